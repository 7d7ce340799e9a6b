// k_bin.cu — the device counting sort that replaces Physics.makeContainers
// (backend/Physics.java:309-354), plus the host-layout conversion kernels.
//
// Per step (after the force kernel of the previous step, or the upload, has
// written every particle's cell and bumped the per-cell counts):
//   scan      counts -> exclusive offsets (Physics.java:334-340), single
//             pass with decoupled look-back
//   scatter   perm[cstart[cell] + r] = i with an in-cell rank r taken from
//             the counts (unstable: atomics order warps; the counts drain
//             back to zero), and the cell of that slot
//   gather    rank_stable(i) = #{members of i's cell with a smaller index};
//             B[cstart[cell] + rank_stable] = A[i]
// The gather makes the sort stable, so the cell-sorted order equals the one
// the reference's sequential scatter (Physics.java:342-348) produces.  The
// stable re-rank costs sum_c n_c^2 compares, a ninth of the force loop's
// sum_c n_c * (9 neighbour cells) candidate tests.
#include "plg_internal.cuh"
#include "plgpu.h"

namespace plg {

namespace {

constexpr int kThreads = 256;
constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;

inline int blocks_for(int n, int threads) { return (n + threads - 1) / threads; }

// ---- upload: host double layout -> FP32 SoA, validation, first binning ----

// The host arrays may be page-locked host memory read in place over the host
// link, so each block moves its particles' interleaved doubles through shared
// memory with warp-contiguous 16-byte accesses (`vec`: the array bases are
// 16-byte aligned; block offsets are multiples of 256 * 24 bytes).
__device__ __forceinline__ void block_copy_in(double* __restrict__ dst, const double* __restrict__ src, int cnt,
                                              bool vec) {
    if (vec) {
        const int c2 = cnt >> 1;
        for (int k = threadIdx.x; k < c2; k += kThreads)
            reinterpret_cast<double2*>(dst)[k] = reinterpret_cast<const double2*>(src)[k];
        if ((cnt & 1) && threadIdx.x == 0) dst[cnt - 1] = src[cnt - 1];
    } else {
        for (int k = threadIdx.x; k < cnt; k += kThreads) dst[k] = src[k];
    }
}

__device__ __forceinline__ void block_copy_out(double* __restrict__ dst, const double* __restrict__ src, int cnt,
                                               bool vec) {
    if (vec) {
        const int c2 = cnt >> 1;
        for (int k = threadIdx.x; k < c2; k += kThreads)
            reinterpret_cast<double2*>(dst)[k] = reinterpret_cast<const double2*>(src)[k];
        if ((cnt & 1) && threadIdx.x == 0) dst[cnt - 1] = src[cnt - 1];
    } else {
        for (int k = threadIdx.x; k < cnt; k += kThreads) dst[k] = src[k];
    }
}

template <int D>
__global__ void __launch_bounds__(kThreads) k_upload(int n, const double* __restrict__ pos,
                                                     const double* __restrict__ vel,
                                                     const int32_t* __restrict__ type, int ntypes,
                                                     StateBuf<D> a, uint32_t* __restrict__ cell,
                                                     uint32_t* counts, Grid g, uint32_t* status, bool vec,
                                                     uint32_t cell_base, int id_base) {
    __shared__ __align__(16) double sp[3 * kThreads];
    __shared__ __align__(16) double sv[3 * kThreads];
    const int i0 = blockIdx.x * kThreads;
    const int m = min(kThreads, n - i0);
    block_copy_in(sp, pos + 3 * (size_t)i0, 3 * m, vec);
    if (vel) block_copy_in(sv, vel + 3 * (size_t)i0, 3 * m, vec);
    __syncthreads();
    const int t = threadIdx.x;
    const int i = i0 + t;
    const bool valid = t < m;
    uint32_t c = 0;
    uint32_t bad = 0;
    if (valid) {
        float p[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            double x = sp[3 * t + k];
            if (k < D && !(x >= 0.0 && x <= 1.0)) {  // also rejects NaN
                bad |= kDevBadPosition;
                x = 0.0;
            }
            p[k] = k < D ? __double2float_rn(x) : 0.0f;
        }
        float v[3] = {0.f, 0.f, 0.f};
        if (vel) {
#pragma unroll
            for (int k = 0; k < D; ++k) {
                double x = sv[3 * t + k];
                if (!isfinite(x)) {
                    bad |= kDevBadVelocity;
                    x = 0.0;
                }
                v[k] = __double2float_rn(x);
            }
        }
        int ty = type[i];
        if (ty < 0 || ty >= ntypes) {
            bad |= kDevBadType;
            ty = 0;
        }
        if constexpr (D == 2) {
            a.pt[i] = make_float4(p[0], p[1], __int_as_float(ty), __int_as_float(id_base + i));
            reinterpret_cast<float2*>(a.vel)[i] = make_float2(v[0], v[1]);
        } else {
            a.pt[i] = make_float4(p[0], p[1], p[2], __int_as_float(ty));
            reinterpret_cast<float4*>(a.vel)[i] = make_float4(v[0], v[1], v[2], __int_as_float(id_base + i));
        }
        c = cell_base + cell_index<D>(p[0], p[1], p[2], g);
        if (bad) atomicOr(status, bad);
    }
    const unsigned mask = __ballot_sync(kFull, valid);
    if (valid) {
        bin_add(counts, c, mask);
        cell[i] = c;
    }
}

// ---- batched worlds ----

template <int D>
__global__ void __launch_bounds__(kThreads) k_batch_move(int n, const int* __restrict__ new_off,
                                                         const int* __restrict__ old_off, int nw, StateBuf<D> a,
                                                         StateBuf<D> b) {
    const int s = blockIdx.x * kThreads + threadIdx.x;
    if (s >= n) return;
    const int k = world_of(new_off, nw, s);
    const int src = __ldg(old_off + k) + (s - __ldg(new_off + k));
    b.pt[s] = a.pt[src];
    b.vel[s] = a.vel[src];
}

template <int D>
__global__ void __launch_bounds__(kThreads) k_batch_rebin(int n, StateBuf<D> a, const ForceParams* __restrict__ worlds,
                                                          const int* __restrict__ wp_off, int nw,
                                                          uint32_t* __restrict__ cell, uint32_t* counts) {
    const int i = blockIdx.x * kThreads + threadIdx.x;
    const bool valid = i < n;
    uint32_t c = 0;
    if (valid) {
        const ForceParams& P = worlds[world_of(wp_off, nw, i)];
        const float4 p = a.pt[i];
        c = P.cell_base + cell_index<D>(p.x, p.y, D == 3 ? p.z : 0.f, P.g);
    }
    const unsigned mask = __ballot_sync(kFull, valid);
    if (valid) {
        bin_add(counts, c, mask);
        cell[i] = c;
    }
}

__global__ void k_batch_tick(int* steps_left, int nworlds) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nworlds && steps_left[k] > 0) steps_left[k] -= 1;
}

// Re-binning of the current state (after an rmax change, or of a world
// generated on the device; cell_base: the world's first global cell).
template <int D>
__global__ void __launch_bounds__(kThreads) k_rebin(int n, StateBuf<D> a, uint32_t* __restrict__ cell,
                                                    uint32_t* counts, Grid g, uint32_t cell_base) {
    const int i = blockIdx.x * kThreads + threadIdx.x;
    const bool valid = i < n;
    uint32_t c = 0;
    if (valid) {
        const float4 p = a.pt[i];
        c = cell_base + cell_index<D>(p.x, p.y, D == 3 ? p.z : 0.f, g);
    }
    const unsigned mask = __ballot_sync(kFull, valid);
    if (valid) {
        bin_add(counts, c, mask);
        cell[i] = c;
    }
}

// ---- download: FP32 SoA -> PhysicsSnapshot layout (app/PhysicsSnapshot.java:50-58) ----

// Like the upload, the interleaved doubles leave through shared memory with
// warp-contiguous 16-byte stores (the destination may be page-locked host
// memory written in place).
template <int D>
__global__ void __launch_bounds__(kThreads) k_download(int n, StateBuf<D> a, double* __restrict__ pos,
                                                       double* __restrict__ vel, int32_t* __restrict__ type,
                                                       int32_t* __restrict__ id, bool vec) {
    __shared__ __align__(16) double sp[3 * kThreads];
    __shared__ __align__(16) double sv[3 * kThreads];
    const int i0 = blockIdx.x * kThreads;
    const int m = min(kThreads, n - i0);
    const int t = threadIdx.x;
    const int i = i0 + t;
    if (t < m) {
        const float4 p = a.pt[i];
        const typename Layout<D>::Vel v = a.vel[i];
        sp[3 * t + 0] = p.x;
        sp[3 * t + 1] = p.y;
        sp[3 * t + 2] = D == 3 ? p.z : 0.0;
        sv[3 * t + 0] = v.x;
        sv[3 * t + 1] = v.y;
        if constexpr (D == 3) {
            sv[3 * t + 2] = v.z;
        } else {
            sv[3 * t + 2] = 0.0;
        }
        if (type) type[i] = Layout<D>::type(p);
        if (id) id[i] = Layout<D>::id(p, v);
    }
    __syncthreads();
    if (pos) block_copy_out(pos + 3 * (size_t)i0, sp, 3 * m, vec);
    if (vel) block_copy_out(vel + 3 * (size_t)i0, sv, 3 * m, vec);
}

// ---- block scan helpers ----

__device__ __forceinline__ uint32_t warp_inclusive(uint32_t v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t t = __shfl_up_sync(kFull, v, d);
        if (lane >= d) v += t;
    }
    return v;
}

// Exclusive scan of one value per thread over a block of kScanThreads;
// returns the exclusive prefix, writes the block total to *total.
__device__ __forceinline__ uint32_t block_exclusive(uint32_t v, uint32_t* total) {
    __shared__ uint32_t warp_sums[kScanThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t inc = warp_inclusive(v);
    if (lane == 31) warp_sums[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        constexpr int kWarps = kScanThreads / 32;
        const uint32_t s = lane < kWarps ? warp_sums[lane] : 0u;
        const uint32_t si = warp_inclusive(s);
        if (lane < kWarps) warp_sums[lane] = si - s;
        if (lane == 31) *total = si;
    }
    __syncthreads();
    const uint32_t r = warp_sums[warp] + inc - v;
    __syncthreads();
    return r;
}

constexpr unsigned long long kTileAggregate = 1ull << 32;  // status word: tile sum published
constexpr unsigned long long kTileInclusive = 2ull << 32;  // status word: prefix through tile
constexpr int kLookbackSpinLimit = 1 << 22;

__device__ __forceinline__ unsigned long long load_volatile(const unsigned long long* p) {
    return *reinterpret_cast<const volatile unsigned long long*>(p);
}

// Single-pass exclusive scan of the per-cell counts (capacity -> index,
// Physics.java:334-340) with decoupled look-back: each block takes the next
// tile id, publishes its tile sum, and adds the sums of earlier tiles until it
// meets a published inclusive prefix.  Tile ids follow block start order, so
// a block only waits on blocks that are already running; every wait is
// bounded and raises kDevSpinLimit instead of hanging.  The counts stay
// (the scatter drains them).  state[0] is the tile counter and
// state[1 + t] the status word of tile t; both start at zero each step.
__global__ void __launch_bounds__(kScanThreads) k_scan(const uint32_t* __restrict__ counts, int ncells,
                                                       uint32_t* __restrict__ cstart, unsigned long long* state,
                                                       uint32_t* status, uint32_t* zero_word) {
    __shared__ uint32_t s_tile, s_prefix, total;
    pdl_release();  // the scatter's blocks may be scheduled as this grid ends
    if (threadIdx.x == 0) s_tile = atomicAdd(reinterpret_cast<unsigned int*>(state), 1u);
    // Launched after the force kernel (launch_scan's `after`), the blocks
    // may start while it drains: the counts and the deferred-target count
    // are read or reset only once it has completed.
    pdl_wait();
    __syncthreads();
    const int tile = (int)s_tile;
    if (tile == 0 && threadIdx.x == 0 && zero_word) *zero_word = 0u;  // the step's deferred-target count
    unsigned long long* flags = state + 1;
    const int base = tile * kScanTile + threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    if (base + kScanItems <= ncells) {
#pragma unroll
        for (int q4 = 0; q4 < kScanItems / 4; ++q4) {
            const uint4 q = *reinterpret_cast<const uint4*>(counts + base + 4 * q4);
            v[4 * q4] = q.x;
            v[4 * q4 + 1] = q.y;
            v[4 * q4 + 2] = q.z;
            v[4 * q4 + 3] = q.w;
        }
    } else {
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) v[k] = base + k < ncells ? counts[base + k] : 0u;
    }
    uint32_t sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) sum += v[k];
    const uint32_t ex = block_exclusive(sum, &total);
    if (threadIdx.x < 32) {
        // Warp-parallel look-back: lanes read the status words of the 32
        // nearest earlier tiles; the sums of tiles up to the nearest one with
        // a published inclusive prefix (tile -1 counts as inclusive 0) are
        // added, otherwise the window moves 32 tiles back.
        const int lane = threadIdx.x;
        uint32_t excl = 0;
        if (tile == 0) {
            if (lane == 0) atomicExch(flags, kTileInclusive | total);
        } else {
            if (lane == 0) atomicExch(flags + tile, kTileAggregate | total);
            for (int p = tile - 1;; p -= 32) {
                const int idx = p - lane;
                unsigned long long f = idx >= 0 ? load_volatile(flags + idx) : kTileInclusive;
                int spins = 0;
                while ((f >> 32) == 0ull) {
                    if (++spins > kLookbackSpinLimit) {
                        atomicOr(status, kDevSpinLimit);
                        f = kTileInclusive;
                        break;
                    }
                    __nanosleep(64);
                    f = load_volatile(flags + idx);
                }
                const unsigned inc = __ballot_sync(kFull, (f >> 32) == 2ull);
                const int last = inc ? __ffs(inc) - 1 : 31;
                uint32_t v = lane <= last ? (uint32_t)f : 0u;
#pragma unroll
                for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(kFull, v, d);
                excl += v;
                if (inc) break;
            }
            if (lane == 0) atomicExch(flags + tile, kTileInclusive | (excl + total));
        }
        if (lane == 0) s_prefix = excl;
    }
    __syncthreads();
    uint32_t run = s_prefix + ex;
    if (base + kScanItems <= ncells) {
#pragma unroll
        for (int q4 = 0; q4 < kScanItems / 4; ++q4) {
            uint4 o;
            o.x = run;
            o.y = o.x + v[4 * q4];
            o.z = o.y + v[4 * q4 + 1];
            o.w = o.z + v[4 * q4 + 2];
            run = o.w + v[4 * q4 + 3];
            *reinterpret_cast<uint4*>(cstart + base + 4 * q4) = o;
        }
        if (base + kScanItems == ncells) cstart[ncells] = run;
    } else {
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            const int c = base + k;
            if (c < ncells) {
                cstart[c] = run;
                if (c == ncells - 1) cstart[ncells] = run + v[k];
            }
            run += v[k];
        }
    }
}

// Each particle takes a slot of its cell (the ranks drain counts back to
// zero for the next counting pass).  kScatterPer particles per thread, their
// atomics in flight together.
constexpr int kScatterPer = 4;
__global__ void __launch_bounds__(kThreads) k_scatter(int n, const uint32_t* __restrict__ cell, uint32_t* counts,
                                                      const uint32_t* __restrict__ cstart,
                                                      uint32_t* __restrict__ perm, uint32_t* __restrict__ slot_cell,
                                                      unsigned long long* zero_state, int nzero) {
    pdl_release();
    const int i0 = blockIdx.x * (kThreads * kScatterPer) + threadIdx.x;
    const int lane = threadIdx.x & 31;
    uint32_t c[kScatterPer], top[kScatterPer];
    unsigned peers[kScatterPer];
    bool v[kScatterPer];
#pragma unroll
    for (int k = 0; k < kScatterPer; ++k) {
        const int i = i0 + k * kThreads;
        v[k] = i < n;
        c[k] = v[k] ? cell[i] : 0u;  // written before the scan: needs no wait
    }
    pdl_wait();  // the scan's offsets, and its reads of the counts, are done
    if (zero_state && blockIdx.x == 0)
        for (int k = threadIdx.x; k < nzero; k += kThreads) zero_state[k] = 0ull;
#pragma unroll
    for (int k = 0; k < kScatterPer; ++k) {
        const unsigned m = __ballot_sync(kFull, v[k]);
        peers[k] = 0u;
        top[k] = 0u;
        if (v[k]) {
            peers[k] = __match_any_sync(m, c[k]);
            if (lane == __ffs(peers[k]) - 1) top[k] = atomicSub(counts + c[k], (uint32_t)__popc(peers[k]));
        }
    }
#pragma unroll
    for (int k = 0; k < kScatterPer; ++k) {
        if (!v[k]) continue;
        const unsigned pk = peers[k];
        const uint32_t t = __shfl_sync(pk, top[k], __ffs(pk) - 1);
        const uint32_t r = t - (uint32_t)__popc(pk) + (uint32_t)__popc(pk & ((1u << lane) - 1u));
        const uint32_t slot = __ldg(cstart + c[k]) + r;
        perm[slot] = (uint32_t)(i0 + k * kThreads);
        if (slot_cell) slot_cell[slot] = c[k];
    }
}

// Places particle i = perm[s] at its rank among its cell's members by
// index: the order of the reference's sequential scatter
// (Physics.java:342-348).
// slot_cell[s] is the cell of slot s (written by the scatter), so the
// cell offsets and the particle's state load in parallel.
template <int D>
__global__ void __launch_bounds__(kThreads) k_gather(int n, const uint32_t* __restrict__ perm,
                                                     const uint32_t* __restrict__ slot_cell,
                                                     const uint32_t* __restrict__ cstart, StateBuf<D> a,
                                                     StateBuf<D> b, int32_t* __restrict__ cell_sorted) {
    pdl_release();
    pdl_wait();  // the scatter's perm and slot_cell
    const int s = blockIdx.x * kThreads + threadIdx.x;
    if (s >= n) return;
    const uint32_t i = perm[s];
    const uint32_t c = slot_cell[s];
    const uint32_t st = cstart[c], en = cstart[c + 1];
    const float4 p = a.pt[i];
    const typename Layout<D>::Vel v = a.vel[i];
    uint32_t r = 0;
    for (uint32_t t = st; t < en; ++t) r += __ldg(perm + t) < i ? 1u : 0u;
    b.pt[st + r] = p;
    b.vel[st + r] = v;
    if (cell_sorted) cell_sorted[st + r] = (int32_t)c;
}

}  // namespace

inline bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

template <int D>
void launch_upload(cudaStream_t st, int n, const double* pos, const double* vel, const int32_t* type, int ntypes,
                   StateBuf<D> a, uint32_t* cell, uint32_t* counts, Grid g, uint32_t* status, uint32_t cell_base,
                   int id_base) {
    if (n <= 0) return;
    const bool vec = aligned16(pos) && aligned16(vel);
    k_upload<D><<<blocks_for(n, kThreads), kThreads, 0, st>>>(n, pos, vel, type, ntypes, a, cell, counts, g, status,
                                                              vec, cell_base, id_base);
}

template <int D>
void launch_batch_move(cudaStream_t st, int n, const int* new_off, const int* old_off, int nw, StateBuf<D> a,
                       StateBuf<D> b) {
    if (n <= 0 || nw <= 0) return;
    k_batch_move<D><<<blocks_for(n, kThreads), kThreads, 0, st>>>(n, new_off, old_off, nw, a, b);
}

template <int D>
void launch_batch_rebin(cudaStream_t st, int n, StateBuf<D> a, const ForceParams* worlds, const int* wp_off, int nw,
                        uint32_t* cell, uint32_t* counts) {
    if (n <= 0 || nw <= 0) return;
    k_batch_rebin<D><<<blocks_for(n, kThreads), kThreads, 0, st>>>(n, a, worlds, wp_off, nw, cell, counts);
}

void launch_batch_tick(cudaStream_t st, int* steps_left, int nworlds) {
    if (nworlds <= 0 || !steps_left) return;
    k_batch_tick<<<blocks_for(nworlds, kThreads), kThreads, 0, st>>>(steps_left, nworlds);
}

template void launch_batch_move<2>(cudaStream_t, int, const int*, const int*, int, StateBuf<2>, StateBuf<2>);
template void launch_batch_move<3>(cudaStream_t, int, const int*, const int*, int, StateBuf<3>, StateBuf<3>);
template void launch_batch_rebin<2>(cudaStream_t, int, StateBuf<2>, const ForceParams*, const int*, int, uint32_t*,
                                    uint32_t*);
template void launch_batch_rebin<3>(cudaStream_t, int, StateBuf<3>, const ForceParams*, const int*, int, uint32_t*,
                                    uint32_t*);

template <int D>
void launch_rebin(cudaStream_t st, int n, StateBuf<D> a, uint32_t* cell, uint32_t* counts, Grid g,
                  uint32_t cell_base) {
    if (n <= 0) return;
    k_rebin<D><<<blocks_for(n, kThreads), kThreads, 0, st>>>(n, a, cell, counts, g, cell_base);
}

template <int D>
void launch_download(cudaStream_t st, int n, StateBuf<D> a, double* pos, double* vel, int32_t* type, int32_t* id) {
    if (n <= 0) return;
    const bool vec = aligned16(pos) && aligned16(vel);
    k_download<D><<<blocks_for(n, kThreads), kThreads, 0, st>>>(n, a, pos, vel, type, id, vec);
}

int scan_blocks(int ncells) { return blocks_for(ncells, kScanTile); }

void launch_scan(cudaStream_t st, const uint32_t* counts, int ncells, uint32_t* cstart, unsigned long long* state,
                 uint32_t* status, uint32_t* zero_word, bool after) {
    if (after)
        launch_after(k_scan, dim3(scan_blocks(ncells)), dim3(kScanThreads), 0, st, counts, ncells, cstart, state,
                     status, zero_word);
    else
        k_scan<<<scan_blocks(ncells), kScanThreads, 0, st>>>(counts, ncells, cstart, state, status, zero_word);
}

void launch_scatter(cudaStream_t st, int n, const uint32_t* cell, uint32_t* counts, const uint32_t* cstart,
                    uint32_t* perm, uint32_t* slot_cell, unsigned long long* zero_state, int nzero) {
    if (n <= 0) return;
    launch_after(k_scatter, dim3(blocks_for(n, kThreads * kScatterPer)), dim3(kThreads), 0, st, n, cell, counts,
                 cstart, perm, slot_cell, zero_state, nzero);
}

template <int D>
void launch_gather(cudaStream_t st, int n, const uint32_t* perm, const uint32_t* slot_cell, const uint32_t* cstart,
                   StateBuf<D> a, StateBuf<D> b, int32_t* cell_sorted) {
    if (n <= 0) return;
    launch_after(k_gather<D>, dim3(blocks_for(n, kThreads)), dim3(kThreads), 0, st, n, perm, slot_cell, cstart, a, b,
                 cell_sorted);
}

template void launch_upload<2>(cudaStream_t, int, const double*, const double*, const int32_t*, int, StateBuf<2>,
                               uint32_t*, uint32_t*, Grid, uint32_t*, uint32_t, int);
template void launch_upload<3>(cudaStream_t, int, const double*, const double*, const int32_t*, int, StateBuf<3>,
                               uint32_t*, uint32_t*, Grid, uint32_t*, uint32_t, int);
template void launch_rebin<2>(cudaStream_t, int, StateBuf<2>, uint32_t*, uint32_t*, Grid, uint32_t);
template void launch_rebin<3>(cudaStream_t, int, StateBuf<3>, uint32_t*, uint32_t*, Grid, uint32_t);
template void launch_download<2>(cudaStream_t, int, StateBuf<2>, double*, double*, int32_t*, int32_t*);
template void launch_download<3>(cudaStream_t, int, StateBuf<3>, double*, double*, int32_t*, int32_t*);
template void launch_gather<2>(cudaStream_t, int, const uint32_t*, const uint32_t*, const uint32_t*, StateBuf<2>,
                               StateBuf<2>, int32_t*);
template void launch_gather<3>(cudaStream_t, int, const uint32_t*, const uint32_t*, const uint32_t*, StateBuf<3>,
                               StateBuf<3>, int32_t*);

}  // namespace plg

// Test hook: the scan's bounded look-back wait runs out on purpose.  One
// block over a two-tile problem whose tile counter starts at 1 takes tile 1
// and waits for tile 0's status word, which no block publishes; after
// kLookbackSpinLimit polls it raises kDevSpinLimit, treats the missing
// prefix as 0 and finishes, so the kernel returns and the context stays
// usable.  Every access stays inside the buffers allocated here.
extern "C" int plg_test_scan_wait(uint32_t* status_out, double* seconds) {
    using namespace plg;
    if (!status_out) return PLG_E_INVALID_ARG;
    const int ncells = 2 * kScanTile;
    uint32_t *counts = nullptr, *cstart = nullptr, *status = nullptr;
    unsigned long long* state = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = PLG_OK;
    auto ok = [&](cudaError_t e) {
        if (e != cudaSuccess && rc == PLG_OK) {
            cudaGetLastError();
            rc = e == cudaErrorMemoryAllocation ? PLG_E_NO_MEMORY : PLG_E_CUDA;
        }
        return rc == PLG_OK;
    };
    const unsigned long long first_tile = 1;
    if (ok(cudaMalloc(&counts, sizeof(uint32_t) * ncells)) &&
        ok(cudaMalloc(&cstart, sizeof(uint32_t) * (ncells + 1))) && ok(cudaMalloc(&status, sizeof(uint32_t))) &&
        ok(cudaMalloc(&state, sizeof(unsigned long long) * 3)) &&
        ok(cudaMemset(counts, 0, sizeof(uint32_t) * ncells)) && ok(cudaMemset(status, 0, sizeof(uint32_t))) &&
        ok(cudaMemset(state, 0, sizeof(unsigned long long) * 3)) &&
        ok(cudaMemcpy(state, &first_tile, sizeof(first_tile), cudaMemcpyHostToDevice)) &&
        ok(cudaEventCreate(&e0)) && ok(cudaEventCreate(&e1)) && ok(cudaEventRecord(e0))) {
        k_scan<<<1, kScanThreads>>>(counts, ncells, cstart, state, status, nullptr);
        if (ok(cudaGetLastError()) && ok(cudaEventRecord(e1)) && ok(cudaEventSynchronize(e1)) &&
            ok(cudaMemcpy(status_out, status, sizeof(uint32_t), cudaMemcpyDeviceToHost))) {
            float ms = 0.f;
            if (seconds && ok(cudaEventElapsedTime(&ms, e0, e1))) *seconds = 1e-3 * ms;
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(counts);
    cudaFree(cstart);
    cudaFree(status);
    cudaFree(state);
    return rc;
}
