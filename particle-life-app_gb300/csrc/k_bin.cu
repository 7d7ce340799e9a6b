// k_bin.cu — the device counting sort that replaces Physics.makeContainers
// (backend/Physics.java:309-354), plus the host-layout conversion kernels.
//
// Per step (after the force kernel of the previous step, or the upload, has
// written every particle's cell and an in-cell rank and bumped the per-cell
// counts):
//   scan_reduce / scan_parts / scan_down  counts -> exclusive offsets
//                                         (Physics.java:334-340); counts reset
//   scatter   perm[cstart[cell]+rank] = i (unstable: atomics order warps)
//   gather    rank_stable(i) = #{members of i's cell with a smaller index};
//             B[cstart[cell] + rank_stable] = A[i]
// The gather makes the sort stable, so the cell-sorted order equals the one
// the reference's sequential scatter (Physics.java:342-348) produces.  The
// stable re-rank costs sum_c n_c^2 compares, a ninth of the force loop's
// sum_c n_c * (9 neighbour cells) candidate tests.
#include "plg_internal.cuh"

namespace plg {

namespace {

constexpr int kThreads = 256;
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

inline int blocks_for(int n, int threads) { return (n + threads - 1) / threads; }

// ---- upload: host double layout -> FP32 SoA, validation, first binning ----

template <int D>
__global__ void __launch_bounds__(kThreads) k_upload(int n, const double* __restrict__ pos,
                                                     const double* __restrict__ vel,
                                                     const int32_t* __restrict__ type, int ntypes,
                                                     StateBuf<D> a, uint32_t* __restrict__ cell,
                                                     uint32_t* __restrict__ rank, uint32_t* counts, Grid g,
                                                     uint32_t* status) {
    const int i = blockIdx.x * kThreads + threadIdx.x;
    const bool valid = i < n;
    uint32_t c = 0;
    uint32_t bad = 0;
    if (valid) {
        float p[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            double x = pos[3 * (size_t)i + k];
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
                double x = vel[3 * (size_t)i + k];
                if (!isfinite(x)) {
                    bad |= kDevBadVelocity;
                    x = 0.0;
                }
                v[k] = __double2float_rn(x);
            }
        }
        int t = type[i];
        if (t < 0 || t >= ntypes) {
            bad |= kDevBadType;
            t = 0;
        }
        if constexpr (D == 2) {
            a.pt[i] = make_float4(p[0], p[1], __int_as_float(t), __int_as_float(i));
            reinterpret_cast<float2*>(a.vel)[i] = make_float2(v[0], v[1]);
        } else {
            a.pt[i] = make_float4(p[0], p[1], p[2], __int_as_float(t));
            reinterpret_cast<float4*>(a.vel)[i] = make_float4(v[0], v[1], v[2], __int_as_float(i));
        }
        c = cell_index<D>(p[0], p[1], p[2], g);
        if (bad) atomicOr(status, bad);
    }
    const unsigned mask = __ballot_sync(kFull, valid);
    if (valid) {
        rank[i] = bin_count(counts, c, mask);
        cell[i] = c;
    }
}

// Re-binning of the current state (after an rmax change).
template <int D>
__global__ void __launch_bounds__(kThreads) k_rebin(int n, StateBuf<D> a, uint32_t* __restrict__ cell,
                                                    uint32_t* __restrict__ rank, uint32_t* counts, Grid g) {
    const int i = blockIdx.x * kThreads + threadIdx.x;
    const bool valid = i < n;
    uint32_t c = 0;
    if (valid) {
        const float4 p = a.pt[i];
        c = cell_index<D>(p.x, p.y, D == 3 ? p.z : 0.f, g);
    }
    const unsigned mask = __ballot_sync(kFull, valid);
    if (valid) {
        rank[i] = bin_count(counts, c, mask);
        cell[i] = c;
    }
}

// ---- download: FP32 SoA -> PhysicsSnapshot layout (app/PhysicsSnapshot.java:50-58) ----

template <int D>
__global__ void __launch_bounds__(kThreads) k_download(int n, StateBuf<D> a, double* __restrict__ pos,
                                                       double* __restrict__ vel, int32_t* __restrict__ type,
                                                       int32_t* __restrict__ id) {
    const int i = blockIdx.x * kThreads + threadIdx.x;
    if (i >= n) return;
    const float4 p = a.pt[i];
    const typename Layout<D>::Vel v = a.vel[i];
    if (pos) {
        pos[3 * (size_t)i + 0] = p.x;
        pos[3 * (size_t)i + 1] = p.y;
        pos[3 * (size_t)i + 2] = D == 3 ? p.z : 0.0;
    }
    if (vel) {
        vel[3 * (size_t)i + 0] = v.x;
        vel[3 * (size_t)i + 1] = v.y;
        if constexpr (D == 3) {
            vel[3 * (size_t)i + 2] = v.z;
        } else {
            vel[3 * (size_t)i + 2] = 0.0;
        }
    }
    if (type) type[i] = Layout<D>::type(p);
    if (id) id[i] = Layout<D>::id(p, v);
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
    if (warp == 0) {  // kScanThreads / 32 == 32 warp sums, one per lane
        const uint32_t s = warp_sums[lane];
        const uint32_t si = warp_inclusive(s);
        warp_sums[lane] = si - s;
        if (lane == 31) *total = si;
    }
    __syncthreads();
    const uint32_t r = warp_sums[warp] + inc - v;
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const uint32_t* __restrict__ counts, int ncells,
                                                              uint32_t* __restrict__ parts) {
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < ncells) s += counts[base + k];
    }
    __shared__ uint32_t red[kScanThreads / 32];
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) s += __shfl_down_sync(kFull, s, d);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        uint32_t t = red[threadIdx.x];
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) t += __shfl_down_sync(kFull, t, d);
        if (threadIdx.x == 0) parts[blockIdx.x] = t;
    }
}

// One block: exclusive scan of the per-tile sums, in place.
__global__ void __launch_bounds__(kScanThreads) k_scan_parts(uint32_t* parts, int nparts) {
    __shared__ uint32_t carry_s;
    __shared__ uint32_t total;
    if (threadIdx.x == 0) carry_s = 0;
    __syncthreads();
    for (int base = 0; base < nparts; base += kScanThreads) {
        const int i = base + threadIdx.x;
        const uint32_t v = i < nparts ? parts[i] : 0u;
        const uint32_t ex = block_exclusive(v, &total);
        const uint32_t carry = carry_s;
        if (i < nparts) parts[i] = carry + ex;
        __syncthreads();
        if (threadIdx.x == 0) carry_s = carry + total;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_down(uint32_t* __restrict__ counts, int ncells,
                                                            const uint32_t* __restrict__ parts,
                                                            uint32_t* __restrict__ cstart) {
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = base + k < ncells ? counts[base + k] : 0u;
        s += v[k];
    }
    __shared__ uint32_t total;
    uint32_t run = block_exclusive(s, &total) + parts[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int c = base + k;
        if (c < ncells) {
            cstart[c] = run;
            counts[c] = 0;  // ready for the next counting pass
            if (c == ncells - 1) cstart[ncells] = run + v[k];
        }
        run += v[k];
    }
}

__global__ void __launch_bounds__(kThreads) k_scatter(int n, const uint32_t* __restrict__ cell,
                                                      const uint32_t* __restrict__ rank,
                                                      const uint32_t* __restrict__ cstart,
                                                      uint32_t* __restrict__ perm) {
    const int i = blockIdx.x * kThreads + threadIdx.x;
    if (i >= n) return;
    perm[cstart[cell[i]] + rank[i]] = (uint32_t)i;
}

template <int D>
__global__ void __launch_bounds__(kThreads) k_gather(int n, const uint32_t* __restrict__ perm,
                                                     const uint32_t* __restrict__ cell,
                                                     const uint32_t* __restrict__ cstart, StateBuf<D> a,
                                                     StateBuf<D> b, int32_t* __restrict__ cell_sorted) {
    const int s = blockIdx.x * kThreads + threadIdx.x;
    if (s >= n) return;
    const uint32_t i = perm[s];
    const uint32_t c = cell[i];
    const uint32_t st = cstart[c], en = cstart[c + 1];
    uint32_t r = 0;
    for (uint32_t t = st; t < en; ++t) r += __ldg(perm + t) < i ? 1u : 0u;
    const uint32_t d = st + r;
    b.pt[d] = a.pt[i];
    b.vel[d] = a.vel[i];
    if (cell_sorted) cell_sorted[d] = (int32_t)c;
}

}  // namespace

template <int D>
void launch_upload(cudaStream_t st, int n, const double* pos, const double* vel, const int32_t* type, int ntypes,
                   StateBuf<D> a, uint32_t* cell, uint32_t* rank, uint32_t* counts, Grid g, uint32_t* status) {
    if (n <= 0) return;
    k_upload<D><<<blocks_for(n, kThreads), kThreads, 0, st>>>(n, pos, vel, type, ntypes, a, cell, rank, counts, g,
                                                              status);
}

template <int D>
void launch_rebin(cudaStream_t st, int n, StateBuf<D> a, uint32_t* cell, uint32_t* rank, uint32_t* counts, Grid g) {
    if (n <= 0) return;
    k_rebin<D><<<blocks_for(n, kThreads), kThreads, 0, st>>>(n, a, cell, rank, counts, g);
}

template <int D>
void launch_download(cudaStream_t st, int n, StateBuf<D> a, double* pos, double* vel, int32_t* type, int32_t* id) {
    if (n <= 0) return;
    k_download<D><<<blocks_for(n, kThreads), kThreads, 0, st>>>(n, a, pos, vel, type, id);
}

int scan_blocks(int ncells) { return blocks_for(ncells, kScanTile); }

void launch_scan_reduce(cudaStream_t st, const uint32_t* counts, int ncells, uint32_t* parts) {
    k_scan_reduce<<<scan_blocks(ncells), kScanThreads, 0, st>>>(counts, ncells, parts);
}

void launch_scan_parts(cudaStream_t st, uint32_t* parts, int nparts) {
    k_scan_parts<<<1, kScanThreads, 0, st>>>(parts, nparts);
}

void launch_scan_down(cudaStream_t st, uint32_t* counts, int ncells, const uint32_t* parts, uint32_t* cstart) {
    k_scan_down<<<scan_blocks(ncells), kScanThreads, 0, st>>>(counts, ncells, parts, cstart);
}

void launch_scatter(cudaStream_t st, int n, const uint32_t* cell, const uint32_t* rank, const uint32_t* cstart,
                    uint32_t* perm) {
    if (n <= 0) return;
    k_scatter<<<blocks_for(n, kThreads), kThreads, 0, st>>>(n, cell, rank, cstart, perm);
}

template <int D>
void launch_gather(cudaStream_t st, int n, const uint32_t* perm, const uint32_t* cell, const uint32_t* cstart,
                   StateBuf<D> a, StateBuf<D> b, int32_t* cell_sorted) {
    if (n <= 0) return;
    k_gather<D><<<blocks_for(n, kThreads), kThreads, 0, st>>>(n, perm, cell, cstart, a, b, cell_sorted);
}

template void launch_upload<2>(cudaStream_t, int, const double*, const double*, const int32_t*, int, StateBuf<2>,
                               uint32_t*, uint32_t*, uint32_t*, Grid, uint32_t*);
template void launch_upload<3>(cudaStream_t, int, const double*, const double*, const int32_t*, int, StateBuf<3>,
                               uint32_t*, uint32_t*, uint32_t*, Grid, uint32_t*);
template void launch_rebin<2>(cudaStream_t, int, StateBuf<2>, uint32_t*, uint32_t*, uint32_t*, Grid);
template void launch_rebin<3>(cudaStream_t, int, StateBuf<3>, uint32_t*, uint32_t*, uint32_t*, Grid);
template void launch_download<2>(cudaStream_t, int, StateBuf<2>, double*, double*, int32_t*, int32_t*);
template void launch_download<3>(cudaStream_t, int, StateBuf<3>, double*, double*, int32_t*, int32_t*);
template void launch_gather<2>(cudaStream_t, int, const uint32_t*, const uint32_t*, const uint32_t*, StateBuf<2>,
                               StateBuf<2>, int32_t*);
template void launch_gather<3>(cudaStream_t, int, const uint32_t*, const uint32_t*, const uint32_t*, StateBuf<3>,
                               StateBuf<3>, int32_t*);

}  // namespace plg
