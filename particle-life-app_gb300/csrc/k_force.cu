// k_force.cu — fused velocity + position phase of the Particle Life step.
//
// One thread per particle of the cell-sorted order B.  It replaces
//   Physics.updateVelocity  (backend/Physics.java:397-441),
//   the default Accelerator (app/Main.java:275-280),
//   Physics.updatePosition  (backend/Physics.java:443-450) with
//   Range.wrap / Range.clamp (backend/Range.java:40-96),
// and, in its epilogue, the counting pass of the next makeContainers
// (Physics.java:328-332) on the new position.
//
// Tiling.  A block takes 128 consecutive targets of the sorted order.  Their
// cells are nondecreasing, so they fall into a few "segments" (targets of one
// grid row: one y in 2D, one (y, z) in 3D).  For each segment the block stages
// into shared memory, with coalesced loads, the 3 (3D: 9) stencil rows over
// the segment's columns plus one halo column each side; every target then
// reads its 3 (9) candidate runs as contiguous shared-memory ranges.  A
// segment whose stencil does not fit falls back to reading the runs from
// global memory (stencil_scan).
//
// Pair test.  The reference keeps a pair when d2 != 0 && d2 <= rmax*rmax in
// FP64, with d = wrapConnection(q - p) (Physics.java:428-432).  Here d2 is
// first formed in FP32 from differences that are exact or rounded once: a
// periodic image is taken by cell, as (q - 1) - p or q - (p - 1), where the
// shifted operand lies in [0.5, 1] and the shift is exact.  The FP32 d2 is
// within 5 ulp of the FP64 one, so a pair with d2 <= lo is inside, a pair
// with d2 >= hi is outside, and only pairs in the band (lo, hi) or below
// `tiny` are re-decided with the reference's exact FP64 operation sequence
// (rare_pair).  The interacting-pair set is therefore bit-identical to the
// FP64 reference run on the same FP32 positions.
//
// Stencil.  The reference scans the 9 (27) cells around floor(x/cs) without
// clamping (Physics.java:404-409).  For a particle in the last partial cell
// [nx*cs, 1) that base is nx, not the binning cell nx-1.  This kernel uses
// the binning cell; the two stencils differ only by column nx-2 (scanned
// here, not there) and column 1 (scanned there, never within rmax).  A pair
// of column nx-2 within rmax lies within 1e-15 relative of rmax^2, so it
// reaches rare_pair, which rejects it like the reference.  Grids with fewer
// than 3 cells per axis, where the reference visits a cell more than once,
// take the literal path (general_scan).
#include <climits>

#include "plg_internal.cuh"

namespace plg {

namespace {

constexpr int kThreads = 256;       // literal-path kernel
constexpr int kTileThreads = 128;   // tiled kernel: targets per block
constexpr int kTileCap = 1280;      // staged candidates per segment
constexpr int kTileCols = 160;      // segment columns incl. both halos
constexpr int kSmemMatrixMax = 16;  // matrix in shared memory up to 16 x 16

template <int D>
struct ForceArgs {
    ForceParams p;
    const float4* __restrict__ bpt;
    const typename Layout<D>::Vel* __restrict__ bvel;
    const uint32_t* __restrict__ cstart;
    float4* __restrict__ apt;
    typename Layout<D>::Vel* __restrict__ avel;
    uint32_t* __restrict__ cell;
    uint32_t* __restrict__ rank;
    uint32_t* counts;
    uint32_t* defer_count;  // deferred-target list: count, then slots
    uint32_t* defer_list;
    const uint32_t* __restrict__ refslot;  // B slot -> slot in the reference order (A)
    DebugOut dbg;
};

struct Acc {
    float x, y, z;
    int pairs;
    unsigned long long hs, hx, cand;
};

__device__ __forceinline__ double wrap_connection(double v) {
    // Range.wrapConnection(double), backend/Range.java:74-81.
    if (v < -0.5) return __dadd_rn(v, 1.0);
    if (v >= 0.5) return __dsub_rn(v, 1.0);
    return v;
}

// The reference's FP64 pair test and Accelerator on the raw FP32 positions
// (upcast).  Returns (acc contribution, 1) if the pair interacts, w = 0 if
// not.  `slmask` bit k: the target lies in the last partial cell of axis k
// and nx >= 4, so candidates of cell nx-2 on that axis are outside the
// reference's stencil.
template <int D>
__device__ __noinline__ float4 rare_pair(const ForceParams& P, float px, float py, float pz, float4 q, float a,
                                         int slmask) {
    double dx = __dsub_rn((double)q.x, (double)px);
    double dy = __dsub_rn((double)q.y, (double)py);
    double dz = D == 3 ? __dsub_rn((double)q.z, (double)pz) : 0.0;
    if (P.wrap) {
        dx = wrap_connection(dx);
        dy = wrap_connection(dy);
        if (D == 3) dz = wrap_connection(dz);
    }
    // lengthSquared: x*x + (y*y + z*z), unfused.
    const double d2 = __dadd_rn(__dmul_rn(dx, dx), __dadd_rn(__dmul_rn(dy, dy), __dmul_rn(dz, dz)));
    if (!(d2 != 0.0 && d2 <= P.rmax2)) return make_float4(0.f, 0.f, 0.f, 0.f);
    if (slmask) {
        const int m2 = P.g.nx - 2;
        if ((slmask & 1) && axis_cell(q.x, P.g) == m2) return make_float4(0.f, 0.f, 0.f, 0.f);
        if ((slmask & 2) && axis_cell(q.y, P.g) == m2) return make_float4(0.f, 0.f, 0.f, 0.f);
        if (D == 3 && (slmask & 4) && axis_cell(q.z, P.g) == m2) return make_float4(0.f, 0.f, 0.f, 0.f);
    }
    // relativePosition.div(rmax); accelerate(a, pos) (app/Main.java:275-280).
    const double rx = __ddiv_rn(dx, P.rmax), ry = __ddiv_rn(dy, P.rmax), rz = __ddiv_rn(dz, P.rmax);
    const double dist = __dsqrt_rn(__dadd_rn(__dmul_rn(rx, rx), __dadd_rn(__dmul_rn(ry, ry), __dmul_rn(rz, rz))));
    const double beta = P.beta_d;
    double f;
    if (dist < beta) {
        f = __dsub_rn(__ddiv_rn(dist, beta), 1.0);
    } else {
        const double t = fabs(__dsub_rn(__dadd_rn(1.0, beta), __dmul_rn(2.0, dist)));
        f = __dmul_rn((double)a, __dsub_rn(1.0, __ddiv_rn(t, __dsub_rn(1.0, beta))));
    }
    const double k = __ddiv_rn(f, dist);
    return make_float4((float)__dmul_rn(rx, k), (float)__dmul_rn(ry, k), (float)__dmul_rn(rz, k), 1.f);
}

template <int D, bool DBG>
__device__ __forceinline__ void add_pair(Acc& acc, float4 c, unsigned long long hid) {
    acc.x += c.x;
    acc.y += c.y;
    if (D == 3) acc.z += c.z;
    if (DBG) {
        const unsigned long long h = mix64(hid);
        acc.pairs++;
        acc.hs += h;
        acc.hx ^= h;
    }
}

// Particle id of sorted slot j (debug outputs only).
template <int D>
__device__ __forceinline__ unsigned long long id_of(const ForceArgs<D>& A, int j) {
    if constexpr (D == 2) return (unsigned long long)(uint32_t)__float_as_int(__ldg(A.bpt + j).w);
    return (unsigned long long)(uint32_t)__float_as_int(reinterpret_cast<const float4*>(A.bvel)[j].w);
}

// FP32 Accelerator for a pair known to interact: adds d * f / |d| to acc.
// f/|d| = 1/(beta rmax) - 1/|d| below beta rmax (linear repulsion), else
// a (1 - |1 + beta - 2 |d|/rmax| / (1 - beta)) / |d|.
__device__ __forceinline__ void fast_pair(const ForceParams& P, float a, float dx, float dy, float dz, float d2,
                                          Acc& acc) {
    const float inv = rsqrtf(d2);
    const float dist = d2 * inv;
    const float t = fmaf(dist, P.m2_inv_rmax, P.one_plus_beta);
    const float u = fmaf(-fabsf(t), P.inv_one_minus_beta, 1.f);
    const float g = dist < P.beta_rmax ? P.k1 - inv : (a * inv) * u;
    acc.x = fmaf(dx, g, acc.x);
    acc.y = fmaf(dy, g, acc.y);
    acc.z = fmaf(dz, g, acc.z);
}

// ---- global-memory stencil (fallback of the tiled kernel) ----

// Candidates j0 + lane, j0 + lane + step, ... < j1 of one run of consecutive
// cells.  (pxe, pye, pze): target position, minus 1 on an axis where the run
// is the periodic image above the box; qo*: -1 on an axis where the run's own
// coordinates must be shifted down (image below the box).  SHQ: some qo* != 0.
template <int D, bool DBG, bool SHQ>
__device__ __forceinline__ void scan_run(const ForceArgs<D>& A, const float* __restrict__ Mrow, int s, int j0,
                                         int j1, float pxe, float pye, float pze, float qox, float qoy, float qoz,
                                         float px, float py, float pz, int slmask, int lane, int step, Acc& acc) {
    const ForceParams& P = A.p;
    for (int j = j0 + lane; j < j1; j += step) {
        const float4 q = __ldg(A.bpt + j);
        const float dx = (SHQ ? q.x + qox : q.x) - pxe;
        const float dy = (SHQ ? q.y + qoy : q.y) - pye;
        float d2;
        float dz = 0.f;
        if (D == 3) {
            dz = (SHQ ? q.z + qoz : q.z) - pze;
            d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        } else {
            d2 = fmaf(dx, dx, dy * dy);
        }
        const bool other = j != s;
        if (DBG && other) acc.cand++;
        if (other && d2 <= P.lo && d2 >= P.tiny) {
            fast_pair(P, Mrow[Layout<D>::type(q)], dx, dy, dz, d2, acc);
            if (DBG) add_pair<D, true>(acc, make_float4(0.f, 0.f, 0.f, 0.f), id_of<D>(A, j));
        } else if (other && d2 < P.hi) {
            const float4 c = rare_pair<D>(P, px, py, pz, q, Mrow[Layout<D>::type(q)], slmask);
            if (c.w != 0.f) add_pair<D, DBG>(acc, c, DBG ? id_of<D>(A, j) : 0ull);
        }
    }
}

template <int D, bool DBG>
__device__ __forceinline__ void run(const ForceArgs<D>& A, const float* Mrow, int s, int j0, int j1, float pxe,
                                    float pye, float pze, float qox, float qoy, float qoz, float px, float py,
                                    float pz, int slmask, int lane, int step, Acc& acc) {
    if (qox != 0.f || qoy != 0.f || qoz != 0.f) {
        scan_run<D, DBG, true>(A, Mrow, s, j0, j1, pxe, pye, pze, qox, qoy, qoz, px, py, pz, slmask, lane, step, acc);
    } else {
        scan_run<D, DBG, false>(A, Mrow, s, j0, j1, pxe, pye, pze, 0.f, 0.f, 0.f, px, py, pz, slmask, lane, step,
                                acc);
    }
}

// nx >= 3: per row (and layer) of the stencil, the three cells cx-1..cx+1 are
// one run of the sorted order unless the row wraps in x.  This lane takes
// every step-th candidate of each run from its offset `lane`.
template <int D, bool DBG>
__device__ __noinline__ Acc stencil_scan(const ForceArgs<D>& A, const float* Mrow, int s, float px, float py,
                                         float pz, int slmask, int lane, int step) {
    const ForceParams& P = A.p;
    Acc acc = {0.f, 0.f, 0.f, 0, 0ull, 0ull, 0ull};
    const int nx = P.g.nx;
    const int cx = axis_cell(px, P.g), cy = axis_cell(py, P.g), cz = D == 3 ? axis_cell(pz, P.g) : 0;
    const uint32_t* __restrict__ cs = A.cstart;
    for (int oz = (D == 3 ? -1 : 0); oz <= (D == 3 ? 1 : 0); ++oz) {
        int rz = cz + oz;
        float qoz = 0.f, pze = pz;
        if (rz < 0) {
            rz += nx;
            if (P.wrap) qoz = -1.f;
        } else if (rz >= nx) {
            rz -= nx;
            if (P.wrap) pze = pz - 1.f;
        }
        for (int oy = -1; oy <= 1; ++oy) {
            int ry = cy + oy;
            float qoy = 0.f, pye = py;
            if (ry < 0) {
                ry += nx;
                if (P.wrap) qoy = -1.f;
            } else if (ry >= nx) {
                ry -= nx;
                if (P.wrap) pye = py - 1.f;
            }
            const int row = (rz * nx + ry) * nx;
            if (cx >= 1 && cx <= nx - 2) {
                run<D, DBG>(A, Mrow, s, __ldg(cs + row + cx - 1), __ldg(cs + row + cx + 2), px, pye, pze, 0.f, qoy,
                            qoz, px, py, pz, slmask, lane, step, acc);
            } else if (cx == 0) {
                run<D, DBG>(A, Mrow, s, __ldg(cs + row + nx - 1), __ldg(cs + row + nx), px, pye, pze,
                            P.wrap ? -1.f : 0.f, qoy, qoz, px, py, pz, slmask, lane, step, acc);
                run<D, DBG>(A, Mrow, s, __ldg(cs + row), __ldg(cs + row + 2), px, pye, pze, 0.f, qoy, qoz, px, py,
                            pz, slmask, lane, step, acc);
            } else {
                run<D, DBG>(A, Mrow, s, __ldg(cs + row + nx - 2), __ldg(cs + row + nx), px, pye, pze, 0.f, qoy,
                            qoz, px, py, pz, slmask, lane, step, acc);
                run<D, DBG>(A, Mrow, s, __ldg(cs + row), __ldg(cs + row + 1), P.wrap ? px - 1.f : px, pye, pze, 0.f,
                            qoy, qoz, px, py, pz, slmask, lane, step, acc);
            }
        }
    }
    return acc;
}

__device__ __forceinline__ int wrap_container(int c, int n) {
    // wrapContainerX / wrapContainerY, Physics.java:377-395.
    return c < 0 ? c + n : (c >= n ? c - n : c);
}

// Literal stencil of Physics.java:404-421 for grids with nx < 3: unclamped
// base cell, every offset visited (a cell may repeat), each candidate decided
// and evaluated in FP64.
template <int D, bool DBG>
__device__ void general_scan(const ForceArgs<D>& A, const float* Mrow, int s, float px, float py, float pz,
                             Acc& acc) {
    const ForceParams& P = A.p;
    const int nx = P.g.nx;
    const int cx0 = axis_cell_unclamped(px, P.g), cy0 = axis_cell_unclamped(py, P.g);
    const int cz0 = D == 3 ? axis_cell_unclamped(pz, P.g) : 0;
    for (int oz = (D == 3 ? -1 : 0); oz <= (D == 3 ? 1 : 0); ++oz) {
        for (int oy = -1; oy <= 1; ++oy) {
            for (int ox = -1; ox <= 1; ++ox) {
                int cx = wrap_container(cx0 + ox, nx), cy = wrap_container(cy0 + oy, nx);
                int cz = D == 3 ? wrap_container(cz0 + oz, nx) : 0;
                if (P.wrap) {
                    cx = wrap_container(cx, nx);
                    cy = wrap_container(cy, nx);
                    if (D == 3) cz = wrap_container(cz, nx);
                } else if (cx < 0 || cx >= nx || cy < 0 || cy >= nx || (D == 3 && (cz < 0 || cz >= nx))) {
                    continue;
                }
                const int ci = cx + (cy + cz * nx) * nx;
                const int j0 = __ldg(A.cstart + ci), j1 = __ldg(A.cstart + ci + 1);
                for (int j = j0; j < j1; ++j) {
                    if (j == s) continue;
                    if (DBG) acc.cand++;
                    const float4 q = __ldg(A.bpt + j);
                    const float4 c = rare_pair<D>(P, px, py, pz, q, Mrow[Layout<D>::type(q)], 0);
                    if (c.w != 0.f) add_pair<D, DBG>(acc, c, DBG ? id_of<D>(A, j) : 0ull);
                }
            }
        }
    }
}

// Range.wrap (repeated +-1 into [0,1)) is x - floor(x) in FP32 with the same
// rounding: every subtraction of 1 from x >= 1 is exact, and for x < 0 the
// repeated additions round once, at the last one.  A result that rounds up
// to 1 is the periodic image 0.  Range.clamp: [0,1].
__device__ __forceinline__ float ensure_position(float x, int wrap) {
    if (wrap) {
        x = x - floorf(x);
        return x >= 1.f ? 0.f : x;
    }
    return fminf(fmaxf(x, 0.f), 1.f);
}

// Epilogue of one target read from B slot s: v = v ff + acc (rmax force dt),
// x = v dt + x, ensurePosition; the next state goes to A[o], o the slot of
// this particle in the reference order.  Returns the new cell.
template <int D, bool DBG>
__device__ __forceinline__ uint32_t integrate(const ForceArgs<D>& A, int s, int o, const float4& me,
                                              const Acc& acc) {
    const ForceParams& P = A.p;
    typename Layout<D>::Vel v = A.bvel[s];
    const float vx = fmaf(acc.x, P.scale, v.x * P.ff);
    const float vy = fmaf(acc.y, P.scale, v.y * P.ff);
    const float nxp = ensure_position(__fadd_rn(__fmul_rn(vx, P.dt), me.x), P.wrap);
    const float nyp = ensure_position(__fadd_rn(__fmul_rn(vy, P.dt), me.y), P.wrap);
    float nzp = 0.f;
    if constexpr (D == 2) {
        A.apt[o] = make_float4(nxp, nyp, me.z, me.w);
        A.avel[o] = make_float2(vx, vy);
    } else {
        const float vz = fmaf(acc.z, P.scale, v.z * P.ff);
        nzp = ensure_position(__fadd_rn(__fmul_rn(vz, P.dt), me.z), P.wrap);
        A.apt[o] = make_float4(nxp, nyp, nzp, me.w);
        A.avel[o] = make_float4(vx, vy, vz, v.w);
    }
    if (DBG) {
        if (A.dbg.pairs) A.dbg.pairs[o] = acc.pairs;
        if (A.dbg.hsum) A.dbg.hsum[o] = acc.hs;
        if (A.dbg.hxor) A.dbg.hxor[o] = acc.hx;
        if (A.dbg.acc) {
            A.dbg.acc[(size_t)D * o + 0] = acc.x;
            A.dbg.acc[(size_t)D * o + 1] = acc.y;
            if (D == 3) A.dbg.acc[(size_t)D * o + 2] = acc.z;
        }
        if (A.dbg.candidates) atomicAdd(A.dbg.candidates, acc.cand);
    }
    return cell_index<D>(nxp, nyp, nzp, A.p.g);
}

template <int D>
__device__ __forceinline__ int sliver_mask(const ForceParams& P, float px, float py, float pz) {
    if (!P.slmask_ok) return 0;
    return (px >= P.g.b_nx ? 1 : 0) | (py >= P.g.b_nx ? 2 : 0) | (D == 3 && pz >= P.g.b_nx ? 4 : 0);
}

// ---- literal-path kernel (nx < 3) ----

template <int D, bool DBG, bool SMEM_M>
__global__ void __launch_bounds__(kThreads) k_force_general(const __grid_constant__ ForceArgs<D> A) {
    const ForceParams& P = A.p;
    extern __shared__ float smat[];
    const float* M = P.matrix;
    if (SMEM_M) {
        const int nn = P.ntypes * P.ntypes;
        for (int k = threadIdx.x; k < nn; k += kThreads) smat[k] = P.matrix[k];
        __syncthreads();
        M = smat;
    }
    const int s = blockIdx.x * kThreads + threadIdx.x;
    const bool valid = s < P.n;
    uint32_t newcell = 0;
    int o = 0;
    if (valid) {
        const float4 me = A.bpt[s];
        o = (int)A.refslot[s];
        Acc acc = {0.f, 0.f, 0.f, 0, 0ull, 0ull, 0ull};
        general_scan<D, DBG>(A, M + Layout<D>::type(me) * P.ntypes, s, me.x, me.y, D == 3 ? me.z : 0.f, acc);
        newcell = integrate<D, DBG>(A, s, o, me, acc);
    }
    const unsigned mask = __ballot_sync(kFull, valid);
    if (valid) {
        A.rank[o] = bin_count(A.counts, newcell, mask);
        A.cell[o] = newcell;
    }
}

// ---- tiled kernel (nx >= 3) ----

template <int D>
struct TileRows {
    static constexpr int R = D == 3 ? 9 : 3;
};

template <int D>
struct TileSmem {
    static constexpr int R = TileRows<D>::R;
    float4 cand[kTileCap];          // staged candidates (x, y, z|type, type|id)
    int coff[R][kTileCols + 1];     // per stencil row: smem start of each column
    int pst[R][4];                  // per row: smem start of left halo, main, right halo; end
    int pgb[R][3];                  // per row: global start of the three pieces
    float tshy[R], tshz[R];         // per row: 1 where the target must use y - 1 (z - 1)
    int rowid[kTileThreads];
    int colid[kTileThreads];
    int seg[kTileThreads + 1];
    int wsum[kTileThreads / 32];
    int nseg;
    int staged;                     // 1: the segment's stencil is in smem
    float mat[kSmemMatrixMax * kSmemMatrixMax];
};

// Stages the stencil of the segment (grid row `srow`, columns cxa..cxb).
template <int D>
__device__ __forceinline__ void stage_segment(const ForceArgs<D>& A, TileSmem<D>& sm, int srow, int cxa, int cxb) {
    constexpr int R = TileRows<D>::R;
    const ForceParams& P = A.p;
    const int nx = P.g.nx;
    const int tid = threadIdx.x;
    const int cy = D == 3 ? srow % nx : srow, cz = D == 3 ? srow / nx : 0;
    const int ncols = cxb - cxa + 1;
    const uint32_t* __restrict__ cs = A.cstart;
    if (tid < 32) {
        int lenL = 0, lenM = 0, lenR = 0, gL = 0, gM = 0, gR = 0;
        float tsy = 0.f, tsz = 0.f;
        if (tid < R) {
            const int oy = tid % 3 - 1, oz = D == 3 ? tid / 3 - 1 : 0;
            int ry = cy + oy, rz = cz + oz;
            if (ry < 0) {
                ry += nx;
            } else if (ry >= nx) {
                ry -= nx;
                if (P.wrap) tsy = 1.f;
            }
            if (rz < 0) {
                rz += nx;
            } else if (rz >= nx) {
                rz -= nx;
                if (P.wrap) tsz = 1.f;
            }
            const int rb = (rz * nx + ry) * nx;
            const int L = cxa > 0 ? cxa - 1 : nx - 1;
            const int Rc = cxb < nx - 1 ? cxb + 1 : 0;
            gL = (int)__ldg(cs + rb + L);
            lenL = (int)__ldg(cs + rb + L + 1) - gL;
            gM = (int)__ldg(cs + rb + cxa);
            lenM = (int)__ldg(cs + rb + cxb + 1) - gM;
            gR = (int)__ldg(cs + rb + Rc);
            lenR = (int)__ldg(cs + rb + Rc + 1) - gR;
        }
        const int len = lenL + lenM + lenR;
        int incl = len;
#pragma unroll
        for (int d = 1; d < 16; d <<= 1) {
            const int t = __shfl_up_sync(kFull, incl, d);
            if (tid >= d) incl += t;
        }
        const int total = __shfl_sync(kFull, incl, R - 1);
        if (tid < R) {
            const int base = incl - len;
            sm.pst[tid][0] = base;
            sm.pst[tid][1] = base + lenL;
            sm.pst[tid][2] = base + lenL + lenM;
            sm.pst[tid][3] = base + len;
            sm.pgb[tid][0] = gL;
            sm.pgb[tid][1] = gM;
            sm.pgb[tid][2] = gR;
            sm.tshy[tid] = tsy;
            sm.tshz[tid] = tsz;
        }
        if (tid == 0) {
            sm.staged = total <= kTileCap && ncols + 2 <= kTileCols;
        }
    }
    __syncthreads();
    if (!sm.staged) return;
    // Column starts: coff[r][0] = left halo, coff[r][1 + i] = column cxa + i,
    // coff[r][ncols + 1] = right halo, coff[r][ncols + 2] = end.
    const int w = ncols + 3;
    for (int it = tid; it < R * w; it += kTileThreads) {
        const int r = it / w, k = it - r * w;
        int v;
        if (k == 0) {
            v = sm.pst[r][0];
        } else if (k <= ncols + 1) {
            const int oy = r % 3 - 1, oz = D == 3 ? r / 3 - 1 : 0;
            int ry = cy + oy, rz = cz + oz;
            ry = ry < 0 ? ry + nx : (ry >= nx ? ry - nx : ry);
            rz = rz < 0 ? rz + nx : (rz >= nx ? rz - nx : rz);
            v = sm.pst[r][1] + ((int)__ldg(cs + (rz * nx + ry) * nx + cxa + k - 1) - sm.pgb[r][1]);
        } else {
            v = sm.pst[r][3];
        }
        sm.coff[r][k] = v;
    }
    // Candidates, with the exact periodic shifts of images below the box.
    const float sxl = (cxa == 0 && P.wrap) ? -1.f : 0.f;
#pragma unroll 1
    for (int r = 0; r < R; ++r) {
        const int oy = r % 3 - 1, oz = D == 3 ? r / 3 - 1 : 0;
        const float sy = (cy + oy < 0 && P.wrap) ? -1.f : 0.f;
        const float sz = (D == 3 && cz + oz < 0 && P.wrap) ? -1.f : 0.f;
        const int p1 = sm.pst[r][1], p2 = sm.pst[r][2], p3 = sm.pst[r][3];
        for (int k = sm.pst[r][0] + tid; k < p3; k += kTileThreads) {
            const int piece = k < p1 ? 0 : (k < p2 ? 1 : 2);
            const int g = sm.pgb[r][piece] + (k - (piece == 0 ? sm.pst[r][0] : (piece == 1 ? p1 : p2)));
            float4 q = __ldg(A.bpt + g);
            q.y += sy;
            if (D == 3) q.z += sz;
            if (piece == 0) q.x += sxl;
            sm.cand[k] = q;
        }
    }
    __syncthreads();
}

// Global sorted slot of staged candidate j of stencil row r.
template <int D>
__device__ __forceinline__ int staged_global(const TileSmem<D>& sm, int r, int j) {
    const int piece = j < sm.pst[r][1] ? 0 : (j < sm.pst[r][2] ? 1 : 2);
    return sm.pgb[r][piece] + (j - sm.pst[r][piece]);
}

// rsqrt.approx.ftz.f32: the fast path only sees d2 >= 2^-100, a normal float.
__device__ __forceinline__ float rsqrt_approx(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// First pass over staged candidates [j0, j1): branch-free, every lane runs
// the FP32 Accelerator and keeps the term only for pairs decided inside.
// Returns true when some candidate needs the FP64 decision (band or tiny).
template <int D, bool DBG>
__device__ __forceinline__ bool tile_run(const ForceArgs<D>& A, const TileSmem<D>& sm, const float* __restrict__ Mrow,
                                         int r, int j0, int j1, int self_j, float pxe, float pye, float pze,
                                         Acc& acc) {
    const ForceParams& P = A.p;
    bool rare = false;
    auto body = [&](int j) {
        const float4 q = sm.cand[j];
        const float dx = q.x - pxe;
        const float dy = q.y - pye;
        float d2;
        float dz = 0.f;
        if (D == 3) {
            dz = q.z - pze;
            d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        } else {
            d2 = fmaf(dx, dx, dy * dy);
        }
        const bool other = j != self_j;
        const bool fast = other && d2 <= P.lo && d2 >= P.tiny;
        rare |= other && !fast && d2 < P.hi;
        const float a = Mrow[Layout<D>::type(q)];
        const float inv = rsqrt_approx(d2);
        const float dist = d2 * inv;
        const float t = fmaf(dist, P.m2_inv_rmax, P.one_plus_beta);
        const float u = fmaf(-fabsf(t), P.inv_one_minus_beta, 1.f);
        float g = dist < P.beta_rmax ? P.k1 - inv : (a * inv) * u;
        g = fast ? g : 0.f;
        acc.x = fmaf(dx, g, acc.x);
        acc.y = fmaf(dy, g, acc.y);
        if (D == 3) acc.z = fmaf(dz, g, acc.z);
        if (DBG) {
            if (other) acc.cand++;
            if (fast) add_pair<D, true>(acc, make_float4(0.f, 0.f, 0.f, 0.f), id_of<D>(A, staged_global(sm, r, j)));
        }
    };
    int j = j0;
    for (; j + 4 <= j1; j += 4) {
        body(j);
        body(j + 1);
        body(j + 2);
        body(j + 3);
    }
    for (; j < j1; ++j) body(j);
    return rare;
}

// First index in [a, b) whose staged x is >= v (> v when UPPER); NaN
// coordinates, staged last, compare as above every bound.
template <bool UPPER>
__device__ __forceinline__ int search_x(const float4* cand, int a, int b, float v) {
    while (a < b) {
        const int m = (a + b) >> 1;
        const float x = cand[m].x;
        if (UPPER ? x <= v : x < v)
            a = m + 1;
        else
            b = m;
    }
    return a;
}

// An x-sorted part [j0, j1) of a run, cut to the candidates within xwin of
// the target in x: every pair that can pass d2 < hi has |dx| < xwin.
template <int D, bool DBG>
__device__ __forceinline__ bool window_run(const ForceArgs<D>& A, const TileSmem<D>& sm, const float* __restrict__ Mrow,
                                           int r, int j0, int j1, int self_j, float pxe, float pye, float pze,
                                           Acc& acc) {
    if (j0 >= j1) return false;
    const int a = search_x<false>(sm.cand, j0, j1, pxe - A.p.xwin);
    const int b = search_x<true>(sm.cand, a, j1, pxe + A.p.xwin);
    return tile_run<D, DBG>(A, sm, Mrow, r, a, b, self_j, pxe, pye, pze, acc);
}

// Appends the lanes with `want` to the deferred-target list (one atomic per
// warp); every lane of the warp must call.
__device__ __forceinline__ void defer_targets(uint32_t* count, uint32_t* list, bool want, int s) {
    const unsigned m = __ballot_sync(kFull, want);
    if (!m) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(count, (uint32_t)__popc(m));
    base = __shfl_sync(kFull, base, leader);
    if (want) list[base + __popc(m & ((1u << lane) - 1u))] = (uint32_t)s;
}

// Main force kernel (nx >= 3).  FP32 only and call-free: a target whose
// first pass meets a candidate that needs the FP64 decision, or whose
// segment did not fit in shared memory, is deferred to k_force_fixup, which
// recomputes it completely.
template <int D, bool DBG, bool SMEM_M>
__global__ void __launch_bounds__(kTileThreads, 8) k_force_tile(const ForceArgs<D> A) {
    constexpr int R = TileRows<D>::R;
    __shared__ TileSmem<D> sm;
    const ForceParams& P = A.p;
    const int tid = threadIdx.x;
    const int nx = P.g.nx;
    if (SMEM_M) {
        const int nn = P.ntypes * P.ntypes;
        for (int k = tid; k < nn; k += kTileThreads) sm.mat[k] = P.matrix[k];
    }
    const float* M = SMEM_M ? sm.mat : P.matrix;
    const int s = blockIdx.x * kTileThreads + tid;
    const bool valid = s < P.n;
    float4 me = make_float4(0.f, 0.f, 0.f, 0.f);
    int cx = 0, cy = 0, cz = 0;
    if (valid) {
        me = A.bpt[s];
        cx = axis_cell(me.x, P.g);
        cy = axis_cell(me.y, P.g);
        if (D == 3) cz = axis_cell(me.z, P.g);
    }
    const float px = me.x, py = me.y, pz = D == 3 ? me.z : 0.f;
    const int row = valid ? cy + cz * nx : INT_MAX;
    sm.rowid[tid] = row;
    sm.colid[tid] = cx;
    __syncthreads();
    // Segments: maximal runs of targets in one grid row (rows are nondecreasing).
    const bool start = valid && (tid == 0 || sm.rowid[tid - 1] != row);
    const unsigned bal = __ballot_sync(kFull, start);
    if ((tid & 31) == 0) sm.wsum[tid >> 5] = __popc(bal);
    __syncthreads();
    int before = 0;
    for (int w = 0; w < (tid >> 5); ++w) before += sm.wsum[w];
    if (start) sm.seg[before + __popc(bal & ((1u << (tid & 31)) - 1u))] = tid;
    if (tid == 0) {
        int t = 0;
        for (int w = 0; w < kTileThreads / 32; ++w) t += sm.wsum[w];
        sm.nseg = t;
        sm.seg[t] = min(kTileThreads, P.n - (int)blockIdx.x * kTileThreads);
    }
    __syncthreads();
    const int nseg = sm.nseg;

    const float* Mrow = M + (valid ? Layout<D>::type(me) : 0) * P.ntypes;
    Acc acc = {0.f, 0.f, 0.f, 0, 0ull, 0ull, 0ull};
    bool defer = false;
    for (int g = 0; g < nseg; ++g) {
        const int ta = sm.seg[g], tb = sm.seg[g + 1];
        const int cxa = sm.colid[ta], cxb = sm.colid[tb - 1];
        stage_segment<D>(A, sm, sm.rowid[ta], cxa, cxb);
        if (tid >= ta && tid < tb) {
            if (sm.staged) {
                const int ncols = cxb - cxa + 1;
                const int k = cx - cxa + 1;
                // Each cell is staged in x order and columns follow in x, so
                // a run is x-sorted except for a halo column that wraps round
                // the row: the left halo of column 0 (in order only when it
                // is shifted down, i.e. periodic) and the right halo of
                // column nx-1 (column 0's cells, reached through the target
                // at x - 1 when periodic).  Those halos are separate parts.
                const bool lsplit = cxa == 0 && k == 1;
                const bool rsplit = cxb == nx - 1 && k == ncols;
                const float pxr = P.wrap ? px - 1.f : px;
#pragma unroll 1
                for (int r = 0; r < R; ++r) {
                    const float pye = py - sm.tshy[r];
                    const float pze = pz - sm.tshz[r];
                    const int j0 = sm.coff[r][k - 1], j1 = sm.coff[r][k + 2];
                    const int jl = lsplit ? sm.coff[r][1] : j0;
                    const int js = rsplit ? sm.coff[r][ncols + 1] : j1;
                    const int self_j = r == R / 2 ? sm.pst[r][1] + (s - sm.pgb[r][1]) : -1;
                    defer |= window_run<D, DBG>(A, sm, Mrow, r, j0, jl, self_j, px, pye, pze, acc);
                    defer |= window_run<D, DBG>(A, sm, Mrow, r, jl, js, self_j, px, pye, pze, acc);
                    defer |= window_run<D, DBG>(A, sm, Mrow, r, js, j1, self_j, pxr, pye, pze, acc);
                }
            } else {
                defer = true;
            }
        }
        if (g + 1 < nseg) __syncthreads();  // staging of the next segment reuses smem
    }
    const bool done = valid && !defer;
    uint32_t newcell = 0;
    int o = 0;
    if (done) {
        o = (int)A.refslot[s];
        newcell = integrate<D, DBG>(A, s, o, me, acc);
    }
    const unsigned mask = __ballot_sync(kFull, done);
    if (done) {
        A.rank[o] = bin_count(A.counts, newcell, mask);
        A.cell[o] = newcell;
    }
    defer_targets(A.defer_count, A.defer_list, valid && defer, s);
}

// Sum of `v` over the warp in a fixed butterfly order (the same bits on
// every run); every lane receives the total.
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(kFull, v, d);
    return v;
}

// Deferred targets, one warp each: the lanes split the candidates of the
// global-memory stencil (with the FP64 decisions), their partial sums are
// combined by warp_sum, and lane 0 runs the epilogue.
template <int D, bool DBG, bool SMEM_M>
__global__ void __launch_bounds__(kThreads) k_force_fixup(const __grid_constant__ ForceArgs<D> A) {
    const ForceParams& P = A.p;
    __shared__ float smat[kSmemMatrixMax * kSmemMatrixMax];
    const float* M = P.matrix;
    if (SMEM_M) {
        const int nn = P.ntypes * P.ntypes;
        for (int k = threadIdx.x; k < nn; k += kThreads) smat[k] = P.matrix[k];
        __syncthreads();
        M = smat;
    }
    const int lane = threadIdx.x & 31;
    const int warps = gridDim.x * (kThreads / 32);
    const int count = (int)*(volatile const uint32_t*)A.defer_count;
    for (int w = blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5); w < count; w += warps) {
        const int s = (int)A.defer_list[w];
        const float4 me = A.bpt[s];
        const float px = me.x, py = me.y, pz = D == 3 ? me.z : 0.f;
        Acc acc = stencil_scan<D, DBG>(A, M + Layout<D>::type(me) * P.ntypes, s, px, py, pz,
                                       sliver_mask<D>(P, px, py, pz), lane, 32);
        acc.x = warp_sum(acc.x);
        acc.y = warp_sum(acc.y);
        if (D == 3) acc.z = warp_sum(acc.z);
        if (DBG) {
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) {
                acc.pairs += __shfl_xor_sync(kFull, acc.pairs, d);
                acc.hs += __shfl_xor_sync(kFull, acc.hs, d);
                acc.hx ^= __shfl_xor_sync(kFull, acc.hx, d);
                acc.cand += __shfl_xor_sync(kFull, acc.cand, d);
            }
        }
        if (lane == 0) {
            const int o = (int)A.refslot[s];
            const uint32_t newcell = integrate<D, DBG>(A, s, o, me, acc);
            A.rank[o] = atomicAdd(A.counts + newcell, 1u);
            A.cell[o] = newcell;
        }
    }
}

template <int D, bool DBG>
void launch_variant(cudaStream_t st, const ForceArgs<D>& A, bool general, int fixup_blocks) {
    const int n = A.p.n;
    const bool smem = A.p.ntypes <= kSmemMatrixMax;
    if (general) {
        const int grid = (n + kThreads - 1) / kThreads;
        const size_t sb = smem ? sizeof(float) * A.p.ntypes * A.p.ntypes : 0;
        if (smem)
            k_force_general<D, DBG, true><<<grid, kThreads, sb, st>>>(A);
        else
            k_force_general<D, DBG, false><<<grid, kThreads, 0, st>>>(A);
    } else if (fixup_blocks == 0) {
        const int grid = (n + kTileThreads - 1) / kTileThreads;
        if (smem)
            k_force_tile<D, DBG, true><<<grid, kTileThreads, 0, st>>>(A);
        else
            k_force_tile<D, DBG, false><<<grid, kTileThreads, 0, st>>>(A);
    } else {
        if (smem)
            k_force_fixup<D, DBG, true><<<fixup_blocks, kThreads, 0, st>>>(A);
        else
            k_force_fixup<D, DBG, false><<<fixup_blocks, kThreads, 0, st>>>(A);
    }
}

template <int D>
ForceArgs<D> make_args(const ForceParams& p, StateBuf<D> b, const uint32_t* cstart, StateBuf<D> a, uint32_t* cell,
                       uint32_t* rank, uint32_t* counts, uint32_t* defer, const uint32_t* refslot,
                       const DebugOut* dbg) {
    ForceArgs<D> A;
    A.p = p;
    A.bpt = b.pt;
    A.bvel = b.vel;
    A.cstart = cstart;
    A.apt = a.pt;
    A.avel = a.vel;
    A.cell = cell;
    A.rank = rank;
    A.counts = counts;
    A.defer_count = defer;
    A.defer_list = defer + 1;
    A.refslot = refslot;
    A.dbg = dbg ? *dbg : DebugOut{nullptr, nullptr, nullptr, nullptr, nullptr};
    return A;
}

}  // namespace

template <int D>
void launch_force(cudaStream_t st, const ForceParams& p, bool general, StateBuf<D> b, const uint32_t* cstart,
                  StateBuf<D> a, uint32_t* cell, uint32_t* rank, uint32_t* counts, uint32_t* defer,
                  const uint32_t* refslot, const DebugOut* dbg) {
    if (p.n <= 0) return;
    const ForceArgs<D> A = make_args<D>(p, b, cstart, a, cell, rank, counts, defer, refslot, dbg);
    if (dbg)
        launch_variant<D, true>(st, A, general, 0);
    else
        launch_variant<D, false>(st, A, general, 0);
}

template <int D>
void launch_force_fixup(cudaStream_t st, const ForceParams& p, bool general, StateBuf<D> b, const uint32_t* cstart,
                        StateBuf<D> a, uint32_t* cell, uint32_t* rank, uint32_t* counts, uint32_t* defer,
                        const uint32_t* refslot, const DebugOut* dbg, int blocks) {
    if (p.n <= 0 || general) return;
    const ForceArgs<D> A = make_args<D>(p, b, cstart, a, cell, rank, counts, defer, refslot, dbg);
    if (dbg)
        launch_variant<D, true>(st, A, false, blocks);
    else
        launch_variant<D, false>(st, A, false, blocks);
}

template void launch_force<2>(cudaStream_t, const ForceParams&, bool, StateBuf<2>, const uint32_t*, StateBuf<2>,
                              uint32_t*, uint32_t*, uint32_t*, uint32_t*, const uint32_t*, const DebugOut*);
template void launch_force<3>(cudaStream_t, const ForceParams&, bool, StateBuf<3>, const uint32_t*, StateBuf<3>,
                              uint32_t*, uint32_t*, uint32_t*, uint32_t*, const uint32_t*, const DebugOut*);
template void launch_force_fixup<2>(cudaStream_t, const ForceParams&, bool, StateBuf<2>, const uint32_t*,
                                    StateBuf<2>, uint32_t*, uint32_t*, uint32_t*, uint32_t*, const uint32_t*,
                                    const DebugOut*, int);
template void launch_force_fixup<3>(cudaStream_t, const ForceParams&, bool, StateBuf<3>, const uint32_t*,
                                    StateBuf<3>, uint32_t*, uint32_t*, uint32_t*, uint32_t*, const uint32_t*,
                                    const DebugOut*, int);

// ---- FP32 FMA throughput probe ----

namespace {

__global__ void __launch_bounds__(256) k_ffma_probe(float* out, int iters, float seed) {
    float a0 = seed + threadIdx.x, a1 = a0 + 1.f, a2 = a0 + 2.f, a3 = a0 + 3.f;
    float a4 = a0 + 4.f, a5 = a0 + 5.f, a6 = a0 + 6.f, a7 = a0 + 7.f;
    const float m = 0.999999f, c = 1e-7f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            a0 = fmaf(a0, m, c);
            a1 = fmaf(a1, m, c);
            a2 = fmaf(a2, m, c);
            a3 = fmaf(a3, m, c);
            a4 = fmaf(a4, m, c);
            a5 = fmaf(a5, m, c);
            a6 = fmaf(a6, m, c);
            a7 = fmaf(a7, m, c);
        }
    }
    const float r = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (r == 12345.678f) out[0] = r;  // keeps the chain live
}

}  // namespace

cudaError_t probe_fp32_peak(double* tflops) {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    float* out = nullptr;
    e = cudaMalloc(&out, sizeof(float));
    if (e != cudaSuccess) return e;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int blocks = sms * 8, threads = 256, iters = 4096;
    k_ffma_probe<<<blocks, threads>>>(out, 64, 1.f);  // warm-up
    cudaEventRecord(e0);
    k_ffma_probe<<<blocks, threads>>>(out, iters, 1.f);
    cudaEventRecord(e1);
    e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e == cudaSuccess) {
        const double flops = 2.0 * 8.0 * 16.0 * iters * (double)blocks * threads;
        *tflops = flops / (ms * 1e-3) / 1e12;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    return e;
}

}  // namespace plg
