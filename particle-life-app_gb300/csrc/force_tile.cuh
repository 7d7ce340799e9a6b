// force_tile.cuh — fused velocity + position phase of the Particle Life step:
// the force kernels and their launchers, instantiated per dimension by
// k_force.cu (2D) and k_force3.cu (3D), which compile in parallel.
//
// One thread per particle of the cell-sorted order B.  It replaces
//   Physics.updateVelocity  (backend/Physics.java:397-441),
//   the default Accelerator (app/Main.java:275-280),
//   Physics.updatePosition  (backend/Physics.java:443-450) with
//   Range.wrap / Range.clamp (backend/Range.java:40-96),
// and, in its epilogue, the counting pass of the next makeContainers
// (Physics.java:328-332) on the new position.
//
// Tiling.  A block takes 128 consecutive targets of the sorted order (tile
// variant 0), one thread each; their cells come from the sort.  The cells are
// nondecreasing, so the targets fall into a few "segments" (targets of one
// grid row: one y in 2D, one (y, z) in 3D).  A target in column cx needs the
// window of columns cx-1..cx+1 over its R stencil rows (3 in 2D, 9 in 3D);
// the block stages the sorted union of its targets' windows into shared
// memory column by column, each column's R cells in turn, so that every
// target's neighbourhood is one contiguous run.  When the whole block's
// windows fit, one staging serves every target; otherwise the block's
// columns are staged in chunks (which may span segments), halved until they
// fit, and a single window that still does not fit (a very dense region) is
// read from global memory in the same candidate order (direct_stencil),
// giving the same bits.  The
// candidate loop is branch-free FP32.  A target that meets a candidate
// needing the FP64 decision is deferred: its warp recomputes it from global
// memory at the end (fixup_target).
//
// Pair test.  The reference keeps a pair when d2 != 0 && d2 <= rmax*rmax in
// FP64, with d = wrapConnection(q - p) (Physics.java:428-432).  Here d2 is
// first formed in FP32 from differences that are exact or rounded once: a
// periodic image is taken by cell, as (q - 1) - p or q - (p - 1), where the
// shifted operand lies in [0.5, 1] and the shift is exact.  The FP32 d2 is
// within 5 ulp of the FP64 one, so a pair with d2 <= lo is inside, a pair
// with d2 >= hi is outside, and only pairs in the band (lo, hi) or below
// `tiny` are re-decided with the reference's exact FP64 operation sequence
// (fp64_keeps).  The interacting-pair set is therefore bit-identical to the
// FP64 reference run on the same FP32 positions.  Only the decision is FP64:
// the term of a kept band pair is FP32 like every other term (the force
// vanishes at rmax, so it is tiny); only a pair whose FP32 d2 underflowed
// (d2 < tiny, distinct particles closer than about 1e-15) takes the FP64 term.
//
// Stencil.  The reference scans the 9 (27) cells around floor(x/cs) without
// clamping (Physics.java:404-409).  For a particle in the last partial cell
// [nx*cs, 1) that base is nx, not the binning cell nx-1.  This kernel uses
// the binning cell; the two stencils differ only by column nx-2 (scanned
// here, not there) and column 1 (scanned there, never within rmax).  A pair
// of column nx-2 within rmax lies within 1e-15 relative of rmax^2, so it
// reaches fp64_keeps, which rejects it like the reference.  Grids with fewer
// than 3 cells per axis, where the reference visits a cell more than once,
// take the literal path (general_scan).
#pragma once

#include "force_common.cuh"

namespace plg {

namespace {

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

// ---- literal-path kernel (nx < 3) ----

template <int D, bool DBG, bool SMEM_M>
__global__ void __launch_bounds__(kThreads) k_force_general(const __grid_constant__ ForceArgs<D> A) {
    pdl_wait();  // the sort before it
    const ForceParams& P = A.p;
    extern __shared__ float smat[];
    const float* M = P.matrix;
    const int nt = P.ntypes, ms = SMEM_M ? smem_matrix_stride<D>(nt) : nt;
    if (SMEM_M) {
        for (int k = threadIdx.x; k < nt * nt; k += kThreads)
            smat[D == 3 ? (k / nt) * ms + k % nt : k] = P.matrix[k];
        __syncthreads();
        M = smat;
    }
    const int s = blockIdx.x * kThreads + threadIdx.x;
    const bool valid = s < P.n;
    uint32_t newcell = 0;
    if (valid) {
        const float4 me = A.bpt[s];
        Acc acc = {0.f, 0.f, 0.f, 0, 0ull, 0ull, 0ull};
        general_scan<D, DBG>(A, M + Layout<D>::type(me) * ms, s, me.x, me.y, D == 3 ? me.z : 0.f, acc);
        newcell = integrate<D, DBG>(A, A.p, s, me, A.bvel[s], acc);
    }
    const unsigned mask = __ballot_sync(kFull, valid);
    if (valid) {
        bin_add(A.counts, newcell, mask);
        A.cell[s] = newcell;
    }
}

// ---- tiled kernel (nx >= 3) ----

// Tile variants (the autotuner's choice, PLG_TILE_*):
//   kTargets    targets per block, one thread each
//   kMinBlocks  resident blocks per SM asked for (caps the registers: more
//               blocks with spilled registers measured slower)
//   kCap        staged candidates per staging
//   kCells      stencil cells per staging (R x columns)
// 2D: both variants are 4 blocks of 256 targets per SM at 64 registers
// (32 warps) with 192 stencil cells (64 columns) per staging.  Variant 0
// stages 1536 candidates (28 KB of shared memory) and suits sparse worlds
// such as the 1M-particle one (95 us per launch against 97 for 8 blocks of
// 128 targets with 256 cells); variant 1 stages 3072 (53 KB) for dense
// worlds (tens to hundreds of particles per cell), where variant 0's
// windows overflow.  Few stencil cells keep variant 1 at 4 blocks per SM
// (with 768 cells and 128 targets only 4 blocks of 4 warps fitted: 15%
// slower on the batched worlds).
// 3D: variant 0 (5 blocks of 128 targets at 96 registers) holds 71 staged
// columns of 9 cells, so that the sparse tails of a blob world stage in one
// or two rounds, and 2176 candidates for the dense cores (on the 4M-blob
// world 1.41 ms per launch against 1.49 with 512 cells and 2048 candidates
// and 1.45 with 384 and 2304; shapes whose shared memory leaves 4 blocks
// per SM lose 5-10%); variant 1 is the smaller tile for sparse worlds.
// Variant 2: 2D, 8 blocks of 128 targets with 256 cells and 1024 candidates,
// for small worlds, which the 256-target tiles cut into too few blocks (the
// 10k-particle world: 40 blocks of 256 on 152 SMs); 3D, 4 blocks of 128
// targets with 2816 candidates, for dense worlds.
template <int D, int V>
struct TileCfg;
template <>
struct TileCfg<2, 0> {
    static constexpr int kTargets = 256, kMinBlocks = 4, kCap = 1536, kCells = 192;
};
template <>
struct TileCfg<2, 1> {
    static constexpr int kTargets = 256, kMinBlocks = 4, kCap = 3072, kCells = 192;
};
template <>
struct TileCfg<2, 2> {
    static constexpr int kTargets = 128, kMinBlocks = 8, kCap = 1024, kCells = 256;
};
template <>
struct TileCfg<3, 0> {
    static constexpr int kTargets = 128, kMinBlocks = 5, kCap = 2176, kCells = 640;
};
template <>
struct TileCfg<3, 1> {
    static constexpr int kTargets = 64, kMinBlocks = 10, kCap = 1024, kCells = 384;
};
template <>
struct TileCfg<3, 2> {
    static constexpr int kTargets = 128, kMinBlocks = 4, kCap = 2816, kCells = 640;
};

// Lives in dynamic shared memory (variant 0: about 28 KB in 2D, 42 KB in 3D).
// Staged columns: the sorted union of the windows cx-1..cx+1 of the staged
// targets, as "virtual" columns -1..nx (-1 and nx being the periodic images
// of columns nx-1 and 0), each with the grid row of its segment.
template <int D, int V>
struct TileSmem {
    static constexpr int kCols = TileCfg<D, V>::kCells / TileRows<D>::R;
    float4 cand[TileCfg<D, V>::kCap];      // staged candidates, column-major by stencil cell
    int coff[TileCfg<D, V>::kCells + 1];   // smem start of stencil cell e = column * R + row
    int cglob[TileCfg<D, V>::kCells];      // sorted-order start of stencil cell e
    int cshift[D == 2 ? TileCfg<D, V>::kCells : 1];  // 2D dense staging: image shifts of cell e (kShift*, kNeg*)
    int colv[kCols];                       // virtual column of staged column ci
    int colrow[kCols];                     // grid row (y, or y + z nx) of staged column ci
    int wsum[TileCfg<D, V>::kTargets / 32];
    int wcol[TileCfg<D, V>::kTargets / 32];
    float mat[kSmemMatrixMax * smem_matrix_stride<D>(kSmemMatrixMax)];
};

// Stages the cells of staged columns 0..ncols-1 (sm.colv, sm.colrow),
// column-major: for each column the cells of its R stencil rows in turn, so
// that the neighbourhood of a target whose window starts at column k is the
// single contiguous range of columns k .. k+2.  Images below the box are
// shifted down by 1 here (exact: their coordinates are >= 0.5); images above
// it are flagged for a target shift instead.  Thread t owns cells
// t*per .. t*per+per-1: it reads their extents, the block scans the
// per-thread sums, and the owner copies its cells.  Returns whether the
// candidates fit (every thread gets the same answer); ncols * R <= kCells
// is the caller's.
template <int D, int V>
__device__ __forceinline__ bool stage_columns(const ForceArgs<D>& A, const ForceParams& P,
                                              const uint32_t* __restrict__ cs, TileSmem<D, V>& sm, int ncols) {
    constexpr int R = TileRows<D>::R;
    constexpr int kT = TileCfg<D, V>::kTargets;
    constexpr int kPer = (TileCfg<D, V>::kCells + kT - 1) / kT;
    const int nx = P.g.nx;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int ncell = R * ncols;
    const int per = (ncell + kT - 1) / kT;
    int g0[kPer], len[kPer];
    int sum = 0;
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
        const int e = tid * per + i;
        g0[i] = 0;
        len[i] = 0;
        if (i < per && e < ncell) {
            const int ci = e / R, r = e - ci * R;
            const int col = wrap_index(sm.colv[ci], nx);
            const int row = sm.colrow[ci];
            const int cy = D == 3 ? row % nx : row, cz = D == 3 ? row / nx : 0;
            const int ry = wrap_index(cy + r % 3 - 1, nx);
            const int rz = D == 3 ? wrap_index(cz + r / 3 - 1, nx) : 0;
            const int c = (rz * nx + ry) * nx + col;
            g0[i] = (int)__ldg(cs + c);
            len[i] = (int)__ldg(cs + c + 1) - g0[i];
        }
        sum += len[i];
    }
    int inc = sum;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int t = __shfl_up_sync(kFull, inc, d);
        if (lane >= d) inc += t;
    }
    if (lane == 31) sm.wsum[warp] = inc;
    __syncthreads();
    int before = 0, total = 0;
#pragma unroll
    for (int w = 0; w < kT / 32; ++w) {
        const int x = sm.wsum[w];
        before += w < warp ? x : 0;
        total += x;
    }
    if (total > TileCfg<D, V>::kCap) return false;  // block-uniform
    // 2D windows of kDenseCell or more candidates per cell on average: each
    // cell is copied by one warp (its lanes take every 32nd member), so that
    // a crowded cell does not hold the block at the barrier behind a single
    // thread; the owners only publish their cells' shifts.  Sparse windows:
    // each owner thread copies its cells.  The same slots either way.
    const bool dense = D == 2 && total >= kDenseCell * ncell;  // block-uniform
    int run = before + inc - sum;
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
        const int e = tid * per + i;
        if (i < per && e < ncell) {
            sm.cglob[e] = g0[i];
            sm.coff[e] = run;
            if (e == ncell - 1) sm.coff[ncell] = run + len[i];
            // The cell's image shifts.
            const int ci = e / R, r = e - ci * R;
            float sx = 0.f, sy = 0.f, sz = 0.f;
            int flags = 0;
            if (P.wrap) {
                const int v = sm.colv[ci], row = sm.colrow[ci];
                const int cy = D == 3 ? row % nx : row, cz = D == 3 ? row / nx : 0;
                const int oy = r % 3 - 1, oz = D == 3 ? r / 3 - 1 : 0;
                if (v < 0) sx = 1.f;
                if (v >= nx) flags |= kShiftX;
                if (cy + oy < 0) sy = 1.f;
                if (cy + oy >= nx) flags |= kShiftY;
                if (D == 3) {
                    if (cz + oz < 0) sz = 1.f;
                    if (cz + oz >= nx) flags |= kShiftZ;
                }
            }
            if (D == 2 && dense) {
                sm.cshift[e] = flags | (sx != 0.f ? kNegX : 0) | (sy != 0.f ? kNegY : 0);
            } else {
                const float4* __restrict__ src = A.bpt + g0[i];
                float4* dst = sm.cand + run;
                const int m = len[i];
                int k = 0;
                for (; k + 4 <= m; k += 4) {
                    float4 q[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) q[u] = __ldg(src + k + u);
#pragma unroll
                    for (int u = 0; u < 4; ++u) dst[k + u] = shift_candidate<D>(q[u], sx, sy, sz, flags);
                }
                for (; k < m; ++k) dst[k] = shift_candidate<D>(__ldg(src + k), sx, sy, sz, flags);
            }
        }
        run += len[i];
    }
    if (D == 2 && dense) {
        __syncthreads();
        for (int e = warp; e < ncell; e += kT / 32) {
            const int d = sm.coff[e], m = sm.coff[e + 1] - d, f = sm.cshift[e];
            const float4* __restrict__ src = A.bpt + sm.cglob[e];
            const float sx = (f & kNegX) ? 1.f : 0.f, sy = (f & kNegY) ? 1.f : 0.f;
            for (int k = lane; k < m; k += 32)
                sm.cand[d + k] = shift_candidate<D>(__ldg(src + k), sx, sy, 0.f, f & (kShiftX | kShiftY));
        }
    }
    __syncthreads();
    return true;
}



// Main force kernel (nx >= 3): one thread per target; a block takes
// kTargets (128 in variant 0) consecutive targets and stages their windows
// so that each target reads one contiguous run (or, where a window does not
// fit, reads the same cells from global memory).  Neighbouring threads mostly share a cell, hence a
// window, so their candidate loads are broadcasts.  FP32 only: a target
// whose neighbourhood holds a candidate that needs the FP64 decision is
// deferred to its warp's closing pass (fixup_target), which recomputes it
// completely.
// BATCH: the sorted order holds many worlds one after another (their cells
// are disjoint ranges of one global cell index).  Tiles are laid out per
// world: block b works on tile b - tile_off[k] of the world k that owns it,
// so a block never mixes worlds and every world is cut into exactly the
// tiles a single-world launch uses: each world computes bit for bit what
// plg_step computes for it, whatever else is in the batch.
//
// SNAP (single world, not instrumented): each warp also writes its slots'
// new state to the snapshot arrays A.snap once its deferred targets are done.
template <int D, bool DBG, bool SMEM_M, bool BATCH, int V, bool SNAP = false>
__global__ void __launch_bounds__(TileCfg<D, V>::kTargets, TileCfg<D, V>::kMinBlocks)
    k_force_tile(const __grid_constant__ ForceArgs<D> A) {
    static_assert(!SNAP || (!DBG && !BATCH), "the snapshot form is the plain single-world kernel");
    constexpr int kT = TileCfg<D, V>::kTargets;
    constexpr int R = TileRows<D>::R;
    extern __shared__ __align__(16) unsigned char smraw[];
    TileSmem<D, V>& sm = *reinterpret_cast<TileSmem<D, V>*>(smraw);
    const int tid = threadIdx.x;
    pdl_wait();  // the sort before it: B, slot_cell, cstart, the drained counts
    pdl_release();  // the next step's scan may be scheduled once every block runs
    int wk = 0, s0 = blockIdx.x * kT, nw = A.p.n;
    if (BATCH) {
        const int q = world_of(A.tile_off, A.nworlds, blockIdx.x);
        wk = __ldg(A.tile_off + A.nworlds + 1 + q);
        const int t = blockIdx.x - __ldg(A.tile_off + q);
        s0 = __ldg(A.wp_off + wk) + t * kT;
        nw = __ldg(A.wp_off + wk + 1) - s0;  // targets of this world from s0 on
    } else {
        nw -= s0;
    }
    const int nvalid = min(kT, nw);
    const bool valid = tid < nvalid;
    const int s = s0 + tid;
    const ForceParams& P = BATCH ? A.worlds[wk] : A.p;
    if (BATCH && A.steps_left && __ldg(A.steps_left + wk) <= 0) {
        // A world that has used up its steps is left exactly as its last
        // step left it: A (its state, in that step's order) is not touched,
        // and the cells that step computed for it are counted again for the
        // next sort (the scan consumed the counts).  A world's slots are the
        // same range in A and B, so this tile's slots are its A slots.
        uint32_t c = 0;
        if (valid) c = A.cell[s];
        const unsigned m = __ballot_sync(kFull, valid);
        if (valid) bin_add(A.counts, c, m);
        return;
    }
    // Autotuner: the block's duration in SM cycles, summed per world.
    const long long t_start = BATCH && A.wcycles ? clock64() : 0;
    const int nt = P.ntypes, ms = SMEM_M ? smem_matrix_stride<D>(nt) : nt;
    if (SMEM_M) {
        for (int k = tid; k < nt * nt; k += kT) sm.mat[D == 3 ? (k / nt) * ms + k % nt : k] = P.matrix[k];
    }
    const float* M = SMEM_M ? sm.mat : P.matrix;
    float4 me = make_float4(0.f, 0.f, 0.f, 0.f);
    typename Layout<D>::Vel vme{};
    const int lane = tid & 31, warp = tid >> 5;
    int cx = 0, row = INT_MAX, prow = INT_MAX, pcx = 0;
    if (valid) {
        // The target's cell is the one the sort binned it by (computed from
        // these same coordinates by the previous epilogue or the upload).
        // The first lane of a warp also reads the cell of the target before
        // it (the other lanes take their neighbour's by a shuffle).
        const uint32_t c = __ldg(A.slot_cell + s) - P.cell_base;
        const uint32_t cp = lane == 0 && tid > 0 ? __ldg(A.slot_cell + s - 1) - P.cell_base : 0u;
        me = A.bpt[s];
        vme = A.bvel[s];  // needed only by the epilogue: loaded early, off its critical path
        const uint32_t nxu = (uint32_t)P.g.nx;
        row = (int)(c / nxu);
        cx = (int)(c - (uint32_t)row * nxu);
        prow = (int)(cp / nxu);
        pcx = (int)(cp - (uint32_t)prow * nxu);
    }
    // Segments: maximal runs of targets in one grid row (rows are
    // nondecreasing, and so are the columns within a segment).  Window
    // columns: each first target of a column adds the columns of its window
    // cx-1..cx+1 that the previous column's window has not added (3 at a
    // segment start); a block-wide scan numbers them, so the target's window
    // starts at staged column kwin = incl - 3.
    {
        const int r_up = __shfl_up_sync(kFull, row, 1), c_up = __shfl_up_sync(kFull, cx, 1);
        if (lane > 0) {
            prow = r_up;
            pcx = c_up;
        }
    }
    const int pcol = tid > 0 ? pcx : 0;
    const bool start = valid && (tid == 0 || prow != row);
    const bool lead = valid && (start || pcol != cx);
    const int newc = !lead ? 0 : (start ? 3 : min(3, cx - pcol));
    int incl = newc;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int t = __shfl_up_sync(kFull, incl, d);
        if (lane >= d) incl += t;
    }
    if (lane == 31) sm.wcol[warp] = incl;
    __syncthreads();
    int cbefore = 0, ncol = 0;
#pragma unroll
    for (int w = 0; w < kT / 32; ++w) {
        const int y = sm.wcol[w];
        cbefore += w < warp ? y : 0;
        ncol += y;
    }
    incl += cbefore;
    const int kwin = incl - 3;
    // Staged columns [cb, ce) of the block numbering, as 0 .. ce-cb-1.
    auto fill_columns = [&](int cb, int ce) {
        for (int i = 0; i < newc; ++i) {
            const int ci = incl - newc + i;
            if (ci >= cb && ci < ce) {
                sm.colv[ci - cb] = cx + 2 - newc + i;
                sm.colrow[ci - cb] = row;
            }
        }
    };
    constexpr int kCols = TileSmem<D, V>::kCols;
    // One staging for the whole block when every window fits; otherwise in
    // chunks of columns (below).
    bool whole = ncol <= kCols;  // block-uniform
    if (whole) fill_columns(0, ncol);
    const int nx = P.g.nx;
    const int cy = D == 3 ? (valid ? row % nx : 0) : row, cz = D == 3 ? (valid ? row / nx : 0) : 0;
    const float px = me.x, py = me.y, pz = D == 3 ? me.z : 0.f;
    const float* Mrow = M + (valid ? Layout<D>::type(me) : 0) * ms;
    Acc acc = {0.f, 0.f, 0.f, 0, 0ull, 0ull, 0ull};
    bool defer = false, direct = false;
    // The target's window: staged columns k .. k+2; the target itself splits
    // its run into [j0, self_j) and (self_j, j1).  Only a target in the last
    // column, row or layer of a periodic box meets candidates flagged for a
    // target shift.
    auto evaluate = [&](int k, int ncell) {
        const int j0 = sm.coff[k * R], j1 = sm.coff[(k + 3) * R];
        const int own = (k + 1) * R + R / 2;
        const int self_j = sm.coff[own] + (s - sm.cglob[own]);
        const bool shift = P.wrap && (cx == nx - 1 || cy == nx - 1 || (D == 3 && cz == nx - 1));
        const int* co = sm.coff;
        const int* cg = sm.cglob;
        // 2D: three runs, before the target's own cell, the own cell (the
        // target itself neutralised in place), after it: every lane of a cell
        // walks the same addresses, so the candidate loads are broadcasts
        // (2.7% faster than splitting at the target).  3D: two runs split at
        // the target (the three-run form measured 8% slower).  Same bits.
        const int o0 = co[own], o1 = co[own + 1];
        if (D == 3) {
            if (shift) {
                defer = cand_range<D, DBG, true>(A, P, sm.cand, co, cg, Mrow, ncell, j0, self_j, px, py, pz, acc);
                defer |= cand_range<D, DBG, true>(A, P, sm.cand, co, cg, Mrow, ncell, self_j + 1, j1, px, py, pz,
                                                  acc);
            } else {
                defer = cand_range<D, DBG, false>(A, P, sm.cand, co, cg, Mrow, ncell, j0, self_j, px, py, pz, acc);
                defer |= cand_range<D, DBG, false>(A, P, sm.cand, co, cg, Mrow, ncell, self_j + 1, j1, px, py, pz,
                                                   acc);
            }
        } else if (shift) {
            defer = cand_range<D, DBG, true>(A, P, sm.cand, co, cg, Mrow, ncell, j0, o0, px, py, pz, acc);
            defer |= cand_range<D, DBG, true, true>(A, P, sm.cand, co, cg, Mrow, ncell, o0, o1, px, py, pz, acc,
                                                    self_j);
            defer |= cand_range<D, DBG, true>(A, P, sm.cand, co, cg, Mrow, ncell, o1, j1, px, py, pz, acc);
        } else {
            defer = cand_range<D, DBG, false>(A, P, sm.cand, co, cg, Mrow, ncell, j0, o0, px, py, pz, acc);
            defer |= cand_range<D, DBG, false, true>(A, P, sm.cand, co, cg, Mrow, ncell, o0, o1, px, py, pz, acc,
                                                     self_j);
            defer |= cand_range<D, DBG, false>(A, P, sm.cand, co, cg, Mrow, ncell, o1, j1, px, py, pz, acc);
        }
    };
    __syncthreads();
    const uint32_t* cs = A.cstart + P.cell_base;
    if (whole) {
        whole = stage_columns<D, V>(A, P, cs, sm, ncol);
        if (whole && valid) evaluate(kwin, R * ncol);
    }
    if (!whole) {
        // Chunks of the block's window columns [a, hi), each serving the
        // targets whose window starts in [a, hi - 3].  A chunk may span
        // segments: its columns are staged one by one with their own rows,
        // and a window never leaves its segment.  A chunk whose candidates do
        // not fit is retried with half as many columns (the width grows back
        // after a success), and a single window that does not fit is read
        // from global memory.  (Per-segment chunks served one segment per
        // staging round: sparse 3D blocks spread over many grid rows.)
        int a = 0, width = kCols;
        while (a <= ncol - 3) {
            const int hi = min(a + width, ncol);
            fill_columns(a, hi);  // the previous staging no longer reads the columns
            __syncthreads();
            const bool staged = stage_columns<D, V>(A, P, cs, sm, hi - a);
            const bool mine = valid && kwin >= a && kwin <= hi - 3;
            if (staged) {
                if (mine) evaluate(kwin - a, R * (hi - a));
                a = hi - 2;
                width = min(kCols, 2 * width);
            } else if (hi - a > 3) {
                width = max(3, (hi - a) / 2);
            } else {
                if (mine) direct = true;  // computed after the loop, off the hot path
                a += 1;
            }
        }
    }
    if (direct) {
        // The window did not fit in shared memory: the same sum from global
        // memory.
        defer = direct_stencil<D, DBG>(A, P, cs, Mrow, s, px, py, pz, cx, cy, cz, acc);
    }
    const bool done = valid && !defer;
    uint32_t newcell = 0;
    if (done) newcell = integrate<D, DBG>(A, P, s, me, vme, acc);
    const unsigned mask = __ballot_sync(kFull, done);
    if (done) {
        bin_add(A.counts, newcell, mask);
        A.cell[s] = newcell;
    }
    // Deferred targets (FP64 band pairs): each warp recomputes its own, one
    // at a time, from global memory.  Most warps have none.
    unsigned dm = __ballot_sync(kFull, valid && defer);
    if (dm && lane == 0) atomicAdd(A.defer_count, (uint32_t)__popc(dm));
    while (dm) {
        const int src = __ffs(dm) - 1;
        dm &= dm - 1;
        fixup_target<D, DBG>(A, P, cs, M, __shfl_sync(kFull, s, src), lane);
    }
    if constexpr (SNAP) write_snapshot_warp<D>(A, s0 + 32 * warp, min(32, nvalid - 32 * warp), lane);
    if (BATCH && A.wcycles) {  // block-uniform
        __syncthreads();
        if (tid == 0) atomicAdd(A.wcycles + wk, (unsigned long long)(clock64() - t_start));
    }
}

template <int D, bool DBG, bool BATCH, int V>
void launch_tile(cudaStream_t st, const ForceArgs<D>& A, bool smem_matrix, int batch_tiles) {
    constexpr int kT = TileCfg<D, V>::kTargets;
    const int grid = BATCH ? batch_tiles : (A.n_total + kT - 1) / kT;
    if (grid <= 0) return;
    const size_t sb = sizeof(TileSmem<D, V>);
    if constexpr (!DBG && !BATCH) {
        if (A.snap.any()) {
            if (smem_matrix)
                launch_after(k_force_tile<D, false, true, false, V, true>, dim3(grid), dim3(kT), sb, st, A);
            else
                launch_after(k_force_tile<D, false, false, false, V, true>, dim3(grid), dim3(kT), sb, st, A);
            return;
        }
    }
    if (smem_matrix)
        launch_after(k_force_tile<D, DBG, true, BATCH, V>, dim3(grid), dim3(kT), sb, st, A);
    else
        launch_after(k_force_tile<D, DBG, false, BATCH, V>, dim3(grid), dim3(kT), sb, st, A);
}

template <int D, bool DBG, bool BATCH>
void launch_tile_variant(cudaStream_t st, const ForceArgs<D>& A, bool smem_matrix, int variant, int batch_tiles) {
    if (variant == 1)
        launch_tile<D, DBG, BATCH, 1>(st, A, smem_matrix, batch_tiles);
    else if (variant == 2)
        launch_tile<D, DBG, BATCH, 2>(st, A, smem_matrix, batch_tiles);
    else
        launch_tile<D, DBG, BATCH, 0>(st, A, smem_matrix, batch_tiles);
}

template <int D, bool DBG>
void launch_variant(cudaStream_t st, const ForceArgs<D>& A, bool general, int variant) {
    const int n = A.p.n;
    const bool smem = A.p.ntypes <= kSmemMatrixMax;
    if (general) {
        const int grid = (n + kThreads - 1) / kThreads;
        const size_t sb = smem ? sizeof(float) * A.p.ntypes * smem_matrix_stride<D>(A.p.ntypes) : 0;
        if (smem)
            launch_after(k_force_general<D, DBG, true>, dim3(grid), dim3(kThreads), sb, st, A);
        else
            launch_after(k_force_general<D, DBG, false>, dim3(grid), dim3(kThreads), 0, st, A);
    } else {
        launch_tile_variant<D, DBG, false>(st, A, smem, variant, 0);
    }
}

}  // namespace

template <int D>
void launch_force(cudaStream_t st, const ForceParams& p, bool general, StateBuf<D> b, const uint32_t* cstart,
                  const uint32_t* slot_cell, StateBuf<D> a, uint32_t* cell, uint32_t* counts, uint32_t* defer,
                  const DebugOut* dbg, int variant, const HostSnap* snap) {
    if (p.n <= 0) return;
    ForceArgs<D> A = make_args<D>(p, b, cstart, slot_cell, a, cell, counts, defer, dbg);
    if (snap && !dbg && !general) A.snap = *snap;
    if (dbg)
        launch_variant<D, true>(st, A, general, variant);
    else
        launch_variant<D, false>(st, A, general, variant);
}

template <int D>
void launch_force_batch(cudaStream_t st, const ForceParams* worlds, const int* wp_off, const int* tile_off,
                        const int* steps_left, int tiles, int nworlds, int n_total, bool smem_matrix, StateBuf<D> b,
                        const uint32_t* cstart, const uint32_t* slot_cell, StateBuf<D> a, uint32_t* cell,
                        uint32_t* counts, uint32_t* defer, const DebugOut* dbg, int variant,
                        unsigned long long* wcycles) {
    if (n_total <= 0 || nworlds <= 0 || tiles <= 0) return;
    ForceParams none{};
    ForceArgs<D> A = make_args<D>(none, b, cstart, slot_cell, a, cell, counts, defer, dbg);
    A.worlds = worlds;
    A.wp_off = wp_off;
    A.tile_off = tile_off;
    A.steps_left = steps_left;
    A.wcycles = wcycles;
    A.nworlds = nworlds;
    A.n_total = n_total;
    if (dbg)
        launch_tile_variant<D, true, true>(st, A, smem_matrix, variant, tiles);
    else
        launch_tile_variant<D, false, true>(st, A, smem_matrix, variant, tiles);
}

// Resident blocks per SM of the batched force kernel of one variant (the
// autotuner turns block cycles into SM time with it).
template <int D, int V>
int batch_blocks_per_sm(bool smem_matrix) {
    int nb = 0;
    const cudaError_t e =
        smem_matrix ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_force_tile<D, false, true, true, V>,
                                                                   TileCfg<D, V>::kTargets, sizeof(TileSmem<D, V>))
                    : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_force_tile<D, false, false, true, V>,
                                                                   TileCfg<D, V>::kTargets, sizeof(TileSmem<D, V>));
    if (e != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    return nb > 0 ? nb : 1;
}

namespace {

// Every tiled kernel of one dimension and variant may use its TileSmem.
template <int D, bool DBG, bool SMEM_M, bool BATCH, int V, bool SNAP = false>
cudaError_t allow_one() {
    return cudaFuncSetAttribute(k_force_tile<D, DBG, SMEM_M, BATCH, V, SNAP>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TileSmem<D, V>));
}

template <int D, int V>
cudaError_t allow_tile_smem() {
    const cudaError_t es[] = {allow_one<D, false, true, false, V>(), allow_one<D, false, false, false, V>(),
                              allow_one<D, true, true, false, V>(),  allow_one<D, true, false, false, V>(),
                              allow_one<D, false, true, true, V>(),  allow_one<D, false, false, true, V>(),
                              allow_one<D, true, true, true, V>(),   allow_one<D, true, false, true, V>(),
                              allow_one<D, false, true, false, V, true>(), allow_one<D, false, false, false, V, true>()};
    for (cudaError_t e : es)
        if (e != cudaSuccess) return e;
    return cudaSuccess;
}

}  // namespace

}  // namespace plg
