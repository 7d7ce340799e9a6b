// force_common.cuh — the building blocks of the force kernels (force_tile.cuh):
// kernel arguments, the FP64 pair decision and term, the candidate
// evaluation over a staged window, the global-memory stencils (the direct
// path and the deferred FP64 pass) and the epilogue.  Every path evaluates a
// target's candidates in the same order with the same arithmetic, so they
// give the same bits.
#pragma once

#include <climits>

#include "plg_internal.cuh"

namespace plg {

// Arguments of every force kernel (one struct, passed as a __grid_constant__).
template <int D>
struct ForceArgs {
    ForceParams p;
    const float4* __restrict__ bpt;
    const typename Layout<D>::Vel* __restrict__ bvel;
    const uint32_t* __restrict__ cstart;
    const uint32_t* __restrict__ slot_cell;  // cell of each slot of B (the sort's), with cell_base
    float4* __restrict__ apt;
    typename Layout<D>::Vel* __restrict__ avel;
    uint32_t* __restrict__ cell;
    uint32_t* counts;
    uint32_t* defer_count;  // targets the tiled kernel deferred this step (statistics)
    DebugOut dbg;
    HostSnap snap;  // snapshot arrays written by the tiled kernel's SNAP form
    // Batched worlds: per-world parameters, first sorted slots
    // (wp_off[k] = worlds[k].p_off, nworlds + 1 entries) and the launch's
    // tile layout: tile_off[q] (q = 0 .. nworlds) is the first tile of the
    // q-th world in launch order and tile_off[nworlds + 1 + q] that world's
    // index (worlds with no tiles in this launch take none).
    const ForceParams* __restrict__ worlds;
    const int* __restrict__ wp_off;
    const int* __restrict__ tile_off;
    const int* __restrict__ steps_left;  // per world; <= 0: frozen this step (may be null)
    unsigned long long* wcycles;         // per world: SM cycles of its blocks (autotuner; may be null)
    int nworlds;
    int n_total;
};

namespace {

constexpr int kThreads = 256;        // literal-path and fixup kernels
constexpr int kSmemMatrixMax = 16;   // matrix in shared memory up to 16 x 16

// Row stride of the matrix in shared memory.  3D: odd, so that the lanes of
// a warp reading one column from different rows (targets of different types
// against one candidate) hit distinct banks (16 types with stride 16 put a
// column in two banks: 3D blobs ran 3% slower).  2D: the plain stride (at
// most 2-way conflicts for 8 types; the padded form measured 1% slower).
template <int D>
__host__ __device__ constexpr int smem_matrix_stride(int ntypes) {
    return D == 3 ? (ntypes | 1) : ntypes;
}



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

// The reference's FP64 pair test on the raw FP32 positions (upcast):
// d = wrapConnection(q - p), keep when d2 != 0 && d2 <= rmax^2
// (Physics.java:428-432), in the reference's operation order.  `slmask` bit
// k: the target lies in the last partial cell of axis k and nx >= 4, so
// candidates of cell nx-2 on that axis are outside the reference's stencil.
// Writes the FP64 difference vector.
template <int D>
__device__ __forceinline__ bool fp64_keeps(const ForceParams& P, float px, float py, float pz, float4 q, int slmask,
                                           double& dx, double& dy, double& dz) {
    dx = __dsub_rn((double)q.x, (double)px);
    dy = __dsub_rn((double)q.y, (double)py);
    dz = D == 3 ? __dsub_rn((double)q.z, (double)pz) : 0.0;
    if (P.wrap) {
        dx = wrap_connection(dx);
        dy = wrap_connection(dy);
        if (D == 3) dz = wrap_connection(dz);
    }
    // lengthSquared: x*x + (y*y + z*z), unfused.
    const double d2 = __dadd_rn(__dmul_rn(dx, dx), __dadd_rn(__dmul_rn(dy, dy), __dmul_rn(dz, dz)));
    if (!(d2 != 0.0 && d2 <= P.rmax2)) return false;
    if (slmask) {
        const int m2 = P.g.nx - 2;
        if ((slmask & 1) && axis_cell(q.x, P.g) == m2) return false;
        if ((slmask & 2) && axis_cell(q.y, P.g) == m2) return false;
        if (D == 3 && (slmask & 4) && axis_cell(q.z, P.g) == m2) return false;
    }
    return true;
}

// The reference's Accelerator term in FP64 for a kept pair:
// relativePosition.div(rmax); accelerate(a, pos) (app/Main.java:275-280).
__device__ __noinline__ float4 fp64_term(const ForceParams& P, double dx, double dy, double dz, float a) {
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

// FP64 decision and FP64 term (the literal path for nx < 3): returns
// (term, 1) when the pair interacts, w = 0 when not.
template <int D>
__device__ __noinline__ float4 rare_pair(const ForceParams& P, float px, float py, float pz, float4 q, float a,
                                         int slmask) {
    double dx, dy, dz;
    if (!fp64_keeps<D>(P, px, py, pz, q, slmask, dx, dy, dz)) return make_float4(0.f, 0.f, 0.f, 0.f);
    return fp64_term(P, dx, dy, dz, a);
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

// ---- global-memory stencil of one target, one warp (fixup of the tiled kernel) ----

// nx >= 3: each row (and layer) of the stencil is at most two runs of the
// sorted order: cells cx-1..cx+1, split in two where the row wraps in x.
// Lane k < 2R (R = 3 rows in 2D, 9 in 3D) describes run k (row k/2, part
// k%2): its first slot, length and periodic shifts; a warp scan gives run
// offsets, and the warp walks the concatenated runs 32 candidates at a time,
// each lane finding its run by a binary search over the offsets.  All
// descriptor loads of a target are issued at once.
//   target side   (pxe, pye, pze): target position, minus 1 on an axis where
//                 the run is the periodic image above the box
//   candidate     (qox, qoy, qoz): -1 on an axis where the run's own
//                 coordinates are shifted down (image below the box)
template <int D, bool DBG>
__device__ __noinline__ Acc warp_stencil(const ForceArgs<D>& A, const ForceParams& P, const uint32_t* cs,
                                         const float* Mrow, int s, float px, float py, float pz, int slmask,
                                         int lane) {
    constexpr int R = D == 3 ? 9 : 3;
    const int nx = P.g.nx;
    const int cx = axis_cell(px, P.g), cy = axis_cell(py, P.g), cz = D == 3 ? axis_cell(pz, P.g) : 0;
    int j0 = 0, len = 0;
    float pxe = px, pye = py, pze = pz, qox = 0.f, qoy = 0.f, qoz = 0.f;
    if (lane < 2 * R) {
        const int row = lane >> 1, part = lane & 1;
        int ry = cy + row % 3 - 1, rz = D == 3 ? cz + row / 3 - 1 : 0;
        if (ry < 0) {
            ry += nx;
            if (P.wrap) qoy = -1.f;
        } else if (ry >= nx) {
            ry -= nx;
            if (P.wrap) pye = py - 1.f;
        }
        if (D == 3) {
            if (rz < 0) {
                rz += nx;
                if (P.wrap) qoz = -1.f;
            } else if (rz >= nx) {
                rz -= nx;
                if (P.wrap) pze = pz - 1.f;
            }
        }
        const int base = (rz * nx + ry) * nx;
        int ca = 0, cb = 0;  // cells [ca, cb) of this row
        if (cx >= 1 && cx <= nx - 2) {
            if (part == 0) ca = cx - 1, cb = cx + 2;
        } else if (cx == 0) {
            if (part == 0) {
                ca = nx - 1, cb = nx;
                if (P.wrap) qox = -1.f;
            } else {
                ca = 0, cb = 2;
            }
        } else {
            if (part == 0) {
                ca = nx - 2, cb = nx;
            } else {
                ca = 0, cb = 1;
                if (P.wrap) pxe = px - 1.f;
            }
        }
        if (cb > ca) {
            j0 = (int)__ldg(cs + base + ca);
            len = (int)__ldg(cs + base + cb) - j0;
        }
    }
    int inc = len;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int t = __shfl_up_sync(kFull, inc, d);
        if (lane >= d) inc += t;
    }
    const int off = inc - len;
    const int total = __shfl_sync(kFull, inc, 31);
    Acc acc = {0.f, 0.f, 0.f, 0, 0ull, 0ull, 0ull};
    for (int k0 = 0; k0 < total; k0 += 32) {
        const int k = k0 + lane;
        int r = 0;  // last run with off <= k (lanes >= 2R have off = total)
#pragma unroll
        for (int step = 16; step > 0; step >>= 1) {
            const int o = __shfl_sync(kFull, off, r + step);
            if (o <= k) r += step;
        }
        const int rj0 = __shfl_sync(kFull, j0, r), roff = __shfl_sync(kFull, off, r);
        const float tx = __shfl_sync(kFull, pxe, r), ty = __shfl_sync(kFull, pye, r);
        const float sx = __shfl_sync(kFull, qox, r), sy = __shfl_sync(kFull, qoy, r);
        float tz = 0.f, sz = 0.f;
        if (D == 3) {
            tz = __shfl_sync(kFull, pze, r);
            sz = __shfl_sync(kFull, qoz, r);
        }
        if (k >= total) continue;
        const int j = rj0 + (k - roff);
        if (j == s) continue;
        const float4 q = __ldg(A.bpt + j);
        const float dx = (q.x + sx) - tx;
        const float dy = (q.y + sy) - ty;
        float d2;
        float dz = 0.f;
        if (D == 3) {
            dz = (q.z + sz) - tz;
            d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        } else {
            d2 = fmaf(dx, dx, dy * dy);
        }
        if (DBG) acc.cand++;
        // FP32 decides where it can; the band (lo, hi) and d2 < tiny are
        // decided in FP64.  A kept pair's term is FP32 unless its FP32 d2
        // lost the difference (d2 < tiny), where only FP64 resolves it.
        bool keep = d2 <= P.lo && d2 >= P.tiny;
        bool f64 = false;
        double ddx = 0.0, ddy = 0.0, ddz = 0.0;
        // Coincident particles: an FP32 difference is zero exactly when the
        // FP64 one is (both are exact or rounded once from a multiple of
        // 2^-149), so the reference's d2 != 0 rejects the pair without FP64.
        const bool same = dx == 0.f && dy == 0.f && (D == 2 || dz == 0.f);
        if (!keep && d2 < P.hi && !same) {
            keep = fp64_keeps<D>(P, px, py, pz, q, slmask, ddx, ddy, ddz);
            f64 = d2 < P.tiny;
        }
        if (keep) {
            const float a = Mrow[Layout<D>::type(q)];
            if (f64) {
                add_pair<D, DBG>(acc, fp64_term(P, ddx, ddy, ddz, a), DBG ? id_of<D>(A, j) : 0ull);
            } else {
                fast_pair(P, a, dx, dy, dz, d2, acc);
                if (DBG) add_pair<D, true>(acc, make_float4(0.f, 0.f, 0.f, 0.f), id_of<D>(A, j));
            }
        }
    }
    return acc;
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

// Epilogue of one target (sorted slot s, velocity v): v = v ff + acc (rmax force dt),
// x = v dt + x, ensurePosition; the next state goes to A[s].  Returns the
// new cell.
template <int D, bool DBG>
__device__ __forceinline__ uint32_t integrate(const ForceArgs<D>& A, const ForceParams& P, int s, const float4& me,
                                              const typename Layout<D>::Vel& v, const Acc& acc) {
    const float vx = fmaf(acc.x, P.scale, v.x * P.ff);
    const float vy = fmaf(acc.y, P.scale, v.y * P.ff);
    const float nxp = ensure_position(__fadd_rn(__fmul_rn(vx, P.dt), me.x), P.wrap);
    const float nyp = ensure_position(__fadd_rn(__fmul_rn(vy, P.dt), me.y), P.wrap);
    float nzp = 0.f;
    if constexpr (D == 2) {
        A.apt[s] = make_float4(nxp, nyp, me.z, me.w);
        A.avel[s] = make_float2(vx, vy);
    } else {
        const float vz = fmaf(acc.z, P.scale, v.z * P.ff);
        nzp = ensure_position(__fadd_rn(__fmul_rn(vz, P.dt), me.z), P.wrap);
        A.apt[s] = make_float4(nxp, nyp, nzp, me.w);
        A.avel[s] = make_float4(vx, vy, vz, v.w);
    }
    if (DBG) {
        if (A.dbg.pairs) A.dbg.pairs[s] = acc.pairs;
        if (A.dbg.hsum) A.dbg.hsum[s] = acc.hs;
        if (A.dbg.hxor) A.dbg.hxor[s] = acc.hx;
        if (A.dbg.acc) {
            A.dbg.acc[(size_t)D * s + 0] = acc.x;
            A.dbg.acc[(size_t)D * s + 1] = acc.y;
            if (D == 3) A.dbg.acc[(size_t)D * s + 2] = acc.z;
        }
        if (A.dbg.candidates) atomicAdd(A.dbg.candidates, acc.cand);
    }
    return P.cell_base + cell_index<D>(nxp, nyp, nzp, P.g);
}

template <int D>
__device__ __forceinline__ int sliver_mask(const ForceParams& P, float px, float py, float pz) {
    if (!P.slmask_ok) return 0;
    return (px >= P.g.b_nx ? 1 : 0) | (py >= P.g.b_nx ? 2 : 0) | (D == 3 && pz >= P.g.b_nx ? 4 : 0);
}

template <int D>
struct TileRows {
    static constexpr int R = D == 3 ? 9 : 3;
};

// Target shifts a staged candidate asks for (bits 16..18 of its type word):
// the target uses x - 1 (y - 1, z - 1) against it, because the candidate is
// the periodic image above the box of a cell near coordinate 0.
constexpr int kShiftX = 1 << 16, kShiftY = 1 << 17, kShiftZ = 1 << 18;
// Staging only (never in a staged word): the cell's image lies below the box
// in x or y and its candidates are shifted down by 1 as they are copied.
constexpr int kNegX = 1 << 20, kNegY = 1 << 21;
// Average staged candidates per cell from which a 2D block copies its cells
// one warp per cell instead of one owner thread per cell.
constexpr int kDenseCell = 16;

__device__ __forceinline__ int wrap_index(int c, int n) { return c < 0 ? c + n : (c >= n ? c - n : c); }

// A staged candidate: coordinates of an image below the box moved down by
// one, target-shift flags (images above the box) in the type word.
template <int D>
__device__ __forceinline__ float4 shift_candidate(float4 q, float sx, float sy, float sz, int flags) {
    q.x -= sx;
    q.y -= sy;
    if (D == 3) q.z -= sz;
    if constexpr (D == 2)
        q.z = __int_as_float(__float_as_int(q.z) | flags);
    else
        q.w = __int_as_float(__float_as_int(q.w) | flags);
    return q;
}

// rsqrt.approx.ftz.f32: a zero or subnormal d2 gives +inf.
__device__ __forceinline__ float rsqrt_approx(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// x * y with subnormal inputs and results flushed to zero.
__device__ __forceinline__ float mul_ftz(float x, float y) {
    float r;
    asm("mul.ftz.f32 %0, %1, %2;" : "=f"(r) : "f"(x), "f"(y));
    return r;
}

// min(m, x) that returns NaN when either is NaN (a running minimum that
// remembers a NaN once it has seen one).
__device__ __forceinline__ float min_nan(float m, float x) {
    float r;
    asm("min.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(m), "f"(x));
    return r;
}

// (qx - px, qy - py) as one packed FP32 subtraction (two lanes of one
// instruction, each rounded like a scalar subtraction).
__device__ __forceinline__ void sub_pair(float qx, float qy, float px, float py, float& dx, float& dy) {
    unsigned long long q, p, d;
    asm("mov.b64 %0, {%1, %2};" : "=l"(q) : "f"(qx), "f"(qy));
    asm("mov.b64 %0, {%1, %2};" : "=l"(p) : "f"(px), "f"(py));
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(q), "l"(p));
    asm("mov.b64 {%0, %1}, %2;" : "=f"(dx), "=f"(dy) : "l"(d));
}

// Loop constants of the candidate evaluation, read once into registers
// (otherwise the compiler re-reads them from the parameter bank per
// candidate).  lo: the FP32 d2 at or below which a pair certainly interacts
// (the debug counts use it); uflag: the threshold of the |u| test below.
//
// A target whose running minimum of |u| ends below uflag, or is NaN, is
// recomputed with the FP64 decisions.  Why that covers every pair the FP32
// d2 cannot decide: with s = |d|/rmax, u = 1 - |1 + beta - 2 s| / (1 - beta)
// is the Accelerator's triangle factor (app/Main.java:275-280), zero at
// s = beta and at s = 1.  A pair in the FP32 decision band lo < d2 < hi (d2
// within 2^-19 relative of rmax^2, kBandRel) has |s - 1| <= 2^-20 + 2^-24,
// so its exact u has |u| <= 2.02e-6 / (1 - beta).  The FP32 u differs from
// it by less than 0.87e-6 / (1 - beta): rsqrt.approx (relative error below
// 2^-22) and the product give dist within 3e-7 relative, the fma for
// t = 1 + beta - 2 dist / rmax adds its rounding and those of -2/rmax and
// 1 + beta (|t| error < 8.3e-7 near s = 1), and the last fma scales it by
// 1/(1 - beta).  So every band pair has |u| < 2.9e-6 / (1 - beta), and
// uflag = 7e-6 / (1 - beta) keeps a factor 2.4 of margin.  A pair whose FP32
// d2 is zero or subnormal (coincident or nearly coincident particles; the
// reference keeps a pair whenever its FP64 d2 != 0) gives
// dist = 0 * inf = NaN, which reaches the running minimum.  Every other pair
// is decided correctly in FP32: d2 <= lo interacts, d2 >= hi does not and
// has u < 0, hence an exact zero term.  A pair near s = beta may raise the
// flag too; that costs a recomputation, never a wrong result.
struct LoopK {
    float lo, m2, opb, iomb, k1, uflag;
    __device__ __forceinline__ explicit LoopK(const ForceParams& P)
        : lo(P.lo), m2(P.m2_inv_rmax), opb(P.one_plus_beta), iomb(P.inv_one_minus_beta), k1(P.k1),
          uflag(7e-6f * P.inv_one_minus_beta) {}
};

// One candidate: d = q - p with the image shifts already applied to q and p,
// the FP32 Accelerator term added to acc, and umin = min(umin, |u|) (NaN
// sticks).  The staged and the direct paths both use it, in the same
// candidate order, so they produce the same bits.  Returns d2.
//
// Force law in FP32, with inv = 1/|d| (rsqrt.approx) and u+ = max(u, 0):
//   below beta rmax   f/|d| = 1/(beta rmax) - 1/|d|   (u+ = 0 there)
//   beta rmax..rmax   f/|d| = a u+ / |d|
// both as g = fma(a u+ - 1, inv, min(k1, inv)), k1 = 1/(beta rmax):
// below beta rmax inv > k1 and a u+ - 1 = -1, giving k1 - inv; above it
// min(k1, inv) = inv, giving (a u+ - 1) inv + inv; beyond rmax (u+ = 0) that
// is fma(-1, inv, inv) = +0 exactly, so a candidate beyond rmax adds an exact
// zero and needs no select.
template <int D>
struct Term {
    float dx, dy, dz, g, d2;
};

// The term of one candidate (not yet added) and umin = min(umin, |u|).
template <int D>
__device__ __forceinline__ Term<D> cand_term(const LoopK& K, float qx, float qy, float qz, float pxe, float pye,
                                             float pze, float a, float& umin) {
    Term<D> r;
    sub_pair(qx, qy, pxe, pye, r.dx, r.dy);
    r.dz = 0.f;
    if (D == 3) {
        r.dz = qz - pze;
        r.d2 = fmaf(r.dx, r.dx, fmaf(r.dy, r.dy, r.dz * r.dz));
    } else {
        r.d2 = fmaf(r.dx, r.dx, r.dy * r.dy);
    }
    const float inv = rsqrt_approx(r.d2);
    const float dist = mul_ftz(r.d2, inv);
    const float t = fmaf(dist, K.m2, K.opb);
    const float u = fmaf(-fabsf(t), K.iomb, 1.f);
    umin = min_nan(umin, fabsf(u));
    const float h = fmaf(a, fmaxf(u, 0.f), -1.f);
    r.g = fmaf(h, inv, fminf(K.k1, inv));
    return r;
}

template <int D>
__device__ __forceinline__ void add_term(Acc& acc, const Term<D>& t) {
    acc.x = fmaf(t.dx, t.g, acc.x);
    acc.y = fmaf(t.dy, t.g, acc.y);
    if (D == 3) acc.z = fmaf(t.dz, t.g, acc.z);
}

template <int D>
__device__ __forceinline__ float eval_candidate(const LoopK& K, float qx, float qy, float qz, float pxe, float pye,
                                                float pze, float a, Acc& acc, float& umin) {
    const Term<D> t = cand_term<D>(K, qx, qy, qz, pxe, pye, pze, a, umin);
    add_term<D>(acc, t);
    return t.d2;
}

// True when the running minimum of |u| asks for the FP64 recomputation.
__device__ __forceinline__ bool needs_fp64(const LoopK& K, float umin) { return !(umin >= K.uflag); }

// Global sorted slot of staged candidate j (rare path and debug only).
__device__ __forceinline__ int staged_global(const int* coff, const int* cglob, int ncell, int j) {
    int lo = 0, hi = ncell;
    while (hi - lo > 1) {
        const int m = (lo + hi) >> 1;
        if (coff[m] <= j)
            lo = m;
        else
            hi = m;
    }
    return cglob[lo] + (j - coff[lo]);
}

// Staged candidates [ja, jb) of the target (a part of its neighbourhood
// without the target itself), from a column-major staging (cand, with cell
// offsets coff and global starts cglob of ncell cells).  Branch-free FP32:
// every lane evaluates the Accelerator for every candidate, and a pair
// beyond rmax adds an exact zero (eval_candidate).  A candidate that needs
// the FP64 decision (the |u| test of LoopK: the decision band around rmax,
// coincident particles) makes the function return true: the caller then
// defers the target to the FP64 fixup, which discards this partial sum.
// SHIFT: some candidates carry target-shift flags.
// SELF: the range holds the target itself at self_j; its copy is moved 8
// units away (an exact zero term, far from both zeros of u), which sums to
// the same bits as leaving it out, without a branch.
template <int D, bool DBG, bool SHIFT, bool SELF = false>
__device__ __forceinline__ bool cand_range(const ForceArgs<D>& A, const ForceParams& P, const float4* cand,
                                           const int* coff, const int* cglob, const float* __restrict__ Mrow,
                                           int ncell, int ja, int jb, float px, float py, float pz, Acc& acc,
                                           int self_j = -1) {
    const float px1 = px - 1.f, py1 = py - 1.f, pz1 = pz - 1.f;
    float umin = INFINITY;
    const LoopK K(P);
    // The term of candidate j, with the staged shifts applied.
    auto term = [&](int j) {
        float4 q = cand[j];
        if (SELF && j == self_j) q.x += 8.f;
        int tb = __float_as_int(D == 3 ? q.w : q.z);
        float pxe = px, pye = py, pze = pz;
        if (SHIFT) {
            pxe = (tb & kShiftX) ? px1 : px;
            pye = (tb & kShiftY) ? py1 : py;
            if (D == 3) pze = (tb & kShiftZ) ? pz1 : pz;
            tb &= 0xffff;
        }
        return cand_term<D>(K, q.x, q.y, q.z, pxe, pye, pze, Mrow[tb], umin);
    };
    auto count = [&](int j, float d2) {
        if (DBG && !(SELF && j == self_j)) {
            acc.cand++;
            if ((d2 <= K.lo) & (d2 > 0.f))
                add_pair<D, true>(acc, make_float4(0.f, 0.f, 0.f, 0.f),
                                  id_of<D>(A, staged_global(coff, cglob, ncell, j)));
        }
    };
    // Two candidates per iteration: their terms are independent chains
    // (shared-memory load, rsqrt, force law) that overlap in one warp; they
    // are added in candidate order, so the sum has the same bits as one
    // candidate at a time.
    constexpr int U = D == 3 ? 4 : 2;
    int j = ja;
    for (; j + U <= jb; j += U) {
        Term<D> t[U];
#pragma unroll
        for (int k = 0; k < U; ++k) t[k] = term(j + k);
#pragma unroll
        for (int k = 0; k < U; ++k) add_term<D>(acc, t[k]);
#pragma unroll
        for (int k = 0; k < U; ++k) count(j + k, t[k].d2);
    }
    for (; j < jb; ++j) {
        const Term<D> t0 = term(j);
        add_term<D>(acc, t0);
        count(j, t0.d2);
    }
    return needs_fp64(K, umin);
}

// The target's neighbourhood read straight from global memory, for segments
// too wide or too full for shared memory: the cells in the staged order
// (columns cx-1..cx+1, and in each the R stencil rows), the same image
// shifts (below the box: the candidate's coordinate minus 1; above: the
// target's) and the same candidate evaluation, so the sum has the same bits
// as the staged path would give.
template <int D, bool DBG>
__device__ __noinline__ bool direct_stencil(const ForceArgs<D>& A, const ForceParams& P,
                                            const uint32_t* __restrict__ cs, const float* __restrict__ Mrow, int s,
                                            float px, float py, float pz, int cx, int cy, int cz, Acc& acc) {
    constexpr int R = D == 3 ? 9 : 3;
    const LoopK K(P);
    const int nx = P.g.nx;
    const bool wrap = P.wrap != 0;
    float umin = INFINITY;
    for (int ci = 0; ci < 3; ++ci) {
        int col = cx - 1 + ci;
        bool qsx = false, tsx = false;
        if (col < 0) {
            col += nx;
            qsx = wrap;
        } else if (col >= nx) {
            col -= nx;
            tsx = wrap;
        }
        const float pxe = tsx ? px - 1.f : px;
        for (int r = 0; r < R; ++r) {
            int ry = cy + r % 3 - 1, rz = D == 3 ? cz + r / 3 - 1 : 0;
            bool qsy = false, qsz = false;
            float pye = py, pze = pz;
            if (ry < 0) {
                ry += nx;
                qsy = wrap;
            } else if (ry >= nx) {
                ry -= nx;
                if (wrap) pye = py - 1.f;
            }
            if (D == 3) {
                if (rz < 0) {
                    rz += nx;
                    qsz = wrap;
                } else if (rz >= nx) {
                    rz -= nx;
                    if (wrap) pze = pz - 1.f;
                }
            }
            const int c = (rz * nx + ry) * nx + col;
            const int j0 = (int)__ldg(cs + c), j1 = (int)__ldg(cs + c + 1);
            for (int j = j0; j < j1; ++j) {
                if (j == s) continue;
                float4 q = __ldg(A.bpt + j);
                if (qsx) q.x -= 1.f;
                if (qsy) q.y -= 1.f;
                if (D == 3 && qsz) q.z -= 1.f;
                const float d2 = eval_candidate<D>(K, q.x, q.y, q.z, pxe, pye, pze, Mrow[Layout<D>::type(q)], acc,
                                                   umin);
                if (DBG) {
                    acc.cand++;
                    if ((d2 <= K.lo) & (d2 > 0.f))
                        add_pair<D, true>(acc, make_float4(0.f, 0.f, 0.f, 0.f), id_of<D>(A, j));
                }
            }
        }
    }
    return needs_fp64(K, umin);
}

// Sum of `v` over the warp in a fixed butterfly order (the same bits on
// every run); every lane receives the total.
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(kFull, v, d);
    return v;
}

// One deferred target, one warp: the lanes split the candidates of the
// global-memory stencil (with the FP64 decisions), their partial sums are
// combined by warp_sum, and lane 0 runs the epilogue and the counting step.
// M: the matrix in global memory (P.matrix) or its shared-memory copy.
template <int D, bool DBG>
__device__ __noinline__ void fixup_target(const ForceArgs<D>& A, const ForceParams& P, const uint32_t* cs,
                                          const float* M, int s, int lane) {
    const int mstride = M == P.matrix ? P.ntypes : smem_matrix_stride<D>(P.ntypes);
    const float4 me = A.bpt[s];
    const float px = me.x, py = me.y, pz = D == 3 ? me.z : 0.f;
    Acc acc = warp_stencil<D, DBG>(A, P, cs, M + Layout<D>::type(me) * mstride, s, px, py, pz,
                                   sliver_mask<D>(P, px, py, pz), lane);
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
        const uint32_t newcell = integrate<D, DBG>(A, P, s, me, A.bvel[s], acc);
        atomicAdd(A.counts + newcell, 1u);
        A.cell[s] = newcell;
    }
}

// The snapshot of one warp's slots w0 .. w0+m-1 (m <= 32; the whole warp
// calls): the values this warp's epilogue and fixups stored in A, read back
// and written in the plg_download layout.  pos and vel are 3 doubles per
// particle, so the warp's 32 particles are 96 consecutive doubles of each;
// lane l writes doubles l, l+32 and l+64 (particle j/3, component j%3,
// fetched from its lane by shuffles), so every store instruction covers
// 256 contiguous bytes.
template <int D>
__device__ __forceinline__ void write_snapshot_warp(const ForceArgs<D>& A, int w0, int m, int lane) {
    if (m <= 0) return;  // warp-uniform
    __syncwarp();        // the lanes' stores to A (epilogue, fixups) are visible to the warp
    float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
    typename Layout<D>::Vel v{};
    const bool mine = lane < m;
    if (mine) {
        p = A.apt[w0 + lane];
        v = A.avel[w0 + lane];
    }
    const float c0 = p.x, c1 = p.y, c2 = D == 3 ? p.z : 0.f;
    float u2 = 0.f;
    if constexpr (D == 3) u2 = v.z;
    const float u0 = v.x, u1 = v.y;
    double* pos = A.snap.pos ? A.snap.pos + 3 * (size_t)w0 : nullptr;
    double* vel = A.snap.vel ? A.snap.vel + 3 * (size_t)w0 : nullptr;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const int j = 32 * r + lane;
        const int q = j / 3, k = j - 3 * q;
        const float a0 = __shfl_sync(kFull, c0, q), a1 = __shfl_sync(kFull, c1, q), a2 = __shfl_sync(kFull, c2, q);
        const float b0 = __shfl_sync(kFull, u0, q), b1 = __shfl_sync(kFull, u1, q), b2 = __shfl_sync(kFull, u2, q);
        if (q < m) {
            if (pos) pos[j] = (double)(k == 0 ? a0 : (k == 1 ? a1 : a2));
            if (vel) vel[j] = (double)(k == 0 ? b0 : (k == 1 ? b1 : b2));
        }
    }
    if (mine) {
        if (A.snap.type) A.snap.type[w0 + lane] = Layout<D>::type(p);
        if (A.snap.id) A.snap.id[w0 + lane] = Layout<D>::id(p, v);
    }
}

template <int D>
ForceArgs<D> make_args(const ForceParams& p, StateBuf<D> b, const uint32_t* cstart, const uint32_t* slot_cell,
                       StateBuf<D> a, uint32_t* cell, uint32_t* counts, uint32_t* defer, const DebugOut* dbg) {
    ForceArgs<D> A;
    A.p = p;
    A.bpt = b.pt;
    A.bvel = b.vel;
    A.cstart = cstart;
    A.slot_cell = slot_cell;
    A.apt = a.pt;
    A.avel = a.vel;
    A.cell = cell;
    A.counts = counts;
    A.defer_count = defer;
    A.dbg = dbg ? *dbg : DebugOut{nullptr, nullptr, nullptr, nullptr, nullptr};
    A.snap = HostSnap{nullptr, nullptr, nullptr, nullptr};
    A.worlds = nullptr;
    A.wp_off = nullptr;
    A.tile_off = nullptr;
    A.steps_left = nullptr;
    A.wcycles = nullptr;
    A.nworlds = 1;
    A.n_total = p.n;
    return A;
}

}  // namespace

}  // namespace plg
