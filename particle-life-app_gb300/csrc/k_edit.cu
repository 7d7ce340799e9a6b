// k_edit.cu — device-side versions of the app's particle mutators, so that a
// host edit does not need a full download / re-upload of the world:
//   cursor selection   app/cursors/Cursor.java:16-35 (isInside, countSelection)
//   cursor MOVE        app/Main.java:540-551: selected p += delta, ensurePosition
//   cursor DELETE      app/Main.java:567-578: keep the unselected in order
//   permute            shuffle / truncate of Physics.setParticleCount
//                      (Physics.java:190-223) and ExtendedPhysics.setTypeCount
//   set types          new types for every particle (ensureTypes, setTypes)
// The selection test runs in FP64 on the upcast FP32 positions, in the
// reference's operation order.
#include "plg_internal.cuh"

namespace plg {

namespace {

constexpr int kThreads = 256;

inline int blocks_for(int n) { return (n + kThreads - 1) / kThreads; }

// Cursor.isInside (Cursor.java:16-35): delta = p - cursor, wrapped
// componentwise as val - floor(val + 0.5) in a periodic box, divided by the
// cursor size, then the shape's test (CircleCursorShape.java:39-41: length
// <= 0.5; SquareCursorShape.java:37-40: |x| <= 0.5 and |y| <= 0.5;
// InfinityCursorShape.java:11-14: everywhere).  A zero size selects nothing.
__device__ __forceinline__ bool cursor_inside(const CursorDev& cu, double x, double y, double z) {
    if (cu.size == 0.0) return false;
    double d[3] = {__dsub_rn(x, cu.x), __dsub_rn(y, cu.y), __dsub_rn(z, cu.z)};
    if (cu.wrap) {
#pragma unroll
        for (int k = 0; k < 3; ++k) d[k] = __dsub_rn(d[k], floor(__dadd_rn(d[k], 0.5)));
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) d[k] = __ddiv_rn(d[k], cu.size);
    if (cu.shape == kCursorCircle) {
        const double l2 = __dadd_rn(__dmul_rn(d[0], d[0]), __dadd_rn(__dmul_rn(d[1], d[1]), __dmul_rn(d[2], d[2])));
        return __dsqrt_rn(l2) <= 0.5;
    }
    if (cu.shape == kCursorSquare) return fabs(d[0]) <= 0.5 && fabs(d[1]) <= 0.5;
    return true;  // infinity
}

template <int D>
__global__ void __launch_bounds__(kThreads) k_cursor_mark(int n, const float4* __restrict__ pt, CursorDev cu,
                                                          uint32_t* __restrict__ flag, unsigned long long* count) {
    const int i = blockIdx.x * kThreads + threadIdx.x;
    bool in = false;
    if (i < n) {
        const float4 p = pt[i];
        in = cursor_inside(cu, p.x, p.y, D == 3 ? p.z : 0.0);
        flag[i] = in ? 1u : 0u;
    }
    const unsigned m = __ballot_sync(kFull, in);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(count, (unsigned long long)__popc(m));
}

// Range.wrap / Range.clamp in FP64 (backend/Range.java:40-96): the repeated
// +-1 of Range.wrap equals x - floor(x) (every step is exact or rounds the
// same way), and a result that rounds up to 1 is the periodic image 0.
__device__ __forceinline__ double ensure_position_f64(double x, int wrap) {
    if (wrap) {
        x = __dsub_rn(x, floor(x));
        return x >= 1.0 ? 0.0 : x;
    }
    return fmin(fmax(x, 0.0), 1.0);
}

template <int D>
__global__ void __launch_bounds__(kThreads) k_cursor_move(int n, float4* __restrict__ pt,
                                                          const uint32_t* __restrict__ flag, double dx, double dy,
                                                          double dz, int wrap) {
    const int i = blockIdx.x * kThreads + threadIdx.x;
    if (i >= n || !flag[i]) return;
    float4 p = pt[i];
    // p.position.add(delta) then physics.ensurePosition (Main.java:546-548)
    p.x = __double2float_rn(ensure_position_f64(__dadd_rn((double)p.x, dx), wrap));
    p.y = __double2float_rn(ensure_position_f64(__dadd_rn((double)p.y, dy), wrap));
    if (D == 3) p.z = __double2float_rn(ensure_position_f64(__dadd_rn((double)p.z, dz), wrap));
    pt[i] = p;
}

// Keeps particle i (flag 0) at slot off[i]: off is the exclusive scan of the
// "keep" marks, so the kept particles stay in their order.
template <int D>
__global__ void __launch_bounds__(kThreads) k_compact(int n, const uint32_t* __restrict__ off, StateBuf<D> a,
                                                      StateBuf<D> b) {
    const int i = blockIdx.x * kThreads + threadIdx.x;
    if (i >= n) return;
    const uint32_t o = off[i];
    if (off[i + 1] == o) return;  // deleted
    b.pt[o] = a.pt[i];
    b.vel[o] = a.vel[i];
}

__global__ void __launch_bounds__(kThreads) k_invert(int n, uint32_t* __restrict__ flag) {
    const int i = blockIdx.x * kThreads + threadIdx.x;
    if (i < n) flag[i] ^= 1u;
}

template <int D>
__global__ void __launch_bounds__(kThreads) k_permute(int n, const int32_t* __restrict__ src, int n_old,
                                                      StateBuf<D> a, StateBuf<D> b, uint32_t* status) {
    const int k = blockIdx.x * kThreads + threadIdx.x;
    if (k >= n) return;
    int j = src[k];
    if (j < 0 || j >= n_old) {
        atomicOr(status, kDevBadIndex);
        j = 0;
    }
    b.pt[k] = a.pt[j];
    b.vel[k] = a.vel[j];
}

template <int D>
__global__ void __launch_bounds__(kThreads) k_set_types(int n, const int32_t* __restrict__ type, int ntypes,
                                                        float4* __restrict__ pt, uint32_t* status) {
    const int i = blockIdx.x * kThreads + threadIdx.x;
    if (i >= n) return;
    int t = type[i];
    if (t < 0 || t >= ntypes) {
        atomicOr(status, kDevBadType);
        return;
    }
    float4 p = pt[i];
    if constexpr (D == 2)
        p.z = __int_as_float(t);
    else
        p.w = __int_as_float(t);
    pt[i] = p;
}

}  // namespace

template <int D>
void launch_cursor_mark(cudaStream_t st, int n, const float4* pt, const CursorDev& cu, uint32_t* flag,
                        unsigned long long* count) {
    if (n <= 0) return;
    k_cursor_mark<D><<<blocks_for(n), kThreads, 0, st>>>(n, pt, cu, flag, count);
}

template <int D>
void launch_cursor_move(cudaStream_t st, int n, float4* pt, const uint32_t* flag, double dx, double dy, double dz,
                        int wrap) {
    if (n <= 0) return;
    k_cursor_move<D><<<blocks_for(n), kThreads, 0, st>>>(n, pt, flag, dx, dy, dz, wrap);
}

void launch_invert(cudaStream_t st, int n, uint32_t* flag) {
    if (n <= 0) return;
    k_invert<<<blocks_for(n), kThreads, 0, st>>>(n, flag);
}

template <int D>
void launch_compact(cudaStream_t st, int n, const uint32_t* off, StateBuf<D> a, StateBuf<D> b) {
    if (n <= 0) return;
    k_compact<D><<<blocks_for(n), kThreads, 0, st>>>(n, off, a, b);
}

template <int D>
void launch_permute(cudaStream_t st, int n, const int32_t* src, int n_old, StateBuf<D> a, StateBuf<D> b,
                    uint32_t* status) {
    if (n <= 0) return;
    k_permute<D><<<blocks_for(n), kThreads, 0, st>>>(n, src, n_old, a, b, status);
}

template <int D>
void launch_set_types(cudaStream_t st, int n, const int32_t* type, int ntypes, float4* pt, uint32_t* status) {
    if (n <= 0) return;
    k_set_types<D><<<blocks_for(n), kThreads, 0, st>>>(n, type, ntypes, pt, status);
}

#define PLG_EDIT_INST(D)                                                                                           \
    template void launch_cursor_mark<D>(cudaStream_t, int, const float4*, const CursorDev&, uint32_t*,            \
                                        unsigned long long*);                                                     \
    template void launch_cursor_move<D>(cudaStream_t, int, float4*, const uint32_t*, double, double, double, int); \
    template void launch_compact<D>(cudaStream_t, int, const uint32_t*, StateBuf<D>, StateBuf<D>);                \
    template void launch_permute<D>(cudaStream_t, int, const int32_t*, int, StateBuf<D>, StateBuf<D>, uint32_t*); \
    template void launch_set_types<D>(cudaStream_t, int, const int32_t*, int, float4*, uint32_t*);
PLG_EDIT_INST(2)
PLG_EDIT_INST(3)
#undef PLG_EDIT_INST

}  // namespace plg
