// k_init.cu — the app's initialiser catalogues as seeded device generators:
//   position setters  app/PositionSetterProvider.java:16-119 (+ the default,
//                     backend/DefaultPositionSetter.java:7-14)
//   type setters      app/TypeSetterProvider.java:11-45 (+ backend/DefaultTypeSetter.java)
// The reference draws from java.util.Random / Math.random; here every
// particle draws from a counter-based generator, Philox4x64-10 (Salmon,
// Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC 2011),
// with key (seed, 0) and counter (particle index, stream, 0, 0): stream 0
// feeds the position setters, 1 the type setters, 2 the third coordinate of
// 3D worlds.  A uniform double is the top 53 bits of a word times 2^-53;
// a normal variate is the cosine branch of Box-Muller on two uniforms.
// Setters then apply ensurePosition (Physics.java:297-303) and zero the
// velocity, as Physics.setPosition does.
#include "plg_internal.cuh"

namespace plg {

namespace {

constexpr int kThreads = 256;

struct Philox4 {
    unsigned long long w[4];
};

// Philox4x64-10: ten rounds of two 64x64->128 multiplies and a key bump.
__host__ __device__ inline Philox4 philox4x64(unsigned long long c0, unsigned long long c1, unsigned long long c2,
                                              unsigned long long c3, unsigned long long k0, unsigned long long k1) {
    const unsigned long long M0 = 0xD2E7470EE14C6C93ull, M1 = 0xCA5A826395121157ull;
    const unsigned long long W0 = 0x9E3779B97F4A7C15ull, W1 = 0xBB67AE8584CAA73Bull;
    for (int r = 0; r < 10; ++r) {
#ifdef __CUDA_ARCH__
        const unsigned long long hi0 = __umul64hi(M0, c0), lo0 = M0 * c0;
        const unsigned long long hi1 = __umul64hi(M1, c2), lo1 = M1 * c2;
#else
        const unsigned __int128 p0 = (unsigned __int128)M0 * c0, p1 = (unsigned __int128)M1 * c2;
        const unsigned long long hi0 = (unsigned long long)(p0 >> 64), lo0 = (unsigned long long)p0;
        const unsigned long long hi1 = (unsigned long long)(p1 >> 64), lo1 = (unsigned long long)p1;
#endif
        const unsigned long long n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += W0;
        k1 += W1;
    }
    return Philox4{{c0, c1, c2, c3}};
}

__device__ __forceinline__ double unit(unsigned long long w) { return (double)(w >> 11) * 0x1.0p-53; }

// Box-Muller, cosine branch: N(0,1) from two uniforms in [0,1).
__device__ __forceinline__ double normal(double u1, double u2) {
    return sqrt(-2.0 * log(1.0 - u1)) * cos(2.0 * M_PI * u2);
}

__device__ __forceinline__ double ensure_pos(double x, int wrap) {
    if (wrap) {
        x = x - floor(x);
        return x >= 1.0 ? 0.0 : x;
    }
    return fmin(fmax(x, 0.0), 1.0);
}

// TypeSetterProvider.mapType: constrain((int) floor(value * nTypes)).
__device__ __forceinline__ int map_type(double v, int n) {
    const double f = floor(v * n);
    return f < 0.0 ? 0 : (f > (double)(n - 1) ? n - 1 : (int)f);
}

// Position of one particle from its setter (coordinates of the setters are
// in [-1,1] and mapped by x * 0.5 + 0.5, as the catalogue does).
__device__ void position_of(int setter, unsigned long long seed, long long i, int type, int ntypes, double& x,
                            double& y) {
    const Philox4 r = philox4x64((unsigned long long)i, 0ull, 0ull, 0ull, seed, 0ull);
    const double u0 = unit(r.w[0]), u1 = unit(r.w[1]), u2 = unit(r.w[2]), u3 = unit(r.w[3]);
    const double two_pi = 2.0 * M_PI;
    const double f03 = (double)0.3f, f05 = (double)0.5f, f01 = (double)0.1f, f02 = (double)0.2f,
                 f015 = (double)0.15f;
    switch (setter) {
        case kPosUniform:
            x = u0;
            y = u1;
            return;
        case kPosCentered:
            x = normal(u0, u1) * f03;
            y = normal(u2, u3) * f03;
            break;
        case kPosUniformCircle: {
            const double a = u0 * two_pi, rad = 0.5 * sqrt(u1);
            x = cos(a) * rad;
            y = sin(a) * rad;
            break;
        }
        case kPosCenteredCircle: {
            const double a = u0 * two_pi, rad = f05 * u1;
            x = cos(a) * rad;
            y = sin(a) * rad;
            break;
        }
        case kPosRing: {
            const double a = u0 * two_pi, rad = 0.7 + 0.02 * normal(u2, u3);
            x = cos(a) * rad;
            y = sin(a) * rad;
            break;
        }
        case kPosRainbowRing: {
            const double a = (0.3 * normal(u0, u1) + type) / ntypes * two_pi, rad = 0.7 + 0.02 * normal(u2, u3);
            x = cos(a) * rad;
            y = sin(a) * rad;
            break;
        }
        case kPosColorBattle: {
            const double ca = type / (double)ntypes * two_pi, cr = f05;
            const double a = u0 * two_pi, rad = u1 * f01;
            x = cr * cos(ca) + cos(a) * rad;
            y = cr * sin(ca) + sin(a) * rad;
            break;
        }
        case kPosColorWheel: {
            const double ca = type / (double)ntypes * two_pi, cr = f03, ir = f02;
            x = cr * cos(ca) + normal(u0, u1) * ir;
            y = cr * sin(ca) + normal(u2, u3) * ir;
            break;
        }
        case kPosLine:
            x = 2 * u0 - 1;
            y = (2 * u1 - 1) * f015;
            break;
        case kPosSpiral: {
            const double f = u0, a = 2.0 * two_pi * f, spread = 0.5 * fmin(f, 0.2);
            const double rad = 0.9 * f + spread * normal(u2, u3) * spread;
            x = rad * cos(a);
            y = rad * sin(a);
            break;
        }
        default: {  // kPosRainbowSpiral
            double f = (type + 1) / (double)(ntypes + 2) + 0.3 / ntypes * normal(u0, u1);
            f = f < 0 ? 0 : (f > 1 ? 1 : f);
            const double a = 2.0 * two_pi * f, spread = 0.5 * fmin(f, 0.2);
            const double rad = 0.9 * f + spread * normal(u2, u3) * spread;
            x = rad * cos(a);
            y = rad * sin(a);
            break;
        }
    }
    x = x * 0.5 + 0.5;
    y = y * 0.5 + 0.5;
}

// Third coordinate of 3D worlds (an extension: the app is 2D): uniform, or
// normal like x for the centred setter.
__device__ double z_of(int setter, unsigned long long seed, long long i) {
    const Philox4 r = philox4x64((unsigned long long)i, 2ull, 0ull, 0ull, seed, 0ull);
    if (setter == kPosCentered) return normal(unit(r.w[0]), unit(r.w[1])) * (double)0.3f * 0.5 + 0.5;
    return unit(r.w[0]);
}

__device__ int type_of(int setter, unsigned long long seed, long long i, double px, double py, double pz, double vx,
                       double vy, double vz, int type, int n) {
    const Philox4 r = philox4x64((unsigned long long)i, 1ull, 0ull, 0ull, seed, 0ull);
    const double v0 = unit(r.w[0]), v1 = unit(r.w[1]);
    switch (setter) {
        case kTypeRandom:
            return (int)floor(v0 * n);
        case kTypeRandomize10:
            return v0 < 0.1 ? map_type(v1, n) : type;
        case kTypeSlices:
            return map_type(px, n);
        case kTypeOnion: {
            const double dx = px - 0.5, dy = py - 0.5, dz = pz;
            return map_type(sqrt(dx * dx + (dy * dy + dz * dz)) * 2, n);
        }
        case kTypeRotate:
            return (type + 1) % n;
        case kTypeFlip:
            return n - 1 - type;
        case kTypeMoreOfFirst:
            return map_type(v0 * v1, n);
        default:  // kTypeKillStill
            return sqrt(vx * vx + (vy * vy + vz * vz)) < 0.01 ? n - 1 : type;
    }
}

// Physics.generateParticle (Physics.java:285-295): the type first (from a
// particle at the origin at rest with type 0), then the position from the
// type; velocity 0; ids 0..n-1.
template <int D>
__global__ void __launch_bounds__(kThreads) k_generate(int n, int pos_setter, int type_setter, unsigned long long seed,
                                                       int ntypes, int wrap, StateBuf<D> a) {
    const int i = blockIdx.x * kThreads + threadIdx.x;
    if (i >= n) return;
    const int t = type_of(type_setter, seed, i, 0, 0, 0, 0, 0, 0, 0, ntypes);
    double x, y;
    position_of(pos_setter, seed, i, t, ntypes, x, y);
    const float fx = __double2float_rn(ensure_pos(x, wrap)), fy = __double2float_rn(ensure_pos(y, wrap));
    if constexpr (D == 2) {
        a.pt[i] = make_float4(fx, fy, __int_as_float(t), __int_as_float(i));
        a.vel[i] = make_float2(0.f, 0.f);
    } else {
        const float fz = __double2float_rn(ensure_pos(z_of(pos_setter, seed, i), wrap));
        a.pt[i] = make_float4(fx, fy, fz, __int_as_float(t));
        a.vel[i] = make_float4(0.f, 0.f, 0.f, __int_as_float(i));
    }
}

// Physics.setPositions (Physics.java:166-168) with a catalogue setter.
template <int D>
__global__ void __launch_bounds__(kThreads) k_apply_positions(int n, int setter, unsigned long long seed, int ntypes,
                                                              int wrap, StateBuf<D> a) {
    const int i = blockIdx.x * kThreads + threadIdx.x;
    if (i >= n) return;
    float4 p = a.pt[i];
    double x, y;
    position_of(setter, seed, i, Layout<D>::type(p), ntypes, x, y);
    p.x = __double2float_rn(ensure_pos(x, wrap));
    p.y = __double2float_rn(ensure_pos(y, wrap));
    if constexpr (D == 2) {
        a.vel[i] = make_float2(0.f, 0.f);
    } else {
        p.z = __double2float_rn(ensure_pos(z_of(setter, seed, i), wrap));
        const float4 v = a.vel[i];
        a.vel[i] = make_float4(0.f, 0.f, 0.f, v.w);
    }
    a.pt[i] = p;
}

// Physics.setTypes (Physics.java:509-511) with a catalogue type setter.
template <int D>
__global__ void __launch_bounds__(kThreads) k_apply_types(int n, int setter, unsigned long long seed, int ntypes,
                                                          StateBuf<D> a) {
    const int i = blockIdx.x * kThreads + threadIdx.x;
    if (i >= n) return;
    float4 p = a.pt[i];
    const typename Layout<D>::Vel v = a.vel[i];
    double vz = 0.0;
    if constexpr (D == 3) vz = v.z;
    const int t = type_of(setter, seed, i, p.x, p.y, D == 3 ? p.z : 0.0, v.x, v.y, vz, Layout<D>::type(p), ntypes);
    if constexpr (D == 2)
        p.z = __int_as_float(t);
    else
        p.w = __int_as_float(t);
    a.pt[i] = p;
}

}  // namespace

template <int D>
void launch_generate(cudaStream_t st, int n, int pos_setter, int type_setter, unsigned long long seed, int ntypes,
                     int wrap, StateBuf<D> a) {
    if (n <= 0) return;
    k_generate<D><<<(n + kThreads - 1) / kThreads, kThreads, 0, st>>>(n, pos_setter, type_setter, seed, ntypes, wrap,
                                                                       a);
}

template <int D>
void launch_apply_positions(cudaStream_t st, int n, int setter, unsigned long long seed, int ntypes, int wrap,
                            StateBuf<D> a) {
    if (n <= 0) return;
    k_apply_positions<D><<<(n + kThreads - 1) / kThreads, kThreads, 0, st>>>(n, setter, seed, ntypes, wrap, a);
}

template <int D>
void launch_apply_types(cudaStream_t st, int n, int setter, unsigned long long seed, int ntypes, StateBuf<D> a) {
    if (n <= 0) return;
    k_apply_types<D><<<(n + kThreads - 1) / kThreads, kThreads, 0, st>>>(n, setter, seed, ntypes, a);
}

// MatrixGeneratorProvider (app/MatrixGeneratorProvider.java:13-79) and
// DefaultMatrix.randomize (backend/DefaultMatrix.java:25-31), on the host:
// entry (i, j) of a random matrix is 2u - 1 with u from the generator at
// counter (i * size + j, 3, 0, 0).
void generate_matrix(int kind, int size, unsigned long long seed, double* m) {
    auto uniform = [&](int i, int j) {
        const Philox4 r = philox4x64((unsigned long long)i * (unsigned long long)size + (unsigned long long)j, 3ull,
                                     0ull, 0ull, seed, 0ull);
        return (double)(r.w[0] >> 11) * 0x1.0p-53;
    };
    for (int i = 0; i < size; ++i)
        for (int j = 0; j < size; ++j) {
            double v = 0.0;
            const bool diag = j == i, next = j == (i + 1) % size, prev = j == (i + size - 1) % size;
            switch (kind) {
                case kMatrixRandom:
                case kMatrixSymmetry:
                    v = 2 * uniform(i, j) - 1;
                    break;
                case kMatrixChains:
                    v = (diag || next || prev) ? 1.0 : -1.0;
                    break;
                case kMatrixChains2:
                    v = diag ? 1.0 : ((next || prev) ? 0.2 : -1.0);
                    break;
                case kMatrixChains3:
                    v = diag ? 1.0 : ((next || prev) ? 0.2 : 0.0);
                    break;
                case kMatrixSnakes:
                    v = diag ? 1.0 : (next ? 0.2 : 0.0);
                    break;
                default:  // kMatrixZero
                    v = 0.0;
            }
            m[(size_t)i * size + j] = v;
        }
    if (kind == kMatrixSymmetry)  // m.set(i, j, m.get(j, i)) for j >= i
        for (int i = 0; i < size; ++i)
            for (int j = i; j < size; ++j) m[(size_t)i * size + j] = m[(size_t)j * size + i];
}

template void launch_generate<2>(cudaStream_t, int, int, int, unsigned long long, int, int, StateBuf<2>);
template void launch_generate<3>(cudaStream_t, int, int, int, unsigned long long, int, int, StateBuf<3>);
template void launch_apply_positions<2>(cudaStream_t, int, int, unsigned long long, int, int, StateBuf<2>);
template void launch_apply_positions<3>(cudaStream_t, int, int, unsigned long long, int, int, StateBuf<3>);
template void launch_apply_types<2>(cudaStream_t, int, int, unsigned long long, int, StateBuf<2>);
template void launch_apply_types<3>(cudaStream_t, int, int, unsigned long long, int, StateBuf<3>);

}  // namespace plg
