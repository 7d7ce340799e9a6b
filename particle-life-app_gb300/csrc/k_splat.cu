// k_splat.cu — headless point splat of the particles into an RGBA8 image,
// restating the app's default particle shaders without a graphics API:
//   default.vert     position and the palette colour of the type
//   default.geom     per particle a square of side `size` around its centre
//                    (minus camTopLeft, wrapped into [0,1) with mod when
//                    `wrap`), plus its periodic copies across the edges it
//                    is within size/2 of (resources/shaders/default.geom:24-88)
//   default.frag     discard where |texCoord| > 1: a disk
//                    (resources/shaders/default.frag:7-12)
// rasterised into 16 samples per pixel with "normal" blending of opaque
// colours, so each sample shows the last particle (in the current order,
// the reference's particle array is in after its per-step container sort,
// which is this library's slot order) covering it, and the samples are averaged
// (the multisample resolve).  As in a rasteriser without per-sample
// shading, the disk test is done once per pixel at its centre (the fragment
// shader's texCoord there) and the square is tested per sample.  Samples sit
// on a 4x4 ordered grid.  Arithmetic is FP32 without contraction, as the
// shader's would be.  Rows run bottom to top (the order glReadPixels
// returns, app/Main.java:1143-1188).
#include "plg_internal.cuh"

namespace plg {

namespace {

constexpr int kThreads = 256;
constexpr int kSamples = 4;  // per axis: 16 per pixel

__device__ __forceinline__ float glsl_mod1(float x) { return __fsub_rn(x, floorf(x)); }

// One square (and its disk) with centre (cx, cy) in world units.
__device__ void splat_one(const SplatParams& S, float cx, float cy, uint32_t tag, uint32_t* __restrict__ winner) {
    const float r = __fmul_rn(0.5f, S.size);
    // world -> pixel: ((w - cam) / dims * 2 + 1) / 2 * width = (w - cam) / dims * width + width / 2
    const float sx = __fdiv_rn((float)S.width, S.cam_w), sy = __fdiv_rn((float)S.height, S.cam_h);
    const float px0 = __fadd_rn(__fmul_rn(__fsub_rn(__fsub_rn(cx, r), S.cam_x), sx), 0.5f * S.width);
    const float px1 = __fadd_rn(__fmul_rn(__fsub_rn(__fadd_rn(cx, r), S.cam_x), sx), 0.5f * S.width);
    const float py0 = __fadd_rn(__fmul_rn(__fsub_rn(__fsub_rn(cy, r), S.cam_y), sy), 0.5f * S.height);
    const float py1 = __fadd_rn(__fmul_rn(__fsub_rn(__fadd_rn(cy, r), S.cam_y), sy), 0.5f * S.height);
    const float pcx = __fadd_rn(__fmul_rn(__fsub_rn(cx, S.cam_x), sx), 0.5f * S.width);
    const float pcy = __fadd_rn(__fmul_rn(__fsub_rn(cy, S.cam_y), sy), 0.5f * S.height);
    const float rpx = __fmul_rn(r, sx), rpy = __fmul_rn(r, sy);
    if (!(isfinite(px0) && isfinite(px1) && isfinite(py0) && isfinite(py1))) return;
    // pixel range, clamped as floats before the conversion to int
    const int i0 = (int)fminf(fmaxf(floorf(px0), 0.f), (float)S.width);
    const int i1 = (int)fmaxf(fminf(floorf(px1), (float)(S.width - 1)), -1.f);
    const int j0 = (int)fminf(fmaxf(floorf(py0), 0.f), (float)S.height);
    const int j1 = (int)fmaxf(fminf(floorf(py1), (float)(S.height - 1)), -1.f);
    for (int j = j0; j <= j1; ++j) {
        for (int i = i0; i <= i1; ++i) {
            // the fragment's texCoord at the pixel centre
            const float tx = __fdiv_rn(__fsub_rn((float)i + 0.5f, pcx), rpx);
            const float ty = __fdiv_rn(__fsub_rn((float)j + 0.5f, pcy), rpy);
            if (__fsqrt_rn(__fadd_rn(__fmul_rn(tx, tx), __fmul_rn(ty, ty))) > 1.0f) continue;  // discard
            for (int b = 0; b < kSamples; ++b) {
                const float yy = (float)j + (b + 0.5f) / kSamples;
                if (yy < py0 || yy >= py1) continue;
                for (int a = 0; a < kSamples; ++a) {
                    const float xx = (float)i + (a + 0.5f) / kSamples;
                    if (xx < px0 || xx >= px1) continue;
                    atomicMax(winner + ((size_t)j * S.width + i) * (kSamples * kSamples) + b * kSamples + a, tag);
                }
            }
        }
    }
}

template <int D>
__global__ void __launch_bounds__(kThreads) k_splat(int n, const float4* __restrict__ pt, SplatParams S,
                                                    uint32_t* __restrict__ winner) {
    const int k = blockIdx.x * kThreads + threadIdx.x;
    if (k >= n) return;
    const float4 p = pt[k];
    float cx = __fsub_rn(p.x, S.top_left_x), cy = __fsub_rn(p.y, S.top_left_y);
    const uint32_t tag = (uint32_t)k + 1u;  // later particles win
    if (S.wrap) {
        cx = glsl_mod1(cx);
        cy = glsl_mod1(cy);
    }
    splat_one(S, cx, cy, tag, winner);
    if (S.wrap) {
        const float r = __fmul_rn(0.5f, S.size);
        const int dx = cx < r ? 1 : (cx > __fsub_rn(1.0f, r) ? -1 : 0);
        const int dy = cy < r ? 1 : (cy > __fsub_rn(1.0f, r) ? -1 : 0);
        if (dx) splat_one(S, __fadd_rn(cx, (float)dx), cy, tag, winner);
        if (dy) splat_one(S, cx, __fadd_rn(cy, (float)dy), tag, winner);
        if (dx && dy) splat_one(S, __fadd_rn(cx, (float)dx), __fadd_rn(cy, (float)dy), tag, winner);
    }
}

// Multisample resolve: the average of the 16 samples, rounded to 8 bits.
template <int D>
__global__ void __launch_bounds__(kThreads) k_resolve(int npix, const uint32_t* __restrict__ winner,
                                                      const float4* __restrict__ pt, const float* __restrict__ palette,
                                                      int ncolors, uint8_t* __restrict__ out) {
    const int q = blockIdx.x * kThreads + threadIdx.x;
    if (q >= npix) return;
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    for (int s = 0; s < kSamples * kSamples; ++s) {
        const uint32_t w = winner[(size_t)q * (kSamples * kSamples) + s];
        if (!w) continue;  // cleared to (0, 0, 0, 0)
        int t = Layout<D>::type(pt[w - 1]);
        t = t < ncolors ? t : ncolors - 1;
        for (int c = 0; c < 4; ++c) acc[c] = __fadd_rn(acc[c], palette[4 * t + c]);
    }
    for (int c = 0; c < 4; ++c) {
        const float v = __fmul_rn(acc[c], 1.0f / (kSamples * kSamples));
        out[4 * (size_t)q + c] = (uint8_t)__float2int_rn(fminf(fmaxf(v, 0.f), 1.f) * 255.0f);
    }
}

}  // namespace

template <int D>
void launch_splat(cudaStream_t st, int n, const float4* pt, const SplatParams& S, uint32_t* winner,
                  const float* palette, int ncolors, uint8_t* out) {
    const int npix = S.width * S.height;
    cudaMemsetAsync(winner, 0, sizeof(uint32_t) * (size_t)npix * kSamples * kSamples, st);
    if (n > 0) k_splat<D><<<(n + kThreads - 1) / kThreads, kThreads, 0, st>>>(n, pt, S, winner);
    k_resolve<D><<<(npix + kThreads - 1) / kThreads, kThreads, 0, st>>>(npix, winner, pt, palette, ncolors, out);
}

int splat_samples_per_pixel() { return kSamples * kSamples; }

template void launch_splat<2>(cudaStream_t, int, const float4*, const SplatParams&, uint32_t*, const float*, int,
                              uint8_t*);
template void launch_splat<3>(cudaStream_t, int, const float4*, const SplatParams&, uint32_t*, const float*, int,
                              uint8_t*);

}  // namespace plg
