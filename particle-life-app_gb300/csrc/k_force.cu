// k_force.cu — the 2D instantiations of the force kernels (force_tile.cuh),
// the start-up shared-memory settings of every tiled kernel, the tile sizes
// the batch host code lays tiles out with, and the FP32 FMA throughput probe
// that serves as the force kernel's roofline denominator.  The 3D
// instantiations are in k_force3.cu, a separate translation unit so the two
// compile in parallel.
#include "force_tile.cuh"

namespace plg {

// k_force3.cu
cudaError_t force_kernels_init_3d();

int tile_targets(int dim, int variant) {
    if (dim == 2)
        return variant == 1 ? TileCfg<2, 1>::kTargets : variant == 2 ? TileCfg<2, 2>::kTargets : TileCfg<2, 0>::kTargets;
    return variant == 1 ? TileCfg<3, 1>::kTargets : variant == 2 ? TileCfg<3, 2>::kTargets : TileCfg<3, 0>::kTargets;
}

template void launch_force_batch<2>(cudaStream_t, const ForceParams*, const int*, const int*, const int*, int, int,
                                    int, bool, StateBuf<2>, const uint32_t*, const uint32_t*, StateBuf<2>, uint32_t*,
                                    uint32_t*, uint32_t*, const DebugOut*, int, unsigned long long*);

// k_force3.cu
int batch_blocks_per_sm_3d(int variant, bool smem_matrix);

int batch_blocks_per_sm(int dim, int variant, bool smem_matrix) {
    if (dim == 3) return batch_blocks_per_sm_3d(variant, smem_matrix);
    return variant == 1   ? batch_blocks_per_sm<2, 1>(smem_matrix)
           : variant == 2 ? batch_blocks_per_sm<2, 2>(smem_matrix)
                          : batch_blocks_per_sm<2, 0>(smem_matrix);
}

template void launch_force<2>(cudaStream_t, const ForceParams&, bool, StateBuf<2>, const uint32_t*, const uint32_t*,
                              StateBuf<2>, uint32_t*, uint32_t*, uint32_t*, const DebugOut*, int,
                              const HostSnap*);

cudaError_t force_kernels_init() {
    cudaError_t e = allow_tile_smem<2, 0>();
    if (e == cudaSuccess) e = allow_tile_smem<2, 1>();
    if (e == cudaSuccess) e = allow_tile_smem<2, 2>();
    if (e == cudaSuccess) e = force_kernels_init_3d();
    return e;
}

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

// The special-function unit: eight independent rsqrt.approx chains per
// thread (the force loop's one SFU operation per candidate).
__global__ void __launch_bounds__(256) k_rsqrt_probe(float* out, int iters, float seed) {
    float a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = seed + threadIdx.x + k;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int r = 0; r < 16; ++r) {
#pragma unroll
            for (int k = 0; k < 8; ++k) asm volatile("rsqrt.approx.ftz.f32 %0, %0;" : "+f"(a[k]));
        }
    }
    float r = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) r += a[k];
    if (r == 12345.678f) out[0] = r;  // keeps the chains live
}

}  // namespace

cudaError_t probe_sfu_peak(double* gops) {
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
    const int blocks = sms * 8, threads = 256, iters = 1024;
    k_rsqrt_probe<<<blocks, threads>>>(out, 16, 1.f);  // warm-up
    cudaEventRecord(e0);
    k_rsqrt_probe<<<blocks, threads>>>(out, iters, 1.f);
    cudaEventRecord(e1);
    e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e == cudaSuccess) *gops = 8.0 * 16.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e9;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    return e;
}

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
