// k_force3.cu — the 3D instantiations of the force kernels (force_tile.cuh)
// and their start-up shared-memory settings; a translation unit of its own so
// that it compiles in parallel with the 2D one (k_force.cu).
#include "force_tile.cuh"

namespace plg {

template void launch_force_batch<3>(cudaStream_t, const ForceParams*, const int*, const int*, const int*, int, int,
                                    int, bool, StateBuf<3>, const uint32_t*, const uint32_t*, StateBuf<3>, uint32_t*,
                                    uint32_t*, uint32_t*, const DebugOut*, int, unsigned long long*);

int batch_blocks_per_sm_3d(int variant, bool smem_matrix) {
    return variant == 1   ? batch_blocks_per_sm<3, 1>(smem_matrix)
           : variant == 2 ? batch_blocks_per_sm<3, 2>(smem_matrix)
                          : batch_blocks_per_sm<3, 0>(smem_matrix);
}

template void launch_force<3>(cudaStream_t, const ForceParams&, bool, StateBuf<3>, const uint32_t*, const uint32_t*,
                              StateBuf<3>, uint32_t*, uint32_t*, uint32_t*, const DebugOut*, int,
                              const HostSnap*);

cudaError_t force_kernels_init_3d() {
    cudaError_t e = allow_tile_smem<3, 0>();
    if (e == cudaSuccess) e = allow_tile_smem<3, 1>();
    if (e == cudaSuccess) e = allow_tile_smem<3, 2>();
    return e;
}

}  // namespace plg
