// k_noalloc.cu — plg_sort_cells_noalloc: the cell sort of makeContainers
// (backend/Physics.java:309-354, getContainerIndex 362-375) over positions
// that already live in caller-owned device memory, with all scratch in one
// fixed file-scope device array instead of allocations.
//
// Who needs it: a caller that must not allocate device memory while it runs
// the sort.  A frame loop that keeps positions in its own device buffer
// cannot afford cudaFree (it waits for the whole device) or a cudaMalloc
// that stalls behind other work in the middle of a frame, and a caller with
// a device-memory budget fixed at start-up cannot let a library grow it.
// Nothing in this file calls cudaMalloc, cudaFree or a library routine that
// allocates; the only device memory used is g_scratch below plus the
// caller's buffers.
//
// Set-up: the first call on a device, with that device current, resolves
// g_scratch's device address with cudaGetSymbolAddress (which may load this
// module) and caches it per device.  Make that first call on every device
// before any stream capture starts.
//
// Scratch contents (32-bit words), all sized for the stated maxima:
//   cell[kMaxParticles]   cell of each particle
//   tmp[kMaxParticles]    unstable cell-sorted order
//   counts[kMaxCells]     per-cell counts; must be zero before counting (the
//                         scatter drains them back to zero)
//   own status word       used when the caller passes no status word
//   scan tile words       (64-bit) look-back state; must be zero before the scan
// Every call zeroes counts and the scan words itself (cudaMemsetAsync on the
// caller's stream), so no earlier call, completed or not, leaves state
// behind.  Calls that overlap in time on one device (any streams, any host
// threads) share this scratch and race; the caller serialises them.
#include "plg_internal.cuh"
#include "plgpu.h"

#include <mutex>

namespace plg {
namespace {

constexpr int kThreads = 256;
constexpr int64_t kMaxParticles = PLG_NOALLOC_MAX_PARTICLES;
constexpr int64_t kMaxCells = PLG_NOALLOC_MAX_CELLS;
constexpr int64_t kOffTmp = kMaxParticles;
constexpr int64_t kOffCounts = 2 * kMaxParticles;
constexpr int64_t kOffStatus = kOffCounts + kMaxCells;
constexpr int64_t kOffScan = kOffStatus + 64;        // 256-byte aligned, 64-bit words from here
constexpr int64_t kScanWords = kMaxCells / 256 + 2;  // enough for scan tiles of >= 256 cells
constexpr int64_t kScratchWords = kOffScan + 2 * kScanWords;
constexpr int kMaxDevices = 64;

static_assert(kOffCounts % 4 == 0, "the scan reads counts as uint4");
static_assert(kOffScan % 64 == 0, "scan words start on a 256-byte boundary");

// About 4.2 MB per device, zero at module load.
static __device__ __align__(256) uint32_t g_scratch[kScratchWords];

std::mutex g_setup_mutex;
uint32_t* g_scratch_ptr[kMaxDevices] = {};

// Per-axis getContainerIndex in FP64 (Physics.java:363-372): (int)(x / cs)
// with the quotient correctly rounded, as in Java, and cx == nx -> nx - 1.
// A position outside [0,1] (or NaN) is clamped into the grid and flagged, so
// no counter outside the grid is ever touched.
__device__ __forceinline__ int axis_cell_f64(double x, double cs, int nx, uint32_t& bad) {
    if (!(x >= 0.0 && x <= 1.0)) {
        bad |= kDevBadPosition;
        x = x > 1.0 ? 1.0 : 0.0;  // NaN -> 0, like Java's (int) of NaN
    }
    const int c = (int)(x / cs);
    return c >= nx ? nx - 1 : c;
}

template <int D>
__global__ void __launch_bounds__(kThreads) k_bin_f64(int n, const double* __restrict__ pos, double cs, int nx,
                                                      uint32_t* __restrict__ cell, uint32_t* counts,
                                                      uint32_t* status) {
    const int i = blockIdx.x * kThreads + threadIdx.x;
    const bool valid = i < n;
    uint32_t c = 0;
    if (valid) {
        uint32_t bad = 0;
        uint32_t stride = 1;
#pragma unroll
        for (int k = 0; k < D; ++k) {
            c += (uint32_t)axis_cell_f64(pos[3 * (size_t)i + k], cs, nx, bad) * stride;
            stride *= (uint32_t)nx;
        }
        if (bad) atomicOr(status, bad);
    }
    const unsigned mask = __ballot_sync(kFull, valid);
    if (valid) {
        bin_add(counts, c, mask);
        cell[i] = c;
    }
}

// perm[cell_start[c] + r] = i with r = the number of members of i's cell with
// a smaller index: the order of the reference's sequential fill loop
// (Physics.java:342-348).
__global__ void __launch_bounds__(kThreads) k_stable_order(int n, const uint32_t* __restrict__ tmp,
                                                           const uint32_t* __restrict__ cell,
                                                           const uint32_t* __restrict__ cell_start,
                                                           uint32_t* __restrict__ perm) {
    const int s = blockIdx.x * kThreads + threadIdx.x;
    if (s >= n) return;
    const uint32_t i = tmp[s];
    const uint32_t c = cell[i];
    const uint32_t st = cell_start[c], en = cell_start[c + 1];
    uint32_t r = 0;
    for (uint32_t t = st; t < en; ++t) r += __ldg(tmp + t) < i ? 1u : 0u;
    perm[st + r] = i;
}

// Device address of g_scratch on the current device, resolved once.
cudaError_t scratch_for_current_device(uint32_t** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
        uint32_t* p = nullptr;
        e = cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}

// True when p is device (or managed) memory of device `dev` with the given
// alignment.
bool device_pointer_ok(const void* p, int dev, size_t align) {
    if (reinterpret_cast<uintptr_t>(p) % align != 0) return false;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeManaged) return true;
    return a.type == cudaMemoryTypeDevice && a.device == dev;
}

}  // namespace
}  // namespace plg

extern "C" int plg_sort_cells_noalloc(int32_t dim, double rmax, int64_t n, const double* pos, uint32_t* perm,
                                      uint32_t* cell_start, uint32_t* status, void* stream) {
    using namespace plg;
    if (dim != 2 && dim != 3) return PLG_E_INVALID_ARG;
    if (n < 0) return PLG_E_INVALID_ARG;
    int32_t nx = 0;
    if (plg_cell_bounds(rmax, &nx, nullptr, 0) != PLG_OK) return PLG_E_INVALID_ARG;
    int64_t ncells = nx;
    for (int k = 1; k < dim; ++k) ncells *= nx;
    if (n > kMaxParticles || ncells > kMaxCells) return PLG_E_CAPACITY;
    if (scan_blocks((int)ncells) + 1 > kScanWords) return PLG_E_CAPACITY;
    if (!cell_start || (n > 0 && (!pos || !perm))) return PLG_E_INVALID_ARG;

    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return PLG_E_CUDA;
    }
    if (!device_pointer_ok(cell_start, dev, 16)) return PLG_E_INVALID_ARG;  // the scan stores uint4
    if (n > 0 && (!device_pointer_ok(pos, dev, 8) || !device_pointer_ok(perm, dev, 4))) return PLG_E_INVALID_ARG;
    if (status && !device_pointer_ok(status, dev, 4)) return PLG_E_INVALID_ARG;

    uint32_t* scratch = nullptr;
    if (scratch_for_current_device(&scratch) != cudaSuccess) {
        cudaGetLastError();
        return PLG_E_CUDA;
    }
    uint32_t* cell = scratch;
    uint32_t* tmp = scratch + kOffTmp;
    uint32_t* counts = scratch + kOffCounts;
    uint32_t* st_word = status ? status : scratch + kOffStatus;
    auto* scan_state = reinterpret_cast<unsigned long long*>(scratch + kOffScan);
    const auto s = static_cast<cudaStream_t>(stream);

    if (cudaMemsetAsync(counts, 0, (size_t)ncells * sizeof(uint32_t), s) != cudaSuccess ||
        cudaMemsetAsync(scan_state, 0, (size_t)(scan_blocks((int)ncells) + 1) * sizeof(unsigned long long), s) !=
            cudaSuccess) {
        cudaGetLastError();
        return PLG_E_CUDA;
    }
    const int ni = (int)n;
    const int blocks = (ni + kThreads - 1) / kThreads;
    const double cs = rmax;  // containerSize = settings.rmax (Physics.java:312)
    if (ni > 0) {
        if (dim == 2) {
            k_bin_f64<2><<<blocks, kThreads, 0, s>>>(ni, pos, cs, nx, cell, counts, st_word);
        } else {
            k_bin_f64<3><<<blocks, kThreads, 0, s>>>(ni, pos, cs, nx, cell, counts, st_word);
        }
    }
    launch_scan(s, counts, (int)ncells, cell_start, scan_state, st_word, nullptr);
    if (ni > 0) {
        launch_scatter(s, ni, cell, counts, cell_start, tmp);
        k_stable_order<<<blocks, kThreads, 0, s>>>(ni, tmp, cell, cell_start, perm);
    }
    if (cudaGetLastError() != cudaSuccess) return PLG_E_CUDA;
    return PLG_OK;
}
