// plg_internal.cuh — device-side types and helpers shared by the kernels of
// the Particle Life physics step (binning, force/integration, conversion).
//
// Data layout in HBM, one world, FP32 structure of arrays:
//   2D: pt  float4 {x, y, type bits, id bits}   vel float2 {vx, vy}
//   3D: pt  float4 {x, y, z, type bits}         vel float4 {vx, vy, vz, id bits}
// Two copies (A = current order, B = cell-sorted order) alternate inside a
// step: the sort gathers A into B, the force kernel reads B and writes the
// next state into A, so positions that the velocity phase still reads are
// never overwritten (the reason Physics.java:122-131 runs two phases).
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>

namespace plg {

// NVTX range over a public call (plg_step, plg_upload, ...), so that a
// profiler can select its kernels (ncu --nvtx); free when no tool is attached.
struct TraceRange {
    explicit TraceRange(const char* name) { nvtxRangePushA(name); }
    ~TraceRange() { nvtxRangePop(); }
    TraceRange(const TraceRange&) = delete;
    TraceRange& operator=(const TraceRange&) = delete;
};

constexpr unsigned kFull = 0xffffffffu;

// Programmatic dependent launch.  A kernel launched with
// launch_after (below) may be scheduled while the kernel before it in the
// stream is still finishing; pdl_wait() returns once that kernel has
// completed and its writes are visible, so every read of its results comes
// after it.  Without the launch attribute pdl_wait() returns at once.
// pdl_release() lets the next kernel's blocks be scheduled as this grid's
// last blocks run (it orders nothing: the next kernel still waits).
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_release() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Launches kernel<<<grid, block, smem, st>>>(args...) as a programmatic
// dependent of the work before it in `st` (the kernel must pdl_wait()
// before it reads that work's results); inside stream capture this becomes
// a programmatic edge of the graph.
template <typename... KArgs, typename... Args>
cudaError_t launch_after(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                         Args... args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// Status bits raised by kernels into the context's device status word.
enum DeviceStatus : uint32_t {
    kDevBadPosition = 1u << 0,  // upload: position outside [0,1] or not finite
    kDevBadType = 1u << 1,      // upload: type outside [0, matrix size)
    kDevBadVelocity = 1u << 2,  // upload: velocity not finite
    kDevSpinLimit = 1u << 3,    // a bounded device wait ran out
    kDevBadIndex = 1u << 4,     // permute: source index outside the particles
};

// Cursor shapes of app/cursors (CircleCursorShape, SquareCursorShape,
// InfinityCursorShape) and a cursor as the device kernels see it.
constexpr int kCursorCircle = 0, kCursorSquare = 1, kCursorInfinity = 2;
struct CursorDev {
    double x, y, z, size;
    int shape;
    int wrap;
};

template <int D>
struct Layout;

template <>
struct Layout<2> {
    using Vel = float2;
    static __device__ __forceinline__ int type(const float4& p) { return __float_as_int(p.z); }
    static __device__ __forceinline__ int id(const float4& p, const Vel&) { return __float_as_int(p.w); }
};

template <>
struct Layout<3> {
    using Vel = float4;
    static __device__ __forceinline__ int type(const float4& p) { return __float_as_int(p.w); }
    static __device__ __forceinline__ int id(const float4&, const Vel& v) { return __float_as_int(v.w); }
};

// Uniform grid of the reference: cell size cs = rmax, nx = floor(1/cs) cells
// per axis (Physics.java:82-85, 312-313).  `bounds` is the exact lookup table
// built on the host: bounds[k] = smallest float x with (int)((double)x/cs) >= k.
struct Grid {
    int nx;
    int ncells;           // nx^D
    float inv_cs;         // (float)(1/cs): first guess only
    float b_nx;           // bounds[nx]: x >= b_nx means (int)(x/cs) == nx
    const float* bounds;  // nx + 1 entries
};

// (int)((double)x / cs) for an FP32 x in [0,1], bit-exact with the
// reference's FP64 expression (Physics.java:363-364, 404-405): a float guess,
// corrected by one table compare each way.  The guess is off by at most one
// for nx < 2^21 (relative error <= 2^-23 of a quotient <= nx + 1).
__device__ __forceinline__ int axis_cell_unclamped(float x, const Grid& g) {
    int c = (int)(x * g.inv_cs);
    c = min(max(c, 0), g.nx);
    if (c > 0 && x < __ldg(g.bounds + c)) {
        --c;
    } else if (c < g.nx && x >= __ldg(g.bounds + c + 1)) {
        ++c;
    }
    return c;
}

// getContainerIndex per axis: clamp cx == nx to nx - 1 (Physics.java:367-372).
__device__ __forceinline__ int axis_cell(float x, const Grid& g) {
    return min(axis_cell_unclamped(x, g), g.nx - 1);
}

template <int D>
__device__ __forceinline__ uint32_t cell_index(float x, float y, float z, const Grid& g) {
    uint32_t c = (uint32_t)axis_cell(x, g) + (uint32_t)axis_cell(y, g) * (uint32_t)g.nx;
    if (D == 3) c += (uint32_t)axis_cell(z, g) * (uint32_t)g.nx * (uint32_t)g.nx;
    return c;
}

// Counting step of makeContainers (Physics.java:328-332) for one particle per
// lane: lanes of a warp with the same cell add once, without waiting for the
// result.  `mask` = lanes taking part (all must call).
__device__ __forceinline__ void bin_add(uint32_t* counts, uint32_t cell, unsigned mask) {
    const unsigned peers = __match_any_sync(mask, cell);
    if ((threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(counts + cell, (uint32_t)__popc(peers));
}

// A rank in [0, counts[cell]) for one particle per lane, distinct for every
// caller of the cell; counts[cell] goes back down to 0 once every member
// has taken one.  The order of the ranks is arbitrary (the gather re-ranks
// the members stably).
__device__ __forceinline__ uint32_t bin_take(uint32_t* counts, uint32_t cell, unsigned mask) {
    const unsigned peers = __match_any_sync(mask, cell);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    const uint32_t k = (uint32_t)__popc(peers);
    uint32_t top = 0;
    if (lane == leader) top = atomicSub(counts + cell, k);
    top = __shfl_sync(peers, top, leader);
    return top - k + (uint32_t)__popc(peers & ((1u << lane) - 1u));
}

// splitmix64 output function (Steele, Lea, Flood 2014) on id + gamma: the
// order-free pair hash of the parity checks.
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t id) {
    uint64_t z = id + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// World of sorted slot s in a batch: the last k with off[k] <= s
// (off: first slot of each world, ascending).
__device__ __forceinline__ int world_of(const int* __restrict__ off, int nworlds, int s) {
    int lo = 0, hi = nworlds;
    while (hi - lo > 1) {
        const int m = (lo + hi) >> 1;
        if (__ldg(off + m) <= s)
            lo = m;
        else
            hi = m;
    }
    return lo;
}

// Parameters of the force / integration kernel, passed by value.
struct ForceParams {
    Grid g;
    int n;
    int wrap;
    int ntypes;
    int slmask_ok;          // nx >= 4: sliver targets need the stencil correction
    const float* matrix;    // ntypes x ntypes, row-major, FP32
    float lo, hi, tiny;     // FP32 d2 decision band around rmax^2
    float inv_rmax;
    float beta, inv_beta, one_plus_beta, inv_one_minus_beta;
    float m2_inv_rmax;      // -2 / rmax
    float beta_rmax;        // beta * rmax: below this distance the linear repulsion applies
    float k1;               // 1 / (beta * rmax): (|d|/(beta rmax) - 1) / |d| = k1 - 1/|d|
    float ff;               // (float) pow(friction, 60 dt)
    float scale;            // (float) (rmax * force * dt)
    float dt;
    double rmax, rmax2, beta_d;
    uint32_t cell_base;     // global index of this world's cell 0 (0 for a single world)
    int p_off;              // first sorted slot of this world (0 for a single world)
};

// Per-particle debug outputs of the instrumented force kernel.
struct DebugOut {
    int32_t* pairs;
    unsigned long long* hsum;
    unsigned long long* hxor;
    float* acc;
    unsigned long long* candidates;
};

// Snapshot arrays the force kernel writes besides the next state, in the
// plg_download layout (pos and vel: 3 doubles per particle, z = 0 in 2D;
// type and id: one int32 each), indexed by sorted slot.  Each pointer is
// device-accessible (page-locked host memory's device alias, or pageable
// memory on a device with coherent pageable access) or null (not written).
struct HostSnap {
    double* pos;
    double* vel;
    int32_t* type;
    int32_t* id;
    __host__ __device__ bool any() const { return pos || vel || type || id; }
};

template <int D>
struct StateBuf {
    float4* pt;
    typename Layout<D>::Vel* vel;
};

// ---- launchers (defined in the .cu files, called by the host library) ----

// cell_base: added to every cell index (a world's first cell in a batch);
// id_base: the id of the first particle (ids are id_base + index).
template <int D>
void launch_upload(cudaStream_t st, int n, const double* pos, const double* vel, const int32_t* type,
                   int ntypes, StateBuf<D> a, uint32_t* cell, uint32_t* counts, Grid g, uint32_t* status,
                   uint32_t cell_base = 0, int id_base = 0);

// ---- initialisers (k_init.cu) ----
// Position setters (app/PositionSetterProvider.java), type setters
// (app/TypeSetterProvider.java) and matrix generators
// (app/MatrixGeneratorProvider.java), numbered as in include/plgpu.h.
enum PositionSetterKind {
    kPosUniform = 0, kPosCentered, kPosUniformCircle, kPosCenteredCircle, kPosRing, kPosRainbowRing,
    kPosColorBattle, kPosColorWheel, kPosLine, kPosSpiral, kPosRainbowSpiral, kPosCount
};
enum TypeSetterKind {
    kTypeRandom = 0, kTypeRandomize10, kTypeSlices, kTypeOnion, kTypeRotate, kTypeFlip, kTypeMoreOfFirst,
    kTypeKillStill, kTypeCount
};
enum MatrixGeneratorKind {
    kMatrixRandom = 0, kMatrixSymmetry, kMatrixChains, kMatrixChains2, kMatrixChains3, kMatrixSnakes, kMatrixZero,
    kMatrixCount
};
template <int D>
void launch_generate(cudaStream_t st, int n, int pos_setter, int type_setter, unsigned long long seed, int ntypes,
                     int wrap, StateBuf<D> a);
template <int D>
void launch_apply_positions(cudaStream_t st, int n, int setter, unsigned long long seed, int ntypes, int wrap,
                            StateBuf<D> a);
template <int D>
void launch_apply_types(cudaStream_t st, int n, int setter, unsigned long long seed, int ntypes, StateBuf<D> a);
void generate_matrix(int kind, int size, unsigned long long seed, double* m);

// ---- headless splat (k_splat.cu) ----
// Camera as the app's NormalizedDeviceCoordinates (centre, dimensions, in
// world units), camTopLeft and wrap as the default geometry shader's
// uniforms, size = the particle diameter in world units.
struct SplatParams {
    int width, height;
    float cam_x, cam_y, cam_w, cam_h;
    float top_left_x, top_left_y;
    float size;
    int wrap;
};
int splat_samples_per_pixel();
// winner: width * height * splat_samples_per_pixel() words of scratch;
// palette: ncolors RGBA floats (device); out: width * height RGBA8 (device).
template <int D>
void launch_splat(cudaStream_t st, int n, const float4* pt, const SplatParams& S, uint32_t* winner,
                  const float* palette, int ncolors, uint8_t* out);

// ---- device-side edits (k_edit.cu) ----
// flag[i] = particle i inside the cursor; *count += the number inside.
template <int D>
void launch_cursor_mark(cudaStream_t st, int n, const float4* pt, const CursorDev& cu, uint32_t* flag,
                        unsigned long long* count);
// Flagged particles move by (dx, dy, dz) (FP64), then wrap or clamp.
template <int D>
void launch_cursor_move(cudaStream_t st, int n, float4* pt, const uint32_t* flag, double dx, double dy, double dz,
                        int wrap);
void launch_invert(cudaStream_t st, int n, uint32_t* flag);
// b[off[i]] = a[i] for every i with off[i + 1] > off[i].
template <int D>
void launch_compact(cudaStream_t st, int n, const uint32_t* off, StateBuf<D> a, StateBuf<D> b);
// b[k] = a[src[k]] for k < n (src on the device, values in [0, n_old)).
template <int D>
void launch_permute(cudaStream_t st, int n, const int32_t* src, int n_old, StateBuf<D> a, StateBuf<D> b,
                    uint32_t* status);
template <int D>
void launch_set_types(cudaStream_t st, int n, const int32_t* type, int ntypes, float4* pt, uint32_t* status);

// Batched worlds: copies surviving worlds to their new places,
// b[s] = a[old_off[k] + s - new_off[k]] for new_off[k] <= s < new_off[k + 1]
// (k < nw; new_off has nw + 1 entries).
template <int D>
void launch_batch_move(cudaStream_t st, int n, const int* new_off, const int* old_off, int nw, StateBuf<D> a,
                       StateBuf<D> b);

// Batched worlds: cell and count of every particle in slots [0, n) with its
// world's grid (worlds[k].cell_base + cell), for the next sort.
template <int D>
void launch_batch_rebin(cudaStream_t st, int n, StateBuf<D> a, const ForceParams* worlds, const int* wp_off, int nw,
                        uint32_t* cell, uint32_t* counts);

template <int D>
void launch_rebin(cudaStream_t st, int n, StateBuf<D> a, uint32_t* cell, uint32_t* counts, Grid g,
                  uint32_t cell_base = 0);

template <int D>
void launch_download(cudaStream_t st, int n, StateBuf<D> a, double* pos, double* vel, int32_t* type,
                     int32_t* id);

int scan_blocks(int ncells);
// state: (scan_blocks + 1) words, zeroed before each launch; *zero_word is
// set to 0 (the step's deferred-target count) when not null.  after: a
// programmatic dependent of the kernel before it in `st` (the force kernel
// of the step before, which releases its dependents once all its blocks
// run); its blocks wait for that kernel before reading anything it wrote.
void launch_scan(cudaStream_t st, const uint32_t* counts, int ncells, uint32_t* cstart, unsigned long long* state,
                 uint32_t* status, uint32_t* zero_word, bool after = false);
// perm[cstart[cell[i]] + r] = i with a rank r taken from counts[cell[i]]
// (bin_take), which leaves counts at zero for the next counting pass.
// slot_cell (may be null): receives the cell of each sorted slot.
// zero_state (may be null): nzero words the scan before it used (its tile
// counter and look-back flags), set back to zero for the next step's scan.
// A programmatic dependent of the scan (launch_after).
void launch_scatter(cudaStream_t st, int n, const uint32_t* cell, uint32_t* counts, const uint32_t* cstart,
                    uint32_t* perm, uint32_t* slot_cell = nullptr, unsigned long long* zero_state = nullptr,
                    int nzero = 0);

template <int D>
void launch_gather(cudaStream_t st, int n, const uint32_t* perm, const uint32_t* slot_cell, const uint32_t* cstart,
                   StateBuf<D> a, StateBuf<D> b, int32_t* cell_sorted);

// slot_cell: the cell of each slot of b, as the scatter wrote it.
// `defer`: one word, zeroed before the step; counts the targets the tiled
// kernel recomputed in its deferred pass.
// variant: tile variant of the force kernel (0 or 1, the autotuner's knob).
// snap (tiled kernel only, not with dbg; may be null): also write the new
// state to these arrays (see HostSnap).
template <int D>
void launch_force(cudaStream_t st, const ForceParams& p, bool general, StateBuf<D> b, const uint32_t* cstart,
                  const uint32_t* slot_cell, StateBuf<D> a, uint32_t* cell, uint32_t* counts, uint32_t* defer,
                  const DebugOut* dbg, int variant = 0, const HostSnap* snap = nullptr);

// Batched worlds: `worlds` (device, nworlds entries) holds each world's
// parameters with its cell_base and p_off; `wp_off` (device, nworlds + 1)
// the first sorted slot of each world and the total; `tile_off` (device,
// nworlds + 1) the first tile of each world for this variant's tile size
// (tile_targets), `tiles` the total.  Every world has nx >= 3.
// smem_matrix: every world has at most 16 types.
// steps_left (device, per world, may be null): a world at <= 0 is frozen
// for the step (its state and order untouched, its cells counted again).
// wcycles (device, per world, may be null): each block adds its duration in
// SM cycles to its world's entry (the per-world autotuner).
template <int D>
void launch_force_batch(cudaStream_t st, const ForceParams* worlds, const int* wp_off, const int* tile_off,
                        const int* steps_left, int tiles, int nworlds, int n_total, bool smem_matrix, StateBuf<D> b,
                        const uint32_t* cstart, const uint32_t* slot_cell, StateBuf<D> a, uint32_t* cell,
                        uint32_t* counts, uint32_t* defer, const DebugOut* dbg, int variant = 0,
                        unsigned long long* wcycles = nullptr);

// Resident blocks per SM of the batched force kernel of a tile variant.
int batch_blocks_per_sm(int dim, int variant, bool smem_matrix);

// Counts every positive steps_left[k] (k < nworlds) down by one.
void launch_batch_tick(cudaStream_t st, int* steps_left, int nworlds);

// The autotuners' choice: the fastest variant `best` replaces the current
// one only when it is at least 2% faster, so timing noise between nearly
// equal variants does not flip the choice.
inline int switch_if_faster(int current, int best, const double* ms_per_step) {
    return ms_per_step[best] < 0.98 * ms_per_step[current] ? best : current;
}

// Targets per block of the force kernel's tile variant.
int tile_targets(int dim, int variant);

// Opts the tiled force kernel in to its dynamic shared memory (> 48 KB) on
// the current device; called once per context.
cudaError_t force_kernels_init();

cudaError_t probe_fp32_peak(double* tflops);
cudaError_t probe_sfu_peak(double* gops);

}  // namespace plg
