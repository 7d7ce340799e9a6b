// plgpu.cu — host side of the C ABI declared in include/plgpu.h.
//
// Owns one world per context: device buffers, the exact cell table, the
// force-kernel parameters derived from PhysicsSettings, and a CUDA graph of
// one step.  See plg_internal.cuh for the device data layout.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "plg_host.h"
#include "plg_internal.cuh"
#include "plgpu.h"

using namespace plg;

namespace plg {

int grid_n(double rmax) { return (int)std::floor(1 / rmax); }

// (int)((double)x/cs) >= k  <=>  (double)x/cs >= k.
void build_bounds(double cs, int nx, float* b) {
    b[0] = 0.f;
    for (int k = 1; k <= nx; ++k) {
        float f = (float)(k * cs);
        while (!((double)f / cs >= (double)k)) f = std::nextafter(f, INFINITY);
        for (;;) {
            const float g = std::nextafter(f, -INFINITY);
            if (g < 0.f || !((double)g / cs >= (double)k)) break;
            f = g;
        }
        b[k] = f;
    }
}

void fill_force_params(const plg_settings& s, int nx, int64_t ncells, int ntypes, float b_nx, ForceParams& p) {
    p.g.nx = nx;
    p.g.ncells = (int)ncells;
    p.g.inv_cs = (float)(1.0 / s.rmax);
    p.g.b_nx = b_nx;
    p.wrap = s.wrap ? 1 : 0;
    p.ntypes = ntypes;
    p.slmask_ok = nx >= 4 ? 1 : 0;
    const double r2 = s.rmax * s.rmax;
    const double lo_d = r2 * (1.0 - kBandRel), hi_d = r2 * (1.0 + kBandRel);
    float lo = (float)lo_d, hi = (float)hi_d;
    if ((double)lo > lo_d) lo = std::nextafter(lo, 0.f);
    if ((double)hi < hi_d) hi = std::nextafter(hi, INFINITY);
    p.lo = lo;
    p.hi = hi;
    p.tiny = std::ldexp(1.0f, -100);
    p.inv_rmax = (float)(1.0 / s.rmax);
    p.beta = (float)s.beta;
    p.inv_beta = (float)(1.0 / s.beta);
    p.one_plus_beta = (float)(1.0 + s.beta);
    p.inv_one_minus_beta = (float)(1.0 / (1.0 - s.beta));
    p.m2_inv_rmax = (float)(-2.0 / s.rmax);
    p.beta_rmax = (float)(s.beta * s.rmax);
    p.k1 = (float)(1.0 / (s.beta * s.rmax));
    p.ff = (float)std::pow(s.friction, 60 * s.dt);
    p.scale = (float)(s.rmax * s.force * s.dt);
    p.dt = (float)s.dt;
    p.rmax = s.rmax;
    p.rmax2 = r2;
    p.beta_d = s.beta;
}

}  // namespace plg

namespace {

constexpr int kRing = 4;  // steps in flight per plg_step call

const char* kKernelNames[PLG_K_COUNT] = {"scan", "scatter", "gather", "force"};

// Staging layout for host <-> device copies: pos[3n] vel[3n] (double), type[n] id[n] (int32).
// Staging rows are padded to an even particle count so that every array
// starts on a 16-byte boundary (the conversion kernels use 16-byte accesses).
size_t stage_rows(int64_t cap) { return ((size_t)cap + 1) & ~(size_t)1; }
size_t stage_bytes(int64_t cap) { return stage_rows(cap) * (3 * 8 + 3 * 8 + 4 + 4); }

// Device address of a page-locked host buffer (cudaHostAlloc / cudaMallocHost
// / cudaHostRegister), or null for pageable memory.  The conversion kernels
// read and write page-locked buffers in place over the host link instead of
// staging them through device memory with separate copies.
template <typename T>
T* host_mapped(T* p) {
    if (!p) return nullptr;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
    return static_cast<T*>(a.devicePointer);
}

// The address a kernel writes host array p through: the device alias of
// page-locked memory, or p itself when it is pageable and the device
// accesses pageable memory coherently.  False: neither (p != NULL).
template <typename T>
bool kernel_writable(T* p, bool pageable, T** out) {
    *out = nullptr;
    if (!p) return true;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeHost && a.devicePointer) {
        *out = static_cast<T*>(a.devicePointer);
        return true;
    }
    if (a.type == cudaMemoryTypeUnregistered && pageable) {
        *out = p;
        return true;
    }
    return false;
}

}  // namespace

struct plg_ctx {
    int dim = 2;
    int64_t cap = 0;
    int64_t n = 0;
    int64_t next_id = 0;  // id of the next particle added (plg_append)
    int device = 0;
    bool pageable = false;  // the device accesses pageable host memory coherently
    cudaStream_t stream = nullptr;

    plg_settings s{};
    bool have_settings = false;
    bool have_matrix = false;
    bool state_valid = false;  // an upload succeeded
    bool bins_dirty = false;   // cell/counts must be recomputed from A

    // grid
    int nx = 0;
    int ncells = 0;
    int nparts = 0;
    std::vector<float> bounds_h;
    float* bounds = nullptr;
    int64_t bounds_cap = 0;
    uint32_t* counts = nullptr;
    uint32_t* cstart = nullptr;
    int64_t cells_cap = 0;
    int64_t cstart_cap = 0;
    unsigned long long* scan_state = nullptr;  // tile counter + look-back status words
    int64_t scan_cap = 0;

    // matrix
    int ntypes = 0;
    float* matrix = nullptr;
    int64_t matrix_cap = 0;

    // particles (A = current order, B = cell-sorted)
    float4* apt = nullptr;
    float4* bpt = nullptr;
    void* avel = nullptr;
    void* bvel = nullptr;
    uint32_t* cell = nullptr;
    uint32_t* perm = nullptr;
    uint32_t* slot_cell = nullptr;  // cell of each sorted slot (scatter -> gather)
    uint32_t* defer = nullptr;  // targets the force kernel deferred in the last step
    unsigned char* stage = nullptr;

    uint32_t* status_d = nullptr;
    uint32_t* status_h = nullptr;

    // device-side edits (allocated on first use)
    uint32_t* edit_flag = nullptr;       // cap: marks / host indices / types
    uint32_t* edit_off = nullptr;        // cap + 1: exclusive scan of the marks
    unsigned long long* edit_scan = nullptr;
    unsigned long long* edit_cnt = nullptr;
    int64_t edit_cap = 0, edit_scan_cap = 0;

    // instrumented step
    int32_t* dbg_pairs = nullptr;
    unsigned long long* dbg_hsum = nullptr;
    unsigned long long* dbg_hxor = nullptr;
    unsigned long long* dbg_cand = nullptr;
    float* dbg_acc = nullptr;
    int32_t* dbg_cell = nullptr;

    // graph of one step
    bool use_graph = true;
    int variant = 0;            // force kernel tile variant (plg_set_tile / plg_autotune)
    bool variant_auto = true;   // neither has been called: the variant follows the size (tile_variant)
    cudaGraphExec_t gexec = nullptr;
    bool graph_dirty = true;

    // profiling
    bool profiling = false;
    cudaEvent_t pev[PLG_K_COUNT][2] = {};
    double prof_ms[PLG_K_COUNT] = {};
    int64_t prof_n[PLG_K_COUNT] = {};

    cudaEvent_t ring[kRing] = {};
    int ring_pos = 0;
    int ring_fill = 0;

    std::atomic<int> stop{0};
    std::string err;
    ForceParams fp{};
    bool general = false;
};

namespace {

int set_err(plg_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}

int cuda_fail(plg_ctx* c, const char* what, cudaError_t e) {
    cudaGetLastError();  // clear a non-sticky error
    return set_err(c, PLG_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(ctx, call)                                          \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess) return cuda_fail(ctx, #call, e_); \
    } while (0)

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int d) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != d) cudaSetDevice(d);
    }
    ~DeviceGuard() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

template <typename T>
int grow(plg_ctx* c, T** p, int64_t* cap, int64_t need, const char* what) {
    if (*p && *cap >= need) return PLG_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    cudaError_t e = cudaMalloc((void**)p, sizeof(T) * (size_t)(need > 0 ? need : 1));
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return set_err(c, PLG_E_NO_MEMORY, std::string("cudaMalloc ") + what + ": " + cudaGetErrorString(e));
    }
    *cap = need;
    return PLG_OK;
}

void destroy_graph(plg_ctx* c) {
    if (c->gexec) cudaGraphExecDestroy(c->gexec);
    c->gexec = nullptr;
    c->graph_dirty = true;
}

template <int D>
StateBuf<D> buf_a(plg_ctx* c) {
    return StateBuf<D>{c->apt, (typename Layout<D>::Vel*)c->avel};
}
template <int D>
StateBuf<D> buf_b(plg_ctx* c) {
    return StateBuf<D>{c->bpt, (typename Layout<D>::Vel*)c->bvel};
}

void compute_force_params(plg_ctx* c) {
    ForceParams& p = c->fp;
    fill_force_params(c->s, c->nx, c->ncells, c->ntypes, c->bounds_h[c->nx], p);
    p.g.bounds = c->bounds;
    p.n = (int)c->n;
    p.matrix = c->matrix;
    p.cell_base = 0;
    p.p_off = 0;
    c->general = c->nx < 3;
}

Grid grid_of(plg_ctx* c) { return c->fp.g; }

// 2D worlds below this many particles default to tile variant 2 (128
// targets per block): with the 256-target variant 0 they fill fewer than
// two waves of blocks (10k particles: 20.7 against 25.0 us per step).
constexpr int64_t kSmallWorld2D = 300000;

// The tile variant a step uses: the one set or tuned, else by size.
int tile_variant(const plg_ctx* c) {
    if (!c->variant_auto) return c->variant;
    return c->dim == 2 && c->n < kSmallWorld2D ? 2 : 0;
}

// Enqueues the body of one step (no rebin) on c->stream.
// snap (may be null): snapshot arrays the force kernel also writes.
template <int D>
void enqueue_body(plg_ctx* c, const DebugOut* dbg, int32_t* cell_sorted, const HostSnap* snap = nullptr) {
    cudaStream_t st = c->stream;
    const int n = (int)c->n;
    auto k0 = [&](int k) {
        if (c->profiling) cudaEventRecord(c->pev[k][0], st);
    };
    auto k1 = [&](int k) {
        if (c->profiling) cudaEventRecord(c->pev[k][1], st);
    };
    // The scan's state (tile counter, look-back flags) starts at zero: the
    // scatter sets it back after each scan; with no particles there is no
    // scatter, and a memset does it.
    const int nstate = c->nparts + 1;
    k0(PLG_K_SCAN);
    launch_scan(st, c->counts, c->ncells, c->cstart, c->scan_state, c->status_d, c->general ? nullptr : c->defer,
                !c->profiling);
    k1(PLG_K_SCAN);
    k0(PLG_K_SCATTER);
    if (n > 0)
        launch_scatter(st, n, c->cell, c->counts, c->cstart, c->perm, c->slot_cell, c->scan_state, nstate);
    else
        cudaMemsetAsync(c->scan_state, 0, sizeof(unsigned long long) * (size_t)nstate, st);
    k1(PLG_K_SCATTER);
    k0(PLG_K_GATHER);
    launch_gather<D>(st, n, c->perm, c->slot_cell, c->cstart, buf_a<D>(c), buf_b<D>(c), cell_sorted);
    k1(PLG_K_GATHER);
    k0(PLG_K_FORCE);
    launch_force<D>(st, c->fp, c->general, buf_b<D>(c), c->cstart, c->slot_cell, buf_a<D>(c), c->cell, c->counts,
                    c->defer, dbg, tile_variant(c), snap);
    k1(PLG_K_FORCE);
}

void enqueue_body_dim(plg_ctx* c, const DebugOut* dbg, int32_t* cell_sorted, const HostSnap* snap = nullptr) {
    if (c->dim == 2)
        enqueue_body<2>(c, dbg, cell_sorted, snap);
    else
        enqueue_body<3>(c, dbg, cell_sorted, snap);
}

// True when the force kernel can write the snapshot arrays itself (the
// tiled kernel runs and every non-null array is kernel-writable); fills hs.
bool snapshot_fusable(plg_ctx* c, double* pos, double* vel, int32_t* type, int32_t* id, HostSnap* hs) {
    return !c->general && c->n > 0 && kernel_writable(pos, c->pageable, &hs->pos) &&
           kernel_writable(vel, c->pageable, &hs->vel) && kernel_writable(type, c->pageable, &hs->type) &&
           kernel_writable(id, c->pageable, &hs->id);
}

int enqueue_rebin(plg_ctx* c) {
    if (!c->bins_dirty) return PLG_OK;
    CK(c, cudaMemsetAsync(c->counts, 0, sizeof(uint32_t) * (size_t)c->ncells, c->stream));
    if (c->dim == 2)
        launch_rebin<2>(c->stream, (int)c->n, buf_a<2>(c), c->cell, c->counts, grid_of(c));
    else
        launch_rebin<3>(c->stream, (int)c->n, buf_a<3>(c), c->cell, c->counts, grid_of(c));
    CK(c, cudaGetLastError());
    c->bins_dirty = false;
    return PLG_OK;
}

int accumulate_profile(plg_ctx* c) {
    CK(c, cudaEventSynchronize(c->pev[PLG_K_COUNT - 1][1]));  // the step's last kernel
    for (int k = 0; k < PLG_K_COUNT; ++k) {
        float ms = 0.f;
        CK(c, cudaEventElapsedTime(&ms, c->pev[k][0], c->pev[k][1]));
        c->prof_ms[k] += ms;
        c->prof_n[k] += 1;
    }
    return PLG_OK;
}

int enqueue_step(plg_ctx* c) {
    int rc = enqueue_rebin(c);
    if (rc) return rc;
    if (c->profiling) {
        enqueue_body_dim(c, nullptr, nullptr);
        CK(c, cudaGetLastError());
        return accumulate_profile(c);
    }
    if (!c->use_graph) {
        enqueue_body_dim(c, nullptr, nullptr);
        CK(c, cudaGetLastError());
        return PLG_OK;
    }
    if (c->graph_dirty || !c->gexec) {
        destroy_graph(c);
        cudaGraph_t g = nullptr;
        CK(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        enqueue_body_dim(c, nullptr, nullptr);
        cudaError_t e = cudaStreamEndCapture(c->stream, &g);
        if (e != cudaSuccess) return cuda_fail(c, "cudaStreamEndCapture", e);
        e = cudaGraphInstantiate(&c->gexec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            c->gexec = nullptr;
            return cuda_fail(c, "cudaGraphInstantiate", e);
        }
        c->graph_dirty = false;
    }
    CK(c, cudaGraphLaunch(c->gexec, c->stream));
    return PLG_OK;
}

int check_ready(plg_ctx* c) {
    if (!c) return PLG_E_INVALID_ARG;
    if (!c->have_settings) return set_err(c, PLG_E_STATE, "plg_set_settings has not been called");
    if (!c->have_matrix) return set_err(c, PLG_E_STATE, "plg_set_matrix has not been called");
    if (!c->state_valid) return set_err(c, PLG_E_STATE, "no valid particle state: call plg_upload");
    return PLG_OK;
}

int wait_stream(plg_ctx* c, double timeout_s) {
    if (timeout_s <= 0) {
        CK(c, cudaStreamSynchronize(c->stream));
    } else {
        const auto t0 = std::chrono::steady_clock::now();
        for (;;) {
            cudaError_t e = cudaStreamQuery(c->stream);
            if (e == cudaSuccess) break;
            if (e != cudaErrorNotReady) return cuda_fail(c, "cudaStreamQuery", e);
            const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            if (el > timeout_s) return set_err(c, PLG_E_TIMEOUT, "device work did not finish within the timeout");
            std::this_thread::sleep_for(std::chrono::microseconds(50));
        }
    }
    c->ring_fill = 0;
    return PLG_OK;
}

int read_status(plg_ctx* c) {
    CK(c, cudaMemcpyAsync(c->status_h, c->status_d, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    const uint32_t st = *c->status_h;
    if (st == 0) return PLG_OK;
    std::string m = "device reported:";
    if (st & kDevBadPosition) m += " position outside [0,1] or not finite;";
    if (st & kDevBadType) m += " type outside [0, matrix size);";
    if (st & kDevBadVelocity) m += " velocity not finite;";
    if (st & kDevSpinLimit) m += " bounded wait ran out;";
    CK(c, cudaMemsetAsync(c->status_d, 0, sizeof(uint32_t), c->stream));
    return set_err(c, (st & (kDevBadPosition | kDevBadType | kDevBadVelocity)) ? PLG_E_INVALID_ARG : PLG_E_DEVICE, m);
}

int free_all(plg_ctx* c) {
    destroy_graph(c);
    void* ptrs[] = {c->bounds,    c->counts,   c->cstart,   c->scan_state, c->matrix,   c->apt,
                    c->bpt,       c->avel,     c->bvel,     c->cell,       c->perm,
                    c->slot_cell, c->defer,    c->stage,    c->status_d,   c->dbg_pairs, c->dbg_hsum,
                    c->dbg_hxor,  c->dbg_cand, c->dbg_acc,  c->dbg_cell, c->edit_flag, c->edit_off,
                    c->edit_scan, c->edit_cnt};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (c->status_h) cudaFreeHost(c->status_h);
    for (int k = 0; k < PLG_K_COUNT; ++k)
        for (int j = 0; j < 2; ++j)
            if (c->pev[k][j]) cudaEventDestroy(c->pev[k][j]);
    for (int k = 0; k < kRing; ++k)
        if (c->ring[k]) cudaEventDestroy(c->ring[k]);
    if (c->stream) cudaStreamDestroy(c->stream);
    return PLG_OK;
}

}  // namespace

extern "C" {

const char* plg_version(void) { return "plgpu 0.1.0 (sm_103a, ABI 1)"; }

const char* plg_status_string(int status) {
    switch (status) {
        case PLG_OK: return "ok";
        case PLG_E_INVALID_ARG: return "invalid argument";
        case PLG_E_UNSUPPORTED: return "unsupported";
        case PLG_E_STATE: return "invalid call order";
        case PLG_E_NO_MEMORY: return "out of memory";
        case PLG_E_CUDA: return "CUDA error";
        case PLG_E_TIMEOUT: return "timeout";
        case PLG_E_STOPPED: return "stopped";
        case PLG_E_DEVICE: return "device error";
        case PLG_E_CAPACITY: return "capacity exceeded";
        default: return "unknown status";
    }
}

int plg_validate_settings(int dim, const plg_settings* s) {
    if (dim != 2 && dim != 3) return PLG_E_INVALID_ARG;
    if (!s) return PLG_E_INVALID_ARG;
    if (s->accel_kind != PLG_ACCEL_PARTICLE_LIFE) return PLG_E_UNSUPPORTED;
    if (!(std::isfinite(s->rmax) && s->rmax > 0 && s->rmax <= 1)) return PLG_E_INVALID_ARG;
    const int nx = grid_n(s->rmax);
    if (nx < 1 || nx > kMaxAxisCells) return PLG_E_INVALID_ARG;
    int64_t cells = (int64_t)nx * nx;
    if (dim == 3) cells *= nx;
    if (cells > kMaxCells) return PLG_E_INVALID_ARG;
    if (!(std::isfinite(s->friction) && s->friction >= 0)) return PLG_E_INVALID_ARG;
    if (!std::isfinite(s->force) || !std::isfinite(s->dt)) return PLG_E_INVALID_ARG;
    if (!(std::isfinite(s->beta) && s->beta > 0 && s->beta < 1)) return PLG_E_INVALID_ARG;
    if (s->wrap != 0 && s->wrap != 1) return PLG_E_INVALID_ARG;
    return PLG_OK;
}

int plg_cell_bounds(double rmax, int32_t* nx_out, float* bounds, int64_t cap) {
    if (!(std::isfinite(rmax) && rmax > 0 && rmax <= 1)) return PLG_E_INVALID_ARG;
    const int nx = grid_n(rmax);
    if (nx < 1 || nx > kMaxAxisCells) return PLG_E_INVALID_ARG;
    if (nx_out) *nx_out = nx;
    if (bounds) {
        if (cap < (int64_t)nx + 1) return PLG_E_INVALID_ARG;
        build_bounds(rmax, nx, bounds);
    }
    return PLG_OK;
}

int plg_create(int dim, int64_t capacity, plg_ctx** out) {
    if (!out) return PLG_E_INVALID_ARG;
    *out = nullptr;
    if ((dim != 2 && dim != 3) || capacity < 1 || capacity > kMaxParticles) return PLG_E_INVALID_ARG;
    plg_ctx* c = new (std::nothrow) plg_ctx();
    if (!c) return PLG_E_NO_MEMORY;
    c->dim = dim;
    c->cap = capacity;
    cudaError_t e = cudaGetDevice(&c->device);
    int pageable = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, c->device);
    if (e != cudaSuccess) {
        cudaGetLastError();
        delete c;
        return PLG_E_CUDA;
    }
    c->pageable = pageable != 0;
    int rc = PLG_OK;
    const size_t vel_sz = dim == 2 ? sizeof(float2) : sizeof(float4);
    auto dmalloc = [&](void** p, size_t bytes) {
        if (rc) return;
        cudaError_t err = cudaMalloc(p, bytes);
        if (err != cudaSuccess) {
            cudaGetLastError();
            *p = nullptr;
            rc = err == cudaErrorMemoryAllocation ? PLG_E_NO_MEMORY : PLG_E_CUDA;
        }
    };
    const size_t cap = (size_t)capacity;
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) rc = PLG_E_CUDA;
    if (!rc && force_kernels_init() != cudaSuccess) rc = PLG_E_CUDA;
    dmalloc((void**)&c->apt, sizeof(float4) * cap);
    dmalloc((void**)&c->bpt, sizeof(float4) * cap);
    dmalloc(&c->avel, vel_sz * cap);
    dmalloc(&c->bvel, vel_sz * cap);
    dmalloc((void**)&c->cell, sizeof(uint32_t) * cap);
    dmalloc((void**)&c->perm, sizeof(uint32_t) * cap);
    dmalloc((void**)&c->slot_cell, sizeof(uint32_t) * cap);
    dmalloc((void**)&c->defer, sizeof(uint32_t));
    dmalloc((void**)&c->stage, stage_bytes(capacity));
    dmalloc((void**)&c->status_d, 64);
    if (!rc && cudaMallocHost((void**)&c->status_h, 64) != cudaSuccess) rc = PLG_E_NO_MEMORY;
    for (int k = 0; k < kRing && !rc; ++k)
        if (cudaEventCreateWithFlags(&c->ring[k], cudaEventDisableTiming) != cudaSuccess) rc = PLG_E_CUDA;
    if (!rc && cudaMemset(c->status_d, 0, 64) != cudaSuccess) rc = PLG_E_CUDA;
    if (rc) {
        cudaGetLastError();
        free_all(c);
        delete c;
        return rc;
    }
    *out = c;
    return PLG_OK;
}

int plg_destroy(plg_ctx* c) {
    if (!c) return PLG_E_INVALID_ARG;
    {
        DeviceGuard g(c->device);
        if (c->stream) cudaStreamSynchronize(c->stream);
        free_all(c);
    }
    delete c;
    return PLG_OK;
}

int plg_set_settings(plg_ctx* c, const plg_settings* s) {
    if (!c || !s) return PLG_E_INVALID_ARG;
    int rc = plg_validate_settings(c->dim, s);
    if (rc == PLG_E_UNSUPPORTED)
        return set_err(c, rc, "only PLG_ACCEL_PARTICLE_LIFE has a device implementation (no CPU fallback)");
    if (rc) return set_err(c, rc, "settings out of the supported range");
    DeviceGuard g(c->device);
    const bool grid_change = !c->have_settings || c->s.rmax != s->rmax;
    if (grid_change) {
        const int nx = grid_n(s->rmax);
        int64_t cells = (int64_t)nx * nx * (c->dim == 3 ? nx : 1);
        CK(c, cudaStreamSynchronize(c->stream));
        if ((rc = grow(c, &c->bounds, &c->bounds_cap, (int64_t)nx + 1, "bounds"))) return rc;
        if ((rc = grow(c, &c->counts, &c->cells_cap, cells, "counts"))) return rc;
        if ((rc = grow(c, &c->cstart, &c->cstart_cap, cells + 1, "cstart"))) return rc;
        const int nparts = scan_blocks((int)cells);
        if ((rc = grow(c, &c->scan_state, &c->scan_cap, (int64_t)nparts + 1, "scan state"))) return rc;
        // Zero before the first scan on this grid; each step's scatter
        // zeroes it again after the scan.
        CK(c, cudaMemset(c->scan_state, 0, sizeof(unsigned long long) * (size_t)(nparts + 1)));
        c->nx = nx;
        c->ncells = (int)cells;
        c->nparts = nparts;
        c->bounds_h.assign((size_t)nx + 1, 0.f);
        build_bounds(s->rmax, nx, c->bounds_h.data());
        CK(c, cudaMemcpy(c->bounds, c->bounds_h.data(), sizeof(float) * (size_t)(nx + 1), cudaMemcpyHostToDevice));
        CK(c, cudaMemset(c->counts, 0, sizeof(uint32_t) * (size_t)cells));
        if (c->state_valid) c->bins_dirty = true;
    }
    c->s = *s;
    c->have_settings = true;
    compute_force_params(c);
    c->graph_dirty = true;
    return PLG_OK;
}

int plg_get_settings(plg_ctx* c, plg_settings* out) {
    if (!c || !out) return PLG_E_INVALID_ARG;
    if (!c->have_settings) return set_err(c, PLG_E_STATE, "plg_set_settings has not been called");
    *out = c->s;
    return PLG_OK;
}

int plg_set_matrix(plg_ctx* c, int32_t n, const double* m) {
    if (!c || !m || n < 1 || n > kMaxTypes) return set_err(c, PLG_E_INVALID_ARG, "matrix size must be 1..1024");
    std::vector<float> f((size_t)n * n);
    for (size_t k = 0; k < f.size(); ++k) {
        if (!std::isfinite(m[k])) return set_err(c, PLG_E_INVALID_ARG, "matrix entries must be finite");
        f[k] = (float)m[k];
    }
    DeviceGuard g(c->device);
    int rc;
    CK(c, cudaStreamSynchronize(c->stream));
    if ((rc = grow(c, &c->matrix, &c->matrix_cap, (int64_t)n * n, "matrix"))) return rc;
    CK(c, cudaMemcpy(c->matrix, f.data(), sizeof(float) * f.size(), cudaMemcpyHostToDevice));
    if (c->ntypes != n || !c->have_matrix) c->graph_dirty = true;
    if (c->have_matrix && n < c->ntypes && c->state_valid) {
        // Types >= n would index outside the matrix: the caller must re-type
        // first (Physics.setMatrixSize -> ensureTypes, Physics.java:238-272).
        c->state_valid = false;
        c->ntypes = n;
        c->have_matrix = true;
        if (c->have_settings) compute_force_params(c);
        return set_err(c, PLG_E_STATE, "matrix shrank below the uploaded types: re-upload with ensured types");
    }
    c->ntypes = n;
    c->have_matrix = true;
    if (c->have_settings) compute_force_params(c);
    c->graph_dirty = true;
    return PLG_OK;
}

int plg_upload(plg_ctx* c, int64_t n, const double* pos, const double* vel, const int32_t* type) {
    const TraceRange tr("plg_upload");
    if (!c) return PLG_E_INVALID_ARG;
    if (n < 0) return set_err(c, PLG_E_INVALID_ARG, "negative particle count");
    if (n > c->cap) return set_err(c, PLG_E_CAPACITY, "more particles than the context capacity");
    if (n > 0 && (!pos || !type)) return set_err(c, PLG_E_INVALID_ARG, "pos and type must not be NULL");
    if (!c->have_settings) return set_err(c, PLG_E_STATE, "plg_set_settings has not been called");
    if (!c->have_matrix) return set_err(c, PLG_E_STATE, "plg_set_matrix has not been called");
    DeviceGuard g(c->device);
    cudaStream_t st = c->stream;
    double* dpos = (double*)c->stage;
    double* dvel = dpos + 3 * stage_rows(c->cap);
    int32_t* dtype = (int32_t*)(dvel + 3 * stage_rows(c->cap));
    c->state_valid = false;
    if (n > 0) {
        // Page-locked arrays are read in place by the upload kernel.
        const double* mpos = host_mapped(pos);
        const double* mvel = host_mapped(vel);
        const int32_t* mtype = host_mapped(type);
        if (mpos)
            dpos = const_cast<double*>(mpos);
        else
            CK(c, cudaMemcpyAsync(dpos, pos, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice, st));
        if (mvel)
            dvel = const_cast<double*>(mvel);
        else if (vel)
            CK(c, cudaMemcpyAsync(dvel, vel, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice, st));
        if (mtype)
            dtype = const_cast<int32_t*>(mtype);
        else
            CK(c, cudaMemcpyAsync(dtype, type, sizeof(int32_t) * (size_t)n, cudaMemcpyHostToDevice, st));
    }
    CK(c, cudaMemsetAsync(c->counts, 0, sizeof(uint32_t) * (size_t)c->ncells, st));
    CK(c, cudaMemsetAsync(c->status_d, 0, sizeof(uint32_t), st));
    if (c->dim == 2)
        launch_upload<2>(st, (int)n, dpos, vel ? dvel : nullptr, dtype, c->ntypes, buf_a<2>(c), c->cell, c->counts,
                         grid_of(c), c->status_d);
    else
        launch_upload<3>(st, (int)n, dpos, vel ? dvel : nullptr, dtype, c->ntypes, buf_a<3>(c), c->cell, c->counts,
                         grid_of(c), c->status_d);
    CK(c, cudaGetLastError());
    int rc = read_status(c);
    if (rc) return rc;
    if (c->n != n) c->graph_dirty = true;
    c->n = n;
    c->next_id = n;
    c->fp.n = (int)n;
    c->bins_dirty = false;
    c->state_valid = true;
    return PLG_OK;
}

int plg_step_async(plg_ctx* c, int32_t nsteps) {
    int rc = check_ready(c);
    if (rc) return rc;
    if (nsteps < 0) return set_err(c, PLG_E_INVALID_ARG, "negative step count");
    DeviceGuard g(c->device);
    for (int32_t k = 0; k < nsteps; ++k) {
        if (c->stop.exchange(0)) return set_err(c, PLG_E_STOPPED, "stopped by plg_request_stop");
        if (c->ring_fill == kRing) {
            CK(c, cudaEventSynchronize(c->ring[c->ring_pos]));
            c->ring_fill--;
        }
        if ((rc = enqueue_step(c))) return rc;
        CK(c, cudaEventRecord(c->ring[c->ring_pos], c->stream));
        c->ring_pos = (c->ring_pos + 1) % kRing;
        c->ring_fill++;
    }
    return PLG_OK;
}

int plg_sync(plg_ctx* c, double timeout_s) {
    if (!c) return PLG_E_INVALID_ARG;
    DeviceGuard g(c->device);
    if (timeout_s <= 0) {
        // The status copy is ordered after all enqueued work, and
        // read_status synchronizes the stream: one wait instead of two.
        c->ring_fill = 0;
        return read_status(c);
    }
    int rc = wait_stream(c, timeout_s);
    if (rc) return rc;
    return read_status(c);
}

int plg_step(plg_ctx* c, int32_t nsteps) {
    const TraceRange tr("plg_step");
    int rc = plg_step_async(c, nsteps);
    if (rc == PLG_E_STOPPED) {
        std::string m = c->err;
        int r2 = plg_sync(c, 0);
        if (r2) return r2;
        c->err = m;
        return rc;
    }
    if (rc) return rc;
    return plg_sync(c, 0);
}

int plg_download(plg_ctx* c, double* pos, double* vel, int32_t* type, int32_t* id) {
    const TraceRange tr("plg_download");
    if (!c) return PLG_E_INVALID_ARG;
    if (!c->state_valid) return set_err(c, PLG_E_STATE, "no valid particle state: call plg_upload");
    DeviceGuard g(c->device);
    cudaStream_t st = c->stream;
    const size_t n = (size_t)c->n;
    double* dpos = (double*)c->stage;
    double* dvel = dpos + 3 * stage_rows(c->cap);
    int32_t* dtype = (int32_t*)(dvel + 3 * stage_rows(c->cap));
    int32_t* did = dtype + stage_rows(c->cap);
    if (n > 0) {
        // Page-locked arrays are written in place by the download kernel;
        // the others go through the staging buffer and a copy.
        double* mpos = host_mapped(pos);
        double* mvel = host_mapped(vel);
        int32_t* mtype = host_mapped(type);
        int32_t* mid = host_mapped(id);
        double* kpos = pos ? (mpos ? mpos : dpos) : nullptr;
        double* kvel = vel ? (mvel ? mvel : dvel) : nullptr;
        int32_t* ktype = type ? (mtype ? mtype : dtype) : nullptr;
        int32_t* kid = id ? (mid ? mid : did) : nullptr;
        if (c->dim == 2)
            launch_download<2>(st, (int)n, buf_a<2>(c), kpos, kvel, ktype, kid);
        else
            launch_download<3>(st, (int)n, buf_a<3>(c), kpos, kvel, ktype, kid);
        CK(c, cudaGetLastError());
        if (pos && !mpos) CK(c, cudaMemcpyAsync(pos, dpos, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st));
        if (vel && !mvel) CK(c, cudaMemcpyAsync(vel, dvel, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st));
        if (type && !mtype) CK(c, cudaMemcpyAsync(type, dtype, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st));
        if (id && !mid) CK(c, cudaMemcpyAsync(id, did, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st));
    }
    CK(c, cudaStreamSynchronize(st));
    return PLG_OK;
}

int plg_step_download_fuses(plg_ctx* c, const double* pos, const double* vel, const int32_t* type,
                            const int32_t* id, int32_t* fused) {
    if (!c || !fused) return PLG_E_INVALID_ARG;
    int rc = check_ready(c);
    if (rc) return rc;
    DeviceGuard g(c->device);
    HostSnap hs{nullptr, nullptr, nullptr, nullptr};
    *fused = snapshot_fusable(c, const_cast<double*>(pos), const_cast<double*>(vel), const_cast<int32_t*>(type),
                              const_cast<int32_t*>(id), &hs)
                 ? 1
                 : 0;
    return PLG_OK;
}

int plg_step_download(plg_ctx* c, int32_t nsteps, double* pos, double* vel, int32_t* type, int32_t* id) {
    const TraceRange tr("plg_step_download");
    int rc = check_ready(c);
    if (rc) return rc;
    if (nsteps < 0) return set_err(c, PLG_E_INVALID_ARG, "negative step count");
    if (nsteps == 0) return plg_download(c, pos, vel, type, id);
    DeviceGuard g(c->device);
    HostSnap hs{nullptr, nullptr, nullptr, nullptr};
    if (!snapshot_fusable(c, pos, vel, type, id, &hs)) {
        if ((rc = plg_step(c, nsteps))) return rc;
        return plg_download(c, pos, vel, type, id);
    }
    auto stopped = [&]() {
        const std::string m = c->err;
        const int r2 = plg_sync(c, 0);
        if (r2) return r2;
        c->err = m;
        return (int)PLG_E_STOPPED;
    };
    rc = plg_step_async(c, nsteps - 1);
    if (rc == PLG_E_STOPPED) return stopped();
    if (rc) return rc;
    if (c->stop.exchange(0)) {
        set_err(c, PLG_E_STOPPED, "stopped by plg_request_stop");
        return stopped();
    }
    // The last step, as plain launches: its force kernel carries the
    // caller's arrays, which change from call to call.
    if ((rc = enqueue_rebin(c))) return rc;
    enqueue_body_dim(c, nullptr, nullptr, &hs);
    CK(c, cudaGetLastError());
    if (c->profiling && (rc = accumulate_profile(c))) return rc;
    return plg_sync(c, 0);
}

}  // extern "C"

namespace {

// Scratch of the device-side edits, sized to the capacity.
int edit_scratch(plg_ctx* c) {
    if (c->edit_flag) return PLG_OK;
    const size_t cap = (size_t)c->cap;
    const int blocks = scan_blocks((int)std::max<int64_t>(c->cap, 1));
    auto dm = [&](void** p, size_t bytes) -> int {
        cudaError_t e = cudaMalloc(p, bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            *p = nullptr;
            return set_err(c, PLG_E_NO_MEMORY, "cudaMalloc (edit scratch)");
        }
        return PLG_OK;
    };
    int rc;
    if ((rc = dm((void**)&c->edit_flag, sizeof(uint32_t) * (cap + 4)))) return rc;
    if ((rc = dm((void**)&c->edit_off, sizeof(uint32_t) * (cap + 4)))) return rc;
    if ((rc = dm((void**)&c->edit_scan, sizeof(unsigned long long) * (size_t)(blocks + 1)))) return rc;
    if ((rc = dm((void**)&c->edit_cnt, sizeof(unsigned long long)))) return rc;
    c->edit_scan_cap = blocks + 1;
    return PLG_OK;
}

CursorDev cursor_dev(const plg_ctx* c, const plg_cursor* k) {
    CursorDev cu;
    cu.x = k->x;
    cu.y = k->y;
    cu.z = k->z;
    cu.size = k->size;
    cu.shape = k->shape;
    cu.wrap = c->s.wrap ? 1 : 0;
    return cu;
}

int check_cursor(plg_ctx* c, const plg_cursor* k) {
    if (!k) return set_err(c, PLG_E_INVALID_ARG, "NULL cursor");
    if (k->shape < PLG_CURSOR_CIRCLE || k->shape > PLG_CURSOR_INFINITY)
        return set_err(c, PLG_E_INVALID_ARG, "unknown cursor shape");
    if (!std::isfinite(k->x) || !std::isfinite(k->y) || !std::isfinite(k->z) || !(k->size >= 0) ||
        !std::isfinite(k->size))
        return set_err(c, PLG_E_INVALID_ARG, "cursor position and size must be finite, size >= 0");
    return PLG_OK;
}

// Marks the particles inside the cursor (edit_flag) and returns how many.
int mark_cursor(plg_ctx* c, const plg_cursor* k, int64_t* count) {
    int rc = edit_scratch(c);
    if (rc) return rc;
    cudaStream_t st = c->stream;
    CK(c, cudaMemsetAsync(c->edit_cnt, 0, sizeof(unsigned long long), st));
    const CursorDev cu = cursor_dev(c, k);
    if (c->dim == 2)
        launch_cursor_mark<2>(st, (int)c->n, c->apt, cu, c->edit_flag, c->edit_cnt);
    else
        launch_cursor_mark<3>(st, (int)c->n, c->apt, cu, c->edit_flag, c->edit_cnt);
    CK(c, cudaGetLastError());
    unsigned long long h = 0;
    CK(c, cudaMemcpyAsync(&h, c->edit_cnt, sizeof(h), cudaMemcpyDeviceToHost, st));
    CK(c, cudaStreamSynchronize(st));
    *count = (int64_t)h;
    return PLG_OK;
}

// After an edit of A: the next step re-bins, and a new particle count or
// swapped buffers mean a new step graph.
void edited(plg_ctx* c, int64_t n) {
    if (n != c->n) c->graph_dirty = true;
    c->n = n;
    c->fp.n = (int)n;
    c->bins_dirty = true;
}

void swap_ab(plg_ctx* c) {
    std::swap(c->apt, c->bpt);
    std::swap(c->avel, c->bvel);
    c->graph_dirty = true;
}

}  // namespace

extern "C" {

int plg_cursor_count(plg_ctx* c, const plg_cursor* k, int64_t* count) {
    int rc = check_ready(c);
    if (rc) return rc;
    if ((rc = check_cursor(c, k))) return rc;
    if (!count) return set_err(c, PLG_E_INVALID_ARG, "NULL count");
    DeviceGuard g(c->device);
    CK(c, cudaStreamSynchronize(c->stream));
    return mark_cursor(c, k, count);
}

int plg_cursor_move(plg_ctx* c, const plg_cursor* k, double dx, double dy, double dz, int64_t* moved) {
    int rc = check_ready(c);
    if (rc) return rc;
    if ((rc = check_cursor(c, k))) return rc;
    if (!std::isfinite(dx) || !std::isfinite(dy) || !std::isfinite(dz))
        return set_err(c, PLG_E_INVALID_ARG, "displacement must be finite");
    DeviceGuard g(c->device);
    CK(c, cudaStreamSynchronize(c->stream));
    int64_t cnt = 0;
    if ((rc = mark_cursor(c, k, &cnt))) return rc;
    if (moved) *moved = cnt;
    if (cnt == 0) return PLG_OK;
    if (c->dim == 2)
        launch_cursor_move<2>(c->stream, (int)c->n, c->apt, c->edit_flag, dx, dy, c->dim == 3 ? dz : 0.0,
                              c->s.wrap ? 1 : 0);
    else
        launch_cursor_move<3>(c->stream, (int)c->n, c->apt, c->edit_flag, dx, dy, dz, c->s.wrap ? 1 : 0);
    CK(c, cudaGetLastError());
    CK(c, cudaStreamSynchronize(c->stream));
    edited(c, c->n);
    return PLG_OK;
}

int plg_cursor_delete(plg_ctx* c, const plg_cursor* k, int64_t* deleted) {
    int rc = check_ready(c);
    if (rc) return rc;
    if ((rc = check_cursor(c, k))) return rc;
    DeviceGuard g(c->device);
    CK(c, cudaStreamSynchronize(c->stream));
    int64_t cnt = 0;
    if ((rc = mark_cursor(c, k, &cnt))) return rc;
    if (deleted) *deleted = cnt;
    if (cnt == 0) return PLG_OK;
    cudaStream_t st = c->stream;
    const int n = (int)c->n;
    launch_invert(st, n, c->edit_flag);  // 1 = keep
    CK(c, cudaMemsetAsync(c->edit_scan, 0, sizeof(unsigned long long) * (size_t)(scan_blocks(n) + 1), st));
    launch_scan(st, c->edit_flag, n, c->edit_off, c->edit_scan, c->status_d, nullptr);
    if (c->dim == 2)
        launch_compact<2>(st, n, c->edit_off, buf_a<2>(c), buf_b<2>(c));
    else
        launch_compact<3>(st, n, c->edit_off, buf_a<3>(c), buf_b<3>(c));
    CK(c, cudaGetLastError());
    if ((rc = read_status(c))) return rc;
    swap_ab(c);
    edited(c, c->n - cnt);
    return PLG_OK;
}

int plg_append(plg_ctx* c, int64_t n, const double* pos, const double* vel, const int32_t* type) {
    int rc = check_ready(c);
    if (rc) return rc;
    if (n < 0) return set_err(c, PLG_E_INVALID_ARG, "negative particle count");
    if (n == 0) return PLG_OK;
    if (!pos || !type) return set_err(c, PLG_E_INVALID_ARG, "pos and type must not be NULL");
    if (c->n + n > c->cap) return set_err(c, PLG_E_CAPACITY, "more particles than the context capacity");
    if (c->next_id + n > INT32_MAX) return set_err(c, PLG_E_CAPACITY, "particle ids exhausted");
    DeviceGuard g(c->device);
    cudaStream_t st = c->stream;
    CK(c, cudaStreamSynchronize(st));
    double* dpos = (double*)c->stage;
    double* dvel = dpos + 3 * stage_rows(c->cap);
    int32_t* dtype = (int32_t*)(dvel + 3 * stage_rows(c->cap));
    const double* mpos = host_mapped(pos);
    const double* mvel = host_mapped(vel);
    const int32_t* mtype = host_mapped(type);
    if (mpos)
        dpos = const_cast<double*>(mpos);
    else
        CK(c, cudaMemcpyAsync(dpos, pos, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice, st));
    if (mvel)
        dvel = const_cast<double*>(mvel);
    else if (vel)
        CK(c, cudaMemcpyAsync(dvel, vel, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice, st));
    if (mtype)
        dtype = const_cast<int32_t*>(mtype);
    else
        CK(c, cudaMemcpyAsync(dtype, type, sizeof(int32_t) * (size_t)n, cudaMemcpyHostToDevice, st));
    CK(c, cudaMemsetAsync(c->status_d, 0, sizeof(uint32_t), st));
    const int64_t off = c->n;
    if (c->dim == 2)
        launch_upload<2>(st, (int)n, dpos, vel ? dvel : nullptr, dtype, c->ntypes,
                         StateBuf<2>{c->apt + off, (float2*)c->avel + off}, c->cell + off, c->counts, grid_of(c),
                         c->status_d, 0, (int)c->next_id);
    else
        launch_upload<3>(st, (int)n, dpos, vel ? dvel : nullptr, dtype, c->ntypes,
                         StateBuf<3>{c->apt + off, (float4*)c->avel + off}, c->cell + off, c->counts, grid_of(c),
                         c->status_d, 0, (int)c->next_id);
    CK(c, cudaGetLastError());
    if ((rc = read_status(c))) return rc;
    c->next_id += n;
    edited(c, c->n + n);
    return PLG_OK;
}

int plg_permute(plg_ctx* c, int64_t n_new, const int32_t* src) {
    int rc = check_ready(c);
    if (rc) return rc;
    if (n_new < 0 || n_new > c->cap) return set_err(c, PLG_E_INVALID_ARG, "bad particle count");
    if (n_new > 0 && !src) return set_err(c, PLG_E_INVALID_ARG, "NULL index array");
    {
        // Distinct indices of the current order: checked before anything changes.
        std::vector<char> seen((size_t)c->n, 0);
        for (int64_t k = 0; k < n_new; ++k) {
            const int32_t j = src[k];
            if (j < 0 || j >= c->n) return set_err(c, PLG_E_INVALID_ARG, "index outside the particles");
            if (seen[(size_t)j]) return set_err(c, PLG_E_INVALID_ARG, "repeated index");
            seen[(size_t)j] = 1;
        }
    }
    DeviceGuard g(c->device);
    if ((rc = edit_scratch(c))) return rc;
    cudaStream_t st = c->stream;
    CK(c, cudaStreamSynchronize(st));
    CK(c, cudaMemsetAsync(c->status_d, 0, sizeof(uint32_t), st));
    if (n_new > 0)
        CK(c, cudaMemcpyAsync(c->edit_flag, src, sizeof(int32_t) * (size_t)n_new, cudaMemcpyHostToDevice, st));
    if (c->dim == 2)
        launch_permute<2>(st, (int)n_new, (const int32_t*)c->edit_flag, (int)c->n, buf_a<2>(c), buf_b<2>(c),
                          c->status_d);
    else
        launch_permute<3>(st, (int)n_new, (const int32_t*)c->edit_flag, (int)c->n, buf_a<3>(c), buf_b<3>(c),
                          c->status_d);
    CK(c, cudaGetLastError());
    if ((rc = read_status(c))) return rc;  // a bad index leaves A untouched
    swap_ab(c);
    edited(c, n_new);
    return PLG_OK;
}

int plg_set_types(plg_ctx* c, const int32_t* type) {
    int rc = check_ready(c);
    if (rc) return rc;
    if (!type) return set_err(c, PLG_E_INVALID_ARG, "NULL type array");
    for (int64_t i = 0; i < c->n; ++i)
        if (type[i] < 0 || type[i] >= c->ntypes) return set_err(c, PLG_E_INVALID_ARG, "type outside [0, matrix size)");
    DeviceGuard g(c->device);
    if ((rc = edit_scratch(c))) return rc;
    cudaStream_t st = c->stream;
    CK(c, cudaStreamSynchronize(st));
    CK(c, cudaMemsetAsync(c->status_d, 0, sizeof(uint32_t), st));
    if (c->n > 0)
        CK(c, cudaMemcpyAsync(c->edit_flag, type, sizeof(int32_t) * (size_t)c->n, cudaMemcpyHostToDevice, st));
    if (c->dim == 2)
        launch_set_types<2>(st, (int)c->n, (const int32_t*)c->edit_flag, c->ntypes, c->apt, c->status_d);
    else
        launch_set_types<3>(st, (int)c->n, (const int32_t*)c->edit_flag, c->ntypes, c->apt, c->status_d);
    CK(c, cudaGetLastError());
    return read_status(c);
}

int plg_generate(plg_ctx* c, int64_t n, int32_t position_setter, int32_t type_setter, uint64_t seed) {
    if (!c) return PLG_E_INVALID_ARG;
    if (n < 0) return set_err(c, PLG_E_INVALID_ARG, "negative particle count");
    if (n > c->cap) return set_err(c, PLG_E_CAPACITY, "more particles than the context capacity");
    if (position_setter < 0 || position_setter >= kPosCount || type_setter < 0 || type_setter >= kTypeCount)
        return set_err(c, PLG_E_INVALID_ARG, "unknown setter");
    if (!c->have_settings) return set_err(c, PLG_E_STATE, "plg_set_settings has not been called");
    if (!c->have_matrix) return set_err(c, PLG_E_STATE, "plg_set_matrix has not been called");
    DeviceGuard g(c->device);
    cudaStream_t st = c->stream;
    CK(c, cudaStreamSynchronize(st));
    if (c->dim == 2)
        launch_generate<2>(st, (int)n, position_setter, type_setter, seed, c->ntypes, c->s.wrap ? 1 : 0, buf_a<2>(c));
    else
        launch_generate<3>(st, (int)n, position_setter, type_setter, seed, c->ntypes, c->s.wrap ? 1 : 0, buf_a<3>(c));
    CK(c, cudaGetLastError());
    CK(c, cudaStreamSynchronize(st));
    if (c->n != n) c->graph_dirty = true;
    c->n = n;
    c->next_id = n;
    c->fp.n = (int)n;
    c->bins_dirty = true;
    c->state_valid = true;
    return PLG_OK;
}

int plg_apply_position_setter(plg_ctx* c, int32_t setter, uint64_t seed) {
    int rc = check_ready(c);
    if (rc) return rc;
    if (setter < 0 || setter >= kPosCount) return set_err(c, PLG_E_INVALID_ARG, "unknown position setter");
    DeviceGuard g(c->device);
    cudaStream_t st = c->stream;
    if (c->dim == 2)
        launch_apply_positions<2>(st, (int)c->n, setter, seed, c->ntypes, c->s.wrap ? 1 : 0, buf_a<2>(c));
    else
        launch_apply_positions<3>(st, (int)c->n, setter, seed, c->ntypes, c->s.wrap ? 1 : 0, buf_a<3>(c));
    CK(c, cudaGetLastError());
    CK(c, cudaStreamSynchronize(st));
    c->bins_dirty = true;
    return PLG_OK;
}

int plg_apply_type_setter(plg_ctx* c, int32_t setter, uint64_t seed) {
    int rc = check_ready(c);
    if (rc) return rc;
    if (setter < 0 || setter >= kTypeCount) return set_err(c, PLG_E_INVALID_ARG, "unknown type setter");
    DeviceGuard g(c->device);
    cudaStream_t st = c->stream;
    if (c->dim == 2)
        launch_apply_types<2>(st, (int)c->n, setter, seed, c->ntypes, buf_a<2>(c));
    else
        launch_apply_types<3>(st, (int)c->n, setter, seed, c->ntypes, buf_a<3>(c));
    CK(c, cudaGetLastError());
    CK(c, cudaStreamSynchronize(st));
    return PLG_OK;
}

int plg_render(plg_ctx* c, const plg_render_params* rp, int32_t ncolors, const float* palette_rgba,
               uint8_t* out_rgba) {
    int rc = check_ready(c);
    if (rc) return rc;
    if (!rp || !palette_rgba || !out_rgba || ncolors < 1) return set_err(c, PLG_E_INVALID_ARG, "NULL argument");
    if (rp->width < 1 || rp->height < 1 || (int64_t)rp->width * rp->height > (1 << 26))
        return set_err(c, PLG_E_INVALID_ARG, "image size must be 1..2^26 pixels");
    if (!(rp->cam_w > 0) || !(rp->cam_h > 0) || !(rp->size >= 0) || !std::isfinite(rp->cam_x) ||
        !std::isfinite(rp->cam_y) || !std::isfinite(rp->size))
        return set_err(c, PLG_E_INVALID_ARG, "camera dimensions must be positive and finite");
    DeviceGuard g(c->device);
    cudaStream_t st = c->stream;
    const size_t npix = (size_t)rp->width * rp->height;
    uint32_t* winner = nullptr;
    float* pal = nullptr;
    uint8_t* img = nullptr;
    auto release = [&] {
        if (winner) cudaFree(winner);
        if (pal) cudaFree(pal);
        if (img) cudaFree(img);
    };
    if (cudaMalloc((void**)&winner, sizeof(uint32_t) * npix * splat_samples_per_pixel()) != cudaSuccess ||
        cudaMalloc((void**)&pal, sizeof(float) * 4 * (size_t)ncolors) != cudaSuccess ||
        cudaMalloc((void**)&img, 4 * npix) != cudaSuccess) {
        cudaGetLastError();
        release();
        return set_err(c, PLG_E_NO_MEMORY, "cudaMalloc (render buffers)");
    }
    SplatParams S;
    S.width = rp->width;
    S.height = rp->height;
    S.cam_x = (float)rp->cam_x;
    S.cam_y = (float)rp->cam_y;
    S.cam_w = (float)rp->cam_w;
    S.cam_h = (float)rp->cam_h;
    S.top_left_x = (float)rp->top_left_x;
    S.top_left_y = (float)rp->top_left_y;
    S.size = (float)rp->size;
    S.wrap = rp->wrap ? 1 : 0;
    cudaError_t e = cudaMemcpyAsync(pal, palette_rgba, sizeof(float) * 4 * (size_t)ncolors, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        if (c->dim == 2)
            launch_splat<2>(st, (int)c->n, c->apt, S, winner, pal, ncolors, img);
        else
            launch_splat<3>(st, (int)c->n, c->apt, S, winner, pal, ncolors, img);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out_rgba, img, 4 * npix, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    release();
    if (e != cudaSuccess) return cuda_fail(c, "plg_render", e);
    return PLG_OK;
}

int plg_generate_matrix(int32_t generator, int32_t size, uint64_t seed, double* out) {
    if (generator < 0 || generator >= kMatrixCount || size < 1 || size > kMaxTypes || !out) return PLG_E_INVALID_ARG;
    generate_matrix(generator, size, seed, out);
    return PLG_OK;
}

int plg_particle_count(plg_ctx* c, int64_t* n) {
    if (!c || !n) return PLG_E_INVALID_ARG;
    *n = c->n;
    return PLG_OK;
}

int plg_request_stop(plg_ctx* c) {
    if (!c) return PLG_E_INVALID_ARG;
    c->stop.store(1);
    return PLG_OK;
}

const char* plg_last_error(plg_ctx* c) { return c ? c->err.c_str() : "null context"; }

int plg_get_stream(plg_ctx* c, void** stream) {
    if (!c || !stream) return PLG_E_INVALID_ARG;
    *stream = (void*)c->stream;
    return PLG_OK;
}

int plg_set_use_graph(plg_ctx* c, int32_t on) {
    if (!c) return PLG_E_INVALID_ARG;
    c->use_graph = on != 0;
    return PLG_OK;
}

int plg_set_tile(plg_ctx* c, int32_t variant) {
    if (!c) return PLG_E_INVALID_ARG;
    if (variant < 0 || variant >= PLG_TILE_VARIANTS) return set_err(c, PLG_E_INVALID_ARG, "unknown tile variant");
    if (variant != tile_variant(c)) c->graph_dirty = true;
    c->variant = variant;
    c->variant_auto = false;
    return PLG_OK;
}

int plg_get_tile(plg_ctx* c, int32_t* variant) {
    if (!c || !variant) return PLG_E_INVALID_ARG;
    *variant = tile_variant(c);
    return PLG_OK;
}

// Times `steps` steps of each tile variant on the world as it is, restoring
// the particle state (A, the next cells and their counts) after each trial,
// and keeps the fastest variant.  The trials allocate a copy of the state
// and free it before returning.
int plg_autotune(plg_ctx* c, int32_t steps, int32_t* chosen, double* ms_per_step) {
    const TraceRange tr("plg_autotune");
    int rc = check_ready(c);
    if (rc) return rc;
    if (steps < 1) return set_err(c, PLG_E_INVALID_ARG, "autotune needs at least one step");
    DeviceGuard g(c->device);
    cudaStream_t st = c->stream;
    if (c->n == 0 || c->general) {  // nothing to time / the literal kernel has no tiles
        if (chosen) *chosen = tile_variant(c);
        return PLG_OK;
    }
    if ((rc = enqueue_rebin(c))) return rc;
    const size_t n = (size_t)c->n, nc = (size_t)c->ncells;
    const size_t vel_sz = c->dim == 2 ? sizeof(float2) : sizeof(float4);
    const size_t bytes[4] = {sizeof(float4) * n, vel_sz * n, 4 * n, 4 * nc};
    void* live[4] = {c->apt, c->avel, c->cell, c->counts};
    void* save[4] = {};
    for (int k = 0; k < 4 && !rc; ++k)
        if (cudaMalloc(&save[k], bytes[k]) != cudaSuccess) {
            cudaGetLastError();
            rc = set_err(c, PLG_E_NO_MEMORY, "cudaMalloc (autotune state copy)");
        }
    auto copy_all = [&](bool restore) -> cudaError_t {
        for (int k = 0; k < 4; ++k) {
            cudaError_t e = cudaMemcpyAsync(restore ? live[k] : save[k], restore ? save[k] : live[k], bytes[k],
                                            cudaMemcpyDeviceToDevice, st);
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    };
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (!rc && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)) {
        cudaGetLastError();
        rc = set_err(c, PLG_E_CUDA, "cudaEventCreate (autotune)");
    }
    if (!rc && copy_all(false) != cudaSuccess) rc = cuda_fail(c, "autotune save", cudaGetLastError());
    const int old = tile_variant(c);
    c->variant = old;
    c->variant_auto = false;
    double best = 1e300;
    double times[PLG_TILE_VARIANTS] = {};
    int best_v = old;
    for (int v = 0; v < PLG_TILE_VARIANTS && !rc; ++v) {
        if (v != c->variant) c->graph_dirty = true;
        c->variant = v;
        if ((rc = enqueue_step(c))) break;  // builds the graph, untimed
        if (cudaEventRecord(e0, st) != cudaSuccess) rc = cuda_fail(c, "autotune timing", cudaGetLastError());
        for (int32_t k = 0; k < steps && !rc; ++k) rc = enqueue_step(c);
        if (rc) break;
        float ms = 0.f;
        if (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
            cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
            rc = cuda_fail(c, "autotune timing", cudaGetLastError());
            break;
        }
        const double per = ms / steps;
        if (ms_per_step) ms_per_step[v] = per;
        times[v] = per;
        if (per < best) {
            best = per;
            best_v = v;
        }
        if (copy_all(true) != cudaSuccess) rc = cuda_fail(c, "autotune restore", cudaGetLastError());
    }
    if (!rc) rc = wait_stream(c, 0);
    if (!rc) rc = read_status(c);
    const int keep = rc ? old : switch_if_faster(old, best_v, times);
    if (keep != c->variant) c->graph_dirty = true;
    c->variant = keep;
    for (void* p : save)
        if (p) cudaFree(p);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (!rc && chosen) *chosen = keep;
    return rc;
}

int plg_profile_enable(plg_ctx* c, int32_t on) {
    if (!c) return PLG_E_INVALID_ARG;
    DeviceGuard g(c->device);
    if (on) {
        for (int k = 0; k < PLG_K_COUNT; ++k) {
            for (int j = 0; j < 2; ++j)
                if (!c->pev[k][j]) CK(c, cudaEventCreate(&c->pev[k][j]));
            c->prof_ms[k] = 0;
            c->prof_n[k] = 0;
        }
    }
    c->profiling = on != 0;
    return PLG_OK;
}

int plg_profile_read(plg_ctx* c, int32_t kernel, double* total_ms, int64_t* launches) {
    if (!c || kernel < 0 || kernel >= PLG_K_COUNT) return PLG_E_INVALID_ARG;
    if (total_ms) *total_ms = c->prof_ms[kernel];
    if (launches) *launches = c->prof_n[kernel];
    return PLG_OK;
}

const char* plg_kernel_name(int32_t kernel) {
    if (kernel < 0 || kernel >= PLG_K_COUNT) return "";
    return kKernelNames[kernel];
}

int plg_debug_step(plg_ctx* c, int32_t* cell, int32_t* pairs, uint64_t* hash_sum, uint64_t* hash_xor, float* acc,
                   int64_t* candidates) {
    int rc = check_ready(c);
    if (rc) return rc;
    DeviceGuard g(c->device);
    const size_t cap = (size_t)c->cap;
    auto dm = [&](void** p, size_t bytes) -> int {
        if (*p) return PLG_OK;
        cudaError_t e = cudaMalloc(p, bytes);
        if (e != cudaSuccess) {
            *p = nullptr;
            return cuda_fail(c, "cudaMalloc (debug buffers)", e);
        }
        return PLG_OK;
    };
    if ((rc = dm((void**)&c->dbg_pairs, sizeof(int32_t) * cap))) return rc;
    if ((rc = dm((void**)&c->dbg_hsum, sizeof(unsigned long long) * cap))) return rc;
    if ((rc = dm((void**)&c->dbg_hxor, sizeof(unsigned long long) * cap))) return rc;
    if ((rc = dm((void**)&c->dbg_cand, sizeof(unsigned long long)))) return rc;
    if ((rc = dm((void**)&c->dbg_acc, sizeof(float) * 3 * cap))) return rc;
    if ((rc = dm((void**)&c->dbg_cell, sizeof(int32_t) * cap))) return rc;
    if ((rc = enqueue_rebin(c))) return rc;
    CK(c, cudaMemsetAsync(c->dbg_cand, 0, sizeof(unsigned long long), c->stream));
    DebugOut d{c->dbg_pairs, c->dbg_hsum, c->dbg_hxor, c->dbg_acc, c->dbg_cand};
    const bool prof = c->profiling;
    c->profiling = false;
    enqueue_body_dim(c, &d, c->dbg_cell);
    c->profiling = prof;
    CK(c, cudaGetLastError());
    const size_t n = (size_t)c->n;
    cudaStream_t st = c->stream;
    unsigned long long cand = 0;
    if (n > 0) {
        if (cell) CK(c, cudaMemcpyAsync(cell, c->dbg_cell, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st));
        if (pairs) CK(c, cudaMemcpyAsync(pairs, c->dbg_pairs, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st));
        if (hash_sum) CK(c, cudaMemcpyAsync(hash_sum, c->dbg_hsum, 8 * n, cudaMemcpyDeviceToHost, st));
        if (hash_xor) CK(c, cudaMemcpyAsync(hash_xor, c->dbg_hxor, 8 * n, cudaMemcpyDeviceToHost, st));
        if (acc)
            CK(c, cudaMemcpyAsync(acc, c->dbg_acc, sizeof(float) * (size_t)c->dim * n, cudaMemcpyDeviceToHost, st));
    }
    CK(c, cudaMemcpyAsync(&cand, c->dbg_cand, sizeof(cand), cudaMemcpyDeviceToHost, st));
    CK(c, cudaStreamSynchronize(st));
    if (candidates) *candidates = (int64_t)cand;
    return read_status(c);
}

int plg_step_stats(plg_ctx* c, int64_t* deferred) {
    if (!c || !deferred) return PLG_E_INVALID_ARG;
    DeviceGuard g(c->device);
    uint32_t v = 0;
    if (!c->general && c->defer) {
        CK(c, cudaMemcpyAsync(c->status_h + 1, c->defer, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
        CK(c, cudaStreamSynchronize(c->stream));
        v = c->status_h[1];
    }
    *deferred = v;
    return PLG_OK;
}

int plg_probe_fp32_peak(double* tflops) {
    if (!tflops) return PLG_E_INVALID_ARG;
    cudaError_t e = probe_fp32_peak(tflops);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return PLG_E_CUDA;
    }
    return PLG_OK;
}

int plg_probe_sfu_peak(double* gops) {
    if (!gops) return PLG_E_INVALID_ARG;
    const cudaError_t e = probe_sfu_peak(gops);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return PLG_E_CUDA;
    }
    return PLG_OK;
}

}  // extern "C"
