// batch.cu — many independent worlds advanced by one step launch.
//
// The worlds of a batch share one set of device arrays.  World k owns the
// sorted slots [p_off, p_off + n) and the global cells [c_off, c_off + nx^D);
// its bounds table and matrix sit at offsets in shared arrays.  Because the
// cell ranges are disjoint and ordered by world, one counting sort over the
// global cell index sorts every world at once and keeps each world's
// particles contiguous, so a batched step is exactly the single-world graph
// (scan, scatter, gather, force) over the concatenation, with the force
// kernel reading each target's world parameters from a device table.  Each
// world computes exactly what a single-world context computes for it.
//
// Membership changes (plg_batch_update) re-lay out the batch in one pass:
// surviving worlds are copied to their new slots (k_batch_move), new worlds
// are converted in place from the caller's buffers, and every particle is
// re-binned with its world's grid.  Their relative particle order is kept,
// so a world's trajectory does not depend on what else is in the batch.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "plg_host.h"
#include "plg_internal.cuh"
#include "plgpu.h"

using namespace plg;

namespace {

struct WorldRec {
    int32_t id = 0;
    int64_t n = 0;
    int ntypes = 0;
    plg_settings s{};
    int nx = 0;
    int64_t ncells = 0;
    std::vector<float> bounds;  // nx + 1
    std::vector<float> matrix;  // ntypes^2
    int64_t p_off = 0, c_off = 0, m_off = 0, b_off = 0;
    int32_t steps_left = INT32_MAX;  // steps before the world freezes (INT32_MAX: no limit)
    bool dead = false;               // retired: frozen in place until the next compaction
    int variant = 0;                 // force kernel tile variant of this world
};

}  // namespace

struct plg_batch {
    int dim = 2;
    int device = 0;
    int64_t pcap = 0, ccap = 0;
    int32_t wcap = 0;
    cudaStream_t stream = nullptr;
    // Force launches of the variants after the first one in use run on
    // streams of their own (forked from and joined back into `stream`), so
    // that one variant's last wave overlaps the others' blocks.
    cudaStream_t vstream[PLG_TILE_VARIANTS] = {};
    cudaEvent_t vfork = nullptr;
    cudaEvent_t vjoin[PLG_TILE_VARIANTS] = {};

    float4* apt = nullptr;
    float4* bpt = nullptr;
    void* avel = nullptr;
    void* bvel = nullptr;
    uint32_t* cell = nullptr;
    uint32_t* perm = nullptr;
    uint32_t* slot_cell = nullptr;
    uint32_t* counts = nullptr;
    uint32_t* cstart = nullptr;
    unsigned long long* scan_state = nullptr;
    uint32_t* defer = nullptr;
    uint32_t* status_d = nullptr;
    uint32_t* status_h = nullptr;

    ForceParams* worlds_d = nullptr;  // wcap
    int* wp_off_d = nullptr;          // wcap + 1
    int* tile_off_d = nullptr;        // PLG_TILE_VARIANTS x (2 wcap + 1): tile layout of each launch
    int* steps_left_d = nullptr;      // wcap: device countdown, a world at 0 is frozen
    int tiles[PLG_TILE_VARIANTS] = {};
    int* move_new_d = nullptr;        // wcap + 1
    int* move_old_d = nullptr;        // wcap
    float* bounds_d = nullptr;
    int64_t bounds_cap = 0;
    float* matrix_d = nullptr;
    int64_t matrix_cap = 0;
    unsigned char* stage = nullptr;  // pageable uploads / downloads
    int64_t stage_cap = 0;           // bytes

    // instrumented step (allocated on first use)
    int32_t* dbg_pairs = nullptr;
    unsigned long long* dbg_hsum = nullptr;
    unsigned long long* dbg_hxor = nullptr;
    unsigned long long* dbg_cand = nullptr;
    float* dbg_acc = nullptr;
    int32_t* dbg_cell = nullptr;

    std::vector<WorldRec> worlds;  // device order
    // Incremental membership (the serving loop): worlds converted into the
    // free tail [n_total, ...) of the arrays while steps run, joining at
    // batch_commit; retired worlds stay frozen in place until batch_compact.
    std::vector<WorldRec> pending;
    int64_t pend_n = 0, pend_c = 0;  // tail particles and cells of the pending worlds
    int64_t tab_b = 0, tab_m = 0;    // next free entry of the bounds and matrix tables
    int64_t dead_n = 0;              // particles of retired worlds still in the layout
    bool pageable = false;           // the device reads and writes pageable host memory
    unsigned char* side_stage = nullptr;  // staging of tail conversions and downloads
    int64_t side_stage_cap = 0;
    int32_t next_id = 1;
    int variant = 0;  // tile variant given to new worlds (plg_batch_set_tile sets every world's)
    unsigned long long* wcycles_d = nullptr;  // wcap: per-world block cycles (per-world autotuner)
    void* tune_save[5] = {};                  // the tuners' copy of the state (kept, grown on demand)
    size_t tune_cap[5] = {};
    int64_t n_total = 0, c_total = 0;
    bool smem_matrix = true;

    bool use_graph = true;
    bool graph_dirty = true;
    cudaGraphExec_t gexec = nullptr;
    std::string err;
};

namespace {

constexpr int kMaxBatchWorlds = 1 << 10;  // world index fits the force kernel's segment key

int berr(plg_batch* b, int code, const std::string& msg) {
    if (b) b->err = msg;
    return code;
}

int bcuda(plg_batch* b, const char* what, cudaError_t e) {
    cudaGetLastError();
    return berr(b, PLG_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define BCK(b, call)                                          \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return bcuda(b, #call, e_);    \
    } while (0)

struct BatchDeviceGuard {
    int prev = -1;
    explicit BatchDeviceGuard(int d) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != d) cudaSetDevice(d);
    }
    ~BatchDeviceGuard() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

template <typename T>
T* mapped_host(T* p) {
    if (!p) return nullptr;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
    return static_cast<T*>(a.devicePointer);
}

template <typename T>
int regrow(plg_batch* b, T** p, int64_t* cap, int64_t need, const char* what) {
    if (*p && *cap >= need) return PLG_OK;
    BCK(b, cudaStreamSynchronize(b->stream));
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    const int64_t want = std::max<int64_t>(need, 1);
    cudaError_t e = cudaMalloc((void**)p, sizeof(T) * (size_t)want);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return berr(b, PLG_E_NO_MEMORY, std::string("cudaMalloc ") + what + ": " + cudaGetErrorString(e));
    }
    *cap = want;
    return PLG_OK;
}

size_t batch_stage_bytes(int64_t rows) { return (size_t)rows * (3 * 8 + 3 * 8 + 4 + 4); }

template <int D>
StateBuf<D> sbuf(float4* pt, void* vel, int64_t off) {
    return StateBuf<D>{pt + off, (typename Layout<D>::Vel*)vel + off};
}

void destroy_batch_graph(plg_batch* b) {
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    b->gexec = nullptr;
    b->graph_dirty = true;
}

void free_batch(plg_batch* b) {
    destroy_batch_graph(b);
    void* ptrs[] = {b->apt,      b->bpt,       b->avel,      b->bvel,        b->cell,
                    b->perm,     b->slot_cell, b->counts,    b->cstart,      b->scan_state, b->defer,
                    b->status_d, b->worlds_d,  b->wp_off_d,  b->move_new_d,  b->move_old_d, b->bounds_d,
                    b->tile_off_d, b->steps_left_d,
                    b->matrix_d, b->stage,     b->dbg_pairs, b->dbg_hsum,    b->dbg_hxor, b->dbg_cand,
                    b->dbg_acc,  b->dbg_cell,  b->side_stage, b->wcycles_d};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    for (void* p : b->tune_save)
        if (p) cudaFree(p);
    if (b->status_h) cudaFreeHost(b->status_h);
    for (int v = 0; v < PLG_TILE_VARIANTS; ++v) {
        if (b->vstream[v]) cudaStreamDestroy(b->vstream[v]);
        if (b->vjoin[v]) cudaEventDestroy(b->vjoin[v]);
    }
    if (b->vfork) cudaEventDestroy(b->vfork);
    if (b->stream) cudaStreamDestroy(b->stream);
}

int find_world(const plg_batch* b, int32_t id) {
    for (size_t k = 0; k < b->worlds.size(); ++k)
        if (b->worlds[k].id == id) return (int)k;
    return -1;
}

// Host-side checks of one world description (the device path has no CPU
// fallback, so anything it cannot run is rejected here).
int check_world(int dim, const plg_world_desc& d, std::string* msg) {
    auto fail = [&](int code, const char* m) {
        if (msg) *msg = m;
        return code;
    };
    int rc = plg_validate_settings(dim, &d.settings);
    if (rc) return fail(rc, "world settings rejected by plg_validate_settings");
    if (grid_n(d.settings.rmax) < 3) return fail(PLG_E_UNSUPPORTED, "batched worlds need rmax <= 1/3 (>= 3 cells per axis)");
    if (d.ntypes < 1 || d.ntypes > kMaxTypes) return fail(PLG_E_INVALID_ARG, "matrix size must be 1..1024");
    if (!d.matrix) return fail(PLG_E_INVALID_ARG, "matrix must not be NULL");
    for (int64_t k = 0; k < (int64_t)d.ntypes * d.ntypes; ++k)
        if (!std::isfinite(d.matrix[k])) return fail(PLG_E_INVALID_ARG, "matrix entries must be finite");
    if (d.n < 0) return fail(PLG_E_INVALID_ARG, "negative particle count");
    if (d.n > kMaxParticles) return fail(PLG_E_CAPACITY, "too many particles");
    if (d.n > 0 && (!d.pos || !d.type)) return fail(PLG_E_INVALID_ARG, "pos and type must not be NULL");
    for (int64_t i = 0; i < d.n; ++i) {
        for (int k = 0; k < dim; ++k) {
            const double x = d.pos[3 * i + k];
            if (!(x >= 0.0 && x <= 1.0)) return fail(PLG_E_INVALID_ARG, "positions must lie in [0,1] (ensurePosition first)");
            if (d.vel && !std::isfinite(d.vel[3 * i + k])) return fail(PLG_E_INVALID_ARG, "velocities must be finite");
        }
        if (d.type[i] < 0 || d.type[i] >= d.ntypes) return fail(PLG_E_INVALID_ARG, "types must lie in [0, matrix size)");
    }
    return PLG_OK;
}

// The checks of a world generated on the device (no particle arrays).
int check_generated(int dim, const plg_world_desc& d, std::string* msg) {
    plg_world_desc e = d;
    e.n = 0;
    e.pos = e.vel = nullptr;
    e.type = nullptr;
    const int rc = check_world(dim, e, msg);
    if (rc) return rc;
    if (d.n < 0) {
        if (msg) *msg = "negative particle count";
        return PLG_E_INVALID_ARG;
    }
    if (d.n > kMaxParticles) {
        if (msg) *msg = "too many particles";
        return PLG_E_CAPACITY;
    }
    return PLG_OK;
}

int check_desc(plg_batch* b, const plg_world_desc& d) {
    std::string msg;
    const int rc = check_world(b->dim, d, &msg);
    return rc ? berr(b, rc, msg) : PLG_OK;
}

// The force kernel's tile tables: for each variant v, the first tile of
// every world in the launch of v's worlds (a world of another variant has
// no tiles there).  A block never spans two worlds, and every world is cut
// into exactly the tiles a single-world launch of its variant uses.
size_t tile_stride(const plg_batch* b) { return 2 * (size_t)b->wcap + 1; }

// Tile layout of each variant's launch: its worlds in decreasing order of
// particles per cell (longest blocks first, so that the launch does not end
// on a straggling dense tile), then the rest with no tiles.
int write_tiles(plg_batch* b) {
    const size_t nw = b->worlds.size();
    const size_t stride = tile_stride(b);
    std::vector<int> toff((size_t)PLG_TILE_VARIANTS * stride, 0);
    std::vector<int> order(nw);
    auto density = [&](size_t k) {
        const WorldRec& w = b->worlds[k];
        return w.dead ? 0.0 : (double)w.n / (double)std::max<int64_t>(w.ncells, 1);
    };
    for (int v = 0; v < PLG_TILE_VARIANTS; ++v) {
        const int kt = tile_targets(b->dim, v);
        for (size_t k = 0; k < nw; ++k) order[k] = (int)k;
        std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
            const bool ix = b->worlds[x].variant == v, iy = b->worlds[y].variant == v;
            if (ix != iy) return ix;
            return ix && density(x) > density(y);
        });
        int* off = toff.data() + (size_t)v * stride;
        int t = 0;
        for (size_t q = 0; q < nw; ++q) {
            const int k = order[q];
            off[q] = t;
            off[nw + 1 + q] = k;
            if (b->worlds[k].variant == v) t += (int)((b->worlds[k].n + kt - 1) / kt);
        }
        off[nw] = t;
        b->tiles[v] = t;
    }
    BCK(b, cudaMemcpyAsync(b->tile_off_d, toff.data(), sizeof(int) * toff.size(), cudaMemcpyHostToDevice, b->stream));
    BCK(b, cudaStreamSynchronize(b->stream));
    destroy_batch_graph(b);
    return PLG_OK;
}

// Writes the device world tables for the current b->worlds layout.
int upload_tables(plg_batch* b) {
    const size_t nw = b->worlds.size();
    int64_t nb = 0, nm = 0;
    for (const WorldRec& w : b->worlds) {
        nb += (int64_t)w.bounds.size();
        nm += (int64_t)w.matrix.size();
    }
    int rc;
    if ((rc = regrow(b, &b->bounds_d, &b->bounds_cap, nb, "bounds"))) return rc;
    if ((rc = regrow(b, &b->matrix_d, &b->matrix_cap, nm, "matrix"))) return rc;
    std::vector<float> bounds((size_t)std::max<int64_t>(nb, 1)), matrix((size_t)std::max<int64_t>(nm, 1));
    std::vector<ForceParams> fp(std::max<size_t>(nw, 1));
    std::vector<int> off(nw + 1, 0);
    b->smem_matrix = true;
    for (size_t k = 0; k < nw; ++k) {
        const WorldRec& w = b->worlds[k];
        std::copy(w.bounds.begin(), w.bounds.end(), bounds.begin() + w.b_off);
        std::copy(w.matrix.begin(), w.matrix.end(), matrix.begin() + w.m_off);
        ForceParams p{};
        fill_force_params(w.s, w.nx, w.ncells, w.ntypes, w.bounds[w.nx], p);
        p.g.bounds = b->bounds_d + w.b_off;
        p.matrix = b->matrix_d + w.m_off;
        p.n = (int)w.n;
        p.cell_base = (uint32_t)w.c_off;
        p.p_off = (int)w.p_off;
        fp[k] = p;
        off[k] = (int)w.p_off;
        if (w.ntypes > 16) b->smem_matrix = false;
    }
    off[nw] = (int)b->n_total;
    if (nb) BCK(b, cudaMemcpyAsync(b->bounds_d, bounds.data(), sizeof(float) * nb, cudaMemcpyHostToDevice, b->stream));
    if (nm) BCK(b, cudaMemcpyAsync(b->matrix_d, matrix.data(), sizeof(float) * nm, cudaMemcpyHostToDevice, b->stream));
    if (nw) BCK(b, cudaMemcpyAsync(b->worlds_d, fp.data(), sizeof(ForceParams) * nw, cudaMemcpyHostToDevice, b->stream));
    BCK(b, cudaMemcpyAsync(b->wp_off_d, off.data(), sizeof(int) * (nw + 1), cudaMemcpyHostToDevice, b->stream));
    std::vector<int> left(std::max<size_t>(nw, 1));
    for (size_t k = 0; k < nw; ++k) left[k] = b->worlds[k].steps_left;
    if (nw) BCK(b, cudaMemcpyAsync(b->steps_left_d, left.data(), sizeof(int) * nw, cudaMemcpyHostToDevice, b->stream));
    // The host vectors die at return: wait for the copies.
    BCK(b, cudaStreamSynchronize(b->stream));
    return write_tiles(b);
}

template <int D>
int relayout(plg_batch* b, const std::vector<int>& survivors, const plg_world_desc* add, int32_t nadd,
             int32_t* ids_out) {
    destroy_batch_graph(b);  // the step graph refers to the old layout
    std::vector<WorldRec> next;
    next.reserve(survivors.size() + (size_t)nadd);
    std::vector<int> mnew, mold;
    int64_t p = 0, c = 0, m = 0, bo = 0;
    for (int k : survivors) {
        WorldRec w = b->worlds[(size_t)k];
        mnew.push_back((int)p);
        mold.push_back((int)w.p_off);
        w.p_off = p;
        w.c_off = c;
        w.m_off = m;
        w.b_off = bo;
        p += w.n;
        c += w.ncells;
        m += (int64_t)w.matrix.size();
        bo += (int64_t)w.bounds.size();
        next.push_back(std::move(w));
    }
    const int64_t n_surv = p;
    mnew.push_back((int)p);
    for (int32_t a = 0; a < nadd; ++a) {
        const plg_world_desc& d = add[a];
        WorldRec w;
        w.id = b->next_id++;
        w.variant = b->variant;
        w.n = d.n;
        w.ntypes = d.ntypes;
        w.s = d.settings;
        w.nx = grid_n(d.settings.rmax);
        w.ncells = (int64_t)w.nx * w.nx * (D == 3 ? w.nx : 1);
        w.bounds.resize((size_t)w.nx + 1);
        build_bounds(d.settings.rmax, w.nx, w.bounds.data());
        w.matrix.resize((size_t)d.ntypes * d.ntypes);
        for (size_t q = 0; q < w.matrix.size(); ++q) w.matrix[q] = (float)d.matrix[q];
        w.p_off = p;
        w.c_off = c;
        w.m_off = m;
        w.b_off = bo;
        p += w.n;
        c += w.ncells;
        m += (int64_t)w.matrix.size();
        bo += (int64_t)w.bounds.size();
        next.push_back(std::move(w));
    }
    if (p > b->pcap) return berr(b, PLG_E_CAPACITY, "batch particle capacity exceeded");
    if (c > b->ccap) return berr(b, PLG_E_CAPACITY, "batch cell capacity exceeded");
    if ((int64_t)next.size() > b->wcap) return berr(b, PLG_E_CAPACITY, "batch world capacity exceeded");

    cudaStream_t st = b->stream;
    int rc;
    // Survivors move A -> B (the tables of the old layout are no longer used).
    if (!survivors.empty()) {
        BCK(b, cudaMemcpyAsync(b->move_new_d, mnew.data(), sizeof(int) * mnew.size(), cudaMemcpyHostToDevice, st));
        BCK(b, cudaMemcpyAsync(b->move_old_d, mold.data(), sizeof(int) * mold.size(), cudaMemcpyHostToDevice, st));
        launch_batch_move<D>(st, (int)n_surv, b->move_new_d, b->move_old_d, (int)survivors.size(),
                             sbuf<D>(b->apt, b->avel, 0), sbuf<D>(b->bpt, b->bvel, 0));
        BCK(b, cudaGetLastError());
    }
    b->worlds = std::move(next);
    b->n_total = p;
    b->c_total = c;
    b->tab_b = bo;
    b->tab_m = m;
    b->dead_n = 0;
    for (const WorldRec& w : b->worlds)
        if (w.dead) b->dead_n += w.n;
    if ((rc = upload_tables(b))) return rc;  // synchronises: the move tables above are consumed
    BCK(b, cudaMemsetAsync(b->counts, 0, sizeof(uint32_t) * (size_t)std::max<int64_t>(c, 1), st));
    BCK(b, cudaMemsetAsync(b->status_d, 0, sizeof(uint32_t), st));
    // New worlds: converted from the caller's buffers straight into B.
    for (int32_t a = 0; a < nadd; ++a) {
        const plg_world_desc& d = add[a];
        const WorldRec& w = b->worlds[survivors.size() + (size_t)a];
        if (ids_out) ids_out[a] = w.id;
        if (w.n == 0) continue;
        const double* dpos = mapped_host(d.pos);
        const double* dvel = mapped_host(d.vel);
        const int32_t* dtype = mapped_host(d.type);
        const int64_t rows = (w.n + 1) & ~(int64_t)1;
        if ((!dpos || (d.vel && !dvel) || !dtype) &&
            (rc = regrow(b, &b->stage, &b->stage_cap, (int64_t)batch_stage_bytes(rows), "staging")))
            return rc;
        double* spos = (double*)b->stage;
        double* svel = spos + 3 * rows;
        int32_t* stype = (int32_t*)(svel + 3 * rows);
        if (!dpos) {
            BCK(b, cudaMemcpyAsync(spos, d.pos, sizeof(double) * 3 * w.n, cudaMemcpyHostToDevice, st));
            dpos = spos;
        }
        if (d.vel && !dvel) {
            BCK(b, cudaMemcpyAsync(svel, d.vel, sizeof(double) * 3 * w.n, cudaMemcpyHostToDevice, st));
            dvel = svel;
        }
        if (!dtype) {
            BCK(b, cudaMemcpyAsync(stype, d.type, sizeof(int32_t) * w.n, cudaMemcpyHostToDevice, st));
            dtype = stype;
        }
        Grid g{};
        g.nx = w.nx;
        g.ncells = (int)w.ncells;
        g.inv_cs = (float)(1.0 / w.s.rmax);
        g.b_nx = w.bounds[w.nx];
        g.bounds = b->bounds_d + w.b_off;
        launch_upload<D>(st, (int)w.n, dpos, dvel, dtype, w.ntypes, sbuf<D>(b->bpt, b->bvel, w.p_off),
                         b->cell + w.p_off, b->counts, g, b->status_d, (uint32_t)w.c_off);
        BCK(b, cudaGetLastError());
    }
    std::swap(b->apt, b->bpt);
    std::swap(b->avel, b->bvel);
    // Survivors: cells in the new global numbering and the next sort's counts.
    if (n_surv > 0) {
        launch_batch_rebin<D>(st, (int)n_surv, sbuf<D>(b->apt, b->avel, 0), b->worlds_d, b->wp_off_d,
                              (int)survivors.size(), b->cell, b->counts);
        BCK(b, cudaGetLastError());
    }
    BCK(b, cudaMemcpyAsync(b->status_h, b->status_d, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    BCK(b, cudaStreamSynchronize(st));
    if (*b->status_h) return berr(b, PLG_E_DEVICE, "a conversion kernel flagged invalid input");
    destroy_batch_graph(b);
    return PLG_OK;
}

// wcycles (may be null): per-world block cycles of the force launches.
template <int D>
void enqueue_batch_step(plg_batch* b, const DebugOut* dbg, int32_t* cell_sorted,
                        unsigned long long* wcycles = nullptr) {
    cudaStream_t st = b->stream;
    const int n = (int)b->n_total;
    const int nc = (int)std::max<int64_t>(b->c_total, 1);
    // The scan's state starts at zero: the scatter sets it back after each
    // scan (the whole state was zeroed at creation); with no particles a
    // memset does it.
    const int nstate = scan_blocks(nc) + 1;
    launch_scan(st, b->counts, nc, b->cstart, b->scan_state, b->status_d, b->defer);
    if (n > 0)
        launch_scatter(st, n, b->cell, b->counts, b->cstart, b->perm, b->slot_cell, b->scan_state, nstate);
    else
        cudaMemsetAsync(b->scan_state, 0, sizeof(unsigned long long) * (size_t)nstate, st);
    launch_gather<D>(st, n, b->perm, b->slot_cell, b->cstart, sbuf<D>(b->apt, b->avel, 0),
                     sbuf<D>(b->bpt, b->bvel, 0), cell_sorted);
    // One force launch per tile variant in use; the launches touch disjoint
    // worlds (their shared outputs, the next counts and the deferred count,
    // are atomics).  The first runs on the step's stream after the gather,
    // the others concurrently on their own streams, joined before the tick.
    auto force = [&](cudaStream_t s, int v) {
        launch_force_batch<D>(s, b->worlds_d, b->wp_off_d, b->tile_off_d + (size_t)v * tile_stride(b),
                              b->steps_left_d, b->tiles[v], (int)b->worlds.size(), n, b->smem_matrix,
                              sbuf<D>(b->bpt, b->bvel, 0), b->cstart, b->slot_cell, sbuf<D>(b->apt, b->avel, 0),
                              b->cell, b->counts, b->defer, dbg, v, wcycles);
    };
    int first = -1;
    for (int v = 0; v < PLG_TILE_VARIANTS; ++v)
        if (b->tiles[v] > 0 && first < 0) first = v;
    bool forked = false;
    for (int v = first + 1; first >= 0 && v < PLG_TILE_VARIANTS; ++v) {
        if (b->tiles[v] <= 0) continue;
        if (!forked) {
            cudaEventRecord(b->vfork, st);
            forked = true;
        }
        cudaStreamWaitEvent(b->vstream[v], b->vfork, 0);
        force(b->vstream[v], v);
        cudaEventRecord(b->vjoin[v], b->vstream[v]);
    }
    if (first >= 0) force(st, first);
    for (int v = first + 1; forked && v < PLG_TILE_VARIANTS; ++v)
        if (b->tiles[v] > 0) cudaStreamWaitEvent(st, b->vjoin[v], 0);
    launch_batch_tick(st, b->steps_left_d, (int)b->worlds.size());
}

int enqueue_step(plg_batch* b) {
    if (b->n_total == 0) return PLG_OK;
    if (!b->use_graph) {
        if (b->dim == 2)
            enqueue_batch_step<2>(b, nullptr, nullptr);
        else
            enqueue_batch_step<3>(b, nullptr, nullptr);
        BCK(b, cudaGetLastError());
        return PLG_OK;
    }
    if (b->graph_dirty || !b->gexec) {
        destroy_batch_graph(b);
        cudaGraph_t g = nullptr;
        BCK(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        if (b->dim == 2)
            enqueue_batch_step<2>(b, nullptr, nullptr);
        else
            enqueue_batch_step<3>(b, nullptr, nullptr);
        cudaError_t e = cudaStreamEndCapture(b->stream, &g);
        if (e != cudaSuccess) return bcuda(b, "cudaStreamEndCapture", e);
        e = cudaGraphInstantiate(&b->gexec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            b->gexec = nullptr;
            return bcuda(b, "cudaGraphInstantiate", e);
        }
        b->graph_dirty = false;
    }
    BCK(b, cudaGraphLaunch(b->gexec, b->stream));
    return PLG_OK;
}

int wait_batch(plg_batch* b, double timeout_s) {
    if (timeout_s <= 0) {
        BCK(b, cudaStreamSynchronize(b->stream));
    } else {
        const auto t0 = std::chrono::steady_clock::now();
        for (;;) {
            cudaError_t e = cudaStreamQuery(b->stream);
            if (e == cudaSuccess) break;
            if (e != cudaErrorNotReady) return bcuda(b, "cudaStreamQuery", e);
            const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            if (dt > timeout_s) return berr(b, PLG_E_TIMEOUT, "batch sync timed out");
            std::this_thread::sleep_for(std::chrono::microseconds(50));
        }
    }
    BCK(b, cudaMemcpy(b->status_h, b->status_d, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    if (*b->status_h & kDevSpinLimit) {
        cudaMemset(b->status_d, 0, sizeof(uint32_t));
        return berr(b, PLG_E_DEVICE, "a bounded device wait ran out (scan look-back)");
    }
    return PLG_OK;
}

}  // namespace

// ---- incremental membership, for the serving loop ----------------------
//
// A batch keeps its worlds at the front of its arrays; the rest is a free
// tail.  batch_append converts (or generates) a new world straight into the
// tail on a side stream while steps run on the batch stream: a step touches
// only slots below n_total and cells below c_total, so the two never meet.
// batch_commit then makes the tail worlds part of the step (tables, graph).
// A finished world is retired in place: its step budget is spent, so the
// step leaves it frozen (its state and order untouched) and it can be
// downloaded on the side stream while later steps run; batch_compact drops
// retired worlds with one re-layout pass once they take too much room.

namespace plg {

namespace {

template <int D>
int append_world(plg_batch* b, const plg_world_desc& d, const WorldGen* gen, int32_t steps, cudaStream_t side,
                 int32_t* id_out) {
    WorldRec w;
    w.variant = b->variant;
    w.n = d.n;
    w.ntypes = d.ntypes;
    w.s = d.settings;
    w.nx = grid_n(d.settings.rmax);
    w.ncells = (int64_t)w.nx * w.nx * (D == 3 ? w.nx : 1);
    const int64_t nbounds = w.nx + 1, nmat = (int64_t)d.ntypes * d.ntypes;
    if (b->n_total + b->pend_n + w.n > b->pcap) return berr(b, PLG_E_CAPACITY, "batch particle capacity exceeded");
    if (b->c_total + b->pend_c + w.ncells > b->ccap) return berr(b, PLG_E_CAPACITY, "batch cell capacity exceeded");
    if ((int64_t)(b->worlds.size() + b->pending.size()) + 1 > b->wcap)
        return berr(b, PLG_E_CAPACITY, "batch world capacity exceeded");
    if (b->tab_b + nbounds > b->bounds_cap || b->tab_m + nmat > b->matrix_cap)
        return berr(b, PLG_E_CAPACITY, "batch tables full (batch_reserve_tables)");
    w.id = b->next_id++;
    w.steps_left = steps < 0 ? INT32_MAX : steps;
    w.bounds.resize((size_t)nbounds);
    build_bounds(d.settings.rmax, w.nx, w.bounds.data());
    w.matrix.resize((size_t)nmat);
    for (size_t q = 0; q < w.matrix.size(); ++q) w.matrix[q] = (float)d.matrix[q];
    w.p_off = b->n_total + b->pend_n;
    w.c_off = b->c_total + b->pend_c;
    w.b_off = b->tab_b;
    w.m_off = b->tab_m;
    // The tail's cells may hold counts of a world a compaction dropped.
    BCK(b, cudaMemsetAsync(b->counts + w.c_off, 0, sizeof(uint32_t) * (size_t)w.ncells, side));
    // Pageable source: copied out before cudaMemcpyAsync returns.
    BCK(b, cudaMemcpyAsync(b->bounds_d + w.b_off, w.bounds.data(), sizeof(float) * nbounds, cudaMemcpyHostToDevice,
                           side));
    Grid g{};
    g.nx = w.nx;
    g.ncells = (int)w.ncells;
    g.inv_cs = (float)(1.0 / w.s.rmax);
    g.b_nx = w.bounds[w.nx];
    g.bounds = b->bounds_d + w.b_off;
    if (w.n > 0 && gen) {
        launch_generate<D>(side, (int)w.n, gen->position_setter, gen->type_setter, gen->seed, w.ntypes,
                           w.s.wrap ? 1 : 0, sbuf<D>(b->apt, b->avel, w.p_off));
        launch_rebin<D>(side, (int)w.n, sbuf<D>(b->apt, b->avel, w.p_off), b->cell + w.p_off, b->counts, g,
                        (uint32_t)w.c_off);
        BCK(b, cudaGetLastError());
    } else if (w.n > 0) {
        // Page-locked arrays are read in place; so is pageable memory on a
        // device that reads it coherently; anything else is staged.
        const double* dpos = mapped_host(d.pos);
        const double* dvel = mapped_host(d.vel);
        const int32_t* dtype = mapped_host(d.type);
        if (b->pageable) {
            if (!dpos) dpos = d.pos;
            if (!dvel) dvel = d.vel;
            if (!dtype) dtype = d.type;
        }
        if (!dpos || (d.vel && !dvel) || !dtype) {
            const int64_t rows = (w.n + 1) & ~(int64_t)1;
            const int64_t need = (int64_t)batch_stage_bytes(rows);
            if (need > b->side_stage_cap) {
                BCK(b, cudaStreamSynchronize(side));
                if (b->side_stage) cudaFree(b->side_stage);
                b->side_stage = nullptr;
                b->side_stage_cap = 0;
                if (cudaMalloc((void**)&b->side_stage, (size_t)need) != cudaSuccess) {
                    cudaGetLastError();
                    return berr(b, PLG_E_NO_MEMORY, "cudaMalloc (side staging)");
                }
                b->side_stage_cap = need;
            }
            double* spos = (double*)b->side_stage;
            double* svel = spos + 3 * rows;
            int32_t* stype = (int32_t*)(svel + 3 * rows);
            if (!dpos) {
                BCK(b, cudaMemcpyAsync(spos, d.pos, sizeof(double) * 3 * w.n, cudaMemcpyHostToDevice, side));
                dpos = spos;
            }
            if (d.vel && !dvel) {
                BCK(b, cudaMemcpyAsync(svel, d.vel, sizeof(double) * 3 * w.n, cudaMemcpyHostToDevice, side));
                dvel = svel;
            }
            if (!dtype) {
                BCK(b, cudaMemcpyAsync(stype, d.type, sizeof(int32_t) * w.n, cudaMemcpyHostToDevice, side));
                dtype = stype;
            }
        }
        launch_upload<D>(side, (int)w.n, dpos, dvel, dtype, w.ntypes, sbuf<D>(b->apt, b->avel, w.p_off),
                         b->cell + w.p_off, b->counts, g, b->status_d, (uint32_t)w.c_off);
        BCK(b, cudaGetLastError());
    }
    b->pend_n += w.n;
    b->pend_c += w.ncells;
    b->tab_b += nbounds;
    b->tab_m += nmat;
    if (id_out) *id_out = w.id;
    b->pending.push_back(std::move(w));
    return PLG_OK;
}

}  // namespace

int batch_append(plg_batch* b, const plg_world_desc& d, const WorldGen* gen, int32_t steps, cudaStream_t side,
                 int32_t* id_out) {
    if (!b) return PLG_E_INVALID_ARG;
    std::string msg;
    const int rc = gen ? check_generated(b->dim, d, &msg) : check_world(b->dim, d, &msg);
    if (rc) return berr(b, rc, msg);
    if (gen && (gen->position_setter < 0 || gen->position_setter >= kPosCount || gen->type_setter < 0 ||
                gen->type_setter >= kTypeCount))
        return berr(b, PLG_E_INVALID_ARG, "unknown setter");
    BatchDeviceGuard g(b->device);
    return b->dim == 2 ? append_world<2>(b, d, gen, steps, side, id_out) : append_world<3>(b, d, gen, steps, side, id_out);
}

bool batch_fits(const plg_batch* b, int64_t n, int64_t cells, bool after_compaction) {
    int64_t live_n = b->n_total + b->pend_n, live_c = b->c_total + b->pend_c;
    int64_t live_w = (int64_t)(b->worlds.size() + b->pending.size());
    if (after_compaction)
        for (const WorldRec& w : b->worlds)
            if (w.dead) {
                live_n -= w.n;
                live_c -= w.ncells;
                live_w -= 1;
            }
    return live_n + n <= b->pcap && live_c + cells <= b->ccap && live_w + 1 <= b->wcap;
}

int batch_reserve_tables(plg_batch* b, int64_t bounds_floats, int64_t matrix_floats) {
    if (!b) return PLG_E_INVALID_ARG;
    BatchDeviceGuard g(b->device);
    const int64_t nb = b->tab_b + bounds_floats, nm = b->tab_m + matrix_floats;
    if (nb <= b->bounds_cap && nm <= b->matrix_cap) return PLG_OK;
    if (!b->pending.empty()) return berr(b, PLG_E_STATE, "tables grow only without pending worlds");
    // The tables move: regrow waits for the batch stream, and the caller's
    // side stream has no tail work (nothing is pending).
    int rc;
    if ((rc = regrow(b, &b->bounds_d, &b->bounds_cap, std::max(nb, 2 * b->bounds_cap), "bounds"))) return rc;
    if ((rc = regrow(b, &b->matrix_d, &b->matrix_cap, std::max(nm, 2 * b->matrix_cap), "matrix"))) return rc;
    return upload_tables(b);  // the committed worlds' tables, at their offsets
}

int batch_commit(plg_batch* b) {
    if (!b) return PLG_E_INVALID_ARG;
    if (b->pending.empty()) return PLG_OK;
    BatchDeviceGuard g(b->device);
    for (WorldRec& w : b->pending) {
        b->n_total += w.n;
        b->c_total += w.ncells;
        b->worlds.push_back(std::move(w));
    }
    b->pending.clear();
    b->pend_n = b->pend_c = 0;
    destroy_batch_graph(b);
    int rc = upload_tables(b);  // synchronises the batch stream
    if (rc) return rc;
    BCK(b, cudaMemcpy(b->status_h, b->status_d, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    if (*b->status_h & (kDevBadPosition | kDevBadType | kDevBadVelocity))
        return berr(b, PLG_E_DEVICE, "a conversion kernel flagged invalid input");
    return PLG_OK;
}

int batch_retire(plg_batch* b, int32_t id) {
    if (!b) return PLG_E_INVALID_ARG;
    const int k = find_world(b, id);
    if (k < 0) return berr(b, PLG_E_INVALID_ARG, "unknown world id " + std::to_string(id));
    WorldRec& w = b->worlds[(size_t)k];
    if (w.dead) return PLG_OK;
    if (w.steps_left != 0) return berr(b, PLG_E_STATE, "only a frozen world (no steps left) can be retired");
    w.dead = true;
    b->dead_n += w.n;
    return PLG_OK;
}

int64_t batch_dead_particles(const plg_batch* b) { return b ? b->dead_n : 0; }

int batch_download_on(plg_batch* b, int32_t id, cudaStream_t st, double* pos, double* vel, int32_t* type,
                      int32_t* pid) {
    if (!b) return PLG_E_INVALID_ARG;
    const int k = find_world(b, id);
    if (k < 0) return berr(b, PLG_E_INVALID_ARG, "unknown world id " + std::to_string(id));
    const WorldRec& w = b->worlds[(size_t)k];
    if (w.n == 0) return PLG_OK;
    BatchDeviceGuard g(b->device);
    double *kpos = mapped_host(pos), *kvel = mapped_host(vel);
    int32_t *ktype = mapped_host(type), *kid = mapped_host(pid);
    if (b->pageable) {
        if (!kpos) kpos = pos;
        if (!kvel) kvel = vel;
        if (!ktype) ktype = type;
        if (!kid) kid = pid;
    }
    const bool staged = (pos && !kpos) || (vel && !kvel) || (type && !ktype) || (pid && !kid);
    const int64_t rows = (w.n + 1) & ~(int64_t)1;
    if (staged && (int64_t)batch_stage_bytes(rows) > b->side_stage_cap) {
        BCK(b, cudaStreamSynchronize(st));
        if (b->side_stage) cudaFree(b->side_stage);
        b->side_stage = nullptr;
        b->side_stage_cap = 0;
        if (cudaMalloc((void**)&b->side_stage, batch_stage_bytes(rows)) != cudaSuccess) {
            cudaGetLastError();
            return berr(b, PLG_E_NO_MEMORY, "cudaMalloc (side staging)");
        }
        b->side_stage_cap = (int64_t)batch_stage_bytes(rows);
    }
    double* spos = (double*)b->side_stage;
    double* svel = spos + 3 * rows;
    int32_t* stype = (int32_t*)(svel + 3 * rows);
    int32_t* sid = stype + rows;
    if (pos && !kpos) kpos = spos;
    if (vel && !kvel) kvel = svel;
    if (type && !ktype) ktype = stype;
    if (pid && !kid) kid = sid;
    if (b->dim == 2)
        launch_download<2>(st, (int)w.n, sbuf<2>(b->apt, b->avel, w.p_off), kpos, kvel, ktype, kid);
    else
        launch_download<3>(st, (int)w.n, sbuf<3>(b->apt, b->avel, w.p_off), kpos, kvel, ktype, kid);
    BCK(b, cudaGetLastError());
    const size_t n = (size_t)w.n;
    if (pos && kpos == spos) BCK(b, cudaMemcpyAsync(pos, spos, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st));
    if (vel && kvel == svel) BCK(b, cudaMemcpyAsync(vel, svel, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st));
    if (type && ktype == stype)
        BCK(b, cudaMemcpyAsync(type, stype, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st));
    if (pid && kid == sid) BCK(b, cudaMemcpyAsync(pid, sid, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st));
    return PLG_OK;
}

int batch_compact(plg_batch* b) {
    if (!b) return PLG_E_INVALID_ARG;
    if (!b->pending.empty()) return berr(b, PLG_E_STATE, "commit pending worlds before a compaction");
    if (b->dead_n == 0) return PLG_OK;
    std::vector<int> survivors;
    for (size_t k = 0; k < b->worlds.size(); ++k)
        if (!b->worlds[k].dead) survivors.push_back((int)k);
    BatchDeviceGuard g(b->device);
    return b->dim == 2 ? relayout<2>(b, survivors, nullptr, 0, nullptr)
                       : relayout<3>(b, survivors, nullptr, 0, nullptr);
}

}  // namespace plg

extern "C" {

int plg_world_check(int32_t dim, const plg_world_desc* d) {
    if (!d || (dim != 2 && dim != 3)) return PLG_E_INVALID_ARG;
    return check_world(dim, *d, nullptr);
}

int64_t plg_world_device_bytes(int32_t dim, const plg_world_desc* d) {
    if (!d || (dim != 2 && dim != 3) || !(d->settings.rmax > 0 && d->settings.rmax <= 1)) return -1;
    const int64_t nx = grid_n(d->settings.rmax);
    const int64_t cells = nx * nx * (dim == 3 ? nx : 1);
    // two copies of position and velocity; cell, sort permutation, slot cell
    const int64_t per_particle = dim == 2 ? 2 * (16 + 8) + 3 * 4 : 2 * (16 + 16) + 3 * 4;
    return d->n * per_particle + cells * 8 + (nx + 1) * 4 + (int64_t)d->ntypes * d->ntypes * 4;
}

int plg_batch_create(int32_t dim, int64_t particle_capacity, int32_t world_capacity, int64_t cell_capacity,
                     plg_batch** out) {
    if (!out) return PLG_E_INVALID_ARG;
    *out = nullptr;
    if (dim != 2 && dim != 3) return PLG_E_INVALID_ARG;
    if (particle_capacity < 1 || particle_capacity > kMaxParticles) return PLG_E_INVALID_ARG;
    if (world_capacity < 1 || world_capacity > kMaxBatchWorlds) return PLG_E_INVALID_ARG;
    if (cell_capacity < 1 || cell_capacity > kMaxCells) return PLG_E_INVALID_ARG;
    plg_batch* b = new plg_batch();
    b->dim = dim;
    b->pcap = particle_capacity;
    b->wcap = world_capacity;
    b->ccap = cell_capacity;
    int pageable = 0;
    if (cudaGetDevice(&b->device) != cudaSuccess ||
        cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, b->device) != cudaSuccess) {
        cudaGetLastError();
        delete b;
        return PLG_E_CUDA;
    }
    b->pageable = pageable != 0;
    int rc = PLG_OK;
    auto dm = [&](void** p, size_t bytes) {
        if (rc) return;
        if (cudaMalloc(p, bytes) != cudaSuccess) {
            cudaGetLastError();
            rc = PLG_E_NO_MEMORY;
        }
    };
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) rc = PLG_E_CUDA;
    if (!rc && cudaEventCreateWithFlags(&b->vfork, cudaEventDisableTiming) != cudaSuccess) rc = PLG_E_CUDA;
    for (int v = 0; v < PLG_TILE_VARIANTS && !rc; ++v)
        if (cudaStreamCreateWithFlags(&b->vstream[v], cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&b->vjoin[v], cudaEventDisableTiming) != cudaSuccess)
            rc = PLG_E_CUDA;
    if (!rc && force_kernels_init() != cudaSuccess) rc = PLG_E_CUDA;
    const size_t pc = (size_t)particle_capacity, cc = (size_t)cell_capacity, wc = (size_t)world_capacity;
    const size_t vel_sz = dim == 2 ? sizeof(float2) : sizeof(float4);
    dm((void**)&b->apt, sizeof(float4) * pc);
    dm((void**)&b->bpt, sizeof(float4) * pc);
    dm(&b->avel, vel_sz * pc);
    dm(&b->bvel, vel_sz * pc);
    dm((void**)&b->cell, sizeof(uint32_t) * pc);
    dm((void**)&b->perm, sizeof(uint32_t) * pc);
    dm((void**)&b->slot_cell, sizeof(uint32_t) * pc);
    dm((void**)&b->counts, sizeof(uint32_t) * cc);
    dm((void**)&b->cstart, sizeof(uint32_t) * (cc + 1));
    dm((void**)&b->scan_state, sizeof(unsigned long long) * (size_t)(scan_blocks((int)cc) + 1));
    dm((void**)&b->defer, sizeof(uint32_t));
    dm((void**)&b->status_d, 64);
    dm((void**)&b->worlds_d, sizeof(ForceParams) * wc);
    dm((void**)&b->wp_off_d, sizeof(int) * (wc + 1));
    dm((void**)&b->tile_off_d, sizeof(int) * PLG_TILE_VARIANTS * (2 * wc + 1));
    dm((void**)&b->steps_left_d, sizeof(int) * wc);
    dm((void**)&b->move_new_d, sizeof(int) * (wc + 1));
    dm((void**)&b->move_old_d, sizeof(int) * wc);
    if (!rc && cudaMallocHost((void**)&b->status_h, 64) != cudaSuccess) rc = PLG_E_NO_MEMORY;
    if (!rc && cudaMemset(b->status_d, 0, 64) != cudaSuccess) rc = PLG_E_CUDA;
    if (!rc && cudaMemset(b->counts, 0, sizeof(uint32_t) * cc) != cudaSuccess) rc = PLG_E_CUDA;
    if (!rc && cudaMemset(b->scan_state, 0, sizeof(unsigned long long) * (size_t)(scan_blocks((int)cc) + 1)) !=
                   cudaSuccess)
        rc = PLG_E_CUDA;
    if (rc) {
        cudaGetLastError();
        free_batch(b);
        delete b;
        return rc;
    }
    *out = b;
    return PLG_OK;
}

int plg_batch_destroy(plg_batch* b) {
    if (!b) return PLG_E_INVALID_ARG;
    BatchDeviceGuard g(b->device);
    cudaStreamSynchronize(b->stream);
    free_batch(b);
    delete b;
    return PLG_OK;
}

int plg_batch_update(plg_batch* b, int32_t nremove, const int32_t* remove_ids, int32_t nadd,
                     const plg_world_desc* add, int32_t* ids_out) {
    const TraceRange tr("plg_batch_update");
    if (!b) return PLG_E_INVALID_ARG;
    if (nremove < 0 || nadd < 0) return berr(b, PLG_E_INVALID_ARG, "negative world count");
    if ((nremove > 0 && !remove_ids) || (nadd > 0 && !add)) return berr(b, PLG_E_INVALID_ARG, "NULL world list");
    if (!b->pending.empty()) return berr(b, PLG_E_STATE, "worlds appended to the tail are not committed yet");
    std::vector<char> gone(b->worlds.size(), 0);
    for (int32_t r = 0; r < nremove; ++r) {
        const int k = find_world(b, remove_ids[r]);
        if (k < 0) return berr(b, PLG_E_INVALID_ARG, "unknown world id " + std::to_string(remove_ids[r]));
        gone[(size_t)k] = 1;
    }
    for (int32_t a = 0; a < nadd; ++a) {
        const int rc = check_desc(b, add[a]);
        if (rc) return rc;
    }
    std::vector<int> survivors;
    for (size_t k = 0; k < b->worlds.size(); ++k)
        if (!gone[k]) survivors.push_back((int)k);
    BatchDeviceGuard g(b->device);
    return b->dim == 2 ? relayout<2>(b, survivors, add, nadd, ids_out) : relayout<3>(b, survivors, add, nadd, ids_out);
}

int plg_batch_step_async(plg_batch* b, int32_t nsteps) {
    if (!b) return PLG_E_INVALID_ARG;
    if (nsteps < 0) return berr(b, PLG_E_INVALID_ARG, "negative step count");
    BatchDeviceGuard g(b->device);
    for (int32_t k = 0; k < nsteps; ++k) {
        const int rc = enqueue_step(b);
        if (rc) return rc;
    }
    for (WorldRec& w : b->worlds)  // mirror of the device countdown
        if (w.steps_left != INT32_MAX) w.steps_left = std::max<int32_t>(0, w.steps_left - nsteps);
    return PLG_OK;
}

int plg_batch_set_steps(plg_batch* b, int32_t id, int32_t steps) {
    if (!b) return PLG_E_INVALID_ARG;
    const int k = find_world(b, id);
    if (k < 0) return berr(b, PLG_E_INVALID_ARG, "unknown world id " + std::to_string(id));
    if (steps < 0) steps = INT32_MAX;
    BatchDeviceGuard g(b->device);
    b->worlds[(size_t)k].steps_left = steps;
    const int v = steps;
    BCK(b, cudaMemcpyAsync(b->steps_left_d + k, &v, sizeof(int), cudaMemcpyHostToDevice, b->stream));
    BCK(b, cudaStreamSynchronize(b->stream));
    return PLG_OK;
}

int plg_batch_steps_left(plg_batch* b, int32_t id, int32_t* steps) {
    if (!b || !steps) return PLG_E_INVALID_ARG;
    const int k = find_world(b, id);
    if (k < 0) return berr(b, PLG_E_INVALID_ARG, "unknown world id " + std::to_string(id));
    *steps = b->worlds[(size_t)k].steps_left == INT32_MAX ? -1 : b->worlds[(size_t)k].steps_left;
    return PLG_OK;
}

int plg_batch_sync(plg_batch* b, double timeout_s) {
    if (!b) return PLG_E_INVALID_ARG;
    BatchDeviceGuard g(b->device);
    return wait_batch(b, timeout_s);
}

int plg_batch_step(plg_batch* b, int32_t nsteps) {
    const TraceRange tr("plg_batch_step");
    const int rc = plg_batch_step_async(b, nsteps);
    if (rc) return rc;
    return plg_batch_sync(b, 0.0);
}

int plg_batch_download(plg_batch* b, int32_t id, double* pos, double* vel, int32_t* type, int32_t* pid) {
    if (!b) return PLG_E_INVALID_ARG;
    const int k = find_world(b, id);
    if (k < 0) return berr(b, PLG_E_INVALID_ARG, "unknown world id " + std::to_string(id));
    const WorldRec& w = b->worlds[(size_t)k];
    BatchDeviceGuard g(b->device);
    cudaStream_t st = b->stream;
    if (w.n == 0) return PLG_OK;
    const int64_t rows = (w.n + 1) & ~(int64_t)1;
    double* mpos = mapped_host(pos);
    double* mvel = mapped_host(vel);
    int32_t* mtype = mapped_host(type);
    int32_t* mid = mapped_host(pid);
    int rc;
    if (((pos && !mpos) || (vel && !mvel) || (type && !mtype) || (pid && !mid)) &&
        (rc = regrow(b, &b->stage, &b->stage_cap, (int64_t)batch_stage_bytes(rows), "staging")))
        return rc;
    double* spos = (double*)b->stage;
    double* svel = spos + 3 * rows;
    int32_t* stype = (int32_t*)(svel + 3 * rows);
    int32_t* sid = stype + rows;
    double* kpos = pos ? (mpos ? mpos : spos) : nullptr;
    double* kvel = vel ? (mvel ? mvel : svel) : nullptr;
    int32_t* ktype = type ? (mtype ? mtype : stype) : nullptr;
    int32_t* kid = pid ? (mid ? mid : sid) : nullptr;
    if (b->dim == 2)
        launch_download<2>(st, (int)w.n, sbuf<2>(b->apt, b->avel, w.p_off), kpos, kvel, ktype, kid);
    else
        launch_download<3>(st, (int)w.n, sbuf<3>(b->apt, b->avel, w.p_off), kpos, kvel, ktype, kid);
    BCK(b, cudaGetLastError());
    const size_t n = (size_t)w.n;
    if (pos && !mpos) BCK(b, cudaMemcpyAsync(pos, spos, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st));
    if (vel && !mvel) BCK(b, cudaMemcpyAsync(vel, svel, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st));
    if (type && !mtype) BCK(b, cudaMemcpyAsync(type, stype, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st));
    if (pid && !mid) BCK(b, cudaMemcpyAsync(pid, sid, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st));
    BCK(b, cudaStreamSynchronize(st));
    return PLG_OK;
}

int plg_batch_set_tile(plg_batch* b, int32_t variant) {
    if (!b) return PLG_E_INVALID_ARG;
    if (variant < 0 || variant >= PLG_TILE_VARIANTS) return berr(b, PLG_E_INVALID_ARG, "unknown tile variant");
    BatchDeviceGuard g(b->device);
    b->variant = variant;
    for (WorldRec& w : b->worlds) w.variant = variant;
    for (WorldRec& w : b->pending) w.variant = variant;
    return write_tiles(b);
}

int plg_batch_get_tile(plg_batch* b, int32_t* variant) {
    if (!b || !variant) return PLG_E_INVALID_ARG;
    *variant = b->variant;
    return PLG_OK;
}

int plg_batch_set_world_tile(plg_batch* b, int32_t id, int32_t variant) {
    if (!b) return PLG_E_INVALID_ARG;
    if (variant < 0 || variant >= PLG_TILE_VARIANTS) return berr(b, PLG_E_INVALID_ARG, "unknown tile variant");
    const int k = find_world(b, id);
    if (k < 0) return berr(b, PLG_E_INVALID_ARG, "unknown world id " + std::to_string(id));
    if (b->worlds[(size_t)k].variant == variant) return PLG_OK;
    BatchDeviceGuard g(b->device);
    b->worlds[(size_t)k].variant = variant;
    return write_tiles(b);
}

int plg_batch_get_world_tile(plg_batch* b, int32_t id, int32_t* variant) {
    if (!b || !variant) return PLG_E_INVALID_ARG;
    const int k = find_world(b, id);
    if (k < 0) return berr(b, PLG_E_INVALID_ARG, "unknown world id " + std::to_string(id));
    *variant = b->worlds[(size_t)k].variant;
    return PLG_OK;
}

namespace {

// The state a trial step changes (A, the next cells and their counts, the
// worlds' step budgets), copied aside and put back, so that a tuner's
// trials leave the batch where it was.  The copy lives in the batch
// (allocated on first use, grown when the batch has grown), so a tuner
// called again, as the serving loop does, allocates nothing.  A and B swap
// only in a re-layout, so the live pointers stay valid across the trials.
struct TrialState {
    static constexpr int kParts = 5;
    plg_batch* b;
    void* live[kParts] = {};
    void* save[kParts] = {};
    size_t bytes[kParts] = {};
    explicit TrialState(plg_batch* bb) : b(bb) {
        const size_t n = (size_t)b->n_total, nc = (size_t)std::max<int64_t>(b->c_total, 1);
        const size_t vel_sz = b->dim == 2 ? sizeof(float2) : sizeof(float4);
        const size_t by[kParts] = {sizeof(float4) * n, vel_sz * n, 4 * n, 4 * nc,
                                   sizeof(int) * std::max<size_t>(b->worlds.size(), 1)};
        void* lv[kParts] = {b->apt, b->avel, b->cell, b->counts, b->steps_left_d};
        for (int k = 0; k < kParts; ++k) {
            bytes[k] = by[k];
            live[k] = lv[k];
        }
    }
    int alloc() {
        for (int k = 0; k < kParts; ++k) {
            if (b->tune_cap[k] < bytes[k]) {
                if (b->tune_save[k]) {
                    BCK(b, cudaStreamSynchronize(b->stream));
                    cudaFree(b->tune_save[k]);
                }
                b->tune_save[k] = nullptr;
                b->tune_cap[k] = 0;
                if (cudaMalloc(&b->tune_save[k], bytes[k]) != cudaSuccess) {
                    cudaGetLastError();
                    b->tune_save[k] = nullptr;
                    return berr(b, PLG_E_NO_MEMORY, "cudaMalloc (tuner state copy)");
                }
                b->tune_cap[k] = bytes[k];
            }
            save[k] = b->tune_save[k];
        }
        return PLG_OK;
    }
    int copy(bool restore) {
        for (int k = 0; k < kParts; ++k)
            BCK(b, cudaMemcpyAsync(restore ? live[k] : save[k], restore ? save[k] : live[k], bytes[k],
                                   cudaMemcpyDeviceToDevice, b->stream));
        return PLG_OK;
    }
};

// `steps` timed steps of the batch as it is (one untimed step first builds
// the graph), then the state restored; *ms: per step.  With wcycles, the
// steps run as plain launches and each world's force-kernel block cycles
// are summed there.
int trial(plg_batch* b, TrialState& ts, int32_t steps, double* ms, unsigned long long* wcycles) {
    cudaStream_t st = b->stream;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = PLG_OK;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) rc = bcuda(b, "event", cudaGetLastError());
    if (!rc && wcycles) {
        if (cudaMemsetAsync(wcycles, 0, sizeof(unsigned long long) * b->worlds.size(), st) != cudaSuccess)
            rc = bcuda(b, "cudaMemsetAsync", cudaGetLastError());
        if (!rc && cudaEventRecord(e0, st) != cudaSuccess) rc = bcuda(b, "event", cudaGetLastError());
        for (int32_t k = 0; k < steps && !rc; ++k) {
            if (b->dim == 2)
                enqueue_batch_step<2>(b, nullptr, nullptr, wcycles);
            else
                enqueue_batch_step<3>(b, nullptr, nullptr, wcycles);
            if (cudaGetLastError() != cudaSuccess) rc = berr(b, PLG_E_CUDA, "tuner step launch");
        }
    } else if (!rc) {
        rc = enqueue_step(b);  // builds the graph, untimed
        if (!rc && cudaEventRecord(e0, st) != cudaSuccess) rc = bcuda(b, "event", cudaGetLastError());
        for (int32_t k = 0; k < steps && !rc; ++k) rc = enqueue_step(b);
    }
    float t = 0.f;
    if (!rc && (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                cudaEventElapsedTime(&t, e0, e1) != cudaSuccess))
        rc = bcuda(b, "tuner timing", cudaGetLastError());
    if (!rc) rc = ts.copy(true);
    if (!rc && cudaStreamSynchronize(st) != cudaSuccess) rc = bcuda(b, "tuner", cudaGetLastError());
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (ms) *ms = t / steps;
    return rc;
}

void set_all_variants(plg_batch* b, int v) {
    for (WorldRec& w : b->worlds) w.variant = v;
}

}  // namespace

// Times `steps` steps of each tile variant on the batch as it is, restoring
// the particle state after each trial, and gives every world the fastest
// variant.  The trials allocate a copy of the state and free it before
// returning.
int plg_batch_autotune(plg_batch* b, int32_t steps, int32_t* chosen, double* ms_per_step) {
    if (!b) return PLG_E_INVALID_ARG;
    if (steps < 1) return berr(b, PLG_E_INVALID_ARG, "autotune needs at least one step");
    if (!b->pending.empty()) return berr(b, PLG_E_STATE, "worlds appended to the tail are not committed yet");
    BatchDeviceGuard g(b->device);
    if (b->n_total == 0) {
        if (chosen) *chosen = b->variant;
        return PLG_OK;
    }
    std::vector<int> before;
    for (const WorldRec& w : b->worlds) before.push_back(w.variant);
    TrialState ts(b);
    int rc = ts.alloc();
    if (!rc) rc = ts.copy(false);
    const int old = b->variant;
    double times[PLG_TILE_VARIANTS] = {};
    int best_v = old;
    double best = 1e300;
    for (int v = 0; v < PLG_TILE_VARIANTS && !rc; ++v) {
        set_all_variants(b, v);
        if ((rc = write_tiles(b))) break;
        rc = trial(b, ts, steps, &times[v], nullptr);
        if (ms_per_step) ms_per_step[v] = times[v];
        if (!rc && times[v] < best) {
            best = times[v];
            best_v = v;
        }
    }
    if (rc) {
        for (size_t k = 0; k < b->worlds.size(); ++k) b->worlds[k].variant = before[k];
        write_tiles(b);
        return rc;
    }
    best_v = switch_if_faster(old, best_v, times);
    b->variant = best_v;
    set_all_variants(b, best_v);
    if (chosen) *chosen = best_v;
    return write_tiles(b);
}

// The per-world tuner.  One trial per variant with every world on it, where
// each world's force blocks add up their SM cycles; a world's cost under a
// variant is its cycles divided by the variant's resident blocks per SM (SM
// time, as the blocks share an SM).  Every world takes its cheapest variant
// (a world keeps its variant unless another is at least 2% cheaper); the
// mixed assignment is then timed whole and kept only if it beats the best
// uniform one, else every world takes that.  ms_by_variant (may be NULL):
// PLG_TILE_VARIANTS uniform times and the mixed one; variants (may be NULL):
// each world's choice, in plg_batch_world_ids order.
int plg_batch_autotune_worlds(plg_batch* b, int32_t steps, int32_t* variants, double* ms_by_variant) {
    if (!b) return PLG_E_INVALID_ARG;
    if (steps < 1) return berr(b, PLG_E_INVALID_ARG, "autotune needs at least one step");
    if (!b->pending.empty()) return berr(b, PLG_E_STATE, "worlds appended to the tail are not committed yet");
    BatchDeviceGuard g(b->device);
    const size_t nw = b->worlds.size();
    if (b->n_total == 0 || nw == 0) return PLG_OK;
    if (!b->wcycles_d && cudaMalloc((void**)&b->wcycles_d, sizeof(unsigned long long) * b->wcap) != cudaSuccess) {
        cudaGetLastError();
        b->wcycles_d = nullptr;
        return berr(b, PLG_E_NO_MEMORY, "cudaMalloc (tuner cycles)");
    }
    std::vector<int> before;
    for (const WorldRec& w : b->worlds) before.push_back(w.variant);
    TrialState ts(b);
    int rc = ts.alloc();
    if (!rc) rc = ts.copy(false);
    std::vector<unsigned long long> cyc(nw);
    std::vector<double> cost((size_t)PLG_TILE_VARIANTS * nw, 0.0);
    double uni[PLG_TILE_VARIANTS] = {};
    for (int v = 0; v < PLG_TILE_VARIANTS && !rc; ++v) {
        set_all_variants(b, v);
        if ((rc = write_tiles(b))) break;
        rc = trial(b, ts, steps, nullptr, b->wcycles_d);  // per-world cycles
        if (!rc && cudaMemcpy(cyc.data(), b->wcycles_d, sizeof(unsigned long long) * nw, cudaMemcpyDeviceToHost) !=
                       cudaSuccess)
            rc = bcuda(b, "tuner cycles", cudaGetLastError());
        if (!rc) rc = trial(b, ts, steps, &uni[v], nullptr);  // the whole batch, as a graph
        const double per_sm = (double)batch_blocks_per_sm(b->dim, v, b->smem_matrix);
        for (size_t k = 0; k < nw && !rc; ++k) cost[(size_t)v * nw + k] = (double)cyc[k] / per_sm;
    }
    std::vector<int> pick(nw);
    for (size_t k = 0; k < nw && !rc; ++k) {
        int best = before[k];
        for (int v = 0; v < PLG_TILE_VARIANTS; ++v)
            if (cost[(size_t)v * nw + k] < 0.98 * cost[(size_t)best * nw + k]) best = v;
        pick[k] = best;
    }
    double mixed = 0;
    if (!rc) {
        for (size_t k = 0; k < nw; ++k) b->worlds[k].variant = pick[k];
        rc = write_tiles(b);
        if (!rc) rc = trial(b, ts, steps, &mixed, nullptr);
    }
    if (rc) {
        for (size_t k = 0; k < nw; ++k) b->worlds[k].variant = before[k];
        write_tiles(b);
        return rc;
    }
    int best_u = 0;
    for (int v = 1; v < PLG_TILE_VARIANTS; ++v)
        if (uni[v] < uni[best_u]) best_u = v;
    if (mixed > uni[best_u]) {  // the mix lost: every world on the best uniform variant
        set_all_variants(b, best_u);
        if ((rc = write_tiles(b))) return rc;
    }
    if (ms_by_variant) {
        for (int v = 0; v < PLG_TILE_VARIANTS; ++v) ms_by_variant[v] = uni[v];
        ms_by_variant[PLG_TILE_VARIANTS] = mixed;
    }
    if (variants)
        for (size_t k = 0; k < nw; ++k) variants[k] = b->worlds[k].variant;
    return PLG_OK;
}

int plg_batch_world_ids(plg_batch* b, int32_t* ids) {
    if (!b || !ids) return PLG_E_INVALID_ARG;
    for (size_t k = 0; k < b->worlds.size(); ++k) ids[k] = b->worlds[k].id;
    return PLG_OK;
}

int plg_batch_world_info(plg_batch* b, int32_t id, int64_t* n, int64_t* first_slot, int64_t* first_cell) {
    if (!b) return PLG_E_INVALID_ARG;
    const int k = find_world(b, id);
    if (k < 0) return berr(b, PLG_E_INVALID_ARG, "unknown world id " + std::to_string(id));
    if (n) *n = b->worlds[(size_t)k].n;
    if (first_slot) *first_slot = b->worlds[(size_t)k].p_off;
    if (first_cell) *first_cell = b->worlds[(size_t)k].c_off;
    return PLG_OK;
}

int plg_batch_counts(plg_batch* b, int32_t* nworlds, int64_t* nparticles, int64_t* ncells) {
    if (!b) return PLG_E_INVALID_ARG;
    if (nworlds) *nworlds = (int32_t)b->worlds.size();
    if (nparticles) *nparticles = b->n_total;
    if (ncells) *ncells = b->c_total;
    return PLG_OK;
}

int plg_batch_set_use_graph(plg_batch* b, int32_t on) {
    if (!b) return PLG_E_INVALID_ARG;
    b->use_graph = on != 0;
    return PLG_OK;
}

int plg_batch_get_stream(plg_batch* b, void** stream) {
    if (!b || !stream) return PLG_E_INVALID_ARG;
    *stream = (void*)b->stream;
    return PLG_OK;
}

const char* plg_batch_last_error(plg_batch* b) { return b ? b->err.c_str() : "null batch"; }

int plg_batch_step_stats(plg_batch* b, int64_t* deferred) {
    if (!b || !deferred) return PLG_E_INVALID_ARG;
    BatchDeviceGuard g(b->device);
    BCK(b, cudaMemcpyAsync(b->status_h + 1, b->defer, sizeof(uint32_t), cudaMemcpyDeviceToHost, b->stream));
    BCK(b, cudaStreamSynchronize(b->stream));
    *deferred = b->status_h[1];
    return PLG_OK;
}

int plg_batch_debug_step(plg_batch* b, int32_t* cell, int32_t* pairs, uint64_t* hash_sum, uint64_t* hash_xor,
                         float* acc, int64_t* candidates) {
    if (!b) return PLG_E_INVALID_ARG;
    BatchDeviceGuard g(b->device);
    const size_t cap = (size_t)b->pcap;
    int rc = PLG_OK;
    auto dm = [&](void** p, size_t bytes) {
        if (rc || *p) return;
        if (cudaMalloc(p, bytes) != cudaSuccess) {
            cudaGetLastError();
            *p = nullptr;
            rc = berr(b, PLG_E_NO_MEMORY, "cudaMalloc (debug buffers)");
        }
    };
    dm((void**)&b->dbg_pairs, sizeof(int32_t) * cap);
    dm((void**)&b->dbg_hsum, sizeof(unsigned long long) * cap);
    dm((void**)&b->dbg_hxor, sizeof(unsigned long long) * cap);
    dm((void**)&b->dbg_cand, sizeof(unsigned long long));
    dm((void**)&b->dbg_acc, sizeof(float) * 3 * cap);
    dm((void**)&b->dbg_cell, sizeof(int32_t) * cap);
    if (rc) return rc;
    cudaStream_t st = b->stream;
    BCK(b, cudaMemsetAsync(b->dbg_cand, 0, sizeof(unsigned long long), st));
    const DebugOut dbg{b->dbg_pairs, b->dbg_hsum, b->dbg_hxor, b->dbg_acc, b->dbg_cand};
    if (b->n_total > 0) {
        if (b->dim == 2)
            enqueue_batch_step<2>(b, &dbg, b->dbg_cell);
        else
            enqueue_batch_step<3>(b, &dbg, b->dbg_cell);
        BCK(b, cudaGetLastError());
    }
    const size_t n = (size_t)b->n_total;
    if (n > 0) {
        if (cell) BCK(b, cudaMemcpyAsync(cell, b->dbg_cell, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st));
        if (pairs) BCK(b, cudaMemcpyAsync(pairs, b->dbg_pairs, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st));
        if (hash_sum) BCK(b, cudaMemcpyAsync(hash_sum, b->dbg_hsum, 8 * n, cudaMemcpyDeviceToHost, st));
        if (hash_xor) BCK(b, cudaMemcpyAsync(hash_xor, b->dbg_hxor, 8 * n, cudaMemcpyDeviceToHost, st));
        if (acc) BCK(b, cudaMemcpyAsync(acc, b->dbg_acc, sizeof(float) * b->dim * n, cudaMemcpyDeviceToHost, st));
    }
    unsigned long long cand = 0;
    BCK(b, cudaMemcpyAsync(&cand, b->dbg_cand, sizeof(cand), cudaMemcpyDeviceToHost, st));
    rc = wait_batch(b, 0.0);
    if (candidates) *candidates = (int64_t)cand;
    return rc;
}

}  // extern "C"
