// serve.cu — the serving loop: simulation requests (a world plus a step
// count) arrive at any time; a native scheduler thread keeps every admitted
// world resident on the device, admits queued requests as memory and batch
// room free up, packs the active worlds into one batch per dimension (each
// on its own stream, so the 2D and 3D batches overlap on the GPU), advances
// them in chunks of steps (a world whose own step count ends inside a chunk
// freezes on the device until the chunk ends), and hands back each world's
// final state.  This is continuous batching: a request that arrives while
// others are running joins at the next chunk boundary, and one that
// finishes leaves at it.
//
// Membership work overlaps the steps.  Each batch has a side stream: an
// admitted world is converted (or generated) into the batch's free tail on
// it while a chunk runs (batch_append), and joins at the next boundary
// (batch_commit: tables and step graph only).  A finished world is frozen by
// its step budget, so it is retired in place and downloaded on the side
// stream while the next chunk runs.  Retired worlds are dropped by one
// re-layout pass (batch_compact) only when they hold a quarter of the
// batch's particles or block the head of the queue.  At a boundary the host
// does a few table copies and a graph rebuild; the GPU keeps stepping the
// other batch meanwhile.
//
// Each result equals the world run alone: batched worlds do not interact and
// the force kernel cuts every world into the same tiles whatever else is in
// the batch, so a world's trajectory is bit for bit independent of the mix.
// No world is ever stepped past its own step count.
//
// Latency is measured per request from plg_server_submit to the moment its
// result is on the host.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include "plg_host.h"
#include "plgpu.h"

namespace {

using Clock = std::chrono::steady_clock;

// A batch is compacted once its retired worlds hold this share of its
// particles (they still cost sort work every step).
constexpr double kCompactShare = 0.25;
// Bounds and matrix table entries reserved per batch at creation.
constexpr int64_t kTableBounds = 1 << 21, kTableMatrix = 1 << 19;

// NVTX range over one scheduler boundary (free when no profiler is attached).
struct BoundaryRange {
    BoundaryRange() { nvtxRangePushA("plg_server boundary"); }
    ~BoundaryRange() { nvtxRangePop(); }
};

struct Request {
    int64_t id = 0;
    int32_t dim = 2;
    int32_t steps = 0;
    int32_t remaining = 0;
    // owned copies of the caller's world
    plg_settings settings{};
    int32_t ntypes = 0;
    std::vector<double> matrix, pos, vel;
    std::vector<int32_t> type;
    bool has_vel = false;
    bool generated = false;
    plg::WorldGen gen{};
    int64_t n = 0;
    int64_t cells = 0;
    int64_t bytes = 0;
    int32_t world = -1;  // id inside its batch while resident
    Clock::time_point submitted, done_at;
    int state = PLG_REQ_QUEUED;
    // result
    std::vector<double> rpos, rvel;
    std::vector<int32_t> rtype, rid;

    plg_world_desc desc() const {
        plg_world_desc d{};
        d.settings = settings;
        d.ntypes = ntypes;
        d.matrix = matrix.data();
        d.n = n;
        d.pos = n && !generated ? pos.data() : nullptr;
        d.vel = has_vel && n ? vel.data() : nullptr;
        d.type = n && !generated ? type.data() : nullptr;
        return d;
    }
};

using ReqPtr = std::shared_ptr<Request>;

// One dimension's batch and what the scheduler knows about it.
struct DimState {
    plg_batch* b = nullptr;
    cudaStream_t stream = nullptr;  // the batch's own stream (steps)
    cudaStream_t side = nullptr;    // tail conversions and downloads
    cudaEvent_t c0 = nullptr, c1 = nullptr;
    cudaEvent_t dl = nullptr;  // recorded on the side stream after a boundary's downloads
    bool running = false;  // a chunk is in flight
    int32_t k = 0;         // its steps
    bool want_compact = false;
    bool want_tables = false;
    std::vector<ReqPtr> active;   // stepping in the batch
    std::vector<ReqPtr> pending;  // in the tail, joining at the next boundary
    std::vector<ReqPtr> leaving;  // retired, download in flight on the side stream
    double busy_s = 0;            // device time of the chunks
    Clock::time_point last_tune{};
};

int64_t cells_of(int dim, double rmax) {
    const int64_t nx = plg::grid_n(rmax);
    return nx * nx * (dim == 3 ? nx : 1);
}

}  // namespace

struct plg_server {
    plg_server_config cfg{};
    int device = 0;
    DimState dims[2];  // [0] 2D, [1] 3D

    std::mutex mu;
    std::condition_variable cv_work;  // scheduler waits for submissions
    std::condition_variable cv_done;  // callers wait for completions
    std::deque<ReqPtr> queue[2];
    std::deque<int64_t> done_ids;  // finished requests in completion order (plg_server_wait_any)
    std::unordered_map<int64_t, ReqPtr> all;
    int64_t next_id = 1;
    bool stop = false;
    int fatal = PLG_OK;
    std::string err;

    // statistics (under mu)
    int64_t submitted = 0, completed = 0, compactions = 0, autotunes = 0;
    int64_t resident_bytes = 0, peak_resident_bytes = 0;
    double particle_steps = 0;
    double busy_dim_s[2] = {0, 0};
    std::vector<double> latencies_ms;
    Clock::time_point started;

    std::thread worker;
};

namespace {

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

bool fail_server(plg_server* s, int code, const std::string& msg) {
    std::lock_guard<std::mutex> lk(s->mu);
    s->fatal = code;
    s->err = msg;
    s->stop = true;
    s->cv_done.notify_all();
    return false;
}

bool cuda_ok(plg_server* s, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    cudaGetLastError();
    return fail_server(s, PLG_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

bool batch_ok(plg_server* s, DimState& S, int rc, const char* what) {
    if (rc == PLG_OK) return true;
    return fail_server(s, rc, std::string(what) + ": " + plg_batch_last_error(S.b));
}

// Enqueues the download of a retired world into its request's result arrays
// on the side stream.
bool start_download(plg_server* s, DimState& S, const ReqPtr& r) {
    r->rpos.assign((size_t)r->n * 3, 0.0);
    r->rvel.assign((size_t)r->n * 3, 0.0);
    r->rtype.assign((size_t)r->n, 0);
    r->rid.assign((size_t)r->n, 0);
    if (!batch_ok(s, S, plg::batch_download_on(S.b, r->world, S.side, r->rpos.data(), r->rvel.data(),
                                               r->rtype.data(), r->rid.data()),
                  "download"))
        return false;
    S.leaving.push_back(r);
    return true;
}

// The side stream has finished: the leaving worlds' results are on the host.
void finish_leaving(plg_server* s, DimState& S) {
    if (S.leaving.empty()) return;
    std::lock_guard<std::mutex> lk(s->mu);
    const auto now = Clock::now();
    for (auto& r : S.leaving) {
        r->done_at = now;
        r->state = PLG_REQ_DONE;
        s->completed++;
        s->resident_bytes -= r->bytes;
        s->latencies_ms.push_back(ms_between(r->submitted, now));
        s->done_ids.push_back(r->id);
        // release the inputs early
        std::vector<double>().swap(r->pos);
        std::vector<double>().swap(r->vel);
        std::vector<int32_t>().swap(r->type);
    }
    S.leaving.clear();
    s->cv_done.notify_all();
}

// A chunk has ended (or none was running): collect it, then at the boundary
// finish downloads, retire finished worlds, commit the tail, compact when
// due, start the next chunk and the new downloads.
bool boundary(plg_server* s, int d, bool* did) {
    DimState& S = s->dims[d];
    if (S.running) {
        const cudaError_t q = cudaEventQuery(S.c1);
        if (q == cudaErrorNotReady) return true;
        if (!cuda_ok(s, q, "chunk")) return false;
        float ms = 0.f;
        if (!cuda_ok(s, cudaEventElapsedTime(&ms, S.c0, S.c1), "chunk timing")) return false;
        if (!batch_ok(s, S, plg_batch_sync(S.b, 0.0), "step")) return false;  // kernel error words
        double ps = 0;
        for (auto& r : S.active) {
            const int32_t done = std::min(r->remaining, S.k);
            r->remaining -= done;
            ps += (double)r->n * done;
        }
        S.busy_s += 1e-3 * ms;
        S.running = false;
        *did = true;
        std::lock_guard<std::mutex> lk(s->mu);
        s->particle_steps += ps;
        s->busy_dim_s[d] = S.busy_s;
    }
    if (S.active.empty() && S.pending.empty() && S.leaving.empty() && !S.want_compact && !S.want_tables) return true;
    const BoundaryRange tr;
    *did = true;
    // Downloads and tail conversions enqueued during the chunk.
    if (!cuda_ok(s, cudaStreamSynchronize(S.side), "side stream")) return false;
    finish_leaving(s, S);
    std::vector<ReqPtr> finished, still;
    for (auto& r : S.active) (r->remaining == 0 ? finished : still).push_back(r);
    for (auto& r : finished)
        if (!batch_ok(s, S, plg::batch_retire(S.b, r->world), "retire")) return false;
    if (!S.pending.empty()) {
        if (!batch_ok(s, S, plg::batch_commit(S.b), "commit")) return false;
        for (auto& r : S.pending) still.push_back(r);
        S.pending.clear();
    }
    {
        std::lock_guard<std::mutex> lk(s->mu);  // plg_server_stats reads the sizes
        S.active.swap(still);
    }
    int64_t n_total = 0;
    plg_batch_counts(S.b, nullptr, &n_total, nullptr);
    const int64_t dead = plg::batch_dead_particles(S.b);
    if (dead > 0 && (S.want_compact || (double)dead >= kCompactShare * (double)n_total)) {
        // Retired worlds leave the layout: their downloads first.
        for (auto& r : finished)
            if (!start_download(s, S, r)) return false;
        finished.clear();
        if (!cuda_ok(s, cudaStreamSynchronize(S.side), "side stream")) return false;
        finish_leaving(s, S);
        if (!batch_ok(s, S, plg::batch_compact(S.b), "compact")) return false;
        S.want_compact = false;
        std::lock_guard<std::mutex> lk(s->mu);
        s->compactions++;
    }
    if (S.want_tables) {
        if (!batch_ok(s, S, plg::batch_reserve_tables(S.b, kTableBounds, kTableMatrix), "tables")) return false;
        S.want_tables = false;
    }
    int32_t k = 0;
    for (auto& r : S.active) k = std::max(k, r->remaining);
    k = std::min(k, s->cfg.max_chunk_steps);
    if (k > 0 && s->cfg.autotune_interval_ms > 0 &&
        ms_between(S.last_tune, Clock::now()) >= (double)s->cfg.autotune_interval_ms) {
        // Every variant gives the same bits: tuning changes speed only.
        if (!batch_ok(s, S, plg_batch_autotune_worlds(S.b, 1, nullptr, nullptr), "autotune")) return false;
        S.last_tune = Clock::now();
        std::lock_guard<std::mutex> lk(s->mu);
        s->autotunes++;
    }
    if (k > 0) {
        if (!cuda_ok(s, cudaEventRecord(S.c0, S.stream), "event")) return false;
        if (!batch_ok(s, S, plg_batch_step_async(S.b, k), "step")) return false;
        if (!cuda_ok(s, cudaEventRecord(S.c1, S.stream), "event")) return false;
        S.running = true;
        S.k = k;
    }
    // Finished worlds are frozen: their downloads overlap the chunk.
    for (auto& r : finished)
        if (!start_download(s, S, r)) return false;
    if (!S.leaving.empty() && !cuda_ok(s, cudaEventRecord(S.dl, S.side), "event")) return false;
    return true;
}

// Hands back results as soon as their downloads are done, without waiting
// for the chunk's end.
bool poll_downloads(plg_server* s, int d, bool* did) {
    DimState& S = s->dims[d];
    if (S.leaving.empty()) return true;
    const cudaError_t q = cudaEventQuery(S.dl);
    if (q == cudaErrorNotReady) return true;
    if (!cuda_ok(s, q, "download")) return false;
    finish_leaving(s, S);
    *did = true;
    return true;
}

// Admits queued requests, first in first out, while the head fits the
// memory budget and its batch's free tail; each admitted world is converted
// (or generated) into the tail on the side stream.
bool admit(plg_server* s, int d, bool* did) {
    DimState& S = s->dims[d];
    for (;;) {
        ReqPtr r;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            if (s->queue[d].empty()) return true;
            r = s->queue[d].front();
            if (s->resident_bytes + r->bytes > s->cfg.memory_budget_bytes) return true;
        }
        if (S.want_tables || S.want_compact) return true;  // room is made at the next boundary
        if (!plg::batch_fits(S.b, r->n, r->cells, false)) {
            if (plg::batch_fits(S.b, r->n, r->cells, true)) S.want_compact = true;
            return true;
        }
        const plg_world_desc wd = r->desc();
        int32_t id = -1;
        const int rc = plg::batch_append(S.b, wd, r->generated ? &r->gen : nullptr, r->remaining, S.side, &id);
        if (rc == PLG_E_CAPACITY) {  // the tables: grown at the next boundary
            S.want_tables = true;
            return true;
        }
        if (!batch_ok(s, S, rc, "append")) return false;
        r->world = id;
        S.pending.push_back(r);
        *did = true;
        std::lock_guard<std::mutex> lk(s->mu);
        s->queue[d].pop_front();
        s->resident_bytes += r->bytes;
        s->peak_resident_bytes = std::max(s->peak_resident_bytes, s->resident_bytes);
        r->state = PLG_REQ_RUNNING;
    }
}

void scheduler(plg_server* s) {
    cudaSetDevice(s->device);
    for (;;) {
        {
            std::lock_guard<std::mutex> lk(s->mu);
            if (s->stop) return;
        }
        bool did = false;
        for (int d = 0; d < 2; ++d)
            if (!boundary(s, d, &did) || !poll_downloads(s, d, &did) || !admit(s, d, &did)) return;
        if (did) continue;
        const bool running = s->dims[0].running || s->dims[1].running;
        std::unique_lock<std::mutex> lk(s->mu);
        if (s->stop) return;
        const bool idle = !running && s->queue[0].empty() && s->queue[1].empty() && s->dims[0].active.empty() &&
                          s->dims[1].active.empty() && s->dims[0].pending.empty() && s->dims[1].pending.empty();
        // Chunks are polled: a short wait keeps a boundary within 0.1 ms of
        // the chunk's end; an idle server sleeps until a submission.
        s->cv_work.wait_for(lk, idle ? std::chrono::microseconds(20000) : std::chrono::microseconds(100));
    }
}

int submit_request(plg_server* s, int32_t dim, const ReqPtr& r, int64_t* id) {
    const int d = dim - 2;
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return s->fatal ? s->fatal : PLG_E_STOPPED;
    if (r->bytes > s->cfg.memory_budget_bytes || r->n > s->cfg.particle_capacity[d] ||
        r->cells > s->cfg.cell_capacity[d])
        return PLG_E_CAPACITY;  // could never be admitted
    r->id = s->next_id++;
    r->submitted = Clock::now();
    s->all[r->id] = r;
    s->queue[d].push_back(r);
    s->submitted++;
    *id = r->id;
    s->cv_work.notify_one();
    return PLG_OK;
}

void destroy_dims(plg_server* s) {
    for (DimState& S : s->dims) {
        if (S.side) cudaStreamSynchronize(S.side);
        if (S.b) plg_batch_destroy(S.b);
        if (S.side) cudaStreamDestroy(S.side);
        if (S.c0) cudaEventDestroy(S.c0);
        if (S.c1) cudaEventDestroy(S.c1);
        if (S.dl) cudaEventDestroy(S.dl);
        S = DimState{};
    }
}

}  // namespace

extern "C" {

int plg_server_create(const plg_server_config* cfg, plg_server** out) {
    if (!cfg || !out) return PLG_E_INVALID_ARG;
    *out = nullptr;
    if (cfg->memory_budget_bytes <= 0 || cfg->max_chunk_steps < 1 || cfg->max_worlds_per_batch < 1 ||
        cfg->max_worlds_per_batch > 1024)
        return PLG_E_INVALID_ARG;
    for (int d = 0; d < 2; ++d)
        if (cfg->particle_capacity[d] < 1 || cfg->cell_capacity[d] < 1) return PLG_E_INVALID_ARG;
    if (cfg->tile_variant < 0 || cfg->tile_variant >= PLG_TILE_VARIANTS) return PLG_E_INVALID_ARG;
    plg_server* s = new plg_server();
    s->cfg = *cfg;
    if (cudaGetDevice(&s->device) != cudaSuccess) {
        cudaGetLastError();
        delete s;
        return PLG_E_CUDA;
    }
    int rc = PLG_OK;
    for (int d = 0; d < 2 && !rc; ++d) {
        DimState& S = s->dims[d];
        rc = plg_batch_create(d + 2, cfg->particle_capacity[d], cfg->max_worlds_per_batch, cfg->cell_capacity[d],
                              &S.b);
        if (!rc) rc = plg_batch_set_tile(S.b, cfg->tile_variant);
        if (!rc) rc = plg_batch_get_stream(S.b, (void**)&S.stream);
        if (!rc && (cudaStreamCreateWithFlags(&S.side, cudaStreamNonBlocking) != cudaSuccess ||
                    cudaEventCreate(&S.c0) != cudaSuccess || cudaEventCreate(&S.c1) != cudaSuccess ||
                    cudaEventCreateWithFlags(&S.dl, cudaEventDisableTiming) != cudaSuccess)) {
            cudaGetLastError();
            rc = PLG_E_CUDA;
        }
        if (!rc) rc = plg::batch_reserve_tables(S.b, kTableBounds, kTableMatrix);
    }
    if (rc) {
        destroy_dims(s);
        delete s;
        return rc;
    }
    s->started = Clock::now();
    s->worker = std::thread(scheduler, s);
    *out = s;
    return PLG_OK;
}

int plg_server_submit(plg_server* s, int32_t dim, const plg_world_desc* world, int32_t steps, int64_t* id) {
    if (!s || !world || !id || (dim != 2 && dim != 3) || steps < 0) return PLG_E_INVALID_ARG;
    int rc = plg_world_check(dim, world);
    if (rc) return rc;
    auto r = std::make_shared<Request>();
    r->dim = dim;
    r->steps = r->remaining = steps;
    r->settings = world->settings;
    r->ntypes = world->ntypes;
    r->matrix.assign(world->matrix, world->matrix + (size_t)world->ntypes * world->ntypes);
    r->n = world->n;
    if (world->n) {
        r->pos.assign(world->pos, world->pos + 3 * (size_t)world->n);
        r->type.assign(world->type, world->type + (size_t)world->n);
        if (world->vel) {
            r->vel.assign(world->vel, world->vel + 3 * (size_t)world->n);
            r->has_vel = true;
        }
    }
    r->bytes = plg_world_device_bytes(dim, world);
    r->cells = cells_of(dim, world->settings.rmax);
    return submit_request(s, dim, r, id);
}

int plg_server_submit_generated(plg_server* s, int32_t dim, const plg_world_gen* g, int32_t steps, int64_t* id) {
    if (!s || !g || !id || (dim != 2 && dim != 3) || steps < 0) return PLG_E_INVALID_ARG;
    if (g->position_setter < 0 || g->position_setter > PLG_POS_RAINBOW_SPIRAL || g->type_setter < 0 ||
        g->type_setter > PLG_TYPE_KILL_STILL)
        return PLG_E_INVALID_ARG;
    plg_world_desc w = g->world;
    const int64_t n = w.n;
    if (n < 0) return PLG_E_INVALID_ARG;
    w.n = 0;  // checks of everything but the particles
    w.pos = w.vel = nullptr;
    w.type = nullptr;
    int rc = plg_world_check(dim, &w);
    if (rc) return rc;
    auto r = std::make_shared<Request>();
    r->dim = dim;
    r->steps = r->remaining = steps;
    r->settings = w.settings;
    r->ntypes = w.ntypes;
    r->matrix.assign(w.matrix, w.matrix + (size_t)w.ntypes * w.ntypes);
    r->n = n;
    r->generated = true;
    r->gen = plg::WorldGen{g->position_setter, g->type_setter, g->seed};
    w.n = n;
    r->bytes = plg_world_device_bytes(dim, &w);
    r->cells = cells_of(dim, w.settings.rmax);
    return submit_request(s, dim, r, id);
}

int plg_server_wait(plg_server* s, int64_t id, double timeout_s, int32_t* state) {
    if (!s) return PLG_E_INVALID_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return PLG_E_INVALID_ARG;
    auto r = it->second;
    auto pred = [&] { return r->state == PLG_REQ_DONE || s->stop; };
    if (timeout_s > 0)
        s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred);
    else
        s->cv_done.wait(lk, pred);
    if (state) *state = r->state;
    if (r->state == PLG_REQ_DONE) return PLG_OK;
    if (s->fatal) return s->fatal;
    return s->stop ? PLG_E_STOPPED : PLG_E_TIMEOUT;
}

int plg_server_wait_any(plg_server* s, double timeout_s, int64_t* id) {
    if (!s || !id) return PLG_E_INVALID_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto pred = [&] { return !s->done_ids.empty() || s->stop; };
    if (timeout_s > 0)
        s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred);
    else
        s->cv_done.wait(lk, pred);
    if (!s->done_ids.empty()) {
        *id = s->done_ids.front();
        s->done_ids.pop_front();
        return PLG_OK;
    }
    if (s->fatal) return s->fatal;
    return s->stop ? PLG_E_STOPPED : PLG_E_TIMEOUT;
}

int plg_server_result(plg_server* s, int64_t id, double* pos, double* vel, int32_t* type, int32_t* pid,
                      int64_t* n, double* latency_ms) {
    if (!s) return PLG_E_INVALID_ARG;
    ReqPtr r;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->all.find(id);
        if (it == s->all.end()) return PLG_E_INVALID_ARG;
        r = it->second;
        if (r->state != PLG_REQ_DONE) return PLG_E_STATE;
        s->all.erase(it);
    }
    const size_t m = (size_t)r->n;
    if (n) *n = r->n;
    if (latency_ms) *latency_ms = ms_between(r->submitted, r->done_at);
    if (pos) std::copy(r->rpos.begin(), r->rpos.begin() + 3 * m, pos);
    if (vel) std::copy(r->rvel.begin(), r->rvel.begin() + 3 * m, vel);
    if (type) std::copy(r->rtype.begin(), r->rtype.begin() + m, type);
    if (pid) std::copy(r->rid.begin(), r->rid.begin() + m, pid);
    return PLG_OK;
}

int plg_server_stats(plg_server* s, plg_server_stats_t* out) {
    if (!s || !out) return PLG_E_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    plg_server_stats_t st{};
    st.submitted = s->submitted;
    st.completed = s->completed;
    st.queued = (int64_t)(s->queue[0].size() + s->queue[1].size());
    for (const DimState& S : s->dims) st.running += (int64_t)(S.active.size() + S.pending.size() + S.leaving.size());
    st.resident_bytes = s->resident_bytes;
    st.peak_resident_bytes = s->peak_resident_bytes;
    st.particle_steps = s->particle_steps;
    st.busy_dim_s[0] = s->busy_dim_s[0];
    st.busy_dim_s[1] = s->busy_dim_s[1];
    st.busy_s = s->busy_dim_s[0] + s->busy_dim_s[1];
    st.compactions = s->compactions;
    st.autotunes = s->autotunes;
    st.wall_s = std::chrono::duration<double>(Clock::now() - s->started).count();
    if (!s->latencies_ms.empty()) {
        std::vector<double> v = s->latencies_ms;
        std::sort(v.begin(), v.end());
        auto pct = [&](double p) {
            const double x = p * (double)(v.size() - 1);
            const size_t i = (size_t)x;
            const double f = x - (double)i;
            return i + 1 < v.size() ? v[i] * (1 - f) + v[i + 1] * f : v[i];
        };
        st.latency_p50_ms = pct(0.50);
        st.latency_p99_ms = pct(0.99);
        double sum = 0;
        for (double x : v) sum += x;
        st.latency_mean_ms = sum / (double)v.size();
    }
    *out = st;
    return s->fatal;
}

const char* plg_server_last_error(plg_server* s) { return s ? s->err.c_str() : "null server"; }

int plg_server_destroy(plg_server* s) {
    if (!s) return PLG_E_INVALID_ARG;
    {
        // Queued and running requests are dropped; their waiters return
        // PLG_E_STOPPED.
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv_done.notify_all();
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();
    destroy_dims(s);
    delete s;
    return PLG_OK;
}

}  // extern "C"
