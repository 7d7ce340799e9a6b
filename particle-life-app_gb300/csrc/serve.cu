// serve.cu — the serving loop: simulation requests (a world plus a step
// count) arrive at any time; a native scheduler thread keeps every admitted
// world resident on the device, admits queued requests as memory and batch
// slots free up, packs the active worlds into one batch per dimension (each
// on its own stream, so the 2D and 3D batches overlap on the GPU), advances
// them in chunks of steps (a world whose own step count ends inside a chunk
// freezes on the device until the chunk ends), and hands back each world's
// final state.  This is
// continuous batching: a request that arrives while others are running joins
// at the next chunk boundary, and one that finishes leaves at it.
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

#include "plgpu.h"

namespace {

using Clock = std::chrono::steady_clock;

// NVTX range over one scheduler chunk (free when no profiler is attached).
struct ChunkRange {
    ChunkRange() { nvtxRangePushA("plg_server chunk"); }
    ~ChunkRange() { nvtxRangePop(); }
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
    int64_t n = 0;
    int64_t bytes = 0;
    int32_t world = -1;  // id inside its batch while resident
    Clock::time_point submitted, done_at;
    int state = PLG_REQ_QUEUED;
    int status = PLG_OK;
    // result
    std::vector<double> rpos, rvel;
    std::vector<int32_t> rtype, rid;

    plg_world_desc desc() const {
        plg_world_desc d{};
        d.settings = settings;
        d.ntypes = ntypes;
        d.matrix = matrix.data();
        d.n = n;
        d.pos = n ? pos.data() : nullptr;
        d.vel = has_vel && n ? vel.data() : nullptr;
        d.type = n ? type.data() : nullptr;
        return d;
    }
};

}  // namespace

struct plg_server {
    plg_server_config cfg{};
    int device = 0;
    plg_batch* batch[2] = {nullptr, nullptr};  // [0] 2D, [1] 3D

    std::mutex mu;
    std::condition_variable cv_work;  // scheduler waits for submissions
    std::condition_variable cv_done;  // callers wait for completions
    std::deque<std::shared_ptr<Request>> queue[2];
    std::unordered_map<int64_t, std::shared_ptr<Request>> all;
    std::vector<std::shared_ptr<Request>> active[2];
    int64_t next_id = 1;
    bool stop = false;
    int fatal = PLG_OK;
    std::string err;

    // statistics (under mu)
    int64_t submitted = 0, completed = 0, failed = 0;
    int64_t resident_bytes = 0, peak_resident_bytes = 0;
    double particle_steps = 0, busy_s = 0;
    std::vector<double> latencies_ms;
    Clock::time_point started;

    std::thread worker;
};

namespace {

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

int fail_server(plg_server* s, int code, const std::string& msg) {
    std::lock_guard<std::mutex> lk(s->mu);
    s->fatal = code;
    s->err = msg;
    s->stop = true;
    s->cv_done.notify_all();
    return code;
}

// Copies finished worlds out, removes them, admits queued requests under the
// budget and the batch capacities, and re-lays out each batch once.
int reshape(plg_server* s, int d) {
    plg_batch* b = s->batch[d];
    std::vector<int32_t> removes;
    std::vector<std::shared_ptr<Request>> finished, admitted;
    {
        // Only this thread changes active[]; it does so under the lock so
        // that plg_server_stats can read the sizes.
        std::vector<std::shared_ptr<Request>> still;
        for (auto& r : s->active[d]) (r->remaining == 0 ? finished : still).push_back(r);
        std::lock_guard<std::mutex> lk(s->mu);
        s->active[d].swap(still);
    }
    for (auto& r : finished) {
        r->rpos.resize((size_t)r->n * 3);
        r->rvel.resize((size_t)r->n * 3);
        r->rtype.resize((size_t)r->n);
        r->rid.resize((size_t)r->n);
        int rc = plg_batch_download(b, r->world, r->rpos.data(), r->rvel.data(), r->rtype.data(), r->rid.data());
        if (rc) return fail_server(s, rc, std::string("download: ") + plg_batch_last_error(b));
        removes.push_back(r->world);
    }
    int32_t nworlds = 0;
    int64_t nparticles = 0, ncells = 0;
    plg_batch_counts(b, &nworlds, &nparticles, &ncells);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        const auto now = Clock::now();
        for (auto& r : finished) {
            r->done_at = now;
            r->state = PLG_REQ_DONE;
            s->completed++;
            s->resident_bytes -= r->bytes;
            s->latencies_ms.push_back(ms_between(r->submitted, now));
            // release the inputs early
            std::vector<double>().swap(r->pos);
            std::vector<double>().swap(r->vel);
            std::vector<int32_t>().swap(r->type);
        }
        nworlds -= (int32_t)finished.size();
        for (auto& r : finished) nparticles -= r->n;
        // FIFO admission: the head of the queue waits until it fits.
        while (!s->queue[d].empty()) {
            auto& r = s->queue[d].front();
            const plg_world_desc wd = r->desc();
            const int64_t cells = [&] {
                const int64_t nx = (int64_t)(1.0 / wd.settings.rmax);
                return nx * nx * (d == 1 ? nx : 1);
            }();
            if (s->resident_bytes + r->bytes > s->cfg.memory_budget_bytes) break;
            if (nworlds + 1 > s->cfg.max_worlds_per_batch) break;
            if (nparticles + r->n > s->cfg.particle_capacity[d]) break;
            if (ncells + cells > s->cfg.cell_capacity[d]) break;
            nworlds++;
            nparticles += r->n;
            ncells += cells;
            s->resident_bytes += r->bytes;
            s->peak_resident_bytes = std::max(s->peak_resident_bytes, s->resident_bytes);
            r->state = PLG_REQ_RUNNING;
            admitted.push_back(r);
            s->queue[d].pop_front();
        }
        if (!finished.empty()) s->cv_done.notify_all();
    }
    if (removes.empty() && admitted.empty()) return PLG_OK;
    std::vector<plg_world_desc> descs;
    for (auto& r : admitted) descs.push_back(r->desc());
    std::vector<int32_t> ids(admitted.size());
    int rc = plg_batch_update(b, (int32_t)removes.size(), removes.data(), (int32_t)descs.size(), descs.data(),
                              ids.data());
    if (rc) return fail_server(s, rc, std::string("batch update: ") + plg_batch_last_error(b));
    for (size_t k = 0; k < admitted.size(); ++k) {
        // The world freezes on the device once its own steps are done, so a
        // chunk can be longer than its remaining steps.
        rc = plg_batch_set_steps(b, ids[k], admitted[k]->remaining);
        if (rc) return fail_server(s, rc, std::string("set steps: ") + plg_batch_last_error(b));
    }
    std::lock_guard<std::mutex> lk(s->mu);
    for (size_t k = 0; k < admitted.size(); ++k) {
        admitted[k]->world = ids[k];
        s->active[d].push_back(admitted[k]);
    }
    return PLG_OK;
}

void scheduler(plg_server* s) {
    cudaSetDevice(s->device);
    for (;;) {
        {
            std::unique_lock<std::mutex> lk(s->mu);
            const bool idle = s->active[0].empty() && s->active[1].empty() && s->queue[0].empty() &&
                              s->queue[1].empty();
            if (s->stop) return;
            if (idle) {
                s->cv_work.wait_for(lk, std::chrono::milliseconds(20));
                continue;
            }
        }
        for (int d = 0; d < 2; ++d)
            if (reshape(s, d)) return;
        // One chunk: up to max_chunk_steps batch steps, both batches at once
        // (each on its own stream).  A world whose own steps run out inside
        // the chunk freezes on the device; the next reshape hands it back.
        int32_t k[2] = {0, 0};
        bool pending = false;
        for (int d = 0; d < 2; ++d) {
            int32_t m = 0;
            for (auto& r : s->active[d]) {
                m = std::max(m, r->remaining);
                pending |= r->remaining == 0;
            }
            k[d] = std::min(m, s->cfg.max_chunk_steps);
        }
        if (!k[0] && !k[1]) {
            if (pending) continue;
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_work.wait_for(lk, std::chrono::milliseconds(1));
            continue;
        }
        const auto t0 = Clock::now();
        const ChunkRange tr;
        for (int d = 0; d < 2; ++d)
            if (k[d] && plg_batch_step_async(s->batch[d], k[d]))
                return (void)fail_server(s, PLG_E_CUDA, std::string("step: ") + plg_batch_last_error(s->batch[d]));
        double ps = 0;
        for (int d = 0; d < 2; ++d) {
            if (!k[d]) continue;
            if (plg_batch_sync(s->batch[d], 0.0))
                return (void)fail_server(s, PLG_E_DEVICE, std::string("sync: ") + plg_batch_last_error(s->batch[d]));
            for (auto& r : s->active[d]) {
                const int32_t done = std::min(r->remaining, k[d]);
                r->remaining -= done;
                ps += (double)r->n * done;
            }
        }
        std::lock_guard<std::mutex> lk(s->mu);
        s->particle_steps += ps;
        s->busy_s += std::chrono::duration<double>(Clock::now() - t0).count();
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
    for (int d = 0; d < 2; ++d) {
        int rc = plg_batch_create(d + 2, cfg->particle_capacity[d], cfg->max_worlds_per_batch, cfg->cell_capacity[d],
                                  &s->batch[d]);
        if (!rc) rc = plg_batch_set_tile(s->batch[d], cfg->tile_variant);
        if (rc) {
            for (plg_batch* b : s->batch)
                if (b) plg_batch_destroy(b);
            delete s;
            return rc;
        }
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
    const int d = dim - 2;
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return s->fatal ? s->fatal : PLG_E_STOPPED;
    const int64_t nx = (int64_t)(1.0 / world->settings.rmax);
    const int64_t cells = nx * nx * (dim == 3 ? nx : 1);
    if (r->bytes > s->cfg.memory_budget_bytes || r->n > s->cfg.particle_capacity[d] ||
        cells > s->cfg.cell_capacity[d])
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

int plg_server_result(plg_server* s, int64_t id, double* pos, double* vel, int32_t* type, int32_t* pid,
                      int64_t* n, double* latency_ms) {
    if (!s) return PLG_E_INVALID_ARG;
    std::shared_ptr<Request> r;
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
    st.running = (int64_t)(s->active[0].size() + s->active[1].size());
    st.resident_bytes = s->resident_bytes;
    st.peak_resident_bytes = s->peak_resident_bytes;
    st.particle_steps = s->particle_steps;
    st.busy_s = s->busy_s;
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
        // Queued and running requests are dropped after the current chunk;
        // their waiters return PLG_E_STOPPED.
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv_done.notify_all();
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();
    for (plg_batch* b : s->batch)
        if (b) plg_batch_destroy(b);
    delete s;
    return PLG_OK;
}

}  // extern "C"
