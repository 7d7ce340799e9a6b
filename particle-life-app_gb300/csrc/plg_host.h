// plg_host.h — host-side helpers shared by the single-world context
// (plgpu.cu) and the batched worlds (batch.cu).
#pragma once

#include <stdint.h>

#include "plg_internal.cuh"
#include "plgpu.h"

namespace plg {

constexpr int64_t kMaxParticles = INT32_MAX / 2;  // 32-bit indices on the device
constexpr int64_t kMaxCells = (int64_t)1 << 30;
constexpr int kMaxAxisCells = 1 << 20;
constexpr int kMaxTypes = 1024;
constexpr double kBandRel = 1.0 / (1 << 19);  // FP32 decision band: 2^-19 relative

// nx = floor(1 / cs) with cs = rmax (Physics.java:82-85, 312-313).
int grid_n(double rmax);

// bounds[k] = smallest float x >= 0 with (double)x / cs >= k (k = 1..nx);
// bounds[0] = 0.
void build_bounds(double cs, int nx, float* b);

// The per-world force parameters that follow from the settings and the grid;
// the caller sets n, matrix, g.bounds, cell_base and p_off.
void fill_force_params(const plg_settings& s, int nx, int64_t ncells, int ntypes, float b_nx, ForceParams& p);

// ---- incremental batch membership (batch.cu), used by the serving loop ----

// A world generated on the device (Physics.setParticleCount from nothing,
// with catalogue setters: plg_generate) instead of uploaded.
struct WorldGen {
    int32_t position_setter, type_setter;
    uint64_t seed;
};

// Converts (gen == nullptr: from d's arrays) or generates a world into the
// batch's free tail on `side`, while steps may run on the batch stream; it
// joins the step at batch_commit, with a budget of `steps` (< 0: none).
// PLG_E_CAPACITY when the tail, the world slots or the tables are full.
int batch_append(plg_batch* b, const plg_world_desc& d, const WorldGen* gen, int32_t steps, cudaStream_t side,
                 int32_t* id);
// Whether a world of n particles and `cells` cells fits the tail now (or
// after batch_compact drops the retired worlds).
bool batch_fits(const plg_batch* b, int64_t n, int64_t cells, bool after_compaction);
// Grows the bounds and matrix tables for appends (no pending worlds; waits
// for the device).
int batch_reserve_tables(plg_batch* b, int64_t bounds_floats, int64_t matrix_floats);
// Pending tail worlds join the step (batch stream idle; side work done).
int batch_commit(plg_batch* b);
// A frozen world (no steps left) is retired: it stays in place, untouched by
// steps, until batch_compact.
int batch_retire(plg_batch* b, int32_t id);
int64_t batch_dead_particles(const plg_batch* b);
// Enqueues a world's download on stream st (no wait); host arrays must stay
// valid until st has finished it.
int batch_download_on(plg_batch* b, int32_t id, cudaStream_t st, double* pos, double* vel, int32_t* type,
                      int32_t* pid);
// Re-lays out the batch without its retired worlds (no pending worlds;
// synchronous).
int batch_compact(plg_batch* b);

}  // namespace plg
