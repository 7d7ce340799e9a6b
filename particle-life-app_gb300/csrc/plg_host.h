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

}  // namespace plg
