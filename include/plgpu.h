/*
 * plgpu.h — C ABI of the GB300-native Particle Life physics step.
 *
 * One context (plg_ctx) holds one world: its particles in FP32 structure-of-
 * arrays form in device memory, its PhysicsSettings mirror and its type
 * matrix.  plg_step() advances the world exactly like
 * com.particle_life.backend.Physics.update() does on the CPU:
 *
 *   makeContainers  (Physics.java:309-354)  -> device stable counting sort
 *   updateVelocity  (Physics.java:397-441)  -> fused force kernel
 *   Accelerator     (app/Main.java:275-280) -> fused into the force kernel
 *   updatePosition  (Physics.java:443-450)  -> force kernel epilogue
 *
 * Reference paths are relative to src/main/java/com/particle_life/ of
 * tom-mohr/particle-life-app.
 *
 * Conventions
 *   - Every function returns a plg_status (0 = PLG_OK).  Nothing throws or
 *     aborts across this boundary.  plg_last_error() gives a message.
 *   - Host buffers are owned by the caller and are never retained after a
 *     call returns.  The library owns all device memory.
 *   - One context is driven by one thread at a time.  plg_request_stop() is
 *     the only call that may come from another thread.
 *   - Positions live in the reference's unit box [0,1)^d (wrap) or [0,1]^d
 *     (clamp).  Host arrays use the PhysicsSnapshot layout
 *     (app/PhysicsSnapshot.java:36-62): double[3n] interleaved x,y,z for
 *     positions and velocities (z = 0 in 2D), int32[n] types.
 *   - Particle ids are the upload index.  Like Physics.particles, the
 *     particle order is permuted by every step (cell-sorted order); ids let a
 *     caller map particles back.
 */
#ifndef PLGPU_H
#define PLGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PLG_ABI_VERSION 1

typedef enum plg_status {
    PLG_OK = 0,
    PLG_E_INVALID_ARG = 1, /* bad pointer, size, range or setting           */
    PLG_E_UNSUPPORTED = 2, /* e.g. an accelerator other than particle-life  */
    PLG_E_STATE = 3,       /* call order: step before settings/matrix/upload */
    PLG_E_NO_MEMORY = 4,   /* device or pinned allocation failed            */
    PLG_E_CUDA = 5,        /* a CUDA runtime call failed (no device, ...)   */
    PLG_E_TIMEOUT = 6,     /* a bounded device wait ran out                 */
    PLG_E_STOPPED = 7,     /* plg_request_stop() ended a multi-step call    */
    PLG_E_DEVICE = 8,      /* a kernel raised its error word                */
    PLG_E_CAPACITY = 9     /* more particles than the context was built for */
} plg_status;

/* The only accelerator with a device implementation: the default lambda of
 * app/Main.java:275-280 with its beta (hard-coded 0.3 there) as a parameter.
 * Any other kind is rejected with PLG_E_UNSUPPORTED: there is no CPU
 * fallback.  Mirrors the Accelerator plug-in (backend/Accelerator.java:16). */
#define PLG_ACCEL_PARTICLE_LIFE 1

/* Mirror of backend/PhysicsSettings.java:8-38 (matrix passed separately). */
typedef struct plg_settings {
    double rmax;       /* interaction radius, also the cell size (0 < rmax <= 1) */
    double friction;   /* per-1/60 s velocity factor, applied as pow(friction, 60 dt) */
    double force;      /* force multiplier                                   */
    double dt;         /* time step in seconds                               */
    double beta;       /* accelerator parameter, 0 < beta < 1                */
    int32_t wrap;      /* 1: periodic box (Range.wrap), 0: clamp (Range.clamp) */
    int32_t accel_kind;/* PLG_ACCEL_PARTICLE_LIFE                            */
} plg_settings;

typedef struct plg_ctx plg_ctx;

/* ---- library --------------------------------------------------------- */

/* Version string of this build.  Host only. */
const char* plg_version(void);

/* Static description of a status code.  Host only. */
const char* plg_status_string(int status);

/* Checks a settings struct without touching a device.  Host only.
 * Replaces nothing in the reference (Java accepts any doubles); it states
 * the ranges the device path supports. */
int plg_validate_settings(int dim, const plg_settings* s);

/* The exact cell lookup table used on the device.  Host only.
 * For cell size cs = rmax, nx = floor(1/cs) (Physics.java:82-85) and
 * bounds[k] (k = 0..nx) = the smallest float x with (int)((double)x/cs) >= k,
 * so that the reference's getContainerIndex (Physics.java:362-375) of an
 * FP32 position equals the number of k >= 1 with x >= bounds[k], clamped to
 * nx-1.  Writes *nx_out; writes bounds when bounds != NULL and cap > nx. */
int plg_cell_bounds(double rmax, int32_t* nx_out, float* bounds, int64_t cap);

/* ---- context ---------------------------------------------------------- */

/* Creates a world of dimension 2 or 3 able to hold `capacity` particles on
 * the current CUDA device.  Replaces the Physics constructor
 * (Physics.java:65-80) minus the host-side setters, which stay in Java. */
int plg_create(int dim, int64_t capacity, plg_ctx** out);

int plg_destroy(plg_ctx* ctx);

/* Settings: Physics.settings (Physics.java:13, PhysicsSettings.java:8-38).
 * A change of rmax re-bins the particles before the next step. */
int plg_set_settings(plg_ctx* ctx, const plg_settings* s);
int plg_get_settings(plg_ctx* ctx, plg_settings* out);

/* Type matrix: settings.matrix (Matrix.java:3-8, DefaultMatrix.java).
 * `m` is row-major n x n doubles, m[i*n+j] = matrix.get(i, j); 1 <= n <= 1024. */
int plg_set_matrix(plg_ctx* ctx, int32_t n, const double* m);

/* Replaces the whole particle state: Physics.particles (Physics.java:15).
 * pos, vel: double[3n] interleaved (z ignored in 2D); type: int32[n] with
 * 0 <= type < matrix size; positions must lie in [0,1] per axis and be
 * finite (use ensurePosition, Physics.java:499-505, before uploading).
 * vel may be NULL (zero velocities).  Ids are assigned 0..n-1. */
int plg_upload(plg_ctx* ctx, int64_t n, const double* pos, const double* vel,
               const int32_t* type);

/* nsteps x Physics.update() (Physics.java:112-134).  Blocks until done.
 * Checks the stop flag between steps: a set flag ends the call early with
 * PLG_E_STOPPED and is cleared (Physics.forceUpdateStop, Physics.java:149). */
int plg_step(plg_ctx* ctx, int32_t nsteps);

/* Enqueues nsteps without waiting; pair with plg_sync. */
int plg_step_async(plg_ctx* ctx, int32_t nsteps);

/* Waits for all enqueued work, polling at most timeout_s seconds
 * (<= 0: no limit), and reports kernel error words.  PLG_E_TIMEOUT when the
 * wait runs out; the context stays usable. */
int plg_sync(plg_ctx* ctx, double timeout_s);

/* Copies the current state to host buffers in the current (cell-sorted)
 * order: the layout of PhysicsSnapshot.write (app/PhysicsSnapshot.java:36-62)
 * plus the particle ids.  Any pointer may be NULL to skip that array. */
int plg_download(plg_ctx* ctx, double* pos, double* vel, int32_t* type,
                 int32_t* id);

/* plg_step(ctx, nsteps) then plg_download(ctx, pos, vel, type, id), with the
 * same results, errors and stop behaviour (a stopped call writes nothing).
 * This is the app's update-then-snapshot pair: updatePhysics
 * (app/Main.java:292-295) followed by physicsSnapshot.take
 * (app/Main.java:600-603, app/PhysicsSnapshot.java:24-62).  When every
 * non-NULL array is device-accessible, the last step's force kernel writes
 * the snapshot as it finishes each particle, so the host-link transfer
 * overlaps the step.
 * Device-accessible means page-locked, or pageable memory on a device with
 * coherent pageable access.  Otherwise the call is plg_step followed by
 * plg_download. */
int plg_step_download(plg_ctx* ctx, int32_t nsteps, double* pos, double* vel,
                      int32_t* type, int32_t* id);

/* *fused = 1 when plg_step_download with these arrays (and the current
 * settings and particle count) writes them from the force kernel, else 0. */
int plg_step_download_fuses(plg_ctx* ctx, const double* pos, const double* vel,
                            const int32_t* type, const int32_t* id,
                            int32_t* fused);

int plg_particle_count(plg_ctx* ctx, int64_t* n);

/* ---- initialisers on the device ------------------------------------------ */

/* The app's catalogues as seeded generators (Philox4x64-10 per particle:
 * key (seed, 0), counter (index, stream, 0, 0)).  Position setters of
 * app/PositionSetterProvider.java:16-119 (UNIFORM is
 * backend/DefaultPositionSetter.java); type setters of
 * app/TypeSetterProvider.java:11-45 (RANDOM is DefaultTypeSetter); matrix
 * generators of app/MatrixGeneratorProvider.java:13-79 (RANDOM is
 * DefaultMatrix.randomize).  3D worlds get a third coordinate (uniform; normal
 * for CENTERED): an extension, the app is 2D. */
#define PLG_POS_UNIFORM 0
#define PLG_POS_CENTERED 1
#define PLG_POS_UNIFORM_CIRCLE 2
#define PLG_POS_CENTERED_CIRCLE 3
#define PLG_POS_RING 4
#define PLG_POS_RAINBOW_RING 5
#define PLG_POS_COLOR_BATTLE 6
#define PLG_POS_COLOR_WHEEL 7
#define PLG_POS_LINE 8
#define PLG_POS_SPIRAL 9
#define PLG_POS_RAINBOW_SPIRAL 10
#define PLG_TYPE_RANDOM 0
#define PLG_TYPE_RANDOMIZE_10 1
#define PLG_TYPE_SLICES 2
#define PLG_TYPE_ONION 3
#define PLG_TYPE_ROTATE 4
#define PLG_TYPE_FLIP 5
#define PLG_TYPE_MORE_OF_FIRST 6
#define PLG_TYPE_KILL_STILL 7
#define PLG_MATRIX_RANDOM 0
#define PLG_MATRIX_SYMMETRY 1
#define PLG_MATRIX_CHAINS 2
#define PLG_MATRIX_CHAINS_2 3
#define PLG_MATRIX_CHAINS_3 4
#define PLG_MATRIX_SNAKES 5
#define PLG_MATRIX_ZERO 6

/* Replaces the particles with n new ones made on the device the way
 * Physics.setParticleCount makes them from nothing (Physics.java:190-196,
 * 285-295): type from the type setter, then position from the position
 * setter, ensurePosition, velocity 0; ids 0..n-1. */
int plg_generate(plg_ctx* ctx, int64_t n, int32_t position_setter, int32_t type_setter,
                 uint64_t seed);
/* Physics.setPositions (Physics.java:166-168) with a catalogue setter. */
int plg_apply_position_setter(plg_ctx* ctx, int32_t setter, uint64_t seed);
/* Physics.setTypes (Physics.java:509-511) with a catalogue type setter. */
int plg_apply_type_setter(plg_ctx* ctx, int32_t setter, uint64_t seed);
/* A catalogue matrix, row-major size x size doubles.  Host only. */
int plg_generate_matrix(int32_t generator, int32_t size, uint64_t seed, double* out);

/* ---- headless splat ------------------------------------------------------ */

/* The app's default particle shaders (resources/shaders/default.vert, .geom,
 * .frag) without a graphics API: each particle a disk of diameter `size`
 * (world units) in its type's palette colour, with periodic copies across
 * the edges when `wrap`; 16 samples per pixel, the last particle in the
 * current order wins each sample (opaque "normal" blending), samples
 * averaged.  Camera as NormalizedDeviceCoordinates: centre (cam_x, cam_y)
 * and dimensions (cam_w, cam_h); top_left is the shader's camTopLeft.  The
 * save thumbnail of app/Main.java:1143-1188 is centre (0.5, 0.5), dims
 * (1, 1), top_left (0, 0), size 0.015, wrap 0. */
typedef struct plg_render_params {
    int32_t width, height;
    double cam_x, cam_y, cam_w, cam_h;
    double top_left_x, top_left_y;
    double size;
    int32_t wrap;
    int32_t reserved;
} plg_render_params;
/* palette_rgba: ncolors x {r, g, b, a} floats in [0, 1] (types beyond the
 * palette take its last colour); out_rgba: width x height x 4 bytes, rows
 * bottom to top. */
int plg_render(plg_ctx* ctx, const plg_render_params* params, int32_t ncolors,
               const float* palette_rgba, uint8_t* out_rgba);

/* ---- edits on the device (no re-upload) --------------------------------- */

/* A cursor of app/cursors/Cursor.java:10-13: position, size and shape
 * (CircleCursorShape, SquareCursorShape, InfinityCursorShape).  A particle
 * is inside when its delta to the cursor (wrapped when settings.wrap),
 * divided by size, passes the shape's test (Cursor.java:16-35). */
#define PLG_CURSOR_CIRCLE 0
#define PLG_CURSOR_SQUARE 1
#define PLG_CURSOR_INFINITY 2
typedef struct plg_cursor {
    double x, y, z;
    double size;
    int32_t shape;
    int32_t reserved;
} plg_cursor;

/* Cursor.countSelection (Cursor.java:44-50). */
int plg_cursor_count(plg_ctx* ctx, const plg_cursor* cursor, int64_t* count);
/* Cursor action MOVE (app/Main.java:540-551): every selected particle moves
 * by (dx, dy, dz) and is wrapped or clamped (ensurePosition). */
int plg_cursor_move(plg_ctx* ctx, const plg_cursor* cursor, double dx, double dy, double dz,
                    int64_t* moved);
/* Cursor action DELETE (app/Main.java:567-578): the unselected particles
 * stay, in their order. */
int plg_cursor_delete(plg_ctx* ctx, const plg_cursor* cursor, int64_t* deleted);
/* Appends particles at the end (cursor action BRUSH, app/Main.java:552-566;
 * growth in Physics.setParticleCount, Physics.java:212-219), in the
 * plg_upload layouts.  Their ids continue after every id handed out so
 * far. */
int plg_append(plg_ctx* ctx, int64_t n, const double* pos, const double* vel,
               const int32_t* type);
/* Reorders and truncates: particle k becomes the old particle src[k]
 * (k < n_new, distinct indices of the current order).  The shuffle and
 * truncation of Physics.setParticleCount (Physics.java:200-211) and of
 * ExtendedPhysics.setTypeCount (app/ExtendedPhysics.java:41-130). */
int plg_permute(plg_ctx* ctx, int64_t n_new, const int32_t* src);
/* New types for all particles, in the current order (Physics.ensureTypes,
 * setTypes: Physics.java:266-272, 509-511). */
int plg_set_types(plg_ctx* ctx, const int32_t* type);

/* Thread-safe stop request: Physics.forceUpdateStop (Physics.java:149-151)
 * and Physics.kill (Physics.java:156-158).  Takes effect between steps. */
int plg_request_stop(plg_ctx* ctx);

/* Message of the last failing call on this context ("" if none). */
const char* plg_last_error(plg_ctx* ctx);

/* The cudaStream_t every kernel of this context is launched on, so a caller
 * can order its own work and record CUDA events against it. */
int plg_get_stream(plg_ctx* ctx, void** stream);

/* 1 (default): each step is one CUDA graph launch.  0: plain launches. */
int plg_set_use_graph(plg_ctx* ctx, int32_t on);

/* ---- measurement ------------------------------------------------------ */

/* Kernel ids for plg_profile_read. */
#define PLG_K_SCAN 0    /* per-cell counts -> offsets (one pass) */
#define PLG_K_SCATTER 1 /* particle index -> its cell's range      */
#define PLG_K_GATHER 2  /* stable in-cell order, A -> B            */
#define PLG_K_FORCE 3   /* neighbour loop + integration + counting */
#define PLG_K_COUNT 4

/* Force kernel tile variant of this world (see PLG_TILE_VARIANTS below).
 * Until plg_set_tile or plg_autotune chooses one, 2D worlds under 300,000
 * particles use variant 2 and all others variant 0.  Every variant gives
 * the same bits. */
int plg_set_tile(plg_ctx* ctx, int32_t variant);
int plg_get_tile(plg_ctx* ctx, int32_t* variant);
/* Times `steps` steps of every tile variant on the world as it is
 * (restoring the particle state after each trial, so the world does not
 * move), keeps the fastest and reports it in *chosen; ms_per_step (may be
 * NULL) receives PLG_TILE_VARIANTS times.  Allocates a temporary copy of the
 * state.  A world below 3 cells per axis has no tiles: *chosen is the
 * current variant. */
int plg_autotune(plg_ctx* ctx, int32_t steps, int32_t* chosen, double* ms_per_step);

/* When on, steps run as plain launches bracketed by CUDA events on the
 * context's stream; plg_profile_read returns per-kernel totals since the
 * last enable.  Turning it on clears the totals. */
int plg_profile_enable(plg_ctx* ctx, int32_t on);
int plg_profile_read(plg_ctx* ctx, int32_t kernel, double* total_ms,
                     int64_t* launches);
const char* plg_kernel_name(int32_t kernel);

/* Runs one step like plg_step with the instrumented force kernel and copies,
 * per particle of the step's cell-sorted order (the order plg_download
 * returns after it):
 *   cell      int32[n]   getContainerIndex of the pre-step position
 *   pairs     int32[n]   interacting pairs (d2 != 0 && d2 <= rmax^2)
 *   hash_sum  uint64[n]  sum of mix64(id_j) over those pairs
 *   hash_xor  uint64[n]  xor of mix64(id_j)
 *   acc       float[dim*n] sum of Accelerator.accelerate(a, r/rmax) before
 *                        the rmax*force*dt scale (Physics.java:435-437)
 * and, in *candidates, the number of pairs tested.  Any pointer may be NULL.
 * mix64 is the splitmix64 finaliser of the id. */
int plg_debug_step(plg_ctx* ctx, int32_t* cell, int32_t* pairs,
                   uint64_t* hash_sum, uint64_t* hash_xor, float* acc,
                   int64_t* candidates);

/* Targets of the last step that the tiled force kernel recomputed in its
 * closing global-memory pass (targets with a pair that needs the FP64
 * decision).  Waits for the context's stream. */
int plg_step_stats(plg_ctx* ctx, int64_t* deferred);

/* Device FP32 FMA throughput microbenchmark on the current device, in
 * TFLOP/s (an FFMA counts 2 flops).  Runs for about 0.1 s. */
int plg_probe_fp32_peak(double* tflops);

/* Device special-function-unit throughput microbenchmark (rsqrt.approx, the
 * force loop's one SFU operation per candidate pair), in Gop/s.  Runs for
 * about 0.1 s. */
int plg_probe_sfu_peak(double* gops);

/* Test hook for the bounded device waits: runs the step's scan kernel on a
 * private two-tile problem where its look-back wait can never be satisfied,
 * so the wait runs out (about 0.3 to 3 s), the kernel raises its error word
 * and returns, and the context stays usable.  *status receives the kernel's
 * error word (bit 3: a bounded wait ran out), *seconds (may be NULL) the
 * kernel's duration.  Uses the current device. */
int plg_test_scan_wait(uint32_t* status, double* seconds);

/* ---- batched worlds ---------------------------------------------------- */

/* Many independent worlds advanced together: one step launch sorts and
 * steps every world (no counterpart in the reference, which runs one
 * Physics at a time; each world computes exactly what plg_step computes for
 * it).  All worlds of a batch have the same dimension and at least 3 cells
 * per axis (rmax <= 1/3).  One thread drives a batch. */
typedef struct plg_batch plg_batch;

/* One world: settings (plg_set_settings), matrix (plg_set_matrix) and its
 * initial particles (plg_upload layouts).  Host buffers are read during the
 * call only; page-locked buffers are read in place. */
typedef struct plg_world_desc {
    plg_settings settings;
    int32_t ntypes;          /* matrix size, 1..1024 (<= 16: matrix in shared memory) */
    const double* matrix;    /* ntypes x ntypes, row-major */
    int64_t n;               /* particles */
    const double* pos;       /* double[3n], each coordinate in [0,1] */
    const double* vel;       /* double[3n] or NULL */
    const int32_t* type;     /* int32[n], 0 <= type < ntypes */
} plg_world_desc;

/* The checks plg_batch_update applies to one world description, without a
 * device: PLG_OK, PLG_E_INVALID_ARG, PLG_E_UNSUPPORTED or PLG_E_CAPACITY.
 * Host only. */
int plg_world_check(int32_t dim, const plg_world_desc* world);
/* Device bytes a world occupies in a batch (particles, cells, tables).
 * Host only; -1 for a bad argument. */
int64_t plg_world_device_bytes(int32_t dim, const plg_world_desc* world);

/* Capacities: particles, worlds (<= 1024) and cells over all worlds. */
int plg_batch_create(int32_t dim, int64_t particle_capacity, int32_t world_capacity,
                     int64_t cell_capacity, plg_batch** out);
int plg_batch_destroy(plg_batch* batch);

/* Removes `nremove` worlds and adds `nadd`, then lays the batch out again
 * (one pass over all particles); ids_out[k] receives the id of add[k].
 * Everything is checked before anything changes: PLG_E_CAPACITY,
 * PLG_E_INVALID_ARG (unknown id, bad description), PLG_E_UNSUPPORTED
 * (rmax > 1/3, accelerator kind). */
int plg_batch_update(plg_batch* batch, int32_t nremove, const int32_t* remove_ids,
                     int32_t nadd, const plg_world_desc* add, int32_t* ids_out);

/* nsteps x Physics.update() for every world; the blocking form waits. */
int plg_batch_step(plg_batch* batch, int32_t nsteps);
int plg_batch_step_async(plg_batch* batch, int32_t nsteps);
int plg_batch_sync(plg_batch* batch, double timeout_s);

/* Step budget of one world: after `steps` more batch steps the world
 * freezes (keeps its state while the others advance).  steps < 0: no limit
 * (the default).  plg_batch_steps_left reports -1 for no limit. */
int plg_batch_set_steps(plg_batch* batch, int32_t id, int32_t steps);
int plg_batch_steps_left(plg_batch* batch, int32_t id, int32_t* steps);

/* One world's state in its cell-sorted order, like plg_download. */
int plg_batch_download(plg_batch* batch, int32_t id, double* pos, double* vel,
                       int32_t* type, int32_t* pid);
/* A world's particle count, first sorted slot and first global cell. */
int plg_batch_world_info(plg_batch* batch, int32_t id, int64_t* n, int64_t* first_slot,
                         int64_t* first_cell);
int plg_batch_counts(plg_batch* batch, int32_t* nworlds, int64_t* nparticles, int64_t* ncells);
int plg_batch_set_use_graph(plg_batch* batch, int32_t on);
int plg_batch_get_stream(plg_batch* batch, void** stream);
const char* plg_batch_last_error(plg_batch* batch);
int plg_batch_step_stats(plg_batch* batch, int64_t* deferred);
/* Force kernel tile variants (threads = targets per block, staging size):
 * 2D: 0 = 256 targets / 1536 staged candidates, 1 = 256 / 3072 (dense
 * worlds), 2 = 128 / 1024 (small worlds); 3D: 0 = 128 / 2176, 1 = 64 / 1024
 * (sparse worlds), 2 = 128 / 2816 (dense worlds).  All give the same bits.  Each world
 * of a batch has its own variant; a step launches the force kernel once per
 * variant in use.  The cell size is not a tuning choice: it is rmax (the
 * sorted order the reference exposes depends on it).  A single world has
 * the same choice: plg_set_tile / plg_autotune. */
#define PLG_TILE_VARIANTS 3
/* Every world (and every world added later) takes `variant`. */
int plg_batch_set_tile(plg_batch* batch, int32_t variant);
int plg_batch_get_tile(plg_batch* batch, int32_t* variant);
/* One world's variant. */
int plg_batch_set_world_tile(plg_batch* batch, int32_t id, int32_t variant);
int plg_batch_get_world_tile(plg_batch* batch, int32_t id, int32_t* variant);
/* The ids of the batch's worlds in device order (plg_batch_counts gives
 * their number). */
int plg_batch_world_ids(plg_batch* batch, int32_t* ids);
/* Autotuner, one variant for the batch: times `steps` steps of every tile
 * variant on the batch as it is (restoring the state after each trial, so
 * no world moves and no step budget is spent), gives every world the
 * fastest and reports it; ms_per_step (may be NULL) receives
 * PLG_TILE_VARIANTS times.  Allocates a temporary copy of the state. */
int plg_batch_autotune(plg_batch* batch, int32_t steps, int32_t* chosen, double* ms_per_step);
/* Autotuner, one variant per world: a trial per variant measures each
 * world's force-kernel SM time (its blocks' cycles over the variant's
 * resident blocks per SM); every world takes its cheapest variant, and the
 * resulting mix is kept only if it times faster than the best single
 * variant (else every world takes that).  State restored as above.
 * ms_by_variant (may be NULL): PLG_TILE_VARIANTS + 1 step times (each
 * variant alone, then the mix); variants (may be NULL): each world's
 * choice in plg_batch_world_ids order. */
int plg_batch_autotune_worlds(plg_batch* batch, int32_t steps, int32_t* variants, double* ms_by_variant);

/* plg_debug_step over the whole batch: per sorted slot (worlds one after
 * another), cell = global cell index (world's first cell + its own). */
int plg_batch_debug_step(plg_batch* batch, int32_t* cell, int32_t* pairs,
                         uint64_t* hash_sum, uint64_t* hash_xor, float* acc,
                         int64_t* candidates);

/* ---- serving ----------------------------------------------------------- */

/* A request loop over batched worlds (no counterpart in the reference):
 * requests (a world and a step count) are submitted from any thread; a
 * native scheduler thread admits them first-in-first-out as the device
 * memory budget and the batch capacities allow, keeps their worlds resident,
 * packs every active world into one batch per dimension (the 2D and 3D
 * batches run concurrently on their own streams), advances them in chunks
 * of at most max_chunk_steps steps (never past a world's own count) and
 * hands back each final state.  Membership changes overlap the steps: an
 * admitted world is converted (or generated) into the batch's free tail on
 * a side stream while a chunk runs and joins at the next chunk boundary; a
 * finished world stays frozen in place and is downloaded on the side stream
 * while the next chunk runs; retired worlds are compacted away in one pass
 * only when they take a quarter of the batch or block an admission.  Each
 * result is bit for bit the world run alone. */
typedef struct plg_server plg_server;

typedef struct plg_server_config {
    int64_t memory_budget_bytes;   /* admission limit: sum of resident worlds' plg_world_device_bytes */
    int64_t particle_capacity[2];  /* batch capacities [2D, 3D] (allocated at create) */
    int64_t cell_capacity[2];
    int32_t max_worlds_per_batch;  /* <= 1024 */
    int32_t max_chunk_steps;       /* steps between admissions */
    int32_t tile_variant;          /* force kernel tile variant of newly admitted worlds */
    int32_t autotune_interval_ms;  /* > 0: at a chunk boundary at least this long after the last,
                                      re-tune the batch per world (plg_batch_autotune_worlds, one
                                      step per trial; results do not change); 0: off */
} plg_server_config;

#define PLG_REQ_QUEUED 0
#define PLG_REQ_RUNNING 1
#define PLG_REQ_DONE 2

typedef struct plg_server_stats_t {
    int64_t submitted, completed, queued, running;
    int64_t resident_bytes, peak_resident_bytes;
    double particle_steps;   /* advanced so far, all worlds */
    double busy_s, wall_s;   /* device time of the step chunks (both batches) / time since create */
    double latency_p50_ms, latency_p99_ms, latency_mean_ms;  /* submit -> result on host */
    double busy_dim_s[2];    /* device time of the step chunks of the 2D and of the 3D batch */
    int64_t compactions;     /* re-layout passes that dropped finished worlds */
    int64_t autotunes;       /* per-world tuner runs */
} plg_server_stats_t;

int plg_server_create(const plg_server_config* cfg, plg_server** out);
/* Copies the world; PLG_E_CAPACITY for a request that could never fit. */
int plg_server_submit(plg_server* server, int32_t dim, const plg_world_desc* world, int32_t steps,
                      int64_t* request_id);

/* A world given by its generator instead of its particles: n particles made
 * on the device at admission exactly as plg_generate makes them in a
 * single-world context (Physics.setParticleCount from nothing with catalogue
 * setters, Physics.java:190-196, 285-295), so a request carries a few bytes
 * however large its world.  `world.pos`, `world.vel` and `world.type` are
 * ignored. */
typedef struct plg_world_gen {
    plg_world_desc world;     /* settings, ntypes, matrix, n */
    int32_t position_setter;  /* PLG_POS_* */
    int32_t type_setter;      /* PLG_TYPE_* */
    uint64_t seed;
} plg_world_gen;
int plg_server_submit_generated(plg_server* server, int32_t dim, const plg_world_gen* world, int32_t steps,
                                int64_t* request_id);
/* Waits for a request (timeout_s <= 0: no limit); *state = PLG_REQ_*. */
int plg_server_wait(plg_server* server, int64_t request_id, double timeout_s, int32_t* state);
/* Waits for any request to finish (timeout_s <= 0: no limit) and gives its
 * id; every finished request is given once, in completion order.
 * PLG_E_TIMEOUT when none finished in time. */
int plg_server_wait_any(plg_server* server, double timeout_s, int64_t* request_id);
/* Copies a finished request's final state (cell-sorted order, like
 * plg_download) and releases it; any pointer may be NULL. */
int plg_server_result(plg_server* server, int64_t request_id, double* pos, double* vel, int32_t* type,
                      int32_t* pid, int64_t* n, double* latency_ms);
int plg_server_stats(plg_server* server, plg_server_stats_t* out);
const char* plg_server_last_error(plg_server* server);
int plg_server_destroy(plg_server* server);

/* ---- cell sort without allocation ------------------------------------- */

/* Capacity of plg_sort_cells_noalloc's fixed device scratch. */
#define PLG_NOALLOC_MAX_PARTICLES (1 << 18)
#define PLG_NOALLOC_MAX_CELLS (1 << 18)

/* No counterpart in the reference.  Computes, for positions already in
 * device memory, the stable cell-sorted order of makeContainers
 * (Physics.java:309-354) with cells from getContainerIndex in FP64
 * (Physics.java:362-375), and allocates nothing: its scratch is one fixed
 * device array of about 4.2 MB per device, for callers that must not
 * allocate device memory while they run (a frame loop owning its position
 * buffer, where cudaFree would wait for the whole device; a fixed memory
 * budget).
 *   pos         device double[3n], PhysicsSnapshot layout (z unused in 2D)
 *   perm        device uint32[n]: perm[s] = index of the particle at sorted
 *               slot s; ties in a cell keep index order
 *   cell_start  device uint32[nx^dim + 1], 16-byte aligned: first slot of
 *               each cell, last = n
 *   status      device uint32 or NULL; the caller zeroes it.  Kernels OR in
 *               1 (a position outside [0,1] or NaN: above the box it is
 *               binned as 1, below it or NaN as 0) and 8 (a bounded device
 *               wait ran out: cell_start is then not valid).  With NULL
 *               neither is reported, so a caller that cannot rule out a
 *               stalled device should pass a status word.
 *   stream      cudaStream_t to enqueue on (NULL: the default stream)
 * Enqueues the work and returns.  n > PLG_NOALLOC_MAX_PARTICLES or
 * nx^dim > PLG_NOALLOC_MAX_CELLS is rejected with PLG_E_CAPACITY, host or
 * other-device pointers with PLG_E_INVALID_ARG, before anything is enqueued.
 * Cost: linear in n except for crowded cells: the in-cell order takes
 * n_c^2 / 32 warp steps for a cell of n_c particles (100,000 particles on
 * one point: about a millisecond; the 2^18 maximum in one cell: several).
 * The first call on a device sets up the scratch address for that device
 * (cudaGetSymbolAddress, which may load the module): make it before any
 * stream capture.  Each call zeroes its own counters on `stream`.  Calls
 * that overlap in time on one device share the scratch and race: serialise
 * them. */
int plg_sort_cells_noalloc(int32_t dim, double rmax, int64_t n,
                           const double* pos, uint32_t* perm,
                           uint32_t* cell_start, uint32_t* status,
                           void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PLGPU_H */
