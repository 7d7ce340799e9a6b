/*
 * plg_oracle.c — CPU FP64 restatement of the Particle Life physics step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: the tests, the smoke
 * check and the bench's CPU-baseline / reference arm load it.  The product
 * path (the CUDA library) never links or calls it.
 *
 * It restates, in plain C with IEEE double arithmetic and no contraction
 * (built with -ffp-contract=off), the step of tom-mohr/particle-life-app
 * (paths relative to src/main/java/com/particle_life/):
 *
 *   backend/Physics.java:112-134   update / updateParticles
 *   backend/Physics.java:309-354   makeContainers (stable counting sort)
 *   backend/Physics.java:362-375   getContainerIndex
 *   backend/Physics.java:377-395   wrapContainerX / wrapContainerY
 *   backend/Physics.java:397-441   updateVelocity
 *   backend/Physics.java:443-450   updatePosition
 *   backend/Physics.java:460-470   connection
 *   backend/Physics.java:499-505   ensurePosition
 *   backend/Range.java:40-96       wrap / wrapConnection / clamp
 *   backend/LoadDistributor.java:37-66  chunking of the parallel phases
 *   app/Main.java:275-280          the default Accelerator lambda
 *
 * Parity status: UNPINNED.  The reference is Java 21 + JOML 1.10.1 and
 * neither a JDK nor JOML is available, and the reference ships no tests or
 * golden vectors.  JOML's vector arithmetic is restated from its published
 * semantics: lengthSquared = x*x + (y*y + z*z) and mulAdd = x*a + b, both
 * unfused (JOML's default, joml.useMathFma=false).  The oracle is
 * cross-checked against an independent pure-Python restatement
 * (tests/golden/make_golden.py) and hand-derived known answers.
 *
 * 2D is the reference's own path (z forced to 0, 9-cell stencil).  3D has no
 * reference path: it extends every per-axis rule to z (27-cell stencil,
 * offsets ordered z-major, then y, then x).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef struct orc_settings {
    double rmax;
    double friction;
    double force;
    double dt;
    double beta;
    int32_t wrap;
    int32_t pad;
} orc_settings;

/* Optional per-particle outputs, indexed in the post-sort order. */
typedef struct orc_debug {
    int32_t* cell;     /* getContainerIndex of each particle (pre-step pos) */
    int32_t* pairs;    /* interacting pairs per particle                    */
    uint64_t* hsum;    /* sum of mix64(id) of interacting partners          */
    uint64_t* hxor;    /* xor of mix64(id)                                  */
    double* acc;       /* dim * n: sum of accelerate(a, r / rmax)           */
    double* fscale;    /* sum over interacting pairs of max(1, |a_ij|): the
                          bound of each term's magnitude |f| and so the
                          scale of its rounding error (f itself vanishes at
                          r = beta and r = 1, so |term| is no error scale) */
    int64_t candidates;/* out: pairs tested (j != i)                        */
} orc_debug;

/* splitmix64 output function (Steele, Lea, Flood 2014) on id + gamma. */
static inline uint64_t mix64(uint64_t id) {
    uint64_t z = id + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

uint64_t orc_mix64(uint64_t id) { return mix64(id); }

/* ---- Range (backend/Range.java) ---------------------------------------- */

/* Range.wrap(double), Range.java:46-57: repeated +-1 into [0,1). */
static double range_wrap(double value) {
    if (value < 0) {
        do {
            value += 1;
        } while (value < 0);
        return value;
    }
    while (value >= 1) {
        value -= 1;
    }
    return value;
}

/* Range.wrapConnection(double), Range.java:74-81: single wind to [-0.5,0.5). */
static double range_wrap_connection(double value) {
    if (value < -0.5) {
        return value + 1;
    } else if (value >= 0.5) {
        return value - 1;
    }
    return value;
}

/* Range.clamp(double), Range.java:89-96. */
static double range_clamp(double val) {
    if (val < 0) {
        return 0;
    } else if (val > 1) {
        return 1;
    }
    return val;
}

double orc_range_wrap(double v) { return range_wrap(v); }
double orc_range_wrap_connection(double v) { return range_wrap_connection(v); }
double orc_range_clamp(double v) { return range_clamp(v); }

/* ---- Accelerator (app/Main.java:275-280) -------------------------------- */

/* accelerate(a, pos): pos is r / rmax (|pos| <= 1).  Writes pos * (f / dist)
 * into out.  dist = pos.length() = sqrt(x*x + (y*y + z*z)). */
static void accelerate(double a, double beta, const double pos[3], double out[3]) {
    double dist = sqrt(pos[0] * pos[0] + (pos[1] * pos[1] + pos[2] * pos[2]));
    double force = dist < beta ? (dist / beta - 1)
                               : a * (1 - fabs(1 + beta - 2 * dist) / (1 - beta));
    double k = force / dist;
    out[0] = pos[0] * k;
    out[1] = pos[1] * k;
    out[2] = pos[2] * k;
}

/* Exposed for the known-answer tests: |accelerate(a, (dist,0,0))| signed. */
double orc_accel_scalar(double a, double beta, double dist) {
    double p[3] = {dist, 0.0, 0.0}, o[3];
    accelerate(a, beta, p, o);
    return o[0];
}

/* ---- grid (Physics.java:82-85, 362-395) --------------------------------- */

/* nx = (int) Math.floor(1 / containerSize), containerSize = rmax. */
int32_t orc_grid_n(double rmax) { return (int32_t)floor(1 / rmax); }

/* getContainerIndex per axis: (int)(x / cs), then cx == nx -> nx - 1.
 * Positions are in [0,1], so the Java (int) truncation equals C's. */
static inline int axis_cell(double x, double cs, int n) {
    int c = (int)(x / cs);
    if (c == n) c = n - 1;
    return c;
}

int32_t orc_container_index(int dim, double x, double y, double z, double rmax) {
    int n = orc_grid_n(rmax);
    int cx = axis_cell(x, rmax, n), cy = axis_cell(y, rmax, n);
    int64_t ci = cx + (int64_t)cy * n;
    if (dim == 3) ci += (int64_t)axis_cell(z, rmax, n) * n * n;
    return (int32_t)ci;
}

/* wrapContainerX/Y, Physics.java:377-395 (single wind). */
static inline int wrap_container(int c, int n) {
    if (c < 0) return c + n;
    if (c >= n) return c - n;
    return c;
}

/* ---- world -------------------------------------------------------------- */

typedef struct world {
    int dim;
    int64_t n;
    double* pos;  /* [3n] */
    double* vel;  /* [3n] */
    int32_t* type;
    int32_t* id;
    int ntypes;
    const double* matrix; /* row-major ntypes x ntypes */
    const orc_settings* s;
    double cs;
    int nx;
    int64_t ncells;
    int64_t* containers; /* end offsets after makeContainers */
    orc_debug* dbg;
    int64_t* cand; /* per-thread candidate counters */
} world;

/* makeContainers, Physics.java:309-354: count, exclusive offsets, stable
 * scatter, swap.  Afterwards containers[c] is the end offset of cell c. */
static int make_containers(world* w) {
    int64_t n = w->n;
    int64_t* cnt = w->containers;
    memset(cnt, 0, sizeof(int64_t) * (size_t)w->ncells);
    int32_t* ci = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    double* p2 = (double*)malloc(sizeof(double) * 3 * (size_t)(n > 0 ? n : 1));
    double* v2 = (double*)malloc(sizeof(double) * 3 * (size_t)(n > 0 ? n : 1));
    int32_t* t2 = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    int32_t* i2 = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    if (!ci || !p2 || !v2 || !t2 || !i2) {
        free(ci); free(p2); free(v2); free(t2); free(i2);
        return -1;
    }
    for (int64_t i = 0; i < n; i++) {
        const double* p = w->pos + 3 * i;
        int64_t c = axis_cell(p[0], w->cs, w->nx) + (int64_t)axis_cell(p[1], w->cs, w->nx) * w->nx;
        if (w->dim == 3) c += (int64_t)axis_cell(p[2], w->cs, w->nx) * w->nx * w->nx;
        ci[i] = (int32_t)c;
        cnt[c]++;
    }
    int64_t offset = 0;
    for (int64_t c = 0; c < w->ncells; c++) {
        int64_t cap = cnt[c];
        cnt[c] = offset;
        offset += cap;
    }
    for (int64_t i = 0; i < n; i++) {
        int64_t d = cnt[ci[i]]++;
        memcpy(p2 + 3 * d, w->pos + 3 * i, 3 * sizeof(double));
        memcpy(v2 + 3 * d, w->vel + 3 * i, 3 * sizeof(double));
        t2[d] = w->type[i];
        i2[d] = w->id[i];
        if (w->dbg && w->dbg->cell) w->dbg->cell[d] = ci[i];
    }
    memcpy(w->pos, p2, sizeof(double) * 3 * (size_t)n);
    memcpy(w->vel, v2, sizeof(double) * 3 * (size_t)n);
    memcpy(w->type, t2, sizeof(int32_t) * (size_t)n);
    memcpy(w->id, i2, sizeof(int32_t) * (size_t)n);
    free(ci); free(p2); free(v2); free(t2); free(i2);
    return 0;
}

/* updateVelocity(i), Physics.java:397-441. */
static void update_velocity(world* w, int64_t i, int64_t* cand) {
    const orc_settings* s = w->s;
    double* v = w->vel + 3 * i;
    const double* p = w->pos + 3 * i;
    const int dim = w->dim, nx = w->nx;

    double friction_factor = pow(s->friction, 60 * s->dt);
    v[0] = v[0] * friction_factor;
    v[1] = v[1] * friction_factor;
    v[2] = v[2] * friction_factor;

    int cx0 = (int)floor(p[0] / w->cs);
    int cy0 = (int)floor(p[1] / w->cs);
    int cz0 = dim == 3 ? (int)floor(p[2] / w->cs) : 0;
    const double rmax = s->rmax;
    const double rmax2 = s->rmax * s->rmax;
    const double scale = s->rmax * s->force * s->dt;
    const int zlo = dim == 3 ? -1 : 0, zhi = dim == 3 ? 1 : 0;

    int32_t npairs = 0;
    uint64_t hs = 0, hx = 0;
    double acc[3] = {0, 0, 0};
    double fscale = 0;

    for (int oz = zlo; oz <= zhi; oz++) {
        for (int oy = -1; oy <= 1; oy++) {
            for (int ox = -1; ox <= 1; ox++) {
                int cx = wrap_container(cx0 + ox, nx);
                int cy = wrap_container(cy0 + oy, nx);
                int cz = dim == 3 ? wrap_container(cz0 + oz, nx) : 0;
                if (s->wrap) {
                    cx = wrap_container(cx, nx);
                    cy = wrap_container(cy, nx);
                    if (dim == 3) cz = wrap_container(cz, nx);
                } else {
                    if (cx < 0 || cx >= nx || cy < 0 || cy >= nx) continue;
                    if (dim == 3 && (cz < 0 || cz >= nx)) continue;
                }
                int64_t ci = cx + (int64_t)cy * nx + (int64_t)cz * nx * nx;
                int64_t start = ci == 0 ? 0 : w->containers[ci - 1];
                int64_t stop = w->containers[ci];
                for (int64_t j = start; j < stop; j++) {
                    if (i == j) continue;
                    (*cand)++;
                    const double* q = w->pos + 3 * j;
                    double r[3];
                    r[0] = q[0] - p[0];
                    r[1] = q[1] - p[1];
                    r[2] = dim == 3 ? q[2] - p[2] : 0.0;
                    if (s->wrap) {
                        r[0] = range_wrap_connection(r[0]);
                        r[1] = range_wrap_connection(r[1]);
                        r[2] = dim == 3 ? range_wrap_connection(r[2]) : 0.0;
                    }
                    double d2 = r[0] * r[0] + (r[1] * r[1] + r[2] * r[2]);
                    if (d2 != 0 && d2 <= rmax2) {
                        r[0] = r[0] / rmax;
                        r[1] = r[1] / rmax;
                        r[2] = r[2] / rmax;
                        double a = w->matrix[(int64_t)w->type[i] * w->ntypes + w->type[j]];
                        double dv[3];
                        accelerate(a, s->beta, r, dv);
                        acc[0] += dv[0];
                        acc[1] += dv[1];
                        acc[2] += dv[2];
                        fscale += fabs(a) > 1 ? fabs(a) : 1.0;
                        v[0] = v[0] + dv[0] * scale;
                        v[1] = v[1] + dv[1] * scale;
                        v[2] = v[2] + dv[2] * scale;
                        npairs++;
                        uint64_t h = mix64((uint64_t)(uint32_t)w->id[j]);
                        hs += h;
                        hx ^= h;
                    }
                }
            }
        }
    }
    if (w->dbg) {
        if (w->dbg->pairs) w->dbg->pairs[i] = npairs;
        if (w->dbg->hsum) w->dbg->hsum[i] = hs;
        if (w->dbg->hxor) w->dbg->hxor[i] = hx;
        if (w->dbg->acc) {
            for (int k = 0; k < dim; k++) w->dbg->acc[(int64_t)dim * i + k] = acc[k];
        }
        if (w->dbg->fscale) w->dbg->fscale[i] = fscale;
    }
}

/* updatePosition(i), Physics.java:443-450, with ensurePosition 499-505. */
static void update_position(world* w, int64_t i) {
    double* p = w->pos + 3 * i;
    const double* v = w->vel + 3 * i;
    const double dt = w->s->dt;
    p[0] = v[0] * dt + p[0];
    p[1] = v[1] * dt + p[1];
    p[2] = v[2] * dt + p[2];
    if (w->s->wrap) {
        p[0] = range_wrap(p[0]);
        p[1] = range_wrap(p[1]);
        p[2] = w->dim == 3 ? range_wrap(p[2]) : 0.0;
    } else {
        p[0] = range_clamp(p[0]);
        p[1] = range_clamp(p[1]);
        p[2] = w->dim == 3 ? range_clamp(p[2]) : 0.0;
    }
}

/* LoadDistributor.distributeLoadEvenly, LoadDistributor.java:37-66:
 * chunks of ceil(n / threads), one task per chunk, joined before return. */
typedef struct task {
    world* w;
    int64_t start, stop;
    int phase;
    int64_t cand;
} task;

static void* run_task(void* arg) {
    task* t = (task*)arg;
    int64_t cand = 0; /* thread-local: task structs share cache lines */
    for (int64_t i = t->start; i < t->stop; i++) {
        if (t->phase == 0)
            update_velocity(t->w, i, &cand);
        else
            update_position(t->w, i);
    }
    t->cand = cand;
    return NULL;
}

static int64_t distribute(world* w, int phase, int threads) {
    int64_t n = w->n;
    if (n <= 0) return 0;
    if (threads < 1) threads = 1;
    int64_t length = (n + threads - 1) / threads;
    int ntask = (int)((n + length - 1) / length);
    task* ts = (task*)calloc((size_t)ntask, sizeof(task));
    pthread_t* th = (pthread_t*)calloc((size_t)ntask, sizeof(pthread_t));
    int64_t cand = 0;
    for (int k = 0; k < ntask; k++) {
        ts[k].w = w;
        ts[k].start = k * length;
        ts[k].stop = (k + 1) * length < n ? (k + 1) * length : n;
        ts[k].phase = phase;
    }
    if (ntask == 1) {
        run_task(&ts[0]);
    } else {
        for (int k = 0; k < ntask; k++) pthread_create(&th[k], NULL, run_task, &ts[k]);
        for (int k = 0; k < ntask; k++) pthread_join(th[k], NULL);
    }
    for (int k = 0; k < ntask; k++) cand += ts[k].cand;
    free(ts);
    free(th);
    return cand;
}

/*
 * One Physics.update() in place.  pos/vel are double[3n] (z kept 0 in 2D),
 * type/id int32[n]; on return the arrays are in the new cell-sorted order.
 * Returns 0, or -1 on bad arguments / allocation failure.
 */
int orc_step(int dim, int64_t n, double* pos, double* vel, int32_t* type, int32_t* id,
             int32_t ntypes, const double* matrix, const orc_settings* s, int32_t threads,
             orc_debug* dbg) {
    if ((dim != 2 && dim != 3) || n < 0 || !s || !(s->rmax > 0) || s->rmax > 1) return -1;
    world w;
    memset(&w, 0, sizeof(w));
    w.dim = dim;
    w.n = n;
    w.pos = pos;
    w.vel = vel;
    w.type = type;
    w.id = id;
    w.ntypes = ntypes;
    w.matrix = matrix;
    w.s = s;
    w.cs = s->rmax;
    w.nx = orc_grid_n(s->rmax);
    w.ncells = (int64_t)w.nx * w.nx * (dim == 3 ? w.nx : 1);
    w.dbg = dbg;
    w.containers = (int64_t*)malloc(sizeof(int64_t) * (size_t)w.ncells);
    if (!w.containers) return -1;
    if (make_containers(&w) != 0) {
        free(w.containers);
        return -1;
    }
    int64_t cand = distribute(&w, 0, threads);
    distribute(&w, 1, threads);
    if (dbg) dbg->candidates = cand;
    free(w.containers);
    return 0;
}

/* Runs `steps` updates and returns the wall time in seconds (CPU baseline). */
double orc_run(int dim, int64_t n, double* pos, double* vel, int32_t* type, int32_t* id,
               int32_t ntypes, const double* matrix, const orc_settings* s, int32_t threads,
               int32_t steps) {
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    for (int k = 0; k < steps; k++) {
        if (orc_step(dim, n, pos, vel, type, id, ntypes, matrix, s, threads, NULL) != 0) return -1.0;
    }
    clock_gettime(CLOCK_MONOTONIC, &t1);
    return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}
