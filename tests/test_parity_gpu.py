"""GPU parity: one instrumented step through the C ABI against the FP64 oracle.

Bit-exact: the sorted order (particle ids after the step), the cell of every
particle, and each particle's interacting-pair set (count, sum and xor of
splitmix64(id)).  Floating point, on the same FP32 start state:
  - accelerations (sum of Accelerator.accelerate terms): norm-wise relative
    error <= 1e-5, and per particle |a - a*| / sum_j max(1, |a_ij|) <= 1e-5
    (each term is f(r) r/|r| with |f| <= max(1, |a_ij|); f vanishes at
    r = beta and r = 1, so |term_j| itself is no error scale);
  - velocities after the step: norm-wise relative error <= 1e-5;
  - positions after the step, per coordinate: periodic distance
    <= 1.2e-7 + dt (1e-5 |v| + 1e-5 rmax force dt sum_j max(1, |a_ij|)):
    FP32 rounding of a coordinate in [0,1) (<= 6e-8) plus dt times the
    velocity error the two tolerances above allow.
The norm-wise acceleration check is skipped for worlds whose every pair sits
at a zero of the force (the exact-rmax lattice), where it is ill-conditioned.
"""
import numpy as np
import pytest

from worlds import (ACC_TOL, WorldSpec, blob_world, compare_with_oracle, f32, norm_rel, run_gpu_debug,
                    run_oracle_debug, uniform_world)

pytestmark = pytest.mark.gpu

def check_step(spec: WorldSpec, gpu, exact_only=False, normwise=True):
    g, state = run_gpu_debug(spec)
    return compare_with_oracle(spec, g, state, exact_only=exact_only, normwise=normwise)


def report(name, r):
    print(f"\n{name}: interacting pairs/particle {r['pairs']:.2f}, acceleration error norm-wise "
          f"{r.get('normwise', float('nan')):.2e}, per particle p99 {r.get('p99', float('nan')):.2e} "
          f"max {r.get('max', float('nan')):.2e}")


def test_cfg1_2d_10k(gpu):
    report("10k 2D", check_step(uniform_world(10_000, 6, 0.02, seed=1, vel_scale=0.01, dt=0.02), gpu))


def test_cfg2_2d_1m(gpu):
    r = check_step(uniform_world(1_000_000, 8, 0.0025, seed=2, vel_scale=0.01, dt=0.01), gpu)
    report("1M 2D", r)
    assert 18 < r["pairs"] < 21  # ~19.6 expected neighbours


def test_cfg3_3d_4m_blobs(gpu):
    """The 3D configuration at full size: 4M particles in 64 blobs, 16 types,
    about 40 neighbours."""
    from plgpu import workloads

    w = workloads.blob_world_3d()
    spec = WorldSpec(3, w.pos, np.zeros_like(w.pos), w.types, w.matrix, w.rmax, w.friction, w.force, w.dt)
    r = check_step(spec, gpu)
    report("4M 3D blobs", r)
    assert 38 < r["pairs"] < 42


def test_2d_clamp_with_walls(gpu):
    spec = uniform_world(20_000, 5, 0.01, seed=3, vel_scale=0.05, wrap=False)
    spec.pos[:200, 0] = 0.0
    spec.pos[200:400, 0] = 1.0
    spec.pos[400:600, 1] = 1.0
    spec.pos[600:800, :2] = 1.0
    check_step(spec, gpu)


def test_2d_last_partial_cell(gpu):
    """rmax with 1/rmax not an integer: a sliver [nx*cs, 1) beyond the last
    full cell, whose stencil differs from the binning cell's."""
    rmax = 0.0031
    spec = uniform_world(50_000, 4, rmax, seed=4)
    rng = np.random.Generator(np.random.Philox(44))
    nx = int(np.floor(1 / rmax))
    lo = nx * rmax
    k = 5000
    spec.pos[:k, 0] = f32(lo + (1 - lo) * rng.random(k))
    spec.pos[k:2 * k, 1] = f32(lo + (1 - lo) * rng.random(k))
    spec.pos[2 * k:3 * k, 0] = f32((nx - 2) * rmax + rmax * rng.random(k))  # column nx-2
    spec.pos[3 * k:3 * k + 500, :2] = f32(lo + (1 - lo) * rng.random((500, 2)))
    spec.pos[:, :2] = np.minimum(spec.pos[:, :2], np.float64(np.nextafter(np.float32(1), np.float32(0))))
    check_step(spec, gpu)


@pytest.mark.parametrize("rmax", [0.3, 0.4, 0.7])
def test_2d_small_grids(gpu, rmax):
    """nx = 3, 2, 1: with nx < 3 the reference visits a cell more than once
    and counts a pair once per visit."""
    check_step(uniform_world(1500, 4, rmax, seed=5, vel_scale=0.01), gpu)


@pytest.mark.parametrize("wrap", [True, False])
def test_2d_small_grid_clamp_and_wrap(gpu, wrap):
    check_step(uniform_world(800, 3, 0.45, seed=6, wrap=wrap), gpu)


def test_2d_many_types_matrix_in_global(gpu):
    check_step(uniform_world(40_000, 100, 0.01, seed=7, vel_scale=0.01), gpu)


def test_2d_lattice_at_exactly_rmax(gpu):
    """Neighbours at exactly rmax (d2 == rmax^2 in FP64) interact (<=);
    one ulp further they do not."""
    rmax = 2.0 ** -6
    k = 64
    xs = (np.arange(k) * rmax).astype(np.float64)
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    pos = np.zeros((k * k, 3))
    pos[:, 0] = X.ravel()
    pos[:, 1] = Y.ravel()
    n = pos.shape[0]
    rng = np.random.Generator(np.random.Philox(8))
    spec = WorldSpec(2, pos, np.zeros((n, 3)), rng.integers(0, 3, n).astype(np.int32),
                     f32(2 * rng.random((3, 3)) - 1), rmax)
    r = check_step(spec, gpu, normwise=False)
    assert r["pairs"] == 4.0
    spec.pos[:, 0] = np.nextafter(spec.pos[:, 0].astype(np.float32), np.float32(2)).astype(np.float64)
    check_step(spec, gpu, normwise=False)


def test_2d_coincident_particles(gpu):
    spec = uniform_world(5000, 4, 0.02, seed=9)
    spec.pos[100:140] = spec.pos[99]
    spec.pos[1000:1003] = spec.pos[2000]
    check_step(spec, gpu)


def test_2d_fast_particles_wrap_many_times(gpu):
    spec = uniform_world(5000, 4, 0.02, seed=10)
    rng = np.random.Generator(np.random.Philox(10))
    spec.vel[:, :2] = f32(rng.uniform(-400, 400, (spec.n, 2)))
    check_step(spec, gpu)


def test_deferred_targets_are_rare_for_uniform_worlds(gpu):
    """Only pairs within 2^-19 of rmax^2 (or coincident) need the FP64 path,
    so the tiled kernel completes nearly every target itself."""
    from plgpu.physics import GpuWorld

    for dim, n, rmax in ((2, 400_000, 0.0025), (3, 200_000, 0.02)):
        spec = uniform_world(n, 8, rmax, seed=15, dim=dim, vel_scale=0.01)
        w = GpuWorld(dim, n)
        w.set_settings(spec.rmax, spec.friction, spec.force, spec.dt, beta=spec.beta, wrap=spec.wrap)
        w.set_matrix(spec.matrix)
        w.upload(spec.pos, spec.vel, spec.types)
        w.step(3)
        assert w.deferred() < n * 1e-3
        w.close()


def test_2d_dense_clusters_overflow_shared_memory(gpu):
    """Clusters far denser than shared memory can stage: those segments are
    computed from global memory in the staged order."""
    spec = blob_world(60_000, 5, 0.01, nblobs=12, sigma=0.004, seed=14, dim=2)
    r = check_step(spec, gpu)
    assert r["pairs"] > 100


def test_3d_uniform(gpu):
    check_step(uniform_world(200_000, 16, 0.02, seed=11, dim=3, vel_scale=0.01, dt=0.01), gpu)


def test_3d_blobs_uneven_cells(gpu):
    """cfg3 shape at 1/10 size: 64 Gaussian blobs, 16 types."""
    check_step(blob_world(400_000, 16, 0.0095, seed=12, dt=0.01), gpu)


def test_empty_and_single(gpu):
    check_step(uniform_world(0, 3, 0.05, seed=13), gpu)
    check_step(uniform_world(1, 3, 0.05, seed=13), gpu)
    check_step(uniform_world(2, 3, 0.5, seed=13), gpu)


@pytest.mark.parametrize("dim", [2, 3])
def test_staged_and_global_memory_paths_agree(gpu, dim):
    """A world whose windows overflow shared memory under one tile variant
    and fit under the other: the staged and the global-memory paths walk the
    same candidates in the same order, so the two runs agree bit for bit."""
    from plgpu.batch import GpuBatch, WorldDesc

    # 2D: ~220 per cell, a 9-cell window of ~1980 candidates overflows variant
    # 0's staging (1536) and fits variant 1's (3072).  3D: ~20 per cell, a
    # 128-target tile of variant 0 stages whole, variant 1 (1024) in chunks.
    spec = (uniform_world(88_000, 5, 0.05, seed=17, vel_scale=0.01) if dim == 2 else
            uniform_world(20_000, 6, 0.1, seed=18, dim=3, vel_scale=0.01))
    runs = []
    for variant in (0, 1):
        b = GpuBatch(dim, spec.n + 1, 4, int(np.floor(1 / spec.rmax)) ** dim + 1)
        (wid,) = b.update(add=[WorldDesc(pos=spec.pos, types=spec.types, matrix=spec.matrix, rmax=spec.rmax,
                                         friction=spec.friction, force=spec.force, dt=spec.dt, beta=spec.beta,
                                         wrap=spec.wrap, vel=spec.vel)])
        b.set_tile(variant)
        b.step(3)
        runs.append(b.download(wid))
        b.close()
    for a, c in zip(*runs):
        assert np.array_equal(a, c)


def test_crowded_clamp_corner(gpu):
    """100,000 particles on one point in a corner of a clamped box (the
    crowded extreme of a clamp-mode world), beside about 20,000 others
    further than rmax from it: coincident particles do not interact (the
    reference keeps a pair only when d2 != 0), the corner cell keeps index
    order, and every other particle steps exactly as in the oracle run
    without the corner pile (the pile is out of their reach).  The step is
    timed: the in-cell ordering and the pile's own pair loop grow with the
    square of its population."""
    import time

    from plgpu.physics import GpuWorld

    rmax = 0.01
    others = uniform_world(20_000, 5, rmax, seed=91, vel_scale=0.01, wrap=False)
    far = np.linalg.norm(others.pos[:, :2], axis=1) > 3 * rmax
    others = WorldSpec(2, others.pos[far], others.vel[far], others.types[far], others.matrix, rmax, wrap=False)
    m = others.n
    pile = 100_000
    spec = WorldSpec(2, np.concatenate([others.pos, np.zeros((pile, 3))]),
                     np.concatenate([others.vel, np.zeros((pile, 3))]),
                     np.concatenate([others.types, np.zeros(pile, np.int32)]), others.matrix, rmax, wrap=False)
    w = GpuWorld(2, spec.n)
    w.set_settings(spec.rmax, spec.friction, spec.force, spec.dt, beta=spec.beta, wrap=spec.wrap)
    w.set_matrix(spec.matrix)
    w.upload(spec.pos, spec.vel, spec.types)
    w.step(1)  # warm
    w.upload(spec.pos, spec.vel, spec.types)
    t0 = time.perf_counter()
    w.step(1)
    dt = time.perf_counter() - t0
    w.upload(spec.pos, spec.vel, spec.types)
    g = w.debug_step()
    gpos, gvel, gtypes, gids = w.download()
    w.close()
    print(f"clamp corner pile of {pile:,}: one step {1e3 * dt:.1f} ms")
    corner = gids >= m
    assert corner.sum() == pile
    assert np.all(g["cell"][corner] == 0) and np.all(np.diff(gids[corner]) > 0)  # index order in the cell
    assert np.all(g["pairs"][corner] == 0) and not g["acc"][corner].any()
    assert not gpos[corner].any() and not gvel[corner].any()
    d, o = run_oracle_debug(others)
    rest = ~corner
    by_id = np.argsort(gids[rest])
    oo = np.argsort(o.ids)
    assert np.array_equal(gids[rest][by_id], o.ids[oo])
    assert np.array_equal(g["pairs"][rest][by_id], d["pairs"][oo])
    assert np.array_equal(g["hsum"][rest][by_id], d["hsum"][oo])
    assert norm_rel(g["acc"][rest][by_id].astype(np.float64), d["acc"][oo]) <= ACC_TOL
    assert dt < 5.0
