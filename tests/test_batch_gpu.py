"""Batched worlds (plg_batch_*): every world of a batch against the oracle
run on that world alone, and the same world's trajectory alone and in a
mix, across membership changes, bit for bit."""
import numpy as np
import pytest

from worlds import WorldSpec, blob_world, compare_with_oracle, uniform_world

pytestmark = pytest.mark.gpu


def desc(spec: WorldSpec):
    from plgpu.batch import WorldDesc

    return WorldDesc(pos=spec.pos, types=spec.types, matrix=spec.matrix, rmax=spec.rmax, friction=spec.friction,
                     force=spec.force, dt=spec.dt, beta=spec.beta, wrap=spec.wrap, vel=spec.vel)


def make_batch(dim, specs, extra_cells=0):
    from plgpu.batch import GpuBatch

    ncap = sum(s.n for s in specs) + 1
    ccap = sum(int(np.floor(1 / s.rmax)) ** dim for s in specs) + extra_cells + 1
    b = GpuBatch(dim, ncap * 2, 64, ccap * 2)
    ids = b.update(add=[desc(s) for s in specs])
    return b, ids


def mixed_2d_specs():
    return [
        uniform_world(30_000, 6, 0.02, seed=41, vel_scale=0.01),
        uniform_world(4_000, 3, 0.05, seed=42, vel_scale=0.02, dt=0.01),
        uniform_world(20_000, 12, 0.0091, seed=43, wrap=False),
        blob_world(15_000, 5, 0.015, nblobs=8, sigma=0.01, seed=44, dim=2),
        uniform_world(1_000, 4, 0.3, seed=45),          # nx = 3
        uniform_world(12_000, 16, 0.0137, seed=46, vel_scale=0.01, dt=0.005),
    ]


@pytest.mark.parametrize("variant", [0, 1])
def test_batch_2d_every_world_matches_the_oracle(gpu, variant):
    specs = mixed_2d_specs()
    b, ids = make_batch(2, specs)
    b.set_tile(variant)
    dbg = b.debug_step()
    for spec, wid in zip(specs, ids):
        g = b.world_debug(dbg, wid)
        compare_with_oracle(spec, g, b.download(wid))
    b.close()


@pytest.mark.parametrize("variant", [0, 1])
def test_batch_3d_every_world_matches_the_oracle(gpu, variant):
    specs = [
        uniform_world(40_000, 8, 0.04, seed=51, dim=3, vel_scale=0.01, dt=0.01),
        blob_world(30_000, 16, 0.02, nblobs=6, sigma=0.02, seed=52, dim=3),
        uniform_world(2_000, 3, 0.26, seed=53, dim=3),
    ]
    b, ids = make_batch(3, specs)
    b.set_tile(variant)
    dbg = b.debug_step()
    for spec, wid in zip(specs, ids):
        compare_with_oracle(spec, b.world_debug(dbg, wid), b.download(wid))
    b.close()


def trajectory(b, wid, steps):
    b.step(steps)
    return b.download(wid)


def test_world_alone_and_in_a_mix_is_bit_identical(gpu):
    specs = mixed_2d_specs()
    target = specs[0]
    alone, (aid,) = make_batch(2, [target])
    ref = trajectory(alone, aid, 6)
    alone.close()
    mix, ids = make_batch(2, specs[3:] + [target] + specs[1:3])
    got = trajectory(mix, ids[3], 6)
    mix.close()
    for a, c in zip(ref, got):
        assert np.array_equal(a, c)


def test_membership_changes_keep_trajectories(gpu):
    """Removing and adding other worlds between steps does not change a world."""
    specs = mixed_2d_specs()
    ref_b, ref_ids = make_batch(2, specs[:2])
    ref_b.step(3)
    ref_b.step(4)
    ref = [ref_b.download(w) for w in ref_ids]
    ref_b.close()

    b, ids = make_batch(2, specs[:4], extra_cells=10 ** 5)
    b.step(3)
    b.update(remove=[ids[2]], add=[desc(specs[5])])
    b.update(remove=[ids[3]])
    b.step(4)
    for w, r in zip(ids[:2], ref):
        for x, y in zip(b.download(w), r):
            assert np.array_equal(x, y)
    assert b.counts()[0] == 3
    b.close()


def test_batch_matches_the_single_world_context(gpu):
    """Same world through plg_step and through a batch: the same arithmetic."""
    from plgpu.physics import GpuWorld

    spec = uniform_world(25_000, 7, 0.017, seed=61, vel_scale=0.01)
    w = GpuWorld(2, spec.n)
    w.set_settings(spec.rmax, spec.friction, spec.force, spec.dt, beta=spec.beta, wrap=spec.wrap)
    w.set_matrix(spec.matrix)
    w.upload(spec.pos, spec.vel, spec.types)
    w.step(5)
    single = w.download()
    w.close()
    b, (_, wid) = make_batch(2, [uniform_world(3_000, 4, 0.05, seed=62), spec])
    got = trajectory(b, wid, 5)
    b.close()
    for a, c in zip(single, got):  # same tiles, same arithmetic
        assert np.array_equal(a, c)


def test_batch_rejects_what_it_cannot_run(gpu):
    from plgpu import _lib

    b, ids = make_batch(2, [uniform_world(1_000, 3, 0.05, seed=71)])
    big = uniform_world(100, 3, 0.5, seed=72)  # nx = 2
    with pytest.raises(_lib.PlgError) as e:
        b.update(add=[desc(big)])
    assert e.value.status == _lib.PLG_E_UNSUPPORTED
    with pytest.raises(_lib.PlgError) as e:
        b.update(remove=[12345])
    assert e.value.status == _lib.PLG_E_INVALID_ARG
    huge = uniform_world(10_000, 3, 0.05, seed=73)
    with pytest.raises(_lib.PlgError) as e:
        b.update(add=[desc(huge)] * 3)  # capacity 2 x 1001 particles
    assert e.value.status == _lib.PLG_E_CAPACITY
    assert b.counts()[0] == 1  # unchanged after the rejections
    b.step(2)
    b.close()


def test_autotune_restores_state_and_variants_agree(gpu):
    from plgpu import _lib

    specs = mixed_2d_specs()[:4]
    b, ids = make_batch(2, specs)
    b.step(2)
    before = [b.download(w) for w in ids]
    v, ms = b.autotune(2)
    assert v == b.tile() and v in range(_lib.PLG_TILE_VARIANTS) and all(m > 0 for m in ms)
    for w, ref in zip(ids, before):
        for x, y in zip(b.download(w), ref):
            assert np.array_equal(x, y)
    b.close()
    runs = []
    for variant in range(_lib.PLG_TILE_VARIANTS):
        bb, ii = make_batch(2, specs)
        bb.set_tile(variant)
        bb.step(4)
        runs.append([bb.download(w) for w in ii])
        bb.close()
    for other in runs[1:]:  # tile variants give the same bits
        for r0, r1 in zip(runs[0], other):
            for a, c in zip(r0, r1):
                assert np.array_equal(a, c)


def test_dense_world_alone_and_in_a_mix_is_bit_identical(gpu):
    """Dense worlds overflow the shared-memory staging; tiles are laid out per
    world, so the same segments take the global-memory path alone and in a
    mix."""
    dense = uniform_world(60_000, 5, 0.05, seed=81, vel_scale=0.01)  # 150 per cell: segments overflow
    others = [uniform_world(7_777, 4, 0.02, seed=82), uniform_world(3_001, 3, 0.04, seed=83)]
    alone, (aid,) = make_batch(2, [dense])
    ref = trajectory(alone, aid, 3)
    alone.close()
    mix, ids = make_batch(2, others[:1] + [dense] + others[1:])
    got = trajectory(mix, ids[1], 3)
    mix.close()
    for a, c in zip(ref, got):
        assert np.array_equal(a, c)


def test_step_budget_freezes_a_world(gpu):
    """A world whose step budget runs out keeps its state while the others
    advance, and continues exactly where it stopped."""
    specs = mixed_2d_specs()[:3]
    ref3 = []
    for spec, n in ((specs[1], 3), (specs[1], 5), (specs[0], 7)):
        b1, (w1,) = make_batch(2, [spec])
        ref3.append(trajectory(b1, w1, n))
        b1.close()
    b, ids = make_batch(2, specs)
    b.set_steps(ids[1], 3)
    b.step(7)
    assert b.steps_left(ids[1]) == 0 and b.steps_left(ids[0]) == -1
    for x, y in zip(b.download(ids[1]), ref3[0]):
        assert np.array_equal(x, y)
    for x, y in zip(b.download(ids[0]), ref3[2]):
        assert np.array_equal(x, y)
    b.set_steps(ids[1], -1)
    b.step(2)
    for x, y in zip(b.download(ids[1]), ref3[1]):
        assert np.array_equal(x, y)
    b.close()


def test_per_world_variants_and_the_per_world_tuner(gpu):
    """Worlds of one batch on different tile variants give the bits of a
    uniform batch (a step launches the force kernel once per variant in
    use); the per-world tuner leaves every world and its step budget where
    they were, and the batch it tunes continues exactly like an untuned
    one."""
    from plgpu import _lib

    specs = mixed_2d_specs() + [uniform_world(40_000, 5, 0.05, seed=84, vel_scale=0.01)]  # a dense world too
    b0, ids0 = make_batch(2, specs)
    b0.set_steps(ids0[2], 2)
    b0.step(4)
    ref = [b0.download(w) for w in ids0]
    b0.close()

    b1, ids1 = make_batch(2, specs)
    b1.set_steps(ids1[2], 2)
    for k, w in enumerate(ids1):
        b1.set_world_tile(w, k % _lib.PLG_TILE_VARIANTS)
    assert [b1.world_tile(w) for w in ids1] == [k % _lib.PLG_TILE_VARIANTS for k in range(len(ids1))]
    b1.step(4)
    for w, r in zip(ids1, ref):
        for a, c in zip(b1.download(w), r):
            assert np.array_equal(a, c)
    b1.close()

    b2, ids2 = make_batch(2, specs)
    b2.set_steps(ids2[2], 2)
    b2.step(1)
    before = [b2.download(w) for w in ids2]
    choice, ms = b2.autotune_worlds(2)
    assert sorted(choice) == sorted(ids2) and set(choice.values()) <= set(range(_lib.PLG_TILE_VARIANTS))
    assert len(ms) == _lib.PLG_TILE_VARIANTS + 1 and all(m > 0 for m in ms)
    assert b2.steps_left(ids2[2]) == 1  # the trials spent no budget
    for w, r in zip(ids2, before):
        for a, c in zip(b2.download(w), r):
            assert np.array_equal(a, c)
    b2.step(3)
    for w, r in zip(ids2, ref):
        for a, c in zip(b2.download(w), r):
            assert np.array_equal(a, c)
    b2.close()
