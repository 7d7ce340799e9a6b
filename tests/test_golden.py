"""The oracle and the GPU path against the committed golden vectors
(tests/golden/*.npz, made by tests/golden/make_golden.py, an independent
pure-Python restatement of the reference step)."""
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = sorted(p.stem for p in GOLDEN.glob("*.npz"))


def load(name):
    return dict(np.load(GOLDEN / f"{name}.npz"))


def settings_of(g):
    dim, rmax, fr, force, dt, beta, wrap = g["params"]
    return int(dim), dict(rmax=float(rmax), friction=float(fr), force=float(force), dt=float(dt), beta=float(beta),
                          wrap=bool(wrap))


def test_golden_cases_present():
    assert len(CASES) >= 6


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_golden(oracle, name):
    g = load(name)
    dim, s = settings_of(g)
    n = g["in_pos"].shape[0]
    w = oracle.World(dim, g["in_pos"], g["in_vel"], g["in_types"], np.arange(n, dtype=np.int32), g["matrix"],
                     oracle.settings(**s))
    steps = sum(1 for k in g if k.startswith("pairs"))
    for k in range(steps):
        d = w.step(debug=True)
        assert np.array_equal(w.ids, g[f"ids{k}"]), f"step {k}: order"
        assert np.array_equal(d["cell"], g[f"cell{k}"]), f"step {k}: cells"
        assert np.array_equal(d["pairs"], g[f"pairs{k}"]), f"step {k}: pair counts"
        assert np.array_equal(d["hsum"], g[f"hsum{k}"]) and np.array_equal(d["hxor"], g[f"hxor{k}"])
        # same IEEE operation sequence; only libm pow may differ by an ulp
        np.testing.assert_allclose(d["acc"], g[f"acc{k}"], rtol=1e-13, atol=1e-13)
        np.testing.assert_allclose(w.vel, g[f"vel{k}"], rtol=1e-12, atol=1e-15)
        np.testing.assert_allclose(w.pos, g[f"pos{k}"], rtol=0, atol=1e-14)


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_gpu_first_step_matches_golden(gpu, name):
    """The golden inputs are FP32-exact, so the GPU's first step must
    reproduce the golden order, cells and pair sets exactly."""
    from worlds import WorldSpec, run_gpu_debug

    g = load(name)
    dim, s = settings_of(g)
    spec = WorldSpec(dim, g["in_pos"], g["in_vel"], g["in_types"], g["matrix"], **s)
    d, (pos, vel, types, ids) = run_gpu_debug(spec)
    assert np.array_equal(ids, g["ids0"])
    assert np.array_equal(d["cell"], g["cell0"])
    assert np.array_equal(d["pairs"], g["pairs0"])
    assert np.array_equal(d["hsum"], g["hsum0"]) and np.array_equal(d["hxor"], g["hxor0"])
    acc = d["acc"].astype(np.float64)
    assert np.linalg.norm(acc - g["acc0"]) <= 1e-5 * np.linalg.norm(g["acc0"])
