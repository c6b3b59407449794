"""tl_simulate_batch: several models and rate sets in one persistent launch.

Each item runs with the same group width (lane units for small models = one
realization per thread, warp units otherwise) and the same Philox streams
as a separate tl_simulate call, so its samples must be bit-identical."""
import numpy as np
import pytest

from tau_leaping_gb300 import Model, _ffi
from tau_leaping_gb300.model import simulate_batch

pytestmark = pytest.mark.gpu


def test_batch_equals_separate_runs():
    dim = Model.generate("dimer", x0_min=3000, x0_max=3000)
    toy = Model.generate("toy", n_species=16, n_channels=24, seed=3, x0_max=2000)
    rng = np.random.default_rng(17)
    dsets = dim.desc()["rate"][None, :] * rng.lognormal(0.0, 0.2, size=(5, 4))
    dtf = rng.uniform(0.5, 2.0, size=5)
    items = [
        dict(model=dim, t_final=1.0, n=333, seed=7, tracked=[0, 1], intervals=2, rate_sets=dsets, t_final_sets=dtf,
             keep_samples=True),
        dict(model=toy, t_final=0.02, n=200, seed=9, tracked=[0, 3, 5], keep_samples=True),
    ]
    out = simulate_batch(items)
    a = dim.simulate(1.0, 333, seed=7, tracked=[0, 1], intervals=2, rate_sets=dsets, t_final_sets=dtf,
                     keep_samples=True, variant=_ffi.VARIANT_THREAD)
    b = toy.simulate(0.02, 200, seed=9, tracked=[0, 3, 5], keep_samples=True, variant=_ffi.VARIANT_WARP)
    assert np.array_equal(out[0]["samples"], a.samples)
    assert np.array_equal(out[1]["samples"], b.samples)
    assert out[0]["leaps"] == a.leaps and out[1]["leaps"] == b.leaps
    assert out[0]["ssa_steps"] == a.ssa_steps and out[1]["ssa_steps"] == b.ssa_steps
    assert np.allclose(out[0]["mean"], a.mean) and np.allclose(out[1]["stddev"], b.stddev)
    assert np.allclose(out[0]["times"][:, -1], dtf)


def test_batch_sensitivity_matches_separate():
    dim = Model.generate("dimer", x0_min=1000, x0_max=1000)
    toy = Model.generate("toy", n_species=12, n_channels=20, seed=5, x0_max=500)
    out = simulate_batch([
        dict(model=dim, t_final=0.5, n=2000, seed=1, tracked=[0], sensitivity=True),
        dict(model=toy, t_final=0.01, n=500, seed=2, tracked=[1], sensitivity=True),
    ])
    g1 = dim.sensitivity(0.5, 2000, seed=1, tracked=[0], variant=_ffi.VARIANT_THREAD)
    g2 = toy.sensitivity(0.01, 500, seed=2, tracked=[1], variant=_ffi.VARIANT_WARP)
    assert np.allclose(out[0]["grad"], g1["grad"], rtol=1e-9, atol=1e-12)
    assert np.allclose(out[1]["grad"], g2["grad"], rtol=1e-9, atol=1e-12)
