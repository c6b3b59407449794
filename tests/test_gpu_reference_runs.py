"""Ensemble parity with the reference's own runs.

tests/golden/ref_runs.npz holds per-realization samples produced by the
reference's Model API (host-built from its sources, logging on; see
tests/golden/make_ref_runs.py) on models where the reference is well
defined.  The engine runs the same model description with its
reference-compatibility switches (TL_FLAG_COMPAT_REFERENCE); mean, variance
and distribution of every tracked species at every grid time must agree at
99% (Welch t, Levene, two-sample KS; fixed seeds, so deterministic).

The reference evaluates the grid by linear interpolation between the states
it logs before each step; the engine ends a leap exactly on each grid time.
Interpolation between states one leap apart lowers the variance, so the
fixtures use many small leaps per grid interval (test_128 at eps 0.03,
the chain at eps 0.003), where the difference is far below the sampling
error of these ensembles.
"""
from pathlib import Path

import numpy as np
import pytest
from scipy import stats

from tau_leaping_gb300 import Model, _ffi

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden" / "ref_runs.npz"


def load(name):
    g = np.load(GOLD)
    d = {k.split("/", 1)[1]: g[k] for k in g.files if k.startswith(name + "/")}
    m = Model.from_arrays(d["x0"], d["rate"], d["col_ptr"], d["row_ind"], d["stoich"])
    return m, d


def agree(ref, eng, label):
    for k in range(ref.shape[1]):
        x, y = ref[:, k].astype(float), eng[:, k].astype(float)
        if np.all(x == x[0]) and np.all(y == y[0]):
            assert x[0] == y[0], label
            continue
        pt = stats.ttest_ind(x, y, equal_var=False).pvalue
        pl = stats.levene(x, y).pvalue
        pk = stats.ks_2samp(x, y).pvalue
        assert min(pt, pl, pk) > 0.01, f"{label} species {k}: t {pt:.3g} levene {pl:.3g} ks {pk:.3g}"


@pytest.mark.parametrize("name", ["test_128", "chain64"])
def test_compat_mode_matches_reference_run(name):
    m, d = load(name)
    T, P = float(d["t_final"]), int(d["intervals"])
    r = m.simulate(T, 20000, seed=21, intervals=P, tracked=d["tracked"], flags=_ffi.FLAG_COMPAT_REFERENCE,
                   keep_samples=True, eps=float(d["eps"]))
    ref = d["samples"]                      # [grid, n, K], grid t_k = k*T/P, k < P
    assert np.allclose(d["times"], r.times[0][: len(d["times"])], atol=1e-6)
    for k in range(1, ref.shape[0]):
        agree(ref[k], r.samples[0, :, k, :], f"{name} t={d['times'][k]:.3g}")


def test_default_mode_matches_reference_run_on_chain():
    """On the chain every rule the reference departs from is inactive (first
    order only, no shared species, Poisson means below 80, no direct-method
    steps), so the default CGP mode must agree with the reference's run."""
    m, d = load("chain64")
    T, P = float(d["t_final"]), int(d["intervals"])
    r = m.simulate(T, 20000, seed=22, intervals=P, tracked=d["tracked"], keep_samples=True, eps=float(d["eps"]))
    assert r.ssa_steps == 0
    for k in range(1, d["samples"].shape[0]):
        agree(d["samples"][k], r.samples[0, :, k, :], f"chain64 default t={d['times'][k]:.3g}")
