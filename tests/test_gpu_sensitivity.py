"""Likelihood-ratio sensitivities (tl_sensitivity) against common-random-
number central finite differences (h = 1e-2 relative) and against the FP64
host estimator of the oracle.  Acceptance: within 3 combined standard
errors."""
import numpy as np
import pytest

from oracle import py as ora
from tau_leaping_gb300 import Model

pytestmark = pytest.mark.gpu


def crn_fd(m, base, j, T, R, seed, tracked, h=1e-2):
    up, dn = base.copy(), base.copy()
    up[j] *= 1 + h
    dn[j] *= 1 - h
    a = m.simulate(T, R, seed=seed, tracked=tracked, rate_sets=up[None], keep_samples=True)
    b = m.simulate(T, R, seed=seed, tracked=tracked, rate_sets=dn[None], keep_samples=True)
    d = (a.samples[0, :, -1, :].astype(float) - b.samples[0, :, -1, :].astype(float)) / (2 * h * base[j])
    return d.mean(0), d.std(0, ddof=1) / np.sqrt(R)


def test_lr_gradient_matches_crn_finite_differences_dimer():
    m = Model.generate("dimer", x0_min=1000, x0_max=1000)
    base = m.desc()["rate"].astype(np.float64)
    T, R, tracked = 1.0, 40000, [0, 1]
    g = m.sensitivity(T, R, seed=3, tracked=tracked)
    assert g["grad"].shape == (1, 2, 4)
    for j in range(4):
        fd, fd_se = crn_fd(m, base, j, T, R, seed=11, tracked=tracked)
        for k in range(2):
            lr, lr_se = g["grad"][0, k, j], g["stderr"][0, k, j]
            tol = 3 * np.hypot(lr_se, fd_se[k])
            assert abs(lr - fd[k]) <= tol, (j, k, lr, lr_se, fd[k], fd_se[k])


def test_lr_gradient_matches_fp64_host_estimator():
    m = Model.generate("dimer", x0_min=500, x0_max=500)
    T, R = 0.5, 20000
    g = m.sensitivity(T, R, seed=5, tracked=[0, 1])
    o = ora.OracleModel.from_desc(m.desc())
    r = o.simulate(T, 8000, seed=6, tracked=[0, 1], threads=8, sens=True)
    x = r["samples"][0, :, -1, :].astype(float)
    sc = r["scores"][0]
    xc, scc = x - x.mean(0), sc - sc.mean(0)
    prod = xc[:, :, None] * scc[:, None, :]          # [n, K, M]
    est = prod.sum(0) / (len(x) - 1)
    se = prod.std(0, ddof=1) / np.sqrt(len(x))
    tol = 3 * np.hypot(g["stderr"][0], se)
    assert np.all(np.abs(g["grad"][0] - est) <= tol), (g["grad"][0], est, tol)


def test_rate_set_batch_gradients_per_set():
    m = Model.generate("dimer", x0_min=1000, x0_max=1000)
    base = m.desc()["rate"]
    rng = np.random.default_rng(17)
    sets = base[None, :] * rng.lognormal(0.0, 0.2, size=(4, 4))
    tf = rng.uniform(0.5, 1.0, size=4)
    g = m.sensitivity(1.0, 8000, seed=2, tracked=[0], rate_sets=sets, t_final_sets=tf)
    assert g["grad"].shape == (4, 1, 4)
    # set 2 alone (same realization ids, same set index -> same streams)
    for s in (0, 3):
        fd, fd_se = crn_fd(m, sets[s].copy(), 0, tf[s], 8000, seed=9, tracked=[0])
        lr, lr_se = g["grad"][s, 0, 0], g["stderr"][s, 0, 0]
        assert abs(lr - fd[0]) <= 3 * np.hypot(lr_se, fd_se[0]), (s, lr, fd)


def test_lr_gradient_toy_network_channels():
    """128 x 256 toy network (the batch workload's second model): LR
    gradients of E[S1(T)] for the channels with the largest estimated
    effect, against CRN central differences."""
    m = Model.generate("toy")
    base = m.desc()["rate"].astype(np.float64)
    T, R = 0.005, 20000
    g = m.sensitivity(T, R, seed=4, tracked=[0])
    order = np.argsort(-np.abs(g["grad"][0, 0]) / np.maximum(g["stderr"][0, 0], 1e-30))
    for j in list(order[:4]) + [int(order[100]), int(order[200])]:
        fd, fd_se = crn_fd(m, base, int(j), T, R, seed=12, tracked=[0])
        lr, lr_se = g["grad"][0, 0, j], g["stderr"][0, 0, j]
        assert abs(lr - fd[0]) <= 3 * np.hypot(lr_se, fd_se[0]), (j, lr, lr_se, fd[0], fd_se[0])
