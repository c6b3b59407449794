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


@pytest.mark.slow
def test_c5_full_configuration_gradients_per_set(capsys):
    """The sensitivity + uneven-batch configuration in full, in one
    tl_simulate_batch launch with sensitivities: the dimerisation decay
    (S1 = 1e5) with 64 rate sets c_j * lognormal(0, 0.2) (seed 17), 4096
    realizations each, t_final uniform in [1, 10]; the 128 x 256 toy network
    with 16 sets, 1024 realizations each, t_final uniform in [0.05, 0.1].

    For every one of the 80 sets, the likelihood-ratio gradient
    dE[S_k(T)]/dc_j of each tracked species is compared with common-random-
    number central finite differences (h = 1e-2 relative; the up and down
    runs of a pair draw the same streams): every channel of the dimer, and
    for the toy network the four channels of that set with the largest
    |gradient| / standard error plus channels 0 and 128.  z = (LR - FD) /
    (combined standard error).  With 704 comparisons some |z| > 3 are
    expected by chance (about 1.9 for unbiased estimators), so the check
    is: at most 1 % of the comparisons beyond 3 standard errors, none beyond
    4.5 (a family-wise level of 0.5 %), and a mean z^2 near 1."""
    from tau_leaping_gb300.model import simulate_batch
    h = 1e-2
    rng = np.random.default_rng(17)
    dim, toy = Model.generate("dimer"), Model.generate("toy")
    ds = dim.desc()["rate"][None, :] * rng.lognormal(0.0, 0.2, size=(64, 4))
    dt = rng.uniform(1.0, 10.0, size=64)
    ts = toy.desc()["rate"][None, :] * rng.lognormal(0.0, 0.2, size=(16, toy.n_channels))
    tt = rng.uniform(0.05, 0.1, size=16)
    lr = simulate_batch([
        dict(model=dim, t_final=10.0, n=4096, seed=1, tracked=[0, 1], rate_sets=ds, t_final_sets=dt,
             sensitivity=True),
        dict(model=toy, t_final=0.1, n=1024, seed=1, tracked=[0, 4], rate_sets=ts, t_final_sets=tt,
             sensitivity=True)])

    def fd_pairs(m, sets, tf, pairs, R, tracked):
        up, dn = [], []
        for s, j in pairs:
            u, d = sets[s].copy(), sets[s].copy()
            u[j] *= 1 + h
            d[j] *= 1 - h
            up.append(u)
            dn.append(d)
        tfr = np.array([tf[s] for s, _ in pairs])
        kw = dict(seed=77, tracked=tracked, keep_samples=True, t_final_sets=tfr)
        a = m.simulate(float(tfr.max()), R, rate_sets=np.array(up), **kw).samples[:, :, -1, :].astype(float)
        b = m.simulate(float(tfr.max()), R, rate_sets=np.array(dn), **kw).samples[:, :, -1, :].astype(float)
        c = np.array([sets[s][j] for s, j in pairs])
        d = (a - b) / (2 * h * c[:, None, None])               # [pairs, R, K]
        return d.mean(1), d.std(1, ddof=1) / np.sqrt(R)

    def zscore(diff, se):
        # both estimates exactly zero (a channel that moves nothing): agreement
        return diff / se if se > 0 else (0.0 if diff == 0 else np.inf)

    z_all = {}
    dpairs = [(s, j) for s in range(64) for j in range(4)]
    fd, fse = fd_pairs(dim, ds, dt, dpairs, 4096, [0, 1])
    g, gse = lr[0]["grad"], lr[0]["stderr"]                     # [S, K, M]
    z_all["dimer"] = np.array([zscore(g[s, k, j] - fd[q, k], np.hypot(gse[s, k, j], fse[q, k]))
                               for q, (s, j) in enumerate(dpairs) for k in range(2)])
    g, gse = lr[1]["grad"], lr[1]["stderr"]
    tpairs = []
    for s in range(16):
        score = np.max(np.abs(g[s]) / np.maximum(gse[s], 1e-300), axis=0)
        pick = list(np.argsort(-score)[:4]) + [0, 128]
        tpairs += [(s, int(j)) for j in dict.fromkeys(pick)]
    fd, fse = fd_pairs(toy, ts, tt, tpairs, 1024, [0, 4])
    z_all["toy"] = np.array([zscore(g[s, k, j] - fd[q, k], np.hypot(gse[s, k, j], fse[q, k]))
                             for q, (s, j) in enumerate(tpairs) for k in range(2)])
    z = np.concatenate(list(z_all.values()))
    with capsys.disabled():
        for name, zz in z_all.items():
            print(f"\nC5 {name}: {len(zz)} LR-vs-CRN-FD comparisons, max |z| {np.abs(zz).max():.2f}, "
                  f"{np.mean(np.abs(zz) > 3):.2%} beyond 3 s.e., mean z^2 {np.mean(zz ** 2):.2f}")
    assert np.all(np.isfinite(z))
    assert np.mean(np.abs(z) > 3) <= 0.01, np.sort(np.abs(z))[-10:]
    assert np.abs(z).max() <= 4.5, np.abs(z).max()
    assert 0.5 <= np.mean(z ** 2) <= 1.5, np.mean(z ** 2)
