"""Pin the FP64 oracle before trusting it.

* Philox4x32-10 known-answer vectors of Random123 (Salmon et al., SC'11).
* tests/golden/ref_functors.npz: outputs of the reference's own functors
  (IsCriticalAndPropensity, CSRMatrixPacked::CompTau, FireReactionsFn,
  pack), generated by tests/golden/make_golden.py.
* The live reference functors (oracle/_ref) when the reference sources are
  present in this environment.
* Statistical sanity of the oracle's tau-leaping against its exact SSA.
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import py as ora
from tau_leaping_gb300 import Model, _ffi

GOLD = Path(__file__).resolve().parent / "golden" / "ref_functors.npz"
COMPAT_TAU = _ffi.FLAG_COMPAT_G | _ffi.FLAG_COMPAT_CRIT | _ffi.FLAG_COMPAT_STOICH

MODELS = {
    "dimer": ("dimer", {}),
    "toy": ("toy", {}),
    "chain64": ("chain", dict(n_species=64)),
    "colloid40": ("colloid", dict(n_species=40)),
}


def test_philox_known_answers():
    ctr = [[0, 0, 0, 0], [0xFFFFFFFF] * 4, [0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344]]
    key = [[0, 0], [0xFFFFFFFF] * 2, [0xA4093822, 0x299F31D0]]
    want = [[0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8],
            [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD],
            [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]]
    assert ora.philox(ctr, key).tolist() == want


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLD))


@pytest.mark.parametrize("name", list(MODELS))
def test_oracle_matches_reference_functors(gold, name):
    fam, kw = MODELS[name]
    m = Model.generate(fam, **kw)
    o = ora.OracleModel.from_desc(m.desc())
    x = gold[f"{name}/x"]
    r = o.eval(x, eps=0.03, flags=COMPAT_TAU, nc=5)
    assert np.array_equal(r["crit"], gold[f"{name}/crit"])
    a_ref = gold[f"{name}/a"].astype(np.float64)
    # reference propensities are FP32 products: <= 3 roundings
    assert np.allclose(r["a"], a_ref, rtol=1e-6, atol=0)
    t_ref = gold[f"{name}/tau1"].astype(np.float64)
    err = np.abs(r["tau1"] - t_ref) / t_ref
    assert err.max() <= 1e-5, err.max()
    # the engine's packed species-row CSR equals the reference's packing
    t = m.tables()
    assert np.array_equal(t["csr_row_ptr"], gold[f"{name}/csr_row_ptr"])
    assert np.array_equal(t["csr_valcol"], gold[f"{name}/csr_valcol"])
    # integer update: bit-exact against FireReactionsFn
    fired = o.replay(gold[f"{name}/x_fire0"], gold[f"{name}/k"], raw=True)
    assert np.array_equal(fired, gold[f"{name}/fired"])
    fired_net = o.replay(gold[f"{name}/x_fire0"], gold[f"{name}/k"], raw=False)
    assert np.array_equal(fired_net, gold[f"{name}/fired"])
    if f"{name}/fired_as_shipped" in gold:
        assert np.array_equal(fired[0], gold[f"{name}/fired_as_shipped"])


def test_oracle_against_live_reference(reference_build):
    """Fresh random states through the reference's functors (oracle/_ref)."""
    import ctypes as C

    from tests.golden import make_golden as mg
    L = mg.load_ref()
    rng = np.random.default_rng(77)
    for name in MODELS:
        m, d, t, ref_order = mg.model_arrays(name)
        o = ora.OracleModel.from_desc(d)
        N, M = m.n_species, m.n_channels
        x = rng.integers(0, 3 * max(int(d["x0"].max()), 30), size=(6, N)).astype(np.int32)
        x[:, ::5] = rng.integers(0, 8, size=x[:, ::5].shape)
        r = o.eval(x.astype(np.int64), eps=0.03, flags=COMPAT_TAU, nc=5)
        pr = C.c_float()
        for s in range(len(x)):
            for j in range(M):
                c = L.ref_propensity(int(ref_order[j]), int(x[s, t["s0"][j]]), int(x[s, t["s1"][j]]), 5,
                                     float(np.float32(d["rate"][j])), C.byref(pr))
                assert c == r["crit"][s, j]
                assert abs(pr.value - r["a"][s, j]) <= 1e-6 * abs(r["a"][s, j]) + 1e-30


def test_oracle_tau_leap_close_to_ssa():
    m = Model.generate("dimer", x0_min=600, x0_max=600)
    o = ora.OracleModel.from_desc(m.desc())
    a = o.simulate(1.0, 3000, seed=1, tracked=[0, 1], threads=8)["samples"][0, :, -1, :].astype(float)
    b = o.simulate(1.0, 3000, seed=2, tracked=[0, 1], method=1, threads=8)["samples"][0, :, -1, :].astype(float)
    for k in range(2):
        se = np.sqrt(a[:, k].var() / len(a) + b[:, k].var() / len(b))
        assert abs(a[:, k].mean() - b[:, k].mean()) <= 0.01 * b[:, k].mean() + 4 * se


def test_oracle_poisson_sampler_moments():
    for mu in (0.5, 7.0, 12.0, 500.0):
        s = ora.poisson(np.full(100_000, mu), seed=3).astype(float)
        assert abs(s.mean() - mu) < 5 * np.sqrt(mu / 1e5)
        assert abs(s.var() - mu) < 5 * np.sqrt((mu + 2 * mu * mu) / 1e5)


def test_oracle_ssa_matches_exact_chain_solution():
    m = Model.generate("chain", n_species=24)
    o = ora.OracleModel.from_desc(m.desc())
    mean, var = ora.chain_exact_moments(m.desc()["x0"], 1.0, 0.4)
    x = o.simulate(0.4, 8000, seed=2, method=1, threads=8)["samples"][0, :, -1, :].astype(float)
    se = np.sqrt(var / len(x))
    assert np.all(np.abs(x.mean(0) - mean) <= 4 * se)
    sev = var * np.sqrt(2.0 / len(x))
    assert np.all(np.abs(x.var(0, ddof=1) - var) <= 4.5 * sev)


@pytest.mark.parametrize("family,kw", [("dimer", {}), ("toy", {}), ("chain", {}), ("colloid", {}),
                                       ("toy", dict(n_species=16, n_channels=32, seed=3, x0_min=0, x0_max=60)),
                                       ("colloid", dict(n_species=60)), ("chain", dict(n_species=48))])
def test_oracle_generator_equals_engine_generator(family, kw):
    """The oracle builds the benchmark models on its own (the CPU reference
    arm never loads the engine): the same description as the engine's
    seeded generator, array for array."""
    from tau_leaping_gb300 import Model
    a = ora.generate(family, **kw)
    b = Model.generate(family, **kw).desc()
    for k in ("x0", "rate", "col_ptr", "row_ind", "stoich"):
        assert np.array_equal(a[k], b[k]), k
