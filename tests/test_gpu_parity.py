"""Parity of the CUDA path (through the C ABI) with the FP64 oracle.

* Philox4x32-10 on the device: Random123 known-answer vectors and the
  oracle's implementation on random counters (bit-exact).
* Leap quantities (propensities, criticality, mu, sigma^2, tau1): within
  1e-5 relative of FP64 (tolerance stated per assertion).
* Integer replay of firing counts: bit-exact, int32 and int64 models,
  raw (reference) and net entries.
* Poisson sampler: moments and chi-square goodness of fit.
"""
import numpy as np
import pytest
from scipy import stats

from oracle import py as ora
from tau_leaping_gb300 import Model, _ffi
from tau_leaping_gb300.model import philox, poisson

pytestmark = pytest.mark.gpu

RTOL = 1e-5  # FP32 device vs FP64 oracle, relative

KAT_CTR = [[0, 0, 0, 0], [0xFFFFFFFF] * 4, [0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344]]
KAT_KEY = [[0, 0], [0xFFFFFFFF] * 2, [0xA4093822, 0x299F31D0]]
KAT_OUT = [[0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8],
           [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD],
           [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]]


def test_philox_known_answers_and_oracle():
    assert philox(KAT_CTR, KAT_KEY).tolist() == KAT_OUT
    rng = np.random.default_rng(5)
    ctr = rng.integers(0, 2**32, size=(4096, 4), dtype=np.uint64).astype(np.uint32)
    key = rng.integers(0, 2**32, size=(4096, 2), dtype=np.uint64).astype(np.uint32)
    assert np.array_equal(philox(ctr, key), ora.philox(ctr, key))


def random_states(m, n, rng, lo_frac=0.0):
    x0 = m.desc()["x0"]
    scale = np.maximum(x0, 20)
    x = (rng.random((n, m.n_species)) * 2 * scale).astype(np.int64)
    # include small populations (critical channels) and zeros
    small = rng.random((n, m.n_species)) < 0.15
    x[small] = rng.integers(0, 12, size=small.sum())
    x[0] = x0
    return x


MODELS = {
    "dimer": lambda: Model.generate("dimer"),
    "toy": lambda: Model.generate("toy"),
    "chain": lambda: Model.generate("chain"),
    "colloid": lambda: Model.generate("colloid"),
}


def rel_err(dev, ref) -> float:
    dev = np.asarray(dev, np.float64)
    ref = np.asarray(ref, np.float64)
    same_inf = np.isinf(dev) & (dev == ref)  # an infinite bound on both sides
    with np.errstate(invalid="ignore"):  # inf - inf of those entries
        err = np.abs(dev - ref) / np.maximum(np.abs(ref), 1e-30)
    err[same_inf] = 0.0
    return float(err.max()) if err.size else 0.0


def rel_close(dev, ref, rtol, what):
    worst = rel_err(dev, ref)
    assert worst <= rtol, f"{what}: max relative error {worst:.3e} > {rtol:.0e}"


@pytest.mark.parametrize("name", list(MODELS))
@pytest.mark.parametrize("flags", [0, _ffi.FLAG_COMPAT_G | _ffi.FLAG_COMPAT_CRIT | _ffi.FLAG_COMPAT_STOICH])
def test_leap_quantities_match_fp64(name, flags, capsys):
    """Propensities, a0 and tau1 within 1e-5 relative of the FP64 oracle on
    random states (small and zero populations included); mu and sigma^2
    against the scale of their summed magnitudes.  The measured maxima are
    printed."""
    m = MODELS[name]()
    o = ora.OracleModel.from_desc(m.desc())
    rng = np.random.default_rng(11)
    x = random_states(m, 8 if name == "colloid" else 64, rng)
    d = m.eval_leap(x, eps=0.03, flags=flags)
    r = o.eval(x, eps=0.03, flags=flags)
    assert np.array_equal(d["crit"], r["crit"])
    # mu / sigma^2 are FP32 sums of signed terms: compare against the scale
    # of the summed magnitudes (cancellation makes pure relative meaningless)
    scale = r["sigma2"] + 1e-30
    mag = np.zeros_like(r["mu"])
    a = r["a"] * (1 - r["crit"])
    desc = m.desc()
    # |mu| error bounded by RTOL * sum_j |v_ij| a_j
    for j in range(m.n_channels):
        for q in range(desc["col_ptr"][j], desc["col_ptr"][j + 1]):
            mag[:, desc["row_ind"][q]] += abs(int(desc["stoich"][q])) * a[:, j]
    e_mu = float(np.max(np.abs(d["mu"] - r["mu"]) / (mag + 1e-30)))
    e_s2 = float(np.max(np.abs(d["sigma2"] - r["sigma2"]) / scale))
    ea, ea0, et = rel_err(d["a"], r["a"]), rel_err(d["a0"], r["a0"]), rel_err(d["tau1"], r["tau1"])
    with capsys.disabled():
        print(f"\nleap quantities {name} flags {flags:#x} vs FP64: a {ea:.2e}, a0 {ea0:.2e}, "
              f"mu {e_mu:.2e} (of sum |v|a), sigma2 {e_s2:.2e}, tau1 {et:.2e}")
    # propensities: products of <= 3 FP32 roundings
    assert ea <= RTOL and ea0 <= RTOL, (ea, ea0)
    assert e_s2 <= RTOL and e_mu <= RTOL, (e_s2, e_mu)
    # tau1: a minimum of ratios of these; relative
    assert et <= RTOL, f"tau1: max relative error {et:.3e} > {RTOL:.0e}"


@pytest.mark.parametrize("name", ["dimer", "toy", "chain", "colloid"])
@pytest.mark.parametrize("raw", [False, True])
def test_replay_bit_exact(name, raw):
    m = MODELS[name]()
    o = ora.OracleModel.from_desc(m.desc())
    rng = np.random.default_rng(3)
    L = 16
    k = rng.integers(0, 50, size=(L, m.n_channels)).astype(np.int32)
    x0 = m.desc()["x0"] + 10**6
    dev = m.replay(x0, k, raw=raw)
    ref = o.replay(x0, k, raw=raw)
    assert np.array_equal(dev, ref)


def test_replay_overflow_reported():
    m = Model.generate("chain", n_species=8)
    k = np.zeros((1, 8), np.int32)
    k[0, 0] = 2**31 - 1   # species 1 gains 2^31-1 on top of >= 1000
    with pytest.raises(_ffi.TLError) as e:
        m.replay(m.desc()["x0"], k)
    assert e.value.status == 4


@pytest.mark.parametrize("mu", [0.0, 0.3, 2.5, 9.99, 10.0, 37.5, 400.0, 2.0e4, 3.0e6])
def test_poisson_sampler_distribution(mu):
    n = 200_000
    s = poisson(np.full(n, mu, np.float32), seed=17, step=3).astype(np.float64)
    if mu == 0.0:
        assert not s.any()
        return
    se_mean = np.sqrt(mu / n)
    assert abs(s.mean() - mu) < 5 * se_mean
    # variance of the sample variance ~ (mu + 2 mu^2)/n
    assert abs(s.var() - mu) < 5 * np.sqrt((mu + 2 * mu * mu) / n)
    # chi-square on the central mass
    lo, hi = int(max(0, np.floor(mu - 4 * np.sqrt(mu)))), int(np.ceil(mu + 4 * np.sqrt(mu))) + 1
    if hi - lo > 200:
        edges = np.linspace(lo, hi, 60).astype(np.int64)
    else:
        edges = np.arange(lo, hi + 1)
    obs, _ = np.histogram(s, bins=edges)
    cdf = stats.poisson.cdf(edges - 1, mu)
    exp = np.diff(cdf) * n
    keep = exp > 20
    chi = ((obs[keep] - exp[keep]) ** 2 / exp[keep]).sum()
    dof = keep.sum() - 1
    assert stats.chi2.sf(chi, dof) > 1e-4, (chi, dof)


def test_poisson_reference_sampler_matches_oracle_law():
    # the reference's Knuth / |Normal| sampler: moments only (it is biased
    # by design above mean 80, where it truncates a normal)
    for mu in (3.0, 50.0):
        s = poisson(np.full(100_000, mu, np.float32), seed=2, compat=True).astype(np.float64)
        r = ora.poisson(np.full(100_000, mu), seed=2, compat=True).astype(np.float64)
        assert abs(s.mean() - r.mean()) < 6 * np.sqrt(2 * mu / 1e5)


GOLD_MODELS = {"dimer": ("dimer", {}), "toy": ("toy", {}), "chain64": ("chain", dict(n_species=64)),
               "colloid40": ("colloid", dict(n_species=40))}


@pytest.mark.parametrize("name", list(GOLD_MODELS))
def test_device_matches_reference_functor_fixtures(name):
    """tests/golden/ref_functors.npz holds the reference's own FP32 outputs
    (IsCriticalAndPropensity, CompTau, FireReactionsFn).  With the compat
    switches the device evaluates the same FP32 expressions in the same
    order, so propensities are bit-identical; tau1 may differ by FMA
    contraction only (relative 1e-6)."""
    from pathlib import Path
    g = np.load(Path(__file__).resolve().parent / "golden" / "ref_functors.npz")
    fam, kw = GOLD_MODELS[name]
    m = Model.generate(fam, **kw)
    flags = _ffi.FLAG_COMPAT_G | _ffi.FLAG_COMPAT_CRIT | _ffi.FLAG_COMPAT_STOICH
    d = m.eval_leap(g[f"{name}/x"], eps=0.03, flags=flags)
    assert np.array_equal(d["crit"], g[f"{name}/crit"])
    assert np.array_equal(d["a"], g[f"{name}/a"])
    t_ref = g[f"{name}/tau1"].astype(np.float64)
    assert np.max(np.abs(d["tau1"] - t_ref) / t_ref) <= 1e-6
    out = m.replay(g[f"{name}/x_fire0"], g[f"{name}/k"], raw=True)
    assert np.array_equal(out, g[f"{name}/fired"])
