"""Paths of the engine that the benchmark configurations rarely or never
take, each driven on purpose and checked through the C ABI:

* sharding: a call over realizations [0, R) equals calls over [0, R/2) and
  [R/2, R) with realization_offset, sample for sample, and tl_merge_moments
  of the halves equals the one-call moments (the reference's serial
  realization loop, tau_leaping/tau_leaping.cpp:144-150, is what is split);
* the rejection regime: leaps whose update leaves a population negative are
  rejected and retried with tau halved (Cao, Gillespie, Petzold 2006, step
  5); the engine and the FP64 oracle, which draws the same streams, agree
  trajectory for trajectory, and an independent oracle ensemble agrees at
  99 % (Welch t, Levene, Kolmogorov-Smirnov) with many rejections;
* small Poisson means on every group kind: the k = 0 / k = 1 tests on the
  shared Philox word, placed differently per group kind, give the oracle's
  firing counts trajectory for trajectory;
* the halving cap: a leap still rejected after max_halvings halvings stops
  its realization and the call returns TL_ERR_NUMERIC;
* the bounded staging wait: with no polls allowed the wait for the model
  tables' shared-memory copy gives up, the call returns
  TL_ERR_WAIT_TIMEOUT, and the next call on the same context succeeds.
"""
import numpy as np
import pytest
from scipy import stats

from oracle import py as ora
from tau_leaping_gb300 import Model, _ffi
from tau_leaping_gb300.shard import merge_moments

pytestmark = pytest.mark.gpu

P99 = 0.01


def compare_final(a, b, label, p=P99):
    for k in range(a.shape[1]):
        x, y = a[:, k].astype(float), b[:, k].astype(float)
        pt = stats.ttest_ind(x, y, equal_var=False).pvalue
        pl = stats.levene(x, y).pvalue
        pk = stats.ks_2samp(x, y).pvalue
        assert pt > p and pl > p and pk > p, f"{label} species {k}: t {pt:.3g} levene {pl:.3g} ks {pk:.3g}"


@pytest.mark.parametrize("family,variant,R,T", [("toy", _ffi.VARIANT_WARP, 4096, 0.004),
                                                ("dimer", _ffi.VARIANT_THREAD, 1001, 1.0),
                                                ("colloid", _ffi.VARIANT_CTA, 257, 0.002)])
def test_sharded_calls_equal_one_call(family, variant, R, T):
    kw = {"colloid": dict(n_species=60), "dimer": dict(x0_min=2000, x0_max=2000)}.get(family, {})
    m = Model.generate(family, **kw)
    tr = [0, 1, 2]
    common = dict(t_final=T, seed=21, tracked=tr, intervals=3, keep_samples=True, variant=variant)
    one = m.simulate(n=R, **common)
    h = R // 2
    lo = m.simulate(n=h, realization_offset=0, **common)
    hi = m.simulate(n=R - h, realization_offset=h, **common)
    assert np.array_equal(np.concatenate([lo.samples, hi.samples], axis=1), one.samples)
    assert lo.leaps + hi.leaps == one.leaps and lo.ssa_steps + hi.ssa_steps == one.ssa_steps
    n, mean, sd = merge_moments([h, R - h], np.stack([lo.mean, hi.mean]), np.stack([lo.stddev, hi.stddev]))
    assert n == R
    assert np.allclose(mean, one.mean, rtol=1e-12, atol=1e-12)
    assert np.allclose(sd, one.stddev, rtol=1e-9, atol=1e-9)


REJ_MODELS = {
    # S1 -> 0 from 40 molecules on one grid interval: at eps = 3 the CGP
    # bound allows a mean of 120 firings, so about half of the attempts are
    # rejected (a finer grid would clamp the leaps and hide them)
    "decay": (lambda: Model.from_arrays([40], [1.0], [0, 1], [0], [-1]), 1),
    # a 16 x 32 random network with first- and second-order channels and
    # populations in [0, 60], two grid intervals
    "toy16": (lambda: Model.generate("toy", n_species=16, n_channels=32, seed=3, x0_min=0, x0_max=60), 2),
}


@pytest.mark.parametrize("name", list(REJ_MODELS))
def test_rejection_regime_matches_oracle(name, capsys):
    """The oracle draws the same Philox streams and halves tau by the same
    rule, so realization for realization the two agree; an independent
    oracle ensemble (other seed) agrees in distribution at a family-wise 99 %
    (Bonferroni over species, grid points and the three tests)."""
    make, P = REJ_MODELS[name]
    m = make()
    tr = [0, 1] if m.n_species > 1 else [0]
    o = ora.OracleModel.from_desc(m.desc())
    g = m.simulate(1.0, 20000, seed=5, eps=3.0, intervals=P, tracked=tr, keep_samples=True)
    paired = o.simulate(1.0, 4000, seed=5, eps=3.0, intervals=P, tracked=tr, threads=8)
    r = o.simulate(1.0, 8000, seed=6, eps=3.0, intervals=P, tracked=tr, threads=8)
    same = np.mean(np.all(paired["samples"][0] == g.samples[0, :4000], axis=(1, 2)))
    with capsys.disabled():
        print(f"\nrejection regime {name}: engine {g.rejections} rejections / {g.leaps} leaps / "
              f"{g.ssa_steps} SSA steps; oracle {r['rejections']} / {r['leaps']} / {r['ssa_steps']}; "
              f"{same:.2%} of 4000 paired trajectories identical")
    assert g.rejections > 0.05 * g.leaps and r["rejections"] > 0.05 * r["leaps"]
    assert same >= 0.99
    level = P99 / (3 * len(tr) * P)
    for pt in range(1, P + 1):
        compare_final(g.samples[0, :, pt, :], r["samples"][0, :, pt, :], f"{name} point {pt}", p=level)
    # rejections per attempt: the same rate in the engine and the oracle
    pg, po = g.rejections / (g.leaps + g.rejections), r["rejections"] / (r["leaps"] + r["rejections"])
    se = np.sqrt(pg * (1 - pg) / (g.leaps + g.rejections) + po * (1 - po) / (r["leaps"] + r["rejections"]))
    assert abs(pg - po) <= 4 * se, (pg, po, se)


@pytest.mark.parametrize("variant", [_ffi.VARIANT_THREAD, _ffi.VARIANT_LANES8, _ffi.VARIANT_LANES16,
                                     _ffi.VARIANT_WARP, _ffi.VARIANT_CTA])
def test_every_group_kind_draws_the_oracles_firings(variant, capsys):
    """Small Poisson means, paired with the oracle.  The 128 x 256 toy
    network runs about 110 leaps per realization to t_final 5e-5; its
    median mean per leap is 0.017, so nearly every draw is settled by q >=
    mu or by the exact k <= 1 tests.  Thread groups run the tests in the
    channel loop after the q >= mu compare, sub-warp and warp groups after
    it, and CTA groups in it.  The oracle draws the same Philox words and
    applies the same rule in FP64, so the trajectories agree realization by
    realization: one wrong count in any leap makes a trajectory differ.
    Only the FP32 propensity sums can still part the two: measured on
    GB300, 0.25 % of the realizations differ (0.05 % of the thread groups'
    on the 16 x 16 network)."""
    if variant == _ffi.VARIANT_THREAD:
        # a thread keeps its whole state in its slot: a 16 x 16 network
        m = Model.generate("toy", n_species=16, n_channels=16, seed=3, x0_min=0, x0_max=2000)
        T = 0.01
    else:
        m = Model.generate("toy")
        T = 5e-5
    tr = list(range(8))
    o = ora.OracleModel.from_desc(m.desc())
    g = m.simulate(T, 2000, seed=9, intervals=1, tracked=tr, variant=variant, keep_samples=True)
    r = o.simulate(T, 2000, seed=9, intervals=1, tracked=tr, threads=8)
    same = np.mean(np.all(r["samples"][0] == g.samples[0], axis=(1, 2)))
    with capsys.disabled():
        print(f"\nvariant {variant}: {g.leaps / 2000:.0f} leaps per realization, {same:.2%} of 2000 paired "
              f"trajectories identical to the oracle")
    assert g.variant == variant
    assert g.leaps >= 100 * 2000
    assert same >= 0.95
    if same == 1.0:
        assert (g.leaps, g.ssa_steps) == (r["leaps"], r["ssa_steps"])


def test_halving_cap_reports_numeric():
    m = REJ_MODELS["decay"][0]()
    # from 40 molecules the first two attempts (tau1 = 3, then 1.5) are both
    # clamped to the end time, a mean of 40 firings, rejected with
    # probability ~0.46 each: a quarter of the realizations need a second
    # halving
    with pytest.raises(_ffi.TLError) as e:
        m.simulate(1.0, 256, seed=5, eps=3.0, tracked=[0], max_halvings=1)
    assert e.value.status == 12 and "halving" in str(e.value)
    ok = m.simulate(1.0, 256, seed=5, eps=3.0, tracked=[0])
    assert ok.status == 0 and ok.rejections > 0


@pytest.mark.parametrize("variant", [_ffi.VARIANT_WARP, _ffi.VARIANT_THREAD])
def test_staging_wait_timeout_is_reported_and_context_survives(variant):
    fam = {_ffi.VARIANT_WARP: ("toy", {}), _ffi.VARIANT_THREAD: ("dimer", dict(x0_min=500, x0_max=500))}[variant]
    m = Model.generate(fam[0], **fam[1])
    kw = dict(t_final=0.002 if fam[0] == "toy" else 0.1, n=512, seed=2, tracked=[0, 1], variant=variant)
    with pytest.raises(_ffi.TLError) as e:
        m.simulate(stage_wait_polls=-1, **kw)
    assert e.value.status == 7
    a = m.simulate(keep_samples=True, **kw)
    b = m.simulate(keep_samples=True, stage_wait_polls=1 << 20, **kw)
    assert a.status == 0 and np.array_equal(a.samples, b.samples)
