"""Simulation-level parity of the CUDA path with the FP64 oracle.

Statistical checks use fixed seeds, so each is deterministic; the
acceptance level is 99% (p > 0.01) unless stated otherwise.
"""
import numpy as np
import pytest
from scipy import stats

from oracle import py as ora
from tau_leaping_gb300 import Model, _ffi

pytestmark = pytest.mark.gpu

P99 = 0.01


def dimer(s1=2000):
    return Model.generate("dimer", x0_min=s1, x0_max=s1)


def compare_final(a, b, label, p=P99):
    """a, b: [R, K] samples at t_final.  Welch t-test on means, Levene on
    variances, two-sample KS on each tracked species."""
    for k in range(a.shape[1]):
        x, y = a[:, k].astype(float), b[:, k].astype(float)
        pt = stats.ttest_ind(x, y, equal_var=False).pvalue
        pl = stats.levene(x, y).pvalue
        pk = stats.ks_2samp(x, y).pvalue
        assert pt > p and pl > p and pk > p, f"{label} species {k}: t {pt:.3g} levene {pl:.3g} ks {pk:.3g}"


@pytest.mark.parametrize("variant", [_ffi.VARIANT_THREAD, _ffi.VARIANT_WARP, _ffi.VARIANT_CTA, _ffi.VARIANT_PLAIN,
                                     _ffi.VARIANT_LANES2, _ffi.VARIANT_LANES4, _ffi.VARIANT_LANES8,
                                     _ffi.VARIANT_LANES16])
def test_dimer_tau_leap_matches_oracle(variant):
    m = dimer()
    o = ora.OracleModel.from_desc(m.desc())
    T = 2.0
    g = m.simulate(T, 20000, seed=5, intervals=4, tracked=[0, 1], variant=variant, keep_samples=True)
    r = o.simulate(T, 4000, seed=99, intervals=4, tracked=[0, 1], threads=8)
    assert g.truncated == 0
    assert g.leaps > 0 and g.ssa_steps > 0
    compare_final(g.samples[0, :, -1, :], r["samples"][0, :, -1, :], f"variant {variant}")
    # intermediate grid point too
    compare_final(g.samples[0, :, 2, :], r["samples"][0, :, 2, :], f"variant {variant} t=T/2")
    # the device reduction equals the host reduction of the same samples
    s = g.samples[0].astype(np.float64)
    assert np.allclose(g.mean[0], s.mean(0), rtol=1e-12)
    assert np.allclose(g.stddev[0], s.std(0, ddof=1), rtol=1e-9)
    assert np.allclose(g.times[0], [0, 0.5, 1.0, 1.5, 2.0])


def test_dimer_tau_leap_close_to_exact_ssa():
    m = dimer(1000)
    o = ora.OracleModel.from_desc(m.desc())
    T = 1.0
    g = m.simulate(T, 100000, seed=3, tracked=[0, 1], keep_samples=True)
    r = o.simulate(T, 20000, seed=4, tracked=[0, 1], method=1, threads=8)
    a, b = g.samples[0, :, -1, :].astype(float), r["samples"][0, :, -1, :].astype(float)
    for k in range(2):
        ma, mb = a[:, k].mean(), b[:, k].mean()
        se = np.sqrt(a[:, k].var() / len(a) + b[:, k].var() / len(b))
        # tau-leaping bias (eps = 0.03) + 4 standard errors
        assert abs(ma - mb) <= 0.01 * abs(mb) + 4 * se, (k, ma, mb, se)
        va, vb = a[:, k].var(ddof=1), b[:, k].var(ddof=1)
        sev = vb * np.sqrt(2 / len(b) + 2 / len(a))
        assert abs(va - vb) <= 0.02 * vb + 4 * sev, (k, va, vb)


def test_deterministic_and_variant_independent_streams():
    m = dimer()
    kw = dict(t_final=1.0, n=512, seed=9, tracked=[0, 1], keep_samples=True, intervals=2)
    a = m.simulate(variant=_ffi.VARIANT_WARP, **kw)
    b = m.simulate(variant=_ffi.VARIANT_WARP, **kw)
    assert np.array_equal(a.samples, b.samples)
    assert (a.leaps, a.ssa_steps, a.rejections) == (b.leaps, b.ssa_steps, b.rejections)
    c = m.simulate(variant=_ffi.VARIANT_WARP, block_threads=64, **kw)
    assert np.array_equal(a.samples, c.samples), "scheduling must not change a realization"
    d = m.simulate(variant=_ffi.VARIANT_LANES4, block_threads=64, **kw)
    e = m.simulate(variant=_ffi.VARIANT_LANES4, block_threads=256, **kw)
    assert np.array_equal(d.samples, e.samples), "scheduling must not change a sub-warp realization"


def test_plain_graph_replay_is_bit_identical():
    """The graph-captured plain step loop launches the same kernels."""
    m = Model.generate("toy")
    kw = dict(t_final=0.01, n=700, seed=4, tracked=[0, 4], keep_samples=True, intervals=3,
              variant=_ffi.VARIANT_PLAIN)
    a = m.simulate(**kw)
    b = m.simulate(flags=_ffi.FLAG_GRAPH, **kw)
    assert np.array_equal(a.samples, b.samples)
    assert (a.leaps, a.ssa_steps, a.rejections) == (b.leaps, b.ssa_steps, b.rejections)
    assert a.launches == b.launches


def test_rate_sets_are_independent_of_batch_neighbours():
    m = dimer()
    base = m.desc()["rate"]
    sets1 = np.stack([base, base * 1.5])
    sets2 = np.stack([base, base * 0.5, base * 2.0])
    kw = dict(t_final=1.0, n=256, seed=4, tracked=[0, 1], keep_samples=True)
    a = m.simulate(rate_sets=sets1, t_final_sets=[1.0, 0.5], **kw)
    b = m.simulate(rate_sets=sets2, t_final_sets=[1.0, 2.0, 3.0], **kw)
    assert np.array_equal(a.samples[0], b.samples[0])
    assert np.allclose(a.times[1], [0.0, 0.5])


def test_edge_cases():
    # nothing can fire: the state holds
    m = Model.from_arrays([0, 0], [1.0], [0, 2], [0, 1], [-1, 1])
    r = m.simulate(5.0, 16, intervals=3, keep_samples=True)
    assert r.leaps == 0 and r.ssa_steps == 0
    assert not r.samples.any()
    # single realization, zero rate channel, source channel (no reactant)
    m2 = Model.from_arrays([10, 0], [0.0, 2.0], [0, 2, 3], [0, 1, 1], [-1, 1, 1])
    r2 = m2.simulate(3.0, 1, intervals=3, keep_samples=True, tracked=[0, 1])
    assert r2.samples[0, 0, :, 0].tolist() == [10, 10, 10, 10]
    assert r2.samples[0, 0, -1, 1] > 0
    # step cap: reported and every realization truncated
    m3 = dimer()
    r3 = m3.simulate(10.0, 64, max_steps=5, allow_truncation=True, tracked=[0])
    assert r3.status == 5 and r3.truncated == 64
    with pytest.raises(_ffi.TLError) as e:
        m3.simulate(10.0, 64, max_steps=5, tracked=[0])
    assert e.value.status == 5
    # invalid configuration
    for bad in (dict(t_final=-1.0, n=4), dict(t_final=1.0, n=0), dict(t_final=1.0, n=4, intervals=0),
                dict(t_final=1.0, n=4, tracked=[7])):
        with pytest.raises(_ffi.TLError) as e:
            m3.simulate(**bad)
        assert e.value.status == 1


@pytest.mark.parametrize("variant", [_ffi.VARIANT_THREAD, _ffi.VARIANT_LANES4, _ffi.VARIANT_LANES16,
                                     _ffi.VARIANT_WARP, _ffi.VARIANT_CTA])
def test_int64_populations_on_every_group_kind(variant):
    """The dimer with 64-bit populations through each group kind: the same
    ensemble statistics as the FP64 oracle, and the same trajectories as the
    32-bit build of the model (its populations stay far below 2^31)."""
    d = dimer(2000).desc()
    m32 = Model.from_arrays(d["x0"], d["rate"], d["col_ptr"], d["row_ind"], d["stoich"], pop_bits=32)
    m64 = Model.from_arrays(d["x0"], d["rate"], d["col_ptr"], d["row_ind"], d["stoich"], pop_bits=64)
    kw = dict(t_final=1.0, n=2048, seed=7, tracked=[0, 1], keep_samples=True, variant=variant)
    a, b = m64.simulate(**kw), m32.simulate(**kw)
    assert np.array_equal(a.samples, b.samples)
    r = ora.OracleModel.from_desc(d).simulate(1.0, 2048, seed=8, tracked=[0, 1], threads=8)
    compare_final(a.samples[0, :, -1, :], r["samples"][0, :, -1, :], f"int64 variant {variant}")


def test_int32_overflow_detected():
    # S1 -> 2 S1 from 2^30: grows past int32 within t=2
    m = Model.from_arrays([2**30], [1.0], [0, 2], [0, 0], [-1, 2], pop_bits=32)
    with pytest.raises(_ffi.TLError) as e:
        m.simulate(2.0, 4, tracked=[0])
    assert e.value.status == 4
    m64 = Model.from_arrays([2**30], [1.0], [0, 2], [0, 0], [-1, 2], pop_bits=64)
    r = m64.simulate(1.0, 256, tracked=[0], keep_samples=True)
    assert r.samples.max() > 2**31
    # explicit tau-leaping grows the mean by (1 + tau) per leap, not e^tau:
    # compare with the FP64 oracle running the same method
    o = ora.OracleModel.from_desc(m64.desc())
    ref = o.simulate(1.0, 256, seed=8, tracked=[0], threads=8)["samples"][0, :, -1, 0].astype(float)
    dev = r.samples[0, :, -1, 0].astype(float)
    se = np.sqrt(dev.var() / len(dev) + ref.var() / len(ref))
    assert abs(dev.mean() - ref.mean()) <= 4 * se + 1e-6 * ref.mean()


def test_chain_mixed_precision_error_vs_ssa():
    m = Model.generate("chain", n_species=64)
    o = ora.OracleModel.from_desc(m.desc())
    tr = list(range(0, 64, 8))
    g = m.simulate(1.0, 20000, seed=2, tracked=tr, keep_samples=True)
    r = o.simulate(1.0, 4000, seed=3, tracked=tr, method=1, threads=8)
    a, b = g.samples[0, :, -1, :].astype(float), r["samples"][0, :, -1, :].astype(float)
    rel_mean = np.abs(a.mean(0) - b.mean(0)) / b.mean(0)
    se = np.sqrt(a.var(0) / len(a) + b.var(0) / len(b)) / b.mean(0)
    assert np.all(rel_mean <= 0.01 + 4 * se), rel_mean


def test_colloid_cta_matches_oracle():
    m = Model.generate("colloid", n_species=60)
    o = ora.OracleModel.from_desc(m.desc())
    g = m.simulate(0.01, 2048, seed=6, tracked=[0, 1, 9], variant=_ffi.VARIANT_CTA, keep_samples=True)
    w = m.simulate(0.01, 2048, seed=6, tracked=[0, 1, 9], variant=_ffi.VARIANT_WARP, keep_samples=True)
    r = o.simulate(0.01, 1024, seed=7, tracked=[0, 1, 9], threads=8)
    compare_final(g.samples[0, :, -1, :], r["samples"][0, :, -1, :], "colloid cta")
    compare_final(w.samples[0, :, -1, :], r["samples"][0, :, -1, :], "colloid warp")


def test_colloid_full_config_within_1pct_of_fp64_oracle(capsys):
    """Colloidal aggregation, 250 species x 31250 channels, int64, t_final
    0.01, 4096 realizations (the full configuration), compared realization
    by realization with the FP64 oracle running the same method: both draw
    realization r from the same Philox stream (same seed, same realization
    ids), so the pairs differ only where FP32 and FP64 arithmetic pick a
    different Poisson count.  The ensemble mean and the variance of every
    species agree within 1 %; the errors are printed.  A second, independent
    oracle ensemble (another seed) checks the statistics at 99 % on two
    species."""
    m = Model.generate("colloid")
    N = m.n_species
    g = m.simulate(0.01, 4096, seed=13, tracked=list(range(N)), keep_samples=True)
    o = ora.OracleModel.from_desc(m.desc())
    r = o.simulate(0.01, 4096, seed=13, tracked=list(range(N)), threads=16)
    a, b = g.samples[0, :, -1, :].astype(float), r["samples"][0, :, -1, :].astype(float)
    ma, mb, va, vb = a.mean(0), b.mean(0), a.var(0, ddof=1), b.var(0, ddof=1)
    rel_m = np.abs(ma - mb) / mb
    rel_v = np.abs(va - vb) / vb
    same = np.mean(np.all(a == b, axis=1))
    with capsys.disabled():
        print(f"\ncolloid-250 vs FP64 oracle, 4096 paired realizations: mean rel err max {rel_m.max():.2e} "
              f"rms {np.sqrt((rel_m ** 2).mean()):.2e}; variance rel err max {rel_v.max():.2e} "
              f"rms {np.sqrt((rel_v ** 2).mean()):.2e}; {same:.1%} of final states identical")
    assert rel_m.max() <= 0.01, rel_m.max()
    assert rel_v.max() <= 0.01, rel_v.max()
    ind = o.simulate(0.01, 2048, seed=14, tracked=[0, 9], threads=16)["samples"][0, :, -1, :]
    compare_final(a[:, [0, 9]], ind, "colloid-250 independent oracle ensemble")


def test_state_larger_than_shared_memory_runs_from_global_slots():
    """Colloidal aggregation with 400 species: 80 000 channels, 320 KB of
    propensities per realization, more than a CTA's shared memory.  CTA
    groups then keep each realization's state in global memory."""
    m = Model.generate("colloid", n_species=400)
    assert m.n_channels == 80000
    g = m.simulate(0.002, 256, seed=4, tracked=[0, 1, 9], keep_samples=True)
    assert g.variant == _ffi.VARIANT_CTA and g.leaps > 0
    o = ora.OracleModel.from_desc(m.desc())
    r = o.simulate(0.002, 256, seed=5, tracked=[0, 1, 9], threads=8)
    compare_final(g.samples[0, :, -1, :], r["samples"][0, :, -1, :], "colloid-400 global slots")
    # the same realizations again: deterministic
    h = m.simulate(0.002, 256, seed=4, tracked=[0, 1, 9], keep_samples=True)
    assert np.array_equal(g.samples, h.samples)


def test_global_slots_are_bit_identical_to_shared_slots():
    """TL_FLAG_GLOBAL_SLOTS moves a CTA group's state to global memory; the
    arithmetic is the same, so the trajectories are too."""
    m = Model.generate("colloid", n_species=60)
    kw = dict(t_final=0.005, n=512, seed=3, tracked=[0, 1, 9], keep_samples=True, intervals=2,
              variant=_ffi.VARIANT_CTA)
    a = m.simulate(**kw)
    b = m.simulate(flags=_ffi.FLAG_GLOBAL_SLOTS, **kw)
    assert np.array_equal(a.samples, b.samples)
    assert (a.leaps, a.ssa_steps, a.rejections) == (b.leaps, b.ssa_steps, b.rejections)


def test_measured_autotuner_picks_a_plan_and_caches_it():
    m = Model.generate("toy", n_species=32, n_channels=64, seed=4, x0_max=3000)
    o = ora.OracleModel.from_desc(m.desc())
    flags = _ffi.FLAG_AUTOTUNE_MEASURE
    a = m.simulate(0.005, 3000, seed=3, tracked=[0, 1], flags=flags, keep_samples=True)
    b = m.simulate(0.005, 3000, seed=3, tracked=[0, 1], flags=flags, keep_samples=True)
    assert a.variant in (_ffi.VARIANT_THREAD, _ffi.VARIANT_WARP, _ffi.VARIANT_CTA, _ffi.VARIANT_LANES2,
                         _ffi.VARIANT_LANES4, _ffi.VARIANT_LANES8, _ffi.VARIANT_LANES16)
    assert (a.variant, a.block_threads) == (b.variant, b.block_threads)
    assert np.array_equal(a.samples, b.samples)
    r = o.simulate(0.005, 1500, seed=4, tracked=[0, 1], threads=8)
    compare_final(a.samples[0, :, -1, :], r["samples"][0, :, -1, :], "autotuned")


@pytest.mark.parametrize("variant,block", [(_ffi.VARIANT_CTA, 64), (_ffi.VARIANT_CTA, 128), (_ffi.VARIANT_CTA, 256),
                                           (_ffi.VARIANT_WARP, 64), (_ffi.VARIANT_THREAD, 32),
                                           (_ffi.VARIANT_LANES2, 64), (_ffi.VARIANT_LANES4, 128),
                                           (_ffi.VARIANT_LANES8, 256), (_ffi.VARIANT_LANES16, 128)])
def test_group_widths_agree_on_chain(variant, block):
    m = Model.generate("chain", n_species=48)
    o = ora.OracleModel.from_desc(m.desc())
    g = m.simulate(0.5, 4096, seed=5, tracked=[0, 7], variant=variant, block_threads=block, keep_samples=True,
                   flags=_ffi.FLAG_NO_STAGE if block == 128 else 0)
    r = o.simulate(0.5, 2048, seed=6, tracked=[0, 7], threads=8)
    compare_final(g.samples[0, :, -1, :], r["samples"][0, :, -1, :], f"chain v{variant} b{block}")


def test_chain_1024_full_config_error_vs_exact_solution(capsys):
    """Cyclic chain, 1024 species, 65536 realizations, t_final 1 (mixed
    precision: FP32 propensities / tau, FP64 time).  Reports the per-species
    error of the ensemble mean and variance against the exact CME solution
    (FP64), and checks that the mixed-precision device run agrees with the
    FP64 oracle running the same tau-leaping method: at eps = 0.03 the chain
    takes ~17 leaps, and the method's own bias (~1 % on means, ~10 % on
    variances, the same in FP64) dominates the error, not the precision."""
    m = Model.generate("chain")
    mean, var = ora.chain_exact_moments(m.desc()["x0"], 1.0, 1.0)
    r = m.simulate(1.0, 65536, seed=11, tracked=list(range(1024)))
    gm, gv = r.mean[0, -1], r.stddev[0, -1] ** 2
    rel_m = np.abs(gm - mean) / mean
    rel_v = np.abs(gv - var) / var
    o = ora.OracleModel.from_desc(m.desc())
    x = o.simulate(1.0, 3000, seed=12, threads=8)["samples"][0, :, -1, :].astype(float)
    om, ov = x.mean(0), x.var(0, ddof=1)
    orm, orv = np.abs(om - mean) / mean, np.abs(ov - var) / var
    with capsys.disabled():
        print(f"\nchain-1024 vs exact CME, device (65536 realizations): mean rel err max {rel_m.max():.2e} "
              f"rms {np.sqrt((rel_m**2).mean()):.2e}; variance rel err max {rel_v.max():.2e} "
              f"rms {np.sqrt((rel_v**2).mean()):.2e}; leaps/realization {r.leaps / 65536:.1f}")
        print(f"chain-1024 vs exact CME, FP64 oracle tau-leaping (3000 realizations): mean rel err max "
              f"{orm.max():.2e} rms {np.sqrt((orm**2).mean()):.2e}; variance rel err rms "
              f"{np.sqrt((orv**2).mean()):.2e}")
    # precision: device and FP64 tau-leaping agree within sampling error
    se = np.sqrt(gv / 65536 + ov / len(x))
    assert np.mean(np.abs(gm - om) <= 4 * se) >= 0.99
    assert np.sqrt(np.mean(((gv - ov) / ov) ** 2)) <= 0.05
    # method accuracy: sanity bounds against the exact solution
    assert rel_m.max() < 0.02
    assert np.sqrt((rel_v ** 2).mean()) < 0.15


def test_heuristic_group_width_follows_model_and_ensemble():
    """The heuristic's group width (the fewest lanes of 8, 16 and 32 with at
    most 16 channels and 8 species rows per lane, on ensembles that fill
    the warp-group slots at least 8 times, unscored runs only), and the
    16-lane plan of the 128 x 256 network against the FP64 oracle."""
    toy = Model.generate("toy")
    big = toy.simulate(0.0005, 100_000, seed=3, tracked=[0, 4])
    assert big.variant == _ffi.VARIANT_LANES16
    assert toy.simulate(0.0005, 20_000, seed=3, tracked=[0, 4]).variant == _ffi.VARIANT_WARP
    assert toy.sensitivity(0.0005, 100_000, seed=3, tracked=[0])["variant"] == _ffi.VARIANT_WARP
    small = Model.generate("toy", n_species=32, n_channels=64, seed=4, x0_max=3000)
    assert small.simulate(0.0005, 100_000, seed=3, tracked=[0]).variant == _ffi.VARIANT_LANES8
    wide = Model.generate("toy", n_species=256, n_channels=512, seed=5)
    assert wide.simulate(0.0002, 100_000, seed=3, tracked=[0]).variant == _ffi.VARIANT_WARP
    g = toy.simulate(0.002, 100_000, seed=6, tracked=[0, 4], keep_samples=True)
    assert g.variant == _ffi.VARIANT_LANES16
    r = ora.OracleModel.from_desc(toy.desc()).simulate(0.002, 4000, seed=7, tracked=[0, 4], threads=16)
    compare_final(g.samples[0, :, -1, :], r["samples"][0, :, -1, :], "toy network, 16-lane plan")
