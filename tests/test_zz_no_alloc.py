"""tl_simulate_static: the no-allocation entry point.

Some callers of this library cannot call cudaMalloc: a host whose GPU memory
a pool allocator has already reserved, or a latency-bound loop that cannot
take cudaMalloc / cudaFree's device-wide synchronisation.  tl_simulate_static
runs the same fused simulation as tl_simulate with all of its device scratch
in one fixed file-scope device array.  These tests call it through the C ABI
and compare it with tl_simulate; they pass alone in a fresh process and after
the rest of the suite (this file is collected last)."""
import numpy as np
import pytest

from tau_leaping_gb300 import Model, _ffi

pytestmark = pytest.mark.gpu


def _free_bytes() -> int:
    import torch
    return int(torch.cuda.mem_get_info(0)[0])


def test_static_entry_matches_simulate_on_two_calls_in_a_row():
    m = Model.generate("toy", n_species=32, n_channels=64, seed=4, x0_max=3000)
    small = dict(t_final=0.005, n=500, seed=3, tracked=[0, 1, 2], intervals=2)
    m.simulate(**small)              # uploads the model's tables (allocates)
    m.simulate_static(**small)       # first call on the device: symbol lookup
    # a larger ensemble and grid than any earlier call on this model: a
    # regression that fell back to the model's grow-only scratch or to
    # cudaMalloc would have to allocate here
    big = dict(t_final=0.005, n=6000, seed=3, tracked=[0, 1, 2], intervals=5)
    free0 = _free_bytes()
    got = [m.simulate_static(**big) for _ in range(2)]   # the second reuses the array
    assert _free_bytes() == free0, "tl_simulate_static changed the device's free memory"
    ref = m.simulate(**big)
    for g in got:
        assert g.status == 0
        assert np.allclose(g.mean, ref.mean, rtol=1e-12, atol=0)
        assert np.allclose(g.stddev, ref.stddev, rtol=1e-12, atol=0)
        assert np.array_equal(g.times, ref.times)
        assert (g.leaps, g.ssa_steps, g.rejections) == (ref.leaps, ref.ssa_steps, ref.rejections)
    d = Model.generate("dimer", x0_min=2000, x0_max=2000)
    dref = d.simulate(1.0, 3000, seed=2, tracked=[0, 1])
    dgot = d.simulate_static(1.0, 3000, seed=2, tracked=[0, 1])
    assert np.allclose(dgot.mean, dref.mean, rtol=1e-12, atol=0)


def test_static_entry_with_compatibility_switches_matches_simulate():
    """A run with reference-compatibility switches takes the general kernel
    build on both entry points."""
    m = Model.generate("toy", n_species=32, n_channels=64, seed=4, x0_max=3000)
    kw = dict(t_final=0.005, n=2000, seed=5, tracked=[0, 1], flags=_ffi.FLAG_COMPAT_REFERENCE)
    ref = m.simulate(**kw)
    got = m.simulate_static(**kw)
    assert np.allclose(got.mean, ref.mean, rtol=1e-12, atol=0)
    assert (got.leaps, got.ssa_steps, got.rejections) == (ref.leaps, ref.ssa_steps, ref.rejections)


def test_static_entry_global_slots_match_simulate():
    """CTA groups whose state lives in global memory: the per-CTA slots come
    out of the fixed array too."""
    m = Model.generate("colloid", n_species=60)
    kw = dict(t_final=0.005, n=512, seed=3, tracked=[0, 1, 9], intervals=2, variant=_ffi.VARIANT_CTA,
              flags=_ffi.FLAG_GLOBAL_SLOTS)
    ref = m.simulate(**kw)
    for _ in range(2):
        got = m.simulate_static(**kw)
        assert np.allclose(got.mean, ref.mean, rtol=1e-12, atol=0)
        assert np.allclose(got.stddev, ref.stddev, rtol=1e-12, atol=0)
        assert (got.leaps, got.ssa_steps, got.rejections) == (ref.leaps, ref.ssa_steps, ref.rejections)


def test_static_entry_limits():
    m = Model.generate("dimer", x0_min=500, x0_max=500)
    with pytest.raises(_ffi.TLError) as e:      # tables not resident yet
        m.simulate_static(0.1, 16, tracked=[0])
    assert e.value.status == 1 and "never allocates" in str(e.value)
    m.simulate(0.1, 16, tracked=[0])
    with pytest.raises(_ffi.TLError) as e:      # scratch beyond the fixed array
        m.simulate_static(0.1, 3_000_000, tracked=[0, 1, 2], intervals=4)
    assert e.value.status == 1 and "bytes of device scratch" in str(e.value)
    with pytest.raises(_ffi.TLError) as e:
        m.simulate_static(0.1, 16, tracked=[0], variant=_ffi.VARIANT_PLAIN)
    assert e.value.status == 3
