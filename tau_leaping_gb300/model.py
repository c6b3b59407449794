"""Python face of the C ABI, shaped like the reference's ``Model`` class
(tau_leaping/model.h:20-98): read a StochKit model, run realizations,
get the per-species statistics.

Every call goes through libtl.so; arrays are numpy and host-resident.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _ffi as F


def _ptr(a: np.ndarray | None, ctype):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ctype))


@dataclass
class SimResult:
    times: np.ndarray            # [S][P]
    mean: np.ndarray             # [S][P][K]
    stddev: np.ndarray           # [S][P][K]
    samples: np.ndarray | None   # [S][R][P][K]
    leaps: int
    ssa_steps: int
    rejections: int
    truncated: int
    kernel_ms: float
    total_ms: float
    variant: int
    block_threads: int
    grid: int
    launches: int
    status: int = 0
    extra: dict = field(default_factory=dict)


class Model:
    """A device-resident reaction network (owns a tl_model handle)."""

    def __init__(self, handle: int):
        self._h = C.c_void_p(handle)
        info = F.ModelInfo()
        F.check(F.lib().tl_model_get_info(self._h, C.byref(info)), "tl_model_get_info")
        self.n_species = info.n_species
        self.n_channels = info.n_channels
        self.nnz_raw = info.nnz_raw
        self.nnz_net = info.nnz_net
        self.pop_bits = info.pop_bits

    # ---- construction -------------------------------------------------
    @classmethod
    def from_stochkit(cls, path: str, pop_bits: int = 0) -> "Model":
        h = C.c_void_p()
        F.check(F.lib().tl_model_from_stochkit(str(path).encode(), pop_bits, C.byref(h)), "tl_model_from_stochkit")
        return cls(h.value)

    @classmethod
    def from_arrays(cls, x0, rate, col_ptr, row_ind, stoich, pop_bits: int = 0) -> "Model":
        x0 = np.ascontiguousarray(x0, dtype=np.int64)
        rate = np.ascontiguousarray(rate, dtype=np.float64)
        col_ptr = np.ascontiguousarray(col_ptr, dtype=np.int32)
        row_ind = np.ascontiguousarray(row_ind, dtype=np.int32)
        stoich = np.ascontiguousarray(stoich, dtype=np.int8)
        d = F.ModelDesc(len(x0), len(rate), len(row_ind), _ptr(x0, C.c_int64), _ptr(rate, C.c_double),
                        _ptr(col_ptr, C.c_int32), _ptr(row_ind, C.c_int32), _ptr(stoich, C.c_int8), pop_bits)
        h = C.c_void_p()
        F.check(F.lib().tl_model_create(C.byref(d), C.byref(h)), "tl_model_create")
        return cls(h.value)

    @classmethod
    def generate(cls, family: str | int, **kw) -> "Model":
        fam = {"dimer": F.GEN_DIMER, "toy": F.GEN_TOY, "chain": F.GEN_CHAIN, "colloid": F.GEN_COLLOID}.get(family, family)
        g = F.GenParams()
        F.lib().tl_gen_params_init(C.byref(g), int(fam))
        for k, v in kw.items():
            if not hasattr(g, k):
                raise TypeError(f"unknown generator parameter {k}")
            setattr(g, k, v)
        h = C.c_void_p()
        F.check(F.lib().tl_model_generate(C.byref(g), C.byref(h)), "tl_model_generate")
        return cls(h.value)

    def close(self) -> None:
        if self._h is not None and self._h.value:
            F.lib().tl_model_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- introspection ------------------------------------------------
    def species_names(self) -> list[str]:
        L = F.lib()
        return [L.tl_model_species_name(self._h, i).decode() for i in range(self.n_species)]

    def species_index(self, name: str) -> int:
        return F.lib().tl_model_species_index(self._h, name.encode())

    def desc(self) -> dict:
        x0 = np.zeros(self.n_species, np.int64)
        rate = np.zeros(self.n_channels, np.float64)
        cp = np.zeros(self.n_channels + 1, np.int32)
        ri = np.zeros(self.nnz_raw, np.int32)
        st = np.zeros(self.nnz_raw, np.int8)
        F.check(F.lib().tl_model_get_desc(self._h, _ptr(x0, C.c_int64), _ptr(rate, C.c_double), _ptr(cp, C.c_int32),
                                          _ptr(ri, C.c_int32), _ptr(st, C.c_int8)), "tl_model_get_desc")
        return {"x0": x0, "rate": rate, "col_ptr": cp, "row_ind": ri, "stoich": st}

    def tables(self) -> dict:
        o = np.zeros(self.n_channels, np.int8)
        s0 = np.zeros(self.n_channels, np.int32)
        s1 = np.zeros(self.n_channels, np.int32)
        rp = np.zeros(self.n_species + 1, np.int32)
        vc = np.zeros(self.nnz_raw, np.int32)
        F.check(F.lib().tl_model_get_tables(self._h, _ptr(o, C.c_int8), _ptr(s0, C.c_int32), _ptr(s1, C.c_int32),
                                            _ptr(rp, C.c_int32), _ptr(vc, C.c_int32)), "tl_model_get_tables")
        return {"order": o, "s0": s0, "s1": s1, "csr_row_ptr": rp, "csr_valcol": vc}

    def write_stochkit(self, path: str) -> None:
        F.check(F.lib().tl_model_write_stochkit(self._h, str(path).encode()), "tl_model_write_stochkit")

    # ---- hot path -----------------------------------------------------
    def _cfg(self, t_final, n, seed, intervals, tracked, eps, variant, flags, rate_sets, t_final_sets,
             max_steps, block_threads, stream, n_critical=0, ssa_factor=0, ssa_block=0, realization_offset=0,
             max_halvings=0, stage_wait_polls=0):
        cfg = F.RunCfg()
        F.lib().tl_run_cfg_init(C.byref(cfg))
        cfg.t_final = float(t_final)
        cfg.eps = float(eps)
        cfg.n_realizations = int(n)
        cfg.seed = int(seed)
        cfg.n_intervals = int(intervals)
        tr = np.ascontiguousarray(tracked if tracked is not None else [], dtype=np.int32)
        cfg.n_tracked = len(tr)
        cfg.tracked = _ptr(tr, C.c_int32) if len(tr) else None
        keep = [tr]
        if rate_sets is not None:
            rs = np.ascontiguousarray(rate_sets, dtype=np.float64).reshape(-1, self.n_channels)
            cfg.n_rate_sets = rs.shape[0]
            cfg.rate_sets = _ptr(rs, C.c_double)
            keep.append(rs)
            if t_final_sets is not None:
                tf = np.ascontiguousarray(t_final_sets, dtype=np.float64)
                assert len(tf) == rs.shape[0]
                cfg.t_final_sets = _ptr(tf, C.c_double)
                keep.append(tf)
        cfg.variant = int(variant)
        cfg.block_threads = int(block_threads)
        cfg.flags = int(flags)
        cfg.max_steps = int(max_steps)
        cfg.n_critical = int(n_critical)
        cfg.ssa_factor = int(ssa_factor)
        cfg.ssa_block = int(ssa_block)
        cfg.stream = stream
        cfg.realization_offset = int(realization_offset)
        cfg.max_halvings = int(max_halvings)
        cfg.stage_wait_polls = int(stage_wait_polls)
        return cfg, keep

    def simulate(self, t_final: float, n: int, seed: int = 1, intervals: int = 1, tracked=None,
                 eps: float = 0.03, variant: int = F.VARIANT_AUTO, flags: int = 0, rate_sets=None,
                 t_final_sets=None, keep_samples: bool = False, max_steps: int = 0, block_threads: int = 0,
                 stream=None, allow_truncation: bool = False, **extra) -> SimResult:
        if tracked is None:
            tracked = list(range(self.n_species))
        tracked = [self.species_index(t) if isinstance(t, str) else int(t) for t in tracked]
        if keep_samples:
            flags |= F.FLAG_KEEP_SAMPLES
        cfg, keep = self._cfg(t_final, n, seed, intervals, tracked, eps, variant, flags, rate_sets, t_final_sets,
                              max_steps, block_threads, stream, **extra)
        S = max(1, cfg.n_rate_sets)
        Pn, K = intervals + 1, len(tracked)
        times = np.zeros((S, Pn))
        mean = np.zeros((S, Pn, K))
        sd = np.zeros((S, Pn, K))
        samples = np.zeros((S, n, Pn, K), np.int64) if keep_samples else None
        res = F.Result()
        res.times = _ptr(times, C.c_double)
        res.mean = _ptr(mean, C.c_double)
        res.stddev = _ptr(sd, C.c_double)
        res.samples = _ptr(samples, C.c_int64)
        st = F.lib().tl_simulate(self._h, C.byref(cfg), C.byref(res))
        if st != F.TL_OK and not (allow_truncation and st == 5):
            F.check(st, "tl_simulate")
        del keep
        return SimResult(times, mean, sd, samples, res.leaps, res.ssa_steps, res.rejections, res.truncated,
                         res.kernel_ms, res.total_ms, res.variant_used, res.block_threads_used, res.grid_used,
                         res.launches, st)

    def simulate_static(self, t_final: float, n: int, seed: int = 1, intervals: int = 1, tracked=None,
                        eps: float = 0.03, variant: int = F.VARIANT_AUTO, flags: int = 0, rate_sets=None,
                        t_final_sets=None, block_threads: int = 0, stream=None) -> SimResult:
        """tl_simulate_static: the same run as simulate() with no device
        allocation (scratch in the library's fixed device array).  For
        callers that cannot call cudaMalloc; the model must already be on the
        device (any earlier simulate() uploads it)."""
        if tracked is None:
            tracked = list(range(self.n_species))
        tracked = [self.species_index(t) if isinstance(t, str) else int(t) for t in tracked]
        cfg, keep = self._cfg(t_final, n, seed, intervals, tracked, eps, variant, flags, rate_sets, t_final_sets, 0,
                              block_threads, stream)
        S = max(1, cfg.n_rate_sets)
        Pn, K = intervals + 1, len(tracked)
        times, mean, sd = np.zeros((S, Pn)), np.zeros((S, Pn, K)), np.zeros((S, Pn, K))
        res = F.Result()
        res.times, res.mean, res.stddev = _ptr(times, C.c_double), _ptr(mean, C.c_double), _ptr(sd, C.c_double)
        st = F.lib().tl_simulate_static(self._h, C.byref(cfg), C.byref(res))
        F.check(st, "tl_simulate_static")
        del keep
        return SimResult(times, mean, sd, None, res.leaps, res.ssa_steps, res.rejections, res.truncated,
                         res.kernel_ms, res.total_ms, res.variant_used, res.block_threads_used, res.grid_used,
                         res.launches, st)

    def sensitivity(self, t_final: float, n: int, seed: int = 1, tracked=None, eps: float = 0.03,
                    variant: int = F.VARIANT_AUTO, flags: int = 0, rate_sets=None, t_final_sets=None,
                    block_threads: int = 0, **extra) -> dict:
        tracked = [self.species_index(t) if isinstance(t, str) else int(t) for t in tracked]
        cfg, keep = self._cfg(t_final, n, seed, 1, tracked, eps, variant, flags, rate_sets, t_final_sets, 0,
                              block_threads, None, **extra)
        S, K, M = max(1, cfg.n_rate_sets), len(tracked), self.n_channels
        g = np.zeros((S, K, M))
        se = np.zeros((S, K, M))
        mf = np.zeros((S, K))
        gr = F.GradResult(_ptr(g, C.c_double), _ptr(se, C.c_double), _ptr(mf, C.c_double))
        res = F.Result()
        F.check(F.lib().tl_sensitivity(self._h, C.byref(cfg), C.byref(res), C.byref(gr)), "tl_sensitivity")
        del keep
        return {"grad": g, "stderr": se, "mean_final": mf, "leaps": res.leaps, "ssa_steps": res.ssa_steps,
                "kernel_ms": res.kernel_ms, "variant": res.variant_used}

    def eval_leap(self, x, eps: float = 0.03, flags: int = 0, n_critical: int = 5) -> dict:
        x = np.ascontiguousarray(np.atleast_2d(x), dtype=np.int64)
        n = x.shape[0]
        a = np.zeros((n, self.n_channels), np.float32)
        cr = np.zeros((n, self.n_channels), np.uint8)
        mu = np.zeros((n, self.n_species), np.float32)
        s2 = np.zeros((n, self.n_species), np.float32)
        tau = np.zeros(n, np.float32)
        a0 = np.zeros(n, np.float64)
        F.check(F.lib().tl_eval_leap(self._h, _ptr(x, C.c_int64), n, eps, flags, n_critical, _ptr(a, C.c_float),
                                     _ptr(cr, C.c_uint8), _ptr(mu, C.c_float), _ptr(s2, C.c_float),
                                     _ptr(tau, C.c_float), _ptr(a0, C.c_double)), "tl_eval_leap")
        return {"a": a, "crit": cr, "mu": mu, "sigma2": s2, "tau1": tau, "a0": a0}

    def replay(self, x0, k, raw: bool = False) -> np.ndarray:
        x0 = np.ascontiguousarray(x0, dtype=np.int64)
        k = np.ascontiguousarray(k, dtype=np.int32).reshape(-1, self.n_channels)
        out = np.zeros((k.shape[0], self.n_species), np.int64)
        F.check(F.lib().tl_replay(self._h, _ptr(x0, C.c_int64), _ptr(k, C.c_int32), k.shape[0], int(raw),
                                  _ptr(out, C.c_int64)), "tl_replay")
        return out


def philox(ctr, key) -> np.ndarray:
    ctr = np.ascontiguousarray(ctr, dtype=np.uint32).reshape(-1, 4)
    key = np.ascontiguousarray(key, dtype=np.uint32).reshape(-1, 2)
    out = np.zeros_like(ctr)
    F.check(F.lib().tl_philox(_ptr(ctr, C.c_uint32), _ptr(key, C.c_uint32), ctr.shape[0], _ptr(out, C.c_uint32)),
            "tl_philox")
    return out


def poisson(mean, seed: int = 1, step: int = 0, compat: bool = False) -> np.ndarray:
    mean = np.ascontiguousarray(mean, dtype=np.float32)
    out = np.zeros(len(mean), np.int32)
    F.check(F.lib().tl_poisson(_ptr(mean, C.c_float), len(mean), seed, step, int(compat), _ptr(out, C.c_int32)),
            "tl_poisson")
    return out


def simulate_batch(items: list[dict], stream=None) -> list[dict]:
    """One launch over several (model, configuration) items (tl_simulate_batch).

    Each item: dict(model=Model, t_final=..., n=..., seed=..., tracked=[...],
    intervals=1, rate_sets=None, t_final_sets=None, sensitivity=False,
    keep_samples=False, flags=0, eps=0.03, realization_offset=0).
    Returns per item a dict with mean / stddev / times (and grad, stderr,
    mean_final with sensitivity, samples with keep_samples) plus counters.
    """
    keep, arr = [], (F.BatchItem * len(items))()
    outs = []
    for k, it in enumerate(items):
        m: Model = it["model"]
        tracked = [m.species_index(t) if isinstance(t, str) else int(t) for t in it["tracked"]]
        intervals = int(it.get("intervals", 1))
        flags = int(it.get("flags", 0)) | (F.FLAG_KEEP_SAMPLES if it.get("keep_samples") else 0)
        cfg, kp = m._cfg(it["t_final"], it["n"], it.get("seed", 1), intervals, tracked, it.get("eps", 0.03), 0, flags,
                         it.get("rate_sets"), it.get("t_final_sets"), it.get("max_steps", 0), 0, None,
                         realization_offset=it.get("realization_offset", 0))
        S, Pn, K, M = max(1, cfg.n_rate_sets), intervals + 1, len(tracked), m.n_channels
        o = {"times": np.zeros((S, Pn)), "mean": np.zeros((S, Pn, K)), "stddev": np.zeros((S, Pn, K))}
        if it.get("keep_samples"):
            o["samples"] = np.zeros((S, it["n"], Pn, K), np.int64)
        res = F.Result()
        res.times, res.mean, res.stddev = _ptr(o["times"], C.c_double), _ptr(o["mean"], C.c_double), \
            _ptr(o["stddev"], C.c_double)
        res.samples = _ptr(o.get("samples"), C.c_int64)
        gr = None
        if it.get("sensitivity"):
            o["grad"], o["stderr"], o["mean_final"] = np.zeros((S, K, M)), np.zeros((S, K, M)), np.zeros((S, K))
            gr = F.GradResult(_ptr(o["grad"], C.c_double), _ptr(o["stderr"], C.c_double),
                              _ptr(o["mean_final"], C.c_double))
        arr[k].model = m._h
        arr[k].cfg = C.pointer(cfg)
        arr[k].result = C.pointer(res)
        arr[k].grad = C.pointer(gr) if gr is not None else None
        keep += [cfg, kp, res, gr]
        outs.append((o, res))
    F.check(F.lib().tl_simulate_batch(arr, len(items), stream), "tl_simulate_batch")
    out = []
    for o, res in outs:
        o.update(leaps=res.leaps, ssa_steps=res.ssa_steps, rejections=res.rejections, truncated=res.truncated,
                 kernel_ms=res.kernel_ms, variant=res.variant_used, grid=res.grid_used,
                 block_threads=res.block_threads_used)
        out.append(o)
    del keep
    return out
