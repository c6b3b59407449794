"""ctypes binding of the oracle (liboracle.so).  Test infrastructure only:
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it as
the checker; the engine never does.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
_lib = None

P = C.POINTER


class OraCfg(C.Structure):
    _fields_ = [("t_final", C.c_double), ("eps", C.c_double), ("R", C.c_int64), ("seed", C.c_uint64),
                ("n_int", C.c_int32), ("K", C.c_int32), ("tracked", P(C.c_int32)), ("S", C.c_int32),
                ("rate_sets", P(C.c_double)), ("t_final_sets", P(C.c_double)), ("flags", C.c_uint32),
                ("nc", C.c_int32), ("ssa_factor", C.c_int32), ("ssa_block", C.c_int32),
                ("max_steps", C.c_int64), ("method", C.c_int32), ("threads", C.c_int32),
                ("r_begin", C.c_int64), ("r_end", C.c_int64), ("sens", C.c_int32)]


def lib():
    global _lib
    if _lib is None:
        path = _HERE / "liboracle.so"
        if not path.exists():
            from . import build
            build.build()
        L = C.CDLL(str(path))
        L.ora_model_new.restype = C.c_void_p
        L.ora_model_new.argtypes = [C.c_int, C.c_int, P(C.c_int64), P(C.c_double), P(C.c_int32), P(C.c_int32),
                                    P(C.c_int8)]
        L.ora_model_free.argtypes = [C.c_void_p]
        L.ora_eval.argtypes = [C.c_void_p, P(C.c_int64), C.c_int, C.c_double, C.c_uint32, C.c_int, P(C.c_double),
                               P(C.c_uint8), P(C.c_double), P(C.c_double), P(C.c_double), P(C.c_double)]
        L.ora_replay.argtypes = [C.c_void_p, P(C.c_int64), P(C.c_int32), C.c_int, C.c_int, P(C.c_int64)]
        L.ora_philox.argtypes = [P(C.c_uint32), P(C.c_uint32), C.c_int, P(C.c_uint32)]
        L.ora_poisson.argtypes = [P(C.c_double), C.c_int, C.c_uint64, C.c_uint32, C.c_int, P(C.c_int64)]
        L.ora_simulate.argtypes = [C.c_void_p, P(OraCfg), P(C.c_int64), P(C.c_double), P(C.c_int64)]
        L.ora_gen_new.restype = C.c_void_p
        L.ora_gen_new.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int64, C.c_int64, C.c_double, C.c_double,
                                  C.c_double, C.c_double, C.c_uint64]
        L.ora_gen_sizes.argtypes = [C.c_void_p, P(C.c_int), P(C.c_int), P(C.c_int)]
        L.ora_gen_copy.argtypes = [C.c_void_p, P(C.c_int64), P(C.c_double), P(C.c_int32), P(C.c_int32),
                                   P(C.c_int8)]
        L.ora_gen_free.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def _p(a, t):
    return None if a is None else a.ctypes.data_as(P(t))


class OracleModel:
    def __init__(self, x0, rate, col_ptr, row_ind, stoich):
        self.x0 = np.ascontiguousarray(x0, np.int64)
        self.rate = np.ascontiguousarray(rate, np.float64)
        self.col_ptr = np.ascontiguousarray(col_ptr, np.int32)
        self.row_ind = np.ascontiguousarray(row_ind, np.int32)
        self.stoich = np.ascontiguousarray(stoich, np.int8)
        self.N, self.M = len(self.x0), len(self.rate)
        self._h = lib().ora_model_new(self.N, self.M, _p(self.x0, C.c_int64), _p(self.rate, C.c_double),
                                      _p(self.col_ptr, C.c_int32), _p(self.row_ind, C.c_int32),
                                      _p(self.stoich, C.c_int8))

    @classmethod
    def from_desc(cls, d: dict) -> "OracleModel":
        return cls(d["x0"], d["rate"], d["col_ptr"], d["row_ind"], d["stoich"])

    def __del__(self):
        try:
            lib().ora_model_free(self._h)
        except Exception:
            pass

    def eval(self, x, eps=0.03, flags=0, nc=5) -> dict:
        x = np.ascontiguousarray(np.atleast_2d(x), np.int64)
        n = x.shape[0]
        out = {"a": np.zeros((n, self.M)), "crit": np.zeros((n, self.M), np.uint8), "mu": np.zeros((n, self.N)),
               "sigma2": np.zeros((n, self.N)), "tau1": np.zeros(n), "a0": np.zeros(n)}
        lib().ora_eval(self._h, _p(x, C.c_int64), n, eps, flags, nc, _p(out["a"], C.c_double),
                       _p(out["crit"], C.c_uint8), _p(out["mu"], C.c_double), _p(out["sigma2"], C.c_double),
                       _p(out["tau1"], C.c_double), _p(out["a0"], C.c_double))
        return out

    def replay(self, x0, k, raw=False) -> np.ndarray:
        x0 = np.ascontiguousarray(x0, np.int64)
        k = np.ascontiguousarray(k, np.int32).reshape(-1, self.M)
        out = np.zeros((k.shape[0], self.N), np.int64)
        lib().ora_replay(self._h, _p(x0, C.c_int64), _p(k, C.c_int32), k.shape[0], int(raw), _p(out, C.c_int64))
        return out

    def simulate(self, t_final, R, seed=1, intervals=1, tracked=None, eps=0.03, flags=0, method=0, threads=1,
                 r_begin=0, r_end=0, rate_sets=None, t_final_sets=None, max_steps=0, sens=False) -> dict:
        tracked = np.ascontiguousarray(tracked if tracked is not None else range(self.N), np.int32)
        cfg = OraCfg()
        cfg.t_final, cfg.eps, cfg.R, cfg.seed = t_final, eps, R, seed
        cfg.n_int, cfg.K, cfg.tracked = intervals, len(tracked), _p(tracked, C.c_int32)
        keep = [tracked]
        S = 1
        if rate_sets is not None:
            rs = np.ascontiguousarray(rate_sets, np.float64).reshape(-1, self.M)
            S = rs.shape[0]
            cfg.rate_sets = _p(rs, C.c_double)
            keep.append(rs)
            if t_final_sets is not None:
                tf = np.ascontiguousarray(t_final_sets, np.float64)
                cfg.t_final_sets = _p(tf, C.c_double)
                keep.append(tf)
        cfg.S, cfg.flags, cfg.method, cfg.threads = S, flags, method, threads
        cfg.max_steps = max_steps
        cfg.r_begin, cfg.r_end = r_begin, (r_end if r_end else R)
        Rn = cfg.r_end - cfg.r_begin
        samples = np.zeros((S, Rn, intervals + 1, len(tracked)), np.int64)
        scores = np.zeros((S, Rn, self.M)) if sens else None
        cnt = np.zeros(4, np.int64)
        lib().ora_simulate(self._h, C.byref(cfg), _p(samples, C.c_int64), _p(scores, C.c_double),
                           _p(cnt, C.c_int64))
        del keep
        return {"samples": samples, "scores": scores, "leaps": int(cnt[0]), "ssa_steps": int(cnt[1]),
                "rejections": int(cnt[2]), "truncated": int(cnt[3])}


# The benchmark configurations' generator parameters per family (the same
# defaults as the engine's tl_gen_params_init).
GEN_FAMILIES = {"dimer": 1, "toy": 2, "chain": 3, "colloid": 4}
GEN_DEFAULTS = {
    "dimer": dict(n_species=3, n_channels=4, x0_min=100000, x0_max=100000, seed=1),
    "toy": dict(n_species=128, n_channels=256, x0_min=0, x0_max=10000, rate_min=1e-3, rate_max=1.0, seed=7),
    "chain": dict(n_species=1024, n_channels=1024, x0_min=1000, x0_max=2000, rate_min=1.0, rate_max=1.0, seed=11),
    "colloid": dict(n_species=250, n_channels=31250, x0_min=1000, x0_max=2000, rate_assoc=1e-4, rate_dissoc=0.1,
                    seed=13),
}


def generate(family: str, **kw) -> dict:
    """Model description {x0, rate, col_ptr, row_ind, stoich} of a seeded
    family, built by the oracle alone (no engine library)."""
    g = dict(n_species=0, n_channels=0, x0_min=0, x0_max=0, rate_min=0.0, rate_max=0.0, rate_assoc=0.0,
             rate_dissoc=0.0, seed=0)
    g.update(GEN_DEFAULTS[family])
    g.update(kw)
    L = lib()
    h = L.ora_gen_new(GEN_FAMILIES[family], g["n_species"], g["n_channels"], g["x0_min"], g["x0_max"],
                      g["rate_min"], g["rate_max"], g["rate_assoc"], g["rate_dissoc"], g["seed"])
    if not h:
        raise ValueError(f"oracle generator rejected {family} {kw}")
    try:
        n, m, z = C.c_int(), C.c_int(), C.c_int()
        L.ora_gen_sizes(h, C.byref(n), C.byref(m), C.byref(z))
        d = {"x0": np.zeros(n.value, np.int64), "rate": np.zeros(m.value), "col_ptr": np.zeros(m.value + 1, np.int32),
             "row_ind": np.zeros(z.value, np.int32), "stoich": np.zeros(z.value, np.int8)}
        L.ora_gen_copy(h, _p(d["x0"], C.c_int64), _p(d["rate"], C.c_double), _p(d["col_ptr"], C.c_int32),
                       _p(d["row_ind"], C.c_int32), _p(d["stoich"], C.c_int8))
    finally:
        L.ora_gen_free(h)
    return d


def philox(ctr, key) -> np.ndarray:
    ctr = np.ascontiguousarray(ctr, np.uint32).reshape(-1, 4)
    key = np.ascontiguousarray(key, np.uint32).reshape(-1, 2)
    out = np.zeros_like(ctr)
    lib().ora_philox(_p(ctr, C.c_uint32), _p(key, C.c_uint32), ctr.shape[0], _p(out, C.c_uint32))
    return out


def poisson(mean, seed=1, step=0, compat=False) -> np.ndarray:
    mean = np.ascontiguousarray(mean, np.float64)
    out = np.zeros(len(mean), np.int64)
    lib().ora_poisson(_p(mean, C.c_double), len(mean), seed, step, int(compat), _p(out, C.c_int64))
    return out


def chain_exact_moments(x0, c: float, t: float):
    """Exact mean and variance of the cyclic chain S_i -> S_(i+1 mod N), rate c
    (closed, first order: every molecule walks the ring independently and
    jumps at rate c).  A molecule starting at i is at j at time t with
    probability q[(j - i) mod N], q[d] = sum_k P(Poisson(c t) = N k + d), so
    the count at j is a sum of binomials:
        mean_j = sum_i x0_i q[j-i],  var_j = sum_i x0_i q[j-i] (1 - q[j-i]).
    FP64, the exact solution of the chemical master equation."""
    from scipy import stats
    x0 = np.asarray(x0, np.float64)
    N = len(x0)
    lam = c * t
    kmax = int(lam + 40 * np.sqrt(lam) + 60)
    pk = stats.poisson.pmf(np.arange(kmax + 1), lam)
    q = np.zeros(N)
    np.add.at(q, np.arange(kmax + 1) % N, pk)
    mean = np.zeros(N)
    var = np.zeros(N)
    for d in range(N):
        if q[d] == 0.0:
            continue
        src = np.roll(x0, d)  # src[j] = x0[(j - d) mod N]
        mean += src * q[d]
        var += src * q[d] * (1.0 - q[d])
    return mean, var
