"""Generate tests/golden/ref_functors.npz from the reference's own functors.

Run where the reference sources are present (they are compiled into
oracle/_ref/libtlref.so by oracle/build_ref.sh):

    python tests/golden/make_golden.py

For four seeded models (dimerisation decay, the 128x256 toy network, a
64-species cyclic chain, a 40-species colloidal aggregation) and random
population states it records, from the reference's code:
  * IsCriticalAndPropensity (functions.h:100-123): a (FP32) and criticality;
  * CSRMatrixPacked::CompTau (CSRMatrixPacked.cu:423-462): tau1 (FP32),
    on a matrix packed by the reference's constructor, with its species-index
    g lookup and n_c = 5;
  * FireReactionsFn (CSRMatrixPacked.cu:464-492) over every species row:
    the state after applying random firing counts;
  * pack() of every raw (species, channel, v) entry.
The fixture then pins the FP64 oracle (tests/test_oracle_cpu.py) and the
CUDA path (tests/test_gpu_parity.py) without the reference present.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

P = C.POINTER


def load_ref():
    from oracle import build
    build.build()
    so = ROOT / "oracle" / "_ref" / "libtlref.so"
    if not so.exists():
        raise SystemExit("reference functors not built (reference sources absent?)")
    L = C.CDLL(str(so))
    L.ref_propensity.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_float, P(C.c_float)]
    L.ref_propensity.restype = C.c_int
    L.ref_pack.argtypes = [C.c_int, C.c_int]
    L.ref_pack.restype = C.c_int
    L.ref_comp_tau.argtypes = [C.c_int, C.c_int, C.c_int, P(C.c_float), P(C.c_int), P(C.c_int), P(C.c_uint8),
                               P(C.c_int), P(C.c_int8), P(C.c_float), C.c_float]
    L.ref_comp_tau.restype = C.c_float
    L.ref_fire_rows.argtypes = [C.c_int, C.c_int, P(C.c_int), P(C.c_int), C.c_int, P(C.c_int), P(C.c_int)]
    L.ref_fire_as_shipped.argtypes = [C.c_int, C.c_int, C.c_int, P(C.c_float), P(C.c_int), P(C.c_int), P(C.c_int),
                                      P(C.c_int)]
    return L


def p(a, t):
    return a.ctypes.data_as(P(t))


MODELS = {
    "dimer": dict(family="dimer", kw={}),
    "toy": dict(family="toy", kw={}),
    "chain64": dict(family="chain", kw=dict(n_species=64)),
    "colloid40": dict(family="colloid", kw=dict(n_species=40)),
}


def model_arrays(name):
    from tau_leaping_gb300 import Model
    spec = MODELS[name]
    m = Model.generate(spec["family"], **spec["kw"])
    d = m.desc()
    t = m.tables()
    # the reference's order detector output (-1, 1, 2, 3)
    cp, ri, st = d["col_ptr"], d["row_ind"], d["stoich"]
    ref_order = np.full(m.n_channels, -1, np.int8)
    for j in range(m.n_channels):
        first = second = 0
        for q in range(cp[j], cp[j + 1]):
            v = int(st[q])
            if v >= 0:
                continue
            if first == 0:
                first = v
            else:
                second = v
        ref_order[j] = 3 if first == -2 else 2 if (first == -1 and second == -1) else 1 if first == -1 else -1
    return m, d, t, ref_order


def species_rows_raw(N, M, cp, ri, st):
    """Raw entries transposed to species rows (stable)."""
    rows = [[] for _ in range(N)]
    for j in range(M):
        for q in range(cp[j], cp[j + 1]):
            rows[ri[q]].append((j, int(st[q])))
    rp = np.zeros(N + 1, np.int32)
    cols, vals = [], []
    for i in range(N):
        rp[i + 1] = rp[i] + len(rows[i])
        for j, v in rows[i]:
            cols.append(j)
            vals.append(v)
    return rp, np.array(cols, np.int32), np.array(vals, np.float32)


def main():
    L = load_ref()
    rng = np.random.default_rng(2024)
    out = {}
    for name in MODELS:
        m, d, t, ref_order = model_arrays(name)
        N, M = m.n_species, m.n_channels
        x0 = d["x0"]
        n_states = 24
        scale = np.maximum(x0, 20)
        xs = (rng.random((n_states, N)) * 2 * scale).astype(np.int64)
        small = rng.random((n_states, N)) < 0.2
        xs[small] = rng.integers(0, 12, size=small.sum())
        xs[0] = x0
        xs = xs.astype(np.int32)
        order, s0, s1 = t["order"], t["s0"], t["s1"]
        rate = d["rate"].astype(np.float32)
        a = np.zeros((n_states, M), np.float32)
        crit = np.zeros((n_states, M), np.uint8)
        pr = C.c_float()
        for s in range(n_states):
            for j in range(M):
                typ = int(ref_order[j])
                crit[s, j] = L.ref_propensity(typ, int(xs[s, s0[j]]), int(xs[s, s1[j]]), 5, float(rate[j]),
                                              C.byref(pr))
                a[s, j] = pr.value
        rp, ci, vals = species_rows_raw(N, M, d["col_ptr"], d["row_ind"], d["stoich"])
        tau = np.zeros(n_states, np.float32)
        typ_arr = np.zeros(max(N, M), np.int8)
        typ_arr[:M] = ref_order
        for s in range(n_states):
            xr = np.ascontiguousarray(xs[s])
            ar = np.ascontiguousarray(a[s])
            cr = np.ascontiguousarray(crit[s])
            tau[s] = L.ref_comp_tau(N, M, len(ci), p(vals, C.c_float), p(rp, C.c_int), p(ci, C.c_int),
                                    p(cr, C.c_uint8), p(xr, C.c_int), p(typ_arr, C.c_int8), p(ar, C.c_float), 0.03)
        # packing of the raw entries
        packed = np.array([L.ref_pack(int(v), int(c)) for c, v in zip(ci, vals)], np.int32)
        # firing: 6 random count vectors applied one after another
        k = rng.integers(0, 40, size=(6, M)).astype(np.int32)
        x = (x0 + 100000).astype(np.int32)
        fired = np.zeros((6, N), np.int64)
        for l in range(6):
            L.ref_fire_rows(N, len(ci), p(packed, C.c_int), p(rp, C.c_int), M, p(np.ascontiguousarray(k[l]), C.c_int),
                            p(x, C.c_int))
            fired[l] = x
        if N == M:
            x2 = (x0 + 100000).astype(np.int32)
            L.ref_fire_as_shipped(N, M, len(ci), p(vals, C.c_float), p(rp, C.c_int), p(ci, C.c_int),
                                  p(np.ascontiguousarray(k[0]), C.c_int), p(x2, C.c_int))
            out[f"{name}/fired_as_shipped"] = x2.astype(np.int64)
        out.update({f"{name}/x": xs.astype(np.int64), f"{name}/a": a, f"{name}/crit": crit,
                    f"{name}/tau1": tau, f"{name}/csr_row_ptr": rp, f"{name}/csr_valcol": packed,
                    f"{name}/k": k, f"{name}/x_fire0": (x0 + 100000).astype(np.int64), f"{name}/fired": fired})
        print(name, "tau1[0] =", tau[0])
    dst = Path(__file__).resolve().parent / "ref_functors.npz"
    np.savez_compressed(dst, **out)
    print("wrote", dst, dst.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
