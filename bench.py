#!/usr/bin/env python3
"""Benchmark of the tau-leaping hot path on GB300.

One "step" = one whole ensemble simulation of the workload: R realizations
from x0 to t_final through tl_simulate (the fused persistent kernel plus the
statistics reduction), model constants already resident on the device.

Default workload (the one the reference's metric is quoted on, fits one
GPU): the 128-species / 256-channel random toy network, generator seed 7,
t_final 0.1, 100000 realizations, tracking S1 and S5, Philox seed 1.

Metric: realization-steps per second, counting every accepted tau-leap and
every direct-method (SSA) step of every realization; both are also reported
separately, with seconds per 1e4 realizations to t_final.

--impl reference times the CPU path (the FP64 oracle port of the
reference's algorithm, all host threads) on a bounded sample of the same
workload and prints the same line with "impl": "reference".

Multi-GPU (torchrun): realizations are sharded by realization id, each rank
runs its own R (weak scaling), no collective on the data path; rank 0 prints
the max-over-ranks timing.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "realization-leaps/sec"
UNIT = "realization-steps/s"

WORKLOADS = {
    # name: generator family, t_final, realizations, tracked species, pop bits
    "toy": dict(family="toy", t_final=0.1, R=100_000, tracked=[0, 4],
                desc="random toy network 128 species x 256 channels (seed 7), t_final 0.1, 1e5 realizations, "
                     "track S1,S5"),
    "dimer": dict(family="dimer", t_final=10.0, R=10_000, tracked=[0, 1],
                  desc="dimerisation decay S1=1e5, t_final 10, 1e4 realizations, track S1,S2"),
    "chain": dict(family="chain", t_final=1.0, R=65_536, tracked=[0, 1],
                  desc="cyclic chain 1024 species (seed 11), t_final 1, 65536 realizations"),
    "colloid": dict(family="colloid", t_final=0.01, R=4096, tracked=[0, 1],
                    desc="colloidal aggregation 250 species x 31250 channels (seed 13), t_final 0.01, "
                         "4096 realizations, int64"),
    "batch": dict(family="batch", t_final=None, R=None, tracked=[0, 1],
                  desc="one launch: dimer-decay 64 rate sets (c x lognormal(0,0.2), seed 17) x 4096 realizations, "
                       "t_final U[1,10]; toy network 16 rate sets x 1024 realizations, t_final U[0.05,0.1]; "
                       "likelihood-ratio sensitivities on"),
}


def batch_items(seed=1, scale=1.0):
    """The sensitivity + uneven-batch workload: dimer-decay (S1 = 1e5) with
    64 rate sets scaled by lognormal(0, 0.2) from seed 17, 4096 realizations
    each, t_final uniform in [1, 10]; the toy network with 16 sets, 1024
    realizations each, t_final uniform in [0.05, 0.1]."""
    from tau_leaping_gb300 import Model
    rng = np.random.default_rng(17)
    dim, toy = Model.generate("dimer"), Model.generate("toy")
    ds = dim.desc()["rate"][None, :] * rng.lognormal(0.0, 0.2, size=(64, 4))
    dt = rng.uniform(1.0, 10.0, size=64)
    ts = toy.desc()["rate"][None, :] * rng.lognormal(0.0, 0.2, size=(16, toy.n_channels))
    tt = rng.uniform(0.05, 0.1, size=16)
    n1, n2 = max(1, int(4096 * scale)), max(1, int(1024 * scale))
    return [dict(model=dim, t_final=10.0, n=n1, seed=seed, tracked=[0, 1], rate_sets=ds, t_final_sets=dt,
                 sensitivity=True),
            dict(model=toy, t_final=0.1, n=n2, seed=seed, tracked=[0, 4], rate_sets=ts, t_final_sets=tt,
                 sensitivity=True)], (dim, toy)


def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "src": "measured", "sm_max_mhz": d.get("sm_max_mhz", 2070.0)}
    return {"hbm_gbs": 6800.0, "src": "fallback", "sm_max_mhz": 2070.0}


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, device: int):
        self.dev = device
        self.proc = None
        self.path = Path(os.environ.get("TL_CLOCKS_CSV", f"/tmp/tl_clocks_{os.getpid()}.csv"))

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev),
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self) -> dict:
        try:
            rows = [r.split(",") for r in self.path.read_text().strip().splitlines() if r.strip()]
        except Exception:
            rows = []
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[0]))
                mx = max(mx, float(r[1]))
                for n, v in zip(names, r[4:8]):
                    if v.strip().lower() == "active":
                        reasons.add(n)
            except Exception:
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def model_bytes(m) -> tuple[int, int]:
    """(device constant bytes, population width) of a model, as uploaded."""
    N, M, nn, nr = m.n_species, m.n_channels, m.nnz_net, m.nnz_raw
    a16 = lambda b: (b + 15) // 16 * 16  # noqa: E731
    w = 8 if m.pop_bits == 64 else 4
    blob = (a16(16 * M) + a16(N) + a16(4 * N) + a16(4 * (N + 1)) + a16(4 * nn) + a16(4 * (M + 1)) + a16(4 * nn) +
            a16(4 * (N + 1)) + a16(4 * nr))
    return blob + N * w + 4 * M, w


def profile_traffic(workload: str):
    """DRAM bytes (read + write) per launch of the fused kernel on this
    workload, from the committed ncu summary (profiles/), or None."""
    p = ROOT / "profiles" / f"k_fused_{workload}.md"
    try:
        for line in p.read_text().splitlines():
            if line.startswith("dram_bytes_per_launch:"):
                return int(float(line.split(":", 1)[1]))
    except OSError:
        pass
    return None


def alg_bytes_per_step(m) -> int:
    """Algorithmic bytes one realization-step moves: the model stream (packed
    CSR, CSC, per-channel constants c/order/s0/s1, row pointers) plus the
    population read and write."""
    w = 8 if m.pop_bits == 64 else 4
    return 4 * m.nnz_net + 4 * m.nnz_net + 13 * m.n_channels + 4 * (m.n_species + 1) + 2 * w * m.n_species


def run_batch_workload(args, wl, rank, world, local_rank):
    """C5: sensitivity + uneven batching in one launch (tl_simulate_batch)."""
    import torch

    from tau_leaping_gb300 import _ffi
    from tau_leaping_gb300.model import simulate_batch
    torch.cuda.set_device(local_rank)
    _ffi.check(_ffi.lib().tl_set_device(local_rank), "tl_set_device")
    items, (dim, toy) = batch_items(args.seed, args.batch_scale)
    stream = torch.cuda.current_stream()
    sptr = C.c_void_p(stream.cuda_stream)
    for it in items:
        it["realization_offset"] = rank * it["n"]
    for _ in range(args.warmup):
        simulate_batch(items, stream=sptr)
    torch.cuda.synchronize()
    times, outs = [], []
    with Clocks(local_rank) as clk:
        for _ in range(args.steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            o = simulate_batch(items, stream=sptr)
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
            outs.append(o)
    tot = float(sum(times))
    steps = sum(it["leaps"] + it["ssa_steps"] for o in outs for it in o)
    o = outs[-1]
    line = {"metric": METRIC, "value": steps / (tot / 1e3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tot / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp32+int32", "data": "synthetic (seeded generator)",
            "config": {"workload": wl["desc"], "variant": "batched (lane units + warp units)",
                       "grid": o[0]["grid"], "block_threads": o[0]["block_threads"]},
            "leaps_per_step": float(sum(it["leaps"] for it in o)),
            "ssa_steps_per_step": float(sum(it["ssa_steps"] for it in o)),
            "gpu_launches": args.steps * (1 + 2 * len(items)),
            "kernel_ms": o[0]["kernel_ms"], "clocks": clk.summary()}
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_ours(args, wl, rank, world, local_rank):
    import torch

    from tau_leaping_gb300 import Model, _ffi
    from tau_leaping_gb300.model import _ptr

    if wl["family"] == "batch":
        return run_batch_workload(args, wl, rank, world, local_rank)
    torch.cuda.set_device(local_rank)
    _ffi.check(_ffi.lib().tl_set_device(local_rank), "tl_set_device")
    m = Model.generate(wl["family"])
    R, T, tracked = args.realizations or wl["R"], args.t_final or wl["t_final"], wl["tracked"]
    stream = torch.cuda.current_stream()
    sptr = C.c_void_p(stream.cuda_stream)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.int32, device="cuda")  # > 129 MB L2
    off = rank * R
    kw = dict(t_final=T, n=R, seed=args.seed, tracked=tracked, variant=args.variant, stream=sptr,
              realization_offset=off)

    def one():
        return m.simulate(**kw)

    for _ in range(args.warmup):
        one()
    torch.cuda.synchronize()
    times, kms, results = [], [], []
    dist = world > 1
    if dist:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with Clocks(local_rank) as clk:
        for _ in range(args.steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            r = one()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
            kms.append(r.kernel_ms)
            results.append(r)
        torch.cuda.synchronize()
        if dist:
            torch.distributed.barrier()
    tot_ms = float(sum(times))
    steps = [r.leaps + r.ssa_steps for r in results]
    if dist:
        t = torch.tensor([tot_ms], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        tot_ms = float(t.item())
        s = torch.tensor([float(sum(steps))], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(s)
        all_steps = float(s.item())
    else:
        all_steps = float(sum(steps))
    value = all_steps / (tot_ms / 1e3)
    r0 = results[-1]
    # dominant kernel: the fused persistent kernel, timed by the library's
    # CUDA events on the same stream
    k_ms = float(np.mean(kms))
    steps_per_launch = float(np.mean(steps))
    alg_per_launch = alg_bytes_per_step(m) * steps_per_launch
    # bytes that must cross HBM per launch: constants once, samples out
    cbytes, w = model_bytes(m)
    hbm_alg = cbytes + R * (1 + 1) * len(tracked) * w
    pk = peaks()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": tot_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32+int32", "data": "synthetic (seeded generator)",
        "config": {"workload": wl["desc"], "realizations_per_gpu": R, "t_final": T,
                   "n_species": m.n_species, "n_channels": m.n_channels, "variant": r0.variant,
                   "grid": r0.grid, "block_threads": r0.block_threads, "l2": "flushed between steps (256 MB write)",
                   "parallelism": f"realizations sharded over {world} GPU(s)"},
        "leaps_per_step": float(np.mean([r.leaps for r in results])),
        "ssa_steps_per_step": float(np.mean([r.ssa_steps for r in results])),
        "rejections_per_step": float(np.mean([r.rejections for r in results])),
        "sec_per_1e4_realizations": (tot_ms / args.steps / 1e3) * 1e4 / R,
        "gpu_launches": args.steps * (r0.launches + 1),
        "roofline": {"bound": "hbm", "achieved": alg_per_launch / (k_ms / 1e3) / 1e9, "peak": pk["hbm_gbs"],
                     "unit": "GB/s", "frac": alg_per_launch / (k_ms / 1e3) / 1e9 / pk["hbm_gbs"],
                     "traffic": profile_traffic(args.workload), "peak_src": pk["src"], "kernel": "k_fused",
                     "kernel_ms": k_ms, "alg_bytes_per_step": alg_bytes_per_step(m),
                     "steps_per_launch": steps_per_launch,
                     "hbm_required_gbs": hbm_alg / (k_ms / 1e3) / 1e9,
                     "note": "achieved = algorithmic bytes per realization-step (model tables + populations "
                             "read/written per leap) x steps per launch / launch time; the fused kernel serves "
                             "them from shared memory, so DRAM traffic (ncu) is only the tables once per CTA "
                             "plus the grid samples; the kernel is bound by instruction issue"},
    }
    # end to end through the C ABI with host buffers
    if rank == 0:
        line["e2e"] = e2e(args, wl, m, R, T, stream, sptr)
        line["clocks"] = clk.summary()
        if world == 1 and not args.no_plain:
            line["plain_form"] = plain_form(args, wl, m, R, T, tot_ms / args.steps, sptr)
        if world == 1 and not args.no_cpu:
            line["cpu_baseline"] = cpu_baseline(args, wl, m, R, check_gpu=True)
        print(json.dumps(line), flush=True)


def plain_form(args, wl, m, R, T, fused_ms, sptr, budget_s: float = 8.0):
    """The plain form (FP32 time, one realization per thread, one launch per
    leap) beside the fused kernel, both on the same sample: all R
    realizations to a t_final shortened, where needed, so that the plain run
    takes about budget_s (its cost is estimated at 40x the fused run's)."""
    from tau_leaping_gb300 import _ffi
    frac = min(1.0, budget_s * 1e3 / max(40.0 * fused_ms, 1e-3))
    Ts = T * frac
    kw = dict(t_final=Ts, n=R, seed=args.seed, tracked=wl["tracked"], stream=sptr,
              realization_offset=0)
    out = {}
    for name, var in (("plain", _ffi.VARIANT_PLAIN), ("fused", args.variant)):
        m.simulate(**{**kw, "t_final": Ts * 0.1}, variant=var)
        r = m.simulate(**kw, variant=var)
        out[name] = dict(value=(r.leaps + r.ssa_steps) / (r.total_ms / 1e3), ms=r.total_ms,
                         launches=r.launches, leaps=r.leaps, ssa_steps=r.ssa_steps)
    return {"value": out["plain"]["value"], "unit": UNIT, "fused_value": out["fused"]["value"],
            "speedup": out["fused"]["value"] / out["plain"]["value"],
            "plain_ms": out["plain"]["ms"], "fused_ms": out["fused"]["ms"],
            "plain_launches": out["plain"]["launches"], "sample": f"{R} realizations to t_final {Ts:.4g}",
            "note": "host wall time of each tl_simulate call (kernels + statistics), same sample"}


def e2e(args, wl, m, R, T, stream, sptr):
    """Same metric through tl_model_create + tl_simulate from host arrays:
    every step uploads the model, runs, and reads the statistics back."""
    import torch

    from tau_leaping_gb300 import Model
    d = m.desc()
    tr = wl["tracked"]
    h2d = model_bytes(m)[0] + 8 * len(tr) + 8
    d2h = 2 * 2 * len(tr) * 8 + 64
    tot, steps = 0.0, 0
    n = 1  # the path is warm from the timed loop; model creation + upload are part of every call
    for i in range(n):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        mm = Model.from_arrays(d["x0"], d["rate"], d["col_ptr"], d["row_ind"], d["stoich"], pop_bits=m.pop_bits)
        r = mm.simulate(T, R, seed=args.seed, tracked=tr, variant=args.variant, stream=sptr)
        mm.close()
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        tot += dt
        steps += r.leaps + r.ssa_steps
    return {"value": steps / tot, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "steps": n, "timing": "host wall clock around model upload + tl_simulate + statistics read-back"}


def cpu_baseline(args, wl, m, R, budget_s: float = 12.0, check_gpu: bool = False):
    """FP64 oracle port of the reference's algorithm on the host cores, on a
    bounded sample (the first realizations of the same ensemble).  With
    check_gpu the same realizations also run on the GPU for fp64_check."""
    from oracle import py as ora
    o = ora.OracleModel.from_desc(m.desc())
    cores = os.cpu_count() or 1
    n = cores
    t0 = time.perf_counter()
    r = o.simulate(wl["t_final"], R, seed=args.seed, tracked=wl["tracked"], threads=cores, r_begin=0, r_end=n)
    dt = time.perf_counter() - t0
    done, steps = n, r["leaps"] + r["ssa_steps"]
    finals = [r["samples"][0, :, -1, :]]
    while dt < budget_s and done < R:
        k = min(R - done, max(cores, int(done * (budget_s - dt) / max(dt, 1e-3) * 0.8)))
        t1 = time.perf_counter()
        r = o.simulate(wl["t_final"], R, seed=args.seed, tracked=wl["tracked"], threads=cores, r_begin=done,
                       r_end=done + k)
        dt += time.perf_counter() - t1
        done += k
        steps += r["leaps"] + r["ssa_steps"]
        finals.append(r["samples"][0, :, -1, :])
    out = {"value": steps / dt, "unit": UNIT, "cores": cores, "kind": "port",
           "sample": f"{done} of {R} realizations of the same workload, FP64 oracle, {cores} threads, {dt:.1f} s"}
    if check_gpu:
        out["fp64_check"] = fp64_check(args, wl, m, done, np.concatenate(finals).astype(np.float64))
    return out


def fp64_check(args, wl, m, n, ora_final):
    """Error of the engine against the FP64 oracle on the baseline's sample:
    the same n realizations (same ids, so the same Philox streams) run on
    the GPU with their samples kept.  Reports, per tracked species, the
    relative difference of the ensemble mean and variance at t_final and the
    share of realizations whose final state is identical."""
    g = m.simulate(wl["t_final"], n, seed=args.seed, tracked=wl["tracked"], keep_samples=True,
                   variant=args.variant)
    gf = g.samples[0, :, -1, :].astype(np.float64)
    rel_mean = np.abs(gf.mean(0) - ora_final.mean(0)) / np.maximum(np.abs(ora_final.mean(0)), 1e-300)
    var_o = ora_final.var(0, ddof=1) if n > 1 else np.zeros(gf.shape[1])
    var_g = gf.var(0, ddof=1) if n > 1 else np.zeros(gf.shape[1])
    rel_var = np.abs(var_g - var_o) / np.maximum(var_o, 1e-300)
    # one standard error of each difference, were the two samples independent
    se_mean = np.sqrt((var_g + var_o) / max(n, 1)) / np.maximum(np.abs(ora_final.mean(0)), 1e-300)
    se_var = np.sqrt(4.0 / max(n - 1, 1)) * np.ones_like(rel_var)
    return {"realizations": int(n), "tracked": wl["tracked"],
            "mean_rel_err": [float(x) for x in rel_mean], "mean_rel_se": [float(x) for x in se_mean],
            "var_rel_err": [float(x) for x in rel_var], "var_rel_se": [float(x) for x in se_var],
            "identical_final_state": float(np.mean(np.all(gf == ora_final, axis=1)))}


def run_reference(args, wl, rank):
    if rank != 0:
        return
    from tau_leaping_gb300 import Model
    m = Model.generate(wl["family"])
    R = args.realizations or wl["R"]
    for _ in range(args.warmup):
        cpu_baseline(args, wl, m, R, budget_s=2.0)
    vals, t_all = [], 0.0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        cb = cpu_baseline(args, wl, m, R, budget_s=8.0)
        t_all += time.perf_counter() - t0
        vals.append(cb["value"])
    v = float(np.mean(vals))
    cb["value"] = v
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t_all / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp64+int64", "data": "synthetic (seeded generator)",
            "config": {"workload": wl["desc"], "realizations_per_gpu": R, "t_final": wl["t_final"]},
            "impl": "reference", "cpu_baseline": cb,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="toy", choices=list(WORKLOADS))
    ap.add_argument("--realizations", type=int, default=0)
    ap.add_argument("--variant", type=int, default=0)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain-form comparison")
    ap.add_argument("--batch-scale", type=float, default=1.0)
    ap.add_argument("--t-final", type=float, default=0.0, help="override t_final (profiling captures)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    wl = WORKLOADS[args.workload]
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    import __graft_entry__
    __graft_entry__.build()
    if args.impl == "reference":
        run_reference(args, wl, rank)
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl", device_id=torch.device(f"cuda:{local_rank}"))
    try:
        run_ours(args, wl, rank, world, local_rank)
    finally:
        if world > 1:
            import torch
            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
