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
workload and prints the same line with "impl": "reference".  That arm builds
its model with the oracle's own generator and never loads the engine.

Multi-GPU (torchrun): realizations are sharded by realization id, each rank
runs its own R (weak scaling), no collective on the data path; rank 0 prints
the max-over-ranks timing.
"""
from __future__ import annotations

import argparse
import ctypes as C
import hashlib
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
    # name: generator family, t_final, realizations, tracked species, sizes
    "toy": dict(family="toy", t_final=0.1, R=100_000, tracked=[0, 4], n_species=128, n_channels=256, pop_bits=32,
                desc="random toy network 128 species x 256 channels (seed 7), t_final 0.1, 1e5 realizations, "
                     "track S1,S5"),
    # 1e4 realizations are two warps per SM: one realization's chain of
    # dependent steps sets the time, not the issue rate
    "dimer": dict(family="dimer", t_final=10.0, R=10_000, tracked=[0, 1], n_species=3, n_channels=4, pop_bits=32,
                  bound="latency", desc="dimerisation decay S1=1e5, t_final 10, 1e4 realizations, track S1,S2"),
    "chain": dict(family="chain", t_final=1.0, R=65_536, tracked=[0, 1], n_species=1024, n_channels=1024,
                  pop_bits=32, desc="cyclic chain 1024 species (seed 11), t_final 1, 65536 realizations"),
    "colloid": dict(family="colloid", t_final=0.01, R=4096, tracked=[0, 1], n_species=250, n_channels=31250,
                    pop_bits=64, desc="colloidal aggregation 250 species x 31250 channels (seed 13), t_final 0.01, "
                                      "4096 realizations, int64"),
    "batch": dict(family="batch", t_final=None, R=None, tracked=[0, 1], n_species=None, n_channels=None, pop_bits=32,
                  desc="one launch: dimer-decay 64 rate sets (c x lognormal(0,0.2), seed 17) x 4096 realizations, "
                       "t_final U[1,10]; toy network 16 rate sets x 1024 realizations, t_final U[0.05,0.1]; "
                       "likelihood-ratio sensitivities on"),
}

BOUND_TEXT = {"issue": "instruction issue", "latency": "the latency of one realization's dependent steps"}


# Element operations of one realization-step (the issue-roof figure): per
# channel a propensity and a Poisson draw, per stored entry the mu and
# sigma^2 FMAs and the integer update.
def ops_per_step(N: int, M: int, nnz: int) -> int:
    return 2 * M + 3 * nnz


def dtype_of(wl) -> str:
    return "fp32+int64" if wl["pop_bits"] == 64 else "fp32+int32"


def workload_config(wl, R, T, world) -> dict:
    """The config both arms report (identical for the same workload)."""
    return {"workload": wl["desc"], "realizations_per_gpu": R, "t_final": T, "n_species": wl["n_species"],
            "n_channels": wl["n_channels"], "population": "int64" if wl["pop_bits"] == 64 else "int32",
            "parallelism": f"realizations sharded over {world} process(es)"}


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
    blob = (a16(8 * M) + a16(M) + a16(N) + a16(4 * N) + a16(4 * (N + 1)) + a16(4 * nn) + a16(4 * (M + 1)) +
            a16(4 * nn) + a16(4 * (N + 1)) + a16(4 * nr))
    return blob + N * w + 4 * M, w


def kernel_source_hash() -> str:
    """sha256 of everything that determines the fused kernel's machine code:
    the CUDA sources, the C ABI header and the nvcc flags."""
    from tau_leaping_gb300 import build as b
    h = hashlib.sha256()
    for p in sorted(b.CSRC.glob("*")) + sorted(b.INC.glob("*.h")):
        h.update(p.name.encode())
        h.update(p.read_bytes())
    h.update(" ".join(f for f in b.NVFLAGS if not f.startswith("/")).encode())  # no machine paths
    return h.hexdigest()


def ncu_record(kernel_tag: str):
    """The ncu figures of the fused kernel on this workload (DRAM bytes per
    launch, issue-slot utilisation), from the record kept beside the
    profile summaries, used only if it was captured from this very kernel
    build (same source hash); otherwise None and the reason."""
    p = ROOT / "profiles" / f"{kernel_tag}.ncu.json"
    try:
        rec = json.loads(p.read_text())
    except (OSError, ValueError):
        return None, "no ncu record for this workload"
    if rec.get("source_sha256") != kernel_source_hash():
        return None, "ncu record is from another kernel build"
    return rec, "ncu capture of this kernel build"


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
            "vs_baseline": None, "dtype": dtype_of(wl), "data": "synthetic (seeded generator)",
            "config": {"workload": wl["desc"], "parallelism": f"realizations sharded over {world} process(es)"},
            "launch": {"variant": "batched (lane units + warp units)", "grid": o[0]["grid"],
                       "block_threads": o[0]["block_threads"]},
            "leaps_per_step": float(sum(it["leaps"] for it in o)),
            "ssa_steps_per_step": float(sum(it["ssa_steps"] for it in o)),
            "gpu_launches": args.steps * (1 + 2 * len(items)),
            "kernel_ms": o[0]["kernel_ms"], "clocks": clk.summary()}
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_ours(args, wl, rank, world, local_rank):
    import torch

    from tau_leaping_gb300 import Model, _ffi

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
    stream_gbs = alg_per_launch / (k_ms / 1e3) / 1e9
    # bytes that must cross HBM per launch: constants once, samples out
    cbytes, w = model_bytes(m)
    hbm_alg = cbytes + R * (1 + 1) * len(tracked) * w
    pk = peaks()
    ops = ops_per_step(m.n_species, m.n_channels, m.nnz_net)
    rec, rec_src = ncu_record(f"k_fused_{args.workload}") if args.variant == 0 and not args.t_final and \
        not args.realizations else (None, "ncu record covers the default launch only")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": tot_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": dtype_of(wl), "data": "synthetic (seeded generator)",
        "config": workload_config(wl, R, T, world),
        "timing": "CUDA events on the library's stream around each tl_simulate call; L2 flushed between steps "
                  "(256 MB write)",
        "launch": {"variant": r0.variant, "grid": r0.grid, "block_threads": r0.block_threads},
        "leaps_per_step": float(np.mean([r.leaps for r in results])),
        "ssa_steps_per_step": float(np.mean([r.ssa_steps for r in results])),
        "rejections_per_step": float(np.mean([r.rejections for r in results])),
        "sec_per_1e4_realizations": (tot_ms / args.steps / 1e3) * 1e4 / R,
        "gpu_launches": args.steps * (r0.launches + 1),
        "roofline": {
            "bound": wl.get("bound", "issue"), "achieved": stream_gbs, "peak": pk["hbm_gbs"], "unit": "GB/s",
            "frac": stream_gbs / pk["hbm_gbs"],
            "traffic": rec["dram_bytes_per_launch"] if rec else None,
            "issue_slots_busy": rec["issue_slots_busy_pct"] / 100.0 if rec else None,
            "l2_traffic": rec.get("lts_bytes_per_launch") if rec else None,
            "ncu_source": rec_src, "ncu_case": rec.get("case") if rec else None,
            "peak_src": pk["src"], "kernel": "k_fused", "kernel_ms": k_ms,
            "alg_bytes_per_step": alg_bytes_per_step(m), "steps_per_launch": steps_per_launch,
            "ops_per_step": ops, "ops_per_s": ops * steps_per_launch / (k_ms / 1e3),
            "hbm_required_gbs": hbm_alg / (k_ms / 1e3) / 1e9,
            "note": f"the fused kernel is bound by {BOUND_TEXT[wl.get('bound', 'issue')]} (issue_slots_busy, "
                    "from ncu on this kernel build); achieved is the algorithmic stream of a realization-step "
                    "(model tables + populations read and written, B_alg) x steps per launch / launch time, "
                    "served from shared memory, L1 and L2 (l2_traffic, where captured), against the HBM copy "
                    "peak as a yardstick; DRAM carries only the tables once per CTA, the grid samples and "
                    "local-memory lines (traffic)"},
    }
    # end to end through the C ABI with host buffers
    if rank == 0:
        line["e2e"] = e2e(args, wl, m, R, T, sptr)
        line["clocks"] = clk.summary()
        if world == 1 and not args.no_plain:
            line["plain_form"] = plain_form(args, wl, m, R, T, tot_ms / args.steps, sptr)
            if args.workload != "colloid":
                line["workloads"] = {"colloid": colloid_target(args, sptr)}
        if world == 1 and not args.no_cpu:
            from oracle import py as ora
            o = ora.OracleModel.from_desc(m.desc())
            line["cpu_baseline"] = cpu_baseline(o, wl, R, T, args.seed)
            line["cpu_baseline"]["fp64_check"] = fp64_check(args, wl, m, line["cpu_baseline"].pop("_finals"))
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


def colloid_target(args, sptr, reps: int = 2):
    """The 250-species colloidal aggregation configuration in full (31250
    channels, int64, 4096 realizations to t_final 0.01): the fused
    persistent kernel against the plain form (one realization per thread,
    one launch per step; the faster of its per-launch and graph-replayed
    loops), each the mean of `reps` calls after one warm-up, timed by the
    host around the whole call (kernels + statistics)."""
    from tau_leaping_gb300 import Model, _ffi
    m = Model.generate("colloid")
    kw = dict(t_final=0.01, n=4096, seed=args.seed, tracked=[0, 1], stream=sptr)
    out = {}
    for name, var, fl in (("fused", 0, 0), ("plain", _ffi.VARIANT_PLAIN, 0),
                          ("plain_graph", _ffi.VARIANT_PLAIN, _ffi.FLAG_GRAPH)):
        m.simulate(**kw, variant=var, flags=fl)
        rs = [m.simulate(**kw, variant=var, flags=fl) for _ in range(reps)]
        st = sum(r.leaps + r.ssa_steps for r in rs)
        ms = sum(r.total_ms for r in rs)
        out[name] = {"value": st / (ms / 1e3), "ms_per_call": ms / reps, "launches": rs[-1].launches,
                     "variant": rs[-1].variant}
    plain = max(out["plain"]["value"], out["plain_graph"]["value"])
    return {"workload": WORKLOADS["colloid"]["desc"], "unit": UNIT, "fused": out["fused"],
            "plain": out["plain"], "plain_graph": out["plain_graph"], "speedup_vs_plain": out["fused"]["value"] / plain,
            "target": ">= 5x the plain form (FP32, one realization per thread, one launch per step)"}


def e2e(args, wl, m, R, T, sptr, n: int = 3):
    """Same metric through tl_model_create + tl_simulate from host arrays:
    every sample uploads the model, runs, and reads the statistics back;
    the mean over n samples."""
    import torch

    from tau_leaping_gb300 import Model
    d = m.desc()
    tr = wl["tracked"]
    h2d = model_bytes(m)[0] + 8 * len(tr) + 8
    d2h = 2 * 2 * len(tr) * 8 + 64
    tot, steps, per = 0.0, 0, []
    for _ in range(n):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        mm = Model.from_arrays(d["x0"], d["rate"], d["col_ptr"], d["row_ind"], d["stoich"], pop_bits=m.pop_bits)
        r = mm.simulate(T, R, seed=args.seed, tracked=tr, variant=args.variant, stream=sptr)
        mm.close()
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        tot += dt
        steps += r.leaps + r.ssa_steps
        per.append((r.leaps + r.ssa_steps) / dt)
    return {"value": steps / tot, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "steps": n, "samples": per,
            "timing": "host wall clock around model upload + tl_simulate + statistics read-back, per sample"}


def cpu_baseline(o, wl, R, T, seed, budget_s: float = 12.0):
    """FP64 oracle port of the reference's algorithm on the host cores, on a
    bounded sample (the first realizations of the same ensemble)."""
    cores = os.cpu_count() or 1
    n = cores
    t0 = time.perf_counter()
    r = o.simulate(T, R, seed=seed, tracked=wl["tracked"], threads=cores, r_begin=0, r_end=n)
    dt = time.perf_counter() - t0
    done, steps = n, r["leaps"] + r["ssa_steps"]
    finals = [r["samples"][0, :, -1, :]]
    while dt < budget_s and done < R:
        k = min(R - done, max(cores, int(done * (budget_s - dt) / max(dt, 1e-3) * 0.8)))
        t1 = time.perf_counter()
        r = o.simulate(T, R, seed=seed, tracked=wl["tracked"], threads=cores, r_begin=done, r_end=done + k)
        dt += time.perf_counter() - t1
        done += k
        steps += r["leaps"] + r["ssa_steps"]
        finals.append(r["samples"][0, :, -1, :])
    return {"value": steps / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{done} of {R} realizations of the same workload, FP64 oracle, {cores} threads, {dt:.1f} s",
            "_finals": np.concatenate(finals).astype(np.float64)}


def fp64_check(args, wl, m, ora_final):
    """Error of the engine against the FP64 oracle on the baseline's sample:
    the same n realizations (same ids, so the same Philox streams) run on
    the GPU with their samples kept.  Reports, per tracked species, the
    relative difference of the ensemble mean and variance at t_final and the
    share of realizations whose final state is identical."""
    n = len(ora_final)
    g = m.simulate(wl["t_final"], n, seed=args.seed, tracked=wl["tracked"], keep_samples=True,
                   variant=args.variant)
    gf = g.samples[0, :, -1, :].astype(np.float64)
    rel_mean = np.abs(gf.mean(0) - ora_final.mean(0)) / np.maximum(np.abs(ora_final.mean(0)), 1e-300)
    var_o = ora_final.var(0, ddof=1) if n > 1 else np.zeros(gf.shape[1])
    var_g = gf.var(0, ddof=1) if n > 1 else np.zeros(gf.shape[1])
    rel_var = np.abs(var_g - var_o) / np.maximum(var_o, 1e-300)
    return {"realizations": int(n), "tracked": wl["tracked"], "paired": "same realization ids and streams",
            "mean_rel_err": [float(x) for x in rel_mean], "var_rel_err": [float(x) for x in rel_var],
            "identical_final_state": float(np.mean(np.all(gf == ora_final, axis=1)))}


def run_reference(args, wl, rank):
    """The reference arm: the FP64 oracle port on all host cores, model built
    by the oracle's own generator (the engine library is never loaded)."""
    if rank != 0:
        return
    if wl["family"] == "batch":
        print(json.dumps({"impl": "reference", "unavailable": "the batched sensitivity workload has no CPU "
                                                             "counterpart in the reference"}), flush=True)
        return
    from oracle import py as ora
    o = ora.OracleModel.from_desc(ora.generate(wl["family"]))
    R, T = args.realizations or wl["R"], args.t_final or wl["t_final"]
    for _ in range(args.warmup):
        cpu_baseline(o, wl, R, T, args.seed, budget_s=2.0)
    vals, t_all = [], 0.0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        cb = cpu_baseline(o, wl, R, T, args.seed, budget_s=8.0)
        t_all += time.perf_counter() - t0
        vals.append(cb["value"])
    cb.pop("_finals")
    v = float(np.mean(vals))
    cb["value"] = v
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t_all / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp64+int64", "data": "synthetic (seeded generator)",
            "config": workload_config(wl, R, T, int(os.environ.get("WORLD_SIZE", "1"))),
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
    ap.add_argument("--no-plain", action="store_true", help="skip the plain-form comparisons")
    ap.add_argument("--batch-scale", type=float, default=1.0)
    ap.add_argument("--t-final", type=float, default=0.0, help="override t_final (profiling captures)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    wl = WORKLOADS[args.workload]
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        from oracle import build as ob
        ob.build()
        run_reference(args, wl, rank)
        return
    import __graft_entry__
    __graft_entry__.build()
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
