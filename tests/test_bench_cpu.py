"""bench.py's host-side figures (no GPU): the algorithmic bytes per
realization-step that the roofline divides by, the config both arms report,
and the rule that ncu figures are used only from the same kernel build."""
import json
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402
from tau_leaping_gb300 import Model  # noqa: E402


def test_algorithmic_bytes_per_step_match_the_design_table():
    # 4 nnz (CSR) + 4 nnz (CSC) + 13 M + 4 (N + 1) + 2 w N
    want = {"dimer": 148, "toy": 10892, "chain": 41988, "colloid": 1159254}
    for fam, b in want.items():
        assert bench.alg_bytes_per_step(Model.generate(fam)) == b, fam


def test_workload_sizes_match_the_generator():
    for name, wl in bench.WORKLOADS.items():
        assert wl["desc"] and wl["family"], name
        if wl["family"] == "batch":
            continue
        m = Model.generate(wl["family"])
        assert (m.n_species, m.n_channels, m.pop_bits) == (wl["n_species"], wl["n_channels"], wl["pop_bits"]), name
        assert bench.dtype_of(wl) == ("fp32+int64" if m.pop_bits == 64 else "fp32+int32")


def test_both_arms_report_the_same_config():
    wl = bench.WORKLOADS["toy"]
    a = bench.workload_config(wl, wl["R"], wl["t_final"], 1)
    b = bench.workload_config(wl, wl["R"], wl["t_final"], 1)
    assert a == b and json.dumps(a) == json.dumps(b)


def test_ncu_record_is_used_only_for_the_same_kernel_build(tmp_path, monkeypatch):
    monkeypatch.setattr(bench, "ROOT", tmp_path)
    (tmp_path / "profiles").mkdir()
    assert bench.ncu_record("k_fused_toy")[0] is None
    rec = {"source_sha256": bench.kernel_source_hash(), "dram_bytes_per_launch": 5, "issue_slots_busy_pct": 70.0}
    (tmp_path / "profiles" / "k_fused_toy.ncu.json").write_text(json.dumps(rec))
    assert bench.ncu_record("k_fused_toy")[0]["dram_bytes_per_launch"] == 5
    rec["source_sha256"] = "0" * 64
    (tmp_path / "profiles" / "k_fused_toy.ncu.json").write_text(json.dumps(rec))
    got, why = bench.ncu_record("k_fused_toy")
    assert got is None and "another kernel build" in why


def test_reference_arm_runs_the_oracle_only():
    """`bench.py --impl reference` builds its model with the oracle's own
    generator and never maps the engine library; its JSON line carries the
    same config as the engine's arm."""
    import subprocess
    code = ("import runpy, sys\n"
            "sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '3',\n"
            "            '--realizations', '64', '--t-final', '0.005']\n"
            "try:\n"
            "    runpy.run_path('bench.py', run_name='__main__')\n"
            "finally:\n"
            "    maps = open('/proc/self/maps').read()\n"
            "    print('MAPS', 'libtl.so' in maps, 'liboracle.so' in maps)\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = r.stdout.strip().splitlines()
    assert lines[-1] == "MAPS False True", lines[-1]
    line = json.loads(lines[-2])
    wl = bench.WORKLOADS["toy"]
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["config"] == bench.workload_config(wl, 64, 0.005, 1)
    assert line["e2e"]["h2d_bytes_per_step"] == 0
