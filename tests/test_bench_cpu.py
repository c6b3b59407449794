"""bench.py's host-side figures (no GPU): the algorithmic bytes per
realization-step that the roofline divides by, and the DRAM traffic it reads
from the committed ncu summaries."""
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


def test_profile_traffic_is_read_from_the_committed_summaries():
    for w in ("toy", "chain", "colloid", "dimer"):
        t = bench.profile_traffic(w)
        assert t is not None and t > 0, w
    assert bench.profile_traffic("no-such-workload") is None


def test_every_workload_has_a_description():
    for name, wl in bench.WORKLOADS.items():
        assert wl["desc"] and wl["family"], name
