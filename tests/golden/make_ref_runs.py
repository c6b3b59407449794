"""Generate tests/golden/ref_runs.npz: per-realization samples from the
reference's own simulation (its Model API, host-built by
oracle/build_ref.sh, logging on), for the statistical comparison of the
engine's reference-compatibility mode with the reference's run.

    python tests/golden/make_ref_runs.py <reference root>

(the reference root is the checkout whose oracle/_ref build this uses; it
supplies examples/test_128.xml; TL_REFERENCE_DIR may give it instead)

Models are those on which the reference is well defined (as many channels
as species, so its FireReactions loop bound is right):
  * test_128  - the reference's examples/test_128.xml (128 x 128);
  * chain64   - this project's seeded 64-species cyclic chain.
For each, the model description (as parsed by the engine's StochKit reader)
and the reference's samples on its statistics grid (AllStat2StepStat, which
interpolates linearly between logged states and stops before t_final) are
stored; the reference's own timing is kept for the record.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

RUNS = {
    # name: (model source, t_final, realizations, intervals, eps, tracked names)
    # The reference interpolates linearly between the states it logs before
    # each step; the chain takes only ~17 leaps at eps 0.03, so it runs at
    # eps 0.003 (tenfold finer leaps) to keep that interpolation far below
    # the sampling error.
    "test_128": ("examples/test_128.xml", 0.1, 400, 4, 0.03, ["S1", "S5"]),
    "chain64": ("chain64", 1.0, 2000, 4, 0.003, ["S1", "S2", "S33"]),
}


def run(name, model_path, T, n, intervals, eps, tracked):
    exe = ROOT / "oracle" / "_ref" / "ref_driver"
    out = subprocess.run([str(exe), str(model_path), str(T), str(n), str(intervals), str(eps), "1", *tracked],
                         capture_output=True, text=True, check=True, cwd=tempfile.gettempdir()).stdout
    times, blocks, cur, secs, steps = [], [], None, 0.0, 0
    for line in out.splitlines():
        if line.startswith("#time"):
            parts = line.split()
            secs, steps = float(parts[1]), int(parts[3])
        elif line.startswith("t "):
            times.append(float(line.split()[1]))
            cur = []
            blocks.append(cur)
        elif cur is not None and line and not line.startswith("#"):
            cur.append([float(v) for v in line.split()])
    samples = np.array(blocks)  # [P', n, K]
    return np.array(times), samples, secs, steps


def main():
    from oracle import build
    from tau_leaping_gb300 import Model
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("TL_REFERENCE_DIR")
    if not ref:
        sys.exit("usage: make_ref_runs.py <reference root>")
    REFERENCE = Path(ref)
    os.environ["TL_REFERENCE_DIR"] = str(REFERENCE)
    build.build()
    out = {}
    with tempfile.TemporaryDirectory() as td:
        for name, (src, T, n, intervals, eps, tracked) in RUNS.items():
            if src.endswith(".xml"):
                path = REFERENCE / src
            else:
                path = Path(td) / f"{name}.xml"
                Model.generate("chain", n_species=64).write_stochkit(path)
            m = Model.from_stochkit(path)
            d = m.desc()
            times, samples, secs, steps = run(name, path, T, n, intervals, eps, tracked)
            idx = np.array([m.species_index(t) for t in tracked], np.int32)
            out.update({f"{name}/{k}": v for k, v in d.items()})
            out.update({f"{name}/times": times, f"{name}/samples": samples.astype(np.float32),
                        f"{name}/tracked": idx, f"{name}/t_final": np.float64(T),
                        f"{name}/intervals": np.int32(intervals), f"{name}/eps": np.float64(eps),
                        f"{name}/ref_seconds": np.float64(secs),
                        f"{name}/ref_logged_steps": np.int64(steps)})
            print(name, "grid", times, "samples", samples.shape, f"{secs:.1f}s")
    dst = Path(__file__).resolve().parent / "ref_runs.npz"
    np.savez_compressed(dst, **out)
    print("wrote", dst, dst.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
