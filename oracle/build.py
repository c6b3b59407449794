"""Build recipe of the oracle (test infrastructure, not part of the engine).

* ``oracle/liboracle.so``  the FP64 host restatement (tl_oracle.cpp).
* ``oracle/_ref/``         when the reference sources are present, the
  reference's own host-compilable functors built by ``build_ref.sh``
  (see that script); skipped silently where the sources are absent.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
REF_DIR = HERE / "_ref"
REFERENCE = Path(os.environ.get("TL_REFERENCE_DIR", "/root/reference"))


def _stale(out: Path, srcs: list[Path]) -> bool:
    sys.path.insert(0, str(HERE.parent))
    from tau_leaping_gb300.build import native_elf
    if not out.exists() or not native_elf(out):
        return True
    return any(s.stat().st_mtime > out.stat().st_mtime for s in srcs)


def build() -> Path:
    src = HERE / "tl_oracle.cpp"
    if _stale(LIB, [src]):
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", str(src), "-o", str(LIB)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("oracle build failed")
    script = HERE / "build_ref.sh"
    if script.exists() and (REFERENCE / "tau_leaping").is_dir():
        r = subprocess.run(["bash", str(script), str(REFERENCE), str(REF_DIR)], capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write("reference oracle build failed (continuing without it):\n" + r.stdout[-2000:] +
                             r.stderr[-2000:])
    return LIB


if __name__ == "__main__":
    print(build())
