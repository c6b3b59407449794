"""Build recipe of the oracle (test infrastructure, not part of the engine).

* ``oracle/liboracle.so``  the FP64 host restatement (tl_oracle.cpp).
* ``oracle/_ref/``         the reference's own host-compilable functors and
  host path, built by ``build_ref.sh`` from the reference's sources where
  they lie (the script finds them; ``TL_REFERENCE_DIR`` overrides); skipped
  where the sources are absent.

Self-contained: building the checker never imports or loads the engine.
"""
from __future__ import annotations

import os
import platform
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
REF_DIR = HERE / "_ref"


def native_elf(path: Path) -> bool:
    """True if path is an ELF object for this machine's architecture."""
    want = {"x86_64": 62, "aarch64": 183, "arm64": 183}.get(platform.machine())
    try:
        with open(path, "rb") as f:
            h = f.read(20)
    except OSError:
        return False
    if len(h) < 20 or h[:4] != b"\x7fELF":
        return False
    return want is None or int.from_bytes(h[18:20], "little") == want


def _stale(out: Path, srcs: list[Path]) -> bool:
    if not out.exists() or not native_elf(out):
        return True
    return any(s.stat().st_mtime > out.stat().st_mtime for s in srcs)


def build(reference: bool = True) -> Path:
    src = HERE / "tl_oracle.cpp"
    if _stale(LIB, [src]):
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", str(src), "-o", str(LIB)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("oracle build failed")
    script = HERE / "build_ref.sh"
    if reference and script.exists():
        args = ["bash", str(script), str(REF_DIR)]
        if os.environ.get("TL_REFERENCE_DIR"):
            args.append(os.environ["TL_REFERENCE_DIR"])
        r = subprocess.run(args, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write("reference oracle build failed (continuing without it):\n" + r.stdout[-2000:] +
                             r.stderr[-2000:])
    return LIB


if __name__ == "__main__":
    print(build())
