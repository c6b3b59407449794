"""Build the engine in-tree: libtl.so (CUDA kernels + C ABI) and the tl_cli
and tl_gen executables.

Every CUDA translation unit is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``); translation units are compiled
in parallel and skipped when their object is newer than every source.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
HOST = PKG / "host"
INC = ROOT / "include"
OBJ = ROOT / "_build"

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
if not Path(NVCC).exists():
    NVCC = shutil.which("nvcc") or NVCC
CXX = os.environ.get("CXX", "g++")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", str(INC)]
# extra nvcc flags for tuning builds, e.g. TL_NVCC_FLAGS="-DTL_WARP_MINB=3"
NVFLAGS += os.environ.get("TL_NVCC_FLAGS", "").split()
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-I", str(INC)]

LIB = PKG / "libtl.so"
CLI = PKG / "tl_cli"
GEN = PKG / "tl_gen"


def _deps() -> list[Path]:
    return sorted(list(CSRC.glob("*")) + list(HOST.glob("*")) + list(INC.glob("*.h")))


def native_elf(path: Path) -> bool:
    """True if path is an ELF object for this machine (x86-64 here, aarch64
    on the GPU hosts); a foreign object is rebuilt, never loaded."""
    import platform
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
    t = out.stat().st_mtime
    return any(s.stat().st_mtime > t for s in srcs)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        raise RuntimeError(f"build step failed: {cmd[0]} {cmd[-1]}")


def build_lib(verbose: bool = False) -> Path:
    OBJ.mkdir(exist_ok=True)
    import fcntl
    with open(OBJ / ".lock", "w") as lk:  # concurrent ranks build once
        fcntl.flock(lk, fcntl.LOCK_EX)
        try:
            return _build_lib()
        finally:
            fcntl.flock(lk, fcntl.LOCK_UN)


def _build_lib() -> Path:
    deps = _deps()
    units = []
    for cu in sorted(CSRC.glob("*.cu")):
        o = OBJ / (cu.stem + ".o")
        units.append((o, [NVCC, *NVFLAGS, "-c", str(cu), "-o", str(o)]))
    for cpp in sorted(HOST.glob("*.cpp")):
        if cpp.name in ("tl_cli.cpp", "tl_gen.cpp"):
            continue
        o = OBJ / (cpp.stem + ".o")
        units.append((o, [CXX, *CXXFLAGS, "-c", str(cpp), "-o", str(o)]))
    todo = [(o, c) for o, c in units if _stale(o, deps)]
    if todo:
        with ThreadPoolExecutor(max_workers=min(8, len(todo))) as ex:
            list(ex.map(lambda oc: _run(oc[1]), todo))
    objs = [str(o) for o, _ in units]
    if todo or _stale(LIB, [Path(o) for o in objs]):
        _run([NVCC, *ARCH, "-shared", "-Xcompiler", "-fPIC", "-o", str(LIB), *objs])
    for exe, src in ((CLI, HOST / "tl_cli.cpp"), (GEN, HOST / "tl_gen.cpp")):
        if src.exists() and (_stale(exe, [src, LIB] + list(INC.glob("*.h")))):
            _run([CXX, *CXXFLAGS, str(src), "-o", str(exe), "-L", str(PKG), "-ltl",
                  "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    build_lib()
    print("built", LIB)
