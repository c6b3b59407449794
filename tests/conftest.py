import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))



def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA path through the C ABI")
    config.addinivalue_line("markers", "slow: long-running statistical test")


def _has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


HAS_GPU = _has_gpu()


def pytest_collection_modifyitems(config, items):
    if HAS_GPU:
        return
    skip = pytest.mark.skip(reason="no CUDA device in this environment")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build libtl.so and the oracle once per session (in-tree, incremental)."""
    from oracle import build as ob
    from tau_leaping_gb300 import build
    build.build_lib()
    ob.build()
    yield


@pytest.fixture(scope="session")
def reference_build():
    """The reference's own host build (oracle/_ref), present only where its
    sources were available to the oracle's build recipe."""
    lib = ROOT / "oracle" / "_ref" / "libtlref.so"
    from oracle.build import native_elf
    if not native_elf(lib):
        pytest.skip("the reference's host build is not present")
    return lib
