"""Shared fixtures.  Markers: `gpu` tests need a CUDA device (GB300) and call
the library through its C ABI; everything else runs on the CPU."""
from __future__ import annotations

import importlib.util
import shutil
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "video-stream-consistency_gb300"
GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(ROOT / "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libvsc.so")


def import_vsc():
    if "vsc_gb300" in sys.modules:
        return sys.modules["vsc_gb300"]
    spec = importlib.util.spec_from_file_location("vsc_gb300", PKG / "__init__.py",
                                                  submodule_search_locations=[str(PKG)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["vsc_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def oracle():
    import oracle as O

    O.build(ref=True)
    return O


@pytest.fixture(scope="session")
def vsc():
    """The package with libvsc.so built (nvcc cross-compiles without a GPU)."""
    mod = import_vsc()
    if shutil.which("nvcc") or Path("/usr/local/cuda/bin/nvcc").exists():
        mod.build()
    mod.load()
    return mod


@pytest.fixture(scope="session")
def cuda(vsc):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    return {p.stem: dict(np.load(p)) for p in GOLDEN.glob("*.npz")}
