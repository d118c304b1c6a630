import importlib.util
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "hpx-fft_gb300")
for p in (os.path.join(PKG, "python"), os.path.join(REPO, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def _load_build():
    spec = importlib.util.spec_from_file_location("hpxfft_build", os.path.join(PKG, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _gpu_present() -> bool:
    if os.path.exists("/dev/nvidia0") or os.path.exists("/dev/nvidiactl"):
        return True
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


def pytest_collection_modifyitems(config, items):
    if _gpu_present():
        return
    skip = pytest.mark.skip(reason="no CUDA device in this machine")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def build_mod():
    return _load_build()


@pytest.fixture(scope="session")
def oracle_lib(build_mod):
    build_mod.build_oracle()
    import oracle

    oracle.load()
    return oracle


@pytest.fixture(scope="session")
def gpu_lib(build_mod):
    """Build (if stale) and load libhpxfft_gb300.so; the import fails loudly if missing."""
    build_mod.build_library()
    import hpxfft

    hpxfft._capi.load()
    return hpxfft


@pytest.fixture(scope="session")
def cuda():
    import torch

    assert torch.cuda.is_available(), "GPU test needs CUDA"
    torch.cuda.init()
    return torch
