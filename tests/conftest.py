"""Test configuration: registers the ``gpu`` marker and puts the repo and the oracle on sys.path.

CPU tests (``-m "not gpu"``) cover the oracle, the settings / JSON host logic, the generator and
the C ABI surface (library loads, every declared symbol is exported). GPU tests (``-m gpu``) are
the parity tests: they call the library through the C ABI and compare with the oracle.
"""

import pathlib
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
for p in (ROOT, ROOT / "oracle", ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests through the C ABI")


@pytest.fixture(scope="session")
def cuda():
    """The GPU tests fail (not skip) when no GPU is visible: a silent skip would hide a missing device."""
    import torch

    assert torch.cuda.is_available(), "GPU test run without a visible CUDA device"
    torch.cuda.init()
    import holovibes_gb300 as hv

    hv.lib()
    return torch


@pytest.fixture(autouse=True)
def _release_device_copies():
    yield
    mod = sys.modules.get("gpu_util")
    if mod is not None:
        mod.release()
