"""Shared fixtures.  GPU tests are marked ``gpu`` and need a CUDA device;
everything else runs on the CPU."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def small_models():
    """Small models used across tests: (name, kwargs, porder, interval mHz)."""
    from normalmodes_gb300.model import Model
    specs = {
        "solid_p1": (dict(n_cells=6, porder=1, fluid_core=0), 1, (0.2, 1.0)),
        "fs_p1": (dict(n_cells=8, porder=1), 1, (0.2, 1.0)),
        "fs_p2": (dict(n_cells=8, porder=2), 2, (0.2, 0.6)),
    }
    out = {}
    for name, (kw, p, iv) in specs.items():
        m = Model.ball(**kw)
        out[name] = {"model": m, "mats": m.operators(), "porder": p, "interval": iv}
    return out
