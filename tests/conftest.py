import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "hartree-fock_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libhfgpu.so")


def load_golden(name):
    d = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    d["soa"] = {k[4:]: v for k, v in d.items() if k.startswith("soa_")}
    return d


# Fock/SCF fixtures of the small systems.  Loaded separately: fd_* (finite-difference gradients), cfg_*
# (the benchmarked sizes, tests/test_gpu_configs.py) and boys_values (tests/test_gpu_boys.py).
GOLDEN_NAMES = sorted(f[:-4] for f in os.listdir(GOLDEN)
                      if f.endswith(".npz") and not f.startswith(("fd_", "cfg_", "boys_")))


@pytest.fixture(scope="session")
def port():
    from oracle import port as p

    p.build()
    return p


def gpu_available():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False
