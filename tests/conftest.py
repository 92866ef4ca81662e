import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) and the built libttg.so")


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def tiny_system():
    from ttdft_public_gb300 import system
    return system.build_system(system.small_spec())


@pytest.fixture(scope="session")
def small_system():
    """~1.7k basis functions, 4 atoms with nonlocal projectors."""
    from ttdft_public_gb300 import system
    spec = system.small_spec(name="small", n_atoms=4, box=12.0, n_el=24, rank=12, n_states=24,
                             degree=12, seed=11)
    return system.build_system(spec)


@pytest.fixture(scope="session")
def atoms8_system():
    from ttdft_public_gb300 import system
    return system.build_system(system.CONFIGS["atoms8"])
