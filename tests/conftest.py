import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the helmgpu kernels)")


@pytest.fixture(scope="session")
def hz():
    """The helmholtz.jl_gb300 package (built library required)."""
    import __graft_entry__ as ge
    ge._load_build_module().build()
    return ge.load_package()


@pytest.fixture(scope="session")
def O():
    import helmholtz_oracle
    return helmholtz_oracle


@pytest.fixture(scope="session")
def cpu_slmg():
    import slmg_cpu
    return slmg_cpu
