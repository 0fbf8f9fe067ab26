import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "planes-rl_gb300")
ORACLE = os.path.join(ROOT, "oracle")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (PKG, ORACLE):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def oracle():
    import oracle_py

    oracle_py.lib()
    return oracle_py


@pytest.fixture(scope="session")
def host_golden():
    return np.load(os.path.join(GOLDEN, "host_golden.npz"))


@pytest.fixture(scope="session")
def built_lib():
    """The C-ABI library, built here if missing (nvcc cross-compiles without a GPU)."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("planes_gb300_build", os.path.join(PKG, "build.py"))
    pkg_build = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(pkg_build)
    return pkg_build.build()


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="session")
def pe(built_lib, cuda):
    import pe as pe_mod

    return pe_mod


@pytest.fixture(scope="session")
def engine(pe):
    """Engine in the default (body-frame) formulation."""
    e = pe.Engine(0)
    yield e
    e.close()


@pytest.fixture(scope="session", params=[0, 1], ids=["reference-arith", "body-frame"])
def any_engine(request, pe):
    """One engine per flight formulation."""
    e = pe.Engine(0)
    e.set_config(formulation=request.param, reg_cap=0, lanes=32 if request.param == 0 else 16)
    yield e
    e.close()
