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
def grad_host():
    """The gradient model (planes-rl_gb300/csrc/pe_grad_model.h) built for the host in double
    and float behind tests/grad_host_harness.cpp."""
    import ctypes as C
    import subprocess

    src = os.path.join(ROOT, "tests", "grad_host_harness.cpp")
    hdr = os.path.join(PKG, "csrc", "pe_grad_model.h")
    out = os.path.join(ROOT, "tests", "_build", "libgrad_host.so")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    if not os.path.exists(out) or os.path.getmtime(out) < max(os.path.getmtime(src), os.path.getmtime(hdr)):
        subprocess.check_call(["g++", "-std=c++17", "-O2", "-shared", "-fPIC", "-ffp-contract=off", src, "-o", out])
    lib = C.CDLL(out)
    vp, i = C.c_void_p, C.c_int
    lib.pgh_plane_data.argtypes = [vp] * 8
    lib.pgh_plane_data.restype = i
    lib.pgh_flight.argtypes = [vp, i, C.c_double, vp, i, vp, vp, vp, i, i, vp, vp, vp, vp, vp, vp, vp]
    lib.pgh_flight.restype = C.c_double
    for name in ("pgh_objective_grad", "pgh_objective_grad_f32"):
        getattr(lib, name).argtypes = [vp, vp, vp, i, i, i, vp, vp, vp, vp, vp]
        getattr(lib, name).restype = i
    return lib


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
