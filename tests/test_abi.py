"""The C-ABI library loads and exports every entry point include/planes_eval.h declares.

No compute calls: these run on hosts without a GPU.
"""
import ctypes as C
import os
import re
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "planes_eval.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pe_[a-z_0-9]+)\s*\(", src)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for n in ("pe_panelbuf_alloc", "pe_panelbuf_free", "pe_prepare", "pe_sim", "pe_eval_batch",
              "pe_evaluate_population", "pe_robust_scores", "pe_engine_create", "pe_autotune"):
        assert n in names


def test_header_is_plain_c():
    r = subprocess.run(["gcc", "-std=c99", "-fsyntax-only", "-Wall", "-Werror", "-x", "c", HEADER],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_library_exports_every_declared_symbol(built_lib):
    lib = C.CDLL(built_lib)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", built_lib], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (pe_[a-z_0-9]+)$", out, flags=re.M))
    assert set(declared_functions()) <= exported


def test_binding_loads_and_reports_errors(built_lib):
    import pe

    assert pe.LIB.pe_version() >= 100
    # argument checks run before any device work
    h = C.c_void_p()
    assert pe.LIB.pe_panelbuf_alloc(0, C.byref(h)) == pe.PE_EINVAL
    assert b"pop" in pe.LIB.pe_last_error()
    assert pe.LIB.pe_panelbuf_free(None) == pe.PE_OK
    assert pe.LIB.pe_robust_scores(None, 1, 1, None, None) == pe.PE_EINVAL


def test_population_bound_is_checked_before_device_work(built_lib):
    """Panel offsets are 32-bit: more than PE_MAX_POP planes in one call is PE_EINVAL, with a message,
    before any device is touched (so it holds on a host without a GPU)."""
    import pe

    src = open(HEADER).read()
    assert int(re.search(r"#define PE_MAX_POP (\d+)", src).group(1)) == pe.MAX_POP
    assert pe.MAX_POP * 344 < 2 ** 31
    h = C.c_void_p()
    assert pe.LIB.pe_panelbuf_alloc(pe.MAX_POP + 1, C.byref(h)) == pe.PE_EINVAL
    assert b"pop must be in 1..4194304" in pe.LIB.pe_last_error()
    assert not h.value
