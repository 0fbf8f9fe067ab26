"""The reference-side binding (planes-rl_gb300/shim/sim_gb300.cpp) compiles against the reference's
own src/sim.h and links against libplanes_gb300.so with no undefined symbol, and the four
definitions it exports carry exactly the signatures sim.h declares (src/sim.h:9-13), so the
reference's callers bind to them.  Needs the reference tree (skipped where it is absent); no GPU."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, "planes-rl_gb300", "shim", "sim_gb300.cpp")
LIBDIR = os.path.join(ROOT, "planes-rl_gb300", "lib")


def _ref_src():
    import importlib.util

    spec = importlib.util.spec_from_file_location("planes_oracle_build", os.path.join(ROOT, "oracle", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return os.path.join(mod.REF_ROOT, "src")


def test_shim_builds_against_reference_header(built_lib, tmp_path):
    src = _ref_src()
    if not os.path.exists(os.path.join(src, "sim.h")):
        pytest.skip("reference tree absent")
    out = str(tmp_path / "libsim_gb300.so")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-Wall", "-Werror", "-isystem", src,
                        "-I" + os.path.join(ROOT, "include"), SHIM, "-L" + LIBDIR, "-lplanes_gb300",
                        "-Wl,--no-undefined", "-o", out], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    nm = subprocess.run(["nm", "-DC", "--defined-only", out], capture_output=True, text=True).stdout
    defined = set(re.findall(r" T (.+)$", nm, flags=re.M))
    want = {"panelbuf_alloc(int)", "panelbuf_free(void*)", "gpu_prepare(Genome const*, void*, int)",
            "gpu_sim(void*, int, int, float*, float8*, int, int, float, int)"}
    assert want <= defined, defined
    # the reference's own declarations mangle to the same symbols: a caller compiled from sim.h
    # (as run_ga is) resolves against the shim
    caller = tmp_path / "caller.cpp"
    caller.write_text('#include "sim.h"\n'
                      'void* use(const Genome* g, float* f) { void* pb = panelbuf_alloc(4); gpu_prepare(g, pb, 4);\n'
                      '  gpu_sim(pb, 4, 1, f, nullptr, 1, 0, 0.0f, 0); panelbuf_free(pb); return pb; }\n')
    exe = str(tmp_path / "libcaller.so")
    r = subprocess.run(["g++", "-std=c++17", "-fPIC", "-shared", "-I" + src, str(caller), out,
                        "-Wl,--no-undefined", "-Wl,-rpath," + LIBDIR, "-L" + LIBDIR, "-lplanes_gb300", "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
