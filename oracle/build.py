"""Build recipe for the oracle -- TEST INFRASTRUCTURE ONLY.

Outputs (all git-ignored):
  oracle/_build/liboracle.so   the C restatement (float + double, OpenMP), built on any host.
  oracle/_ref/libref_host.so   the reference's own src/common.h (+ src/designs.cu, src/stl.cu for
                               its preset genomes) behind oracle/ref_host_harness.cpp.  Built only
                               where the reference tree exists (this x86 container); it is used to
                               record tests/golden/host_golden.npz.
  oracle/_ref/ref_sim.ptx      the reference's src/sim.cu device code (k_prepare, k_sim), compiled
                               with the reference's flags (-O3 -use_fast_math) for compute_103a.
                               tests/golden/make_ref_cuda_golden.py JIT-loads it on a GB300 through
                               oracle/ref_cuda_runner.cpp to record the reference CUDA build's
                               outputs and timings.

The reference sources are compiled where they lie; nothing from them is copied.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference checkout: $PLANES_REF_ROOT, else a directory named "reference" beside this
# repository.  Where neither exists (the GPU host), only the oracle and the runner are built.
REF_ROOT = os.environ.get("PLANES_REF_ROOT") or os.path.normpath(
    os.path.join(HERE, os.pardir, os.pardir, "reference"))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")

ORACLE_SRC = ["oracle_f32.c", "oracle_f64.c", "oracle_common.c"]
ORACLE_LIB = os.path.join(BUILD, "liboracle.so")
RUNNER_BIN = os.path.join(BUILD, "ref_cuda_runner")


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))


def build_oracle(force=False):
    """gcc -O3 -fopenmp, no FP contraction: float results match the reference's x86-64 host build."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, s) for s in ORACLE_SRC]
    deps = srcs + [os.path.join(HERE, "oracle.h"), os.path.join(HERE, "oracle_impl.h")]
    if force or _stale(ORACLE_LIB, deps):
        _run(["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
              "-fno-fast-math", "-o", ORACLE_LIB] + srcs + ["-lm"])
    return ORACLE_LIB


def build_ref_cuda_runner(force=False):
    """Driver-API host program that runs the reference's k_prepare/k_sim from ref_sim.ptx.

    Built on whichever host runs it (it needs only libcuda), including the host of the GPU it drives.
    """
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "ref_cuda_runner.cpp")
    if not os.path.exists(src):
        return None
    if force or _stale(RUNNER_BIN, [src]):
        _run(["g++", "-O2", "-std=c++17", "-I/usr/local/cuda/include", "-o", RUNNER_BIN, src,
              "-L/usr/local/cuda/lib64", "-L/usr/local/cuda/lib64/stubs", "-lcuda"])
    return RUNNER_BIN


def have_reference():
    return os.path.exists(os.path.join(REF_ROOT, "src", "common.h"))


def build_ref(force=False):
    """Compile the reference's own sources into oracle/_ref (only where the tree exists)."""
    if not have_reference():
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    src = os.path.join(REF_ROOT, "src")
    lib = os.path.join(REF_OUT, "libref_host.so")
    harness = os.path.join(HERE, "ref_host_harness.cpp")
    host_deps = [harness, os.path.join(src, "common.h"), os.path.join(src, "designs.cu"),
                 os.path.join(src, "stl.cu")]
    if force or _stale(lib, host_deps):
        # the reference's own host-test recipe (Makefile:63-65) builds these two files with
        # g++ -x c++; -ffp-contract=off keeps float results identical on any host ISA.
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
              "-I" + src, "-x", "c++", os.path.join(src, "stl.cu"), os.path.join(src, "designs.cu"),
              harness, "-o", lib])
    ptx = os.path.join(REF_OUT, "ref_sim.ptx")
    sim_deps = [os.path.join(src, "sim.cu"), os.path.join(src, "common.h"), os.path.join(src, "sim.h")]
    if force or _stale(ptx, sim_deps):
        # reference flags, Makefile:3 (-O3 -use_fast_math -std=c++17 -lineinfo), for compute_103a
        _run(["nvcc", "-ptx", "-O3", "-use_fast_math", "-std=c++17", "-lineinfo",
              "-arch=compute_103a", "-I" + src, os.path.join(src, "sim.cu"), "-o", ptx])
    return lib


def build_all(force=False):
    out = {"oracle": build_oracle(force)}
    out["ref"] = build_ref(force)
    try:
        out["runner"] = build_ref_cuda_runner(force)
    except RuntimeError as e:  # needs libcuda headers; optional for the CPU tests
        out["runner"] = None
        sys.stderr.write(str(e))
    return out


if __name__ == "__main__":
    print(build_all(force="--force" in sys.argv))
