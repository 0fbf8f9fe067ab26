"""Build recipe for planes-rl_gb300: CUDA kernels + C ABI -> lib/libplanes_gb300.so, and the
`planes` command-line driver -> bin/planes.

Every CUDA translation unit is compiled for sm_103a only, with the reference's numeric flags
(-O3 -use_fast_math, Makefile:3 of the reference) except the gradient (IEEE math), in parallel;
objects are linked with the static CUDA runtime so the library needs only the driver at run time.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB_DIR = os.path.join(HERE, "lib")
BIN_DIR = os.path.join(HERE, "bin")
LIB = os.path.join(LIB_DIR, "libplanes_gb300.so")
CLI = os.path.join(BIN_DIR, "planes")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_FLAGS = ["-O3", "-use_fast_math", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-warn-spills"]
CU_SOURCES = ["pe_prepare.cu", "pe_flight.cu", "pe_flight_fast.cu", "pe_scores.cu", "pe_api.cu", "pe_probe.cu",
              "pe_noalloc.cu", "pe_grad.cu", "pe_objective.cu", "pe_ga.cu", "pe_audit.cu"]
# The gradient and the objective it differentiates are built without fast math: they are checked
# against FP64 finite differences, and the FP64 objective must stay FP64.
PRECISE_SOURCES = {"pe_grad.cu", "pe_objective.cu"}
HOST_SOURCES = ["pe_host.cpp", "pe_drivers.cpp"]
CLI_SOURCES = ["pe_cli.cpp"]
HEADERS = ["pe_model.cuh", "pe_internal.cuh", "pe_grad_model.h", "pe_f32x2.cuh"]


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def _compile_cu(src, verbose=False):
    out = os.path.join(OBJ, os.path.splitext(src)[0] + ".o")
    deps = [os.path.join(CSRC, src)] + [os.path.join(CSRC, h) for h in HEADERS]
    deps.append(os.path.join(ROOT, "include", "planes_eval.h"))
    if _stale(out, deps):
        extra = ["-Xptxas", "-v"] if verbose else []
        flags = [f for f in CU_FLAGS if f != "-use_fast_math"] if src in PRECISE_SOURCES else CU_FLAGS
        log = _run([NVCC] + ARCH + flags + extra + ["-I" + os.path.join(ROOT, "include"), "-c",
                    os.path.join(CSRC, src), "-o", out])
        if verbose:
            sys.stderr.write(log)
    return out


def _compile_host(src):
    out = os.path.join(OBJ, os.path.splitext(src)[0] + ".o")
    deps = [os.path.join(CSRC, src), os.path.join(ROOT, "include", "planes_eval.h")]
    if os.path.exists(os.path.join(CSRC, src)) and _stale(out, deps):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include"),
              "-I/usr/local/cuda/include", "-c", os.path.join(CSRC, src), "-o", out])
    return out if os.path.exists(os.path.join(CSRC, src)) else None


def build(force=False, verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    os.makedirs(BIN_DIR, exist_ok=True)
    if force:
        for f in os.listdir(OBJ):
            os.remove(os.path.join(OBJ, f))
    with cf.ThreadPoolExecutor(max_workers=len(CU_SOURCES) + len(HOST_SOURCES)) as ex:
        futs = [ex.submit(_compile_cu, s, verbose) for s in CU_SOURCES]
        futs += [ex.submit(_compile_host, s) for s in HOST_SOURCES]
        objs = [f.result() for f in futs]
    objs = [o for o in objs if o]
    if _stale(LIB, objs):
        _run([NVCC] + ARCH + ["-shared", "-cudart", "static", "-o", LIB] + objs)
    cli_src = [os.path.join(CSRC, s) for s in CLI_SOURCES if os.path.exists(os.path.join(CSRC, s))]
    if cli_src and _stale(CLI, cli_src + [LIB]):
        _run(["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), "-o", CLI] + cli_src +
             ["-L" + LIB_DIR, "-lplanes_gb300", "-Wl,-rpath,$ORIGIN/../lib"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
