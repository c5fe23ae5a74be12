"""Build of the psvwave_gb300 C-ABI library (libpsvwave_gb300.so) for sm_103a.

Compiles the CUDA kernels and the C++ host core with nvcc, one process per
translation unit, and links them into psvwave_gb300/_build/. The FP64 solver
and the FP64 helpers are compiled with -fmad=false so that no multiply-add is
contracted and their arithmetic rounds exactly as the reference's double
code does.
"""
import concurrent.futures
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
LIB_NAME = "libpsvwave_gb300.so"
LIB_PATH = os.path.join(BUILD, LIB_NAME)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code never contracts a*b+c into a fused multiply-add (g++ does by
# default on aarch64): the setup tables (Ricker wavelets, taper) must round
# exactly as the reference's double code does.
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler",
          "-ffp-contract=off", "-I", CSRC, "-I", INCLUDE]

# (source, extra flags)
UNITS = [
    ("psv_solver_f64.cu", ["-fmad=false"]),
    ("psv_solver_f32.cu", []),
    ("psv_fast_f32.cu", []),
    ("psv_tma_f32.cu", []),
    ("psv_exact_tma.cu", []),
    ("psv_cluster_f32.cu", []),
    ("psv_aux.cu", ["-fmad=false"]),
    ("psv_noalloc.cu", []),
    ("psv_config.cpp", []),
    ("psv_model.cpp", []),
    ("psv_batch.cpp", []),
    ("psv_capi.cpp", []),
    ("psv_cnn.cu", []),
    ("psv_surrogate_capi.cpp", []),
]


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the psvwave_gb300 CUDA library cannot be built")


def _sources():
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)
            if f.endswith((".cu", ".cuh", ".cpp", ".hpp"))]
    deps.append(os.path.join(INCLUDE, "psvwave.h"))
    deps.append(os.path.abspath(__file__))
    return deps


def up_to_date():
    if not os.path.exists(LIB_PATH):
        return False
    t = os.path.getmtime(LIB_PATH)
    return all(os.path.getmtime(p) <= t for p in _sources())


def _compile(args):
    src, flags, obj = args
    cmd = [nvcc()] + ARCH + COMMON + flags + ["-c", os.path.join(CSRC, src), "-o", obj]
    if src.endswith(".cpp"):
        cmd = [nvcc()] + COMMON + flags + ["-x", "c++", "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compiling %s failed:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return obj


def build(force=False, verbose=False):
    """Compile and link the library unless it is newer than every source."""
    if not force and up_to_date():
        return LIB_PATH
    os.makedirs(BUILD, exist_ok=True)
    units = [(s, f, os.path.join(BUILD, os.path.splitext(s)[0] + ".o"))
             for s, f in UNITS if os.path.exists(os.path.join(CSRC, s))]
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(units)) as ex:
        objs = list(ex.map(_compile, units))
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-Xcompiler", "-fPIC", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("linking failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, LIB_PATH)
    if verbose:
        print("built", LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    build(force=True, verbose=True)
