"""Build libnspipe_gb300.so in place (nvcc for sm_103a; g++ for the host setup).

    python nspipe-gpu_gb300/build.py                 # incremental build
    python nspipe-gpu_gb300/build.py --force         # rebuild everything
    python nspipe-gpu_gb300/build.py --bounds-check  # the bounds-checked library

Objects go to nspipe-gpu_gb300/_build/ (git-ignored), the library to
nspipe-gpu_gb300/libnspipe_gb300.so.  Translation units compile in parallel.  The
bounds-checked build (-DNSP_BOUNDS_CHECK, csrc/nsp_bounds.cuh) goes to _build_bc/ and
libnspipe_gb300_bc.so: the same entry points, with every computed global index of the
step kernels checked (nsp_bounds_report).
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libnspipe_gb300.so")
BUILD_BC = os.path.join(HERE, "_build_bc")
LIB_BC = os.path.join(HERE, "libnspipe_gb300_bc.so")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
            "--expt-relaxed-constexpr", "-I", os.path.join(HERE, "..", "include")] + ARCH
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-I", os.path.join(CUDA, "include"),
             "-I", os.path.join(HERE, "..", "include")]

CU_UNITS = ["nsp_api.cu", "nsp_linear.cu", "nsp_transform.cu", "nsp_noalloc.cu", "nsp_theta_tc.cu", "nsp_remesh.cu",
            "nsp_setup_dev.cu"]
# Per-unit extra flags.  nsp_setup_dev.cu builds the operator tables that nsp_setup.cpp
# builds on the host (-ffp-contract=off): without FMA contraction both give the same bits.
CU_EXTRA = {"nsp_setup_dev.cu": ["-fmad=false"]}
CXX_UNITS = ["nsp_setup.cpp", "nsp_run.cpp"]
HEADERS = ["nsp_internal.h", "nsp_setup_mode.h", "nsp_fft.cuh", "nsp_cvt.cuh", "nsp_state.cuh", "nsp_tc.cuh",
           "nsp_bounds.cuh", "nsp_df.cuh", os.path.join("..", "..", "include", "nspipe_gb300.h")]


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, h) for h in HEADERS]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force=False, verbose=False, bounds_check=False):
    bdir, lib = (BUILD_BC, LIB_BC) if bounds_check else (BUILD, LIB)
    defs = ["-DNSP_BOUNDS_CHECK"] if bounds_check else []
    os.makedirs(bdir, exist_ok=True)
    jobs = []
    for u in CU_UNITS:
        src, obj = os.path.join(CSRC, u), os.path.join(bdir, u + ".o")
        if force or _stale(obj, src):
            jobs.append([NVCC] + CU_FLAGS + defs + CU_EXTRA.get(u, []) + ["-c", src, "-o", obj])
    for u in CXX_UNITS:
        src, obj = os.path.join(CSRC, u), os.path.join(bdir, u + ".o")
        if force or _stale(obj, src):
            jobs.append(["g++"] + CXX_FLAGS + defs + ["-c", src, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s" % (" ".join(cmd), p.stdout + p.stderr))
        return p.stdout + p.stderr

    with ThreadPoolExecutor(max(1, len(jobs))) as ex:
        for out in ex.map(run, jobs):
            if verbose and out.strip():
                print(out)
    objs = [os.path.join(bdir, u + ".o") for u in CU_UNITS + CXX_UNITS]
    if force or jobs or not os.path.exists(lib):
        run([NVCC] + ARCH + ["-shared", "-cudart", "shared", "-o", lib] + objs)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, bounds_check="--bounds-check" in sys.argv))
