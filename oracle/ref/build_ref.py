"""Build recipe for the reference nsPipe-CUDA binary (the end-to-end oracle).

TEST INFRASTRUCTURE.  The reference is configured only by #defines in
Main_Code/src/head.h (head.h:16-61), so every configuration is a separate
build.  This script

  stage()            copies Main_Code/src from the read-only reference checkout
                     into oracle/_ref/src (git-ignored; it travels with the
                     working tree so the GPU host can compile it there),
  build(cfg, mode)   copies oracle/_ref/src into oracle/_ref/<cfg>/<mode>/,
                     rewrites the parameter #defines of head.h, and compiles
                     every reference source except main.cu together with
                     oracle/ref/ref_driver.cu (nvcc, sm_103a, -lcufft -lcublas),
                     wrapping nonlinear() at link time to count calls,
  run(cfg, mode, ..) runs it in oracle/_ref/<cfg>/<mode>/run/ on given u?_s.bin.

Modes: 'trace' (nsteps=1, integrate() called once per step), 'time' (nsteps=N,
one integrate() call, output files off) and 'io' (as 'time', with the output
schedule IO_SCHEDULE patched into head.h:33-40 so that integrate() writes its
io_*.txt files into the run directory).

No reference source is modified other than the #define values; nothing is
copied into the tracked tree.
"""
import os
import re
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
REF_OUT = os.path.join(ORACLE, "_ref")
# Checkout of the reference project: $NSP_REFERENCE_ROOT, else the container's read-only copy.
REF_ROOT = os.environ.get("NSP_REFERENCE_ROOT") or "/root/reference"
REF_SRC_DEFAULT = os.path.join(REF_ROOT, "Main_Code", "src")
REMESH_SRC_DEFAULT = os.path.join(REF_ROOT, "tools", "Re_Mesh", "src")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

# name -> (NR, NT, NZ, LZ expression, Re, dt in code units)
CONFIGS = {
    "s1": (24, 8, 9, "(1.0*PI2)", 1000.0, 0.01),
    "s2": (32, 16, 17, "(2.0*PI2)", 3000.0, 0.005),
    "c0": (48, 32, 65, "(2.0*PI2)", 2000.0, 0.01),
    "c1": (96, 128, 257, "(2.5*PI2)", 5300.0, 0.004),
    # the turbulent shape with half its time step (0.001 R/U_b): a long run that stays stable
    "c1h": (96, 128, 257, "(2.5*PI2)", 5300.0, 0.002),
    "c4b": (64, 48, 129, "(2.0*PI2)", 2700.0, 0.006),
    "c4c": (96, 96, 193, "(2.0*PI2)", 3500.0, 0.006),
}


def stage(src=None):
    """Copy the reference sources next to the build outputs (once, where the reference exists)."""
    src = src or REF_SRC_DEFAULT
    dst = os.path.join(REF_OUT, "src")
    if not os.path.isdir(src):
        if os.path.isdir(dst):
            return dst
        raise FileNotFoundError("reference sources not found: %s" % src)
    os.makedirs(dst, exist_ok=True)
    for f in os.listdir(src):
        shutil.copy2(os.path.join(src, f), os.path.join(dst, f))
        os.chmod(os.path.join(dst, f), 0o644)
    return dst


# mode 'io': dt_frc, dt_qcr, dt_mnp (head.h:33,36,39) and the rows buffered per write
# dc_frc = dc_qcr = dc_mnp (head.h:34,37,40).  With dt = 0.005 (s2) the accumulated
# time reaches 0.05 only after 11 steps (ten additions of 0.005 fall short of 0.05).
IO_SCHEDULE = (0.015, 0.05, 0.035, 4)


def _patch_header(text, NR, NT, NZ, LZ, Re, dt, nsteps, io=None):
    def sub(name, value):
        nonlocal text
        pat = re.compile(r"^#define\s+%s\b.*$" % re.escape(name), re.M)
        assert pat.search(text), name
        text = pat.sub("#define %s %s" % (name, value), text, count=1)

    sub("NR", NR)
    sub("NT", NT)
    sub("NZ", NZ)
    sub("LZ", LZ)
    sub("Re", "(%r)" % float(Re))
    sub("restart", 1)
    for k, v in zip(("dt_frc", "dt_qcr", "dt_mnp"), io[:3] if io else (1e30,) * 3):
        sub(k, repr(float(v)))
    if io:
        for k in ("dc_frc", "dc_qcr", "dc_mnp"):
            sub(k, int(io[3]))
    sub("dt", repr(float(dt)))
    sub("nsteps", nsteps)
    return text


def build(cfg, mode="trace", nsteps=None, jobs=8):
    """Compile oracle/_ref/<cfg>/<mode>/Pipe.  mode 'trace' builds nsteps=1."""
    NR, NT, NZ, LZ, Re, dt = CONFIGS[cfg]
    if mode == "trace":
        nsteps = 1
    assert nsteps is not None
    src = stage()
    out = os.path.join(REF_OUT, cfg, "%s%s" % (mode, "" if mode == "trace" else nsteps))
    os.makedirs(out, exist_ok=True)
    exe = os.path.join(out, "Pipe")
    if os.path.exists(exe):
        return exe
    for f in os.listdir(src):
        shutil.copy2(os.path.join(src, f), os.path.join(out, f))
    with open(os.path.join(out, "head.h")) as fh:
        hdr = fh.read()
    with open(os.path.join(out, "head.h"), "w") as fh:
        fh.write(_patch_header(hdr, NR, NT, NZ, LZ, Re, dt, nsteps, IO_SCHEDULE if mode == "io" else None))
    shutil.copy2(os.path.join(HERE, "ref_driver.cu"), os.path.join(out, "ref_driver.cu"))
    units = sorted(f for f in os.listdir(out) if f.endswith(".cu") and f != "main.cu")

    def cc(u):
        subprocess.run(["nvcc", "-O3", ARCH, "-I", out, "-c", os.path.join(out, u), "-o",
                        os.path.join(out, u[:-3] + ".o")], check=True)

    with ThreadPoolExecutor(jobs) as ex:
        list(ex.map(cc, units))
    objs = [os.path.join(out, u[:-3] + ".o") for u in units]
    subprocess.run(["nvcc", ARCH, "-o", exe] + objs + ["-Xlinker", "--wrap=_Z9nonlinear6vfieldS_",
                                                        "-lcufft", "-lcublas"], check=True)
    return exe


def run(cfg, mode, fields_dir, nsteps, snaps=None, nsteps_build=None):
    """Run the reference on u?_s.bin from fields_dir; returns the run directory."""
    exe = build(cfg, mode, nsteps=nsteps_build if mode != "trace" else None)
    rundir = os.path.join(os.path.dirname(exe), "run")
    os.makedirs(rundir, exist_ok=True)
    for c in "rtz":
        shutil.copy2(os.path.join(fields_dir, "u%s_s.bin" % c), os.path.join(rundir, "u%s_s.bin" % c))
    args = [exe, "trace" if mode == "trace" else "time", str(nsteps)] + ([",".join(str(s) for s in snaps)] if snaps else [])
    p = subprocess.run(args, cwd=rundir, capture_output=True, text=True)
    with open(os.path.join(rundir, "stdout.txt"), "w") as fh:
        fh.write(p.stdout + p.stderr)
    if p.returncode != 0:
        raise RuntimeError("reference run failed (%d): %s" % (p.returncode, (p.stdout + p.stderr)[-2000:]))
    return rundir


# ---- the reference's main.cu linked, unchanged, against the GB300 stepper's head.h shim

def build_shim(cfg, nsteps, io=False):
    """Compile main.cu (unchanged; head.h patched as for the reference builds) with
    nspipe-gpu_gb300/headshim/nsp_headshim.cu against libnspipe_gb300.so:
    oracle/_ref/<cfg>/shim[io]<nsteps>/Pipe.  The library must be built first."""
    NR, NT, NZ, LZ, Re, dt = CONFIGS[cfg]
    src = stage()
    repo = os.path.dirname(ORACLE)
    lib = os.path.join(repo, "nspipe-gpu_gb300")
    out = os.path.join(REF_OUT, cfg, "shim%s%d" % ("io" if io else "", nsteps))
    exe = os.path.join(out, "Pipe")
    if os.path.exists(exe):
        return exe
    os.makedirs(out, exist_ok=True)
    shutil.copy2(os.path.join(src, "main.cu"), os.path.join(out, "main.cu"))
    with open(os.path.join(src, "head.h")) as fh:
        hdr = fh.read()
    with open(os.path.join(out, "head.h"), "w") as fh:
        fh.write(_patch_header(hdr, NR, NT, NZ, LZ, Re, dt, nsteps, IO_SCHEDULE if io else None))
    shim = os.path.join(lib, "headshim", "nsp_headshim.cu")
    objs = [os.path.join(out, "main.o"), os.path.join(out, "shim.o")]
    subprocess.run(["nvcc", "-O3", ARCH, "-I", out, "-c", os.path.join(out, "main.cu"), "-o", objs[0]], check=True)
    subprocess.run(["nvcc", "-O3", "-std=c++17", ARCH, "-I", out, "-I", os.path.join(repo, "include"), "-c", shim,
                    "-o", objs[1]], check=True)
    subprocess.run(["nvcc", ARCH, "-o", exe] + objs + ["-L", lib, "-lnspipe_gb300", "-Xlinker", "-rpath=" + lib],
                   check=True)
    return exe


def run_exe(exe, fields_dir, rundir):
    """Run a build in rundir on u?_s.bin from fields_dir; returns (returncode, output)."""
    os.makedirs(rundir, exist_ok=True)
    for c in "rtz":
        shutil.copy2(os.path.join(fields_dir, "u%s_s.bin" % c), os.path.join(rundir, "u%s_s.bin" % c))
    p = subprocess.run([exe], cwd=rundir, capture_output=True, text=True)
    return p.returncode, p.stdout + p.stderr


# ---- the Re_Mesh tool (tools/Re_Mesh/src): mod_remesh.cu + mod_io.cu + remesh_driver.cu

def stage_remesh(src=None):
    """Copy the Re_Mesh sources to oracle/_ref/remesh_src (once, where the reference exists)."""
    src = src or REMESH_SRC_DEFAULT
    dst = os.path.join(REF_OUT, "remesh_src")
    if not os.path.isdir(src):
        if os.path.isdir(dst):
            return dst
        raise FileNotFoundError("Re_Mesh sources not found: %s" % src)
    os.makedirs(dst, exist_ok=True)
    for f in os.listdir(src):
        shutil.copy2(os.path.join(src, f), os.path.join(dst, f))
        os.chmod(os.path.join(dst, f), 0o644)
    return dst


def build_remesh(old, new, iw=3):
    """Compile oracle/_ref/remesh/<tag>/Remesh for old=(NR, NT, NZ) -> new=(Nrd, Ntd, Nzd)."""
    src = stage_remesh()
    tag = "%dx%dx%d_%dx%dx%d_iw%d" % (tuple(old) + tuple(new) + (iw,))
    out = os.path.join(REF_OUT, "remesh", tag)
    exe = os.path.join(out, "Remesh")
    if os.path.exists(exe):
        return exe
    os.makedirs(out, exist_ok=True)
    for f in ("head.h", "mod_remesh.cu", "mod_io.cu"):
        shutil.copy2(os.path.join(src, f), os.path.join(out, f))
    with open(os.path.join(out, "head.h")) as fh:
        text = fh.read()
    for name, value in zip(("NR", "NT", "NZ", "Nrd", "Ntd", "Nzd", "iw"), tuple(old) + tuple(new) + (iw,)):
        pat = re.compile(r"^#define\s+%s\b.*$" % name, re.M)
        assert pat.search(text), name
        text = pat.sub("#define %s %d" % (name, value), text, count=1)
    with open(os.path.join(out, "head.h"), "w") as fh:
        fh.write(text)
    shutil.copy2(os.path.join(HERE, "remesh_driver.cu"), os.path.join(out, "remesh_driver.cu"))
    objs = []
    for u in ("mod_remesh.cu", "mod_io.cu", "remesh_driver.cu"):
        obj = os.path.join(out, u[:-3] + ".o")
        subprocess.run(["nvcc", "-O3", ARCH, "-I", out, "-c", os.path.join(out, u), "-o", obj], check=True)
        objs.append(obj)
    subprocess.run(["nvcc", ARCH, "-o", exe] + objs, check=True)
    return exe


def run_remesh(old, new, iw, fields):
    """Run the tool on fields (3 complex arrays of shape old); returns the 3 new arrays."""
    import numpy as np
    exe = build_remesh(old, new, iw)
    rundir = os.path.join(os.path.dirname(exe), "run")
    os.makedirs(rundir, exist_ok=True)
    for c, a in zip("rtz", fields):
        np.ascontiguousarray(a, np.complex128).tofile(os.path.join(rundir, "u%s_o.bin" % c))
    p = subprocess.run([exe], cwd=rundir, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("Re_Mesh failed (%d): %s" % (p.returncode, (p.stdout + p.stderr)[-2000:]))
    return [np.fromfile(os.path.join(rundir, "u%s_s.bin" % c), np.complex128).reshape(new) for c in "rtz"]


if __name__ == "__main__":
    if sys.argv[1] == "stage":
        print(stage())
    elif sys.argv[1] == "build":
        print(build(sys.argv[2], sys.argv[3], int(sys.argv[4]) if len(sys.argv) > 4 else None))
