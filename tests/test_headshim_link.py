"""CPU check of the head.h shim: the reference's own main.cu (staged in
oracle/_ref/src) compiles unchanged and links against nspipe-gpu_gb300/headshim and
libnspipe_gb300.so, i.e. the shim provides every entry point main.cu calls.  (The
run itself is the GPU test test_gpu_headshim.py.)"""
import os
import shutil

import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "oracle", "_ref", "src")


def test_reference_main_links_against_shim(tmp_path, monkeypatch):
    if not os.path.exists(os.path.join(SRC, "main.cu")):
        pytest.skip("reference sources not staged (oracle/_ref/src)")
    if not shutil.which("nvcc"):
        pytest.skip("nvcc not found")
    import sys
    sys.path.insert(0, os.path.join(ROOT, "nspipe-gpu_gb300"))
    sys.path.insert(0, os.path.join(ROOT, "oracle", "ref"))
    import build as nbuild
    import build_ref
    nbuild.build()
    shutil.copytree(SRC, str(tmp_path / "src"))
    monkeypatch.setattr(build_ref, "REF_OUT", str(tmp_path))
    monkeypatch.setattr(build_ref, "REF_SRC_DEFAULT", str(tmp_path / "absent"))
    exe = build_ref.build_shim("s2", 20)
    assert os.path.exists(exe) and os.access(exe, os.X_OK)


def test_integration_example_compiles(tmp_path):
    """The hand-written integrate() replacement in the integration notes (the ```cpp block
    that defines integrate_gb300(vfield u)) compiles against the reference's head.h: its
    macros share the C ABI's field names, and the example shows the way round them."""
    import re
    import subprocess
    if not os.path.exists(os.path.join(SRC, "head.h")):
        pytest.skip("reference sources not staged (oracle/_ref/src)")
    if not shutil.which("nvcc"):
        pytest.skip("nvcc not found")
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    code = [b for b in re.findall(r"```cpp\n(.*?)```", text, re.S) if "integrate_gb300(vfield u)" in b][0]
    src = tmp_path / "example.cu"
    src.write_text(code)
    p = subprocess.run(["nvcc", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", "-I", SRC, "-I",
                        os.path.join(ROOT, "include"), "-c", str(src), "-o", str(tmp_path / "example.o")],
                       capture_output=True, text=True)
    assert p.returncode == 0, p.stdout + p.stderr
