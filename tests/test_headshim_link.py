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
