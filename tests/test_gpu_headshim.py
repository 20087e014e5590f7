"""The literal drop-in test: the reference's own main.cu (Main_Code/src/main.cu,
unchanged; head.h patched as for the reference builds) compiled against the GB300
stepper through the head.h shim (nspipe-gpu_gb300/headshim/nsp_headshim.cu) and
run as the reference program: restart files in, the io_*.txt files and
ur.bin/ut.bin/uz.bin out.  Its final state is checked against the reference build's
golden fixture (config s2, 20 steps, relative L2 <= 1e-12) and its output files
against the ones the reference build wrote (config s2, 100 steps, the short output
schedule of tests/golden/io_s2/).  Needs the staged reference sources
(oracle/_ref/src, present where the reference checkout was)."""
import os
import shutil

import numpy as np
import pytest

from conftest import ROOT, rel
from test_gpu_parity import CFG, golden, init, nsp  # noqa: F401  (fixtures)
from test_run_host import IO, lines

pytestmark = pytest.mark.gpu

SRC = os.path.join(ROOT, "oracle", "_ref", "src", "main.cu")


@pytest.fixture(scope="module")
def br():
    if not os.path.exists(SRC):
        pytest.skip("reference sources not staged (oracle/_ref/src)")
    import sys
    sys.path.insert(0, os.path.join(ROOT, "oracle", "ref"))
    import build_ref
    return build_ref


def fields_dir(nsp, tmp_path):
    d = str(tmp_path / "init")
    nsp.write_state(init(nsp, "s2"), d)
    return d


def test_reference_main_on_gb300_stepper_s2(nsp, br, tmp_path):
    exe = br.build_shim("s2", 20)
    rc, out = br.run_exe(exe, fields_dir(nsp, tmp_path), str(tmp_path / "run"))
    assert rc == 0, out[-2000:]
    NR, NT, NZ = CFG["s2"][:3]
    u = nsp.read_state(str(tmp_path / "run"), (NR, NT, NZ), suffix="")
    assert rel(np.stack(u), golden("s2")["u_20"]) < 1e-12


def test_reference_main_output_files_s2(nsp, br, tmp_path):
    exe = br.build_shim("s2", 100, io=True)
    run = str(tmp_path / "run")
    rc, out = br.run_exe(exe, fields_dir(nsp, tmp_path), run)
    assert rc == 0, out[-2000:]
    assert " Step 3 of 100" in out  # the reference's progress lines at each friction row
    for name in ("io_friction.txt", "io_qcross.txt", "io_ucross.txt", "io_meanpr.txt"):
        ref = lines(name)
        with open(os.path.join(run, name)) as fh:
            mine = fh.read().split("\n")[:-1]
        assert len(mine) >= len(ref), name
        for a, b in zip(mine, ref):
            assert a.split("  ")[0] == b.split("  ")[0], name
            va, vb = np.array([float(x) for x in a.split()]), np.array([float(x) for x in b.split()])
            assert np.all(np.abs(va - vb) <= 1.5e-8 * np.abs(vb) + 1e-300), (name, a, b)
