"""The run driver (nsp_run_*) on the GPU: the output files against the ones the
reference build wrote for the same run (tests/golden/io_s2/), and checkpoint /
resume against an uninterrupted run.

File parity: header rows and row times identical as text; values equal to the
printed precision (%.8e: 9 significant digits, so within 1.5e-8 relative, the
FP64 fields agreeing to ~1e-12).  The reference writes only whole blocks of
rows_per_write rows; its rows are a prefix of the driver's, which writes the last
partial block when the run closes.
"""
import os

import numpy as np
import pytest

from test_gpu_parity import CFG, init, nsp, stepper  # noqa: F401  (fixtures)
from test_run_host import INTERVAL, IO, NSTEPS, ROWS_PER_WRITE, lines

pytestmark = pytest.mark.gpu

FILES = ("io_friction.txt", "io_qcross.txt", "io_ucross.txt", "io_meanpr.txt")


def read_rows(path):
    with open(path) as fh:
        text = fh.read()
    assert text.endswith("\n")
    return text.split("\n")[:-1]


def values(row):
    return np.array([float(x) for x in row.split()])


def test_output_files_match_reference_build_s2(nsp, tmp_path):
    st = stepper(nsp, "s2", nsp.NSP_FP64)
    st.set_state(0, init(nsp, "s2"))
    out = str(tmp_path / "out")
    run = nsp.Run(st, out_dir=out, dt_frc=INTERVAL["io_friction.txt"], dt_qcr=INTERVAL["io_qcross.txt"],
                  dt_mnp=INTERVAL["io_meanpr.txt"], rows_per_write=ROWS_PER_WRITE)
    iters = run.advance(NSTEPS)
    assert iters.shape == (NSTEPS, 1) and (iters >= 1).all()
    t, n = run.time(0)
    t_ref = 0.0
    for _ in range(NSTEPS):
        t_ref += CFG["s2"][5]  # t += dt per step (mod_integrate.cu:131)
    assert n == NSTEPS and t == t_ref
    run.close()
    for name in FILES:
        ref = lines(name)
        mine = read_rows(os.path.join(out, name))
        head = 0 if name == "io_friction.txt" else 1
        if head:
            assert mine[0] == ref[0], name
        due, _ = nsp.output_schedule(CFG["s2"][5], INTERVAL[name], NSTEPS)
        assert len(mine) - head == int(due.sum()), name  # every row, the last partial block too
        for a, b in zip(mine[head:], ref[head:]):
            assert a.split("  ")[0] == b.split("  ")[0], name  # times, as text
            va, vb = values(a), values(b)
            assert va.shape == vb.shape, name
            assert np.all(np.abs(va - vb) <= 1.5e-8 * np.abs(vb) + 1e-300), (name, a, b)
    # the final state dump (main.cu:42-44) holds the state the context ends with
    u = st.get_state(0)
    for c, comp in zip("rtz", u):
        assert open(os.path.join(out, "u%s.bin" % c), "rb").read() == comp.tobytes()
    st.close()


def test_output_rows_are_the_diagnostics(nsp, tmp_path):
    """Each row carries nsp_diag / nsp_cross_sections / nsp_mean_profile of the state
    after the step it is stamped with."""
    st = stepper(nsp, "s2", nsp.NSP_FP64)
    st.set_state(0, init(nsp, "s2"))
    out = str(tmp_path / "o")
    run = nsp.Run(st, out_dir=out, dt_frc=0.05, dt_qcr=0.05, dt_mnp=0.05, rows_per_write=1, final_state=False)
    run.advance(11)  # ten additions of 0.005 fall short of 0.05: the first rows follow step 11
    d = st.diag(0)
    q, uu = st.cross_sections(0)
    prof = st.mean_profile(0)
    fr = read_rows(os.path.join(out, "io_friction.txt"))
    assert fr == ["%.8e  %.8e  %.8e" % (run.time(0)[0], d.u_centre, d.u_tau)]
    for name, v in (("io_qcross.txt", q), ("io_ucross.txt", uu), ("io_meanpr.txt", prof)):
        rows = read_rows(os.path.join(out, name))
        assert len(rows) == 2
        assert rows[1] == "".join("%.8e  " % x for x in [run.time(0)[0]] + list(v)), name
    run.close()
    assert not os.path.exists(os.path.join(out, "ur.bin"))
    st.close()


def ensemble(nsp, precision=0):
    NR, NT, NZ, LZ, Re, dt, _, _ = CFG["s2"]
    st = nsp.Stepper([nsp.make_params(NR, NT, NZ, Re, dt, LZ), nsp.make_params(NR, NT, NZ, Re * 1.1, dt, LZ)],
                     precision=precision)
    return st


def tree(d):
    out = {}
    for root, _, files in os.walk(d):
        for f in files:
            p = os.path.join(root, f)
            out[os.path.relpath(p, d)] = open(p, "rb").read()
    return out


@pytest.mark.parametrize("precision", [0, 1])
def test_resume_reproduces_uninterrupted_run(nsp, tmp_path, monkeypatch, precision):
    """A run interrupted after its step-20 checkpoint and resumed from it writes the
    same output files, byte for byte, and ends in the same state as a run that was
    never interrupted."""
    monkeypatch.setenv("NSP_AUTOTUNE", "0")  # the same block shapes in every context
    kw = dict(dt_frc=0.015, dt_qcr=0.035, dt_mnp=0.05, rows_per_write=3, ckpt_every=10, ckpt_keep=2)
    u0 = [init(nsp, "s2", m) for m in range(2)]

    st = ensemble(nsp, precision)
    for m in range(2):
        st.set_state(m, u0[m])
    with nsp.Run(st, out_dir=str(tmp_path / "a"), ckpt_dir=str(tmp_path / "ca"), **kw) as run:
        run.advance(30)
    ua = [np.stack(st.get_state(m)) for m in range(2)]
    st.close()
    assert sorted(os.listdir(tmp_path / "ca")) == ["step_0000000020", "step_0000000030"]  # ckpt_keep=2

    st = ensemble(nsp, precision)
    for m in range(2):
        st.set_state(m, u0[m])
    run = nsp.Run(st, out_dir=str(tmp_path / "b"), ckpt_dir=str(tmp_path / "cb"), **kw)
    run.advance(27)  # rows of steps 21..27 reach the files; the process "dies" here
    run.close()
    st.close()
    info, where = nsp.checkpoint_info(str(tmp_path / "cb"))
    assert info["step"] == 20 and where.endswith("step_0000000020")
    assert [m["dir"] for m in info["members"]] == ["member_0000", "member_0001"]

    st = ensemble(nsp, precision)  # a fresh context; the state comes from the checkpoint
    run = nsp.Run(st, out_dir=str(tmp_path / "b"), ckpt_dir=str(tmp_path / "cb"), resume=str(tmp_path / "cb"), **kw)
    assert run.time(1)[1] == 20
    run.advance(10)
    run.close()
    ub = [np.stack(st.get_state(m)) for m in range(2)]
    st.close()
    for m in range(2):
        assert np.array_equal(ua[m], ub[m]), m
    a, b = tree(str(tmp_path / "a")), tree(str(tmp_path / "b"))
    assert sorted(a) == sorted(b) and len(a) == 2 * 7
    for k in a:
        assert a[k] == b[k], k


def test_resume_rejects_other_parameters_and_corrupt_files(nsp, tmp_path):
    st = stepper(nsp, "s2", nsp.NSP_FP64)
    st.set_state(0, init(nsp, "s2"))
    ck = str(tmp_path / "ck")
    with nsp.Run(st, out_dir=None, ckpt_dir=ck) as run:
        run.advance(3)
        run.checkpoint()
    st.close()
    step = os.path.join(ck, "step_0000000003")
    assert sorted(os.listdir(step)) == ["checkpoint.json", "ur_s.bin", "ut_s.bin", "uz_s.bin"]
    # resuming from an older checkpoint abandons the later ones at its first checkpoint
    st = stepper(nsp, "s2", nsp.NSP_FP64)
    with nsp.Run(st, out_dir=None, resume=step, ckpt_dir=ck) as run:
        run.advance(3)
        run.checkpoint()  # step 6
    with nsp.Run(st, out_dir=None, resume=step, ckpt_dir=ck) as run:
        run.advance(1)
        run.checkpoint()  # step 4: step 6 is from the abandoned timeline
    assert sorted(os.listdir(ck)) == ["step_0000000003", "step_0000000004"]
    st.close()
    # a one-member checkpoint is a restart directory of the reference
    st = stepper(nsp, "s2", nsp.NSP_FP64)
    st.load(0, step)
    NR, NT, NZ, LZ, Re, dt, _, _ = CFG["s2"]
    other = nsp.Stepper([nsp.make_params(NR, NT, NZ, Re + 1.0, dt, LZ)])
    with pytest.raises(nsp.NspError) as e:
        nsp.Run(other, out_dir=None, resume=ck)
    assert e.value.code == nsp.NSP_ERR_ARG and "Re" in str(e.value)
    other.close()
    with open(os.path.join(step, "uz_s.bin"), "r+b") as fh:
        fh.seek(100)
        b = fh.read(1)
        fh.seek(100)
        fh.write(bytes([b[0] ^ 0x40]))
    with pytest.raises(nsp.NspError) as e:
        nsp.Run(st, out_dir=None, resume=step)
    assert e.value.code == nsp.NSP_ERR_IO and "checksum" in str(e.value)
    st.close()
