"""CPU checks of the run driver's host logic (no GPU): the output cadence and the
header rows against the files the reference build wrote (tests/golden/io_s2/:
config s2, 100 steps of dt = 0.005, rows every 0.015 / 0.05 / 0.035 time units,
4 rows per write, so the reference kept only whole blocks of 4 rows), and the
checkpoint lookup and validation of nsp_checkpoint_info on hand-made checkpoints."""
import json
import os
import shutil

import numpy as np
import pytest

from conftest import PI2, ROOT

IO = os.path.join(ROOT, "tests", "golden", "io_s2")
NR, NT, NZ, LZ, DT, NSTEPS = 32, 16, 17, 2 * PI2, 0.005, 100
INTERVAL = {"io_friction.txt": 0.015, "io_qcross.txt": 0.05, "io_ucross.txt": 0.05, "io_meanpr.txt": 0.035}
ROWS_PER_WRITE = 4


@pytest.fixture(scope="module")
def nsp():
    import sys
    sys.path.insert(0, os.path.join(ROOT, "nspipe-gpu_gb300"))
    import build as nbuild
    nbuild.build()
    import nspipe_gb300
    return nspipe_gb300


def test_fixture_schedule_is_the_reference_build_schedule():
    import sys
    sys.path.insert(0, os.path.join(ROOT, "oracle", "ref"))
    import build_ref
    assert build_ref.IO_SCHEDULE == (INTERVAL["io_friction.txt"], INTERVAL["io_qcross.txt"],
                                     INTERVAL["io_meanpr.txt"], ROWS_PER_WRITE)
    assert build_ref.CONFIGS["s2"][:3] == (NR, NT, NZ) and build_ref.CONFIGS["s2"][5] == DT


def lines(name):
    with open(os.path.join(IO, name)) as fh:
        return fh.read().split("\n")[:-1]


@pytest.mark.parametrize("name", sorted(INTERVAL))
def test_cadence_matches_reference_rows(nsp, name):
    """Row times: steps where the accumulated dt reaches the interval (double additions,
    reset to 0 after a row) and t accumulated step by step, printed %.8e."""
    due, _ = nsp.output_schedule(DT, INTERVAL[name], NSTEPS)
    t, times = 0.0, []
    for j in range(NSTEPS):
        t += DT
        if due[j]:
            times.append("%.8e" % t)
    rows = lines(name)[0 if name == "io_friction.txt" else 1:]
    assert len(rows) == len(times) // ROWS_PER_WRITE * ROWS_PER_WRITE  # whole blocks only
    assert [r.split("  ")[0] for r in rows] == times[: len(rows)]
    if name.startswith("io_q"):  # ten additions of 0.005 fall short of 0.05: the first row is at step 11
        assert int(np.flatnonzero(due)[0]) == 10


def test_schedule_edge_cases(nsp):
    due, acc = nsp.output_schedule(0.5, 0.5, 4)
    assert due.tolist() == [True] * 4 and acc == 0.0
    due, acc = nsp.output_schedule(0.01, -1.0, 7)  # a negative interval: no rows
    assert not due.any()
    due, acc = nsp.output_schedule(0.25, 0.5, 3, acc=0.25)  # continues from a saved accumulator
    assert due.tolist() == [True, False, True] and acc == 0.0
    assert nsp.output_schedule(0.1, 0.0, 0) [0].size == 0


def test_header_rows_match_reference(oracle_lib):
    """Axial points z_n = LZ n / NZR of the cross-section files and the radial grid of
    io_meanpr.txt, each row led by 0, values as "%.8e  "."""
    NZR = 3 * (NZ - 1)
    z = [LZ * float(i) / float(NZR) for i in range(NZR)]
    row = "".join("%.8e  " % v for v in [0.0] + z)
    assert lines("io_qcross.txt")[0] == row
    assert lines("io_ucross.txt")[0] == row
    r = oracle_lib.Oracle(NR, NT, NZ, Re=3000.0, dt=DT, LZ=LZ).grid()["r"]
    assert lines("io_meanpr.txt")[0] == "".join("%.8e  " % v for v in [0.0] + list(r))
    assert all(len(x.split("  ")) == 3 for x in lines("io_friction.txt"))


def fnv1a64(data):
    h = 14695981039346656037
    for b in data:
        h = ((h ^ b) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return "%016x" % h


def make_checkpoint(root, step, members=1, size=48, sidecar=True, version=1):
    d = os.path.join(root, "step_%010d" % step)
    recs = []
    rng = np.random.default_rng(step)
    for m in range(members):
        sub = "." if members == 1 else "member_%04d" % m
        os.makedirs(os.path.join(d, sub), exist_ok=True)
        state = []
        for f in ("ur_s.bin", "ut_s.bin", "uz_s.bin"):
            data = rng.standard_normal(2 * size).tobytes()
            with open(os.path.join(d, sub, f), "wb") as fh:
                fh.write(data)
            state.append({"file": f, "bytes": len(data), "fnv1a64": fnv1a64(data)})
        recs.append({"dir": sub, "NR": 4, "NT": 4, "NZ": 3, "t": 0.1 * step, "step": step, "state": state,
                     "outputs": {}})
    if sidecar:
        with open(os.path.join(d, "checkpoint.json"), "w") as fh:
            json.dump({"format": "nspipe-gb300 checkpoint", "version": version, "precision": "fp64",
                       "step": step, "members": recs}, fh, indent=1)
    return d


def test_checkpoint_info_resolution_and_validation(nsp, tmp_path):
    root = str(tmp_path / "ckpt")
    d10 = make_checkpoint(root, 10, members=2)
    d20 = make_checkpoint(root, 20, members=2)
    make_checkpoint(root, 30, members=2, sidecar=False)  # interrupted while writing: skipped
    info, where = nsp.checkpoint_info(root)
    assert where == d20 and info["step"] == 20 and len(info["members"]) == 2
    info, where = nsp.checkpoint_info(d10)
    assert where == d10 and info["step"] == 10
    # a flipped byte, a short file, a foreign sidecar: NSP_ERR_IO
    f = os.path.join(d20, "member_0001", "ut_s.bin")
    data = bytearray(open(f, "rb").read())
    data[17] ^= 1
    open(f, "wb").write(bytes(data))
    with pytest.raises(nsp.NspError) as e:
        nsp.checkpoint_info(d20)
    assert e.value.code == nsp.NSP_ERR_IO
    open(f, "wb").write(bytes(data[:-16]))
    with pytest.raises(nsp.NspError):
        nsp.checkpoint_info(d20)
    d40 = make_checkpoint(root, 40, version=2)
    with pytest.raises(nsp.NspError):
        nsp.checkpoint_info(d40)
    shutil.rmtree(d40)
    with pytest.raises(nsp.NspError):
        nsp.checkpoint_info(str(tmp_path / "missing"))
    # a one-member checkpoint keeps the reference's restart names in the step directory itself
    d = make_checkpoint(str(tmp_path / "one"), 5)
    assert sorted(x for x in os.listdir(d) if x.endswith(".bin")) == ["ur_s.bin", "ut_s.bin", "uz_s.bin"]
    assert nsp.checkpoint_info(d)[1] == d


@pytest.mark.parametrize("text", ['{"format": "nspipe-gb300 checkpoint", "version": 1, "members": [',
                                  'not json at all',
                                  '{"format": "nspipe-gb300 checkpoint", "version": "1", "members": []}',
                                  '{"format": "nspipe-gb300 checkpoint", "version": 1, "members": [{"dir": "."}]}',
                                  '{"format": "nspipe-gb300 checkpoint", "version": 1, "members": [{"dir": ".", '
                                  '"state": [{"file": "ur_s.bin"}, {}, {}]}]}',
                                  '[1, 2, 3]', ''])
def test_checkpoint_info_rejects_malformed_sidecars(nsp, tmp_path, text):
    d = tmp_path / "step_0000000001"
    d.mkdir()
    (d / "checkpoint.json").write_text(text)
    with pytest.raises(nsp.NspError) as e:
        nsp.checkpoint_info(str(d))
    assert e.value.code == nsp.NSP_ERR_IO
    assert str(d) in nsp.host_error() or "checkpoint" in nsp.host_error()


def test_checkpoint_info_buffer_too_small(nsp, tmp_path):
    import ctypes
    d = make_checkpoint(str(tmp_path), 2)
    small = ctypes.create_string_buffer(8)
    rc = nsp.lib().nsp_checkpoint_info(d.encode(), small, len(small), None, 0)
    assert rc == nsp.NSP_ERR_ARG
