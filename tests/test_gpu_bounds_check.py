"""The bounds-checked build (libnspipe_gb300_bc.so, -DNSP_BOUNDS_CHECK): every global
index the step kernels compute is checked against the extent it addresses, and an
access outside it is skipped and recorded (nsp_bounds_report).  The reference's
kernels have no such checks; this build stands in for a memory checker.

The small and edge shapes (the s1 pipe, the smallest accepted grid, an odd azimuthal
length, run-time transform lengths, a tall radial grid), an uneven batch and the
tensor-core shape (NR=48, 32 x 64 modes) are stepped in both precisions through the
checked library in a child process (the normal library is loaded in this one), and
must record no violation while matching the oracle: FP64 relative L2 <= 1e-12 with the
oracle's iteration counts, mixed <= 1e-6.
"""
import json
import os
import subprocess
import sys

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

CHILD = r'''
import json, sys
import numpy as np
import nspipe_gb300 as nsp
import oracle
PI2 = nsp.PI2
assert nsp.LIB_PATH.endswith("_bc.so"), nsp.LIB_PATH
out = []

def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))

cases = [  # NR, NT, NZ, Re, dt, LZ, amplitude, seed, steps
    (24, 8, 9, 1000.0, 0.01, PI2, 0.05, 11, 3),
    (8, 4, 3, 1000.0, 0.005, PI2, 0.05, 7, 3),
    (24, 6, 5, 1000.0, 0.005, PI2, 0.05, 7, 3),
    (24, 12, 13, 1500.0, 0.01, PI2, 0.05, 31, 3),
    (256, 8, 9, 1000.0, 0.005, PI2, 0.05, 7, 2),
    (48, 32, 65, 2000.0, 0.01, 2 * PI2, 1e-3, 2000, 2),
]
for NR, NT, NZ, Re, dt, LZ, amp, seed, n in cases:
    u0 = nsp.seeded_field(NR, NT, NZ, LZ, amp, seed)
    o = oracle.Oracle(NR, NT, NZ, Re=Re, dt=dt, LZ=LZ)
    uo, ito, _ = o.step([a.copy() for a in u0], n)
    o.close()
    for prec in (nsp.NSP_FP64, nsp.NSP_MIXED):
        st = nsp.Stepper([nsp.make_params(NR, NT, NZ, Re, dt, LZ)] * 2, precision=prec)
        st.set_state(0, u0)
        st.set_state(1, u0)
        it = st.step(n)
        u = np.stack(st.get_state(0))
        st.step_host(1, st.pack([u0, u0]))  # the chunked host path too
        out.append(dict(shape=[NR, NT, NZ], prec=prec, err=rel(u, np.stack(uo)), iters=it[:, 0].tolist(),
                        oracle_iters=list(map(int, ito)), theta=st.describe()["groups"][0]["theta"],
                        bounds=list(st.bounds_report())))
        st.close()
# an uneven batch: three shapes, two Re values
prm = [nsp.make_params(24, 8, 9, 1000.0, 0.01, PI2), nsp.make_params(32, 16, 17, 3000.0, 0.01, 2 * PI2),
       nsp.make_params(24, 8, 9, 1200.0, 0.01, PI2), nsp.make_params(16, 12, 13, 900.0, 0.01, PI2)]
for prec in (nsp.NSP_FP64, nsp.NSP_MIXED):
    st = nsp.Stepper(prm, precision=prec)
    for m, p in enumerate(prm):
        st.set_state(m, nsp.seeded_field(p.NR, p.NT, p.NZ, p.LZ, 0.05, 40 + m))
    st.step(2)
    st.diag_all()
    out.append(dict(shape="uneven", prec=prec, err=0.0, iters=[], oracle_iters=[], theta="",
                    bounds=list(st.bounds_report())))
    st.close()
print("RESULT " + json.dumps(out))
'''


@pytest.fixture(scope="module")
def results():
    sys.path.insert(0, os.path.join(ROOT, "nspipe-gpu_gb300"))
    import build as nbuild
    lib = nbuild.build(bounds_check=True)
    env = dict(os.environ, NSP_LIBRARY=lib,
               PYTHONPATH=os.pathsep.join([os.path.join(ROOT, "nspipe-gpu_gb300"), os.path.join(ROOT, "oracle")]))
    p = subprocess.run([sys.executable, "-c", CHILD], env=env, capture_output=True, text=True, timeout=900)
    assert p.returncode == 0, p.stdout[-3000:] + p.stderr[-3000:]
    line = [x for x in p.stdout.splitlines() if x.startswith("RESULT ")][-1]
    return json.loads(line[len("RESULT "):])


def test_bounds_checked_build_records_no_violation(results):
    for r in results:
        assert r["bounds"][4] == 1, r  # the checked build was loaded
        assert r["bounds"][0] == 0, r  # (count, site, index, extent)


def test_bounds_checked_build_matches_oracle(results):
    for r in results:
        if r["shape"] == "uneven":
            continue
        if r["prec"] == 0:
            assert r["err"] < 1e-12, r
            assert r["iters"] == r["oracle_iters"], r
        else:
            assert r["err"] < 1e-6, r
    assert any(r["theta"] == "tcgen05-3xtf32" for r in results)
