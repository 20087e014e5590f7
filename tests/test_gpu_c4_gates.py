"""Accuracy gates of the uneven mixed batch: three resolutions (NR=48 x 32 x 64 modes,
NR=64 x 48 x 128, NR=96 x 96 x 192), Re spread within each group, dt = 0.003 R/U_b
(0.006 code units), L = 4 pi R, seeded perturbations of amplitude 0.05.

  * The plain FP64 form against the reference build (tests/golden/ref_c4b.npz and
    ref_c4c.npz: one member of the NR=64 and of the NR=96 group, 100 steps): relative
    L2 <= 1e-12 of the low-mode block, the mean profile, the per-component norms and the
    seeded projections at steps 1, 10, 50 and 100, the reference's iteration counts,
    wall divergence <= 1e-10.
  * The mixed form against the FP64 form, both ends of each group's Re range, in one
    uneven context per form, at 50 and 100 steps: velocity relative L2 <= 1e-6 and
    the mean profile <= 1e-4 (the spec gate), Re_tau <= 1e-4, and the error of
    the perturbation alone (the mean mode (m, k_z) = (0, 0) removed, the part of the
    field that carries the flow's dynamics) <= 1e-6.
"""
import numpy as np
import pytest

from conftest import PI2, rel
from test_gpu_parity import golden, nsp  # noqa: F401  (fixtures)

pytestmark = pytest.mark.gpu

C4 = {  # name: NR, NT, NZ, LZ, Re, dt, amplitude, seed (the reference fixtures)
    "c4b": (64, 48, 129, 2 * PI2, 2700.0, 0.006, 0.05, 4100),
    "c4c": (96, 96, 193, 2 * PI2, 3500.0, 0.006, 0.05, 4200),
}
GROUPS = [(48, 32, 65, 2000.0, 2400.0), (64, 48, 129, 2400.0, 3000.0), (96, 96, 193, 3000.0, 4000.0)]


def perturbation(u):
    """The field without its mean mode (m, k_z) = (0, 0)."""
    v = np.array(u, copy=True)
    v[:, :, 0, 0] = 0
    return v


@pytest.mark.parametrize("name", ["c4b", "c4c"])
def test_c4_fp64_matches_reference_build(nsp, name):
    from make_golden import projection_weights
    g = golden(name)
    NR, NT, NZ, LZ, Re, dt, amp, seed = C4[name]
    st = nsp.Stepper(nsp.make_params(NR, NT, NZ, Re, dt, LZ), precision=nsp.NSP_FP64)
    st.set_state(0, nsp.seeded_field(NR, NT, NZ, LZ, amp, seed))
    w = projection_weights(NR * NT * NZ, seed)
    slots = [0, 1, 2, 3, 4, NT - 4, NT - 3, NT - 2, NT - 1]
    done, iters = 0, []
    for s in (1, 10, 50, 100):
        iters += list(st.step(s - done)[:, 0])
        done = s
        u = st.get_state(0)
        assert rel(np.stack([a[:, slots, :6] for a in u]), g["low_%d" % s]) < 1e-12, s
        assert rel(u[2][:, 0, 0], g["mean_%d" % s]) < 1e-12, s
        proj = np.stack([w @ a.reshape(-1) for a in u])
        assert np.abs(proj - g["proj_%d" % s]).max() <= 1e-11 * np.abs(g["proj_%d" % s]).max(), s
        norms = np.array([np.linalg.norm(a) for a in u])
        assert np.all(np.abs(norms - g["norm_%d" % s]) <= 1e-12 * g["norm_%d" % s]), s
        assert st.diag(0).div_wall <= 1e-10, s
    assert iters == list(g["iters"][:done])
    st.close()


def test_c4_mixed_form_gate(nsp):
    prm, fields = [], []
    for gi, (nr, nt, nz, lo, hi) in enumerate(GROUPS):
        for j, re in enumerate((lo, hi)):
            prm.append(nsp.make_params(nr, nt, nz, re, 0.006, 2 * PI2))
            fields.append(nsp.seeded_field(nr, nt, nz, 2 * PI2, 0.05, 4300 + 10 * gi + j))
    res = {}
    for prec in (nsp.NSP_FP64, nsp.NSP_MIXED):
        st = nsp.Stepper(prm, precision=prec)
        for m, f in enumerate(fields):
            st.set_state(m, f)
        done = 0
        for s in (50, 100):
            st.step(s - done)
            done = s
            res[prec, s] = ([np.stack(st.get_state(m)) for m in range(len(prm))], st.diag_all())
        if prec == nsp.NSP_MIXED:
            assert [g["theta"] for g in st.describe()["groups"]] == ["tcgen05-3xtf32", "fft-fp32", "fft-fp32"]
        st.close()
    for s in (50, 100):
        for m in range(len(prm)):
            a, b = res[nsp.NSP_FP64, s][0][m], res[nsp.NSP_MIXED, s][0][m]
            da, db = res[nsp.NSP_FP64, s][1][m], res[nsp.NSP_MIXED, s][1][m]
            tag = (s, m, prm[m].NR, prm[m].Re)
            assert rel(b, a) <= 1e-6, tag
            assert rel(perturbation(b), perturbation(a)) <= 1e-6, tag
            assert rel(b[2, :, 0, 0], a[2, :, 0, 0]) <= 1e-4, tag
            assert abs(db.re_tau - da.re_tau) <= 1e-4 * da.re_tau, tag
            assert db.div_wall <= 1e-10 and db.status == 0, tag
