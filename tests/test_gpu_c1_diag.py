"""Diagnostics (divergence, mean profile, friction Reynolds number) against the
oracle, and the turbulent configuration NR=96 x 128 theta x 256 axial modes,
Re_b=5300, L=5piR, dt=0.002 R/U_b, seeded perturbation of amplitude 0.1, against
the reference build's golden fixture.

That configuration is numerically unstable: from about step 38 the corrector's
convergence measure grows ~4.7x per step in the reference, in the oracle and here
alike (a round-off-seeded instability; the reference hits maxit from step 50), so
round-off differences of 1e-15 are amplified by ~1e10 by step 50 (the oracle,
1.6e-15 from the reference at step 10, is 5.3e-5 from it at step 50).  Parity is
therefore gated on the stable stretch: relative L2 <= 1e-12 at steps 1 and 10, the
identical iteration sequence through step 50 (49 single corrector passes, then
maxit), and a wall divergence <= 1e-10.  The mixed form's FP32 noise seeds the same
instability ~1e7 times higher, so it is compared with the FP64 form over 10 steps.
"""
import numpy as np
import pytest

from conftest import PI2, rel
from test_gpu_parity import CFG, golden, init, nsp, orc, stepper  # noqa: F401  (fixtures)

pytestmark = pytest.mark.gpu

C1 = (96, 128, 257, 2.5 * PI2, 5300.0, 0.004, 0.1, 5300)  # NR, NT, NZ, LZ, Re, dt, amplitude, seed


def c1_stepper(nsp, precision):
    NR, NT, NZ, LZ, Re, dt, _, _ = C1
    return nsp.Stepper([nsp.make_params(NR, NT, NZ, Re, dt, LZ)], precision=precision)


def c1_init(nsp):
    NR, NT, NZ, LZ, Re, dt, amp, seed = C1
    return nsp.seeded_field(NR, NT, NZ, LZ, amp, seed)


def test_diag_matches_oracle(nsp, orc):
    name = "c0"
    o = orc(name)
    NR = CFG[name][0]
    Re = CFG[name][4]
    st = stepper(nsp, name, nsp.NSP_FP64)
    st.set_state(0, init(nsp, name))
    st.step(3)
    u = st.get_state(0)
    d = st.diag(0)
    div = o.divergence(*u)
    assert abs(d.div_max - np.abs(div[: NR - 1]).max()) <= 1e-10 * max(1.0, np.abs(div[: NR - 1]).max())
    assert abs(d.div_wall - np.abs(o.div_wall(*u)).max()) <= 1e-13
    assert d.div_wall <= 1e-10
    prof = st.mean_profile(0)
    assert np.array_equal(prof, u[2][:, 0, 0].real)
    ucen, utau = o.friction(u[2])
    assert abs(d.u_centre - ucen) <= 1e-13 * abs(ucen)
    assert abs(d.u_tau - utau) <= 1e-13 * abs(utau)
    assert abs(d.re_tau - Re * d.u_tau) <= 1e-12 * d.re_tau
    st.close()


def test_cross_sections_match_oracle(nsp, orc):
    """q and u cross-section rows (the reference's wrt_qcr / wrt_ucr data) against the
    oracle's physical-space levels: r-weighted theta means of u_r^2 + u_theta^2, u_z^2."""
    name = "c0"
    o = orc(name)
    NR = CFG[name][0]
    st = stepper(nsp, name, nsp.NSP_FP64)
    st.set_state(0, init(nsp, name))
    st.step(2)
    u = st.get_state(0)
    q, uu = st.cross_sections(0)
    rdr = o.grid()["rdr"]
    q_ref, u_ref = np.zeros_like(q), np.zeros_like(uu)
    for i in range(NR):
        pr, pt, pz = (o.level_backward(a[i]) for a in u)  # [NTP][NZR] physical values
        q_ref += rdr[i] * (pr ** 2 + pt ** 2).mean(axis=0)
        u_ref += rdr[i] * (pz ** 2).mean(axis=0)
    assert rel(q, q_ref) < 1e-12
    assert rel(uu, u_ref) < 1e-12
    st.close()


def _low(u, NT):
    m_slots = [0, 1, 2, 3, 4, NT - 4, NT - 3, NT - 2, NT - 1]
    return np.stack([a[:, m_slots, :6] for a in u])


def test_fp64_matches_reference_build_c1(nsp):
    from make_golden import projection_weights
    g = golden("c1")
    NR, NT, NZ = C1[:3]
    st = c1_stepper(nsp, nsp.NSP_FP64)
    st.set_state(0, c1_init(nsp))
    w = projection_weights(NR * NT * NZ, C1[7])
    done, iters = 0, []
    for s in (1, 10):
        iters += list(st.step(s - done)[:, 0])
        done = s
        u = st.get_state(0)
        assert rel(_low(u, NT), g["low_%d" % s]) < 1e-12, s
        assert rel(u[2][:, 0, 0], g["mean_%d" % s]) < 1e-12, s
        proj = np.stack([w @ a.reshape(-1) for a in u])
        assert np.abs(proj - g["proj_%d" % s]).max() <= 1e-11 * np.abs(g["proj_%d" % s]).max(), s
        norms = np.array([np.linalg.norm(a) for a in u])
        assert np.all(np.abs(norms - g["norm_%d" % s]) <= 1e-12 * g["norm_%d" % s]), s
        d = st.diag(0)
        assert d.div_wall <= 1e-10, s
        assert d.status == 0
    iters += list(st.step(50 - done)[:, 0])
    assert iters == list(g["iters"][:50])
    assert iters[-1] == 10  # the first step of the instability reaches maxit, as in the reference
    st.close()


def test_mixed_close_to_fp64_c1(nsp):
    u0 = c1_init(nsp)
    res, dg = {}, {}
    for prec in (nsp.NSP_FP64, nsp.NSP_MIXED):
        st = c1_stepper(nsp, prec)
        st.set_state(0, u0)
        st.step(10)
        res[prec] = np.stack(st.get_state(0))
        dg[prec] = st.diag(0)
        st.close()
    assert rel(res[nsp.NSP_MIXED], res[nsp.NSP_FP64]) < 1e-6
    assert rel(res[nsp.NSP_MIXED][2, :, 0, 0], res[nsp.NSP_FP64][2, :, 0, 0]) < 1e-4
    assert dg[nsp.NSP_MIXED].div_wall <= 1e-10
    assert abs(dg[nsp.NSP_MIXED].re_tau - dg[nsp.NSP_FP64].re_tau) <= 1e-4 * dg[nsp.NSP_FP64].re_tau
