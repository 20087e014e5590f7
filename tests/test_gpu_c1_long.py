"""A long run of the turbulent shape: NR=96 x 128 theta x 256 axial modes, Re_b=5300,
L=5piR, seeded perturbation of amplitude 0.1, with half the specified time step
(dt = 0.001 R/U_b, 0.002 code units; at the specified 0.002 R/U_b the run is unstable in
the reference build as well), 500 steps against the reference build's fixture
(tests/golden/ref_c1h.npz: low-mode block, mean profile, norms and projections at steps
1, 10, 50, 100, 200, 300, 400, 500, and every step's iteration count).

The flow goes chaotic from about step 150: an FP64 run whose initial state is changed by
1e-13 (relative, per coefficient) ends 1e-3 away at step 500, so trajectories are
compared while they are predictable and statistics after that:

  * FP64 form: relative L2 <= 1e-12 of every fixture quantity through step 100; the
    reference's iteration count at every one of the 500 steps; wall divergence <= 1e-10
    at every snapshot; the mean profile and Re_tau at step 500 within 1e-5 of the
    reference build's (measured 2.5e-7 and below).
  * Mixed form: relative L2 <= 1e-6 of the FP64 form's state at step 50; at steps 100 and
    500 the mean profile and Re_tau within 1e-4 of the FP64 form's.
"""
import numpy as np
import pytest

from conftest import PI2, rel
from test_gpu_parity import golden, nsp  # noqa: F401  (fixtures)

pytestmark = pytest.mark.gpu

C1H = (96, 128, 257, 2.5 * PI2, 5300.0, 0.002, 0.1, 5300)  # NR, NT, NZ, LZ, Re, dt, amplitude, seed
SNAPS = (1, 10, 50, 100, 200, 300, 400, 500)


def run(nsp, precision):
    """Steps to every snapshot; returns {step: (state or None, mean profile, diag)} (the
    state kept through step 100 only) and the iteration counts."""
    NR, NT, NZ, LZ, Re, dt, amp, seed = C1H
    st = nsp.Stepper(nsp.make_params(NR, NT, NZ, Re, dt, LZ), precision=precision)
    st.set_state(0, nsp.seeded_field(NR, NT, NZ, LZ, amp, seed))
    out, iters, done = {}, [], 0
    for s in SNAPS:
        iters += list(st.step(s - done)[:, 0])
        done = s
        u = st.get_state(0)
        out[s] = (u if s <= 100 else None, u[2][:, 0, 0].copy(), st.diag(0))
    st.close()
    return out, iters


def re_tau_of_profile(nsp, mean):
    """Re_tau of a mean axial-velocity profile, by the product's own friction rule."""
    NR, NT, NZ, LZ, Re, dt, _, _ = C1H
    st = nsp.Stepper(nsp.make_params(NR, NT, NZ, Re, dt, LZ), precision=nsp.NSP_FP64)
    u = [np.zeros((NR, NT, NZ), np.complex128) for _ in range(3)]
    u[2][:, 0, 0] = mean
    st.set_state(0, u)
    t = st.diag(0).re_tau
    st.close()
    return t


@pytest.fixture(scope="module")
def fp64_run(nsp):
    return run(nsp, nsp.NSP_FP64)


def test_c1h_fp64_matches_reference_build(nsp, fp64_run):
    from make_golden import projection_weights
    g = golden("c1h")
    NR, NT, NZ, _, _, _, _, seed = C1H
    out, iters = fp64_run
    assert iters == list(g["iters"][:500])
    w = projection_weights(NR * NT * NZ, seed)
    slots = [0, 1, 2, 3, 4, NT - 4, NT - 3, NT - 2, NT - 1]
    for s in SNAPS:
        u, _, d = out[s]
        assert d.div_wall <= 1e-10 and d.status == 0, s
        if s > 100:
            continue
        assert rel(np.stack([a[:, slots, :6] for a in u]), g["low_%d" % s]) < 1e-12, s
        assert rel(u[2][:, 0, 0], g["mean_%d" % s]) < 1e-12, s
        proj = np.stack([w @ a.reshape(-1) for a in u])
        assert np.abs(proj - g["proj_%d" % s]).max() <= 1e-11 * np.abs(g["proj_%d" % s]).max(), s
        norms = np.array([np.linalg.norm(a) for a in u])
        assert np.all(np.abs(norms - g["norm_%d" % s]) <= 1e-12 * g["norm_%d" % s]), s
    _, mean, d = out[500]
    assert rel(mean, g["mean_500"]) <= 1e-5
    assert abs(d.re_tau - re_tau_of_profile(nsp, g["mean_500"])) <= 1e-5 * d.re_tau


def test_c1h_mixed_form_against_fp64(nsp, fp64_run):
    ref, _ = fp64_run
    out, iters = run(nsp, nsp.NSP_MIXED)
    assert max(iters) <= 3
    assert rel(np.stack(out[50][0]), np.stack(ref[50][0])) <= 1e-6
    for s in (100, 500):
        _, mean, d = out[s]
        _, mean_ref, da = ref[s]
        assert rel(mean, mean_ref) <= 1e-4, s
        assert abs(d.re_tau - da.re_tau) <= 1e-4 * da.re_tau, s
        assert d.div_wall <= 1e-10 and d.status == 0, s
