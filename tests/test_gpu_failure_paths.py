"""Failure paths of the step, made on the host (no GPU fault): a member whose input holds
a NaN or an Inf, and corrector loops that stop at maxit without converging.

The reference exits on CUDA errors (head.h:64-70) and says nothing when its corrector
loop stops at maxit (mod_integrate.cu:120); a NaN in its state simply propagates.
Here a non-finite member is reported as NSP_ERR_NONFINITE by both stepping entry
points while the other members advance exactly as they would without it, and a step
that stops at maxit with err > tol is counted per member (nsp_diag) and, in strict
mode, reported as NSP_ERR_MAXIT, with the states unchanged from a non-strict run.
"""
import numpy as np
import pytest

from conftest import rel
from test_gpu_parity import CFG, init, nsp, orc, stepper  # noqa: F401  (fixtures)

pytestmark = pytest.mark.gpu


def spoiled(u, value):
    """A copy of the field u with one coefficient of u_theta replaced by value."""
    v = [a.copy() for a in u]
    v[1][5, 3, 2] = complex(value, 0.0)
    return v


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("value", [np.nan, np.inf])
def test_nonfinite_member_reported_others_unaffected(nsp, precision, value):
    name, n = "s2", 3
    u = [init(nsp, name, m) for m in range(n)]
    clean = stepper(nsp, name, precision, members=n)
    for m in range(n):
        clean.set_state(m, u[m])
    it_clean = clean.step(2)
    want = [np.stack(clean.get_state(m)) for m in range(n)]
    clean.close()

    st = stepper(nsp, name, precision, members=n)
    for m in range(n):
        st.set_state(m, spoiled(u[m], value) if m == 1 else u[m])
    with pytest.raises(nsp.NspError) as e:
        st.step(2)
    assert e.value.code == nsp.NSP_ERR_NONFINITE and "member 1" in str(e.value)
    assert st.diag(1).status == nsp.NSP_ERR_NONFINITE
    it = st.step(0, check=False)  # (no steps: the status stays)
    assert it.shape == (0, n)
    for m in (0, 2):
        assert st.diag(m).status == nsp.NSP_OK
        assert np.array_equal(np.stack(st.get_state(m)), want[m]), m
    # a clean state clears the member's status; the context steps on normally
    st.set_state(1, u[1])
    st.step(1)
    assert all(d.status == nsp.NSP_OK for d in st.diag_all())
    st.close()
    assert it_clean.shape == (2, n)


@pytest.mark.parametrize("precision", [0, 1])
def test_nonfinite_member_through_step_host(nsp, precision):
    name, n = "s2", 4
    u = [init(nsp, name, m) for m in range(n)]
    st = stepper(nsp, name, precision, members=n)
    want, _ = st.step_host(2, st.pack(u))
    bad = st.pack([spoiled(u[m], np.nan) if m == 2 else u[m] for m in range(n)])
    out = np.zeros_like(bad)
    with pytest.raises(nsp.NspError) as e:
        st.step_host(2, bad, out)
    assert e.value.code == nsp.NSP_ERR_NONFINITE and "member 2" in str(e.value)
    got, exp = st.unpack(out), st.unpack(want)
    for m in (0, 1, 3):
        for c in range(3):
            assert np.array_equal(got[m][c], exp[m][c]), (m, c)
    assert not np.all(np.isfinite(np.stack(got[2])))
    # the next call from clean states succeeds and repeats the first result
    again, _ = st.step_host(2, st.pack(u))
    assert np.array_equal(again, want)
    st.close()


def test_maxit_counted_and_strict_mode_reports_it(nsp, orc):
    """tol = 1e-30 is never met: every step stops at maxit = 3.  The states and
    iteration counts are the oracle's with the same maxit / tol (FP64 form, 1e-12)."""
    name, nsteps, maxit = "s2", 3, 3
    NR, NT, NZ, LZ, Re, dt, _, _ = CFG[name]
    prm = nsp.make_params(NR, NT, NZ, Re, dt, LZ, maxit=maxit, tol=1e-30)
    u0 = init(nsp, name)
    st = nsp.Stepper(prm, precision=nsp.NSP_FP64)
    st.set_state(0, u0)
    it = st.step(nsteps)
    assert list(it[:, 0]) == [maxit] * nsteps
    assert st.diag(0).unconverged_steps == nsteps
    assert st.diag_all()[0].unconverged_steps == nsteps
    lax = np.stack(st.get_state(0))

    import oracle
    o = oracle.Oracle(NR, NT, NZ, Re=Re, dt=dt, LZ=LZ, maxit=maxit, tol=1e-30)
    uo, ito, _ = o.step([a.copy() for a in u0], nsteps)
    o.close()
    assert list(ito) == [maxit] * nsteps
    assert rel(lax, np.stack(uo)) < 1e-12

    st.set_strict(True)
    st.set_state(0, u0)
    with pytest.raises(nsp.NspError) as e:
        st.step(nsteps)
    assert e.value.code == nsp.NSP_ERR_MAXIT and "maxit = 3" in str(e.value)
    assert np.array_equal(np.stack(st.get_state(0)), lax)
    with pytest.raises(nsp.NspError) as e:
        st.step_host(nsteps, st.pack([u0]))
    assert e.value.code == nsp.NSP_ERR_MAXIT
    st.close()

    # a converging run counts nothing, strict or not
    ok = stepper(nsp, name, nsp.NSP_FP64)
    ok.set_strict(True)
    ok.set_state(0, u0)
    ok.step(nsteps)
    assert ok.diag(0).unconverged_steps == 0
    ok.close()


def test_maxit_ends_a_strict_run_after_its_rows(nsp, tmp_path):
    name = "s2"
    NR, NT, NZ, LZ, Re, dt, _, _ = CFG[name]
    st = nsp.Stepper(nsp.make_params(NR, NT, NZ, Re, dt, LZ, maxit=2, tol=1e-30), precision=nsp.NSP_FP64)
    st.set_state(0, init(nsp, name))
    st.set_strict(True)
    run = nsp.Run(st, out_dir=str(tmp_path), dt_frc=2 * dt, dt_qcr=-1, dt_mnp=-1, final_state=False)
    with pytest.raises(nsp.NspError) as e:
        run.advance(6)
    assert e.value.code == nsp.NSP_ERR_MAXIT
    rows = open(tmp_path / "io_friction.txt").read().split("\n")
    assert len([r for r in rows if r.strip()]) == 1  # the row due after the first chunk
    assert run.time(0)[1] == 2
    run.close()
    st.close()
