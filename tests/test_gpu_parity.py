"""GPU parity tests: the CUDA stepper (through the C ABI) against the oracle on the
same seeded inputs, and against the reference build's golden fixtures.

Tolerances: plain FP64 form, relative L2 <= 1e-12 against the oracle and the
reference (the spec gate); mixed form, relative L2 <= 1e-6 after the
stated number of steps.  Iteration counts per step must match exactly in FP64.
"""
import os

import numpy as np
import pytest

from conftest import PI2, ROOT, rel

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(ROOT, "tests", "golden")
CFG = {  # name: NR, NT, NZ, LZ, Re, dt, amplitude, seed
    "s1": (24, 8, 9, PI2, 1000.0, 0.01, 0.05, 11),
    "s2": (32, 16, 17, 2 * PI2, 3000.0, 0.005, 0.1, 12),
    "c0": (48, 32, 65, 2 * PI2, 2000.0, 0.01, 1e-3, 2000),
}


@pytest.fixture(scope="module")
def nsp():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import nspipe_gb300
    nspipe_gb300.lib()
    return nspipe_gb300


@pytest.fixture(scope="module")
def orc(oracle_lib):
    cache = {}

    def get(name):
        if name not in cache:
            NR, NT, NZ, LZ, Re, dt, _, _ = CFG[name]
            cache[name] = oracle_lib.Oracle(NR, NT, NZ, Re=Re, dt=dt, LZ=LZ)
        return cache[name]
    return get


def stepper(nsp, name, precision, members=1):
    NR, NT, NZ, LZ, Re, dt, _, _ = CFG[name]
    return nsp.Stepper([nsp.make_params(NR, NT, NZ, Re, dt, LZ) for _ in range(members)], precision=precision)


def init(nsp, name, m=0):
    NR, NT, NZ, LZ, Re, dt, amp, seed = CFG[name]
    return nsp.seeded_field(NR, NT, NZ, LZ, amp * (1 + 0.01 * m), seed + m)


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("name", ["s1", "c0"])
@pytest.mark.parametrize("kind", [0, 1, 2, 3])
def test_banded_solve_matches_oracle(nsp, orc, name, kind):
    import torch
    o = orc(name)
    st = stepper(nsp, name, nsp.NSP_FP64)
    rng = np.random.default_rng(kind)
    b = rng.standard_normal(o.shape) + 1j * rng.standard_normal(o.shape)
    sol = torch.zeros(o.shape, dtype=torch.complex128, device="cuda")
    st.lusolve(0, kind, dev(b), sol)
    ref = o.lusolve_p(b) if kind == 3 else o.lusolve_u(b, kind)
    assert rel(sol.cpu().numpy(), ref) < 1e-13
    st.close()


@pytest.mark.parametrize("name", ["s1", "c0"])
def test_double_float_solves_close_to_fp64(nsp, name):
    """The mixed form's corrector solves in double-float (FP32 pairs, kinds 4..7) against
    the FP64 solves of the same factors: relative L2 <= 1e-12 for the Helmholtz operators,
    <= 1e-9 for the pressure operator (condition numbers up to ~1e6 on its high-m lines)."""
    import torch
    st = stepper(nsp, name, nsp.NSP_MIXED)
    NR, NT, NZ = CFG[name][:3]
    rng = np.random.default_rng(7)
    for kind in range(4):
        b = rng.standard_normal((NR, NT, NZ)) + 1j * rng.standard_normal((NR, NT, NZ))
        x64 = torch.zeros(b.shape, dtype=torch.complex128, device="cuda")
        xdf = torch.zeros_like(x64)
        st.lusolve(0, kind, dev(b), x64)
        st.lusolve(0, kind + 4, dev(b), xdf)
        err = rel(xdf.cpu().numpy(), x64.cpu().numpy())
        assert err <= (1e-9 if kind == 3 else 1e-12), (kind, err)
    st.close()
    st = stepper(nsp, name, nsp.NSP_FP64)
    with pytest.raises(nsp.NspError):
        st.lusolve(0, 4, dev(np.zeros((NR, NT, NZ), complex)), torch.zeros((NR, NT, NZ), dtype=torch.complex128, device="cuda"))
    st.close()


@pytest.mark.parametrize("name", ["s1", "s2", "c0"])
@pytest.mark.parametrize("precision,tol", [(0, 1e-13), (1, 2e-6)])
def test_nonlinear_matches_oracle(nsp, orc, name, precision, tol):
    import torch
    o = orc(name)
    u0 = init(nsp, name)
    st = stepper(nsp, name, precision)
    n = [torch.zeros(o.shape, dtype=torch.complex128, device="cuda") for _ in range(3)]
    st.nonlinear(0, [dev(a) for a in u0], n)
    ref = o.nonlinear(u0)
    for c in range(3):
        assert rel(n[c].cpu().numpy(), ref[c]) < tol, c
    st.close()


@pytest.mark.parametrize("name,nsteps", [("s1", 5), ("s2", 5), ("c0", 3)])
def test_fp64_steps_match_oracle(nsp, orc, name, nsteps):
    o = orc(name)
    u0 = init(nsp, name)
    st = stepper(nsp, name, nsp.NSP_FP64)
    st.set_state(0, u0)
    it = st.step(nsteps)
    ug = np.stack(st.get_state(0))
    uo, ito, _ = o.step([a.copy() for a in u0], nsteps)
    assert list(it[:, 0]) == list(ito)
    assert rel(ug, np.stack(uo)) < 1e-12
    assert st.kernel_launches() > 0
    st.close()


def test_mixed_steps_close_to_fp64(nsp, orc):
    name, nsteps = "c0", 10
    o = orc(name)
    u0 = init(nsp, name)
    st = stepper(nsp, name, nsp.NSP_MIXED)
    st.set_state(0, u0)
    st.step(nsteps)
    ug = np.stack(st.get_state(0))
    uo, _, _ = o.step([a.copy() for a in u0], nsteps)
    assert rel(ug, np.stack(uo)) < 1e-6
    st.close()


def test_mixed_increment_correctors_follow_fp64(nsp):
    """The mixed form's correctors advance by increments (d_im/2) L(N_i - N_{i-1}), with
    the previous pass's N kept between passes.  With tol = 1e-14 every step takes
    several corrector passes, so the chain of increments runs past the first
    corrector; the states and iteration counts follow the FP64 form's full passes."""
    NR, NT, NZ, LZ, Re, dt, _, _ = CFG["c0"]
    res, its = {}, {}
    for prec in (nsp.NSP_FP64, nsp.NSP_MIXED):
        st = nsp.Stepper([nsp.make_params(NR, NT, NZ, Re, dt, LZ, tol=1e-14) for _ in range(2)], precision=prec)
        for m in range(2):
            st.set_state(m, init(nsp, "c0", m))
        its[prec] = st.step(20)
        res[prec] = [np.stack(st.get_state(m)) for m in range(2)]
        st.close()
    assert its[nsp.NSP_FP64].min() >= 2, its[nsp.NSP_FP64]
    assert np.array_equal(its[nsp.NSP_MIXED], its[nsp.NSP_FP64]), (its[nsp.NSP_MIXED], its[nsp.NSP_FP64])
    for m in range(2):
        assert rel(res[nsp.NSP_MIXED][m], res[nsp.NSP_FP64][m]) < 1e-6


def test_ensemble_members_independent(nsp):
    """A batched context gives each member the result of a single-member context."""
    name, M, nsteps = "s2", 5, 3
    batch = stepper(nsp, name, nsp.NSP_FP64, members=M)
    for m in range(M):
        batch.set_state(m, init(nsp, name, m))
    itb = batch.step(nsteps)
    for m in (0, 3):
        one = stepper(nsp, name, nsp.NSP_FP64)
        one.set_state(0, init(nsp, name, m))
        it1 = one.step(nsteps)
        assert list(it1[:, 0]) == list(itb[:, m])
        assert rel(np.stack(batch.get_state(m)), np.stack(one.get_state(0))) < 1e-14
        one.close()
    batch.close()


def test_uneven_batch(nsp, orc):
    """Members of different shapes and Re in one context each match their own oracle."""
    prm, states, names = [], [], ["s1", "s2", "s1"]
    for k, name in enumerate(names):
        NR, NT, NZ, LZ, Re, dt, _, _ = CFG[name]
        prm.append(nsp.make_params(NR, NT, NZ, Re * (1 + 0.1 * k), dt, LZ))
        states.append(init(nsp, name, k))
    st = nsp.Stepper(prm, precision=nsp.NSP_FP64)
    for m, u in enumerate(states):
        st.set_state(m, u)
    st.step(2)
    import oracle
    for m, name in enumerate(names):
        NR, NT, NZ, LZ, Re, dt, _, _ = CFG[name]
        o = oracle.Oracle(NR, NT, NZ, Re=Re * (1 + 0.1 * m), dt=dt, LZ=LZ)
        uo, _, _ = o.step([a.copy() for a in states[m]], 2)
        assert rel(np.stack(st.get_state(m)), np.stack(uo)) < 1e-12
    st.close()


def golden(name):
    path = os.path.join(GOLDEN, "ref_%s.npz" % name)
    if not os.path.exists(path):
        pytest.skip("golden fixture %s missing" % path)
    return np.load(path)


@pytest.mark.parametrize("name", ["s2"])
def test_fp64_matches_reference_build_full_field(nsp, name):
    g = golden(name)
    st = stepper(nsp, name, nsp.NSP_FP64)
    u0 = list(g["init"])
    st.set_state(0, u0)
    done = 0
    snaps = sorted(int(k.split("_")[1]) for k in g.files if k.startswith("u_"))
    iters = []
    for s in snaps:
        iters += list(st.step(s - done)[:, 0])
        done = s
        assert rel(np.stack(st.get_state(0)), g["u_%d" % s]) < 1e-12, s
    assert iters == list(g["iters"][:done])
    st.close()


def test_fp64_matches_reference_build_c0(nsp):
    from make_golden import projection_weights
    g = golden("c0")
    name = "c0"
    NR, NT, NZ, LZ, Re, dt, amp, seed = CFG[name]
    st = stepper(nsp, name, nsp.NSP_FP64)
    st.set_state(0, init(nsp, name))
    snaps = sorted(int(k.split("_")[1]) for k in g.files if k.startswith("mean_"))
    w = projection_weights(NR * NT * NZ, seed)
    done, iters = 0, []
    m_slots = [0, 1, 2, 3, 4, NT - 4, NT - 3, NT - 2, NT - 1]
    for s in snaps:
        iters += list(st.step(s - done)[:, 0])
        done = s
        u = st.get_state(0)
        low = np.stack([a[:, m_slots, :6] for a in u])
        assert rel(low, g["low_%d" % s]) < 1e-12, s
        assert rel(u[2][:, 0, 0], g["mean_%d" % s]) < 1e-12
        proj = np.stack([w @ a.reshape(-1) for a in u])
        assert np.abs(proj - g["proj_%d" % s]).max() <= 1e-12 * np.abs(g["proj_%d" % s]).max() * 10
    assert iters == list(g["iters"][:done])
    st.close()
