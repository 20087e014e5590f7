"""Uneven batches: members of several shapes and Reynolds numbers in one context.
Members sharing a shape form one group (one launch per stage) whatever their Re;
each distinct Re is an operator parameter set of the group; the groups run as
parallel branches of the step graph.  Every member must match its own oracle."""
import numpy as np
import pytest

from conftest import rel
from test_gpu_parity import CFG, dev, init, nsp, orc  # noqa: F401  (fixtures)

pytestmark = pytest.mark.gpu

NAMES = ["s1", "s2", "s1", "s1", "s2"]
SCALE = [1.0, 1.0, 1.2, 1.0, 1.3]  # Re multipliers: s1 has two sets (1.0 twice, 1.2), s2 two sets


def batch(nsp, precision):
    prm, states = [], []
    for k, name in enumerate(NAMES):
        NR, NT, NZ, LZ, Re, dt, _, _ = CFG[name]
        prm.append(nsp.make_params(NR, NT, NZ, Re * SCALE[k], dt, LZ))
        states.append(init(nsp, name, k))
    st = nsp.Stepper(prm, precision=precision)
    for m, u in enumerate(states):
        st.set_state(m, u)
    return st, states


def member_oracle(name, k):
    import oracle
    NR, NT, NZ, LZ, Re, dt, _, _ = CFG[name]
    return oracle.Oracle(NR, NT, NZ, Re=Re * SCALE[k], dt=dt, LZ=LZ)


def test_uneven_groups_sets_and_parity(nsp):
    st, states = batch(nsp, nsp.NSP_FP64)
    d = st.describe()
    assert [g["members"] for g in d["groups"]] == [3, 2]
    its = st.step(3)
    for m, name in enumerate(NAMES):
        o = member_oracle(name, m)
        uo, ito, _ = o.step([a.copy() for a in states[m]], 3)
        assert rel(np.stack(st.get_state(m)), np.stack(uo)) < 1e-12, m
        assert list(its[:, m]) == list(ito), m
        o.close()
    st.close()


def test_uneven_single_member_calls_use_member_operators(nsp):
    import torch
    st, states = batch(nsp, nsp.NSP_FP64)
    m, name = 2, "s1"  # second parameter set of the s1 group
    o = member_oracle(name, m)
    shape = o.shape
    rng = np.random.default_rng(5)
    b = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    sol = torch.zeros(shape, dtype=torch.complex128, device="cuda")
    st.lusolve(m, 0, dev(b), sol)
    assert rel(sol.cpu().numpy(), o.lusolve_u(b, 0)) < 1e-13
    n = [torch.zeros(shape, dtype=torch.complex128, device="cuda") for _ in range(3)]
    st.nonlinear(m, [dev(a) for a in states[m]], n)
    ref = o.nonlinear(states[m])
    for c in range(3):
        assert rel(n[c].cpu().numpy(), ref[c]) < 1e-13, c
    o.close()
    st.close()


def test_uneven_mixed_close_to_fp64(nsp):
    res = {}
    for prec in (nsp.NSP_FP64, nsp.NSP_MIXED):
        st, _ = batch(nsp, prec)
        st.step(5)
        res[prec] = [np.stack(st.get_state(m)) for m in range(len(NAMES))]
        st.close()
    for m in range(len(NAMES)):
        assert rel(res[nsp.NSP_MIXED][m], res[nsp.NSP_FP64][m]) < 1e-6, m


def test_all_member_transfers_interleaved_groups(nsp):
    """NSP_ALL_MEMBERS transfers (one pitched copy per component per run of members
    stored together) on members whose groups interleave in user order: the arrays
    hold each member's component back to back in user order, both directions."""
    from conftest import PI2
    shapes = [(24, 8, 9), (32, 16, 17), (24, 8, 9), (24, 8, 9), (32, 16, 17)]
    st = nsp.Stepper([nsp.make_params(*s, 1000.0 + 50 * k, 0.005, PI2) for k, s in enumerate(shapes)])
    fields = [nsp.seeded_field(*s, PI2, 0.05, 60 + k) for k, s in enumerate(shapes)]
    flat = [np.concatenate([f[c].reshape(-1) for f in fields]) for c in range(3)]
    st.set_states_all(flat)
    for k, f in enumerate(fields):
        got = st.get_state(k)
        for c in range(3):
            assert np.array_equal(got[c], f[c]), (k, c)
    st.step(2)
    back = st.get_states_all()
    off = 0
    for k, s in enumerate(shapes):
        n = int(np.prod(s))
        one = st.get_state(k)
        for c in range(3):
            assert np.array_equal(back[c][off:off + n].reshape(s), one[c]), (k, c)
        off += n
    st.close()


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("nsteps", [1, 3])
def test_step_host_matches_step(nsp, precision, nsteps):
    """nsp_step_host (members stepped in chunks, copies overlapping compute) gives the
    states and iteration counts of set_states_all + step + get_states_all bit for bit,
    on 17 members of two interleaved shapes (chunks straddle the groups), and leaves
    the context ready for further steps."""
    from conftest import PI2
    shapes = [(24, 8, 9) if k % 3 else (32, 16, 17) for k in range(17)]
    prm = [nsp.make_params(*s, 1000.0 + 10 * k, 0.005, PI2) for k, s in enumerate(shapes)]
    fields = [nsp.seeded_field(*s, PI2, 0.05, 80 + k) for k, s in enumerate(shapes)]
    flat = [np.concatenate([f[c].reshape(-1) for f in fields]) for c in range(3)]
    a = nsp.Stepper(prm, precision=precision)
    a.set_states_all(flat)
    it_a = a.step(nsteps)
    out_a = a.get_states_all()
    b = nsp.Stepper(prm, precision=precision)
    out_b, it_b = b.step_host(nsteps, b.pack(fields))
    for m, f in enumerate(b.unpack(out_b)):  # member-major out vs component-major out_a
        n = f[0].size
        off = sum(int(np.prod(s)) for s in shapes[:m])
        for c in range(3):
            assert np.array_equal(f[c].reshape(-1), out_a[c][off:off + n]), (m, c)
    assert np.array_equal(it_a, it_b)
    same, _ = b.step_host(0, out_b)  # zero steps: in -> state -> out
    assert np.array_equal(same, out_b)
    a.step(2)
    b.step(2)
    for c, (x, y) in enumerate(zip(a.get_states_all(), b.get_states_all())):
        assert np.array_equal(x, y), c
    a.close()
    b.close()


@pytest.mark.parametrize("name", ["s1", "s2", "c0"])
def test_mirror_refresh_matches_linear_pass(nsp, name):
    """Mixed form: the FP32 mirror of the state and its d_r are kept current by the
    linear pass between steps and rebuilt by their own kernel after the state is
    written from outside (NR = 24, 32, 48: one, two partial and two full level tiles).
    Both must give the same bits, so stepping on and re-setting the same state before
    the next step agree exactly."""
    NR, NT, NZ, LZ, Re, dt, _, _ = CFG[name]
    prm = [nsp.make_params(NR, NT, NZ, Re * (1 + 0.1 * k), dt, LZ) for k in range(3)]
    u0 = [init(nsp, name, k) for k in range(3)]
    a = nsp.Stepper(prm, precision=nsp.NSP_MIXED)
    b = nsp.Stepper(prm, precision=nsp.NSP_MIXED)
    for k in range(3):
        a.set_state(k, u0[k])
        b.set_state(k, u0[k])
    a.step(3)
    b.step(1)
    for k in range(3):
        b.set_state(k, b.get_state(k))
    b.step(2)
    for k in range(3):
        assert np.array_equal(np.stack(a.get_state(k)), np.stack(b.get_state(k))), k
    a.close()
    b.close()


def test_mirror_refreshed_after_device_writes(nsp):
    """A state written device to device (nsp_set_state_device) also marks the FP32
    mirror stale: stepping on from it equals stepping a context that never had the
    member's other state."""
    import torch
    NR, NT, NZ, LZ, Re, dt, _, _ = CFG["c0"]
    prm = [nsp.make_params(NR, NT, NZ, Re, dt, LZ) for _ in range(2)]
    u0, u1 = init(nsp, "c0", 0), init(nsp, "c0", 1)
    a = nsp.Stepper(prm, precision=nsp.NSP_MIXED)
    b = nsp.Stepper(prm, precision=nsp.NSP_MIXED)
    for m in range(2):
        a.set_state(m, u0)
        b.set_state(m, u1 if m == 1 else u0)
    a.step(1)  # a's mirror of member 1 is now the one the linear pass kept (u0's successor)
    d = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in u1]
    a.set_state_device(1, *d)
    a.step(2)
    b.step(2)
    assert np.array_equal(np.stack(a.get_state(1)), np.stack(b.get_state(1)))
    a.close()
    b.close()


@pytest.mark.parametrize("weights", ["3:1", "1:0:2", "5", "2:3:3:2:9"])
def test_step_host_chunk_weights(nsp, monkeypatch, weights):
    """nsp_step_host's member chunks (the NSP_HOST_CHUNKS override: equal chunks or a
    weight pattern; chunks that round to no member are dropped) change only the
    overlap of copies and compute, never the results."""
    from conftest import PI2
    shapes = [(24, 8, 9) if k % 3 else (32, 16, 17) for k in range(11)]
    prm = [nsp.make_params(*s, 1000.0 + 10 * k, 0.005, PI2) for k, s in enumerate(shapes)]
    fields = [nsp.seeded_field(*s, PI2, 0.05, 90 + k) for k, s in enumerate(shapes)]
    ref = nsp.Stepper(prm, precision=nsp.NSP_MIXED)
    out_ref, it_ref = ref.step_host(2, ref.pack(fields))
    ref.close()
    monkeypatch.setenv("NSP_HOST_CHUNKS", weights)
    st = nsp.Stepper(prm, precision=nsp.NSP_MIXED)
    out, it = st.step_host(2, st.pack(fields))
    st.close()
    assert np.array_equal(out, out_ref) and np.array_equal(it, it_ref)


def test_batched_diagnostics_equal_per_member(nsp):
    """nsp_diag_all / nsp_mean_profile_all / nsp_cross_sections_all (one launch per group
    and kernel) give each member's per-member values bit for bit."""
    from conftest import PI2
    shapes = [(24, 8, 9), (32, 16, 17), (24, 8, 9), (32, 16, 17), (32, 16, 17)]
    st = nsp.Stepper([nsp.make_params(*s, 1200.0 + 100 * k, 0.005, PI2) for k, s in enumerate(shapes)])
    for k, s in enumerate(shapes):
        st.set_state(k, nsp.seeded_field(*s, PI2, 0.05, 90 + k))
    st.step(3)
    d_all = st.diag_all()
    p_all = st.mean_profile_all()
    q_all, u_all = st.cross_sections_all()
    for m in range(len(shapes)):
        d = st.diag(m)
        for f, _ in nsp.NspDiag._fields_:
            assert getattr(d_all[m], f) == getattr(d, f), (m, f)
        assert np.array_equal(p_all[m], st.mean_profile(m)), m
        q, u = st.cross_sections(m)
        assert np.array_equal(q_all[m], q) and np.array_equal(u_all[m], u), m
    st.close()
