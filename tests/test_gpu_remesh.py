"""Re_Mesh on the GPU (nsp_remesh_*): the batched kernel against the reference tool's
outputs and the oracle, the file tool, batching, and remeshing context members
between two groups of an uneven ensemble.  Tolerance: relative L2 <= 1e-13 (the
tables agree with the tool's to rounding; each output is a <= 2 iw term FMA chain)."""
import os

import numpy as np
import pytest

from conftest import PI2, rel
from test_gpu_parity import nsp  # noqa: F401  (fixture)
from test_remesh_host import cases, golden  # noqa: F401  (fixtures)

pytestmark = pytest.mark.gpu


def dev3(u):
    import torch
    return torch.from_numpy(np.ascontiguousarray(np.stack(u)).reshape(-1)).cuda()


def host3(t, shape):
    return [a for a in t.cpu().numpy().reshape((3,) + tuple(shape))]


@pytest.mark.parametrize("name", ["up", "down", "radial_iw2"])
def test_device_remesh_matches_reference_tool(nsp, golden, name):
    import torch
    import remesh as R
    from make_golden import remesh_input
    old, new, iw, seed = cases()[name]
    u = remesh_input(old, seed)
    p = nsp.Remesh(old, new, iw)
    out = torch.full((3 * int(np.prod(new)),), float("nan"), dtype=torch.complex128, device="cuda")
    p.device([dev3(u)], [out])
    got = np.stack(host3(out, new))
    assert np.isfinite(got).all()  # every destination value written
    assert rel(got, golden[name]) < 1e-13
    assert rel(got, np.stack(R.remesh(u, new, iw))) < 1e-13
    assert np.all(got[0, :, 0, 0] == 0) and np.all(got[1:, :, 0, 0].imag == 0)
    p.close()


def test_files_tool_and_batching(nsp, tmp_path):
    import torch
    from make_golden import remesh_input
    old, new, iw, _ = cases()["up"]
    fields = [remesh_input(old, 500 + k) for k in range(3)]
    p = nsp.Remesh(old, new, iw)
    outs = [torch.zeros(3 * int(np.prod(new)), dtype=torch.complex128, device="cuda") for _ in range(3)]
    p.device([dev3(f) for f in fields], outs)  # one launch, three members
    batched = [np.stack(host3(o, new)) for o in outs]
    for k in range(3):
        one = torch.zeros_like(outs[0])
        p.device([dev3(fields[k])], [one])
        assert np.array_equal(np.stack(host3(one, new)), batched[k]), k
    # the tool: u?_o.bin in, u?_s.bin out
    d = str(tmp_path)
    for c, a in zip("rtz", fields[1]):
        np.ascontiguousarray(a).tofile(os.path.join(d, "u%s_o.bin" % c))
    p.files(d, d)
    fromfile = np.stack([np.fromfile(os.path.join(d, "u%s_s.bin" % c), np.complex128).reshape(new) for c in "rtz"])
    assert np.array_equal(fromfile, batched[1])
    with pytest.raises(nsp.NspError) as e:
        p.files(str(tmp_path / "missing"), d)
    assert e.value.code == nsp.NSP_ERR_IO
    p.close()


def test_members_between_groups_of_an_uneven_ensemble(nsp):
    """A coarse group's state refined into a fine group of the same context, then both
    stepped: the refined member starts from the oracle's remesh of the coarse state."""
    import remesh as R
    old, new = (24, 8, 9), (32, 16, 17)
    Re, dt = 1000.0, 0.005
    coarse = nsp.make_params(*old, Re, dt, PI2)
    fine = nsp.make_params(*new, Re, dt, PI2)
    st = nsp.Stepper([coarse, coarse, fine, fine], precision=nsp.NSP_FP64)
    u0 = [nsp.seeded_field(*old, PI2, 0.05, 7 + m) for m in range(2)]
    for m in range(2):
        st.set_state(m, u0[m])
    st.step(3)
    src = [st.get_state(m) for m in range(2)]
    p = nsp.Remesh(old, new, 3)
    p.members(st, [0, 1], st, [3, 2])
    for m, k in ((0, 3), (1, 2)):
        assert rel(np.stack(st.get_state(k)), np.stack(R.remesh(src[m], new, 3))) < 1e-13
    iters = st.step(3)
    assert (iters >= 1).all()
    for k in range(4):
        d = st.diag(k)
        assert d.status == 0 and np.isfinite(d.u_tau) and d.div_wall < 1e-9, k
    with pytest.raises(nsp.NspError):  # shapes must be the plan's
        p.members(st, [2], st, [3])
    with pytest.raises(nsp.NspError):  # a member cannot be its own destination
        q = nsp.Remesh(new, new, 3)
        q.members(st, [2], st, [2])
    p.close()
    st.close()
