"""The allocation-free nonlinear entry point (nsp_nonlinear_static).

It exists for callers that cannot allocate device memory while they run: hosts with
a device-memory budget fixed after start-up, applications whose own pool allocator
owns the device memory, and loops that cannot afford cudaMalloc/cudaFree (which may
synchronise the device).  Its intermediates live in a fixed 32 MiB __device__ array
shared by all calls.  These tests call it through the C ABI and compare it with
the allocating entry point nsp_nonlinear, on two calls in a row; they run last
(file name) and also pass on their own in a fresh process.
"""
import numpy as np
import pytest

from conftest import PI2, rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nsp():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import nspipe_gb300
    nspipe_gb300.lib()
    return nspipe_gb300


def dev3(u):
    import torch
    return torch.from_numpy(np.ascontiguousarray(np.stack(u))).cuda()


@pytest.mark.parametrize("precision,tol", [(0, 1e-13), (1, 1e-6)])
def test_static_scratch_matches_allocating_entry_point(nsp, precision, tol):
    import torch
    NR, NT, NZ, LZ, Re, dt = 48, 32, 65, 2 * PI2, 2000.0, 0.01
    st = nsp.Stepper(nsp.make_params(NR, NT, NZ, Re, dt, LZ), precision=precision)
    for call, seed in enumerate((2000, 2001)):  # two calls in a row, different inputs
        u = nsp.seeded_field(NR, NT, NZ, LZ, 1e-3 * (1 + call), seed)
        u3 = dev3(u)
        ref = [torch.zeros((NR, NT, NZ), dtype=torch.complex128, device="cuda") for _ in range(3)]
        st.nonlinear(0, [u3[0], u3[1], u3[2]], ref)
        n3 = torch.full((3, NR, NT, NZ), float("nan"), dtype=torch.complex128, device="cuda")
        st.nonlinear_static(0, u3, n3)
        got = n3.cpu().numpy()
        for c in range(3):
            assert rel(got[c], ref[c].cpu().numpy()) < tol, (call, c)
    st.close()


def test_static_scratch_rejects_members_beyond_the_limit(nsp):
    import torch
    NR, NT, NZ = 64, 48, 129  # intermediates need ~114 MB in FP64
    st = nsp.Stepper(nsp.make_params(NR, NT, NZ, 2700.0, 0.006, 2 * PI2), precision=nsp.NSP_FP64)
    u3 = torch.zeros((3, NR, NT, NZ), dtype=torch.complex128, device="cuda")
    n3 = torch.zeros_like(u3)
    with pytest.raises(nsp.NspError) as e:
        st.nonlinear_static(0, u3, n3)
    assert e.value.code == nsp.NSP_ERR_ARG
    assert "fixed limit" in str(e.value)
    st.close()
