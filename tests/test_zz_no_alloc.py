"""The allocation-free nonlinear entry point (nsp_nonlinear_static).

It exists for callers that cannot allocate device memory while they run: hosts with
a device-memory budget fixed after start-up, applications whose own pool allocator
owns the device memory, and loops that cannot afford cudaMalloc/cudaFree (which may
synchronise the device).  Its intermediates live in a fixed 32 MiB __device__ array
shared by all calls.  These tests call it through the C ABI and compare it with
the allocating entry point nsp_nonlinear (bit for bit) and with the oracle, on two
calls in a row; they run last (file name) and also pass on their own in a fresh
process.
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


@pytest.fixture(scope="module")
def orc_c0(oracle_lib):
    o = oracle_lib.Oracle(48, 32, 65, Re=2000.0, dt=0.01, LZ=2 * PI2)
    yield o
    o.close()


@pytest.mark.parametrize("precision,tol", [(0, 1e-13), (1, 2e-6)])
def test_static_scratch_matches_allocating_entry_point(nsp, orc_c0, precision, tol):
    """Same kernels on the same input as nsp_nonlinear, only the intermediates live in
    the fixed array: the results are equal bit for bit, on two calls in a row (the
    second call finds the first call's intermediates in the array).  Each result is
    also checked against the oracle (FP64 form 1e-13, mixed form 2e-6 relative)."""
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
        want = orc_c0.nonlinear(u)
        for c in range(3):
            assert np.array_equal(got[c], ref[c].cpu().numpy()), (call, c)
            assert rel(got[c], want[c]) < tol, (call, c)
    st.close()


def test_static_scratch_rejects_overlapping_buffers(nsp):
    import torch
    NR, NT, NZ = 24, 8, 9
    st = nsp.Stepper(nsp.make_params(NR, NT, NZ, 1000.0, 0.01, PI2), precision=nsp.NSP_FP64)
    buf = torch.zeros((4, NR, NT, NZ), dtype=torch.complex128, device="cuda")
    with pytest.raises(nsp.NspError) as e:
        st.nonlinear_static(0, buf[0:3], buf[1:4])
    assert e.value.code == nsp.NSP_ERR_ARG and "overlap" in str(e.value)
    st.close()


def test_static_scratch_reports_a_device_wait_that_ran_out(nsp):
    """The mixed form's tensor-core transforms, made to run out of their bounded wait
    (nsp_debug_inject, no GPU fault): the call reports NSP_ERR_DEVICE, and the next
    call, without the injection, succeeds and matches nsp_nonlinear bit for bit."""
    import torch
    NR, NT, NZ, LZ = 48, 32, 65, 2 * PI2
    st = nsp.Stepper(nsp.make_params(NR, NT, NZ, 2000.0, 0.01, LZ), precision=nsp.NSP_MIXED)
    if st.describe()["groups"][0]["theta"] != "tcgen05-3xtf32":
        pytest.skip("tensor-core theta transforms not selected")
    u3 = dev3(nsp.seeded_field(NR, NT, NZ, LZ, 1e-3, 2000))
    n3 = torch.zeros_like(u3)
    st.debug_inject(1)
    with pytest.raises(nsp.NspError) as e:
        st.nonlinear_static(0, u3, n3)
    assert e.value.code == nsp.NSP_ERR_DEVICE
    st.debug_inject(0)
    st.nonlinear_static(0, u3, n3)
    ref = [torch.zeros((NR, NT, NZ), dtype=torch.complex128, device="cuda") for _ in range(3)]
    st.nonlinear(0, [u3[0], u3[1], u3[2]], ref)
    for c in range(3):
        assert torch.equal(n3[c], ref[c]), c
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
