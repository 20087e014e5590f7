"""Transform lengths without a compiled kernel specialisation (the run-time FFT
kernels): NT=12 (NTP=18) and NZ=13 (NZR=36), NR=24, against the oracle.  Same gates
as the compiled lengths: FP64 relative L2 <= 1e-12 with identical iteration counts,
mixed <= 2e-6 for the nonlinear term and <= 1e-6 after 10 steps."""
import numpy as np
import pytest

from conftest import PI2, rel
from test_gpu_parity import dev, nsp  # noqa: F401  (fixture)

pytestmark = pytest.mark.gpu

NR, NT, NZ, Re, dt, LZ = 24, 12, 13, 1500.0, 0.01, PI2


@pytest.fixture(scope="module")
def o(oracle_lib):
    orc = oracle_lib.Oracle(NR, NT, NZ, Re=Re, dt=dt, LZ=LZ)
    yield orc
    orc.close()


def field(nsp, seed=31):
    return nsp.seeded_field(NR, NT, NZ, LZ, 0.05, seed)


def stepper(nsp, precision):
    st = nsp.Stepper(nsp.make_params(NR, NT, NZ, Re, dt, LZ), precision=precision)
    g = st.describe()["groups"][0]
    assert g["theta"] in ("fft-fp64", "fft-fp32")
    return st


@pytest.mark.parametrize("precision,tol", [(0, 1e-13), (1, 2e-6)])
def test_nonlinear_generic_lengths(nsp, o, precision, tol):
    import torch
    u0 = field(nsp)
    st = stepper(nsp, precision)
    n = [torch.zeros(o.shape, dtype=torch.complex128, device="cuda") for _ in range(3)]
    st.nonlinear(0, [dev(a) for a in u0], n)
    ref = o.nonlinear(u0)
    for c in range(3):
        assert rel(n[c].cpu().numpy(), ref[c]) < tol, c
    st.close()


def test_steps_generic_lengths(nsp, o):
    u0 = field(nsp)
    uo, ito, _ = o.step([a.copy() for a in u0], 10)
    for precision, tol in ((0, 1e-12), (1, 1e-6)):
        st = stepper(nsp, precision)
        st.set_state(0, u0)
        it = st.step(10)
        if precision == 0:
            assert list(it[:, 0]) == list(ito)
        assert rel(np.stack(st.get_state(0)), np.stack(uo)) < tol, precision
        st.close()
