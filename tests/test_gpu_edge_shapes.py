"""Shapes at the edges of what nsp_create accepts, against the oracle: the smallest
grid (NR=8: every radial row within the stencil's reach of the axis or the wall;
NT=4, NZ=3: transforms of 6 points), an odd azimuthal length (NT=6: NTP=9), and a
tall radial grid (NR=256, the linear pass's smaller blocks).  FP64 relative L2 <= 1e-12
with identical iteration counts after 3 steps; mixed <= 1e-6."""
import numpy as np
import pytest

from conftest import PI2, rel
from test_gpu_parity import nsp  # noqa: F401  (fixture)

pytestmark = pytest.mark.gpu

SHAPES = [(8, 4, 3), (24, 6, 5), (256, 8, 9)]


@pytest.mark.parametrize("shape", SHAPES)
def test_edge_shape_matches_oracle(nsp, oracle_lib, shape):
    NR, NT, NZ = shape
    Re, dt = 1000.0, 0.005
    u0 = nsp.seeded_field(NR, NT, NZ, PI2, 0.05, 7)
    o = oracle_lib.Oracle(NR, NT, NZ, Re=Re, dt=dt, LZ=PI2)
    uo, ito, _ = o.step([a.copy() for a in u0], 3)
    o.close()
    for precision, tol in ((nsp.NSP_FP64, 1e-12), (nsp.NSP_MIXED, 1e-6)):
        st = nsp.Stepper(nsp.make_params(NR, NT, NZ, Re, dt, PI2), precision=precision)
        st.set_state(0, u0)
        it = st.step(3)
        u = np.stack(st.get_state(0))
        if precision == nsp.NSP_FP64:
            assert list(it[:, 0]) == list(ito)
        assert rel(u, np.stack(uo)) < tol, (shape, precision)
        assert st.diag(0).div_wall < 1e-10
        st.close()
