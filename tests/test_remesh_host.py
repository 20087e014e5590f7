"""CPU checks of Re_Mesh (no GPU): the oracle against the reference tool's outputs
(tests/golden/remesh.npz), the product's interpolation tables against the oracle's,
and argument checks of the plan."""
import os

import numpy as np
import pytest

from conftest import ROOT, rel


@pytest.fixture(scope="module")
def nsp():
    import sys
    sys.path.insert(0, os.path.join(ROOT, "nspipe-gpu_gb300"))
    import build as nbuild
    nbuild.build()
    import nspipe_gb300
    return nspipe_gb300


@pytest.fixture(scope="module")
def golden():
    return np.load(os.path.join(ROOT, "tests", "golden", "remesh.npz"))


def cases():
    from make_golden import REMESH_CASES
    return REMESH_CASES


@pytest.mark.parametrize("name", ["up", "down", "radial_iw2"])
def test_oracle_matches_reference_tool(golden, name):
    import remesh as R
    from make_golden import remesh_input
    old, new, iw, seed = cases()[name]
    out = np.stack(R.remesh(remesh_input(old, seed), new, iw))
    assert out.shape == golden[name].shape
    assert rel(out, golden[name]) < 1e-13
    # modes the old grid lacks are exactly zero; mode (0,0) as modeZZ_k leaves it
    assert np.all(golden[name][0, :, 0, 0] == 0)
    assert np.all(golden[name][1:, :, 0, 0].imag == 0)


@pytest.mark.parametrize("name", ["up", "down", "radial_iw2"])
def test_plan_tables_match_oracle(nsp, name):
    import remesh as R
    old, new, iw, _ = cases()[name]
    p = nsp.Remesh(old, new, iw)
    RM = p.matrix()
    ref = R.remesh_matrix(old[0], new[0], iw)
    assert np.abs(RM - ref).max() <= 1e-15
    assert RM[0, -1, -1] == 1.0 and RM[1, -1, -1] == 1.0
    # every row interpolates: the even table reproduces constants away from the axis
    assert np.allclose(RM[0, :, :].sum(axis=1)[new[0] // 2:], 1.0, atol=1e-12)
    assert ((RM != 0).sum(axis=2) <= 2 * iw).all()
    p.close()


@pytest.mark.parametrize("args,needle", [((24, 8, 9, 32, 12, 13, 0), "iw"), ((24, 8, 9, 32, 12, 13, 9), "iw"),
                                         ((24, 7, 9, 32, 12, 13, 3), "NT"), ((2, 8, 9, 32, 12, 13, 3), "NR"),
                                         ((24, 8, 0, 32, 12, 13, 3), "NZ")])
def test_plan_rejects_bad_shapes(nsp, args, needle):
    with pytest.raises(nsp.NspError) as e:
        nsp.Remesh(args[:3], args[3:6], args[6])
    assert e.value.code == nsp.NSP_ERR_ARG and needle in str(e.value)
