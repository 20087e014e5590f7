"""Pins the oracle to the reference: the FP64 C restatement (oracle/) against the
golden outputs of the reference nsPipe-CUDA build (tests/golden/ref_*.npz, made
by tests/golden/make_golden.py on a GB300 from the same seeded restart files).

Gate: relative L2 <= 1e-12 and identical corrector-iteration sequences."""
import os

import numpy as np
import pytest

from conftest import ROOT, rel

GOLDEN = os.path.join(ROOT, "tests", "golden")


def load(name):
    path = os.path.join(GOLDEN, "ref_%s.npz" % name)
    if not os.path.exists(path):
        pytest.skip("fixture %s missing" % path)
    g = np.load(path)
    NR, NT, NZ, Re, dt, LZ, amp, seed, nsteps = g["params"]
    return g, int(NR), int(NT), int(NZ), Re, dt, LZ, amp, int(seed)


def test_oracle_matches_reference_full_field_s2(oracle_lib):
    g, NR, NT, NZ, Re, dt, LZ, amp, seed = load("s2")
    o = oracle_lib.Oracle(NR, NT, NZ, Re=Re, dt=dt, LZ=LZ)
    u = list(g["init"])
    # the fixture's initial field is the seeded generator's output (to the last bits of
    # the host's libm, which may differ between the x86 and aarch64 hosts)
    from nspipe_gb300.initfield import seeded_field
    for a, b in zip(u, seeded_field(NR, NT, NZ, LZ, amp, seed)):
        assert rel(a, b) < 1e-15
    done, iters = 0, []
    for s in sorted(int(k.split("_")[1]) for k in g.files if k.startswith("u_")):
        u, it, _ = o.step(u, s - done)
        iters += list(it)
        done = s
        assert rel(np.stack(u), g["u_%d" % s]) < 1e-12, s
    assert iters == list(g["iters"][:done])


def test_oracle_matches_reference_c0_100_steps(oracle_lib):
    from make_golden import projection_weights
    from nspipe_gb300.initfield import seeded_field
    g, NR, NT, NZ, Re, dt, LZ, amp, seed = load("c0")
    o = oracle_lib.Oracle(NR, NT, NZ, Re=Re, dt=dt, LZ=LZ)
    u = seeded_field(NR, NT, NZ, LZ, amp, seed)
    w = projection_weights(NR * NT * NZ, seed)
    slots = [0, 1, 2, 3, 4, NT - 4, NT - 3, NT - 2, NT - 1]
    done, iters = 0, []
    for s in sorted(int(k.split("_")[1]) for k in g.files if k.startswith("mean_")):
        u, it, _ = o.step(u, s - done)
        iters += list(it)
        done = s
        assert rel(np.stack([a[:, slots, :6] for a in u]), g["low_%d" % s]) < 1e-12
        assert rel(u[2][:, 0, 0], g["mean_%d" % s]) < 1e-12
        proj = np.stack([w @ a.reshape(-1) for a in u])
        assert np.abs(proj - g["proj_%d" % s]).max() < 1e-12 * np.abs(g["proj_%d" % s]).max()
        assert np.allclose([np.linalg.norm(a) for a in u], g["norm_%d" % s], rtol=1e-12, atol=0)
    assert iters == list(g["iters"][:done])


@pytest.mark.parametrize("name,nsteps", [("c4b", 10), ("c4c", 1), ("c1h", 1)])
def test_oracle_matches_reference_larger_shapes(oracle_lib, name, nsteps):
    """The larger shapes of the uneven batch (NR=64 x 48 x 128 modes, NR=96 x 96 x 192)
    and the turbulent shape at half its time step (NR=96 x 128 x 256), over their first
    steps (the oracle is single-pipe C: a few seconds per step at the largest shape)."""
    from make_golden import projection_weights
    from nspipe_gb300.initfield import seeded_field
    g, NR, NT, NZ, Re, dt, LZ, amp, seed = load(name)
    o = oracle_lib.Oracle(NR, NT, NZ, Re=Re, dt=dt, LZ=LZ)
    u, it, _ = o.step(seeded_field(NR, NT, NZ, LZ, amp, seed), nsteps)
    o.close()
    slots = [0, 1, 2, 3, 4, NT - 4, NT - 3, NT - 2, NT - 1]
    assert rel(np.stack([a[:, slots, :6] for a in u]), g["low_%d" % nsteps]) < 1e-12
    assert rel(u[2][:, 0, 0], g["mean_%d" % nsteps]) < 1e-12
    w = projection_weights(NR * NT * NZ, seed)
    proj = np.stack([w @ a.reshape(-1) for a in u])
    assert np.abs(proj - g["proj_%d" % nsteps]).max() < 1e-12 * np.abs(g["proj_%d" % nsteps]).max()
    assert list(it) == list(g["iters"][:nsteps])
