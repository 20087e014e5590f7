"""Operator tables built on the device (one thread per parameter set and mode) against
the host build: the same per-mode code, compiled without FMA contraction on both
sides, so the tables must agree bit for bit.  Checked through the entry points that
read them -- the four banded solves (the factors) and time steps (the influence-matrix
profiles) -- on an uneven ensemble with several Re per shape, in both precisions."""
import time

import numpy as np
import pytest

from conftest import PI2
from test_gpu_parity import dev, nsp  # noqa: F401  (fixture)

pytestmark = pytest.mark.gpu

SHAPES = [((24, 8, 9), (1000.0, 1100.0, 1250.0)), ((48, 32, 65), (2000.0, 2200.0))]


def build(nsp, monkeypatch, device_setup, precision):
    monkeypatch.setenv("NSP_DEVICE_SETUP", "1" if device_setup else "0")
    monkeypatch.setenv("NSP_AUTOTUNE", "0")
    prm = [nsp.make_params(*shape, Re, 0.01, 2 * PI2) for shape, res in SHAPES for Re in res]
    t0 = time.perf_counter()
    st = nsp.Stepper(prm, precision=precision)
    dt = time.perf_counter() - t0
    d = st.describe()
    assert [g["setup"] for g in d["groups"]] == ["device" if device_setup else "host"] * 2
    assert [g["parameter_sets"] for g in d["groups"]] == [3, 2]
    return st, dt


@pytest.mark.parametrize("precision", [0, 1])
def test_device_setup_bit_identical_to_host(nsp, monkeypatch, precision):
    import torch
    sts = {}
    for flag in (False, True):
        sts[flag], _ = build(nsp, monkeypatch, flag, precision)
    rng = np.random.default_rng(5)
    for m in range(sts[True].n):
        shape = sts[True].shape(m)
        b = dev(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
        for kind in range(4):
            out = {}
            for flag, st in sts.items():
                x = torch.zeros(shape, dtype=torch.complex128, device="cuda")
                st.lusolve(m, kind, b, x)
                out[flag] = x.cpu().numpy()
            assert np.array_equal(out[True], out[False]), (m, kind)
        u0 = nsp.seeded_field(*shape, 2 * PI2, 0.05, 40 + m)
        for st in sts.values():
            st.set_state(m, u0)
    res = {}
    for flag, st in sts.items():
        iters = st.step(4)
        res[flag] = ([np.stack(st.get_state(m)) for m in range(st.n)], iters)
    for m in range(sts[True].n):
        assert np.array_equal(res[True][0][m], res[False][0][m]), m
    assert np.array_equal(res[True][1], res[False][1])
    for st in sts.values():
        st.close()


def test_device_setup_time(nsp, monkeypatch):
    """Record the set-up time of both paths (the device path must not be slower)."""
    times = {}
    for flag in (False, True):
        st, times[flag] = build(nsp, monkeypatch, flag, 0)
        st.close()
    print("setup seconds: host %.3f device %.3f" % (times[False], times[True]))
    assert times[True] <= times[False] * 1.5 + 0.5
