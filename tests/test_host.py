"""CPU checks of the host-side logic: the seeded initial field and the raw
restart-file format (rBufferBinary / wBufferBinary, mod_io_nonlinear.cu:528-565)."""
import numpy as np
import pytest

from conftest import PI2
from nspipe_gb300 import initfield as inf


def test_seeded_field_is_deterministic_and_hermitian():
    a = inf.seeded_field(48, 32, 65, 2 * PI2, 1e-3, 7)
    b = inf.seeded_field(48, 32, 65, 2 * PI2, 1e-3, 7)
    c = inf.seeded_field(48, 32, 65, 2 * PI2, 1e-3, 8)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    assert not np.array_equal(a[0], c[0])
    NT = 32
    for u in a:
        for it in range(1, NT // 2):
            assert np.array_equal(u[:, NT - it, 0], np.conj(u[:, it, 0]))
        assert np.all(u[:, NT // 2, :] == 0)     # theta Nyquist slot
        assert np.all(u[:, :, -1] == 0)          # l = NZ-1 (zeroed by padBackward)
        assert np.all(u[-1] == 0)                # no-slip wall (r = 1)
    r = inf.radial_grid(48)
    pert = [x.copy() for x in a]
    pert[2][:, 0, 0] -= 1 - r * r
    assert abs(max(np.abs(x).max() for x in pert) - 1e-3) < 1e-18
    assert np.all(a[0][:, 0, 0] == 0)


def test_seeded_field_is_solenoidal_in_the_continuum():
    # divergence (1/r) d(r u_r)/dr + i m u_t / r + i k_z u_z of the analytic profiles, by
    # finite differences on a fine auxiliary grid: vanishes to discretisation error.
    NR, NT, NZ, LZ = 400, 16, 9, PI2
    u = inf.seeded_field(NR, NT, NZ, LZ, 1.0, 3, base_flow=False)
    r = inf.radial_grid(NR)
    for it in range(NT):
        m = it if it < NT // 2 else it - NT
        for l in range(NZ):
            ur, ut, uz = u[0][:, it, l], u[1][:, it, l], u[2][:, it, l]
            if not (np.any(ur) or np.any(ut) or np.any(uz)):
                continue
            kz = PI2 / LZ * l
            div = np.gradient(r * ur, r) / r + 1j * m * ut / r + 1j * kz * uz
            scale = max(np.abs(ur).max(), np.abs(ut).max(), np.abs(uz).max())
            assert np.abs(div[5:-5]).max() < 1e-3 * scale * max(1, abs(m), kz)


def test_restart_files_roundtrip_and_layout(tmp_path):
    u = inf.seeded_field(24, 8, 9, PI2, 0.05, 11)
    inf.write_state(u, str(tmp_path))
    raw = (tmp_path / "ur_s.bin").read_bytes()
    assert len(raw) == 24 * 8 * 9 * 16
    # double2 layout: (re, im) pairs, little-endian, index i*NT*NZ + it*NZ + l
    first = np.frombuffer(raw[:32], "<f8")
    assert first[0] == u[0][0, 0, 0].real and first[1] == u[0][0, 0, 0].imag
    assert first[2] == u[0][0, 0, 1].real
    v = inf.read_state(str(tmp_path), (24, 8, 9))
    for a, b in zip(u, v):
        assert np.array_equal(a, b)


def test_short_restart_file_is_rejected(tmp_path):
    u = inf.seeded_field(24, 8, 9, PI2, 0.05, 11)
    inf.write_state(u, str(tmp_path))
    p = tmp_path / "ut_s.bin"
    p.write_bytes(p.read_bytes()[:-16])
    with pytest.raises(ValueError):
        inf.read_state(str(tmp_path), (24, 8, 9))


def test_splitmix_reference_values():
    # SplitMix64 published test vector for seed 1234567.
    g = inf.SplitMix64(1234567)
    assert [g.next() for _ in range(3)] == [6457827717110365317, 3203168211198807973, 9817491932198370423]
