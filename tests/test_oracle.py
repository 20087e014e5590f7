"""CPU checks of the oracle (the FP64 C restatement in oracle/): transforms against
numpy, radial operators against exact polynomial derivatives, the banded
solves against an independently assembled operator, and the invariants the
reference's step enforces (wall no-slip, wall divergence, prescribed flux)."""
import numpy as np
import pytest

from conftest import PI2, rel


@pytest.fixture(scope="module")
def o_s1(oracle_lib):
    return oracle_lib.Oracle(24, 8, 9, Re=1000.0, dt=0.01, LZ=PI2)


@pytest.fixture(scope="module")
def o_c0(oracle_lib):
    return oracle_lib.Oracle(48, 32, 65, Re=2000.0, dt=0.01, LZ=2 * PI2)


def hermitian_level(NT, NZ, rng):
    spec = rng.standard_normal((NT, NZ)) + 1j * rng.standard_normal((NT, NZ))
    spec[NT // 2, :] = 0
    spec[:, NZ - 1] = 0
    for it in range(1, NT // 2):
        spec[NT - it, 0] = np.conj(spec[it, 0])
    spec[0, 0] = spec[0, 0].real
    return spec


@pytest.mark.parametrize("shape", [(8, 9), (32, 65), (48, 129), (16, 17)])
def test_level_transforms_match_numpy(oracle_lib, shape):
    NT, NZ = shape
    o = oracle_lib.Oracle(16, NT, NZ, Re=1000.0, dt=0.01, LZ=PI2)
    rng = np.random.default_rng(NT * 1000 + NZ)
    spec = hermitian_level(NT, NZ, rng)
    phys = o.level_backward(spec)
    NTP, NZP, NZR = o.NTP, o.NZP, o.NZR
    pad = np.zeros((NTP, NZP), complex)
    pad[: NT // 2, :NZ] = spec[: NT // 2]
    pad[NTP - NT // 2:, :NZ] = spec[NT // 2:]
    ref = np.fft.irfft2(pad, s=(NTP, NZR)) * NTP * NZR
    assert np.abs(phys - ref).max() <= 1e-14 * np.abs(ref).max()
    back = o.level_forward(phys)
    assert np.abs(back - spec).max() <= 1e-14 * np.abs(spec).max()
    # forward of an arbitrary real field: numpy rfft2, scaled, truncated (padBackward)
    x = rng.standard_normal((NTP, NZR))
    F = np.fft.rfft2(x) / (NTP * NZR)
    exp = np.zeros((NT, NZ), complex)
    exp[: NT // 2] = F[: NT // 2, :NZ]
    exp[NT // 2:] = F[NTP - NT // 2:, :NZ]
    exp[NT // 2, :] = 0
    exp[:, NZ - 1] = 0
    got = o.level_forward(x)
    assert np.abs(got - exp).max() <= 1e-15


def test_grid_and_quadrature(o_c0):
    g = o_c0.grid()
    r = g["r"]
    assert np.all(np.diff(r) > 0) and r[0] > 0 and abs(r[-1] - 1.0) < 1e-15
    assert abs(r[0] - 6.3671e-3) < 1e-6  # wall-clustered grid of init_fd at NR=48
    assert abs(g["rdr"].sum() - 1.0) < 1e-13  # (1/pi) int int r dr dtheta = 1


def apply_rows(table, f, NR):
    out = np.zeros(NR)
    for i in range(NR):
        left, right = max(0, i - 3), min(i + 3, NR - 1)
        i0 = i + 3 - right
        for j in range(right + 1 - left):
            out[i] += table[i, j + i0] * f[left + j]
    return out


def test_derivative_tables_exact_on_polynomials(o_c0):
    g = o_c0.grid()
    r, D = g["r"], g["D"]
    NR = len(r)
    # even table (index 0): even functions; odd table (index 1): odd functions.
    for deg in (2, 4):
        d = apply_rows(D[0], r ** deg, NR)
        assert np.abs(d[:-1] - deg * r[:-1] ** (deg - 1)).max() < 1e-9
    for deg in (1, 3):
        d = apply_rows(D[1], r ** deg, NR)
        assert np.abs(d[:-1] - deg * r[:-1] ** (deg - 1)).max() < 1e-9
    # one-sided wall row: exact up to degree 3
    assert abs(apply_rows(D[0], r ** 2, NR)[-1] - 2.0) < 1e-10


def assemble(o, kind, it, l, g):
    """Dense operator of LUsolve_* for one mode, assembled from the grid tables."""
    NR, NT = o.NR, o.NT
    m = it if it < NT // 2 else it - NT
    kt, kz = float(m), (PI2 / o.prm.LZ) * l
    odd = 1 if kind <= 1 else 0
    tab = abs(abs(m) % 2 - odd)
    T = g["Lp"][tab] if kind == 3 else g["Lu"][tab]
    A = np.zeros((NR, NR))
    r = g["r"]
    for i in range(NR):
        left, right = max(0, i - 3), min(i + 3, NR - 1)
        i0 = i + 3 - right
        for j in range(right + 1 - left):
            A[i, left + j] = T[i, j + i0]
        if i < NR - 1:
            r2 = r[i] ** 2
            diag = -kz * kz - kt * kt / r2
            if kind == 0:
                diag += -1 / r2 - 2 * kt / r2
            elif kind == 1:
                diag += -1 / r2 + 2 * kt / r2
            if kind == 3:
                A[i, i] += diag
            else:
                A[i, :] *= -o.prm.d_im / o.prm.Re
                A[i, i] += 1 / o.prm.dt - o.prm.d_im / o.prm.Re * diag
    if kind == 3 and m == 0 and l == 0:
        A[NR - 1, :] = 0
        A[NR - 1, NR - 1] = 1
    return A


@pytest.mark.parametrize("kind", [0, 1, 2, 3])
def test_banded_solves_against_dense_operator(o_s1, kind):
    o = o_s1
    g = o.grid()
    rng = np.random.default_rng(kind)
    b = rng.standard_normal(o.shape) + 1j * rng.standard_normal(o.shape)
    x = o.lusolve_p(b) if kind == 3 else o.lusolve_u(b, kind)
    for it in range(o.NT):
        for l in range(o.NZ):
            A = assemble(o, kind, it, l, g)
            res = A @ x[:, it, l] - b[:, it, l]
            assert np.abs(res).max() <= 1e-9 * (np.abs(A).max() * np.abs(x[:, it, l]).max() + 1)


def test_step_invariants(oracle_lib, o_s1):
    import nspipe_gb300.initfield as inf
    o = o_s1
    u0 = inf.seeded_field(o.NR, o.NT, o.NZ, PI2, 0.05, 11)
    u, iters, errs = o.step(u0, 3)
    g = o.grid()
    assert all(1 <= i <= 10 for i in iters)
    # no-slip at the wall and prescribed flux Q = 0.5 (adj_flux)
    for a in u:
        assert np.abs(a[-1]).max() < 1e-12
    assert abs((g["rdr"] * u[2][:, 0, 0].real).sum() - 0.5) < 1e-13
    # wall divergence removed by the influence-matrix correction
    dw = o.div_wall(*u)
    assert np.abs(dw).max() < 1e-9 * np.abs(u[2]).max()
    # mode (0,0) constraints (modeZZ)
    assert np.all(u[0][:, 0, 0] == 0) and np.all(u[1][:, 0, 0].imag == 0) and np.all(u[2][:, 0, 0].imag == 0)
    # Hermitian symmetry of the l = 0 plane is preserved
    for it in range(1, o.NT // 2):
        for a in u:
            assert np.abs(a[:, o.NT - it, 0] - np.conj(a[:, it, 0])).max() < 1e-12
