"""Seeded initial fields and the raw spectral checkpoint format.

The reference starts either from a built-in deterministic perturbation
(initField, mod_io_nonlinear.cu:424-449) or from raw restart files u?_s.bin
(rBufferBinary, :550-565).  Ensembles need a *seeded* perturbation, which the
reference does not have, so this module generates one and writes it in the
restart format; both the reference build and this stepper read the same files.

Construction (divergence-free in the continuous sense, no-slip at r = 1):
for every retained mode (m, l) with 0 < |m|+l, |m| <= mmax, l <= lmax,

    psi = a (1-r^2)^2 r^|m|       ->  u_r = i m psi / r,   u_th = -d psi/dr
    chi = b (1-r^2)^2 r^(|m|+1)   ->  u_r = -i k_z chi,    u_z = (1/r) d(r chi)/dr

(the curls of psi e_z and chi e_th), with complex normal a, b drawn from a
SplitMix64 stream (Box-Muller).  The l = 0 plane is made Hermitian
(u(-m,0) = conj u(m,0)).  The perturbation is scaled so that its largest
spectral coefficient has modulus `amplitude`, and the Hagen-Poiseuille
profile u_z(0,0) = 1 - r^2 (base_k, mod_io_nonlinear.cu:9-16) is added.
"""
import math
import os

import numpy as np

PI2 = 6.283185307179586  # the reference's constant (head.h:12)
_M64 = (1 << 64) - 1


class SplitMix64:
    def __init__(self, seed):
        self.s = seed & _M64

    def next(self):
        self.s = (self.s + 0x9E3779B97F4A7C15) & _M64
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
        return z ^ (z >> 31)

    def uniform(self):
        return ((self.next() >> 11) + 0.5) * (1.0 / 9007199254740992.0)

    def normal(self):
        u1, u2 = self.uniform(), self.uniform()
        return math.sqrt(-2.0 * math.log(u1)) * math.cos(PI2 * u2)


def radial_grid(NR):
    """Wall-clustered radial grid of init_fd (mod_radialFD.cu:211-216)."""
    N_p = NR + int(math.sqrt(float(NR)))
    r = np.zeros(NR)
    for i in range(N_p - NR, N_p):
        ir = N_p - i - 1
        r[i - N_p + NR] = 0.5 * (1.0 + math.cos(0.5 * PI2 * (float(ir) / float(N_p))))
    for _ in range(10):
        dr = 1.5 * r[0] - 0.5 * r[1]
        r = r * (1.0 + dr) - dr
    return r


def seeded_field(NR, NT, NZ, LZ, amplitude, seed, mmax=4, lmax=4, base_flow=True):
    """Return [ur, ut, uz], complex128 arrays (NR, NT, NZ) in the reference layout."""
    r = radial_grid(NR)
    u = [np.zeros((NR, NT, NZ), np.complex128) for _ in range(3)]
    rng = SplitMix64(seed)
    mmax = min(mmax, NT // 2 - 1)
    lmax = min(lmax, NZ - 2)
    one = 1.0 - r * r
    for l in range(0, lmax + 1):
        for m in range(-mmax, mmax + 1):
            if l == 0 and m <= 0:
                continue
            a = complex(rng.normal(), rng.normal()) / math.sqrt(2.0)
            b = complex(rng.normal(), rng.normal()) / math.sqrt(2.0)
            n = abs(m)
            kz = (PI2 / LZ) * l
            f_over_r = one ** 2 * r ** (n - 1) if n > 0 else np.zeros(NR)
            fp = (n * r ** (n - 1) if n > 0 else 0.0) * one ** 2 - 4.0 * r ** (n + 1) * one
            g = one ** 2 * r ** (n + 1)
            uz_chi = (n + 2) * r ** n * one ** 2 - 4.0 * r ** (n + 2) * one
            ur = 1j * m * a * f_over_r - 1j * kz * b * g
            ut = -a * fp
            uz = b * uz_chi
            it = m % NT
            u[0][:, it, l] = ur
            u[1][:, it, l] = ut
            u[2][:, it, l] = uz
            if l == 0:
                u[0][:, (-m) % NT, 0] = np.conj(ur)
                u[1][:, (-m) % NT, 0] = np.conj(ut)
                u[2][:, (-m) % NT, 0] = np.conj(uz)
    peak = max(np.abs(x).max() for x in u)
    if peak > 0:
        for x in u:
            x *= amplitude / peak
    if base_flow:
        u[2][:, 0, 0] += one
    return u


def write_state(u, directory, suffix="_s"):
    """Write ur<suffix>.bin, ut<suffix>.bin, uz<suffix>.bin (wBufferBinary layout)."""
    os.makedirs(directory, exist_ok=True)
    for c, a in zip("rtz", u):
        np.ascontiguousarray(a, np.complex128).astype("<c16").tofile(os.path.join(directory, "u%s%s.bin" % (c, suffix)))


def read_state(directory, shape, suffix="_s"):
    """Read the three raw double2[NR][NT][NZ] files (rBufferBinary layout)."""
    out = []
    for c in "rtz":
        path = os.path.join(directory, "u%s%s.bin" % (c, suffix))
        a = np.fromfile(path, dtype="<c16")
        if a.size != int(np.prod(shape)):
            raise ValueError("%s: %d values, expected %d" % (path, a.size, int(np.prod(shape))))
        out.append(a.reshape(shape).astype(np.complex128))
    return out
