"""ctypes binding of the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE: the FP64 CPU restatement of the nsPipe-CUDA step used as
the parity checker by tests/, __graft_entry__.smoke() and the CPU legs of
bench.py.  Nothing in the product package imports this module.

Spectral fields are numpy complex128 arrays of shape (NR, NT, NZ), the
reference's double2[NR][NT][NZ] layout (head.h:73, mod_deriv.cu:15-17).
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


class OrcParams(ctypes.Structure):
    _fields_ = [
        ("NR", ctypes.c_int), ("NT", ctypes.c_int), ("NZ", ctypes.c_int),
        ("LT", ctypes.c_double), ("LZ", ctypes.c_double),
        ("Re", ctypes.c_double),
        ("dt", ctypes.c_double), ("d_im", ctypes.c_double),
        ("maxit", ctypes.c_int),
        ("tol", ctypes.c_double),
        ("sten", ctypes.c_int),
        ("nthreads", ctypes.c_int),
    ]


def build():
    """Compile liboracle.so in place (gcc; a few seconds)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        vp, dp, ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
        L.orc_create.restype = vp
        L.orc_create.argtypes = [ctypes.POINTER(OrcParams)]
        L.orc_destroy.argtypes = [vp]
        L.orc_get_grid.argtypes = [vp] + [dp] * 6
        L.orc_get_setup.argtypes = [vp] + [dp] * 9
        L.orc_derivr.argtypes = [vp, dp, dp, ctypes.c_int]
        L.orc_lusolve_u.argtypes = [vp, dp, dp, ctypes.c_int]
        L.orc_lusolve_p.argtypes = [vp, dp, dp]
        L.orc_add_laplacian.argtypes = [vp, dp, dp, ctypes.c_int]
        L.orc_divergence.argtypes = [vp, dp, dp, dp, dp]
        L.orc_div_wall.argtypes = [vp, dp, dp, dp, dp]
        L.orc_nonlinear.argtypes = [vp] + [dp] * 6
        L.orc_level_backward.argtypes = [vp, dp, dp]
        L.orc_level_forward.argtypes = [vp, dp, dp]
        L.orc_step.argtypes = [vp, dp, dp, dp, ctypes.c_int, ip, dp]
        L.orc_step.restype = ctypes.c_int
        L.orc_friction.argtypes = [vp, dp, dp, dp]
        _LIB = L
    return _LIB


def _p(a):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Oracle:
    """One pipe with the reference's compile-time parameters given at run time."""

    def __init__(self, NR, NT, NZ, Re, dt, LZ, LT=None, d_im=0.51, maxit=10, tol=5e-8, sten=7, nthreads=0):
        PI2 = 6.283185307179586
        self.NR, self.NT, self.NZ = NR, NT, NZ
        self.NTP = 3 * NT // 2
        self.NZP = 3 * (NZ - 1) // 2 + 1
        self.NZR = 2 * self.NZP - 2
        self.sten = sten
        self.prm = OrcParams(NR, NT, NZ, PI2 if LT is None else LT, LZ, Re, dt, d_im, maxit, tol, sten, nthreads)
        self.h = lib().orc_create(ctypes.byref(self.prm))

    def close(self):
        if self.h:
            lib().orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def shape(self):
        return (self.NR, self.NT, self.NZ)

    def zeros(self):
        return np.zeros(self.shape, np.complex128)

    def grid(self):
        NR, s = self.NR, self.sten
        r, rdr = np.zeros(NR), np.zeros(NR)
        D, Lu, Lp = np.zeros((2, NR, s)), np.zeros((2, NR, s)), np.zeros((2, NR, s))
        dr0 = np.zeros(s // 2 + 1)
        lib().orc_get_grid(self.h, _p(r), _p(rdr), _p(D), _p(Lu), _p(Lp), _p(dr0))
        return dict(r=r, rdr=rdr, D=D, Lu=Lu, Lp=Lp, dr0=dr0)

    def setup(self):
        uc, Qc = np.zeros(self.NR), np.zeros(1)
        invM = np.zeros((self.NT * self.NZ, 16), np.complex128)
        f = [self.zeros() for _ in range(6)]
        lib().orc_get_setup(self.h, _p(uc), _p(Qc), _p(invM), *[_p(a) for a in f])
        return dict(uc=uc, Qc=Qc[0], invM=invM, uh=f[:3], uhP=f[3:])

    def derivr(self, u, flag):
        out = self.zeros()
        lib().orc_derivr(self.h, _p(out), _p(np.ascontiguousarray(u)), flag)
        return out

    def lusolve_u(self, rhs, flag):
        out = self.zeros()
        lib().orc_lusolve_u(self.h, _p(out), _p(np.ascontiguousarray(rhs)), flag)
        return out

    def lusolve_p(self, rhs):
        out = self.zeros()
        lib().orc_lusolve_p(self.h, _p(out), _p(np.ascontiguousarray(rhs)))
        return out

    def add_laplacian(self, rhs, u, flag):
        out = np.array(rhs, np.complex128, copy=True)
        lib().orc_add_laplacian(self.h, _p(out), _p(np.ascontiguousarray(u)), flag)
        return out

    def divergence(self, ur, ut, uz):
        out = self.zeros()
        lib().orc_divergence(self.h, _p(out), *[_p(np.ascontiguousarray(a)) for a in (ur, ut, uz)])
        return out

    def div_wall(self, ur, ut, uz):
        out = np.zeros((self.NT, self.NZ), np.complex128)
        lib().orc_div_wall(self.h, _p(out), *[_p(np.ascontiguousarray(a)) for a in (ur, ut, uz)])
        return out

    def nonlinear(self, u):
        out = [self.zeros() for _ in range(3)]
        lib().orc_nonlinear(self.h, *[_p(np.ascontiguousarray(a)) for a in u], *[_p(a) for a in out])
        return out

    def level_backward(self, spec):
        out = np.zeros((self.NTP, self.NZR))
        lib().orc_level_backward(self.h, _p(np.ascontiguousarray(spec, np.complex128)), _p(out))
        return out

    def level_forward(self, phys):
        out = np.zeros((self.NT, self.NZ), np.complex128)
        lib().orc_level_forward(self.h, _p(np.ascontiguousarray(phys, np.float64)), _p(out))
        return out

    def step(self, u, nsteps):
        """Advance u = [ur, ut, uz] in place by nsteps; returns (iters, errs)."""
        u = [np.ascontiguousarray(a, np.complex128) for a in u]
        iters = np.zeros(nsteps, np.int32)
        errs = np.zeros(nsteps)
        lib().orc_step(self.h, _p(u[0]), _p(u[1]), _p(u[2]), nsteps,
                       iters.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _p(errs))
        return u, iters, errs

    def friction(self, uz):
        uc, ut = ctypes.c_double(), ctypes.c_double()
        lib().orc_friction(self.h, _p(np.ascontiguousarray(uz)), ctypes.byref(uc), ctypes.byref(ut))
        return uc.value, ut.value
