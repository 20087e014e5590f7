"""Python binding of the GB300 pipe-flow stepper (libnspipe_gb300.so, include/nspipe_gb300.h).

Host-side mirror of the nsPipe-CUDA driver interface: parameters as in head.h,
the (u_r, u_theta, u_z) spectral state as complex128 arrays of shape
(NR, NT, NZ) (the reference's double2[NR][NT][NZ] layout), restart files in the
reference's raw format, and the per-step entry points.  All numerics run in the
CUDA library; if it is missing this module raises instead of falling back.
"""
import ctypes
import json
import os

import numpy as np

from .initfield import PI2, radial_grid, read_state, seeded_field, write_state  # noqa: F401

_HERE = os.path.dirname(os.path.abspath(__file__))
# $NSP_LIBRARY selects another build of the library, e.g. the bounds-checked
# libnspipe_gb300_bc.so (nspipe-gpu_gb300/build.py --bounds-check).
LIB_PATH = os.environ.get("NSP_LIBRARY") or os.path.join(os.path.dirname(_HERE), "libnspipe_gb300.so")

(NSP_OK, NSP_ERR_ARG, NSP_ERR_CUDA, NSP_ERR_IO, NSP_ERR_NONFINITE, NSP_ERR_STATE, NSP_ERR_NOMEM, NSP_ERR_DEVICE,
 NSP_ERR_MAXIT) = range(9)
NSP_FP64, NSP_MIXED = 0, 1

EXPORTS = [
    "nsp_default_params", "nsp_create", "nsp_setup", "nsp_load_state", "nsp_save_state",
    "nsp_set_state_host", "nsp_get_state_host", "nsp_set_state_device", "nsp_get_state_device",
    "nsp_step", "nsp_nonlinear", "nsp_lusolve", "nsp_diag", "nsp_grid", "nsp_kernel_launches",
    "nsp_sync", "nsp_last_error", "nsp_destroy", "nsp_set_stream", "nsp_profile_stages",
    "nsp_measure_fp64_peak", "nsp_nonlinear_static", "nsp_describe", "nsp_mean_profile", "nsp_cross_sections",
    "nsp_get_params", "nsp_info", "nsp_run_default_opts", "nsp_run_open", "nsp_run_resume", "nsp_run_advance",
    "nsp_run_checkpoint", "nsp_run_time", "nsp_run_close", "nsp_checkpoint_info", "nsp_output_schedule",
    "nsp_remesh_create", "nsp_remesh_matrix", "nsp_remesh_device", "nsp_remesh_members", "nsp_remesh_files",
    "nsp_remesh_destroy", "nsp_step_host", "nsp_diag_all", "nsp_mean_profile_all", "nsp_cross_sections_all",
    "nsp_debug_inject", "nsp_set_strict", "nsp_profile_linear", "nsp_bounds_report",
]


class NspParams(ctypes.Structure):
    _fields_ = [
        ("NR", ctypes.c_int), ("NT", ctypes.c_int), ("NZ", ctypes.c_int),
        ("LT", ctypes.c_double), ("LZ", ctypes.c_double),
        ("Re", ctypes.c_double), ("dt", ctypes.c_double), ("d_im", ctypes.c_double),
        ("maxit", ctypes.c_int), ("tol", ctypes.c_double), ("sten", ctypes.c_int),
        ("Qdes", ctypes.c_double),
    ]


class NspDiag(ctypes.Structure):
    _fields_ = [
        ("u_centre", ctypes.c_double), ("u_tau", ctypes.c_double), ("flux", ctypes.c_double),
        ("last_err", ctypes.c_double), ("last_iters", ctypes.c_int), ("status", ctypes.c_int),
        ("re_tau", ctypes.c_double), ("div_max", ctypes.c_double), ("div_wall", ctypes.c_double),
        ("unconverged_steps", ctypes.c_int),
    ]


class NspRunOpts(ctypes.Structure):
    _fields_ = [
        ("out_dir", ctypes.c_char_p), ("dt_frc", ctypes.c_double), ("dt_qcr", ctypes.c_double),
        ("dt_mnp", ctypes.c_double), ("rows_per_write", ctypes.c_int), ("ckpt_dir", ctypes.c_char_p),
        ("ckpt_every", ctypes.c_int), ("ckpt_keep", ctypes.c_int), ("final_state", ctypes.c_int),
        ("verbose", ctypes.c_int),
    ]


class NspError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("nspipe error %d: %s" % (code, msg))
        self.code = code


_LIB = None


def lib():
    """Load libnspipe_gb300.so (raises if it has not been built)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("%s not found: run nspipe-gpu_gb300/build.py" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        vp, ip, dp = ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)
        L.nsp_default_params.argtypes = [ctypes.POINTER(NspParams)]
        L.nsp_create.argtypes = [ctypes.POINTER(NspParams), ip, ip, ip, ctypes.POINTER(vp)]
        L.nsp_setup.argtypes = [vp]
        L.nsp_load_state.argtypes = [vp, ip, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p]
        L.nsp_save_state.argtypes = [vp, ip, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p]
        L.nsp_set_state_host.argtypes = [vp, ip, dp, dp, dp]
        L.nsp_get_state_host.argtypes = [vp, ip, dp, dp, dp]
        L.nsp_set_state_device.argtypes = [vp, ip, vp, vp, vp]
        L.nsp_get_state_device.argtypes = [vp, ip, vp, vp, vp]
        L.nsp_step.argtypes = [vp, ip, ctypes.POINTER(ctypes.c_int)]
        L.nsp_step_host.argtypes = [vp, ip, dp, dp, ctypes.POINTER(ctypes.c_int)]
        L.nsp_nonlinear.argtypes = [vp, ip, vp, vp, vp, vp, vp, vp]
        L.nsp_lusolve.argtypes = [vp, ip, ip, vp, vp]
        L.nsp_diag.argtypes = [vp, ip, ctypes.POINTER(NspDiag)]
        L.nsp_grid.argtypes = [vp, ip, dp, dp]
        L.nsp_kernel_launches.argtypes = [vp]
        L.nsp_kernel_launches.restype = ctypes.c_longlong
        L.nsp_sync.argtypes = [vp]
        L.nsp_set_stream.argtypes = [vp, vp]
        L.nsp_profile_stages.argtypes = [vp, ip, dp]
        L.nsp_measure_fp64_peak.argtypes = [vp, dp]
        L.nsp_nonlinear_static.argtypes = [vp, ip, vp, vp]
        L.nsp_describe.argtypes = [vp, ctypes.c_char_p, ip]
        L.nsp_mean_profile.argtypes = [vp, ip, dp]
        L.nsp_diag_all.argtypes = [vp, ctypes.POINTER(NspDiag)]
        L.nsp_mean_profile_all.argtypes = [vp, dp]
        L.nsp_cross_sections_all.argtypes = [vp, dp, dp]
        L.nsp_cross_sections.argtypes = [vp, ip, dp, dp]
        L.nsp_get_params.argtypes = [vp, ip, ctypes.POINTER(NspParams)]
        L.nsp_info.argtypes = [vp, ctypes.POINTER(ip), ctypes.POINTER(ip)]
        L.nsp_run_default_opts.argtypes = [ctypes.POINTER(NspRunOpts)]
        L.nsp_run_open.argtypes = [vp, ctypes.POINTER(NspRunOpts), ctypes.POINTER(vp)]
        L.nsp_run_resume.argtypes = [vp, ctypes.POINTER(NspRunOpts), ctypes.c_char_p, ctypes.POINTER(vp)]
        L.nsp_run_advance.argtypes = [vp, ip, ctypes.POINTER(ip)]
        L.nsp_run_checkpoint.argtypes = [vp]
        L.nsp_run_time.argtypes = [vp, ip, dp, ctypes.POINTER(ctypes.c_longlong)]
        L.nsp_run_close.argtypes = [vp]
        L.nsp_checkpoint_info.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ip, ctypes.c_char_p, ip]
        L.nsp_output_schedule.argtypes = [ctypes.c_double, ctypes.c_double, ip, dp, ctypes.POINTER(ctypes.c_ubyte)]
        L.nsp_remesh_create.argtypes = [ip, ip, ip, ip, ip, ip, ip, ip, ctypes.POINTER(vp)]
        L.nsp_remesh_matrix.argtypes = [vp, dp]
        L.nsp_remesh_device.argtypes = [vp, ip, ctypes.POINTER(vp), ctypes.POINTER(vp), vp]
        L.nsp_remesh_members.argtypes = [vp, vp, ctypes.POINTER(ip), vp, ctypes.POINTER(ip), ip]
        L.nsp_remesh_files.argtypes = [vp, ctypes.c_char_p, ctypes.c_char_p]
        L.nsp_remesh_destroy.argtypes = [vp]
        L.nsp_debug_inject.argtypes = [vp, ip]
        L.nsp_set_strict.argtypes = [vp, ip]
        L.nsp_profile_linear.argtypes = [vp, ip, dp]
        L.nsp_bounds_report.argtypes = [vp, ctypes.POINTER(ctypes.c_longlong)]
        L.nsp_last_error.argtypes = [vp]
        L.nsp_last_error.restype = ctypes.c_char_p
        L.nsp_destroy.argtypes = [vp]
        _LIB = L
    return _LIB


def default_params(**kw):
    """Reference defaults (head.h:16-61) with keyword overrides."""
    p = NspParams()
    lib().nsp_default_params(ctypes.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def make_params(NR, NT, NZ, Re, dt, LZ, LT=PI2, d_im=0.51, maxit=10, tol=5e-8, Qdes=0.5):
    return default_params(NR=NR, NT=NT, NZ=NZ, Re=float(Re), dt=float(dt), LZ=float(LZ), LT=float(LT),
                          d_im=d_im, maxit=maxit, tol=tol, Qdes=Qdes)


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ptr(x):
    return x if isinstance(x, int) else x.data_ptr()


class Stepper:
    """An ensemble of independent pipes advanced together on one GPU."""

    def __init__(self, params, precision=NSP_FP64, device=0, setup=True):
        if isinstance(params, NspParams):
            params = [params]
        self.params = list(params)
        self.n = len(self.params)
        self._total = sum(p.NR * p.NT * p.NZ for p in self.params)  # values per component, all members
        arr = (NspParams * self.n)(*self.params)
        self._h = ctypes.c_void_p()
        rc = lib().nsp_create(arr, self.n, precision, device, ctypes.byref(self._h))
        if rc != NSP_OK:
            msg = self.last_error()
            self.close()
            raise NspError(rc, msg)
        self.precision = precision
        if setup:
            self._check(lib().nsp_setup(self._h))

    # -- plumbing
    def last_error(self):
        return lib().nsp_last_error(self._h).decode() if self._h else "closed"

    def _check(self, rc):
        if rc != NSP_OK:
            raise NspError(rc, self.last_error())
        return rc

    def close(self):
        if self._h:
            lib().nsp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def shape(self, m=0):
        p = self.params[m]
        return (p.NR, p.NT, p.NZ)

    # -- state
    def set_state(self, m, u):
        u = [np.ascontiguousarray(a, np.complex128) for a in u]
        for a in u:
            if a.shape != self.shape(m):
                raise ValueError("state shape %s != %s" % (a.shape, self.shape(m)))
        self._check(lib().nsp_set_state_host(self._h, m, _dp(u[0]), _dp(u[1]), _dp(u[2])))

    def get_state(self, m, out=None):
        u = out if out is not None else [np.zeros(self.shape(m), np.complex128) for _ in range(3)]
        for a in u:
            if a.dtype != np.complex128 or not a.flags["C_CONTIGUOUS"] or a.size != int(np.prod(self.shape(m))):
                raise ValueError("output must be C-contiguous complex128 of the member's shape")
        self._check(lib().nsp_get_state_host(self._h, m, _dp(u[0]), _dp(u[1]), _dp(u[2])))
        return u

    def _all_size(self):
        return self._total

    def set_states_all(self, u_all):
        """All members at once: u_all[c] holds component c of every member back to back."""
        u_all = [np.ascontiguousarray(a, np.complex128) for a in u_all]
        for a in u_all:
            if a.size != self._all_size():
                raise ValueError("expected %d values per component" % self._all_size())
        self._check(lib().nsp_set_state_host(self._h, -1, _dp(u_all[0]), _dp(u_all[1]), _dp(u_all[2])))

    def get_states_all(self, out=None):
        u = out if out is not None else [np.zeros(self._all_size(), np.complex128) for _ in range(3)]
        for a in u:
            if a.dtype != np.complex128 or not a.flags["C_CONTIGUOUS"] or a.size != self._all_size():
                raise ValueError("output must be C-contiguous complex128 with every member")
        self._check(lib().nsp_get_state_host(self._h, -1, _dp(u[0]), _dp(u[1]), _dp(u[2])))
        return u

    def set_state_device(self, m, ur, ut, uz):
        self._check(lib().nsp_set_state_device(self._h, m, _ptr(ur), _ptr(ut), _ptr(uz)))

    def get_state_device(self, m, ur, ut, uz):
        self._check(lib().nsp_get_state_device(self._h, m, _ptr(ur), _ptr(ut), _ptr(uz)))

    def load(self, m, directory, suffix="_s"):
        f = [os.path.join(directory, "u%s%s.bin" % (c, suffix)).encode() for c in "rtz"]
        self._check(lib().nsp_load_state(self._h, m, *f))

    def save(self, m, directory, suffix=""):
        os.makedirs(directory, exist_ok=True)
        f = [os.path.join(directory, "u%s%s.bin" % (c, suffix)).encode() for c in "rtz"]
        self._check(lib().nsp_save_state(self._h, m, *f))

    # -- stepping and operators
    def step(self, nsteps=1, check=True):
        iters = np.zeros((nsteps, self.n), np.int32)
        rc = lib().nsp_step(self._h, nsteps, iters.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
        if check:
            self._check(rc)
        return iters

    def member_major_size(self):
        return 3 * self._all_size()

    def pack(self, fields):
        """Member-major array (each member's u_r, u_theta, u_z back to back) of per-member fields."""
        return np.concatenate([np.ascontiguousarray(a, np.complex128).reshape(-1) for f in fields for a in f])

    def unpack(self, flat):
        """Per-member [u_r, u_theta, u_z] views of a member-major array."""
        out, off = [], 0
        for m in range(self.n):
            n = int(np.prod(self.shape(m)))
            out.append([flat[off + c * n: off + (c + 1) * n].reshape(self.shape(m)) for c in range(3)])
            off += 3 * n
        return out

    def step_host(self, nsteps, u, out=None, check=True):
        """Host-resident steps (nsp_step_host) on a member-major array; returns (out, iters).
        Copies overlap compute member chunk by chunk (pin the arrays for the overlap)."""
        u = np.ascontiguousarray(u, np.complex128)
        out = out if out is not None else np.zeros(self.member_major_size(), np.complex128)
        for a in (u, out):
            if a.size != self.member_major_size() or a.dtype != np.complex128 or not a.flags["C_CONTIGUOUS"]:
                raise ValueError("expected C-contiguous complex128 arrays of %d values" % self.member_major_size())
        iters = np.zeros((nsteps, self.n), np.int32)
        rc = lib().nsp_step_host(self._h, nsteps, _dp(u), _dp(out), iters.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
        if check:
            self._check(rc)
        return out, iters

    def kernel_launches(self):
        return lib().nsp_kernel_launches(self._h)

    def describe(self):
        """Execution choices of the context (precision, graph, per-group block shape, theta path)."""
        buf = ctypes.create_string_buffer(4096)
        self._check(lib().nsp_describe(self._h, buf, len(buf)))
        return json.loads(buf.value.decode())

    def nonlinear(self, m, u_dev, n_dev):
        self._check(lib().nsp_nonlinear(self._h, m, *[_ptr(a) for a in u_dev], *[_ptr(a) for a in n_dev]))

    def nonlinear_static(self, m, u3_dev, n3_dev):
        """Nonlinear term without device allocation; u3/n3 hold (r, theta, z) back to back."""
        self._check(lib().nsp_nonlinear_static(self._h, m, _ptr(u3_dev), _ptr(n3_dev)))

    def lusolve(self, m, kind, rhs_dev, sol_dev):
        self._check(lib().nsp_lusolve(self._h, m, kind, _ptr(rhs_dev), _ptr(sol_dev)))

    def diag(self, m):
        d = NspDiag()
        self._check(lib().nsp_diag(self._h, m, ctypes.byref(d)))
        return d

    def friction(self, m=0):
        """(u_centre, u_tau) of member m (nsp_diag): the data of the friction file's rows."""
        d = self.diag(m)
        return d.u_centre, d.u_tau

    def mean_profile(self, m=0):
        """Re u_z(0,0)(r_i), i < NR (the data row of the reference's mean-profile file)."""
        out = np.zeros(self.params[m].NR)
        self._check(lib().nsp_mean_profile(self._h, m, _dp(out)))
        return out

    def cross_sections(self, m=0):
        """(q, u): r-integrated theta means of u_r^2 + u_theta^2 and of u_z^2 at the NZR
        physical axial points (the data rows of the reference's q / u cross-section files)."""
        nzr = 3 * (self.params[m].NZ - 1)
        q, u = np.zeros(nzr), np.zeros(nzr)
        self._check(lib().nsp_cross_sections(self._h, m, _dp(q), _dp(u)))
        return q, u

    def diag_all(self):
        """nsp_diag of every member in one pass: a list of NspDiag in member order."""
        out = (NspDiag * self.n)()
        self._check(lib().nsp_diag_all(self._h, out))
        return list(out)

    def mean_profile_all(self):
        """Mean profiles of every member (list of arrays of NR_m values)."""
        sizes = [p.NR for p in self.params]
        flat = np.zeros(sum(sizes))
        self._check(lib().nsp_mean_profile_all(self._h, _dp(flat)))
        return np.split(flat, np.cumsum(sizes)[:-1])

    def cross_sections_all(self):
        """(q, u) cross sections of every member (lists of arrays of NZR_m values)."""
        sizes = [3 * (p.NZ - 1) for p in self.params]
        q, u = np.zeros(sum(sizes)), np.zeros(sum(sizes))
        self._check(lib().nsp_cross_sections_all(self._h, _dp(q), _dp(u)))
        cut = np.cumsum(sizes)[:-1]
        return np.split(q, cut), np.split(u, cut)

    def grid(self, m=0):
        NR = self.params[m].NR
        r, rdr = np.zeros(NR), np.zeros(NR)
        self._check(lib().nsp_grid(self._h, m, _dp(r), _dp(rdr)))
        return r, rdr

    def set_stream(self, stream_handle):
        """Launch on a given cudaStream_t (int handle, e.g. torch.cuda.Stream().cuda_stream)."""
        self._check(lib().nsp_set_stream(self._h, stream_handle or None))

    def profile_stages(self, reps=5):
        """Average ms per launch: [theta-inverse, z stage, theta-forward, linear pass, converge]."""
        ms = np.zeros(5)
        self._check(lib().nsp_profile_stages(self._h, reps, _dp(ms)))
        return ms

    def profile_linear(self, reps=5):
        """Average ms per launch of the linear pass: [predictor pass, corrector pass]."""
        ms = np.zeros(2)
        self._check(lib().nsp_profile_linear(self._h, reps, _dp(ms)))
        return ms

    def fp64_peak_tflops(self):
        """Measured FP64 multiply-add throughput of the device (TFLOP/s)."""
        t = ctypes.c_double()
        self._check(lib().nsp_measure_fp64_peak(self._h, ctypes.byref(t)))
        return t.value

    def bounds_report(self):
        """(violations, first site, its index, its extent, bounds-checked build?) of nsp_bounds_report."""
        out = (ctypes.c_longlong * 5)()
        self._check(lib().nsp_bounds_report(self._h, out))
        return tuple(out)

    def set_strict(self, strict=True):
        """Strict convergence: steps that stop at maxit with err > tol raise NSP_ERR_MAXIT."""
        self._check(lib().nsp_set_strict(self._h, int(bool(strict))))

    def debug_inject(self, flags):
        """Test hook of the device-side failure path (nsp_debug_inject)."""
        self._check(lib().nsp_debug_inject(self._h, flags))

    def sync(self):
        self._check(lib().nsp_sync(self._h))


def output_schedule(dt, interval, nsteps, acc=0.0):
    """The output cadence of the run driver: (due, acc) where due[j] is True when a row
    is written after step j+1 (accumulator += dt per step, row when >= interval)."""
    due = np.zeros(nsteps, np.uint8)
    a = ctypes.c_double(acc)
    rc = lib().nsp_output_schedule(dt, interval, nsteps, ctypes.byref(a),
                                   due.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)))
    if rc != NSP_OK:
        raise NspError(rc, "nsp_output_schedule")
    return due.astype(bool), a.value


def host_error():
    """Message of the last failed context-free call in this thread (nsp_last_error(NULL))."""
    return lib().nsp_last_error(None).decode()


def checkpoint_info(path):
    """(sidecar dict, resolved checkpoint directory) of a checkpoint, after checking its
    state files against the sidecar; NspError(NSP_ERR_IO) if missing or corrupt."""
    js = ctypes.create_string_buffer(1 << 20)
    where = ctypes.create_string_buffer(4096)
    rc = lib().nsp_checkpoint_info(os.fsencode(path), js, len(js), where, len(where))
    if rc != NSP_OK:
        raise NspError(rc, host_error())
    return json.loads(js.value.decode()), where.value.decode()


class Run:
    """The reference's integrate() around a Stepper: the output files io_friction.txt,
    io_qcross.txt, io_ucross.txt, io_meanpr.txt at their cadence, periodic checkpoints
    with a JSON sidecar, and resume (include/nspipe_gb300.h, nsp_run_*).

    Keyword arguments are the fields of nsp_run_opts; resume= names a checkpoint (a
    step_* directory or a checkpoint directory) to continue from."""

    def __init__(self, stepper, out_dir=".", dt_frc=0.5, dt_qcr=0.5, dt_mnp=0.5, rows_per_write=100,
                 ckpt_dir=None, ckpt_every=0, ckpt_keep=2, final_state=True, verbose=False, resume=None):
        self.stepper = stepper
        o = NspRunOpts()
        lib().nsp_run_default_opts(ctypes.byref(o))
        self._strings = [os.fsencode(out_dir) if out_dir is not None else None,
                         os.fsencode(ckpt_dir) if ckpt_dir is not None else None]
        o.out_dir, o.ckpt_dir = self._strings
        o.dt_frc, o.dt_qcr, o.dt_mnp = float(dt_frc), float(dt_qcr), float(dt_mnp)
        o.rows_per_write, o.ckpt_every, o.ckpt_keep = rows_per_write, ckpt_every, ckpt_keep
        o.final_state, o.verbose = int(bool(final_state)), int(bool(verbose))
        self._h = ctypes.c_void_p()
        if resume is None:
            rc = lib().nsp_run_open(stepper._h, ctypes.byref(o), ctypes.byref(self._h))
        else:
            rc = lib().nsp_run_resume(stepper._h, ctypes.byref(o), os.fsencode(resume), ctypes.byref(self._h))
        stepper._check(rc)

    def advance(self, nsteps):
        iters = np.zeros((nsteps, self.stepper.n), np.int32)
        self.stepper._check(lib().nsp_run_advance(self._h, nsteps, iters.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
        return iters

    def checkpoint(self):
        self.stepper._check(lib().nsp_run_checkpoint(self._h))

    def time(self, m=0):
        t, n = ctypes.c_double(), ctypes.c_longlong()
        self.stepper._check(lib().nsp_run_time(self._h, m, ctypes.byref(t), ctypes.byref(n)))
        return t.value, n.value

    def close(self):
        if self._h:
            h, self._h = self._h, None
            self.stepper._check(lib().nsp_run_close(h))

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Remesh:
    """A Re_Mesh plan (nsp_remesh_*): fields of shape old = (NR, NT, NZ) to new =
    (Nrd, Ntd, Nzd), radial Lagrange interpolation on 2*iw points, theta / z modes
    truncated or zero-padded, batched over members in one launch."""

    def __init__(self, old, new, iw=3, device=0):
        self.old, self.new, self.iw = tuple(old), tuple(new), iw
        self._h = ctypes.c_void_p()
        rc = lib().nsp_remesh_create(*self.old, *self.new, iw, device, ctypes.byref(self._h))
        if rc != NSP_OK:
            raise NspError(rc, host_error())

    def _check(self, rc):
        if rc != NSP_OK:
            raise NspError(rc, host_error())

    def matrix(self):
        """RM[2][Nrd][NR]: 0 even folding, 1 odd folding."""
        out = np.zeros((2, self.new[0], self.old[0]))
        self._check(lib().nsp_remesh_matrix(self._h, _dp(out)))
        return out

    def device(self, src, dst, stream=None):
        """src / dst: sequences of device buffers (torch tensors or int pointers), each a
        member's three components back to back; one launch for all of them."""
        n = len(src)
        if len(dst) != n:
            raise ValueError("src and dst lengths differ")
        sp = (ctypes.c_void_p * max(n, 1))(*[_ptr(x) for x in src])
        dp_ = (ctypes.c_void_p * max(n, 1))(*[_ptr(x) for x in dst])
        self._check(lib().nsp_remesh_device(self._h, n, sp, dp_, stream))

    def members(self, src, src_members, dst, dst_members):
        """State of src member src_members[k] -> state of dst member dst_members[k]."""
        n = len(src_members)
        a = (ctypes.c_int * max(n, 1))(*src_members)
        b = (ctypes.c_int * max(n, 1))(*dst_members)
        rc = lib().nsp_remesh_members(self._h, src._h, a, dst._h, b, n)
        if rc != NSP_OK:
            raise NspError(rc, dst.last_error())

    def files(self, dir_in, dir_out):
        """The tool: u?_o.bin in dir_in -> u?_s.bin in dir_out."""
        self._check(lib().nsp_remesh_files(self._h, os.fsencode(dir_in), os.fsencode(dir_out)))

    def close(self):
        if self._h:
            lib().nsp_remesh_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
