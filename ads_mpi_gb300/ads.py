"""Python mirror of the reference's ADSS module over the C-ABI (include/ads_gpu.h).

The reference drives a time step with ``initialize(n, p, ads, ads_data,
mierr)``, ``Step(iter, RHS_fun, ads, ads_data, l2norm, mierr)`` and
``Cleanup(ads, ads_data, mierr)`` (src/ADS.F90:11, :437, :802).  ``ADS`` keeps
those names and argument meanings; the RHS_fun callback is replaced by
``set_form`` (an integrand form plus per-quadrature-point arrays), since a GPU
kernel cannot call back into host code.  Errors are raised as ``ADSError``
carrying the C status code; the library never exits the process.
"""
import ctypes
import os

import numpy as np

from . import build as _build

PREC_FP64 = 0
PREC_MIXED = 1
PREC_MIXED_FAST = 2
FORM_PROJECT = 0
FORM_HEAT = 1
FORM_OIL = 2
REORDER_FOR_Y = 0
REORDER_FOR_Z = 1
REORDER_FOR_X = 2

_lib = None
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


class ADSError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"ADS status {status}: {msg}")
        self.status = status


class Opts(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int), ("refine_tol", ctypes.c_double),
                ("max_refine", ctypes.c_int), ("device", ctypes.c_int)]


class Stats(ctypes.Structure):
    _fields_ = [("l2norm", ctypes.c_double), ("rel_residual", ctypes.c_double),
                ("refinements", ctypes.c_int), ("converged", ctypes.c_int), ("fp64_residuals", ctypes.c_int),
                ("host_path", ctypes.c_int)]


# (name, argtypes, restype) of every entry point declared in include/ads_gpu.h
ABI = [
    ("ads_default_opts", [ctypes.POINTER(Opts)], ctypes.c_int),
    ("ads_create", [_ip, _ip, ctypes.POINTER(Opts), ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    ("ads_destroy", [ctypes.c_void_p], ctypes.c_int),
    ("ads_last_error", [ctypes.c_void_p], ctypes.c_char_p),
    ("ads_status_string", [ctypes.c_int], ctypes.c_char_p),
    ("ads_dims", [ctypes.c_void_p, _ip, _ip, _ip], ctypes.c_int),
    ("ads_qp_points", [ctypes.c_void_p, ctypes.c_int, _dp], ctypes.c_int),
    ("ads_axis_tables", [ctypes.c_void_p, ctypes.c_int, _dp, _ip, _dp, _dp, _dp], ctypes.c_int),
    ("ads_set_form", [ctypes.c_void_p, ctypes.c_int, _dp, _dp, ctypes.c_double, ctypes.c_double], ctypes.c_int),
    ("ads_set_oil", [ctypes.c_void_p, _dp, ctypes.c_double], ctypes.c_int),
    ("ads_get_drained", [ctypes.c_void_p, _dp], ctypes.c_int),
    ("ads_save_spline_plot", [ctypes.c_void_p, ctypes.c_char_p, _dp, _ip, _dp], ctypes.c_int),
    ("ads_write_vti", [ctypes.c_char_p, _ip, _dp], ctypes.c_int),
    ("ads_set_coeffs", [ctypes.c_void_p, _dp], ctypes.c_int),
    ("ads_get_coeffs", [ctypes.c_void_p, _dp], ctypes.c_int),
    ("ads_step", [ctypes.c_void_p, _dp], ctypes.c_int),
    ("ads_step_host", [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, _dp], ctypes.c_int),
    ("ads_steps", [ctypes.c_void_p, ctypes.c_int, _dp], ctypes.c_int),
    ("ads_multistep", [ctypes.c_void_p, _dp, _dp], ctypes.c_int),
    ("ads_get_stats", [ctypes.c_void_p, ctypes.POINTER(Stats)], ctypes.c_int),
    ("ads_assemble", [ctypes.c_void_p, _dp, _dp], ctypes.c_int),
    ("ads_solve", [ctypes.c_void_p, _dp, _dp], ctypes.c_int),
    ("ads_apply_mass", [ctypes.c_void_p, _dp, _dp], ctypes.c_int),
    ("ads_reorder", [ctypes.c_void_p, ctypes.c_int, _dp, _dp], ctypes.c_int),
    ("ads_set_coeffs_device", [ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    ("ads_get_coeffs_device", [ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    ("ads_residual_noalloc", [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, _dp],
     ctypes.c_int),
    ("ads_heat_adjoint", [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, _dp, _dp], ctypes.c_int),
    ("ads_heat_jvp", [ctypes.c_void_p, ctypes.c_int, _dp, _dp, _dp, _dp, _dp], ctypes.c_int),
    ("ads_axis_setup", [ctypes.c_int, ctypes.c_int, _dp, _ip, _dp, _dp, _dp, _dp, _dp, _dp, _dp], ctypes.c_int),
    ("ads_fma_peak", [ctypes.c_int, ctypes.c_int, _dp], ctypes.c_int),
    ("ads_get_stream", [ctypes.c_void_p], ctypes.c_void_p),
    ("ads_set_stream", [ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    ("ads_timing_enable", [ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
    ("ads_timing_read", [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, _dp, _ip, ctypes.c_int, _ip], ctypes.c_int),
    ("ads_timing_reset", [ctypes.c_void_p], ctypes.c_int),
    ("ads_phase_timing_read", [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, _dp, _ip, ctypes.c_int, _ip],
     ctypes.c_int),
    ("ads_launch_count", [ctypes.c_void_p], ctypes.c_longlong),
    ("ads_launch_count_reset", [ctypes.c_void_p], ctypes.c_int),
]


def write_vti(name, vals):
    """VtkOutput (src/vtk.F90:15-77): vals shaped (resz, resy, resx) into name.vti."""
    v = np.ascontiguousarray(vals, dtype=np.float64)
    res = np.array([v.shape[2], v.shape[1], v.shape[0]], dtype=np.int32)
    st = load().ads_write_vti(os.fsencode(name), res.ctypes.data_as(_ip), v.ctypes.data_as(_dp))
    if st != 0:
        raise ADSError(st, f"cannot write {name}.vti")


def lib_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load libadsgpu.so (building it first if it is missing or stale)."""
    global _lib
    if _lib is None:
        path = _build.LIB
        if build_if_missing:
            _build.build()
        if not os.path.exists(path):
            raise ADSError(-1, f"CUDA extension {path} is missing; run ads_mpi_gb300.build.build()")
        L = ctypes.CDLL(path)
        for name, args, res in ABI:
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def _ptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(_dp)


def _c64(a):
    return np.ascontiguousarray(a, dtype=np.float64).ravel()


def axis_setup(n, p):
    """Host setup tables of one axis (no GPU needed); see ads_axis_setup in include/ads_gpu.h."""
    L = load()
    E = n - p + 1
    q = p + 1
    U = np.zeros(n + p + 2)
    O = np.zeros(E, dtype=np.int32)
    J = np.zeros(E)
    W = np.zeros(q)
    X = np.zeros(E * q)
    NN = np.zeros(E * q * (p + 1) * 2)
    band = np.zeros((2 * p + 1) * (n + 1))
    fac = np.zeros((2 * p + 2) * (n + 1))
    tfac = np.zeros((2 * p + 2) * (n + 1))
    st = L.ads_axis_setup(n, p, _ptr(U), O.ctypes.data_as(_ip), _ptr(J), _ptr(W), _ptr(X), _ptr(NN),
                          _ptr(band), _ptr(fac), _ptr(tfac))
    if st != 0:
        raise ADSError(st, L.ads_status_string(st).decode())
    return dict(U=U, O=O, J=J, W=W, X=X.reshape(E, q), NN=NN.reshape(E, q, p + 1, 2),
                band=band.reshape(2 * p + 1, n + 1), fac=fac.reshape(2 * p + 2, n + 1),
                tfac=tfac.reshape(2 * p + 2, n + 1))


def fma_peak(fp64, device=0):
    """Measured FP32/FP64 FMA throughput of a device in TFLOP/s (diagnostic)."""
    L = load()
    t = ctypes.c_double(0.0)
    st = L.ads_fma_peak(device, int(bool(fp64)), ctypes.byref(t))
    if st != 0:
        raise ADSError(st, L.ads_status_string(st).decode())
    return t.value


class ADS:
    """One ADS configuration on one GPU (ADS_setup + ADS_compute_data of one rank)."""

    def __init__(self, n, p, precision=PREC_FP64, refine_tol=1e-13, max_refine=3, device=0):
        L = load()
        o = Opts()
        L.ads_default_opts(ctypes.byref(o))
        o.precision = precision
        o.refine_tol = refine_tol
        o.max_refine = max_refine
        o.device = device
        n3 = (ctypes.c_int * 3)(*n)
        p3 = (ctypes.c_int * 3)(*p)
        h = ctypes.c_void_p()
        st = L.ads_create(n3, p3, ctypes.byref(o), ctypes.byref(h))
        if st != 0:
            raise ADSError(st, L.ads_status_string(st).decode())
        self._L = L
        self.h = h
        ne = (ctypes.c_int * 3)()
        nd = (ctypes.c_int * 3)()
        nq = (ctypes.c_int * 3)()
        L.ads_dims(h, ne, nd, nq)
        self.nelem, self.ndof, self.nq = tuple(ne), tuple(nd), tuple(nq)
        self.n, self.p = tuple(n), tuple(p)
        self.precision = precision
        self.N = int(np.prod(self.ndof))
        self.nqp = int(np.prod(self.nelem)) * int(np.prod(self.nq))

    # reference name: initialize (src/ADS.F90:11)
    @classmethod
    def initialize(cls, n, p, **kw):
        return cls(n, p, **kw)

    def _check(self, st):
        if st != 0:
            msg = self._L.ads_last_error(self.h).decode() or self._L.ads_status_string(st).decode()
            raise ADSError(st, msg)

    # reference name: Cleanup (src/ADS.F90:802)
    def cleanup(self):
        if self.h:
            self._L.ads_destroy(self.h)
            self.h = None

    close = cleanup

    def __del__(self):
        try:
            self.cleanup()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.cleanup()

    def qp_points(self, axis):
        X = np.zeros(self.nelem[axis] * self.nq[axis])
        self._check(self._L.ads_qp_points(self.h, axis, _ptr(X)))
        return X.reshape(self.nelem[axis], self.nq[axis])

    def qp_coords(self):
        """x, y, z at every quadrature point, shaped (Ez, Ey, Ex, q, q, q) = the
        (kx,ky,kz,ex,ey,ez) column-major layout of the per-point arrays."""
        X, Y, Z = (self.qp_points(a) for a in range(3))
        x = X[None, None, :, None, None, :]
        y = Y[None, :, None, None, :, None]
        z = Z[:, None, None, :, None, None]
        shape = (self.nelem[2], self.nelem[1], self.nelem[0], self.nq[2], self.nq[1], self.nq[0])
        return (np.broadcast_to(x, shape), np.broadcast_to(y, shape), np.broadcast_to(z, shape))

    def axis_tables(self, axis):
        E, q, p = self.nelem[axis], self.nq[axis], self.p[axis]
        U = np.zeros(self.n[axis] + p + 2)
        O = np.zeros(E, dtype=np.int32)
        J = np.zeros(E)
        W = np.zeros(q)
        NN = np.zeros(E * q * (p + 1) * 2)
        self._check(self._L.ads_axis_tables(self.h, axis, _ptr(U), O.ctypes.data_as(_ip), _ptr(J), _ptr(W), _ptr(NN)))
        return dict(U=U, O=O, J=J, W=W, NN=NN.reshape(E, q, p + 1, 2))

    def set_form(self, form, f_qp=None, kappa_qp=None, kappa=1.0, dt=0.0):
        f = None if f_qp is None else _c64(f_qp)
        k = None if kappa_qp is None else _c64(kappa_qp)
        for a in (f, k):
            if a is not None and a.size != self.nqp:
                raise ValueError(f"per-point array must have {self.nqp} entries")
        self._check(self._L.ads_set_form(self.h, form, _ptr(f), _ptr(k), float(kappa), float(dt)))

    def set_oil(self, drain_qp, mu=10.0):
        """The oil problem's draining weight w at the points (draining(u, X) =
        w(X) u, problems/oil/input_data.F90:265-283) and mi (exp(mi u),
        :297-303); with set_form(FORM_OIL, f_qp=pumping, kappa_qp=Kq, dt=Dt)."""
        w = _c64(drain_qp)
        if w.size != self.nqp:
            raise ValueError(f"per-point array must have {self.nqp} entries")
        self._check(self._L.ads_set_oil(self.h, _ptr(w), float(mu)))

    def save_spline_plot(self, name=None, rng=(0.0, 1.0, 0.0, 1.0, 0.0, 1.0), res=(31, 31, 31)):
        """SaveSplinePlot (src/plot.F90:111-140) of the current coefficients:
        the spline at an res grid over rng, returned shaped (resz, resy, resx)
        and, with a name, written to name.vti as VtkOutput does."""
        r = np.ascontiguousarray(rng, dtype=np.float64)
        rs = np.ascontiguousarray(res, dtype=np.int32)
        vals = np.zeros(int(np.prod(res)))
        nm = None if name is None else os.fsencode(name)
        self._check(self._L.ads_save_spline_plot(self.h, nm, _ptr(r), rs.ctypes.data_as(_ip), _ptr(vals)))
        return vals.reshape(res[2], res[1], res[0])

    # reference name: PrintSolution (src/ADS.F90:955-989)
    def print_solution(self, iter, directory="."):
        """The solution sampled on 31^3 points of [0,1]^3 into <directory>/step<iter>.vti."""
        return self.save_spline_plot(os.path.join(directory, f"step{iter}"))

    def drained(self):
        """The oil problem's drained total since set_oil (ComputeResults)."""
        v = ctypes.c_double(0.0)
        self._check(self._L.ads_get_drained(self.h, ctypes.byref(v)))
        return v.value

    def set_coeffs(self, u):
        u = _c64(u)
        if u.size != self.N:
            raise ValueError(f"coefficients must have {self.N} entries")
        self._check(self._L.ads_set_coeffs(self.h, _ptr(u)))

    def coeffs(self):
        u = np.zeros(self.N)
        self._check(self._L.ads_get_coeffs(self.h, _ptr(u)))
        return u

    def coeffs_into(self, out):
        """Copy the coefficients into a caller-provided contiguous float64 array."""
        if out.dtype != np.float64 or not out.flags["C_CONTIGUOUS"] or out.size != self.N:
            raise ValueError("out must be a contiguous float64 array of ndof entries")
        self._check(self._L.ads_get_coeffs(self.h, _ptr(out)))
        return out

    # reference name: Step (src/ADS.F90:437); returns l2norm
    def step(self):
        l2 = ctypes.c_double(0.0)
        self._check(self._L.ads_step(self.h, ctypes.byref(l2)))
        return l2.value

    def step_host(self, u, out=None):
        """One Step from the float64 array u into out (u itself when out is
        None, the reference's in-place Step); returns l2norm.  Pinned (or, where
        the device reads pageable memory, any) host arrays are read and written
        in place by the step's kernels."""
        out = u if out is None else out
        for a in (u, out):
            if not isinstance(a, np.ndarray) or a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"] \
                    or a.size != self.N:
                raise ValueError("u and out must be contiguous float64 arrays of ndof entries")
        if not out.flags["WRITEABLE"]:
            raise ValueError("out must be writeable")
        l2 = ctypes.c_double(0.0)
        self._check(self._L.ads_step_host(self.h, ctypes.c_void_p(u.ctypes.data), ctypes.c_void_p(out.ctypes.data),
                                          ctypes.byref(l2)))
        return l2.value

    def steps(self, k):
        out = np.zeros(max(k, 1))
        self._check(self._L.ads_steps(self.h, k, _ptr(out)))
        return out[:k]

    # reference name: MultiStep (src/ADS.F90:391-429); returns l2norm
    def multistep(self, mix):
        """Three substeps with the 1-D matrix mixes mix[s] = (M, K, B, BT)
        weights of substep s (the reference's mix(4,3), one row per substep)."""
        m = np.ascontiguousarray(mix, dtype=np.float64).reshape(3, 4)
        l2 = ctypes.c_double(0.0)
        self._check(self._L.ads_multistep(self.h, _ptr(m), ctypes.byref(l2)))
        return l2.value

    def stats(self):
        s = Stats()
        self._check(self._L.ads_get_stats(self.h, ctypes.byref(s)))
        return dict(l2norm=s.l2norm, rel_residual=s.rel_residual, refinements=s.refinements,
                    converged=bool(s.converged), fp64_residuals=s.fp64_residuals, host_path=s.host_path)

    def assemble(self):
        F = np.zeros(self.N)
        l2 = ctypes.c_double(0.0)
        self._check(self._L.ads_assemble(self.h, _ptr(F), ctypes.byref(l2)))
        return F, l2.value

    def solve(self, F):
        F = _c64(F)
        u = np.zeros(self.N)
        self._check(self._L.ads_solve(self.h, _ptr(F), _ptr(u)))
        return u

    def apply_mass(self, u):
        u = _c64(u)
        out = np.zeros(self.N)
        self._check(self._L.ads_apply_mass(self.h, _ptr(u), _ptr(out)))
        return out

    def reorder(self, kind, arr):
        a = _c64(arr)
        out = np.zeros_like(a)
        self._check(self._L.ads_reorder(self.h, kind, _ptr(a), _ptr(out)))
        return out

    def heat_adjoint(self, K, checkpoint_every, u0, u_target, grad=True, grad_kappa=False):
        u0 = _c64(u0)
        ut = _c64(u_target)
        loss = ctypes.c_double(0.0)
        g = np.zeros(self.N) if grad else None
        gk = np.zeros(self.nqp) if grad_kappa else None
        self._check(self._L.ads_heat_adjoint(self.h, K, checkpoint_every, _ptr(u0), _ptr(ut),
                                             ctypes.byref(loss), _ptr(g), _ptr(gk)))
        return loss.value, g, gk

    def heat_jvp(self, K, u0, du0=None, dkappa=None):
        """Tangent-linear model of K heat steps: (u^K, du^K) with du^K the
        derivative of u^K along du0 (initial state) and dkappa (per-point
        conductivity, quadrature-point layout); either may be None."""
        u0 = _c64(u0)
        du0 = None if du0 is None else _c64(du0)
        dk = None if dkappa is None else _c64(dkappa)
        uK = np.zeros(self.N)
        duK = np.zeros(self.N)
        self._check(self._L.ads_heat_jvp(self.h, K, _ptr(u0), _ptr(du0), _ptr(dk), _ptr(uK), _ptr(duK)))
        return uK, duK

    # device interop
    def stream(self):
        return self._L.ads_get_stream(self.h)

    def set_stream(self, ptr):
        self._check(self._L.ads_set_stream(self.h, ctypes.c_void_p(ptr)))

    def set_coeffs_device(self, ptr):
        self._check(self._L.ads_set_coeffs_device(self.h, ctypes.c_void_p(ptr)))

    def get_coeffs_device(self, ptr):
        self._check(self._L.ads_get_coeffs_device(self.h, ctypes.c_void_p(ptr)))

    def timing(self, on=True):
        self._check(self._L.ads_timing_enable(self.h, int(on)))

    def timing_reset(self):
        self._check(self._L.ads_timing_reset(self.h))

    def timing_read(self, max_kernels=64):
        names = ctypes.create_string_buffer(8192)
        t = np.zeros(max_kernels)
        c = np.zeros(max_kernels, dtype=np.int32)
        n = ctypes.c_int(0)
        self._check(self._L.ads_timing_read(self.h, names, 8192, _ptr(t), c.ctypes.data_as(_ip), max_kernels,
                                            ctypes.byref(n)))
        nm = names.value.decode().split(",") if n.value else []
        return {nm[i]: (float(t[i]), int(c[i])) for i in range(n.value)}

    def phase_timing_read(self, max_phases=16):
        """Per-phase CUDA-event totals {name: (ms, launches)} under the
        reference's PERFORMANCE names ("Form 3D RHS", "Solve 1", ...)."""
        names = ctypes.create_string_buffer(1024)
        t = np.zeros(max_phases)
        c = np.zeros(max_phases, dtype=np.int32)
        n = ctypes.c_int(0)
        self._check(self._L.ads_phase_timing_read(self.h, names, 1024, _ptr(t), c.ctypes.data_as(_ip), max_phases,
                                                  ctypes.byref(n)))
        nm = names.value.decode().split(",") if n.value else []
        return {nm[i]: (float(t[i]), int(c[i])) for i in range(n.value)}

    def launch_count(self):
        return int(self._L.ads_launch_count(self.h))

    def launch_count_reset(self):
        self._check(self._L.ads_launch_count_reset(self.h))
