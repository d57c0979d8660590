"""ctypes wrapper of the CPU oracle (test infrastructure only).

The oracle (oracle/ads_oracle.cpp) restates the IGA-ADS FP64 time-step path on
the CPU.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
import this module; the product (ads_mpi_gb300) never does.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lib = None

FORM_PROJECT = 0
FORM_HEAT = 1
FORM_OIL = 2

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def build(force=False):
    """Compile oracle/liboracle.so with oracle/Makefile."""
    if force or not os.path.exists(_LIB_PATH) or (
        os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "ads_oracle.cpp"))
    ):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        L.orc_fill_open_knot.argtypes = [ctypes.c_int, ctypes.c_int, _dp]
        L.orc_count_spans.argtypes = [ctypes.c_int, ctypes.c_int, _dp]
        L.orc_count_spans.restype = ctypes.c_int
        L.orc_prepare_knot.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _ip]
        L.orc_gauss_rule.argtypes = [ctypes.c_int, _dp, _dp]
        L.orc_ders_basis_funs.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int, _dp, _dp]
        L.orc_basis_data.argtypes = [ctypes.c_int, ctypes.c_int, _dp, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_int, _ip, _dp, _dp, _dp, _dp]
        L.orc_dgbsv.argtypes = [ctypes.c_int] * 4 + [_dp, ctypes.c_int, _ip, _dp, ctypes.c_int]
        L.orc_dgbsv.restype = ctypes.c_int
        L.orc_create.argtypes = [_ip, _ip]
        L.orc_create.restype = ctypes.c_void_p
        L.orc_destroy.argtypes = [ctypes.c_void_p]
        L.orc_dims.argtypes = [ctypes.c_void_p, _ip, _ip, _ip]
        L.orc_axis_tables.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _ip, _dp, _dp, _dp, _dp]
        L.orc_set_coeffs.argtypes = [ctypes.c_void_p, _dp]
        L.orc_get_coeffs.argtypes = [ctypes.c_void_p, _dp]
        L.orc_get_F.argtypes = [ctypes.c_void_p, _dp]
        L.orc_step.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _dp, ctypes.c_double,
                               ctypes.c_double, ctypes.c_int, _dp]
        L.orc_step.restype = ctypes.c_int
        L.orc_assemble.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _dp, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_int]
        L.orc_assemble.restype = ctypes.c_double
        L.orc_step_oil.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, ctypes.c_double, ctypes.c_double, _dp, _dp]
        L.orc_step_oil.restype = ctypes.c_int
        L.orc_assemble_oil.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, ctypes.c_double, ctypes.c_double, _dp]
        L.orc_assemble_oil.restype = ctypes.c_double
        L.orc_find_span.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, _dp]
        L.orc_find_span.restype = ctypes.c_int
        L.orc_eval_spline_grid.argtypes = [ctypes.c_void_p, _dp, _ip, _dp]
        L.orc_multistep.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _dp, ctypes.c_double, ctypes.c_double,
                                    _dp, _dp]
        L.orc_multistep.restype = ctypes.c_int
        L.orc_solve_F.argtypes = [ctypes.c_void_p, _dp]
        L.orc_solve_F.restype = ctypes.c_int
        L.orc_pivoted.argtypes = [ctypes.c_void_p, _ip]
        L.orc_heat_initial_qp.argtypes = [ctypes.c_void_p, _dp]
        L.orc_heat_initial_state.argtypes = [ctypes.c_double] * 3
        L.orc_heat_initial_state.restype = ctypes.c_double
        L.orc_mkbbt_band.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _dp]
        L.orc_apply_mass.argtypes = [ctypes.c_void_p, _dp, _dp]
        L.orc_heat_adjoint.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _dp, _dp,
                                       ctypes.c_double, ctypes.c_double, _dp, _dp, _dp]
        L.orc_heat_adjoint.restype = ctypes.c_int
        for nm in ("orc_reorder_for_y", "orc_reorder_for_z", "orc_reorder_for_x"):
            getattr(L, nm).argtypes = [_ip, _dp, _dp]
        L.orc_num_threads.restype = ctypes.c_int
        L.orc_set_num_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def _p(a, ty=_dp):
    if a is None:
        return None
    return a.ctypes.data_as(ty)


def fill_open_knot(n, p):
    U = np.zeros(max(n + p + 2, 0))
    lib().orc_fill_open_knot(n, p, _p(U))
    return U


def count_spans(n, p, U):
    U = np.ascontiguousarray(U, dtype=np.float64)
    return lib().orc_count_spans(n, p, _p(U))


def prepare_knot(n, p):
    U = np.zeros(max(n + p + 2, 0))
    ne = ctypes.c_int(0)
    lib().orc_prepare_knot(n, p, _p(U), ctypes.byref(ne))
    return U, ne.value


def gauss_rule(q):
    X = np.zeros(q)
    W = np.zeros(q)
    lib().orc_gauss_rule(q, _p(X), _p(W))
    return X, W


def dgbsv(A_band, kl, ku, B):
    """Banded solve; A_band in LAPACK layout (2kl+ku+1, n), B (n, nrhs)."""
    AB = np.asfortranarray(A_band, dtype=np.float64).copy(order="F")
    n = AB.shape[1]
    Bf = np.asfortranarray(B, dtype=np.float64).copy(order="F")
    if Bf.ndim == 1:
        Bf = Bf.reshape(n, 1, order="F")
    ipiv = np.zeros(n, dtype=np.int32)
    info = lib().orc_dgbsv(n, kl, ku, Bf.shape[1], _p(AB), AB.shape[0], _p(ipiv, _ip), _p(Bf), n)
    return info, Bf, ipiv


class Oracle:
    """One-rank restatement of initialize/Step/Cleanup (src/ADS.F90)."""

    def __init__(self, n, p):
        L = lib()
        n3 = (ctypes.c_int * 3)(*n)
        p3 = (ctypes.c_int * 3)(*p)
        self.h = L.orc_create(n3, p3)
        if not self.h:
            raise ValueError(f"oracle rejected n={n} p={p}")
        ne = (ctypes.c_int * 3)()
        nd = (ctypes.c_int * 3)()
        nq = (ctypes.c_int * 3)()
        L.orc_dims(self.h, ne, nd, nq)
        self.nelem, self.ndof, self.nq = tuple(ne), tuple(nd), tuple(nq)
        self.p = tuple(p)
        self.N = int(np.prod(self.ndof))
        self.nqp = int(np.prod(self.nelem)) * int(np.prod(self.nq))

    def close(self):
        if self.h:
            lib().orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def axis_tables(self, axis):
        E, q, p = self.nelem[axis], self.nq[axis], self.p[axis]
        n = self.ndof[axis] - 1
        U = np.zeros(n + p + 2)
        O = np.zeros(E, dtype=np.int32)
        J = np.zeros(E)
        W = np.zeros(q)
        X = np.zeros(q * E)
        NN = np.zeros(2 * (p + 1) * q * E)
        lib().orc_axis_tables(self.h, axis, _p(U), _p(O, _ip), _p(J), _p(W), _p(X), _p(NN))
        return dict(U=U, O=O, J=J, W=W, X=X.reshape(E, q), NN=NN.reshape(E, q, p + 1, 2))

    def set_coeffs(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64).ravel()
        assert u.size == self.N
        lib().orc_set_coeffs(self.h, _p(u))

    def coeffs(self):
        u = np.zeros(self.N)
        lib().orc_get_coeffs(self.h, _p(u))
        return u

    def F(self):
        u = np.zeros(self.N)
        lib().orc_get_F(self.h, _p(u))
        return u

    def step(self, form, fqp=None, kappa_qp=None, kappa=1.0, dt=0.0, heat_initial=False):
        fqp = None if fqp is None else np.ascontiguousarray(fqp, dtype=np.float64).ravel()
        kq = None if kappa_qp is None else np.ascontiguousarray(kappa_qp, dtype=np.float64).ravel()
        l2 = ctypes.c_double(0.0)
        info = lib().orc_step(self.h, form, _p(fqp), _p(kq), kappa, dt, int(heat_initial), ctypes.byref(l2))
        if info:
            raise RuntimeError(f"oracle step failed: info={info}")
        return l2.value

    def assemble(self, form, fqp=None, kappa_qp=None, kappa=1.0, dt=0.0, heat_initial=False):
        fqp = None if fqp is None else np.ascontiguousarray(fqp, dtype=np.float64).ravel()
        kq = None if kappa_qp is None else np.ascontiguousarray(kappa_qp, dtype=np.float64).ravel()
        l2 = lib().orc_assemble(self.h, form, _p(fqp), _p(kq), kappa, dt, int(heat_initial))
        return self.F(), l2

    def step_oil(self, pump_qp, kq_qp, drain_qp, mu, dt):
        """One oil-problem step (problems/oil/RHS_eq.F90:69-92); returns (l2norm, drained)."""
        arrs = [np.ascontiguousarray(a, dtype=np.float64).ravel() for a in (pump_qp, kq_qp, drain_qp)]
        l2, dr = ctypes.c_double(0.0), ctypes.c_double(0.0)
        info = lib().orc_step_oil(self.h, _p(arrs[0]), _p(arrs[1]), _p(arrs[2]), mu, dt, ctypes.byref(l2),
                                  ctypes.byref(dr))
        if info:
            raise RuntimeError(f"oracle step failed: info={info}")
        return l2.value, dr.value

    def assemble_oil(self, pump_qp, kq_qp, drain_qp, mu, dt):
        """The oil assembly only; returns (F, l2norm, drained)."""
        arrs = [np.ascontiguousarray(a, dtype=np.float64).ravel() for a in (pump_qp, kq_qp, drain_qp)]
        dr = ctypes.c_double(0.0)
        l2 = lib().orc_assemble_oil(self.h, _p(arrs[0]), _p(arrs[1]), _p(arrs[2]), mu, dt, ctypes.byref(dr))
        return self.F(), l2, dr.value

    def eval_spline_grid(self, rng=(0.0, 1.0, 0.0, 1.0, 0.0, 1.0), res=(31, 31, 31)):
        """SaveSplinePlot's samples of the current coefficients (x fastest), shaped (resz, resy, resx)."""
        r = np.ascontiguousarray(rng, dtype=np.float64)
        rs = np.ascontiguousarray(res, dtype=np.int32)
        vals = np.zeros(int(np.prod(res)))
        lib().orc_eval_spline_grid(self.h, _p(r), _p(rs, _ip), _p(vals))
        return vals.reshape(res[2], res[1], res[0])

    def multistep(self, form, mix, fqp=None, kappa_qp=None, kappa=1.0, dt=0.0):
        """MultiStep (src/ADS.F90:391-429) with mix(4,3) given as a (3, 4) array of
        substep rows (M, K, B, BT weights); returns the l2norm."""
        m = np.ascontiguousarray(mix, dtype=np.float64).ravel()
        fqp = None if fqp is None else np.ascontiguousarray(fqp, dtype=np.float64).ravel()
        kq = None if kappa_qp is None else np.ascontiguousarray(kappa_qp, dtype=np.float64).ravel()
        l2 = ctypes.c_double(0.0)
        info = lib().orc_multistep(self.h, form, _p(fqp), _p(kq), kappa, dt, _p(m), ctypes.byref(l2))
        if info:
            raise RuntimeError(f"oracle MultiStep failed: info={info}")
        return l2.value

    def solve(self, F):
        F = np.ascontiguousarray(F, dtype=np.float64).ravel().copy()
        info = lib().orc_solve_F(self.h, _p(F))
        if info:
            raise RuntimeError(f"oracle solve failed: info={info}")
        return F

    def pivoted(self):
        piv = (ctypes.c_int * 3)()
        lib().orc_pivoted(self.h, piv)
        return tuple(piv)

    def heat_initial_qp(self):
        f = np.zeros(self.nqp)
        lib().orc_heat_initial_qp(self.h, _p(f))
        return f

    def mkbbt_band(self, axis, mix=(1.0, 0.0, 0.0, 0.0)):
        p = self.p[axis]
        n1 = self.ndof[axis]
        AB = np.zeros((n1, 3 * p + 1))  # C view of a Fortran (3p+1, n1) array
        mixa = np.asarray(mix, dtype=np.float64)
        lib().orc_mkbbt_band(self.h, axis, _p(mixa), _p(AB))
        return AB.T.copy()  # (3p+1, n1) LAPACK band layout

    def apply_mass(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64).ravel()
        out = np.zeros(self.N)
        lib().orc_apply_mass(self.h, _p(u), _p(out))
        return out

    def heat_adjoint(self, K, u0, ut, kappa_qp=None, kappa=1.0, dt=1e-5, want_grad=True,
                     want_kappa_grad=False):
        u0 = np.ascontiguousarray(u0, dtype=np.float64).ravel()
        ut = np.ascontiguousarray(ut, dtype=np.float64).ravel()
        kq = None if kappa_qp is None else np.ascontiguousarray(kappa_qp, dtype=np.float64).ravel()
        loss = ctypes.c_double(0.0)
        g = np.zeros(self.N) if want_grad else None
        gk = np.zeros(self.nqp) if want_kappa_grad else None
        info = lib().orc_heat_adjoint(self.h, K, _p(u0), _p(ut), _p(kq), kappa, dt,
                                      ctypes.byref(loss), _p(g), _p(gk))
        if info:
            raise RuntimeError(f"oracle adjoint failed: info={info}")
        return loss.value, g, gk


def reorder(kind, s, F):
    s3 = (ctypes.c_int * 3)(*s)
    F = np.ascontiguousarray(F, dtype=np.float64).ravel()
    out = np.zeros_like(F)
    getattr(lib(), f"orc_reorder_for_{kind}")(s3, _p(F), _p(out))
    return out


def num_threads():
    return lib().orc_num_threads()


def set_num_threads(n):
    lib().orc_set_num_threads(n)
