"""TEST INFRASTRUCTURE: ctypes front end of the CPU oracle (oracle/ikarus_oracle.cpp).

The oracle restates the reference's FP64 CPU algorithm for the Newton-Raphson / LoadControl
hot path.  Only tests/, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use it,
and only as the checker or the reported CPU baseline; the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_UNFUSED_PATH = os.path.join(_HERE, "_build", "liboracle_unfused.so")
_lib = None
_lib_unfused = None

EAS_NONE, EAS_GL, EAS_H, EAS_HT = 0, 1, 2, 3
DBC_RAW, DBC_REDUCED, DBC_FULL = 0, 1, 2
SOLVER_BANDED_LDLT, SOLVER_CG_JACOBI = 0, 1
MATERIAL_NEOHOOKE, MATERIAL_SVK, MATERIAL_BLATZKO, MATERIAL_HYPERELASTIC = 0, 1, 2, 3
DEV_NONE, DEV_BLATZKO, DEV_OGDEN_TOTAL, DEV_OGDEN_DEVIATORIC, DEV_INVARIANT_BASED, DEV_ARRUDA_BOYCE, DEV_GENT = range(7)
HYPER_MAX_TERMS = 4
PF_ARC_LENGTH, PF_LOAD_CONTROL, PF_DISPLACEMENT_CONTROL = 0, 1, 2
ERRORS = {-1: "ARG", -2: "NOT_IMPLEMENTED", -3: "NONPOSITIVE_DETC", -4: "SINGULAR", -5: "NOT_CONVERGED"}


class OracleError(RuntimeError):
    def __init__(self, code, what=""):
        super().__init__(f"oracle {what} failed: {ERRORS.get(code, code)}")
        self.code = code


def build():
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib(unfused=False):
    """The oracle library; unfused=True: the same restatement compiled without contracting multiply-adds to fused
    multiply-adds (a second valid FP64 evaluation, for FP64 floors of ill-conditioned quantities)."""
    global _lib, _lib_unfused
    if unfused:
        if _lib_unfused is None:
            if not os.path.exists(_UNFUSED_PATH):
                build()
            _lib_unfused = _declare(C.CDLL(_UNFUSED_PATH))
        return _lib_unfused
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        _lib = _declare(C.CDLL(_LIB_PATH))
    return _lib


def _declare(L):
    dp, ip, up, lp = (C.POINTER(C.c_double), C.POINTER(C.c_int32), C.POINTER(C.c_uint8), C.POINTER(C.c_int64))
    vp = C.c_void_p
    L.orc_problem_create.restype = vp
    L.orc_problem_create.argtypes = [C.c_int, dp, C.c_int, ip, C.c_double, C.c_double, C.c_int, C.c_int]
    L.orc_problem_destroy.argtypes = [vp]
    L.orc_set_dirichlet.argtypes = [vp, up]
    L.orc_add_neumann.argtypes = [vp, C.c_int, ip, ip, dp]
    L.orc_add_point_loads.argtypes = [vp, C.c_int, ip, dp]
    L.orc_set_faithful_moduli.argtypes = [vp, C.c_int]
    L.orc_get_alpha.argtypes = [vp, dp]
    L.orc_set_alpha.argtypes = [vp, dp]
    L.orc_element_vector.argtypes = [vp, C.c_int, dp, C.c_double, dp]
    L.orc_element_matrix.argtypes = [vp, C.c_int, dp, C.c_double, dp]
    L.orc_element_energy.argtypes = [vp, C.c_int, dp, C.c_double, dp]
    L.orc_update_state.argtypes = [vp, dp, C.c_double, dp]
    L.orc_assemble_vector.argtypes = [vp, dp, C.c_double, C.c_int, dp]
    L.orc_pattern_nnz.restype = C.c_int64
    L.orc_pattern_nnz.argtypes = [vp, C.c_int]
    L.orc_reduced_size.argtypes = [vp]
    L.orc_assemble_matrix_csc.argtypes = [vp, dp, C.c_double, C.c_int, lp, ip, dp]
    L.orc_set_dirichlet_values.argtypes = [vp, dp]
    L.orc_set_material.argtypes = [vp, C.c_int]
    L.orc_set_hyperelastic.argtypes = [vp, C.POINTER(OrcHyper)]
    L.orc_hyper_deviatoric.argtypes = [C.POINTER(OrcHyper), dp, dp]
    L.orc_hyper_volumetric.argtypes = [C.c_int, C.c_double, C.c_double, dp]
    L.orc_material_point.argtypes = [C.c_int, C.c_double, C.c_double, C.POINTER(OrcHyper), dp, dp]
    L.orc_calculate_at.argtypes = [vp, C.c_int, dp, C.c_int, dp, dp]
    L.orc_cg_jacobi_csc.argtypes = [C.c_int, lp, ip, dp, dp, dp, C.c_double, C.c_int, C.POINTER(C.c_int)]
    L.orc_load_control.argtypes = [vp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, C.c_int,
                                   C.c_double, dp, dp, ip, dp, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.orc_path_following.argtypes = [vp, C.c_int, C.c_int, C.c_double, C.c_int, ip, C.c_int, C.c_double, C.c_int,
                                     C.c_int, C.c_double, dp, dp, ip, dp, dp, dp, C.POINTER(C.c_int),
                                     C.POINTER(C.c_int)]
    L.orc_set_threads.argtypes = [C.c_int]
    L.orc_add_volume_load.argtypes = [vp, _ORC_POINT_FN, vp]
    L.orc_set_dirichlet_function.argtypes = [vp, _ORC_POINT_FN, _ORC_POINT_FN, vp]
    L.orc_add_neumann_function.argtypes = [vp, C.c_int, ip, ip, _ORC_POINT_FN, vp]
    L.orc_constraints_below.argtypes = [vp, ip]
    L.orc_load_step.argtypes = [vp, C.c_double, C.c_double, C.c_int, C.c_int, C.c_int, C.c_double, dp, dp, dp]
    L.orc_path_following_toy.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_double, C.c_int, dp,
                                         dp, ip, dp, dp, C.POINTER(C.c_int)]
    return L


class OrcHyper(C.Structure):
    """orc_hyper: Hyperelastic<Deviatoric<DF>, Volumetric<VF>> (materials/hyperelastic/interface.hh)."""
    _fields_ = [("deviatoric", C.c_int32), ("n_terms", C.c_int32), ("mu", C.c_double * HYPER_MAX_TERMS),
                ("alpha", C.c_double * HYPER_MAX_TERMS), ("p", C.c_int32 * HYPER_MAX_TERMS),
                ("q", C.c_int32 * HYPER_MAX_TERMS), ("param", C.c_double), ("volumetric", C.c_int32),
                ("reserved", C.c_int32), ("K", C.c_double), ("beta", C.c_double)]


def hyper(deviatoric, mu=(), alpha=(), p=(), q=(), param=0.0, volumetric=0, K=0.0, beta=0.0):
    """An orc_hyper from plain values (mu: the deviatoric function's moduli or coefficients)."""
    h = OrcHyper()
    h.deviatoric, h.n_terms = int(deviatoric), len(mu)
    for i, v in enumerate(mu):
        h.mu[i] = v
    for i, v in enumerate(alpha):
        h.alpha[i] = v
    for i, v in enumerate(p):
        h.p[i] = v
    for i, v in enumerate(q):
        h.q[i] = v
    h.param, h.volumetric, h.K, h.beta = float(param), int(volumetric), float(K), float(beta)
    return h


def _as_hyper(h):
    return h if isinstance(h, OrcHyper) else hyper(**h)


def hyper_deviatoric(h, stretches):
    """(W, dW/dlambda (3), secondDerivative (3x3)) of the deviatoric function at the principal stretches."""
    hh = _as_hyper(h)
    lam = np.ascontiguousarray(stretches, dtype=np.float64)
    out = np.zeros(13)
    _check(lib().orc_hyper_deviatoric(C.byref(hh), _p(lam, C.c_double), _p(out, C.c_double)), "hyper_deviatoric")
    return out[0], out[1:4].copy(), out[4:].reshape(3, 3).copy()


def hyper_volumetric(vf, J, beta=0.0):
    """(U, U', U'') of volumetric function VF<vf> at J."""
    out = np.zeros(3)
    _check(lib().orc_hyper_volumetric(int(vf), float(beta), float(J), _p(out, C.c_double)), "hyper_volumetric")
    return tuple(out)


def material_point(material, Cmat, lam=0.0, mu=0.0, h=None, unfused=False):
    """(psi, S Voigt (6), moduli Voigt (6x6)) of a material law at the right Cauchy-Green tensor C (3x3)."""
    hh = _as_hyper(h) if h is not None else OrcHyper()
    c = np.ascontiguousarray(Cmat, dtype=np.float64).reshape(9)
    out = np.zeros(43)
    _check(lib(unfused).orc_material_point(int(material), float(lam), float(mu), C.byref(hh), _p(c, C.c_double),
                                           _p(out, C.c_double)), "material_point")
    return out[0], out[1:7].copy(), out[7:].reshape(6, 6).copy()


_ORC_POINT_FN = C.CFUNCTYPE(None, C.c_int32, C.POINTER(C.c_double), C.c_double, C.POINTER(C.c_double), C.c_void_p)


def _point_fn(fn):
    def tramp(n, X, lam, out, _user):
        x = np.ctypeslib.as_array(X, shape=(n, 3))
        np.ctypeslib.as_array(out, shape=(n, 3))[:] = np.asarray(fn(x, lam), dtype=np.float64).reshape(n, 3)
    return _ORC_POINT_FN(tramp)


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t)) if a is not None else None


def _check(code, what):
    if code != 0:
        raise OracleError(code, what)


def set_threads(n):
    """Threads of the oracle's CG (assembly stays serial); results depend only on the count."""
    _check(lib().orc_set_threads(int(n)), "set_threads")


def cg_jacobi(col_ptr, row_idx, values, b, rtol, max_iter):
    """The oracle's Jacobi-preconditioned CG on a CSC matrix: (x, iterations, converged)."""
    n = len(col_ptr) - 1
    cp = np.ascontiguousarray(col_ptr, dtype=np.int64)
    ri = np.ascontiguousarray(row_idx, dtype=np.int32)
    v = np.ascontiguousarray(values, dtype=np.float64)
    bb = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros(n)
    its = C.c_int(0)
    code = lib().orc_cg_jacobi_csc(n, _p(cp, C.c_int64), _p(ri, C.c_int32), _p(v, C.c_double), _p(bb, C.c_double),
                                   _p(x, C.c_double), rtol, max_iter, C.byref(its))
    if code not in (0, -5):
        raise OracleError(code, "cg_jacobi")
    return x, its.value, code == 0


def path_following_toy(kind=PF_ARC_LENGTH, idbc=False, steps=5, step_size=0.1, target_iterations=0, tol=1e-8,
                       max_iter=20):
    """The oracle's path-following routine on the reference's two-dof test operator
    (tests/src/testpathfollowing.cpp:26-40), starting from D = 0, lambda = 0."""
    d = np.zeros(2)
    lam = np.zeros(1)
    its = np.zeros(steps + 1, dtype=np.int32)
    lams = np.zeros(steps + 1)
    ds = np.zeros((steps + 1, 2))
    ns = C.c_int(0)
    code = lib().orc_path_following_toy(kind, int(idbc), steps, step_size, target_iterations, tol, max_iter,
                                        _p(d, C.c_double), _p(lam, C.c_double), _p(its, C.c_int32),
                                        _p(lams, C.c_double), _p(ds, C.c_double), C.byref(ns))
    _check(code, "path_following_toy")
    return dict(d=d, lam=float(lam[0]), iterations=its[: ns.value].tolist(), lambdas=lams[: ns.value],
                d_steps=ds[: ns.value])


def from_problem(p, faithful=False, unfused=False):
    """Oracle twin of an ``ikarus_gb300.problems.Problem`` definition (plain data, no GPU objects); unfused: evaluated
    by the build of the oracle without fused multiply-adds."""
    o = OracleProblem(p.mesh.coords, p.mesh.conn, p.lam, p.mu, p.eas if p.n_eas else EAS_NONE, p.n_eas,
                      unfused=unfused)
    o.set_dirichlet(p.fixed)
    if getattr(p, "hyper", None) is not None:  # a description with oracle_terms(), or the terms themselves
        o.set_hyperelastic(p.hyper.oracle_terms() if hasattr(p.hyper, "oracle_terms") else p.hyper)
    elif getattr(p, "material", 0):
        o.set_material(p.material)
    if p.face_elem is not None and len(p.face_elem):
        o.add_neumann(p.face_elem, p.face_local, p.face_traction)
    if p.pl_dofs is not None:
        o.add_point_loads(p.pl_dofs, p.pl_values)
    if faithful:
        o.set_faithful_moduli(True)
    return o


class OracleProblem:
    """One mesh + NeoHooke material + EAS choice, with Dirichlet flags and dead loads."""

    def __init__(self, coords, conn, lam, mu, eas_kind=EAS_NONE, n_alpha=0, unfused=False):
        self.coords = np.ascontiguousarray(coords, dtype=np.float64)
        self.conn = np.ascontiguousarray(conn, dtype=np.int32)
        self.n_nodes, self.n_elems = self.coords.shape[0], self.conn.shape[0]
        self.n_dofs = 3 * self.n_nodes
        self.n_alpha = n_alpha
        self._L = L = lib(unfused)
        self.h = L.orc_problem_create(self.n_nodes, _p(self.coords, C.c_double), self.n_elems,
                                      _p(self.conn, C.c_int32), lam, mu, eas_kind, n_alpha)
        if not self.h:
            raise OracleError(-1, "create")

    def __del__(self):
        if getattr(self, "h", None) and getattr(self, "_L", None) is not None:
            self._L.orc_problem_destroy(self.h)
            self.h = None

    def set_dirichlet(self, fixed):
        f = np.ascontiguousarray(fixed, dtype=np.uint8)
        _check(self._L.orc_set_dirichlet(self.h, _p(f, C.c_uint8)), "set_dirichlet")

    def calculate_at(self, e, u, result_type, xi=(0.5, 0.5, 0.5)):
        """Stress of element e at local xi: result_type 0 PK2, 1 Kirchhoff, 2 Cauchy (Voigt, 6 values)."""
        uu = self._u(u)
        x = np.ascontiguousarray(xi, dtype=np.float64)
        out = np.zeros(6)
        _check(self._L.orc_calculate_at(self.h, e, _p(uu, C.c_double), result_type, _p(x, C.c_double),
                                      _p(out, C.c_double)), "calculate_at")
        return out

    def set_material(self, material):
        """MATERIAL_NEOHOOKE (default) or MATERIAL_SVK for all elements."""
        _check(self._L.orc_set_material(self.h, int(material)), "set_material")

    def set_hyperelastic(self, h):
        """MATERIAL_HYPERELASTIC with the functions of h (an OrcHyper or the keyword arguments of ``hyper``)."""
        self._hyper = _as_hyper(h)
        _check(self._L.orc_set_hyperelastic(self.h, C.byref(self._hyper)), "set_hyperelastic")

    def set_dirichlet_values(self, rate):
        """Inhomogeneous Dirichlet values lambda * rate on constrained dofs (None removes them)."""
        if rate is None:
            _check(self._L.orc_set_dirichlet_values(self.h, None), "set_dirichlet_values")
            return
        r = np.ascontiguousarray(rate, dtype=np.float64)
        _check(self._L.orc_set_dirichlet_values(self.h, _p(r, C.c_double)), "set_dirichlet_values")

    def add_neumann(self, face_elem, face_local, traction):
        fe = np.ascontiguousarray(face_elem, dtype=np.int32)
        fl = np.ascontiguousarray(face_local, dtype=np.int32)
        t = np.ascontiguousarray(np.broadcast_to(np.asarray(traction, dtype=np.float64), (len(fe), 3)))
        _check(self._L.orc_add_neumann(self.h, len(fe), _p(fe, C.c_int32), _p(fl, C.c_int32), _p(t, C.c_double)),
               "add_neumann")

    def set_dirichlet_function(self, value, derivative):
        """Inhomogeneous Dirichlet values value(X (n, 3), lambda) at every node, lambda-derivative derivative(X,
        lambda) (used at lambda = 1 for the IDBC forces)."""
        cv, cd = _point_fn(value), _point_fn(derivative)
        self._cbs = getattr(self, "_cbs", []) + [cv, cd]
        _check(self._L.orc_set_dirichlet_function(self.h, cv, cd, None), "set_dirichlet_function")

    def add_volume_load(self, fn):
        """VolumeLoad with fn(X (n, 3), lambda) -> body forces (n, 3)."""
        cb = _point_fn(fn)
        self._cbs = getattr(self, "_cbs", []) + [cb]
        _check(self._L.orc_add_volume_load(self.h, cb, None), "add_volume_load")

    def add_neumann_function(self, face_elem, face_local, fn):
        """Neumann faces with a traction function fn(X (n, 3), lambda) -> (n, 3)."""
        fe = np.ascontiguousarray(face_elem, dtype=np.int32)
        fl = np.ascontiguousarray(face_local, dtype=np.int32)
        cb = _point_fn(fn)
        self._cbs = getattr(self, "_cbs", []) + [cb]
        _check(self._L.orc_add_neumann_function(self.h, len(fe), _p(fe, C.c_int32), _p(fl, C.c_int32), cb, None),
               "add_neumann_function")

    def add_point_loads(self, dofs, values):
        d = np.ascontiguousarray(dofs, dtype=np.int32)
        v = np.ascontiguousarray(values, dtype=np.float64)
        _check(self._L.orc_add_point_loads(self.h, len(d), _p(d, C.c_int32), _p(v, C.c_double)), "add_point_loads")

    def set_faithful_moduli(self, on=True):
        _check(self._L.orc_set_faithful_moduli(self.h, int(on)), "faithful")

    @property
    def alpha(self):
        a = np.zeros(self.n_elems * self.n_alpha)
        if a.size:
            _check(self._L.orc_get_alpha(self.h, _p(a, C.c_double)), "get_alpha")
        return a.reshape(self.n_elems, self.n_alpha)

    @alpha.setter
    def alpha(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64).ravel()
        _check(self._L.orc_set_alpha(self.h, _p(a, C.c_double)), "set_alpha")

    def _u(self, u):
        return np.ascontiguousarray(u if u is not None else np.zeros(self.n_dofs), dtype=np.float64)

    def element_vector(self, e, u=None, lam=0.0):
        u = self._u(u)
        out = np.zeros(24)
        _check(self._L.orc_element_vector(self.h, e, _p(u, C.c_double), lam, _p(out, C.c_double)), "element_vector")
        return out

    def element_matrix(self, e, u=None, lam=0.0):
        u = self._u(u)
        out = np.zeros(576)
        _check(self._L.orc_element_matrix(self.h, e, _p(u, C.c_double), lam, _p(out, C.c_double)), "element_matrix")
        return out.reshape(24, 24).T.copy()  # stored column-major

    def element_energy(self, e, u=None, lam=0.0):
        u = self._u(u)
        out = np.zeros(1)
        _check(self._L.orc_element_energy(self.h, e, _p(u, C.c_double), lam, _p(out, C.c_double)), "element_energy")
        return float(out[0])

    def update_state(self, u, correction, lam=0.0):
        u = self._u(u)
        c = np.ascontiguousarray(correction, dtype=np.float64)
        _check(self._L.orc_update_state(self.h, _p(u, C.c_double), lam, _p(c, C.c_double)), "update_state")

    def constraints_below(self):
        out = np.zeros(self.n_dofs, dtype=np.int32)
        _check(self._L.orc_constraints_below(self.h, _p(out, C.c_int32)), "constraints_below")
        return out

    def reduced_size(self):
        return self._L.orc_reduced_size(self.h)

    def assemble_vector(self, u=None, lam=0.0, dbc=DBC_FULL):
        u = self._u(u)
        n = self.reduced_size() if dbc == DBC_REDUCED else self.n_dofs
        out = np.zeros(n)
        _check(self._L.orc_assemble_vector(self.h, _p(u, C.c_double), lam, dbc, _p(out, C.c_double)), "assemble_vector")
        return out

    def assemble_matrix_csc(self, u=None, lam=0.0, dbc=DBC_FULL):
        """Returns (col_ptr int64, row_idx int32, values float64, n)."""
        u = self._u(u)
        n = self.reduced_size() if dbc == DBC_REDUCED else self.n_dofs
        nnz = self._L.orc_pattern_nnz(self.h, dbc)
        cp = np.zeros(n + 1, dtype=np.int64)
        ri = np.zeros(nnz, dtype=np.int32)
        v = np.zeros(nnz)
        _check(self._L.orc_assemble_matrix_csc(self.h, _p(u, C.c_double), lam, dbc, _p(cp, C.c_int64),
                                             _p(ri, C.c_int32), _p(v, C.c_double)), "assemble_matrix")
        return cp, ri, v, n

    def assemble_matrix_dense(self, u=None, lam=0.0, dbc=DBC_FULL):
        cp, ri, v, n = self.assemble_matrix_csc(u, lam, dbc)
        A = np.zeros((n, n))
        for c in range(n):
            A[ri[cp[c]:cp[c + 1]], c] = v[cp[c]:cp[c + 1]]
        return A

    def load_control(self, steps, t_begin=0.0, t_end=1.0, tol=1e-10, tol_mode=0, max_iter=20,
                     solver=SOLVER_BANDED_LDLT, cg_rtol=1e-12, u0=None, lam0=0.0, allow_failure=False):
        u = self._u(u0).copy()
        lam = np.array([lam0])
        its = np.zeros(steps + 1, dtype=np.int32)
        rn = np.zeros(steps + 1)
        ns, tot = C.c_int(0), C.c_int(0)
        code = self._L.orc_load_control(self.h, steps, t_begin, t_end, tol, tol_mode, max_iter, solver, cg_rtol,
                                      _p(u, C.c_double), _p(lam, C.c_double), _p(its, C.c_int32), _p(rn, C.c_double),
                                      C.byref(ns), C.byref(tot))
        if code != 0 and not (allow_failure and code == -5):
            raise OracleError(code, "load_control")
        return dict(u=u, lam=float(lam[0]), iterations=its[: ns.value], res_norms=rn[: ns.value],
                    total_iterations=tot.value, success=(code == 0))

    def load_step(self, u, lam, dlambda, tol=1e-8, tol_mode=1, max_iter=30, solver=SOLVER_CG_JACOBI, cg_rtol=1e-10):
        """One LoadControl step from (u, lam): lambda += dlambda and Newton to the tolerance.  Returns (u, lambda,
        stats) with stats = dict(newton, cg, t_residual, t_tangent, t_solve, residual_norm)."""
        uu = self._u(u).copy()
        lm = np.array([lam], dtype=np.float64)
        st = np.zeros(6)
        code = self._L.orc_load_step(self.h, dlambda, tol, tol_mode, max_iter, solver, cg_rtol, _p(uu, C.c_double),
                                   _p(lm, C.c_double), _p(st, C.c_double))
        _check(code, "load_step")
        return uu, float(lm[0]), dict(zip(("newton", "cg", "t_residual", "t_tangent", "t_solve", "residual_norm"),
                                          st.tolist()))

    def path_following(self, steps, step_size, kind=PF_ARC_LENGTH, controlled=None, target_iterations=0, tol=1e-8,
                       max_iter=20, solver=SOLVER_BANDED_LDLT, cg_rtol=1e-12, u0=None, lam0=0.0,
                       allow_failure=False):
        """PathFollowing::run with NewtonRaphsonWithSubsidiaryFunction (pathfollowing.inl:25-73); entry k of the
        per-solve arrays belongs to load step k - 1."""
        u = self._u(u0).copy()
        lam = np.array([lam0])
        its = np.zeros(steps + 1, dtype=np.int32)
        rn = np.zeros(steps + 1)
        lams = np.zeros(steps + 1)
        psi = np.zeros(1)
        ci = np.ascontiguousarray(controlled if controlled is not None else [], dtype=np.int32)
        ns, tot = C.c_int(0), C.c_int(0)
        code = self._L.orc_path_following(self.h, kind, steps, step_size, len(ci), _p(ci, C.c_int32) if len(ci) else None,
                                        target_iterations, tol, max_iter, solver, cg_rtol, _p(u, C.c_double),
                                        _p(lam, C.c_double), _p(its, C.c_int32), _p(rn, C.c_double),
                                        _p(lams, C.c_double), _p(psi, C.c_double), C.byref(ns), C.byref(tot))
        if code != 0 and not (allow_failure and code == -5):
            raise OracleError(code, "path_following")
        return dict(u=u, lam=float(lam[0]), iterations=its[: ns.value], res_norms=rn[: ns.value],
                    lambdas=lams[: ns.value], psi=float(psi[0]), total_iterations=tot.value, success=(code == 0))
