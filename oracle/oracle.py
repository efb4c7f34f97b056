"""ctypes front-end of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline legs of bench.py.  The product path (ugcore_gb300) never imports
this module.  The C sources cite the ugcore files they restate.
"""
import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

ORC_QUAD, ORC_HEX, ORC_TET, ORC_TRI = 0, 1, 2, 3


class LineSearch(C.Structure):
    """StandardLineSearch parameters (orc_line_search)"""
    _fields_ = [("max_steps", C.c_int), ("lambda_start", C.c_double), ("lambda_reduce", C.c_double),
                ("alpha", C.c_double), ("max_defect", C.c_double), ("accept_best", C.c_int),
                ("check_all", C.c_int)]


class Params(C.Structure):
    _fields_ = [
        ("elem_type", C.c_int), ("mx", C.c_int), ("my", C.c_int), ("mz", C.c_int), ("nref", C.c_int),
        ("seed", C.c_uint64),
        ("coef_kind", C.c_int), ("coef_modes", C.c_int), ("coef_kmax", C.c_double),
        ("vel_kind", C.c_int), ("vel_modes", C.c_int),
        ("vel_kmax", C.c_double), ("diffusion", C.c_double), ("peclet", C.c_double),
        ("solver", C.c_int), ("smoother", C.c_int), ("damp", C.c_double),
        ("nu1", C.c_int), ("nu2", C.c_int), ("cycle", C.c_int), ("base", C.c_int),
        ("maxit", C.c_int), ("rel_red", C.c_double), ("min_defect", C.c_double),
        ("rap", C.c_int), ("bicg_restart", C.c_int), ("bicg_min_ortho", C.c_double),
        ("damp_prol", C.c_double), ("damp_res", C.c_double),
        ("post_smoother", C.c_int), ("post_damp", C.c_double), ("base_steps", C.c_int),
    ]


def build():
    """Compile liboracle.so in place (plain C, seconds); a library left from
    another host architecture is rebuilt."""
    import platform
    stamp = os.path.join(_HERE, ".build_arch")
    arch = platform.machine()
    if not os.path.exists(stamp) or open(stamp).read().strip() != arch:
        subprocess.check_call(["make", "-s", "-C", _HERE, "clean"])
        with open(stamp, "w") as fh:
            fh.write(arch)
    subprocess.check_call(["make", "-s", "-C", _HERE, "liboracle.so"])


def lib():
    global _LIB
    if _LIB is None:
        # UG4GB_ORACLE_LIB: another build of the same sources (the sanitizer
        # build of tests/test_sanitizers.py)
        path = os.environ.get("UG4GB_ORACLE_LIB") or os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        P = C.c_void_p
        dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
        ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
        L.orc_prob_create.restype = P
        L.orc_prob_create.argtypes = [C.POINTER(Params), P, P]
        for name in ("orc_prob_num_levels",):
            getattr(L, name).argtypes = [P]
        L.orc_prob_level_nv.argtypes = [P, C.c_int]
        L.orc_prob_level_ne.argtypes = [P, C.c_int]
        L.orc_prob_level_nnz.argtypes = [P, C.c_int]
        L.orc_prob_level_nnz.restype = C.c_int64
        L.orc_prob_level_matrix.argtypes = [P, C.c_int, ip, ip, dp]
        L.orc_prob_level_coef.argtypes = [P, C.c_int, dp]
        L.orc_prob_level_elems.argtypes = [P, C.c_int, P, P, P]
        L.orc_prob_rhs.argtypes = [P, dp]
        L.orc_prob_source.argtypes = [P, dp]
        L.orc_prob_transfer_nnz.argtypes = [P, C.c_int, C.c_int]
        L.orc_prob_transfer_nnz.restype = C.c_int64
        L.orc_prob_transfer.argtypes = [P, C.c_int, C.c_int, ip, ip, dp]
        L.orc_prob_theta_system.argtypes = [P, C.c_double, C.c_double, dp, ip, ip, dp, dp]
        L.orc_prob_theta_steps.argtypes = [P, C.c_double, C.c_double, C.c_int, dp, ip]
        L.orc_prob_theta_jacobian.argtypes = [P, C.c_int, C.c_double, C.c_double, ip, ip, dp]
        L.orc_prob_create_ext.restype = P
        L.orc_prob_create_ext.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_prob_defect.argtypes = [P, C.c_double, C.c_double, C.c_void_p, dp, dp]
        L.orc_prob_newton.argtypes = [P, C.c_double, C.c_double, C.c_void_p, dp, C.c_int, C.c_double, C.c_double,
                                      ip, ip, dp]
        L.orc_prob_newton_ls.argtypes = [P, C.c_double, C.c_double, C.c_void_p, dp, C.c_int, C.c_double,
                                         C.c_double, C.c_void_p, ip, ip, dp, ip, dp]
        L.orc_prob_gmg_level_nnz.argtypes = [P, C.c_int]
        L.orc_prob_gmg_level_nnz.restype = C.c_int64
        L.orc_prob_gmg_level.argtypes = [P, C.c_int, ip, ip, dp]
        L.orc_prob_apply_gmg.argtypes = [P, dp, dp]
        L.orc_prob_solve.argtypes = [P, dp, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                     C.POINTER(C.c_double), P, C.c_int]
        L.orc_prob_adjoint.argtypes = [P, dp, dp, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                       C.POINTER(C.c_double)]
        L.orc_prob_grad_logk.argtypes = [P, dp, dp, dp]
        L.orc_prob_grad_source.argtypes = [P, dp, dp]
        L.orc_prob_free.argtypes = [P]
        L.orc_transpose_nnz.argtypes = [C.c_int, C.c_int, ip, ip, dp, C.c_int]
        L.orc_transpose_nnz.restype = C.c_int64
        L.orc_geometry.argtypes = [C.c_int, dp, dp, dp, dp, ip, ip, dp]
        _LIB = L
    return _LIB


def make_params(elem_type=ORC_QUAD, mx=2, my=2, mz=2, nref=6, seed=1, coef_kind=0, coef_modes=64,
                coef_kmax=8.0, vel_kind=0, vel_modes=16, vel_kmax=2.0, diffusion=1.0, peclet=10.0,
                solver=0, smoother=0, damp=0.6, nu1=2, nu2=2, cycle=1, base=0, maxit=200,
                rel_red=1e-10, min_defect=1e-300, rap=0, bicg_restart=0, bicg_min_ortho=0.0, damp_prol=1.0,
                damp_res=1.0, post_smoother=-1, post_damp=1.0, base_steps=0):
    return Params(elem_type, mx, my, mz, nref, seed, coef_kind, coef_modes, coef_kmax, vel_kind,
                  vel_modes, vel_kmax, diffusion, peclet, solver, smoother, damp, nu1, nu2, cycle,
                  base, maxit, rel_red, min_defect, rap, bicg_restart, bicg_min_ortho, damp_prol, damp_res,
                  post_smoother, post_damp, base_steps)


class Problem:
    """One assemble-and-solve problem held by the oracle.  levels: optional
    hierarchy [(coords, elems, bnd, npar, par), ...] coarse to fine (an
    unstructured hierarchy exported by the library; npar/par None on level 0)
    instead of the structured one the parameters describe."""

    def __init__(self, params, m_top=None, f_top=None, levels=None):
        L = lib()
        self.params = params
        self._m = None if m_top is None else np.ascontiguousarray(m_top, dtype=np.float64)
        self._f = None if f_top is None else np.ascontiguousarray(f_top, dtype=np.float64)
        if levels is not None:
            self._lv = [tuple(None if a is None else np.ascontiguousarray(a) for a in lev) for lev in levels]
            n = len(levels)
            nv = (C.c_int * n)(*[len(lv[0]) for lv in self._lv])
            ne = (C.c_int * n)(*[len(lv[1]) for lv in self._lv])
            ptrs = []
            for j in range(5):
                arr = (C.c_void_p * n)(*[None if lv[j] is None else lv[j].ctypes.data for lv in self._lv])
                ptrs.append(arr)
            self._ptrs = ptrs
            self.h = L.orc_prob_create_ext(C.byref(params), n, nv, ne, *ptrs,
                                           None if self._m is None else self._m.ctypes.data,
                                           None if self._f is None else self._f.ctypes.data)
        else:
            self.h = L.orc_prob_create(C.byref(params),
                                       None if self._m is None else self._m.ctypes.data,
                                       None if self._f is None else self._f.ctypes.data)
        if not self.h:
            raise RuntimeError("oracle problem setup failed")
        self.nlev = L.orc_prob_num_levels(self.h)
        self.top = self.nlev - 1

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_prob_free(self.h)
            self.h = None

    def nv(self, l=None):
        return lib().orc_prob_level_nv(self.h, self.top if l is None else l)

    def ne(self, l=None):
        return lib().orc_prob_level_ne(self.h, self.top if l is None else l)

    def matrix(self, l=None):
        l = self.top if l is None else l
        L = lib()
        n = self.nv(l)
        nnz = L.orc_prob_level_nnz(self.h, l)
        rp = np.zeros(n + 1, np.int32)
        ci = np.zeros(nnz, np.int32)
        va = np.zeros(nnz, np.float64)
        L.orc_prob_level_matrix(self.h, l, rp, ci, va)
        return rp, ci, va

    def theta_system(self, theta, dt, u_old):
        """top-level (M + theta dt A, rhs) of one theta step from u_old"""
        rp, ci, va = self.matrix()
        va = np.zeros_like(va)
        b = np.zeros(self.nv())
        rc = lib().orc_prob_theta_system(self.h, theta, dt, np.ascontiguousarray(u_old, np.float64), rp, ci, va, b)
        if rc:
            raise RuntimeError("theta assembly failed")
        return (rp, ci, va), b

    def defect(self, u, theta=None, dt=0.0, u_old=None):
        """top-level defect of u: stationary, or of one theta step from u_old"""
        d = np.zeros(self.nv())
        uo = None if u_old is None else np.ascontiguousarray(u_old, np.float64)
        rc = lib().orc_prob_defect(self.h, -1.0 if theta is None else theta, dt,
                                   None if uo is None else uo.ctypes.data_as(C.c_void_p),
                                   np.ascontiguousarray(u, np.float64), d)
        if rc:
            raise RuntimeError("defect failed")
        return d

    def newton(self, u0, maxit=10, min_defect=1e-50, reduction=1e-10, theta=None, dt=0.0, u_old=None,
               line_search=None):
        """NewtonSolver on the stationary operator or one theta step, with
        line_search = dict(max_steps, lambda_start, lambda_reduce, alpha,
        max_defect, accept_best, check_all) or None; returns (u, rc, steps,
        linear steps per step, defects), plus (tries, lambdas) per step with a
        line search"""
        u = np.array(u0, dtype=np.float64, copy=True)
        steps = np.zeros(1, np.int32)
        ls = np.zeros(maxit + 1, np.int32)
        defs = np.zeros(maxit + 1)
        tries = np.zeros(maxit + 1, np.int32)
        lams = np.zeros(maxit + 1)
        uo = None if u_old is None else np.ascontiguousarray(u_old, np.float64)
        ptr = None
        if line_search is not None:
            p = dict(max_steps=10, lambda_start=1.0, lambda_reduce=0.5, alpha=0.25, max_defect=1e10,
                     accept_best=0, check_all=0)
            p.update(line_search)
            lsp = LineSearch(int(p["max_steps"]), p["lambda_start"], p["lambda_reduce"], p["alpha"],
                             p["max_defect"], int(p["accept_best"]), int(p["check_all"]))
            ptr = C.cast(C.pointer(lsp), C.c_void_p)
        rc = lib().orc_prob_newton_ls(self.h, -1.0 if theta is None else theta, dt,
                                      None if uo is None else uo.ctypes.data_as(C.c_void_p), u, maxit, min_defect,
                                      reduction, ptr, steps, ls, defs, tries, lams)
        if rc < 0:
            raise RuntimeError("Newton set-up failed %d" % rc)
        n = int(steps[0])
        if line_search is None:
            return u, rc, n, ls[:n], defs[:n + 1]
        nt = n + (1 if rc == 3 else 0)
        return u, rc, n, ls[:n], defs[:n + 1], (tries[:nt].tolist(), lams[:nt].tolist())

    def theta_jacobian(self, l, theta, dt):
        """level l's M + theta dt A (CRS pattern = the level's)"""
        rp, ci, va = self.matrix(l)
        va = np.zeros_like(va)
        if lib().orc_prob_theta_jacobian(self.h, l, theta, dt, rp, ci, va):
            raise RuntimeError("theta jacobian failed")
        return rp, ci, va

    def theta_steps(self, theta, dt, nsteps, u0):
        """nsteps theta steps from u0; (u, iterations per step)"""
        u = np.array(u0, dtype=np.float64, copy=True)
        steps = np.zeros(nsteps, np.int32)
        rc = lib().orc_prob_theta_steps(self.h, theta, dt, nsteps, u, steps)
        if rc:
            raise RuntimeError("theta steps failed %d" % rc)
        return u, steps

    def gmg_level_matrix(self, l):
        """the multigrid's operator of level l (R A P of the level above with rap)"""
        L = lib()
        n = self.nv(l)
        nnz = L.orc_prob_gmg_level_nnz(self.h, l)
        if nnz < 0:
            raise RuntimeError("gmg init failed")
        rp = np.zeros(n + 1, np.int32)
        ci = np.zeros(nnz, np.int32)
        va = np.zeros(nnz, np.float64)
        L.orc_prob_gmg_level(self.h, l, rp, ci, va)
        return rp, ci, va

    def transfer(self, l, which):
        """which = 0: P (fine l x coarse l-1), 1: R."""
        L = lib()
        nnz = L.orc_prob_transfer_nnz(self.h, l, which)
        nrow = self.nv(l) if which == 0 else self.nv(l - 1)
        rp = np.zeros(nrow + 1, np.int32)
        ci = np.zeros(nnz, np.int32)
        va = np.zeros(nnz, np.float64)
        L.orc_prob_transfer(self.h, l, which, rp, ci, va)
        return rp, ci, va

    def level_geometry(self, l=None):
        """(coords nv x dim, elems ne x k, Dirichlet flags nv) of level l"""
        l = self.top if l is None else l
        L = lib()
        n, ne = self.nv(l), self.ne(l)
        dim = 2 if self.params.elem_type in (ORC_QUAD, ORC_TRI) else 3
        k = 8 if self.params.elem_type == ORC_HEX else (3 if self.params.elem_type == ORC_TRI else 4)
        coords = np.zeros(n * dim)
        elems = np.zeros(ne * k, np.int32)
        bnd = np.zeros(n, np.uint8)
        L.orc_prob_level_elems(self.h, l, elems.ctypes.data, coords.ctypes.data, bnd.ctypes.data)
        return coords.reshape(n, dim), elems.reshape(ne, k), bnd

    def coef(self, l=None):
        l = self.top if l is None else l
        K = np.zeros(self.ne(l))
        lib().orc_prob_level_coef(self.h, l, K)
        return K

    def rhs(self):
        b = np.zeros(self.nv())
        lib().orc_prob_rhs(self.h, b)
        return b

    def source(self):
        f = np.zeros(self.nv())
        lib().orc_prob_source(self.h, f)
        return f

    def apply_gmg(self, d):
        c = np.zeros(self.nv())
        rc = lib().orc_prob_apply_gmg(self.h, c, np.ascontiguousarray(d, np.float64))
        if rc:
            raise RuntimeError("gmg init failed %d" % rc)
        return c

    def solve(self, hist_cap=0):
        x = np.zeros(self.nv())
        steps = C.c_int()
        d0, d1 = C.c_double(), C.c_double()
        hist = np.zeros(max(hist_cap, 1))
        rc = lib().orc_prob_solve(self.h, x, C.byref(steps), C.byref(d0), C.byref(d1),
                                  hist.ctypes.data if hist_cap else None, hist_cap)
        return dict(x=x, steps=steps.value, d0=d0.value, d1=d1.value, converged=(rc == 0),
                    history=hist[:min(steps.value + 1, hist_cap)] if hist_cap else None)

    def adjoint(self, g):
        lam = np.zeros(self.nv())
        steps = C.c_int()
        d0, d1 = C.c_double(), C.c_double()
        rc = lib().orc_prob_adjoint(self.h, np.ascontiguousarray(g, np.float64), lam, C.byref(steps),
                                    C.byref(d0), C.byref(d1))
        return dict(lam=lam, steps=steps.value, d0=d0.value, d1=d1.value, converged=(rc == 0))

    def grad_logk(self, u, lam):
        g = np.zeros(self.ne())
        lib().orc_prob_grad_logk(self.h, np.ascontiguousarray(u, np.float64),
                                 np.ascontiguousarray(lam, np.float64), g)
        return g

    def grad_source(self, lam):
        g = np.zeros(self.nv())
        lib().orc_prob_grad_source(self.h, np.ascontiguousarray(lam, np.float64), g)
        return g


def transpose_nnz(rowptr, col, val, n_cols, keep_zeros):
    rowptr = np.ascontiguousarray(rowptr, np.int32)
    return lib().orc_transpose_nnz(len(rowptr) - 1, n_cols, rowptr, np.ascontiguousarray(col, np.int32),
                                   np.ascontiguousarray(val, np.float64), int(keep_zeros))


def geometry(elem_type, corners):
    """FV1 geometry of one element: SCVF area normals, integration points,
    shape gradients at them, from/to corners, and the SCV volumes"""
    dim = 2 if elem_type in (ORC_QUAD, ORC_TRI) else 3
    k = {ORC_QUAD: 4, ORC_HEX: 8, ORC_TET: 4, ORC_TRI: 3}[elem_type]
    nf = {ORC_QUAD: 4, ORC_HEX: 12, ORC_TET: 6, ORC_TRI: 3}[elem_type]
    corners = np.ascontiguousarray(corners, np.float64).reshape(-1)
    normals = np.zeros(nf * dim)
    ips = np.zeros(nf * dim)
    vols = np.zeros(k)
    grads = np.zeros(nf * k * dim)
    fr = np.zeros(nf, np.int32)
    to = np.zeros(nf, np.int32)
    lib().orc_geometry(elem_type, corners, normals, vols, grads, fr, to, ips)
    return dict(normals=normals.reshape(nf, dim), vols=vols, grads=grads.reshape(nf, k, dim),
                frm=fr, to=to, ips=ips.reshape(nf, dim))
