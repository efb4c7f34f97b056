"""Python mirror of ugcore's assemble-and-solve interface over libug4gb.

Class and method names follow the ugcore objects a Lua script drives through
the registry (bridge/algebra_bridges/solver_bridge.cpp, preconditioner_bridge.cpp,
disc_bridges/multigrid_bridge.cpp, domain_disc_bridge.cpp):

    ugcore (Lua)                          here
    ------------------------------------  -------------------------------------
    InitUG(dim, AlgebraType("GPU", 1))    Context(device)
    util.CreateDomain + refinement        StructuredHierarchy(ctx, "hex", 2, 2, 2, 6)
    DomainDiscretization + FV1 ConvDiff   DomainDiscretization(hier) .set_* ...
    + DirichletBoundary (0 on boundary)
    GridFunction / Vector                 GPUVector
    AssembledLinearOperator / matrix      GPUSparseMatrix
    GeometricMultiGrid(approxSpace)       GeometricMultiGrid(disc)
    Jacobi(0.6) / GaussSeidel()           Jacobi(0.6) / GaussSeidel() (multicolour)
    BackwardGaussSeidel / SGS / ILU       BackwardGaussSeidel() / SymmetricGaussSeidel() / ILU()
    gmg:set_presmoother / postsmoother    GeometricMultiGrid.set_presmoother / set_postsmoother
    StdTransfer                           StdTransfer (P1 prolongation, R = P^T, dampings)
    LU (base solver)                      LU() (dense, the default)
    LinearSolver + ConvCheck(k, 0, 0)     BaseSmoothing(k) (k pre-smoother steps)
    CG() / BiCGStab()                     CG() / BiCGStab()
    ConvCheck(maxit, minDef, red)         StdConvCheck(maxit, minDef, red)

All work happens on the GPU; errors raised by the C ABI become UG4GBError.
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import check, lib

_ELEM = {"quad": _lib.QUAD, "quadrilateral": _lib.QUAD, "hex": _lib.HEX, "hexahedron": _lib.HEX,
         "tet": _lib.TET, "tetrahedron": _lib.TET, "tri": _lib.TRI, "triangle": _lib.TRI}


def _ptr(a):
    """data pointer of a numpy array or a torch tensor (host or device)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    return C.c_void_p(a.ctypes.data)


def _f64(a):
    if hasattr(a, "data_ptr"):
        return a
    return np.ascontiguousarray(a, dtype=np.float64)


class Context:
    """One GPU, one stream (InitUG with the GPU algebra)."""

    def __init__(self, device=0):
        h = C.c_void_p()
        rc = lib().ug4gb_create(device, C.byref(h))
        if rc != 0:
            raise _lib.UG4GBError(rc, "cannot create context on device %d" % device)
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().ug4gb_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def synchronize(self):
        check(lib().ug4gb_synchronize(self.h), self.h)

    def kernel_launches(self):
        return lib().ug4gb_kernel_launches(self.h)

    def set_operator_format(self, fmt):
        """'auto' (diagonal layout for structured operators) or 'sell'."""
        check(lib().ug4gb_set_operator_format(self.h, {"auto": 0, "sell": 1}[fmt]), self.h)

    def set_tuning(self, pdl=None, sweep_fusion=None, sweep_planes=None, row_assembly=None, sweep_wait_test=None,
                   coarse_levels=None):
        """performance switches:
        pdl: programmatic dependent launch of the solve kernels;
        sweep_fusion: bit mask (1 on, 2 every level size) of the
        two-Jacobi-steps-per-pass smoother of structured 3D FP32 levels;
        sweep_planes: z planes per block of that smoother (these three leave
        results bit-identical);
        row_assembly: stationary assembly of structured levels row by row
        from the per-class element geometry (True or 1), in addition from
        the one interior stencil when the coefficient is constant and there
        is no convection (2, the default), or element by element (False or
        0); the same values to rounding;
        coarse_levels: levels above the base that one launch cycles at the
        coarse end of a V-cycle (-1 as many as pay, the default; 0 none;
        bit-identical corrections; multigrids set up afterwards)."""
        if sweep_wait_test is not None:
            # failure test of the fused sweeps' bounded waits only
            check(lib().ug4gb_set_tuning(self.h, _lib.TUNE_SWEEP_WAIT_TEST, int(sweep_wait_test)), self.h)
        if row_assembly is not None:
            check(lib().ug4gb_set_tuning(self.h, _lib.TUNE_ROW_ASSEMBLY, int(row_assembly)), self.h)
        if pdl is not None:
            check(lib().ug4gb_set_tuning(self.h, _lib.TUNE_PDL, int(bool(pdl))), self.h)
        if sweep_fusion is not None:
            check(lib().ug4gb_set_tuning(self.h, _lib.TUNE_SWEEP_FUSION, int(sweep_fusion)), self.h)
        if sweep_planes is not None:
            check(lib().ug4gb_set_tuning(self.h, _lib.TUNE_SWEEP_PLANES, int(sweep_planes)), self.h)
        if coarse_levels is not None:
            check(lib().ug4gb_set_tuning(self.h, _lib.TUNE_COARSE_LEVELS, int(coarse_levels)), self.h)

    def profile_begin(self):
        check(lib().ug4gb_profile_begin(self.h), self.h)

    def profile_end(self):
        """{ 'tag|kernel': (launches, total_ms) } of the launches since profile_begin"""
        buf = C.create_string_buffer(1 << 20)
        check(lib().ug4gb_profile_end(self.h, buf, len(buf)), self.h)
        out = {}
        for line in buf.value.decode().splitlines():
            name, cnt, ms = line.split("\t")
            out[name] = (int(cnt), float(ms))
        return out

    @property
    def stream(self):
        return lib().ug4gb_stream(self.h)


class _Hierarchy:
    """Multigrid hierarchy of a grid (levels 0 .. num_levels - 1)."""

    def _init(self, ctx, elem_type, h):
        self.ctx = ctx
        self.elem_type = int(elem_type)
        self.h = h
        self.num_levels = lib().ug4gb_grid_num_levels(h)
        self.top = self.num_levels - 1
        self.dim = 2 if self.elem_type in (_lib.QUAD, _lib.TRI) else 3
        self.structured = lib().ug4gb_grid_is_structured(h) == 1

    def __del__(self):
        if getattr(self, "h", None):
            lib().ug4gb_grid_destroy(self.h)
            self.h = None

    def level_info(self, level=None):
        level = self.top if level is None else level
        nv, ne, k, dim = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        check(lib().ug4gb_grid_level_info(self.h, level, C.byref(nv), C.byref(ne), C.byref(k), C.byref(dim)))
        return dict(num_vertices=nv.value, num_elements=ne.value, corners=k.value, dim=dim.value)

    def num_vertices(self, level=None):
        return self.level_info(level)["num_vertices"]

    def num_elements(self, level=None):
        return self.level_info(level)["num_elements"]

    def export(self, level=None):
        level = self.top if level is None else level
        info = self.level_info(level)
        coords = np.zeros((info["num_vertices"], info["dim"]))
        elems = np.zeros((info["num_elements"], info["corners"]), np.int32)
        bnd = np.zeros(info["num_vertices"], np.uint8)
        check(lib().ug4gb_grid_level_export(self.h, level, _ptr(coords), _ptr(elems), _ptr(bnd)), self.ctx.h)
        return coords, elems, bnd

    def parents(self, level=None):
        """(npar, par): parents of the vertices of `level` >= 1 in level - 1"""
        level = self.top if level is None else level
        nv = self.num_vertices(level)
        npar = np.zeros(nv, np.int32)
        par = np.zeros((nv, 8), np.int32)
        check(lib().ug4gb_grid_level_parents(self.h, level, _ptr(npar), _ptr(par)), self.ctx.h)
        return npar, par


class StructuredHierarchy(_Hierarchy):
    """Uniformly refined unit square/cube: levels 0..num_refinements."""

    def __init__(self, ctx, elem, mx, my, mz=1, num_refinements=0):
        et = _ELEM[elem] if isinstance(elem, str) else int(elem)
        h = C.c_void_p()
        check(lib().ug4gb_grid_create_structured(ctx.h, et, mx, my, mz, num_refinements, C.byref(h)), ctx.h)
        self._init(ctx, et, h)


class UnstructuredHierarchy(_Hierarchy):
    """Regular refinements of an unstructured coarse grid (a UGX file, as
    util.refinement.CreateRegularHierarchy / GlobalMultiGridRefiner, or
    arrays).  dirichlet: subset names (UGX) whose objects carry the zero
    Dirichlet condition; None = the topological boundary."""

    def __init__(self, ctx, elem_type, h):
        self._init(ctx, elem_type, h)

    @classmethod
    def from_ugx(cls, ctx, filename, num_refinements=0, dirichlet=None):
        names = None if dirichlet is None else (dirichlet if isinstance(dirichlet, str) else ",".join(dirichlet))
        h = C.c_void_p()
        check(lib().ug4gb_grid_create_ugx(ctx.h, filename.encode(), num_refinements,
                                          None if names is None else names.encode(), C.byref(h)), ctx.h)
        info = C.c_int()
        k = C.c_int()
        lib().ug4gb_grid_level_info(h, 0, None, None, C.byref(k), C.byref(info))
        et = {(2, 3): _lib.TRI, (2, 4): _lib.QUAD, (3, 4): _lib.TET, (3, 8): _lib.HEX}[(info.value, k.value)]
        return cls(ctx, et, h)

    @classmethod
    def from_arrays(cls, ctx, elem, coords, elems, dirichlet_vertices=None, dirichlet_edges=None,
                    dirichlet_faces=None, num_refinements=0):
        et = _ELEM[elem] if isinstance(elem, str) else int(elem)
        x = np.ascontiguousarray(coords, np.float64)
        el = np.ascontiguousarray(elems, np.int32)
        dv = None if dirichlet_vertices is None else np.ascontiguousarray(dirichlet_vertices, np.uint8)
        de = np.zeros((0, 2), np.int32) if dirichlet_edges is None else np.ascontiguousarray(dirichlet_edges, np.int32)
        df = np.zeros((0, 4), np.int32) if dirichlet_faces is None else np.ascontiguousarray(dirichlet_faces, np.int32)
        h = C.c_void_p()
        check(lib().ug4gb_grid_create_unstructured(ctx.h, et, x.shape[0], _ptr(x), el.shape[0], _ptr(el),
                                                   None if dv is None else _ptr(dv), de.shape[0],
                                                   _ptr(de) if de.size else None, df.shape[0],
                                                   _ptr(df) if df.size else None, num_refinements, C.byref(h)),
              ctx.h)
        return cls(ctx, et, h)


class GPUVector:
    """Device vector of doubles (ug::Vector<double>)."""

    def __init__(self, ctx, n=None, wrap=None):
        self.ctx = ctx
        h = C.c_void_p()
        if wrap is not None:
            # wrap a CUDA torch tensor (float64, contiguous) without copying
            self._keep = wrap
            check(lib().ug4gb_vector_wrap(ctx.h, C.c_void_p(wrap.data_ptr()), wrap.numel(), C.byref(h)), ctx.h)
        else:
            check(lib().ug4gb_vector_create(ctx.h, int(n), C.byref(h)), ctx.h)
        self.h = h
        self.n = lib().ug4gb_vector_size(h)

    def __del__(self):
        if getattr(self, "h", None):
            lib().ug4gb_vector_destroy(self.h)
            self.h = None

    def __len__(self):
        return self.n

    def size(self):
        return self.n

    def data_ptr(self):
        return lib().ug4gb_vector_data(self.h)

    def set(self, value):
        check(lib().ug4gb_vector_set(self.h, float(value)), self.ctx.h)
        return self

    def copy_from(self, src):
        src = _f64(src)
        check(lib().ug4gb_vector_copy_from(self.h, _ptr(src)), self.ctx.h)
        return self

    def copy_to(self, dst=None):
        if dst is None:
            dst = np.zeros(self.n)
        check(lib().ug4gb_vector_copy_to(self.h, _ptr(dst)), self.ctx.h)
        return dst

    def numpy(self):
        return self.copy_to()

    def norm(self):
        out = C.c_double()
        check(lib().ug4gb_vector_norm(self.h, C.byref(out)), self.ctx.h)
        return out.value

    def maxnorm(self):
        out = C.c_double()
        check(lib().ug4gb_vector_maxnorm(self.h, C.byref(out)), self.ctx.h)
        return out.value

    def get_values(self, idx):
        i = np.ascontiguousarray(idx, np.int32)
        out = np.zeros(len(i))
        check(lib().ug4gb_vector_get_values(self.h, len(i), _ptr(i), _ptr(out)), self.ctx.h)
        return out

    def set_values(self, idx, vals):
        i = np.ascontiguousarray(idx, np.int32)
        v = np.ascontiguousarray(vals, np.float64)
        check(lib().ug4gb_vector_set_values(self.h, len(i), _ptr(i), _ptr(v)), self.ctx.h)

    def dot(self, other):
        out = C.c_double()
        check(lib().ug4gb_vector_dot(self.h, other.h, C.byref(out)), self.ctx.h)
        return out.value

    def scale_add(self, alpha, a, beta, b):
        check(lib().ug4gb_vector_scale_add(self.h, alpha, a.h, beta, b.h), self.ctx.h)
        return self

    def clone(self):
        v = GPUVector(self.ctx, self.n)
        v.scale_add(1.0, self, 0.0, self)
        return v

    def clone_without_values(self):
        return GPUVector(self.ctx, self.n)


class GPUSparseMatrix:
    """Device CRS matrix (ug::SparseMatrix<double>, defragmented form)."""

    def __init__(self, ctx):
        self.ctx = ctx
        h = C.c_void_p()
        check(lib().ug4gb_matrix_create(ctx.h, C.byref(h)), ctx.h)
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            lib().ug4gb_matrix_destroy(self.h)
            self.h = None

    def info(self):
        r, c, nnz = C.c_int(), C.c_int(), C.c_int64()
        check(lib().ug4gb_matrix_info(self.h, C.byref(r), C.byref(c), C.byref(nnz)))
        return r.value, c.value, nnz.value

    def num_rows(self):
        return self.info()[0]

    def num_cols(self):
        return self.info()[1]

    def total_num_connections(self):
        return self.info()[2]

    def set_csr(self, rowptr, col, val, num_cols=None):
        rowptr = np.ascontiguousarray(rowptr, np.int32)
        col = np.ascontiguousarray(col, np.int32)
        val = np.ascontiguousarray(val, np.float64)
        n = len(rowptr) - 1
        check(lib().ug4gb_matrix_set_csr(self.h, n, n if num_cols is None else num_cols, len(col), _ptr(rowptr),
                                         _ptr(col), _ptr(val)), self.ctx.h)
        return self

    def export_csr(self):
        r, _, nnz = self.info()
        rp = np.zeros(r + 1, np.int32)
        ci = np.zeros(nnz, np.int32)
        va = np.zeros(nnz)
        check(lib().ug4gb_matrix_export_csr(self.h, _ptr(rp), _ptr(ci), _ptr(va)), self.ctx.h)
        return rp, ci, va

    def axpy(self, dest, alpha1, v1, beta1, w1):
        """dest = alpha1*v1 + beta1*A*w1"""
        check(lib().ug4gb_matrix_axpy(self.h, dest.h, alpha1, v1.h if v1 is not None else None, beta1, w1.h),
              self.ctx.h)

    def axpy_transposed(self, dest, alpha1, v1, beta1, w1):
        check(lib().ug4gb_matrix_axpy_transposed(self.h, dest.h, alpha1, v1.h if v1 is not None else None, beta1,
                                                 w1.h), self.ctx.h)

    def apply(self, f, u):
        """f = A u"""
        self.axpy(f, 0.0, None, 1.0, u)

    def apply_transposed(self, f, u):
        self.axpy_transposed(f, 0.0, None, 1.0, u)

    def matmul_minus(self, res, x):
        """res -= A x"""
        self.axpy(res, 1.0, res, -1.0, x)

    def resize_and_clear(self, num_rows, num_cols):
        check(lib().ug4gb_matrix_resize_and_clear(self.h, num_rows, num_cols), self.ctx.h)
        return self

    def clear_retain_structure(self):
        check(lib().ug4gb_matrix_clear_retain_structure(self.h), self.ctx.h)
        return self

    def set_as_copy_of(self, B, scale=1.0):
        check(lib().ug4gb_matrix_set_as_copy_of(self.h, B.h, float(scale)), self.ctx.h)
        return self

    def scale(self, alpha):
        check(lib().ug4gb_matrix_scale(self.h, float(alpha)), self.ctx.h)
        return self

    def apply_ignore_zero_rows(self, dest, beta, w):
        check(lib().ug4gb_matrix_apply_ignore_zero_rows(self.h, dest.h, float(beta), w.h), self.ctx.h)

    def row(self, r):
        """(columns, values) of row r, copied to the host"""
        n = lib().ug4gb_matrix_get_row(self.h, r, None, None, 0)
        check(min(n, 0), self.ctx.h)
        ci, va = np.zeros(n, np.int32), np.zeros(n)
        lib().ug4gb_matrix_get_row(self.h, r, _ptr(ci) if n else None, _ptr(va) if n else None, n)
        return ci, va

    def add_entries(self, rows, cols, vals):
        """A(r, c) += v for entries of the existing pattern"""
        r = np.ascontiguousarray(rows, np.int32)
        c = np.ascontiguousarray(cols, np.int32)
        v = np.ascontiguousarray(vals, np.float64)
        check(lib().ug4gb_matrix_add_entries(self.h, len(r), _ptr(r), _ptr(c), _ptr(v)), self.ctx.h)

    def set_as_transpose_of(self, B, keep_zeros=True):
        check(lib().ug4gb_matrix_set_as_transpose_of(self.h, B.h, 1 if keep_zeros else 0), self.ctx.h)
        return self


class DomainDiscretization:
    """DomainDiscretization with one FV1 convection-diffusion element disc
    (-div(K grad u) + div(v u) = f) and zero Dirichlet values on the whole
    boundary."""

    def __init__(self, hier):
        self.ctx = hier.ctx
        self.hier = hier
        h = C.c_void_p()
        check(lib().ug4gb_disc_create(self.ctx.h, hier.h, C.byref(h)), self.ctx.h)
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            lib().ug4gb_disc_destroy(self.h)
            self.h = None

    def set_diffusion(self, K):
        check(lib().ug4gb_disc_set_diffusion_constant(self.h, float(K)), self.ctx.h)

    def set_diffusion_field(self, field, factor=2.0):
        """K = exp(factor * g(centroid)) for a fields.ScalarField g."""
        self._kk = np.ascontiguousarray(field.k, np.float64)
        self._kp = np.ascontiguousarray(field.phase, np.float64)
        check(lib().ug4gb_disc_set_diffusion_fourier(self.h, field.nmodes, _ptr(self._kk), _ptr(self._kp),
                                                     field.amp, factor), self.ctx.h)

    def set_log_diffusion(self, m_top):
        """K = exp(m) per top-level element (host array or CUDA tensor)."""
        m_top = _f64(m_top)
        check(lib().ug4gb_disc_set_log_diffusion_elements(self.h, _ptr(m_top)), self.ctx.h)

    def set_velocity_field(self, field, scale):
        """v = scale * field(x) for a fields.CurlField (already normalised to |v| <= 1)."""
        self._vk = np.ascontiguousarray(field.k, np.float64)
        self._vc = np.ascontiguousarray(field.c, np.float64)
        self._vp = np.ascontiguousarray(field.phase, np.float64)
        check(lib().ug4gb_disc_set_velocity_fourier_curl(self.h, field.nmodes, _ptr(self._vk), _ptr(self._vc),
                                                         _ptr(self._vp), field.scale * scale), self.ctx.h)

    def set_upwind(self, upwind="full"):
        check(lib().ug4gb_disc_set_upwind(self.h, _lib.UPWIND_FULL if upwind in ("full", 1, True) else
                                          _lib.UPWIND_NONE), self.ctx.h)

    def set_source(self, f_top):
        f_top = _f64(f_top)
        check(lib().ug4gb_disc_set_source_vertices(self.h, _ptr(f_top)), self.ctx.h)

    def set_source_uniform(self, seed):
        check(lib().ug4gb_disc_set_source_uniform(self.h, int(seed)), self.ctx.h)

    def assemble_linear(self, A, b, level=None):
        level = self.hier.top if level is None else level
        check(lib().ug4gb_disc_assemble_linear(self.h, level, A.h, b.h), self.ctx.h)

    def assemble_jacobian(self, A, level=None):
        level = self.hier.top if level is None else level
        check(lib().ug4gb_disc_assemble_jacobian(self.h, level, A.h), self.ctx.h)

    def assemble_defect(self, d, u, level=None):
        """d = A(u) u - f element by element, 0 at Dirichlet vertices"""
        level = self.hier.top if level is None else level
        check(lib().ug4gb_disc_assemble_defect(self.h, level, u.h, d.h), self.ctx.h)

    def adjust_solution(self, u, level=None):
        """Dirichlet values (0) into u"""
        level = self.hier.top if level is None else level
        check(lib().ug4gb_disc_adjust_solution(self.h, level, u.h), self.ctx.h)

    def adjoint_operator(self, A, AT, level=None):
        """AT = A^T with Dirichlet rows reset to identity."""
        level = self.hier.top if level is None else level
        check(lib().ug4gb_disc_adjoint_operator(self.h, level, A.h, AT.h), self.ctx.h)
        return AT

    def coefficients(self, level=None):
        level = self.hier.top if level is None else level
        K = np.zeros(self.hier.num_elements(level))
        check(lib().ug4gb_disc_export_coefficients(self.h, level, _ptr(K)), self.ctx.h)
        return K

    def grad_logk(self, u, lam, out=None):
        if out is None:
            out = np.zeros(self.hier.num_elements())
        check(lib().ug4gb_disc_grad_logk(self.h, u.h, lam.h, _ptr(out)), self.ctx.h)
        return out

    def grad_source(self, lam, out=None):
        if out is None:
            out = np.zeros(self.hier.num_vertices())
        check(lib().ug4gb_disc_grad_source(self.h, lam.h, _ptr(out)), self.ctx.h)
        return out


class ThetaTimeStep:
    """ThetaTimeStep(domainDisc) (theta_time_step.h:165): the theta scheme
    (M + theta dt A) u_new = M u_old - (1 - theta) dt A u_old + dt f with the
    lumped FV1 mass; theta = 1 implicit Euler, 0.5 Crank-Nicolson."""

    def __init__(self, disc, theta=1.0):
        self.ctx = disc.ctx
        self.disc = disc
        h = C.c_void_p()
        check(lib().ug4gb_timedisc_create(self.ctx.h, disc.h, C.byref(h)), self.ctx.h)
        self.h = h
        self.set_theta(theta)

    def __del__(self):
        if getattr(self, "h", None):
            lib().ug4gb_timedisc_destroy(self.h)
            self.h = None

    def set_theta(self, theta):
        check(lib().ug4gb_timedisc_set_theta(self.h, float(theta)), self.ctx.h)

    def prepare_step(self, u_old, t_old, dt):
        """previous solution (GPUVector of the top level), its time, the step size"""
        check(lib().ug4gb_timedisc_prepare_step(self.h, u_old.h, float(t_old), float(dt)), self.ctx.h)

    def future_time(self):
        t = C.c_double()
        check(lib().ug4gb_timedisc_future_time(self.h, C.byref(t)), self.ctx.h)
        return t.value

    def assemble_linear(self, A, b, level=None):
        level = self.disc.hier.num_levels - 1 if level is None else level
        check(lib().ug4gb_timedisc_assemble_linear(self.h, level, A.h, b.h), self.ctx.h)

    def assemble_jacobian(self, A, level=None):
        level = self.disc.hier.num_levels - 1 if level is None else level
        check(lib().ug4gb_timedisc_assemble_jacobian(self.h, level, A.h), self.ctx.h)

    def assemble_defect(self, d, u):
        """time-discrete defect of u at the future time (top level)"""
        check(lib().ug4gb_timedisc_assemble_defect(self.h, self.disc.hier.num_levels - 1, u.h, d.h), self.ctx.h)


class Jacobi:
    """damped Jacobi smoother (jacobi.h); damp is the ugcore damping factor"""

    def __init__(self, damp=1.0):
        self.kind, self.damp = _lib.SMOOTHER_JACOBI, float(damp)


class _SorRelax:
    def set_sor_relax(self, relax):
        """GaussSeidelBase::set_sor_relax (gauss_seidel.h:96)"""
        self.damp = float(relax)
        return self


class GaussSeidel(_SorRelax):
    """multicolour Gauss-Seidel smoother (opt-in GPU variant of gauss_seidel.h)"""

    def __init__(self, relax=1.0):
        self.kind, self.damp = _lib.SMOOTHER_MCGS, float(relax)


class BackwardGaussSeidel(_SorRelax):
    """backward multicolour Gauss-Seidel: colours in decreasing order (GPU
    variant of BackwardGaussSeidel, gauss_seidel.h:316)"""

    def __init__(self, relax=1.0):
        self.kind, self.damp = _lib.SMOOTHER_MCBGS, float(relax)


class LU:
    """dense partially pivoted LU as the multigrid's base solver (lu.h:50;
    the default, base levels of at most 4096 unknowns)"""
    kind, steps = _lib.BASE_LU, 0


class BaseSmoothing:
    """the base solver as `steps` steps of the multigrid's pre-smoother from
    a zero correction: ugcore's LinearSolver with that smoother and
    StdConvCheck(steps, 0, 0) whose unsuccessful end is suppressed
    (convergence_check.h:191); for base levels too large for the dense LU"""

    def __init__(self, steps=10):
        self.kind, self.steps = _lib.BASE_SMOOTHER, int(steps)


class ILU:
    """ILU(0) smoother in multicolour order (GPU variant of ILU, ilu.h);
    damp scales the correction"""

    def __init__(self, damp=1.0):
        self.kind, self.damp = _lib.SMOOTHER_ILU, float(damp)


class SymmetricGaussSeidel(_SorRelax):
    """symmetric multicolour Gauss-Seidel: forward, then backward colour sweep
    (GPU variant of SymmetricGaussSeidel, gauss_seidel.h:350)"""

    def __init__(self, relax=1.0):
        self.kind, self.damp = _lib.SMOOTHER_MCSGS, float(relax)


class DofPermutation:
    """DoF permutation between the engine's vertex numbering of a level and
    an external numbering (ugcore's DoFDistribution): perm[i] = engine index
    of external DoF i.  No ugcore counterpart."""

    def __init__(self, ctx, perm=None, hier=None, level=None, positions=None, tol=1e-9):
        self.ctx = ctx
        h = C.c_void_p()
        if perm is not None:
            self._perm = np.ascontiguousarray(perm, np.int32)
            check(lib().ug4gb_perm_create(ctx.h, len(self._perm), _ptr(self._perm), C.byref(h)), ctx.h)
        else:
            level = hier.top if level is None else level
            x = np.ascontiguousarray(positions, np.float64)
            check(lib().ug4gb_perm_from_positions(ctx.h, hier.h, level, x.shape[0], _ptr(x), float(tol),
                                                  C.byref(h)), ctx.h)
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            lib().ug4gb_perm_destroy(self.h)
            self.h = None

    def vector(self, src, dst, to_external=True):
        check(lib().ug4gb_perm_vector(self.h, int(bool(to_external)), src.h, dst.h), self.ctx.h)
        return dst

    def matrix(self, A, B, to_external=True):
        check(lib().ug4gb_perm_matrix(self.h, int(bool(to_external)), A.h, B.h), self.ctx.h)
        return B


class StdTransfer:
    """StdTransfer (lib_disc/operator/linear_operator/std_transfer.h:57): P1
    prolongation / restriction between the levels of the hierarchy.  The
    damping factors scale the applied transfers (not the assembled
    matrices).  enable_p1_lagrange_optimization selects ugcore's assembly
    shortcut for P1 elements under regular refinement; the hierarchies here
    are always regularly refined, where both assembly paths give the same P,
    so the flag is kept but changes nothing."""

    def __init__(self):
        self.prolongation_damping = 1.0
        self.restriction_damping = 1.0
        self.p1_lagrange_optimization = True

    def set_prolongation_damping(self, damp):
        self.prolongation_damping = float(damp)

    def set_restriction_damping(self, damp):
        self.restriction_damping = float(damp)

    def enable_p1_lagrange_optimization(self, enable=True):
        self.p1_lagrange_optimization = bool(enable)


class GeometricMultiGrid:
    """AssembledMultiGridCycle: V/W cycle, re-assembled level operators,
    StdTransfer, LU base solver."""

    def __init__(self, disc):
        self.ctx = disc.ctx
        self.disc = disc
        h = C.c_void_p()
        check(lib().ug4gb_gmg_create(self.ctx.h, disc.h, C.byref(h)), self.ctx.h)
        self.h = h
        self.set_smoother(Jacobi(0.6))

    def __del__(self):
        if getattr(self, "h", None):
            lib().ug4gb_gmg_destroy(self.h)
            self.h = None

    def set_smoother(self, sm):
        check(lib().ug4gb_gmg_set_smoother(self.h, sm.kind, sm.damp), self.ctx.h)

    def set_presmoother(self, sm):
        """set_presmoother (mg_solver.h:179-183); Gauss-Seidel kinds and ILU
        combine freely with a different post-smoother, Jacobi only with the
        same Jacobi"""
        check(lib().ug4gb_gmg_set_presmoother(self.h, sm.kind, sm.damp), self.ctx.h)

    def set_postsmoother(self, sm):
        check(lib().ug4gb_gmg_set_postsmoother(self.h, sm.kind, sm.damp), self.ctx.h)

    def set_cycle_type(self, cycle):
        """"V" (1), "W" (2), gamma up to 4, or "F" (-1), as set_cycle_type"""
        c = {"V": 1, "W": 2, "F": -1}[cycle] if isinstance(cycle, str) else int(cycle)
        check(lib().ug4gb_gmg_set_cycle_type(self.h, c), self.ctx.h)

    def set_num_presmooth(self, n):
        check(lib().ug4gb_gmg_set_num_presmooth(self.h, n), self.ctx.h)

    def set_num_postsmooth(self, n):
        check(lib().ug4gb_gmg_set_num_postsmooth(self.h, n), self.ctx.h)

    def set_base_level(self, level):
        check(lib().ug4gb_gmg_set_base_level(self.h, level), self.ctx.h)

    def set_base_solver(self, solver):
        """set_base_solver (mg_solver.h:136): LU() or BaseSmoothing(steps)"""
        check(lib().ug4gb_gmg_set_base_solver(self.h, solver.kind, solver.steps), self.ctx.h)

    def set_precision(self, prec):
        p = {"fp64": _lib.PREC_FP64, "mixed": _lib.PREC_MIXED, 0: 0, 1: 1}[prec]
        check(lib().ug4gb_gmg_set_precision(self.h, p), self.ctx.h)

    def set_discretization(self, td):
        """assemble the coarse levels with a ThetaTimeStep's jacobian (None: the
        stationary discretisation); init() follows its prepare_step"""
        check(lib().ug4gb_gmg_set_time_disc(self.h, td.h if td is not None else None), self.ctx.h)
        self._td = td

    def set_rap(self, flag=True):
        """Galerkin coarse operators R A P instead of re-assembly (set_rap)"""
        check(lib().ug4gb_gmg_set_rap(self.h, int(bool(flag))), self.ctx.h)

    def set_transposed(self, flag=True):
        check(lib().ug4gb_gmg_set_transposed(self.h, 1 if flag else 0), self.ctx.h)

    def set_transfer(self, transfer):
        """AssembledMultiGridCycle::set_transfer (mg_solver.h:146) with a
        StdTransfer: its prolongation and restriction damping"""
        self.transfer_op = transfer
        check(lib().ug4gb_gmg_set_prolongation_damping(self.h, float(transfer.prolongation_damping)), self.ctx.h)
        check(lib().ug4gb_gmg_set_restriction_damping(self.h, float(transfer.restriction_damping)), self.ctx.h)

    def init(self, A):
        check(lib().ug4gb_gmg_init(self.h, A.h), self.ctx.h)

    def apply(self, c, d):
        check(lib().ug4gb_gmg_apply(self.h, c.h, d.h), self.ctx.h)

    def transfer(self, level, which):
        """(rowptr, col, val) of P (which=0) or R (which=1) of fine level `level`."""
        r, cc, nnz = C.c_int(), C.c_int(), C.c_int64()
        check(lib().ug4gb_gmg_transfer_info(self.h, level, which, C.byref(r), C.byref(cc), C.byref(nnz)),
              self.ctx.h)
        rp = np.zeros(r.value + 1, np.int32)
        ci = np.zeros(nnz.value, np.int32)
        va = np.zeros(nnz.value)
        check(lib().ug4gb_gmg_export_transfer(self.h, level, which, _ptr(rp), _ptr(ci), _ptr(va)), self.ctx.h)
        return rp, ci, va

    def level_matrix(self, level):
        """(rowptr, col, val) of the multigrid's FP64 operator of `level`
        (re-assembled, or R A P with set_rap)."""
        r, nnz = C.c_int(), C.c_int64()
        check(lib().ug4gb_gmg_level_info(self.h, level, C.byref(r), C.byref(nnz)), self.ctx.h)
        rp = np.zeros(r.value + 1, np.int32)
        ci = np.zeros(nnz.value, np.int32)
        va = np.zeros(nnz.value)
        check(lib().ug4gb_gmg_export_level(self.h, level, _ptr(rp), _ptr(ci), _ptr(va)), self.ctx.h)
        return rp, ci, va


class StdConvCheck:
    def __init__(self, max_steps=100, min_defect=1e-300, rel_reduction=1e-10):
        self.max_steps, self.min_defect, self.rel_reduction = int(max_steps), float(min_defect), float(rel_reduction)


class _Krylov:
    KIND = None

    def __init__(self, ctx):
        self.ctx = ctx
        h = C.c_void_p()
        check(lib().ug4gb_solver_create(ctx.h, self.KIND, C.byref(h)), ctx.h)
        self.h = h
        self.pre = None
        self.set_convergence_check(StdConvCheck())

    def __del__(self):
        if getattr(self, "h", None):
            lib().ug4gb_solver_destroy(self.h)
            self.h = None

    def set_preconditioner(self, gmg):
        self.pre = gmg
        check(lib().ug4gb_solver_set_preconditioner(self.h, gmg.h if gmg is not None else None), self.ctx.h)

    def set_convergence_check(self, cc):
        self.conv = cc
        check(lib().ug4gb_solver_set_convergence_check(self.h, cc.max_steps, cc.min_defect, cc.rel_reduction),
              self.ctx.h)

    def init(self, A):
        self.A = A
        check(lib().ug4gb_solver_init(self.h, A.h), self.ctx.h)

    def apply_return_defect(self, x, b, raise_on_failure=True):
        rc = lib().ug4gb_solver_apply_return_defect(self.h, x.h, b.h)
        return self._finish(rc, raise_on_failure)

    def apply(self, x, b, raise_on_failure=True):
        rc = lib().ug4gb_solver_apply(self.h, x.h, b.h)
        return self._finish(rc, raise_on_failure)

    def solve_host(self, b_host, x_host, raise_on_failure=True):
        """b, x: host arrays (numpy or pinned torch); x = A^{-1} b from x0 = 0."""
        rc = lib().ug4gb_solver_solve_host(self.h, _ptr(b_host), _ptr(x_host))
        return self._finish(rc, raise_on_failure)

    def _finish(self, rc, raise_on_failure):
        if rc != 0 and (raise_on_failure or rc not in (_lib.ERR_NOT_CONVERGED, _lib.ERR_BREAKDOWN)):
            check(rc, self.ctx.h)
        return rc == 0

    def stats(self):
        steps, d0, d1, conv = C.c_int(), C.c_double(), C.c_double(), C.c_int()
        check(lib().ug4gb_solver_get_stats(self.h, C.byref(steps), C.byref(d0), C.byref(d1), C.byref(conv)))
        return dict(steps=steps.value, initial_defect=d0.value, defect=d1.value, converged=bool(conv.value))

    def history(self):
        cap = self.conv.max_steps + 2
        buf = np.zeros(cap)
        n = lib().ug4gb_solver_get_history(self.h, _ptr(buf), cap)
        return buf[:max(n, 0)]


class AssembledOperator:
    """AssembledOperator(domainDisc | timeDisc): the nonlinear operator N(u)
    whose defect and jacobian the discretisation assembles"""

    def __init__(self, disc):
        self.disc = disc


class StandardLineSearch:
    """StandardLineSearch (line_search.h:115-400): the constructor's defaults
    and its setters; handed to NewtonSolver.set_line_search."""

    def __init__(self, max_steps=10, lambda_start=1.0, lambda_reduce=0.5, accept_best=False, check_all=False):
        self.max_steps = int(max_steps)
        self.lambda_start = float(lambda_start)
        self.lambda_reduce = float(lambda_reduce)
        self.suff_descent_factor = 0.25
        self.accept_best = bool(accept_best)
        self.check_all = bool(check_all)
        self.max_defect = 1e10

    def set_maximum_steps(self, steps):
        self.max_steps = int(steps)

    def set_lambda_start(self, start):
        self.lambda_start = float(start)

    def set_reduce_factor(self, factor):
        self.lambda_reduce = float(factor)

    def set_suff_descent_factor(self, factor):
        self.suff_descent_factor = float(factor)

    def set_accept_best(self, b):
        self.accept_best = bool(b)

    def set_check_all(self, b):
        self.check_all = bool(b)

    def set_maximum_defect(self, d):
        self.max_defect = float(d)


class NewtonSolver:
    """NewtonSolver (newton.h:62): set_linear_solver, set_convergence_check,
    set_line_search (StandardLineSearch or None), init(AssembledOperator),
    prepare(u), apply(u)."""

    def __init__(self, ctx):
        self.ctx = ctx
        h = C.c_void_p()
        check(lib().ug4gb_newton_create(ctx.h, C.byref(h)), ctx.h)
        self.h = h
        self.conv = StdConvCheck(10, 1e-50, 1e-10)
        check(lib().ug4gb_newton_set_convergence_check(self.h, 10, 1e-50, 1e-10), ctx.h)

    def __del__(self):
        if getattr(self, "h", None):
            lib().ug4gb_newton_destroy(self.h)
            self.h = None

    def set_linear_solver(self, solver):
        self._lin = solver
        check(lib().ug4gb_newton_set_linear_solver(self.h, solver.h), self.ctx.h)

    def set_convergence_check(self, cc):
        self.conv = cc
        check(lib().ug4gb_newton_set_convergence_check(self.h, cc.max_steps, cc.min_defect, cc.rel_reduction),
              self.ctx.h)

    def set_line_search(self, ls):
        if ls is None:
            check(lib().ug4gb_newton_clear_line_search(self.h), self.ctx.h)
            return
        check(lib().ug4gb_newton_set_line_search(self.h, ls.max_steps, ls.lambda_start, ls.lambda_reduce,
                                                 ls.suff_descent_factor, int(ls.accept_best), int(ls.check_all),
                                                 ls.max_defect), self.ctx.h)

    def set_reassemble_J_freq(self, freq):
        """assemble the jacobian only in steps 0, freq, 2 freq, ... (0: every step)"""
        check(lib().ug4gb_newton_set_reassemble_J_freq(self.h, int(freq)), self.ctx.h)

    def num_jacobian_assemblies(self):
        return lib().ug4gb_newton_num_jacobian_assemblies(self.h)

    def line_search_history(self):
        """per Newton step of the last apply: (tries evaluated, accepted lambda)"""
        cap = self.conv.max_steps + 1
        tries = np.zeros(cap, np.int32)
        lam = np.zeros(cap)
        n = lib().ug4gb_newton_get_line_search_history(self.h, _ptr(tries), _ptr(lam), cap)
        return tries[:max(n, 0)].tolist(), lam[:max(n, 0)].tolist()

    def init(self, op):
        d = op.disc if isinstance(op, AssembledOperator) else op
        self._op = d
        if isinstance(d, ThetaTimeStep):
            check(lib().ug4gb_newton_init(self.h, None, d.h), self.ctx.h)
        else:
            check(lib().ug4gb_newton_init(self.h, d.h, None), self.ctx.h)

    def prepare(self, u):
        check(lib().ug4gb_newton_prepare(self.h, u.h), self.ctx.h)

    def apply(self, u, raise_on_failure=True):
        rc = lib().ug4gb_newton_apply(self.h, u.h)
        if rc != 0 and (raise_on_failure or rc != _lib.ERR_NOT_CONVERGED):
            check(rc, self.ctx.h)
        return rc == 0

    def stats(self):
        steps, d0, d1 = C.c_int(), C.c_double(), C.c_double()
        ls = np.zeros(self.conv.max_steps + 1, np.int32)
        check(lib().ug4gb_newton_get_stats(self.h, C.byref(steps), C.byref(d0), C.byref(d1), _ptr(ls), len(ls)))
        return dict(steps=steps.value, initial_defect=d0.value, defect=d1.value,
                    linear_steps=[int(x) for x in ls[:steps.value]])

    def history(self):
        buf = np.zeros(self.conv.max_steps + 2)
        n = lib().ug4gb_newton_get_history(self.h, _ptr(buf), len(buf))
        return buf[:max(n, 0)]


class CG(_Krylov):
    KIND = _lib.SOLVER_CG


class BiCGStab(_Krylov):
    KIND = _lib.SOLVER_BICGSTAB

    def set_restart(self, num_restarts):
        """restart every num_restarts steps of the convergence check (which
        counts half steps); 0 = never (bicgstab.h:387)"""
        check(lib().ug4gb_solver_set_restart(self.h, int(num_restarts)), self.ctx.h)

    def set_min_orthogonality(self, min_ortho):
        """restart when |(r, r0)| <= min_ortho |r| |r0| (bicgstab.h:390)"""
        check(lib().ug4gb_solver_set_min_orthogonality(self.h, float(min_ortho)), self.ctx.h)
