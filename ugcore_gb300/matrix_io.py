"""Matrix and vector files in ugcore's formats, through the C ABI.

Function names follow the ugcore registry:

    ugcore (Lua)                                  here
    --------------------------------------------  ------------------------------------------
    SaveMatrixToMTX(filename, A, comment)         SaveMatrixToMTX(filename, A, comment)
      (bridge/disc_bridges/output_bridge.cpp:309-315)
    MatrixIOMtx(filename):read_into(A)            ReadMatrixFromMTX(filename, A)
    SaveMatrixForConnectionViewer(u, A, file)     SaveMatrixForConnectionViewer(hier, A, file, level)
    SaveVectorForConnectionViewer(u, file)        SaveVectorForConnectionViewer(hier, v, file, level)
    LoadVector(u, file)                           LoadVector(v, file)
      (output_bridge.cpp:212-240)

ugcore takes the vertex positions from the GridFunction's approximation
space; here they come from a StructuredHierarchy level (the top level by
default).  The host-array functions (write_mtx, read_mtx, write_cv_matrix,
write_cv_vector, read_cv_vector) need neither a context nor a GPU.
"""
import ctypes as C

import numpy as np

from ._lib import UG4GBError, check, lib

_ERRCAP = 512


def _raise(rc, err):
    if rc != 0:
        raise UG4GBError(rc, err.value.decode(errors="replace"))


def _p(a):
    return C.c_void_p(a.ctypes.data) if a is not None and a.size else None


def _csr(rowptr, col, val):
    return (np.ascontiguousarray(rowptr, np.int32), np.ascontiguousarray(col, np.int32),
            np.ascontiguousarray(val, np.float64))


def _enc(s):
    return None if s is None else s.encode()


# ---- host arrays --------------------------------------------------------
def write_mtx(filename, rowptr, col, val, num_cols=None, comment=None):
    """MatrixMarket file of a host CRS (columns strictly increasing per row)."""
    rp, ci, va = _csr(rowptr, col, val)
    n = len(rp) - 1
    err = C.create_string_buffer(_ERRCAP)
    _raise(lib().ug4gb_io_write_mtx(n, n if num_cols is None else int(num_cols), _p(rp), _p(ci), _p(va),
                                    filename.encode(), _enc(comment), err, _ERRCAP), err)


def read_mtx(filename):
    """(rowptr, col, val, num_cols) read as MatrixIOMtx::read_into does."""
    err = C.create_string_buffer(_ERRCAP)
    r, c, nnz = C.c_int(), C.c_int(), C.c_int64()
    _raise(lib().ug4gb_io_read_mtx_info(filename.encode(), C.byref(r), C.byref(c), C.byref(nnz), err, _ERRCAP), err)
    rp = np.zeros(r.value + 1, np.int32)
    ci = np.zeros(max(nnz.value, 1), np.int32)
    va = np.zeros(max(nnz.value, 1))
    _raise(lib().ug4gb_io_read_mtx(filename.encode(), _p(rp), _p(ci), _p(va), err, _ERRCAP), err)
    return rp, ci[:nnz.value], va[:nnz.value], c.value


def write_cv_matrix(filename, rowptr, col, val, positions):
    """ConnectionViewer .mat of a host CRS; positions: (num_rows, dim)."""
    rp, ci, va = _csr(rowptr, col, val)
    pos = np.ascontiguousarray(positions, np.float64)
    err = C.create_string_buffer(_ERRCAP)
    _raise(lib().ug4gb_io_write_cv_matrix(len(rp) - 1, _p(rp), _p(ci), _p(va), pos.shape[1], _p(pos),
                                          filename.encode(), err, _ERRCAP), err)


def write_cv_vector(filename, values, positions):
    v = np.ascontiguousarray(values, np.float64)
    pos = np.ascontiguousarray(positions, np.float64)
    err = C.create_string_buffer(_ERRCAP)
    _raise(lib().ug4gb_io_write_cv_vector(len(v), _p(v), pos.shape[1], _p(pos), filename.encode(), err, _ERRCAP),
           err)


def read_cv_vector(filename, n):
    v = np.zeros(n)
    err = C.create_string_buffer(_ERRCAP)
    _raise(lib().ug4gb_io_read_cv_vector(filename.encode(), n, _p(v) if n else None, err, _ERRCAP), err)
    return v


# ---- device objects (ugcore's names) -------------------------------------
def SaveMatrixToMTX(filename, A, comment="%Generated with ug4."):
    check(lib().ug4gb_matrix_write_mtx(A.h, filename.encode(), _enc(comment)), A.ctx.h)


def ReadMatrixFromMTX(filename, A):
    check(lib().ug4gb_matrix_read_mtx(A.h, filename.encode()), A.ctx.h)
    return A


def SaveMatrixForConnectionViewer(hier, A, filename, level=None):
    level = hier.num_levels - 1 if level is None else level
    check(lib().ug4gb_matrix_write_cv(A.h, hier.h, level, filename.encode()), A.ctx.h)


def SaveVectorForConnectionViewer(hier, v, filename, level=None):
    level = hier.num_levels - 1 if level is None else level
    check(lib().ug4gb_vector_write_cv(v.h, hier.h, level, filename.encode()), v.ctx.h)


def SaveVectorDiffForConnectionViewer(hier, a, b, filename, level=None):
    """a - b as a .vec file (output_bridge.cpp:226-232; WriteVector with a
    compare vector, connection_viewer_output.h:413-418)"""
    from .algebra import GPUVector
    d = GPUVector(a.ctx, len(a))
    d.scale_add(1.0, a, -1.0, b)
    SaveVectorForConnectionViewer(hier, d, filename, level)


def LoadVector(v, filename):
    check(lib().ug4gb_vector_read_cv(v.h, filename.encode()), v.ctx.h)
    return v


# ---- UGX coarse grids (host only) -----------------------------------------
def ugx_level(filename, num_refinements, level, dirichlet=None):
    """Level `level` of the hierarchy ug4gb_grid_create_ugx builds, computed
    on the host (no context, no GPU): dict with elem_type, coords, elems,
    dirichlet (vertex flags), npar, par (level >= 1)."""
    names = None if dirichlet is None else (dirichlet if isinstance(dirichlet, str) else ",".join(dirichlet))
    nb = None if names is None else names.encode()
    err = C.create_string_buffer(_ERRCAP)
    et, nv, ne = C.c_int(), C.c_int(), C.c_int()
    _raise(lib().ug4gb_io_ugx_level(filename.encode(), num_refinements, nb, level, C.byref(et), C.byref(nv),
                                    C.byref(ne), None, None, None, None, None, err, _ERRCAP), err)
    dim = 2 if et.value in (0, 3) else 3
    k = {0: 4, 1: 8, 2: 4, 3: 3}[et.value]
    coords = np.zeros((nv.value, dim))
    elems = np.zeros((ne.value, k), np.int32)
    bnd = np.zeros(nv.value, np.uint8)
    npar = np.zeros(nv.value, np.int32)
    par = np.zeros((nv.value, 8), np.int32)
    _raise(lib().ug4gb_io_ugx_level(filename.encode(), num_refinements, nb, level, C.byref(et), C.byref(nv),
                                    C.byref(ne), _p(coords), _p(elems), _p(bnd),
                                    _p(npar) if level else None, _p(par) if level else None, err, _ERRCAP), err)
    return dict(elem_type=et.value, coords=coords, elems=elems, dirichlet=bnd,
                npar=npar if level else None, par=par if level else None)
