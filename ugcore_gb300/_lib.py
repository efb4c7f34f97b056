"""ctypes binding of libug4gb.so (the C ABI declared in include/ug4gb.h).

Loading fails loudly when the library has not been built: there is no CPU
fallback anywhere in this package.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
# UG4GB_LIB_PATH: another build of the same sources (the sanitizer build
# tests/test_sanitizers.py loads); the default is the in-tree library
LIB_PATH = os.environ.get("UG4GB_LIB_PATH") or os.path.join(HERE, "libug4gb.so")

OK = 0
ERR_INVALID, ERR_CUDA, ERR_NOMEM, ERR_SINGULAR, ERR_NOT_CONVERGED, ERR_BREAKDOWN, ERR_STATE = -1, -2, -3, -4, -5, -6, -7
QUAD, HEX, TET, TRI = 0, 1, 2, 3
SMOOTHER_JACOBI, SMOOTHER_MCGS, SMOOTHER_MCSGS, SMOOTHER_ILU, SMOOTHER_MCBGS = 0, 1, 2, 3, 4
BASE_LU, BASE_SMOOTHER = 0, 1
PREC_FP64, PREC_MIXED = 0, 1
SOLVER_CG, SOLVER_BICGSTAB = 0, 1
UPWIND_NONE, UPWIND_FULL = 0, 1
TUNE_PDL = 1
TUNE_SWEEP_FUSION = 2
TUNE_SWEEP_PLANES = 3
TUNE_ROW_ASSEMBLY = 4
TUNE_SWEEP_WAIT_TEST = 5
TUNE_COARSE_LEVELS = 6

_ERRNAMES = {ERR_INVALID: "invalid argument", ERR_CUDA: "CUDA error", ERR_NOMEM: "out of device memory",
             ERR_SINGULAR: "singular base matrix", ERR_NOT_CONVERGED: "not converged",
             ERR_BREAKDOWN: "Krylov breakdown", ERR_STATE: "wrong call order"}


class UG4GBError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (_ERRNAMES.get(code, "error"), code, msg))
        self.code = code


P = C.c_void_p
I = C.c_int
D = C.c_double
I64 = C.c_int64
PP = C.POINTER(C.c_void_p)
PI = C.POINTER(C.c_int)
PD = C.POINTER(C.c_double)
PI64 = C.POINTER(C.c_int64)

# name: (restype, argtypes)
_SIGS = {
    "ug4gb_create": (I, [I, PP]),
    "ug4gb_destroy": (None, [P]),
    "ug4gb_last_error": (C.c_char_p, [P]),
    "ug4gb_synchronize": (I, [P]),
    "ug4gb_stream": (P, [P]),
    "ug4gb_kernel_launches": (I64, [P]),
    "ug4gb_set_operator_format": (I, [P, I]),
    "ug4gb_set_tuning": (I, [P, I, I]),
    "ug4gb_profile_begin": (I, [P]),
    "ug4gb_profile_end": (I, [P, C.c_char_p, I]),
    "ug4gb_debug_guard_check": (I, [C.c_char_p, I]),
    "ug4gb_grid_create_structured": (I, [P, I, I, I, I, I, PP]),
    "ug4gb_grid_num_levels": (I, [P]),
    "ug4gb_grid_level_info": (I, [P, I, PI, PI, PI, PI]),
    "ug4gb_grid_level_export": (I, [P, I, P, P, P]),
    "ug4gb_grid_destroy": (None, [P]),
    "ug4gb_grid_create_ugx": (I, [P, C.c_char_p, I, C.c_char_p, PP]),
    "ug4gb_grid_create_unstructured": (I, [P, I, I, P, I, P, P, I, P, I, P, I, PP]),
    "ug4gb_grid_is_structured": (I, [P]),
    "ug4gb_grid_level_parents": (I, [P, I, P, P]),
    "ug4gb_io_ugx_level": (I, [C.c_char_p, I, C.c_char_p, I, PI, PI, PI, P, P, P, P, P, C.c_char_p, I]),
    "ug4gb_vector_create": (I, [P, I, PP]),
    "ug4gb_vector_wrap": (I, [P, P, I, PP]),
    "ug4gb_vector_size": (I, [P]),
    "ug4gb_vector_data": (P, [P]),
    "ug4gb_vector_set": (I, [P, D]),
    "ug4gb_vector_copy_from": (I, [P, P]),
    "ug4gb_vector_copy_to": (I, [P, P]),
    "ug4gb_vector_norm": (I, [P, PD]),
    "ug4gb_vector_dot": (I, [P, P, PD]),
    "ug4gb_vector_scale_add": (I, [P, D, P, D, P]),
    "ug4gb_vector_destroy": (None, [P]),
    "ug4gb_vector_dot_noalloc": (I, [P, P, I64, P, P, C.c_char_p, I]),
    "ug4gb_matrix_create": (I, [P, PP]),
    "ug4gb_matrix_set_csr": (I, [P, I, I, I64, P, P, P]),
    "ug4gb_matrix_info": (I, [P, PI, PI, PI64]),
    "ug4gb_matrix_export_csr": (I, [P, P, P, P]),
    "ug4gb_matrix_axpy": (I, [P, P, D, P, D, P]),
    "ug4gb_matrix_axpy_transposed": (I, [P, P, D, P, D, P]),
    "ug4gb_matrix_set_as_transpose_of": (I, [P, P, I]),
    "ug4gb_matrix_destroy": (None, [P]),
    "ug4gb_disc_create": (I, [P, P, PP]),
    "ug4gb_disc_set_diffusion_constant": (I, [P, D]),
    "ug4gb_disc_set_diffusion_fourier": (I, [P, I, P, P, D, D]),
    "ug4gb_disc_set_log_diffusion_elements": (I, [P, P]),
    "ug4gb_disc_set_velocity_fourier_curl": (I, [P, I, P, P, P, D]),
    "ug4gb_disc_set_upwind": (I, [P, I]),
    "ug4gb_disc_set_source_vertices": (I, [P, P]),
    "ug4gb_disc_set_source_uniform": (I, [P, C.c_uint64]),
    "ug4gb_disc_assemble_linear": (I, [P, I, P, P]),
    "ug4gb_disc_assemble_jacobian": (I, [P, I, P]),
    "ug4gb_disc_export_coefficients": (I, [P, I, P]),
    "ug4gb_disc_adjoint_operator": (I, [P, I, P, P]),
    "ug4gb_disc_destroy": (None, [P]),
    "ug4gb_gmg_create": (I, [P, P, PP]),
    "ug4gb_gmg_set_smoother": (I, [P, I, D]),
    "ug4gb_gmg_set_presmoother": (I, [P, I, D]),
    "ug4gb_gmg_set_base_solver": (I, [P, I, I]),
    "ug4gb_gmg_set_postsmoother": (I, [P, I, D]),
    "ug4gb_gmg_set_cycle_type": (I, [P, I]),
    "ug4gb_gmg_set_num_presmooth": (I, [P, I]),
    "ug4gb_gmg_set_num_postsmooth": (I, [P, I]),
    "ug4gb_gmg_set_base_level": (I, [P, I]),
    "ug4gb_gmg_set_precision": (I, [P, I]),
    "ug4gb_gmg_set_transposed": (I, [P, I]),
    "ug4gb_gmg_set_rap": (I, [P, I]),
    "ug4gb_gmg_set_prolongation_damping": (I, [P, D]),
    "ug4gb_gmg_set_restriction_damping": (I, [P, D]),
    "ug4gb_gmg_set_time_disc": (I, [P, P]),
    "ug4gb_timedisc_create": (I, [P, P, P]),
    "ug4gb_timedisc_set_theta": (I, [P, D]),
    "ug4gb_timedisc_prepare_step": (I, [P, P, D, D]),
    "ug4gb_timedisc_future_time": (I, [P, P]),
    "ug4gb_timedisc_assemble_linear": (I, [P, I, P, P]),
    "ug4gb_timedisc_assemble_jacobian": (I, [P, I, P]),
    "ug4gb_timedisc_assemble_defect": (I, [P, I, P, P]),
    "ug4gb_timedisc_destroy": (None, [P]),
    "ug4gb_disc_assemble_defect": (I, [P, I, P, P]),
    "ug4gb_disc_adjust_solution": (I, [P, I, P]),
    "ug4gb_newton_create": (I, [P, PP]),
    "ug4gb_newton_set_linear_solver": (I, [P, P]),
    "ug4gb_newton_set_convergence_check": (I, [P, I, D, D]),
    "ug4gb_newton_init": (I, [P, P, P]),
    "ug4gb_newton_prepare": (I, [P, P]),
    "ug4gb_newton_apply": (I, [P, P]),
    "ug4gb_newton_get_stats": (I, [P, PI, PD, PD, P, I]),
    "ug4gb_newton_get_history": (I, [P, P, I]),
    "ug4gb_newton_set_line_search": (I, [P, I, D, D, D, I, I, D]),
    "ug4gb_newton_clear_line_search": (I, [P]),
    "ug4gb_newton_set_reassemble_J_freq": (I, [P, I]),
    "ug4gb_newton_num_jacobian_assemblies": (I, [P]),
    "ug4gb_newton_get_line_search_history": (I, [P, P, P, I]),
    "ug4gb_newton_destroy": (None, [P]),
    "ug4gb_gmg_level_info": (I, [P, I, P, P]),
    "ug4gb_gmg_export_level": (I, [P, I, P, P, P]),
    "ug4gb_gmg_init": (I, [P, P]),
    "ug4gb_gmg_apply": (I, [P, P, P]),
    "ug4gb_gmg_transfer_info": (I, [P, I, I, PI, PI, PI64]),
    "ug4gb_gmg_export_transfer": (I, [P, I, I, P, P, P]),
    "ug4gb_gmg_destroy": (None, [P]),
    "ug4gb_solver_create": (I, [P, I, PP]),
    "ug4gb_solver_set_preconditioner": (I, [P, P]),
    "ug4gb_solver_set_convergence_check": (I, [P, I, D, D]),
    "ug4gb_solver_init": (I, [P, P]),
    "ug4gb_solver_set_restart": (I, [P, I]),
    "ug4gb_perm_create": (I, [P, I, P, C.POINTER(P)]),
    "ug4gb_perm_from_positions": (I, [P, P, I, I, P, D, C.POINTER(P)]),
    "ug4gb_perm_vector": (I, [P, I, P, P]),
    "ug4gb_perm_matrix": (I, [P, I, P, P]),
    "ug4gb_perm_destroy": (None, [P]),
    "ug4gb_solver_set_min_orthogonality": (I, [P, D]),
    "ug4gb_solver_apply_return_defect": (I, [P, P, P]),
    "ug4gb_solver_apply": (I, [P, P, P]),
    "ug4gb_solver_solve_host": (I, [P, P, P]),
    "ug4gb_solver_get_stats": (I, [P, PI, PD, PD, PI]),
    "ug4gb_solver_get_history": (I, [P, P, I]),
    "ug4gb_solver_destroy": (None, [P]),
    "ug4gb_disc_grad_logk": (I, [P, P, P, P]),
    "ug4gb_disc_grad_source": (I, [P, P, P]),
    "ug4gb_matrix_resize_and_clear": (I, [P, I, I]),
    "ug4gb_matrix_clear_retain_structure": (I, [P]),
    "ug4gb_matrix_set_as_copy_of": (I, [P, P, D]),
    "ug4gb_matrix_scale": (I, [P, D]),
    "ug4gb_matrix_apply_ignore_zero_rows": (I, [P, P, D, P]),
    "ug4gb_matrix_get_row": (I, [P, I, P, P, I]),
    "ug4gb_matrix_add_entries": (I, [P, I, P, P, P]),
    "ug4gb_vector_maxnorm": (I, [P, PD]),
    "ug4gb_vector_get_values": (I, [P, I, P, P]),
    "ug4gb_vector_set_values": (I, [P, I, P, P]),
    "ug4gb_io_write_mtx": (I, [I, I, P, P, P, C.c_char_p, C.c_char_p, C.c_char_p, I]),
    "ug4gb_io_read_mtx_info": (I, [C.c_char_p, PI, PI, PI64, C.c_char_p, I]),
    "ug4gb_io_read_mtx": (I, [C.c_char_p, P, P, P, C.c_char_p, I]),
    "ug4gb_io_write_cv_matrix": (I, [I, P, P, P, I, P, C.c_char_p, C.c_char_p, I]),
    "ug4gb_io_write_cv_vector": (I, [I, P, I, P, C.c_char_p, C.c_char_p, I]),
    "ug4gb_io_read_cv_vector": (I, [C.c_char_p, I, P, C.c_char_p, I]),
    "ug4gb_matrix_write_mtx": (I, [P, C.c_char_p, C.c_char_p]),
    "ug4gb_matrix_read_mtx": (I, [P, C.c_char_p]),
    "ug4gb_matrix_write_cv": (I, [P, P, I, C.c_char_p]),
    "ug4gb_vector_write_cv": (I, [P, P, I, C.c_char_p]),
    "ug4gb_vector_read_cv": (I, [P, C.c_char_p]),
}

_lib = None


def exported_symbols():
    """Names the C header declares (for the symbol-export test)."""
    return sorted(_SIGS)


def lib():
    """Load libug4gb.so; raises if it was not built (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libug4gb.so not built: run __graft_entry__.build() or "
                              "python -m ugcore_gb300.build")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc, ctx=None):
    if rc != OK and rc is not None:
        msg = lib().ug4gb_last_error(ctx).decode() if ctx else ""
        raise UG4GBError(rc, msg)
    return rc


def debug_guard_check():
    """(damaged zones, report) of a guarded build (ug4gb_debug_guard_check);
    (None, "") for a normal build"""
    buf = C.create_string_buffer(1 << 16)
    n = lib().ug4gb_debug_guard_check(buf, len(buf))
    if n == ERR_STATE:
        return None, ""
    return n, buf.value.decode()
