"""ctypes binding of libchefsi_gb300.so (the C ABI declared in include/chefsi.h).

Loading fails loudly: there is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libchefsi_gb300.so")

CHEFSI_OK = 0
CHEFSI_ERR_INVALID = 1
CHEFSI_ERR_CUDA = 2
CHEFSI_ERR_NOT_SPD = 3
CHEFSI_ERR_NO_CONVERGENCE = 4
CHEFSI_ERR_ALLOC = 5
CHEFSI_ERR_TIMEOUT = 6
CHEFSI_ERR_NAN = 7
CHEFSI_ERR_UNSUPPORTED = 8

PREC_FP64, PREC_MIXED, PREC_FP32, PREC_FP32_TC = 0, 1, 2, 3
PRECISIONS = {"fp64": PREC_FP64, "mixed": PREC_MIXED, "fp32": PREC_FP32, "fp32tc": PREC_FP32_TC}

_ERRNAMES = {1: "INVALID", 2: "CUDA", 3: "NOT_SPD", 4: "NO_CONVERGENCE", 5: "ALLOC",
             6: "TIMEOUT", 7: "NAN", 8: "UNSUPPORTED"}

# every symbol include/chefsi.h declares
EXPORTS = [
    "chefsi_last_error", "chefsi_version", "chefsi_launch_count", "chefsi_operator_create", "chefsi_operator_destroy",
    "chefsi_operator_info", "chefsi_hx", "chefsi_overlap", "chefsi_xthx",
    "chefsi_chebyshev_filter", "chefsi_lanczos_bounds", "chefsi_syevd", "chefsi_heevd", "chefsi_syevd_noalloc",
    "chefsi_cholesky_gs",
    "chefsi_rayleigh_ritz", "chefsi_rayleigh_ritz_spectrum_split",
    "chefsi_density_matrix_first_order_response", "chefsi_residual_norms",
    "chefsi_solver_create",
    "chefsi_solver_destroy", "chefsi_solver_reinit_spectrum_bounds", "chefsi_solver_get_bounds",
    "chefsi_solver_timings", "chefsi_solver_set_profiling", "chefsi_solver_hx_stats",
    "chefsi_solve", "chefsi_solve_spectrum_split", "chefsi_solve_batched", "chefsi_solve_no_rr", "chefsi_chebyshev_order", "chefsi_gemm",
    "chefsi_axpby", "chefsi_convert_block", "chefsi_density", "chefsi_assemble_cell_hamiltonians",
    "chefsi_assemble_cell_hamiltonians_bloch", "chefsi_assemble_cell_hamiltonians_gga",
    "chefsi_assemble_cell_hamiltonians_bloch_gga", "chefsi_assemble_cell_hamiltonians_geometry",
    "chefsi_operator_update_cell_matrices",
    "chefsi_cell_outer_accumulate", "chefsi_cell_quadrature_contract", "chefsi_set_wait_limits",
]
DEFAULT_WAIT_TRIES = 65536
DEFAULT_BARRIER_SPINS = 1 << 26


class ChefsiError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"CHEFSI_ERR_{_ERRNAMES.get(code, code)}: {msg}")
        self.code = code


class OperatorDesc(ctypes.Structure):
    _fields_ = [
        ("n_dofs", ctypes.c_int64), ("n_cells", ctypes.c_int32),
        ("nodes_per_cell", ctypes.c_int32), ("is_complex", ctypes.c_int32),
        ("cell_dof_map", ctypes.c_void_p), ("cell_matrices", ctypes.c_void_p),
        ("sqrt_mass", ctypes.c_void_p), ("inv_sqrt_mass", ctypes.c_void_p),
        ("n_constrained", ctypes.c_int32), ("constrained_ids", ctypes.c_void_p),
        ("constraint_ptr", ctypes.c_void_p), ("master_ids", ctypes.c_void_p),
        ("master_weights", ctypes.c_void_p),
        ("n_atoms", ctypes.c_int32), ("n_proj", ctypes.c_int32),
        ("atom_dof_ptr", ctypes.c_void_p), ("atom_dofs", ctypes.c_void_p),
        ("atom_proj", ctypes.c_void_p), ("couplings", ctypes.c_void_p),
    ]


class Params(ctypes.Structure):
    _fields_ = [
        ("chebyshev_degree", ctypes.c_int32), ("cheby_wfc_block", ctypes.c_int32),
        ("wfc_block", ctypes.c_int32), ("precision", ctypes.c_int32),
        ("lanczos_steps", ctypes.c_int32), ("reproducible", ctypes.c_int32),
        ("first_scf_degree_scale", ctypes.c_double), ("keep_hx", ctypes.c_int32),
        ("rr_precision", ctypes.c_int32), ("ss_frac_reduced", ctypes.c_int32),
        ("rr_block", ctypes.c_int32), ("rr_slab_rows", ctypes.c_int32),
        ("filter_variant", ctypes.c_int32),
    ]


_lib = None


def load(path: str | None = None) -> ctypes.CDLL:
    """Load the CUDA library; raises if it is missing (build with dftfe_gb300.build.build())."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"libchefsi_gb300.so not found at {p}: run "
                           "`python -c 'import __graft_entry__ as g; g.build()'` first "
                           "(the CheFSI path has no CPU fallback)")
    lib = ctypes.CDLL(p)
    vp, i32, i64, f64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_double
    sig = {
        "chefsi_last_error": ([], ctypes.c_char_p),
        "chefsi_version": ([], ctypes.c_char_p),
        "chefsi_launch_count": ([], ctypes.c_uint64),
        "chefsi_operator_create": ([ctypes.POINTER(OperatorDesc), ctypes.POINTER(vp)], ctypes.c_int),
        "chefsi_operator_destroy": ([vp], ctypes.c_int),
        "chefsi_operator_info": ([vp, vp, vp, vp, vp], ctypes.c_int),
        "chefsi_hx": ([vp, vp, i64, vp, i64, i32, f64, i32, i32, vp], ctypes.c_int),
        "chefsi_overlap": ([vp, vp, i64, i32, vp, i32, vp], ctypes.c_int),
        "chefsi_xthx": ([vp, vp, i64, i32, vp, i32, vp], ctypes.c_int),
        "chefsi_chebyshev_filter": ([vp, vp, i64, i32, i32, f64, f64, f64, i32, vp], ctypes.c_int),
        "chefsi_lanczos_bounds": ([vp, i32, i32, vp, ctypes.c_uint64, vp, vp, vp], ctypes.c_int),
        "chefsi_syevd": ([i32, vp, vp, vp, vp], ctypes.c_int),
        "chefsi_heevd": ([i32, vp, vp, vp, vp], ctypes.c_int),
        "chefsi_syevd_noalloc": ([i32, vp, vp, vp, vp], ctypes.c_int),
        "chefsi_cholesky_gs": ([vp, vp, i64, i32, i32, vp], ctypes.c_int),
        "chefsi_rayleigh_ritz": ([vp, vp, i64, i32, vp, vp, vp, i32, vp], ctypes.c_int),
        "chefsi_rayleigh_ritz_spectrum_split": ([vp, vp, i64, i32, i32, vp, i64, vp, vp, i32, i32,
                                                 vp], ctypes.c_int),
        "chefsi_gemm": ([ctypes.c_char, ctypes.c_char, i64, i32, i32, f64, vp, i64, vp, i64, f64,
                         vp, i64, i32, vp], ctypes.c_int),
        "chefsi_axpby": ([i64, i32, f64, vp, i64, f64, vp, i64, vp], ctypes.c_int),
        "chefsi_convert_block": ([i32, vp, i64, i32, vp, i64, i64, i32, f64, vp], ctypes.c_int),
        "chefsi_density": ([vp, vp, i64, i32, vp, i32, vp, vp, vp, i32, i32, vp], ctypes.c_int),
        "chefsi_assemble_cell_hamiltonians": ([i32, i32, i32, vp, vp, vp, vp, vp], ctypes.c_int),
        "chefsi_assemble_cell_hamiltonians_gga": ([i32, i32, i32, vp, vp, vp, vp, vp, vp, vp],
                                                  ctypes.c_int),
        "chefsi_assemble_cell_hamiltonians_geometry": ([i32, i32, i32, vp, vp, vp, vp, vp, vp],
                                                       ctypes.c_int),
        "chefsi_assemble_cell_hamiltonians_bloch_gga": ([i32, i32, i32, vp, vp, vp, vp, vp, vp, i32,
                                                         vp, vp, vp], ctypes.c_int),
        "chefsi_assemble_cell_hamiltonians_bloch": ([i32, i32, i32, vp, vp, vp, vp, vp, i32, vp, vp,
                                                     vp], ctypes.c_int),
        "chefsi_operator_update_cell_matrices": ([vp, vp, vp], ctypes.c_int),
        "chefsi_cell_outer_accumulate": ([vp, vp, vp, i64, i32, f64, vp, vp], ctypes.c_int),
        "chefsi_cell_quadrature_contract": ([i32, i32, i32, vp, vp, vp, vp, vp], ctypes.c_int),
        "chefsi_residual_norms": ([vp, vp, i64, i32, vp, vp, vp], ctypes.c_int),
        "chefsi_solver_create": ([ctypes.POINTER(Params), ctypes.POINTER(vp)], ctypes.c_int),
        "chefsi_solver_destroy": ([vp], ctypes.c_int),
        "chefsi_solver_reinit_spectrum_bounds": ([vp, f64, f64, f64], ctypes.c_int),
        "chefsi_solver_get_bounds": ([vp, vp, vp, vp, vp], ctypes.c_int),
        "chefsi_solver_timings": ([vp, vp], ctypes.c_int),
        "chefsi_solver_set_profiling": ([vp, i32], ctypes.c_int),
        "chefsi_solver_hx_stats": ([vp, vp, vp], ctypes.c_int),
        "chefsi_density_matrix_first_order_response": ([vp, vp, i64, i32, vp, f64, f64, vp, i32,
                                                        vp], ctypes.c_int),
        "chefsi_solve": ([vp, vp, vp, i32, vp, vp, i32, i32, vp], ctypes.c_int),
        "chefsi_solve_spectrum_split": ([vp, vp, vp, i32, i32, vp, vp, vp, i32, i32, vp],
                                        ctypes.c_int),
        "chefsi_solve_batched": ([i32, vp, vp, vp, vp, vp, vp, i32, i32, i32, i32], ctypes.c_int),
        "chefsi_solve_no_rr": ([vp, vp, vp, i32, i32, i32, vp], ctypes.c_int),
        "chefsi_chebyshev_order": ([f64], i32),
        "chefsi_set_wait_limits": ([ctypes.c_uint32, ctypes.c_uint32], ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def check(rc: int) -> None:
    if rc != CHEFSI_OK:
        msg = load().chefsi_last_error()
        raise ChefsiError(rc, msg.decode() if msg else "")
