"""ctypes binding of the C-ABI in ``include/fgpu.h`` (``_lib/libfgpu.so``).

The library is the product: there is no CPU fallback. If the shared library
is missing or cannot be loaded, importing this module raises.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libfgpu.so")

FGPU_OK = 0
F64, F32, DF64 = 0, 1, 2
FORM_LAPLACE_MASS, FORM_ELASTICITY = 0, 1
RANGE_ELEMENTS, RANGE_BOUNDARY_FACES, RANGE_MARKED_FACES = 0, 1, 2
ALGO_AUTO, ALGO_GATHER, ALGO_COLOUR, ALGO_GATHER_NATIVE_F64, ALGO_TWO_PHASE, ALGO_STREAMED = 0, 1, 2, 3, 4, 5
TC_F32, TC_DF64 = 1, 2
HOST_TRANSFER_AUTO, HOST_TRANSFER_COPY, HOST_TRANSFER_DIRECT = 0, 1, 2
RHS_SINE, RHS_CONST_VEC, RHS_CONST, RHS_FACE = 0, 1, 2, 3
ON_ELIMINATION, ON_ELIMINATION_SYMMETRIC, ON_ELIMINATION_KEEP_DIAGONAL = 0, 1, 2
PC_NONE, PC_JACOBI, PC_CHEB_JACOBI, PC_GAMG, PC_PMG = 0, 1, 2, 3, 4
ARITH_F64, ARITH_DF64 = 0, 1

ERROR_NAMES = {1: "FGPU_ERR_INVALID", 2: "FGPU_ERR_CUDA", 3: "FGPU_ERR_BAD_ELEMENT", 4: "FGPU_ERR_OUT_OF_RANGE",
               5: "FGPU_ERR_NOT_CONVERGED", 6: "FGPU_ERR_BREAKDOWN", 7: "FGPU_ERR_PATTERN", 8: "FGPU_ERR_ALLOC"}


class FgpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERROR_NAMES.get(code, "?"), code, msg))
        self.code = code


class Config(C.Structure):
    _fields_ = [("device", C.c_int), ("stream", C.c_void_p), ("profile", C.c_int), ("host_threads", C.c_int),
                ("host_setup", C.c_int), ("tune", C.c_int), ("tune_cache", C.c_char_p)]


class FormDesc(C.Structure):
    _fields_ = [("kind", C.c_int), ("kappa", C.c_double), ("kappa_elem", C.c_void_p), ("mass", C.c_double),
                ("lam", C.c_double), ("mu", C.c_double), ("quad_degree", C.c_int), ("algo", C.c_int),
                ("kappa_scale", C.c_void_p), ("range", C.c_int), ("range_xmax", C.c_double), ("mass_h", C.c_double),
                ("dn_trial", C.c_double), ("dn_test", C.c_double)]


class RhsDesc(C.Structure):
    _fields_ = [("kind", C.c_int), ("c", C.c_double * 3), ("quad_degree", C.c_int), ("range", C.c_int),
                ("range_xmax", C.c_double)]


class SolverCfg(C.Structure):
    _fields_ = [("rtol", C.c_double), ("maxit", C.c_int), ("pc", C.c_int), ("mixed", C.c_int),
                ("inner_rtol", C.c_double), ("check_every", C.c_int), ("arith", C.c_int),
                ("cheb_degree", C.c_int), ("cheb_ratio", C.c_double)]


class AmgCfg(C.Structure):
    _fields_ = [("threshold", C.c_double), ("max_levels", C.c_int), ("coarse_eq_lim", C.c_int), ("agg_smooths", C.c_int),
                ("smoother_degree", C.c_int), ("setup_on_host", C.c_int), ("block_size", C.c_int), ("nns_count", C.c_int),
                ("nns", C.c_void_p), ("nns_host", C.c_void_p)]


class PmgCfg(C.Structure):
    _fields_ = [("smoother_degree", C.c_int), ("coarse_cycles", C.c_int)]


class SolveStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("outer", C.c_int), ("rel_residual", C.c_double), ("time_ms", C.c_double),
                ("eig_max", C.c_double), ("fallback", C.c_int), ("fallback_iterations", C.c_int)]


P = C.c_void_p
PP = C.POINTER(C.c_void_p)
i32, i64, f64 = C.c_int, C.c_int64, C.c_double
I64P = C.POINTER(C.c_int64)
IP = C.POINTER(C.c_int)
DP = C.POINTER(C.c_double)

SIGNATURES = {
    "fgpu_create": (i32, [C.POINTER(Config), PP]),
    "fgpu_destroy": (i32, [P]),
    "fgpu_last_error": (C.c_char_p, [P]),
    "fgpu_sync": (i32, [P]),
    "fgpu_launch_count": (i64, [P]),
    "fgpu_mesh_upload": (i32, [P, i64, P, i64, P, PP]),
    "fgpu_mesh_upload_hex": (i32, [P, i64, P, i64, P, PP]),
    "fgpu_host_hex_dof_table": (i32, [i64, i64, P, i32, P, C.POINTER(i64)]),
    "fgpu_host_hex_ref_tables": (i32, [i32, i32, P, P, P, P, P, C.POINTER(i32)]),
    "fgpu_mesh_cell_vertices": (i32, [P, C.POINTER(i32)]),
    "fgpu_mesh_set_coords": (i32, [P, P]),
    "fgpu_mesh_destroy": (i32, [P]),
    "fgpu_space_create": (i32, [P, P, i32, i32, PP]),
    "fgpu_space_ndof": (i32, [P, I64P, IP]),
    "fgpu_space_l2g": (i32, [P, P]),
    "fgpu_space_boundary_dofs": (i32, [P, i32, f64, I64P, P]),
    "fgpu_space_destroy": (i32, [P]),
    "fgpu_matrix_create": (i32, [P, P, P, i32, PP]),
    "fgpu_matrix_create_like": (i32, [P, i32, PP]),
    "fgpu_matrix_info": (i32, [P, I64P, I64P, IP]),
    "fgpu_matrix_get_csr": (i32, [P, P, P, P]),
    "fgpu_matrix_get_csr32": (i32, [P, P, P, P]),
    "fgpu_matrix_values_device": (i32, [P, PP]),
    "fgpu_matrix_zero": (i32, [P]),
    "fgpu_matrix_convert": (i32, [P, P]),
    "fgpu_matrix_destroy": (i32, [P]),
    "fgpu_assemble_matrix": (i32, [P, P, C.POINTER(FormDesc), i32]),
    "fgpu_assemble_matrix_dev": (i32, [P, P, C.POINTER(FormDesc), P, i32]),
    "fgpu_vector_create": (i32, [P, i64, PP]),
    "fgpu_vector_upload": (i32, [P, P]),
    "fgpu_vector_download": (i32, [P, P]),
    "fgpu_vector_zero": (i32, [P]),
    "fgpu_vector_device": (i32, [P, PP]),
    "fgpu_vector_destroy": (i32, [P]),
    "fgpu_assemble_vector": (i32, [P, P, C.POINTER(RhsDesc), P, i32]),
    "fgpu_dirichlet": (i32, [P, P, P, i64, P, P, i32, f64]),
    "fgpu_matrix_mult": (i32, [P, P, P, P]),
    "fgpu_solve_cg": (i32, [P, P, P, P, P, C.POINTER(SolverCfg), C.POINTER(SolveStats)]),
    "fgpu_solve_cg_refine_dd": (i32, [P, P, P, P, P, P, C.POINTER(SolverCfg), C.c_double, C.POINTER(SolveStats)]),
    "fgpu_amg_create": (i32, [P, P, C.POINTER(AmgCfg), PP]),
    "fgpu_amg_update": (i32, [P]),
    "fgpu_amg_info": (i32, [P, C.POINTER(C.c_int), P, P, DP]),
    "fgpu_amg_setup_info": (i32, [P, C.POINTER(C.c_int), P]),
    "fgpu_amg_destroy": (i32, [P]),
    "fgpu_mesh_set_ho_nodes": (i32, [P, P]),
    "fgpu_assemble_matrix_host": (i32, [P, P, C.POINTER(FormDesc), P]),
    "fgpu_solve_gmres": (i32, [P, P, P, P, P, C.POINTER(SolverCfg), i32, C.POINTER(SolveStats)]),
    "fgpu_set_host_transfer": (i32, [P, i32]),
    "fgpu_set_tensor_cores": (i32, [P, i32]),
    "fgpu_export_ensight": (i32, [P, C.c_char_p, i32, P, P]),
    "fgpu_pmg_create": (i32, [P, P, P, P, C.POINTER(PmgCfg), PP]),
    "fgpu_pmg_info": (i32, [P, DP, P, DP]),
    "fgpu_pmg_destroy": (i32, [P]),
    "fgpu_solve_cg_operator_pmg": (i32, [P, P, P, P, P, P, C.POINTER(SolverCfg), C.POINTER(SolveStats)]),
    "fgpu_solve_cg_amg": (i32, [P, P, P, P, P, C.POINTER(SolverCfg), C.POINTER(SolveStats)]),
    "fgpu_amg_host_build": (i32, [i64, P, P, P, C.POINTER(AmgCfg), i32, PP]),
    "fgpu_amg_host_levels": (i32, [P]),
    "fgpu_amg_host_level": (i32, [P, i32, P, P, P, P, DP]),
    "fgpu_amg_host_export": (i32, [P, i32, P, P, P, P, P, P, P]),
    "fgpu_amg_host_coarse_inverse": (i32, [P, P]),
    "fgpu_amg_host_destroy": (i32, [P]),
    "fgpu_amg_device_build": (i32, [P, P, C.POINTER(AmgCfg), PP]),
    "fgpu_amg_host_device_levels": (i32, [P]),
    "fgpu_space_rigid_body_modes": (i32, [P, P]),
    "fgpu_norms_sine": (i32, [P, P, P, i32, DP, DP]),
    "fgpu_operator_create": (i32, [P, P, C.POINTER(FormDesc), i32, PP]),
    "fgpu_operator_set_dirichlet": (i32, [P, i64, P]),
    "fgpu_operator_apply": (i32, [P, P, P, P]),
    "fgpu_operator_destroy": (i32, [P]),
    "fgpu_operator_set_tensor_cores": (i32, [P, i32]),
    "fgpu_operator_set_algo": (i32, [P, i32]),
    "fgpu_tc_selftest": (i32, [P, P, P, P]),
    "fgpu_solve_cg_operator": (i32, [P, P, P, P, P, C.POINTER(SolverCfg), C.POINTER(SolveStats)]),
    "fgpu_host_dof_table": (i32, [i64, i64, P, i32, i32, P, I64P]),
    "fgpu_host_pattern": (i32, [i64, i64, P, i32, i32, P, P, I64P]),
    "fgpu_host_ref_tables": (i32, [i32, i32, P, P, P, P, P, IP]),
    "fgpu_assemble_vector_noalloc": (i32, [P, C.POINTER(RhsDesc), P, i32, P]),
    "fgpu_host_df64_ops": (i32, [i32, i64, P, P, P]),
    "fgpu_bc_create": (i32, [P, i64, i64, P, P, PP]),
    "fgpu_bc_apply": (i32, [P, P, P, P, i32, f64]),
    "fgpu_bc_destroy": (i32, [P]),
    "fgpu_vector_axpby": (i32, [P, f64, P, f64, P]),
    "fgpu_vector_copy": (i32, [P, P, P]),
    "fgpu_graph_begin": (i32, [P]),
    "fgpu_graph_end": (i32, [P, PP]),
    "fgpu_graph_launch": (i32, [P, P, i32]),
    "fgpu_graph_destroy": (i32, [P]),
    "fgpu_batch_create": (i32, [P, i32, P, P, P, PP]),
    "fgpu_batch_assemble": (i32, [P, P, i32]),
    "fgpu_batch_set_launch": (i32, [P, i32, i32]),
    "fgpu_batch_get_launch": (i32, [P, IP, IP, IP]),
    "fgpu_batch_set_algo": (i32, [P, i32]),
    "fgpu_batch_destroy": (i32, [P]),
    "fgpu_prof_reset": (i32, [P]),
    "fgpu_prof_get": (i32, [P, C.c_char_p, I64P, DP]),
}

_lib = None


def load(path=None):
    """Load the compiled library (raises OSError when it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise OSError("feelpp_gb300: CUDA library %s is missing; run __graft_entry__.build()" % path)
    L = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(rc, ctx=None):
    if rc != FGPU_OK:
        msg = load().fgpu_last_error(ctx).decode() if ctx else ""
        raise FgpuError(rc, msg)
