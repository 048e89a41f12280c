"""ctypes binding of libasgkron.so (the C ABI declared in include/asgkron.h).

The library must have been built (``asgkron._build.build()`` or ``__graft_entry__.build()``);
loading fails loudly otherwise -- there is no CPU fallback for any entry point.
"""
import ctypes as C
import os

from . import _build

ASG_OK = 0
ASG_ERR_INVALID = 1
ASG_ERR_UNSUPPORTED = 2
ASG_ERR_CUDA = 3
ASG_ERR_NOMEM = 4
ASG_ERR_TIMEOUT = 5
ASG_ERR_CAPACITY = 6
_NAMES = {1: "ASG_ERR_INVALID", 2: "ASG_ERR_UNSUPPORTED", 3: "ASG_ERR_CUDA", 4: "ASG_ERR_NOMEM",
          5: "ASG_ERR_TIMEOUT", 6: "ASG_ERR_CAPACITY"}

ASG_STRUCT_NONE = 0
ASG_STRUCT_DETECT = 1
ASG_GRID_SG = 0
ASG_GRID_FG = 1
KERNEL_CHAIN_WARP, KERNEL_CHAIN_CTA, KERNEL_SINGLE_MODE, KERNEL_SINGLE_TMA, KERNEL_SINGLE_TMA3 = 0, 1, 2, 3, 4
KERNEL_SINGLE_TMA_ROWS, KERNEL_SINGLE_SMALL, KERNEL_STREAM, KERNEL_SINGLE_TMA_X2 = 5, 6, 7, 8
KERNEL_NAMES = ["warp_chain", "cta_chain", "single_mode", "single_mode_tma", "single_mode_tma_3cta", "single_mode_tma_rows",
                "single_mode_small", "stream", "single_mode_tma_x2"]


class AsgError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (_NAMES.get(status, status), msg))
        self.status = status


class PlanDesc(C.Structure):
    _fields_ = [
        ("num_dims", C.c_int),
        ("deg", C.c_int),
        ("num_terms", C.c_int),
        ("num_elems", C.c_int),
        ("index_base", C.c_int),
        ("idx1d", C.POINTER(C.c_int)),
        ("row_ptr", C.POINTER(C.c_longlong)),
        ("cols", C.POINTER(C.c_int)),
        ("ops", C.POINTER(C.POINTER(C.c_double))),
        ("op_ld", C.POINTER(C.c_int)),
        ("structure", C.c_int),
        ("drop_tol", C.c_double),
    ]


class PlanExt(C.Structure):
    _fields_ = [("row_begin", C.c_int), ("row_end", C.c_int), ("op_blocks", C.POINTER(C.c_int))]


class PartialTermDesc(C.Structure):
    _fields_ = [
        ("kind", C.c_int),
        ("LF", C.c_double),
        ("bcl", C.c_char),
        ("bcr", C.c_char),
        ("g_quad", C.POINTER(C.c_double)),
        ("g_face", C.POINTER(C.c_double)),
    ]


class PlanStats(C.Structure):
    _fields_ = [
        ("num_pairs", C.c_longlong),
        ("num_entries", C.c_longlong),
        ("dof", C.c_longlong),
        ("flops_reference", C.c_double),
        ("flops_executed", C.c_double),
        ("op_bytes_f64", C.c_longlong),
        ("kernel_kind", C.c_int),
        ("active_modes_max", C.c_int),
    ]


class GemmDesc(C.Structure):
    _fields_ = [
        ("level", C.c_int), ("m", C.c_int), ("n", C.c_int), ("k", C.c_int),
        ("trans_a", C.c_char), ("trans_b", C.c_char), ("alpha", C.c_double), ("beta", C.c_double),
        ("a_operand", C.c_int), ("b_operand", C.c_int), ("c_operand", C.c_int),
        ("a_offset", C.c_longlong), ("b_offset", C.c_longlong), ("c_offset", C.c_longlong),
        ("lda", C.c_int), ("ldb", C.c_int), ("ldc", C.c_int),
    ]


class GmresOpts(C.Structure):
    _fields_ = [("restart", C.c_int), ("max_outer", C.c_int), ("tol", C.c_double), ("inner_reduction", C.c_double),
                ("mixed", C.c_int)]


class GmresInfo(C.Structure):
    _fields_ = [("outer_iters", C.c_int), ("inner_iters", C.c_int), ("converged", C.c_int),
                ("rel_residual", C.c_double)]


_P = C.c_void_p
_I = C.POINTER(C.c_int)
_D = C.POINTER(C.c_double)

# name -> (restype, argtypes); every symbol include/asgkron.h declares
SIGNATURES = {
    "asg_version": (C.c_char_p, []),
    "asg_last_error": (C.c_int, [C.c_char_p, C.c_size_t]),
    "asg_plan_create": (C.c_int, [C.POINTER(PlanDesc), C.POINTER(C.c_void_p)]),
    "asg_plan_destroy": (C.c_int, [C.c_void_p]),
    "asg_plan_stats_get": (C.c_int, [C.c_void_p, C.POINTER(PlanStats)]),
    "asg_plan_update_ops": (C.c_int, [C.c_void_p, C.POINTER(C.POINTER(C.c_double)), C.POINTER(C.c_int)]),
    "asg_plan_create_ex": (C.c_int, [C.POINTER(PlanDesc), C.POINTER(PlanExt), C.POINTER(C.c_void_p)]),
    "asg_plan_halo": (C.c_int, [C.c_void_p, _I, C.c_longlong, C.POINTER(C.c_longlong)]),
    "asg_plan_row_entries": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong)]),
    "asg_plan_update_elements": (C.c_int, [C.c_void_p, C.c_int, _I, C.POINTER(C.c_longlong), _I]),
    "asg_plan_set_kernel": (C.c_int, [C.c_void_p, C.c_int]),
    "asg_plan_tune": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_float),
                                C.POINTER(C.c_float)]),
    "asg_plan_kernel_for": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int)]),
    "asg_probe_gather_f32": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    "asg_probe_fma": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_void_p, C.POINTER(C.c_double), C.c_void_p]),
    "asg_plan_active": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint)]),
    "asg_plan_device_status": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "asg_apply_f64": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "asg_apply_f32": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "asg_apply_residual_f64": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "asg_apply_residual_f32": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "asg_apply_T_f64": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "asg_apply_T_f32": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "asg_grad_ops_f64": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_int),
                                   C.c_void_p]),
    "asg_grad_ops_f32": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_int),
                                   C.c_void_p]),
    "asg_apply_host_f64": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "asg_apply_host_f32": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "asg_apply_T_host_f64": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "asg_assemble_bsr_f64": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong), C.POINTER(C.c_int), C.c_void_p,
                                       C.c_longlong, C.POINTER(C.c_longlong), C.c_void_p]),
    "asg_grad_ops_host_f64": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p),
                                        C.POINTER(C.c_int)]),
    "asg_hash_table_sparse_nd": (C.c_int, [C.c_int, C.POINTER(C.c_int), C.c_int, C.c_int, C.POINTER(C.c_int),
                                           C.POINTER(C.c_int), C.POINTER(C.c_ulonglong), C.c_longlong,
                                           C.POINTER(C.c_longlong)]),
    "asg_hash_table_nd": (C.c_int, [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_longlong,
                                    C.POINTER(C.c_longlong)]),
    "asg_element_idx1d": (C.c_int, [C.c_int, C.c_longlong, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                    C.POINTER(C.c_int)]),
    "asg_connect_nd": (C.c_int, [C.c_int, C.c_longlong, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int, C.c_int,
                                 C.c_int, C.POINTER(C.c_longlong), C.POINTER(C.c_int), C.c_longlong,
                                 C.POINTER(C.c_longlong)]),
    "asg_gemm_vbatched_f64": (C.c_int, [C.c_char, C.c_char, _P, _P, _P, C.c_double, _P, _P, _P, _P, C.c_double, _P, _P,
                                        C.c_int, _P]),
    "asg_gemm_vbatched_f32": (C.c_int, [C.c_char, C.c_char, _P, _P, _P, C.c_float, _P, _P, _P, _P, C.c_float, _P, _P,
                                        C.c_int, _P]),
    "asg_kron_plan_create": (C.c_int, [C.c_int, _I, _I, C.c_longlong, C.POINTER(C.c_void_p)]),
    "asg_kron_plan_destroy": (C.c_int, [C.c_void_p]),
    "asg_kron_plan_workspace": (C.c_int, [C.c_void_p, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
    "asg_kron_plan_lists": (C.c_int, [C.c_void_p, C.POINTER(GemmDesc), C.c_int, _I]),
    "asg_kron_batch_f64": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), _P, _P, _P, C.c_size_t, _P]),
    "asg_kron_batch_f32": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), _P, _P, _P, C.c_size_t, _P]),
    "asg_kron_batch_static_f64": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), _P, _P, _P]),
    "asg_krond_f64": (C.c_int, [C.c_int, _I, _I, C.POINTER(C.c_void_p), _P, _P]),
    "asg_batch_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.POINTER(C.c_void_p)]),
    "asg_batch_destroy": (C.c_int, [C.c_void_p]),
    "asg_batch_set_io_f64": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
    "asg_batch_set_io_f32": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
    "asg_batch_prepare": (C.c_int, [C.c_void_p, C.c_int]),
    "asg_batch_apply": (C.c_int, [C.c_void_p, C.c_int, _P]),
    "asg_batch_tune": (C.c_int, [C.c_void_p, C.c_int, _P, C.POINTER(C.c_float)]),
    "asg_batch_configure": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "asg_batch_info": (C.c_int, [C.c_void_p, _I, _I, C.POINTER(C.c_double)]),
    "asg_rk3_step_f64": (C.c_int, [C.c_void_p, _P, C.c_double, C.POINTER(C.c_void_p), _P, C.c_size_t, _P]),
    "asg_rk3_step_f32": (C.c_int, [C.c_void_p, _P, C.c_double, C.POINTER(C.c_void_p), _P, C.c_size_t, _P]),
    "asg_rk3_step_sources_f64": (C.c_int, [C.c_void_p, _P, C.c_double, C.c_int, _P, _P, _P, C.c_size_t, _P]),
    "asg_rk3_step_sources_f32": (C.c_int, [C.c_void_p, _P, C.c_double, C.c_int, _P, _P, _P, C.c_size_t, _P]),
    "asg_lincomb_f64": (C.c_int, [C.c_longlong, C.c_int, _P, _P, _P, _P]),
    "asg_be_workspace": (C.c_int, [C.c_void_p, C.POINTER(GmresOpts), C.POINTER(C.c_size_t)]),
    "asg_be_solve": (C.c_int, [C.c_void_p, C.c_double, _P, _P, C.POINTER(GmresOpts), C.POINTER(GmresInfo), _P,
                               C.c_size_t, _P]),
    "asg_debug_withhold_arrival": (C.c_int, [C.c_int]),
    "asg_gauss_legendre_f64": (C.c_int, [C.c_int, C.c_double, C.c_double, _D, _D]),
    "asg_multiwavelet_filters_f64": (C.c_int, [C.c_int, _D, _D]),
    "asg_fmwt_matrix_f64": (C.c_int, [C.c_int, C.c_int, _D]),
    "asg_coeff_matrix_f64": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_int,
                                       C.POINTER(PartialTermDesc), _D]),
}

_LIB = None


def lib():
    """The loaded library (built on first use if the sources are newer)."""
    global _LIB
    if _LIB is None:
        path = _build.LIB_PATH
        if not os.path.exists(path):
            _build.build()
        if not os.path.exists(path):
            raise ImportError("libasgkron.so is missing; run __graft_entry__.build()")
        L = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def last_error():
    buf = C.create_string_buffer(1024)
    lib().asg_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def check(status):
    if status != ASG_OK:
        raise AsgError(status, last_error())
    return status
