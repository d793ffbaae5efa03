"""ctypes binding of the C ABI declared in ``include/ds_gb300.h``.

The library is the in-tree ``libdsgb300.so`` built by ``dachshund_gb300.build``.
There is no CPU fallback: if the library is missing or fails to load, every
entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

LIB_PATH = _build.LIB

DS_OK = 0
DS_ERR_ARG = 1
DS_ERR_CUDA = 2
DS_ERR_NOT_CONVERGED = 3
DS_ERR_NORM_B = 4
DS_ERR_OOM = 5
DS_ERR_NO_DEVICE = 6
DS_ERR_STATE = 7
DS_ERR_TIMEOUT = 8

DS_FORM_SN = 0
DS_FORM_W = 1
DS_EVAL_TABLE = 0
DS_EVAL_EXACT = 1
DS_TABLE_N = 200
DS_INNER_AUTO = 0
DS_INNER_CUDA_CORE = 1
DS_INNER_TENSOR = 2
DS_INNER_STRUCTURED = 3
DS_ITER_AUTO = 0
DS_ITER_GRAPH = 1
DS_BATCH_AUTO = -1
DS_BATCH_CUDA_CORE = 0
DS_BATCH_TENSOR = 1


class KernelParamsC(C.Structure):
    _fields_ = [
        ("var_s", C.c_double),
        ("l_perp", C.c_double),
        ("l_para", C.c_double),
        ("eval", C.c_int),
        ("exact_cutoff", C.c_double),
        ("table", C.POINTER(C.c_double)),
    ]


class PcgParamsC(C.Structure):
    _fields_ = [
        ("max_iter", C.c_int),
        ("step_r", C.c_int),
        ("tol", C.c_double),
        ("verbose", C.c_int),
    ]


class PcgResultC(C.Structure):
    _fields_ = [
        ("success", C.c_int),
        ("num_iters", C.c_int),
        ("norm_b", C.c_double),
        ("final_norm", C.c_double),
        ("n_outer", C.c_int),
        ("n_inner", C.c_int),
        ("seconds", C.c_double),
    ]


class MixedParamsC(C.Structure):
    _fields_ = [
        ("max_iter", C.c_int),
        ("tol", C.c_double),
        ("reliable_delta", C.c_double),
        ("inner_cutoff", C.c_double),
        ("verbose", C.c_int),
    ]


class OperatorInfoC(C.Structure):
    _fields_ = [
        ("n", C.c_int),
        ("n_pad", C.c_int),
        ("tile", C.c_int),
        ("n_tiles", C.c_int),
        ("n_tile_pairs", C.c_longlong),
        ("evaluated_pairs", C.c_longlong),
    ]


class BatchInfoC(C.Structure):
    _fields_ = [
        ("n_chunks", C.c_int),
        ("n_rhs", C.c_int),
        ("n_total", C.c_int),
        ("n_pad", C.c_int),
        ("n_tiles", C.c_int),
        ("inner_tile_pairs", C.c_longlong),
        ("outer_tile_pairs", C.c_longlong),
        ("inner_evaluated", C.c_longlong),
        ("outer_evaluated", C.c_longlong),
        ("variant", C.c_int),
        ("rhs_block", C.c_int),
        ("graph_replays", C.c_int),
    ]


class ProfileC(C.Structure):
    _fields_ = [
        ("pair_launches", C.c_longlong),
        ("pair_ms", C.c_double),
        ("pair_evaluated", C.c_double),
        ("kernel_launches", C.c_longlong),
        ("f64_launches", C.c_longlong),
        ("f64_ms", C.c_double),
        ("f64_evaluated", C.c_double),
        ("f32_launches", C.c_longlong),
        ("f32_ms", C.c_double),
        ("f32_evaluated", C.c_double),
        ("map_launches", C.c_longlong),
        ("map_ms", C.c_double),
        ("map_evaluated", C.c_double),
        ("dense_launches", C.c_longlong),
        ("dense_ms", C.c_double),
        ("dense_entries", C.c_double),
    ]


_vp = C.c_void_p
_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int)
_i = C.c_int
_d = C.c_double

# name -> (restype, argtypes).  Every function declared in include/ds_gb300.h.
SIGNATURES = {
    "ds_status_string": (C.c_char_p, [_i]),
    "ds_table_init": (None, [_dp, _dp]),
    "ds_signal_covar": (_i, [C.POINTER(KernelParamsC), _i, _dp, _dp, _dp]),
    "ds_context_create": (_i, [_i, C.POINTER(_vp)]),
    "ds_context_destroy": (None, [_vp]),
    "ds_context_stream": (_vp, [_vp]),
    "ds_context_synchronize": (_i, [_vp]),
    "ds_context_last_error": (C.c_char_p, [_vp]),
    "ds_context_set_profiling": (_i, [_vp, _i]),
    "ds_context_set_wait_limit": (_i, [_vp, C.c_longlong]),
    "ds_context_get_profile": (_i, [_vp, C.POINTER(ProfileC)]),
    "ds_operator_create": (_i, [_vp, _i, _i, _dp, C.POINTER(KernelParamsC), C.POINTER(_vp)]),
    "ds_operator_destroy": (None, [_vp]),
    "ds_operator_get_info": (_i, [_vp, C.POINTER(OperatorInfoC)]),
    "ds_A_product": (_i, [_vp, _dp, _dp]),
    "ds_A_product_dev": (_i, [_vp, _vp, _vp]),
    "ds_A_residual": (_i, [_vp, _dp, _dp]),
    "ds_A_residual_dev": (_i, [_vp, _vp, _vp]),
    "ds_preconditioner_solve": (_i, [_vp, _dp, _dp]),
    "ds_norm_b": (_i, [_vp, _dp]),
    "ds_A_entries": (_i, [_vp, _i, _i, _ip, _ip, _dp]),
    "ds_operator_set_dense": (_i, [_vp, _i]),
    "ds_operator_set_dense_arith": (_i, [_vp, _i]),
    "ds_operator_get_dense_arith": (_i, [_vp, C.POINTER(C.c_int)]),
    "ds_operator_set_inner_matvec": (_i, [_vp, _i]),
    "ds_operator_set_iteration_form": (_i, [_vp, _i]),
    "ds_operator_get_persistent_profile": (_i, [_vp, C.POINTER(C.c_double), _i, _i,
                                              C.POINTER(C.c_int)]),
    "ds_solve_cf": (_i, [_vp, _i, _i, _dp, C.POINTER(KernelParamsC), _dp]),
    "ds_map_covar_diag": (_i, [_vp, _i, _dp, _i, _dp, C.POINTER(KernelParamsC),
                               C.POINTER(PcgParamsC), _dp, _ip, _ip]),
    "ds_solve_pcg": (_i, [_vp, C.POINTER(PcgParamsC), _dp, C.POINTER(PcgResultC), _dp]),
    "ds_solve_pcg_dev": (_i, [_vp, C.POINTER(PcgParamsC), _vp, C.POINTER(PcgResultC), _dp]),
    "ds_solve_pcg_noalloc": (_i, [_i, _i, _vp, C.POINTER(KernelParamsC), C.POINTER(PcgParamsC),
                                  _vp, C.POINTER(PcgResultC), _dp, _vp]),
    "ds_A_residual_ff": (_i, [_vp, _dp, _dp]),
    "ds_solve_mixed": (_i, [_vp, C.POINTER(MixedParamsC), _dp, C.POINTER(PcgResultC), _dp]),
    "ds_solve_mixed_dev": (_i, [_vp, C.POINTER(MixedParamsC), _vp, C.POINTER(PcgResultC), _dp]),
    "ds_map_product_f32": (_i, [_vp, _vp, _d, _dp, _dp]),
    "ds_map_product_f32_dev": (_i, [_vp, _vp, _d, _vp, _vp]),
    "ds_batch_create": (_i, [_vp, _i, _i, _ip, _dp, C.POINTER(KernelParamsC), _i, _d,
                             C.POINTER(_vp)]),
    "ds_batch_destroy": (None, [_vp]),
    "ds_batch_get_info": (_i, [_vp, C.POINTER(BatchInfoC)]),
    "ds_batch_set_variant": (_i, [_vp, _i, _i]),
    "ds_batch_solve_mixed": (_i, [_vp, C.POINTER(MixedParamsC), _dp, _dp, _ip, _ip, _ip, _dp,
                                  _dp]),
    "ds_batch_solve_mixed_dev": (_i, [_vp, C.POINTER(MixedParamsC), _vp, _vp, _ip, _ip, _ip,
                                      _dp, _dp]),
    "ds_batch_product_f32_dev": (_i, [_vp, _vp, _vp]),
    "ds_learned_create": (_i, [_vp, C.POINTER(KernelParamsC), _i, _i, C.c_uint,
                               C.POINTER(_vp)]),
    "ds_learned_destroy": (None, [_vp]),
    "ds_learned_num_params": (_i, [_vp, C.POINTER(C.c_longlong)]),
    "ds_learned_get_params": (_i, [_vp, _fp]),
    "ds_learned_set_params": (_i, [_vp, _fp]),
    "ds_learned_get_grads": (_i, [_vp, _fp]),
    "ds_learned_save": (_i, [_vp, C.c_char_p]),
    "ds_learned_load": (_i, [_vp, C.c_char_p]),
    "ds_learned_set_inference": (_i, [_vp, _i]),
    "ds_learned_forward_dev": (_i, [_vp, _i, _i, _vp, _vp, _vp]),
    "ds_learned_train_step_dev": (_i, [_vp, _i, _i, _vp, _vp, _vp, C.c_float, C.c_float,
                                       C.c_float, _i, _dp]),
    "ds_operator_set_skewer_preconditioner": (_i, [_vp, _i, _i, _i, _vp]),
    "ds_operator_set_cluster_preconditioner": (_i, [_vp, _i, _i, _i, _i, _vp]),
    "ds_operator_set_skewer_grid": (_i, [_vp, _i, _i]),
    "ds_map_set_column_grid": (_i, [_vp, _i, _i]),
    "ds_operator_skewer_product_dev": (_i, [_vp, _i, _vp, _vp]),
    "ds_map_create": (_i, [_vp, _i, _dp, C.POINTER(_vp)]),
    "ds_map_destroy": (None, [_vp]),
    "ds_map_product": (_i, [_vp, _vp, _dp, _dp]),
    "ds_map_product_dev": (_i, [_vp, _vp, _vp, _vp]),
    "ds_smp_product": (_i, [_vp, _i, _dp, _i, _dp, C.POINTER(KernelParamsC), _dp, _dp]),
    "ds_sigma_m_noise_dom": (_i, [_vp, _i, _dp, _i, _dp, C.POINTER(KernelParamsC), _dp]),
}

_lib = None


def load(build_if_missing: bool = True):
    """Load (building first if needed) the CUDA library; raises on failure."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise RuntimeError(f"dachshund-gb300: {LIB_PATH} is not built")
        _build.build()
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class DsError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def status_string(code: int) -> str:
    return load().ds_status_string(code).decode()
