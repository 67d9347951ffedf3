"""ctypes binding of libqtt_gb300.so (include/qtt_gb300.h).

The library is built in-tree by ``quantit_gb300.build``.  Loading fails loudly
when it is missing: there is no CPU fallback for any operation.
"""
import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libqtt_gb300.so")

QTT_OK = 0
ERRORS = {
    1: ValueError,      # std::invalid_argument
    2: IndexError,      # std::out_of_range
    3: ValueError,      # std::domain_error
    4: RuntimeError,    # std::logic_error
    5: RuntimeError,    # std::runtime_error
    6: RuntimeError,    # CUDA failure
    7: MemoryError,     # device allocation failure
    8: RuntimeError,    # c10::Error (TORCH_CHECK)
    9: RuntimeError,    # structure-only btensor in a numeric call
}

i32, i64, f64, vp = C.c_int32, C.c_int64, C.c_double, C.c_void_p
P = C.POINTER
bt = C.c_void_p

# name: (restype, argtypes)
SIGNATURES = {
    "qtt_last_error": (C.c_char_p, []),
    "qtt_version": (C.c_char_p, []),
    "qtt_init": (C.c_int, [C.c_int]),
    "qtt_set_stream": (C.c_int, [vp]),
    "qtt_get_stream": (vp, []),
    "qtt_synchronize": (C.c_int, []),
    "qtt_set_gemm_mode": (C.c_int, [C.c_int]),
    "qtt_set_jacobi_kernel": (C.c_int, [C.c_int]),
    "qtt_set_autotune": (C.c_int, [C.c_int]),
    "qtt_set_svd_deflation": (C.c_int, [C.c_int]),
    "qtt_set_planner": (C.c_int, [C.c_int, i64]),
    "qtt_planner_stats": (C.c_int, [P(i64), P(C.c_double), C.c_int]),
    "qtt_set_persistent_gemm": (C.c_int, [C.c_int]),
    "qtt_autotune_report": (C.c_int, [C.c_char_p, i64, P(i64)]),
    "qtt_device_memory": (C.c_int, [P(i64), P(i64)]),
    "qtt_get_gemm_mode": (C.c_int, []),
    "qtt_bt_create": (C.c_int, [i32, P(i64), P(i64), i32, P(C.c_uint16), P(C.c_int16), P(C.c_int16), i32, P(bt)]),
    "qtt_bt_set_blocks": (C.c_int, [bt, i64, P(i64), vp]),
    "qtt_bt_set_blocks_device": (C.c_int, [bt, i64, P(i64), vp]),
    "qtt_bt_set_block_structure": (C.c_int, [bt, i64, P(i64)]),
    "qtt_bt_destroy": (C.c_int, [bt]),
    "qtt_bt_clone": (C.c_int, [bt, P(bt)]),
    "qtt_bt_meta": (C.c_int, [bt, P(i32), P(i64), P(i32), P(i64), P(i64), P(i32), P(i32)]),
    "qtt_bt_structure": (C.c_int, [bt, P(i64), P(i64), P(C.c_int16), P(C.c_int16), P(C.c_uint16)]),
    "qtt_bt_blocks": (C.c_int, [bt, P(i64), P(i64)]),
    "qtt_bt_download": (C.c_int, [bt, vp, i64]),
    "qtt_bt_check": (C.c_int, [bt, C.c_char_p, i64]),
    "qtt_permute": (C.c_int, [bt, P(i64), P(bt)]),
    "qtt_reshape": (C.c_int, [bt, i32, P(i64), P(bt)]),
    "qtt_reshape_as": (C.c_int, [bt, bt, P(bt)]),
    "qtt_conj": (C.c_int, [bt, P(bt)]),
    "qtt_inverse_cvals": (C.c_int, [bt, P(bt)]),
    "qtt_tensordot": (C.c_int, [bt, bt, i32, P(i64), P(i64), P(bt)]),
    "qtt_tensorgdot": (C.c_int, [bt, bt, bt, i32, P(i64), P(i64), f64, f64, P(bt)]),
    "qtt_tensorgdot_": (C.c_int, [bt, bt, bt, i32, P(i64), P(i64), f64, f64]),
    "qtt_add": (C.c_int, [bt, bt, f64, P(bt)]),
    "qtt_mul_scalar": (C.c_int, [bt, f64, P(bt)]),
    "qtt_dot_all": (C.c_int, [bt, bt, P(f64)]),
    "qtt_mul_lastleg": (C.c_int, [bt, bt, P(bt)]),
    "qtt_svd": (C.c_int, [bt, P(bt), P(bt), P(bt)]),
    "qtt_svd_split": (C.c_int, [bt, i64, P(bt), P(bt), P(bt)]),
    "qtt_svd_truncate": (C.c_int, [bt, i64, f64, i64, i64, f64, P(bt), P(bt), P(bt)]),
    "qtt_truncate": (C.c_int, [bt, bt, bt, i64, i64, f64, f64, P(bt), P(bt), P(bt)]),
    "qtt_eigh": (C.c_int, [bt, i32, P(bt), P(bt)]),
    "qtt_eigh_split": (C.c_int, [bt, i64, P(bt), P(bt)]),
    "qtt_dmrg_options_default": (None, [vp]),
    "qtt_compute_2sites_hamil": (C.c_int, [bt, bt, P(bt)]),
    "qtt_hamil2site_times_state": (C.c_int, [bt, bt, bt, bt, P(bt)]),
    "qtt_one_step_lanczos": (C.c_int, [bt, bt, bt, bt, P(bt), P(f64), P(f64), P(f64)]),
    "qtt_eig2x2": (C.c_int, [f64, f64, f64, P(f64), P(f64), P(f64)]),
    "qtt_compute_left_env": (C.c_int, [bt, bt, bt, P(bt)]),
    "qtt_compute_right_env": (C.c_int, [bt, bt, bt, P(bt)]),
    "qtt_dmrg": (C.c_int, [i32, P(bt), P(bt), P(i64), vp, vp, vp, P(f64)]),
    "qtt_mps_energy": (C.c_int, [i32, P(bt), P(bt), P(f64), P(f64)]),
    "qtt_stats_enable": (C.c_int, [C.c_int]),
    "qtt_stats_reset": (C.c_int, []),
    "qtt_stats_get": (C.c_int, [C.c_int, P(f64), P(f64), P(i64)]),
    "qtt_launch_count": (i64, []),
    "qtt_last_svd_sweeps": (C.c_int, [P(i32), i32, P(i32)]),
    "qtt_last_svd_fp32_sweeps": (C.c_int, [P(i32), i32, P(i32)]),
    "qtt_svd_dense_noalloc": (C.c_int, [vp, i64, i64, vp, vp, vp, vp]),
    "qtt_dmrg_logged": (C.c_int, [i32, P(vp), P(vp), P(i64), vp, vp, P(f64)]),
    "qtt_trivial_edge": (C.c_int, [vp, i32, vp, i32, P(vp)]),
    "qtt_random_mps": (C.c_int, [i32, P(vp), i64, P(C.c_int16), C.c_uint64, P(vp)]),
}


class DmrgOptionsC(C.Structure):
    _fields_ = [("cutoff", f64), ("convergence_criterion", f64), ("maximum_bond", i64), ("minimum_bond", i64),
                ("maximum_iterations", i64), ("gemm_mode", i32), ("final_energy_fp64", i32),
                ("lanczos_steps", i32), ("cuda_graphs", i32), ("svd_warm_start", i32), ("pad", i32)]


LOG_FN = C.CFUNCTYPE(None, vp, i64, f64, f64)
LOG_INIT = C.CFUNCTYPE(None, vp, vp)
LOG_IT = C.CFUNCTYPE(None, vp, i64, f64, f64, f64, i32, P(vp), i64)
LOG_END = C.CFUNCTYPE(None, vp, i64, f64, i32, P(vp), i64)


class DmrgLoggerC(C.Structure):
    _fields_ = [("user", vp), ("init", LOG_INIT), ("it_log_all", LOG_IT), ("end_log_all", LOG_END)]

_lib = None


def lib():
    """The loaded library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with `python -m quantit_gb300.build`")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status):
    if status != QTT_OK:
        msg = lib().qtt_last_error().decode(errors="replace")
        raise ERRORS.get(status, RuntimeError)(msg)


def call(name, *args):
    check(getattr(lib(), name)(*args))


def i64_array(values):
    values = [int(v) for v in values]
    return (i64 * max(len(values), 1))(*values)


_initialised = False


def ensure_init(device=0):
    global _initialised
    if not _initialised:
        call("qtt_init", device)
        _initialised = True
