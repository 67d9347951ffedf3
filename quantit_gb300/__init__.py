"""quantit_gb300: QuantiT's block-sparse tensor hot path on GB300 (sm_103a).

The package mirrors the Python API of QuantiT (module ``quantit``) for the
accelerated path -- ``btensor`` contraction, sector SVD / eigh with truncation,
and two-site DMRG -- over the C-ABI of libqtt_gb300.so (include/qtt_gb300.h).
All arithmetic runs in CUDA kernels; nothing falls back to the CPU.
"""
from . import algorithms, conserved, linalg, networks
from ._lib import LIB_PATH, ensure_init, lib
from .tensor import btensor, dot_all, from_blocks, tensordot, tensorgdot, tensorgdot_

__all__ = ["algorithms", "conserved", "linalg", "networks", "btensor", "dot_all", "from_blocks", "tensordot",
           "tensorgdot", "tensorgdot_", "LIB_PATH", "ensure_init", "lib", "stats", "set_gemm_mode"]


def set_gemm_mode(mode):
    """Block-GEMM precision: 'f64' (drop-in), 'tf32x3' or 'bf16x3'."""
    from ._lib import call
    call("qtt_set_gemm_mode", algorithms.GEMM_MODES[mode] if isinstance(mode, str) else int(mode))


def set_autotune(on):
    """Turn the sector-SVD block-width autotuner on (default) or off."""
    from ._lib import call
    call("qtt_set_autotune", 1 if on else 0)


def set_svd_deflation(on):
    """Under a truncating svd, numerically null columns (norm at the sweeps' FP32 / FP64
    resolution) leave the sector-SVD sweeps (on by default)."""
    from ._lib import call
    call("qtt_set_svd_deflation", 1 if on else 0)


def set_planner(mode="host", auto_blocks=3000):
    """Block-sparsity planner of tensordot: "host" (the default), "device" (wherever the
    device planner's limits allow) or "auto" (device for contractions of at least
    ``auto_blocks`` blocks in both operands together)."""
    from ._lib import call
    modes = {"host": 0, "device": 1, "auto": 2}
    if mode not in modes:
        raise ValueError(f"planner mode must be one of {sorted(modes)}")
    call("qtt_set_planner", modes[mode], int(auto_blocks))


def planner_stats(reset=False):
    """{"host_calls", "device_calls", "device_fallbacks", "host_s", "device_s"}: planner
    calls and the host wall seconds spent planning on each path."""
    import ctypes as C
    from ._lib import call
    calls = (C.c_int64 * 3)()
    secs = (C.c_double * 2)()
    call("qtt_planner_stats", calls, secs, 1 if reset else 0)
    return {"host_calls": calls[0], "device_calls": calls[1], "device_fallbacks": calls[2], "host_s": secs[0],
            "device_s": secs[1]}


def set_persistent_gemm(on):
    """Persistent split-TF32 GEMM for launches of many tiles (on by default)."""
    from ._lib import call
    call("qtt_set_persistent_gemm", 1 if on else 0)


def autotune_report():
    """The autotuner's decisions, one line per class of decomposition."""
    import ctypes as C
    from ._lib import call
    n = C.c_int64()
    call("qtt_autotune_report", None, 0, C.byref(n))
    buf = C.create_string_buffer(n.value + 1)
    call("qtt_autotune_report", buf, n.value + 1, C.byref(n))
    return buf.value.decode()


def set_jacobi_kernel(which):
    """Sector-SVD Jacobi kernel: 'block' (block-cyclic wherever it fits, the
    default) or 'scalar' (one column pair per warp and grid step)."""
    from ._lib import call
    call("qtt_set_jacobi_kernel", {"block": 0, "scalar": 1}[which] if isinstance(which, str) else int(which))


class stats:
    """Per-kernel-class device time (CUDA events) and algorithmic work."""
    KINDS = {"gemm": 0, "permute": 1, "svd": 2, "elementwise": 3, "pack": 4, "svd_fp64": 5, "jacobi_fp32": 6,
             "jacobi_fp64": 7}

    @staticmethod
    def enable(on=True):
        from ._lib import call
        call("qtt_stats_enable", int(bool(on)))

    @staticmethod
    def reset():
        from ._lib import call
        call("qtt_stats_reset")

    @staticmethod
    def get(kind):
        import ctypes as C
        from ._lib import call
        ms, work, n = C.c_double(), C.c_double(), C.c_int64()
        call("qtt_stats_get", stats.KINDS[kind], C.byref(ms), C.byref(work), C.byref(n))
        return {"ms": ms.value, "work": work.value, "launches": n.value}

    @staticmethod
    def launches():
        return int(lib().qtt_launch_count())
