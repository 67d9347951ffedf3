"""Sector decompositions, mirroring ``quantit.linalg`` (python_binding/linalg.cpp:14-111)."""
import ctypes as C

from . import _lib
from .tensor import btensor

SIZE_MAX = 2 ** 63 - 1


def _out3(name, *args):
    U, d, V = C.c_void_p(), C.c_void_p(), C.c_void_p()
    _lib.call(name, *args, C.byref(U), C.byref(d), C.byref(V))
    return btensor._wrap(U), btensor._wrap(d), btensor._wrap(V)


def svd(tensor, split=None, tol=None, *, min_size=1, max_size=SIZE_MAX, pow=2):
    """svd(tensor) | svd(tensor, split) | svd(tensor, split, tol, min_size=, max_size=, pow=).

    Returns (U, d, V) with tensor = U * diag(d) * V^H sector by sector."""
    if split is None:
        return _out3("qtt_svd", tensor._h)
    if tol is None:
        return _out3("qtt_svd_split", tensor._h, int(split))
    return _out3("qtt_svd_truncate", tensor._h, int(split), float(tol), int(min_size), int(min(max_size, SIZE_MAX)),
                 float(pow))


def truncate(U, d, V, max_size, min_size, tol, pow=2):
    """truncate(U, d, V, max, min, tol, pow) (blockTensor/LinearAlgebra.h:246)."""
    Uo, do, Vo = C.c_void_p(), C.c_void_p(), C.c_void_p()
    _lib.call("qtt_truncate", U._h, d._h, V._h if V is not None else None, int(min(max_size, SIZE_MAX)),
              int(min_size), float(tol), float(pow), C.byref(Uo), C.byref(do), C.byref(Vo))
    return btensor._wrap(Uo), btensor._wrap(do), (btensor._wrap(Vo) if V is not None else None)


def eigh(tensor, split=None, upper=False):
    """eigh(tensor, upper) or eigh(tensor, split): (eigenvalues d, eigenvectors U)."""
    d, U = C.c_void_p(), C.c_void_p()
    if split is None:
        _lib.call("qtt_eigh", tensor._h, int(bool(upper)), C.byref(d), C.byref(U))
    else:
        _lib.call("qtt_eigh_split", tensor._h, int(split), C.byref(d), C.byref(U))
    return btensor._wrap(d), btensor._wrap(U)


def last_svd_sweeps(fp32_stage=False):
    """Jacobi sweeps each sector needed in the calling thread's most recent
    decomposition: the FP64 sweeps that produced the factors, or with fp32_stage
    the FP32 sweeps the mixed path ran before them (empty after a plain FP64
    decomposition).  No reference counterpart; synchronises."""
    name = "qtt_last_svd_fp32_sweeps" if fp32_stage else "qtt_last_svd_sweeps"
    n = C.c_int32()
    _lib.call(name, None, 0, C.byref(n))
    buf = (C.c_int32 * max(n.value, 1))()
    _lib.call(name, buf, n.value, C.byref(n))
    return list(buf[:n.value])
