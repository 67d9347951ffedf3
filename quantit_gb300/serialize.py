"""Block-list serialisation of btensors, MPS and MPO (checkpoint / resume).

The reference has no on-disk format for block tensors.  This one stores, per
tensor, the structure exactly as the C-ABI describes it (sections per leg,
section sizes, charges [section][component], selection rule, group moduli) plus
the block list [block][rank] and ONE contiguous data array in block-list order,
so a tensor is written with a single device-to-host copy and read back with a
single upload.  A file is a NumPy ``.npz`` archive (no pickling) holding:

  ``format``  the string ``qtt-blocklist-1``
  ``kind``    ``btensor``, ``bMPS`` or ``bMPO``; ``count`` tensors;
  ``oc``      the orthogonality centre of a bMPS;
  ``t{i}_sbd``, ``t{i}_ssz``, ``t{i}_cv``, ``t{i}_sel``, ``t{i}_mods``,
  ``t{i}_bidx``, ``t{i}_data`` (absent for a structure-only tensor), ``t{i}_dtype``.
"""
import ctypes as C

import numpy as np

from . import _lib
from .tensor import btensor

FORMAT = "qtt-blocklist-1"
_NPDT = {0: np.float64, 1: np.float32}


def _p(a, ctype):
    """Typed pointer to a contiguous array (a one-element dummy for an empty one)."""
    if a.size == 0:
        a = np.zeros(1, dtype=a.dtype)
    return a.ctypes.data_as(C.POINTER(ctype)), a


def tensor_arrays(t):
    """The structure and data of one btensor as NumPy arrays (one download)."""
    r, ns, nc, nb, nnz, dt, hd = t._meta()
    sbd = np.zeros(max(r, 1), dtype=np.int64)
    ssz = np.zeros(max(ns, 1), dtype=np.int64)
    cv = np.zeros(max(ns * nc, 1), dtype=np.int16)
    sel1 = np.zeros(max(nc, 1), dtype=np.int16)
    mods1 = np.zeros(max(nc, 1), dtype=np.uint16)
    _lib.call("qtt_bt_structure", t._h, sbd.ctypes.data_as(C.POINTER(C.c_int64)),
              ssz.ctypes.data_as(C.POINTER(C.c_int64)), cv.ctypes.data_as(C.POINTER(C.c_int16)),
              sel1.ctypes.data_as(C.POINTER(C.c_int16)), mods1.ctypes.data_as(C.POINTER(C.c_uint16)))
    sel, mods = sel1[:nc], mods1[:nc]
    bidx = np.zeros(max(nb * r, 1), dtype=np.int64)
    numel = np.zeros(max(nb, 1), dtype=np.int64)
    _lib.call("qtt_bt_blocks", t._h, bidx.ctypes.data_as(C.POINTER(C.c_int64)),
              numel.ctypes.data_as(C.POINTER(C.c_int64)))
    out = {"sbd": sbd[:r], "ssz": ssz[:ns], "cv": cv[:ns * nc].reshape(ns, nc), "sel": sel, "mods": mods,
           "bidx": bidx[:nb * r].reshape(nb, r), "dtype": np.int32(dt)}
    if hd:
        data = np.empty(max(nnz, 1), dtype=_NPDT[dt])
        if nnz:
            _lib.call("qtt_bt_download", t._h, data.ctypes.data_as(C.c_void_p), C.c_int64(data.nbytes))
        out["data"] = data[:nnz]
    return out


def tensor_from_arrays(d):
    """A btensor from ``tensor_arrays`` output (one upload when data is present)."""
    sbd = np.ascontiguousarray(d["sbd"], dtype=np.int64)
    ssz = np.ascontiguousarray(d["ssz"], dtype=np.int64)
    cv = np.ascontiguousarray(d["cv"], dtype=np.int16).reshape(-1)
    sel = np.ascontiguousarray(d["sel"], dtype=np.int16)
    mods = np.ascontiguousarray(d["mods"], dtype=np.uint16)
    bidx = np.ascontiguousarray(d["bidx"], dtype=np.int64)
    rank = int(sbd.size)
    nc = int(mods.size)
    if rank and int(np.sum(sbd)) != ssz.size:
        raise ValueError("corrupt block list: section counts and sizes disagree")
    if cv.size != ssz.size * nc or sel.size != nc:
        raise ValueError("corrupt block list: charge arrays have the wrong length")
    h = C.c_void_p()
    keep = []  # the arrays behind the pointers stay alive for the calls

    def ptr(a, ctype):
        p, arr = _p(a, ctype)
        keep.append(arr)
        return p

    _lib.call("qtt_bt_create", rank, ptr(sbd, C.c_int64), ptr(ssz, C.c_int64), nc, ptr(mods, C.c_uint16),
              ptr(cv, C.c_int16), ptr(sel, C.c_int16), int(d.get("dtype", 0)), C.byref(h))
    t = btensor._wrap(h)
    nb = bidx.shape[0] if bidx.ndim == 2 else 0
    if "data" in d:
        data = np.ascontiguousarray(d["data"], dtype=_NPDT[int(d.get("dtype", 0))])
        if data.size == 0:
            data = np.zeros(1, dtype=data.dtype)
        _lib.call("qtt_bt_set_blocks", t._h, int(nb), ptr(bidx.reshape(-1), C.c_int64),
                  data.ctypes.data_as(C.c_void_p))
    else:
        _lib.call("qtt_bt_set_block_structure", t._h, int(nb), ptr(bidx.reshape(-1), C.c_int64))
    return t


def save(path, obj):
    """Write a btensor, a bMPS (with its orthogonality centre) or a bMPO / list."""
    from .networks import bMPO, bMPS
    if isinstance(obj, btensor):
        kind, tensors, oc = "btensor", [obj], 0
    elif isinstance(obj, bMPS):
        kind, tensors, oc = "bMPS", list(obj), int(obj.orthogonality_center)
    else:
        kind, tensors, oc = "bMPO", list(obj), 0
    arrays = {"format": np.array(FORMAT), "kind": np.array(kind), "count": np.int64(len(tensors)), "oc": np.int64(oc)}
    for i, t in enumerate(tensors):
        for k, v in tensor_arrays(t).items():
            arrays[f"t{i}_{k}"] = v
    with open(path, "wb") as f:
        np.savez(f, **arrays)


def load(path):
    """Read what ``save`` wrote: a btensor, a bMPS or a bMPO."""
    from .networks import bMPO, bMPS
    with np.load(path, allow_pickle=False) as z:
        if str(z["format"]) != FORMAT:
            raise ValueError(f"{path}: not a {FORMAT} file")
        kind, n, oc = str(z["kind"]), int(z["count"]), int(z["oc"])
        tensors = []
        for i in range(n):
            pre = f"t{i}_"
            d = {k[len(pre):]: z[k] for k in z.files if k.startswith(pre)}
            tensors.append(tensor_from_arrays(d))
    if kind == "btensor":
        return tensors[0]
    if kind == "bMPS":
        return bMPS(tensors, oc)
    return bMPO(tensors)
