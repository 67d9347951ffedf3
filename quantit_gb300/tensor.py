"""The ``btensor`` handle class: QuantiT's block-sparse tensor on a GB300.

Mirrors the Python binding's ``quantit.btensor`` (python_binding/quantt.cpp:77-750)
for the operations of the accelerated path.  Block data lives in device memory;
``blocks()`` downloads it.  Every operation goes through libqtt_gb300.so.
"""
import ctypes as C

import numpy as np

from . import _lib
from .conserved import quantity

F64, F32 = 0, 1


def _dt_code(dtype):
    if dtype in (None, np.float64, "float64", "f64", float):
        return F64
    if dtype in (np.float32, "float32", "f32"):
        return F32
    raise ValueError(f"unsupported dtype {dtype}")


class btensor:
    """Block-sparse tensor handle (immutable; operations return new handles)."""

    __slots__ = ("_h",)

    def __init__(self, legs=None, selection_rule=None, dtype=None, _handle=None):
        if _handle is not None:
            self._h = _handle
            return
        if legs is None:
            raise ValueError("btensor needs its legs: [[(size, quantity), ...], ...]")
        rank = len(legs)
        sel = selection_rule if selection_rule is not None else legs[0][0][1].neutral()
        mods = sel.mods
        sbd = [len(l) for l in legs]
        ssz = [int(s) for l in legs for s, _ in l]
        cv = []
        for l in legs:
            for _, q in l:
                if q.mods != mods:
                    raise TypeError("every charge needs the selection rule's group")
                cv.extend(q.values)
        nc = len(mods)
        h = C.c_void_p()
        _lib.call("qtt_bt_create", rank, _lib.i64_array(sbd), _lib.i64_array(ssz), nc,
                  (C.c_uint16 * nc)(*mods), (C.c_int16 * max(len(cv), 1))(*[_s16(v) for v in cv]),
                  (C.c_int16 * nc)(*[_s16(v) for v in sel.values]), _dt_code(dtype), C.byref(h))
        self._h = h

    # ------------------------------------------------------------- lifetime
    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _lib._lib is not None:
            _lib.lib().qtt_bt_destroy(h)
            self._h = None

    @staticmethod
    def _wrap(h):
        return btensor(_handle=h)

    # ------------------------------------------------------------- structure
    def _meta(self):
        r, ns, nc, nb, nnz, dt, hd = (C.c_int32(), C.c_int64(), C.c_int32(), C.c_int64(), C.c_int64(),
                                      C.c_int32(), C.c_int32())
        _lib.call("qtt_bt_meta", self._h, C.byref(r), C.byref(ns), C.byref(nc), C.byref(nb), C.byref(nnz),
                  C.byref(dt), C.byref(hd))
        return r.value, ns.value, nc.value, nb.value, nnz.value, dt.value, hd.value

    def dim(self):
        return self._meta()[0]

    def structure(self):
        """(sections_by_dim, section_sizes, c_vals as quantities, selection_rule)."""
        r, ns, nc, nb, nnz, dt, hd = self._meta()
        sbd = (C.c_int64 * max(r, 1))()
        ssz = (C.c_int64 * max(ns, 1))()
        cv = (C.c_int16 * max(ns * nc, 1))()
        sel = (C.c_int16 * nc)()
        mods = (C.c_uint16 * nc)()
        _lib.call("qtt_bt_structure", self._h, sbd, ssz, cv, sel, mods)
        mods_t = tuple(int(m) for m in mods)

        def q(vals):
            return quantity._raw(tuple((v & 0xFFFF) if m else int(v) for v, m in zip(vals, mods_t)), mods_t)
        cvals = [q(cv[i * nc:(i + 1) * nc]) for i in range(ns)]
        return list(sbd[:r]), list(ssz[:ns]), cvals, q(sel[:nc])

    @property
    def sections_by_dim(self):
        return self.structure()[0]

    @property
    def section_sizes(self):
        return self.structure()[1]

    @property
    def c_vals(self):
        return self.structure()[2]

    @property
    def selection_rule(self):
        return self.structure()[3]

    @property
    def dtype(self):
        return np.float64 if self._meta()[5] == F64 else np.float32

    def sizes(self):
        sbd, ssz, _, _ = self.structure()
        out, a = [], 0
        for n in sbd:
            out.append(int(sum(ssz[a:a + n])))
            a += n
        return out

    def block_indices(self):
        r, ns, nc, nb, nnz, dt, hd = self._meta()
        idx = (C.c_int64 * max(nb * r, 1))()
        _lib.call("qtt_bt_blocks", self._h, idx, None)
        return [tuple(idx[b * r:(b + 1) * r]) for b in range(nb)]

    def _sizes(self):
        """(sections_by_dim, section_sizes) without the charges."""
        r, ns, nc, nb, nnz, dt, hd = self._meta()
        sbd = (C.c_int64 * max(r, 1))()
        ssz = (C.c_int64 * max(ns, 1))()
        cv = (C.c_int16 * max(ns * nc, 1))()
        sel = (C.c_int16 * max(nc, 1))()
        mods = (C.c_uint16 * max(nc, 1))()
        _lib.call("qtt_bt_structure", self._h, sbd, ssz, cv, sel, mods)
        return list(sbd[:r]), list(ssz[:ns])

    @staticmethod
    def _shape_of(sizes, idx):
        sbd, ssz = sizes
        shp, a = [], 0
        for d, i in enumerate(idx):
            shp.append(ssz[a + i])
            a += sbd[d]
        return tuple(shp)

    def block_shape(self, idx):
        return self._shape_of(self._sizes(), idx)

    def has_data(self):
        return bool(self._meta()[6])

    def nnz(self):
        return self._meta()[4]

    def blocks(self):
        """[(block index, numpy array)] in block-list order (downloads from the device)."""
        r, ns, nc, nb, nnz, dt, hd = self._meta()
        idx = (C.c_int64 * max(nb * r, 1))()
        numel = (C.c_int64 * max(nb, 1))()
        _lib.call("qtt_bt_blocks", self._h, idx, numel)
        npdt = np.float64 if dt == F64 else np.float32
        flat = np.empty(max(nnz, 1), dtype=npdt)
        if nnz:
            _lib.call("qtt_bt_download", self._h, flat.ctypes.data_as(C.c_void_p), flat.nbytes)
        sizes = self._sizes()
        out, o = [], 0
        for b in range(nb):
            key = tuple(idx[b * r:(b + 1) * r])
            n = numel[b]
            out.append((key, flat[o:o + n].reshape(self._shape_of(sizes, key)).copy()))
            o += n
        return out

    def block_at(self, idx):
        """Data of one block; IndexError when the block is absent (btensor::block_at)."""
        for k, v in self.blocks():
            if k == tuple(idx):
                return v
        raise IndexError(f"no block at {tuple(idx)}")

    def check(self):
        buf = C.create_string_buffer(1 << 14)
        _lib.call("qtt_bt_check", self._h, buf, len(buf))
        return buf.value.decode()

    # ------------------------------------------------------------- construction
    def set_blocks(self, blocks):
        """Replace the block list with [(index, array)] (uploads to the device)."""
        sizes = self._sizes()
        dt = self.dtype
        idx, arrs = [], []
        for k, v in blocks:
            idx.extend(int(i) for i in k)
            shp = self._shape_of(sizes, tuple(k))
            a = np.ascontiguousarray(v, dtype=dt)
            if a.shape != shp:
                raise ValueError(f"block {tuple(k)} has shape {a.shape}, {shp} expected")
            arrs.append(a.ravel())
        data = np.concatenate(arrs) if arrs else np.zeros(1, dtype=dt)
        _lib.call("qtt_bt_set_blocks", self._h, len(arrs), _lib.i64_array(idx),
                  data.ctypes.data_as(C.c_void_p))
        return self

    def set_block_structure(self, indices):
        """Block list without data (structure-only tensor, no GPU needed)."""
        flat = [int(i) for k in indices for i in k]
        _lib.call("qtt_bt_set_block_structure", self._h, len(indices), _lib.i64_array(flat))
        return self

    def copy_structure(self):
        sbd, ssz, cv, sel = self.structure()
        legs, a = [], 0
        for n in sbd:
            legs.append([(ssz[a + i], cv[a + i]) for i in range(n)])
            a += n
        return btensor(legs, sel, dtype=self.dtype)

    # ------------------------------------------------------------- operations
    def _unary(self, name, *args):
        h = C.c_void_p()
        _lib.call(name, self._h, *args, C.byref(h))
        return btensor._wrap(h)

    def tensordot(self, other, dims):
        """tensordot(other, (dims_self, dims_other)) or tensordot(other, n)."""
        if isinstance(dims, int):
            da = list(range(self.dim() - dims, self.dim()))
            db = list(range(dims))
        else:
            da, db = dims
        if len(da) != len(db):
            raise RuntimeError("both dimension lists should have the same length.")
        h = C.c_void_p()
        _lib.call("qtt_tensordot", self._h, other._h, len(da), _lib.i64_array(da), _lib.i64_array(db), C.byref(h))
        return btensor._wrap(h)

    def permute(self, perm):
        return self._unary("qtt_permute", _lib.i64_array(perm))

    def reshape(self, index_groups):
        return self._unary("qtt_reshape", len(index_groups), _lib.i64_array(index_groups))

    def reshape_as(self, other):
        return self._unary("qtt_reshape_as", other._h)

    def conj(self):
        return self._unary("qtt_conj")

    def inverse_cvals(self):
        return self._unary("qtt_inverse_cvals")

    def add(self, other, alpha=1.0):
        return self._unary("qtt_add", other._h, float(alpha))

    def sub(self, other, alpha=1.0):
        return self.add(other, -alpha)

    def mul(self, other):
        if isinstance(other, btensor):
            return self._unary("qtt_mul_lastleg", other._h)
        return self._unary("qtt_mul_scalar", float(other))

    def __add__(self, other):
        return self.add(other)

    def __sub__(self, other):
        return self.sub(other)

    def __mul__(self, other):
        return self.mul(other)

    __rmul__ = __mul__

    def __truediv__(self, s):
        return self.mul(1.0 / float(s))

    def __repr__(self):
        try:
            sbd, ssz, cv, sel = self.structure()
            return f"btensor(sections={sbd}, sizes={ssz}, selection_rule={sel}, blocks={len(self.block_indices())})"
        except Exception:  # pragma: no cover
            return "btensor(<invalid>)"


def _s16(v):
    v = int(v)
    return v - 65536 if v >= 32768 else v


def from_blocks(legs, selection_rule, blocks, dtype=None):
    return btensor(legs, selection_rule, dtype=dtype).set_blocks(blocks)


def tensordot(a, b, dims_a, dims_b):
    return a.tensordot(b, (list(dims_a), list(dims_b)))


def tensorgdot(add, mul1, mul2, dims1, dims2, beta=1.0, alpha=1.0):
    """beta*add + alpha*tensordot(mul1, mul2, dims1, dims2) (addmm semantics)."""
    h = C.c_void_p()
    _lib.call("qtt_tensorgdot", add._h, mul1._h, mul2._h, len(dims1), _lib.i64_array(dims1), _lib.i64_array(dims2),
              float(beta), float(alpha), C.byref(h))
    return btensor._wrap(h)


def tensorgdot_(add, mul1, mul2, dims1, dims2, beta=1.0, alpha=1.0):
    _lib.call("qtt_tensorgdot_", add._h, mul1._h, mul2._h, len(dims1), _lib.i64_array(dims1), _lib.i64_array(dims2),
              float(beta), float(alpha))
    return add


def dot_all(a, b):
    """tensordot(a, b.conj(), all legs).item()."""
    out = C.c_double()
    _lib.call("qtt_dot_all", a._h, b._h, C.byref(out))
    return out.value
