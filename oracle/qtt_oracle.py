"""CPU oracle for the block-sparse DMRG hot path -- TEST INFRASTRUCTURE ONLY.

This module is a plain numpy restatement of QuantiT's algorithms for the path
that the GPU library accelerates.  It exists to check the CUDA path: only the
tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may
import it.  The product (``quantit_gb300``) never calls it.

Parity pinning: the restatement is checked against every known-answer case of
the reference's own unit tests for this path (block lists, reshape charges and
sizes, sector order, the exact L=3 Heisenberg matrix, the 2x2 eigenproblem, the
Lanczos identities, the truncation bound); see ``tests/golden``.  The reference
itself needs libtorch to build, so it is not compiled here.

Each function cites the reference routine it restates (paths relative to the
QuantiT source tree).  Charges are tuples of ints, one entry per group factor;
``mods`` gives the factor kinds: 0 for U(1) (``conserved::Z``, int16) and N>0 for
Z(N) (``conserved::C<N>``, uint16 in [0,N)).
"""
from __future__ import annotations

import itertools
import math
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

Charge = Tuple[int, ...]
Index = Tuple[int, ...]

# --------------------------------------------------------------------------
# charges  (include/Conserved/quantity.h classes C, Z; Composite/quantity_impl.h)
# --------------------------------------------------------------------------


def _wrap16(v: int) -> int:
    return ((v + 32768) % 65536) - 32768


def make_C(v: int, n: int) -> int:
    """conserved::C<N>(int16) constructor, include/Conserved/quantity.h:96.

    ``val = (v != -N)*(v < 0)*N + (v % N)`` with C++ truncating modulo, stored in
    a uint16."""
    r = abs(v) % n
    if v < 0:
        r = -r
    return ((int(v != -n) * int(v < 0)) * n + r) & 0xFFFF


def make_charge(values: Sequence[int], mods: Sequence[int]) -> Charge:
    out = []
    for v, m in zip(values, mods):
        out.append(make_C(int(v), m) if m else _wrap16(int(v)))
    return tuple(out)


def q_add(a: Charge, b: Charge, mods: Sequence[int]) -> Charge:
    """Group operation: Z adds (int16), C<N> adds modulo N (quantity.h:116-134,196-203)."""
    return tuple(((x + y) % m) if m else _wrap16(x + y) for x, y, m in zip(a, b, mods))


def q_inv(a: Charge, mods: Sequence[int]) -> Charge:
    """inverse_(): Z negates, C<N> maps v -> (v != 0)*(N - v) (quantity.h:135-143,212-220)."""
    return tuple(((m - x) if x else 0) if m else _wrap16(-x) for x, m in zip(a, mods))


def q_neutral(mods: Sequence[int]) -> Charge:
    return tuple(0 for _ in mods)


# Charge order is tuple-lexicographic (Composite/quantity_impl.h:326-329) with
# signed compare for Z and unsigned compare for C<N>; python tuple order on the
# stored values is exactly that.


# --------------------------------------------------------------------------
# btensor structure  (include/blockTensor/btensor.h:105-169,821-837)
# --------------------------------------------------------------------------


@dataclass
class BTensor:
    mods: Tuple[int, ...]
    sbd: List[int]                  # sections_by_dim
    ssz: List[int]                  # packed sections_sizes
    cv: List[Charge]                # packed c_vals
    sel: Charge                     # selection_rule
    blocks: List[Tuple[Index, np.ndarray]] = field(default_factory=list)
    dtype: type = np.float64

    @property
    def rank(self) -> int:
        return len(self.sbd)

    def addr(self, d: int) -> int:
        return int(sum(self.sbd[:d]))

    def sec_sizes(self, d: int) -> List[int]:
        a = self.addr(d)
        return self.ssz[a:a + self.sbd[d]]

    def sec_charges(self, d: int) -> List[Charge]:
        a = self.addr(d)
        return self.cv[a:a + self.sbd[d]]

    def block_shape(self, idx: Index) -> Tuple[int, ...]:
        return tuple(self.ssz[self.addr(d) + i] for d, i in enumerate(idx))

    def block_charge_sum(self, idx: Index) -> Charge:
        q = q_neutral(self.mods)
        for d, i in enumerate(idx):
            q = q_add(q, self.cv[self.addr(d) + i], self.mods)
        return q

    def allowed(self, idx: Index) -> bool:
        """block_conservation_rule_test, sources/btensor.cpp:363-372."""
        return self.block_charge_sum(idx) == self.sel

    def sizes(self) -> List[int]:
        return [int(sum(self.sec_sizes(d))) for d in range(self.rank)]

    def block_dict(self) -> Dict[Index, np.ndarray]:
        return {k: v for k, v in self.blocks}

    def empty_like(self) -> "BTensor":
        return BTensor(self.mods, list(self.sbd), list(self.ssz), list(self.cv), self.sel, [], self.dtype)

    def copy(self) -> "BTensor":
        out = self.empty_like()
        out.blocks = [(k, v.copy()) for k, v in self.blocks]
        return out

    def check(self) -> str:
        """check_tensor, sources/btensor.cpp:405-467 (returns '' when consistent)."""
        msg = []
        if sum(self.sbd) != len(self.ssz) or len(self.ssz) != len(self.cv):
            msg.append("section tables inconsistent")
        for idx, b in self.blocks:
            if len(idx) != self.rank:
                msg.append(f"block {idx}: wrong rank")
                continue
            if any(i >= s or i < 0 for i, s in zip(idx, self.sbd)):
                msg.append(f"block {idx}: index out of range")
                continue
            if not self.allowed(idx):
                msg.append(f"block {idx}: incompatible with selection rule")
            if tuple(b.shape) != self.block_shape(idx):
                msg.append(f"block {idx}: shape {b.shape} != {self.block_shape(idx)}")
        return "\n".join(msg)

    def nnz(self) -> int:
        return int(sum(b.size for _, b in self.blocks))


def btensor(legs: Sequence[Sequence[Tuple[int, Sequence[int]]]], sel: Sequence[int],
            mods: Sequence[int], dtype=np.float64) -> BTensor:
    """btensor(vec_list_t, selection_rule) constructor (sources/btensor.cpp:299-313): an
    empty block list over the given legs [(section size, charge), ...]."""
    mods = tuple(mods)
    sbd = [len(l) for l in legs]
    ssz = [int(s) for l in legs for s, _ in l]
    cv = [make_charge(q if isinstance(q, (list, tuple)) else [q], mods) for l in legs for _, q in l]
    return BTensor(mods, sbd, ssz, cv, make_charge(sel if isinstance(sel, (list, tuple)) else [sel], mods),
                   [], dtype)


def allowed_blocks(t: BTensor) -> List[Index]:
    """Every block index allowed by the selection rule, in lexicographic order
    (the set factory_wrap fills, sources/btensor.cpp:2341-2354)."""
    out = []
    for idx in itertools.product(*[range(s) for s in t.sbd]):
        if t.allowed(idx):
            out.append(tuple(idx))
    return out


def fill(t: BTensor, gen) -> BTensor:
    """Fill every allowed block with ``gen(shape)``, in lexicographic block order."""
    out = t.empty_like()
    for idx in allowed_blocks(t):
        out.blocks.append((idx, np.asarray(gen(t.block_shape(idx)), dtype=t.dtype)))
    return out


def randn_like(t: BTensor, rng: np.random.Generator) -> BTensor:
    return fill(t, lambda s: rng.standard_normal(s))


def to_dense(t: BTensor) -> np.ndarray:
    """to_dense, sources/btensor.cpp:2491."""
    out = np.zeros(t.sizes(), dtype=t.dtype)
    offs = [np.concatenate([[0], np.cumsum(t.sec_sizes(d))]).astype(int) for d in range(t.rank)]
    for idx, b in t.blocks:
        sl = tuple(slice(offs[d][i], offs[d][i + 1]) for d, i in enumerate(idx))
        out[sl] = b
    return out


# --------------------------------------------------------------------------
# permute / conj  (sources/btensor.cpp:1754-1804, 2156-2172)
# --------------------------------------------------------------------------


def permute(t: BTensor, perm: Sequence[int]) -> BTensor:
    """btensor::permute, sources/btensor.cpp:1754-1804."""
    r = t.rank
    perm = [p + r if p < 0 else p for p in perm]
    out = BTensor(t.mods, [t.sbd[p] for p in perm],
                  [s for p in perm for s in t.sec_sizes(p)],
                  [q for p in perm for q in t.sec_charges(p)], t.sel, [], t.dtype)
    blocks = [(tuple(idx[p] for p in perm), np.ascontiguousarray(b.transpose(perm))) for idx, b in t.blocks]
    blocks.sort(key=lambda kv: kv[0])
    out.blocks = blocks
    return out


def inverse_cvals(t: BTensor) -> BTensor:
    """inverse_cvals_, sources/btensor.cpp:2163-2172 (shares the block data)."""
    out = BTensor(t.mods, list(t.sbd), list(t.ssz), [q_inv(q, t.mods) for q in t.cv],
                  q_inv(t.sel, t.mods), list(t.blocks), t.dtype)
    return out


def conj(t: BTensor) -> BTensor:
    """btensor::conj = conj_only().inverse_cvals_(), sources/btensor.cpp:2156."""
    c = inverse_cvals(t)
    c.blocks = [(k, np.conj(v)) for k, v in t.blocks]
    return c


# --------------------------------------------------------------------------
# tensordot  (sources/btensor.cpp:783-883, 1843-1935, 1971-2119)
# --------------------------------------------------------------------------


class ContractionError(ValueError):
    pass


def tdot_structure(A: BTensor, B: BTensor, dA: Sequence[int], dB: Sequence[int]):
    """compute_tdot_shape + check_product_compat + compute_tdot_cval_sectSize
    (sources/btensor.cpp:783-883,1908-1935).  Returns (p1, p2, empty output)."""
    dA = [d + A.rank if d < 0 else d for d in dA]
    dB = [d + B.rank if d < 0 else d for d in dB]
    if len(dA) != len(dB):
        raise ContractionError("both dimension lists should have the same length.")
    if A.mods != B.mods:
        raise ContractionError("the two tensors have different type of conserved quantities")
    neut = q_neutral(A.mods)
    for a, b in zip(dA, dB):
        if A.sbd[a] != B.sbd[b]:
            raise ContractionError(f"contracted dimensions need to match, but first has {A.sbd[a]} sections along "
                                   f"dim {a} and second has {B.sbd[b]} sections along dim {b}")
        for qa, qb in zip(A.sec_charges(a), B.sec_charges(b)):
            if q_add(qa, qb, A.mods) != neut:
                raise ContractionError(f"contracted conserved numbers need to sum to zero, but there is a violation "
                                       f"when contracting dim {a} of the left tensor with dim {b} of the right tensor")
        if A.sec_sizes(a) != B.sec_sizes(b):
            raise ContractionError(f"contracted section sizes differ between dim {a} and dim {b}")
    freeA = [i for i in range(A.rank) if i not in dA]
    freeB = [i for i in range(B.rank) if i not in dB]
    p1 = freeA + dA
    p2 = dB + freeB
    out = BTensor(A.mods, [A.sbd[i] for i in freeA] + [B.sbd[i] for i in freeB],
                  [s for i in freeA for s in A.sec_sizes(i)] + [s for i in freeB for s in B.sec_sizes(i)],
                  [q for i in freeA for q in A.sec_charges(i)] + [q for i in freeB for q in B.sec_charges(i)],
                  q_add(A.sel, B.sel, A.mods), [], np.result_type(A.dtype, B.dtype).type)
    return p1, p2, dA, dB, freeA, freeB, out


def _permute_bl(t: BTensor, block_perm: Sequence[int], tensor_perm: Sequence[int], split: int):
    """permute_bl, sources/btensor.cpp:1843-1894: permute each block's index and data,
    reshape the data to a (split | rest) matrix, re-sort the list."""
    out = []
    for idx, b in t.blocks:
        nidx = tuple(idx[p] for p in block_perm)
        m = b.transpose(tensor_perm)
        a = int(np.prod(m.shape[:split])) if split > 0 else 1
        c = int(np.prod(m.shape[split:])) if split < m.ndim else 1
        out.append((nidx, m.reshape(a, c)))
    out.sort(key=lambda kv: kv[0])
    return out


def tdot_plan(A: BTensor, B: BTensor, dA: Sequence[int], dB: Sequence[int]):
    """The merge-join of btensor::tensordot (sources/btensor.cpp:1998-2114) on block
    indices only.  Returns the output structure and, per output block in emission
    order, the list of (A block position, B block position) pairs in accumulation
    order (positions refer to A.blocks / B.blocks)."""
    p1, p2, dA, dB, freeA, freeB, out = tdot_structure(A, B, dA, dB)
    dl = len(dA)
    p2p = p2[dl:] + p2[:dl]
    t1 = sorted([(tuple(idx[p] for p in p1), n) for n, (idx, _) in enumerate(A.blocks)])
    t2 = sorted([(tuple(idx[p] for p in p2p), n) for n, (idx, _) in enumerate(B.blocks)])
    nfa = A.rank - dl
    nfb = B.rank - dl

    def runs(lst, nf):
        res = []
        i = 0
        while i < len(lst):
            j = i + 1
            if dl == 0:
                pass  # every block is its own run (next_index increments the last entry)
            else:
                while j < len(lst) and lst[j][0][:nf] == lst[i][0][:nf]:
                    j += 1
            res.append((i, j))
            i = j
        return res

    plan = []
    for (a0, a1) in runs(t1, nfa):
        for (b0, b1) in runs(t2, nfb):
            ia, ib = a0, b0
            pairs = []
            while ia < a1 and ib < b1:
                sa = t1[ia][0][nfa:]
                sb = t2[ib][0][nfb:]
                if sa < sb:
                    ia += 1
                elif sb < sa:
                    ib += 1
                else:
                    pairs.append((t1[ia][1], t2[ib][1]))
                    ia += 1
                    ib += 1
            if pairs:
                oidx = tuple(t1[a0][0][:nfa]) + tuple(t2[b0][0][:nfb])
                plan.append((oidx, pairs))
    return out, plan, p1, p2


def tensordot(A: BTensor, B: BTensor, dA: Sequence[int], dB: Sequence[int]) -> BTensor:
    """btensor::tensordot, sources/btensor.cpp:1971-2119.

    Output blocks exist only where at least one (A, B) block pair matches on the
    contracted legs; each is mm of the first pair plus addmm_ of the others."""
    out, plan, p1, p2 = tdot_plan(A, B, dA, dB)
    dl = len(dA)
    split1 = A.rank - dl
    blocks = []
    for oidx, pairs in plan:
        acc = None
        for na, nb in pairs:
            ma = A.blocks[na][1].transpose(p1)
            ma = ma.reshape(int(np.prod(ma.shape[:split1])) if split1 else 1, -1 if ma.size else 0)
            mb = B.blocks[nb][1].transpose(p2)
            mb = mb.reshape(int(np.prod(mb.shape[:dl])) if dl else 1, -1 if mb.size else 0)
            prod = ma @ mb
            acc = prod if acc is None else acc + prod
        blocks.append((oidx, acc.reshape(out.block_shape(oidx))))
    blocks.sort(key=lambda kv: kv[0])
    out.blocks = blocks
    return out


def tensorgdot(add: BTensor, A: BTensor, B: BTensor, dA, dB, beta: float = 1.0, alpha: float = 1.0) -> BTensor:
    """C = beta*add + alpha*tensordot(A, B): the addmm semantics of the dense
    tensorgdot_out (sources/tensorgdot.cpp:102-117) lifted to btensors (the btensor
    overloads declared at include/blockTensor/btensor.h:624-627,1247-1268 have no
    definition in the reference)."""
    prod = tensordot(A, B, dA, dB)
    if prod.sbd != add.sbd or prod.ssz != add.ssz or prod.cv != add.cv or prod.sel != add.sel:
        raise ContractionError("the add tensor's shape differs from the contraction's output shape")
    return add_scaled(add, prod, beta, alpha)


# --------------------------------------------------------------------------
# elementwise algebra  (sources/btensor.cpp:2666-2760, 1205-1290)
# --------------------------------------------------------------------------


def same_shape(a: BTensor, b: BTensor) -> bool:
    return a.sbd == b.sbd and a.ssz == b.ssz and a.cv == b.cv and a.sel == b.sel


def add_scaled(a: BTensor, b: BTensor, ca: float, cb: float) -> BTensor:
    """ca*a + cb*b over the union of the block lists (flat_map::merge, btensor::add
    sources/btensor.cpp:2666-2760)."""
    if not same_shape(a, b):
        raise ValueError("incompatible btensors for addition")
    da = a.block_dict()
    db = b.block_dict()
    out = a.empty_like()
    for k in sorted(set(da) | set(db)):
        if k in da and k in db:
            v = ca * da[k] + cb * db[k]
        elif k in da:
            v = ca * da[k]
        else:
            v = cb * db[k]
        out.blocks.append((k, v))
    return out


def scale(a: BTensor, c: float) -> BTensor:
    out = a.empty_like()
    out.blocks = [(k, c * v) for k, v in a.blocks]
    return out


def dot_all(a: BTensor, b: BTensor) -> float:
    """tensordot over every leg with matching block indices (the a0/b/a1 inner
    products of sources/dmrg.cpp:593,596,605).  Returns 0 when no block matches."""
    db = b.block_dict()
    s = 0.0
    for k, v in a.blocks:
        if k in db:
            s += float(np.dot(v.ravel(), db[k].ravel()))
    return s


def mul_lastleg(u: BTensor, d: BTensor) -> BTensor:
    """u.mul(d) for a rank-1 neutral d broadcast on u's last leg
    (broadcast_operation, sources/btensor.cpp:1205-1290): only blocks whose last
    section has a d block survive."""
    dd = d.block_dict()
    out = u.empty_like()
    out.sel = q_add(u.sel, d.sel, u.mods)
    last = u.addr(u.rank - 1)
    # charges of the broadcast leg are combined with d's (neutral) charges
    for i in range(u.sbd[-1]):
        out.cv[last + i] = q_add(u.cv[last + i], d.cv[i], u.mods)
    for k, v in u.blocks:
        if (k[-1],) in dd:
            out.blocks.append((k, v * dd[(k[-1],)]))
    return out


# --------------------------------------------------------------------------
# reshape  (sources/btensor.cpp:2762-3087)
# --------------------------------------------------------------------------


def reshape(t: BTensor, groups: Sequence[int]) -> BTensor:
    """btensor::reshape(index_groups), sources/btensor.cpp:2986-3026.

    New sections are the Cartesian product of the grouped legs' sections in
    right-major order, with charges combined and sizes multiplied
    (reshape_block_prop :2791-2830)."""
    m = [0] + list(groups) + [t.rank]
    sbd, ssz, cv = [], [], []
    for g in range(len(m) - 1):
        dims = list(range(m[g], m[g + 1]))
        n = 1
        for d in dims:
            n *= t.sbd[d]
        sbd.append(n)
        for combo in itertools.product(*[range(t.sbd[d]) for d in dims]):
            s = 1
            q = q_neutral(t.mods)
            for d, i in zip(dims, combo):
                s *= t.ssz[t.addr(d) + i]
                q = q_add(q, t.cv[t.addr(d) + i], t.mods)
            ssz.append(s)
            cv.append(q)
    out = BTensor(t.mods, sbd, ssz, cv, t.sel, [], t.dtype)
    blocks = []
    for idx, b in t.blocks:
        nidx = []
        for g in range(len(m) - 1):
            f = 0
            for d in range(m[g], m[g + 1]):
                f = f * t.sbd[d] + idx[d]
            nidx.append(f)
        nidx = tuple(nidx)
        blocks.append((nidx, b.reshape(out.block_shape(nidx))))
    blocks.sort(key=lambda kv: kv[0])
    out.blocks = blocks
    return out


def _flat(idx, sbd):
    f = 0
    for i, s in zip(idx, sbd):
        f = f * s + i
    return f


def _unflat(f, sbd):
    out = []
    for s in reversed(sbd):
        out.append(f % s)
        f //= s
    return tuple(reversed(out))


def reshape_as(t: BTensor, other: BTensor) -> BTensor:
    """btensor::reshape_as<dims_only>, sources/btensor.cpp:3027-3087: the block
    index is flattened over t's sections and unflattened over other's; the result
    takes other's sections and charges and keeps t's selection rule."""
    if int(np.prod(t.sbd)) != int(np.prod(other.sbd)):
        raise ValueError(f"incompatible sections layouts {t.sbd} and {other.sbd}")
    # compatible_c_vals / compatible_block_size (:2876-2934), over every block position
    for f in range(int(np.prod(t.sbd))):
        it = _unflat(f, t.sbd)
        io = _unflat(f, other.sbd)
        if t.block_charge_sum(it) != other.block_charge_sum(io):
            raise ValueError("incompatible conserved quantities")
        if int(np.prod(t.block_shape(it))) != int(np.prod(other.block_shape(io))):
            raise ValueError("incompatible block dimensions")
    out = BTensor(t.mods, list(other.sbd), list(other.ssz), list(other.cv), t.sel, [], t.dtype)
    blocks = []
    for idx, b in t.blocks:
        nidx = _unflat(_flat(idx, t.sbd), other.sbd)
        blocks.append((nidx, b.reshape(other.block_shape(nidx))))
    blocks.sort(key=lambda kv: kv[0])
    out.blocks = blocks
    return out


def shape_keep(t: BTensor, keep: Sequence[int], invert: bool = False) -> BTensor:
    """Structure made of t's legs ``keep`` (shape_from with -1 on those legs), optionally
    with inverted charges; used to rebuild the U/V shapes of svd(A, split)."""
    cv = [q for d in keep for q in t.sec_charges(d)]
    if invert:
        cv = [q_inv(q, t.mods) for q in cv]
    return BTensor(t.mods, [t.sbd[d] for d in keep], [s for d in keep for s in t.sec_sizes(d)], cv,
                   q_neutral(t.mods), [], t.dtype)


def concat_shapes(*shapes: BTensor) -> BTensor:
    out = BTensor(shapes[0].mods, [], [], [], q_neutral(shapes[0].mods), [], shapes[0].dtype)
    for s in shapes:
        out.sbd += s.sbd
        out.ssz += s.ssz
        out.cv += s.cv
        out.sel = q_add(out.sel, s.sel, out.mods)
    return out


# --------------------------------------------------------------------------
# sector decompositions  (sources/btensor_linalg.cpp:30-534)
# --------------------------------------------------------------------------


def reorder_by_cvals(t: BTensor):
    """reorder_by_cvals, sources/btensor_linalg.cpp:30-67: stable sort of the block
    list by (row charge, column charge) of the last two legs."""
    r = t.rank
    rowq = t.sec_charges(r - 2)
    colq = t.sec_charges(r - 1)
    return sorted(t.blocks, key=lambda kv: (rowq[kv[0][r - 2]], colq[kv[0][r - 1]]))


@dataclass
class Sector:
    other: Index                         # leading block index (rank > 2 batching)
    rows: List[Tuple[int, int, int]]     # (row section, start, stop) in first-appearance order
    cols: List[Tuple[int, int, int]]     # (col section, start, stop); offsets by first appearance,
                                         # list kept sorted by section (compact_dense_single :82-150)
    mat: np.ndarray


def compact_dense(t: BTensor) -> List[Sector]:
    """compact_dense + compact_dense_single, sources/btensor_linalg.cpp:82-255."""
    r = t.rank
    rowq = t.sec_charges(r - 2)
    colq = t.sec_charges(r - 1)
    lst = reorder_by_cvals(t)
    groups = []
    i = 0
    while i < len(lst):
        j = i + 1
        k0 = lst[i][0]
        while j < len(lst):
            k1 = lst[j][0]
            if k1[:r - 2] == k0[:r - 2] and rowq[k1[r - 2]] == rowq[k0[r - 2]] and colq[k1[r - 1]] == colq[k0[r - 1]]:
                j += 1
            else:
                break
        groups.append(lst[i:j])
        i = j
    sectors = []
    for g in groups:
        first = g[0]
        lead_shape = first[1].shape[:r - 2]
        rows = []
        cols = []   # sorted by col index, each (col, start, stop)
        row_acc = 0
        col_acc = 0
        cur_row = first[0][r - 2]
        rows.append((cur_row, 0, first[1].shape[r - 2]))
        row_acc = first[1].shape[r - 2]
        for idx, b in g:
            c = idx[r - 1]
            pos = 0
            while pos < len(cols) and cols[pos][0] < c:
                pos += 1
            if pos == len(cols) or cols[pos][0] != c:
                cols.insert(pos, (c, col_acc, col_acc + b.shape[r - 1]))
                col_acc += b.shape[r - 1]
            if cur_row != idx[r - 2]:
                cur_row = idx[r - 2]
                rows.append((cur_row, row_acc, row_acc + b.shape[r - 2]))
                row_acc += b.shape[r - 2]
        mat = np.zeros(tuple(lead_shape) + (row_acc, col_acc), dtype=t.dtype)
        rmap = {rr: (a, b_) for rr, a, b_ in rows}
        cmap = {cc: (a, b_) for cc, a, b_ in cols}
        for idx, b in g:
            ra, rb = rmap[idx[r - 2]]
            ca, cb = cmap[idx[r - 1]]
            mat[..., ra:rb, ca:cb] = b
        sectors.append(Sector(tuple(first[0][:r - 2]), rows, cols, mat))
    return sectors


def _svd_sector(m: np.ndarray):
    u, s, vh = np.linalg.svd(m, full_matrices=False)
    return u, s, np.swapaxes(vh, -1, -2).conj()


def svd(t: BTensor):
    """svd(btensor, some=true), sources/btensor_linalg.cpp:390-502.  Returns (U, d, V)
    with t = U * diag(d) * V^H per sector; V is returned inverse_cvals()'d."""
    r = t.rank
    secs = compact_dense(t)
    colq = t.sec_charges(r - 1)
    neut = q_neutral(t.mods)
    dq = [colq[s.cols[0][0]] for s in secs]             # :411 right_D_cvals
    dsz = [min(s.mat.shape[-1], s.mat.shape[-2]) for s in secs]
    lead = list(range(r - 2))
    # U: leading legs + row leg + D leg; selection rule of t (:441-442)
    U = concat_shapes(shape_keep(t, lead + [r - 2]),
                      BTensor(t.mods, [len(secs)], dsz, dq, neut, [], t.dtype))
    U.sel = t.sel
    # V: neutral leading legs, col leg, D leg with inverted charges; then inverse_cvals_ (:447-453,501)
    lead_shape = shape_keep(t, lead)
    lead_shape.cv = [neut for _ in lead_shape.cv]
    V = concat_shapes(lead_shape, shape_keep(t, [r - 1]),
                      BTensor(t.mods, [len(secs)], dsz, [q_inv(q, t.mods) for q in dq], neut, [], t.dtype))
    V.sel = neut
    d = concat_shapes(shape_keep(t, lead), BTensor(t.mods, [len(secs)], dsz, [neut] * len(secs), neut, [], t.dtype))
    d.cv = [neut for _ in d.cv]
    d.sel = neut
    ub, vb, db = [], [], []
    for bi, s in enumerate(secs):
        u, sv, v = _svd_sector(s.mat)
        for row, a, b in s.rows:
            ub.append((s.other + (row, bi), np.ascontiguousarray(u[..., a:b, :])))
        for col, a, b in s.cols:
            vb.append((s.other + (col, bi), np.ascontiguousarray(v[..., a:b, :])))
        db.append((s.other + (bi,), sv))
    U.blocks = sorted(ub, key=lambda kv: kv[0])
    V.blocks = sorted(vb, key=lambda kv: kv[0])
    d.blocks = sorted(db, key=lambda kv: kv[0])
    return U, d, inverse_cvals(V)


def svd_split(t: BTensor, split: int):
    """svd(A, split), sources/btensor_linalg.cpp:503-534: reshape to a matrix, sector
    SVD, reshape U and V back."""
    rt = reshape(t, [split])
    rU, d, rV = svd(rt)
    Ushape = concat_shapes(shape_keep(t, list(range(split))), shape_keep(rU, [1]))
    Vshape = concat_shapes(shape_keep(t, list(range(split, t.rank)), invert=True), shape_keep(rV, [1]))
    U = reshape_as(rU, Ushape)
    V = reshape_as(rV, Vshape)
    return U, d, V


def compute_last_index(vd: np.ndarray, tol: float, pw: float, min_size: int, max_size: int) -> int:
    """compute_last_index, sources/LinearAlgebra.cpp:57-75 (vd sorted descending)."""
    n = vd.shape[-1]
    toln = float(tol) ** float(pw)
    last = n - 1
    if n == 0:
        return -1
    trunc = abs(vd[last]) ** pw
    while last >= min_size:
        if trunc > toln and last < max_size:
            break
        last -= 1
        trunc += abs(vd[last]) ** pw
    return last


def _remove_unit_blocks(blocks: list, sector: int):
    """remove_unit_blocks lambda, sources/btensor_linalg.cpp:688-709, restated step
    by step (including its handling of consecutive matching blocks)."""
    n = len(blocks)
    src = 0
    dest = 0
    while dest != n:
        dest_last = blocks[dest][0][-1]
        dest += int(dest_last == sector)
        if dest != src and dest != n:
            blocks[dest], blocks[src] = blocks[src], blocks[dest]
        dest += int(dest != n)
        src += 1
    del blocks[len(blocks) - (dest - src):]


def truncate(U: BTensor, d: BTensor, V: Optional[BTensor], max_size: int, min_size: int, tol: float,
             pw: float = 2.0):
    """truncate_impl, sources/btensor_linalg.cpp:658-755.

    All singular values are sorted descending in float64; compute_last_index gives
    the smallest kept value s; every value > s*(1-2*eps(dtype)) is kept, sector by
    sector walking backwards; a sector with nothing kept is erased from d and from
    the unitaries (its section stays, with its old size)."""
    U = U.copy()
    V = V.copy() if V is not None else None
    d = d.copy()
    if d.blocks:
        vd = np.sort(np.concatenate([np.asarray(b, dtype=np.float64).ravel() for _, b in d.blocks]))[::-1]
    else:
        vd = np.zeros(0)
    eps = float(np.finfo(d.dtype).eps)
    li = compute_last_index(vd, tol, pw, min_size, max_size)
    smallest = vd[li] if vd.size else 0.0
    smallest = smallest - 2 * smallest * eps
    # the discarded weight the threshold bounds (sum of dropped |s|^pow), relative to
    # the total: reported by the GPU driver's logger, kept here as an attribute
    allw = np.abs(vd) ** pw
    dropped_rel = float(np.sum(allw[~(vd > smallest)]) / np.sum(allw)) if vd.size and np.sum(allw) > 0 else 0.0
    unitaries = [x for x in (U, V) if x is not None]
    pos = len(d.blocks)
    while pos > 0:
        pos -= 1
        didx, db = d.blocks[pos]
        k = 0
        while k < db.shape[0] and db[k] > smallest:
            k += 1
        sector = didx[-1]
        if k == 0:
            for un in unitaries:
                _remove_unit_blocks(un.blocks, sector)
            del d.blocks[pos]
        else:
            d.blocks[pos] = (didx, db[:k])
            d.ssz[d.addr(d.rank - 1) + sector] = k
            for un in unitaries:
                un.ssz[len(un.ssz) - (len(d.ssz) - sector)] = k
                un.blocks[:] = [(ui, (ub[..., :k] if ui[-1] == sector else ub)) for ui, ub in un.blocks]
    d.discarded_rel = dropped_rel
    return U, d, V


def svd_truncated(t: BTensor, split: int, tol: float, min_size: int, max_size: int, pw: float = 2.0):
    """svd(A, split, tol, min, max, pow), sources/btensor_linalg.cpp:805-809."""
    U, d, V = svd_split(t, split)
    return truncate(U, d, V, max_size, min_size, tol, pw)


def eigh(t: BTensor, upper: bool = True):
    """eigh(btensor), sources/btensor_linalg.cpp:294-368: per sector eigenvalues in
    ascending order and eigenvectors (d, U)."""
    r = t.rank
    secs = compact_dense(t)
    colq = t.sec_charges(r - 1)
    neut = q_neutral(t.mods)
    dq = [colq[s.cols[0][0]] for s in secs]
    dsz = [s.mat.shape[-1] for s in secs]
    lead = list(range(r - 2))
    U = concat_shapes(shape_keep(t, lead + [r - 2]),
                      BTensor(t.mods, [len(secs)], dsz, dq, neut, [], t.dtype))
    # U carries t's selection rule.  (The reference shifts it by the inverse of the
    # first column charge twice, :325-327, so its block() insertion throws unless that
    # charge is neutral; for those inputs both agree.)
    U.sel = t.sel
    d = concat_shapes(shape_keep(t, lead), BTensor(t.mods, [len(secs)], dsz, [neut] * len(secs), neut, [], t.dtype))
    d.cv = [neut for _ in d.cv]
    d.sel = neut
    ub, db = [], []
    for bi, s in enumerate(secs):
        w, v = np.linalg.eigh(s.mat, UPLO="U" if upper else "L")
        for row, a, b in s.rows:
            ub.append((s.other + (row, bi), np.ascontiguousarray(v[..., a:b, :])))
        db.append((s.other + (bi,), w))
    U.blocks = sorted(ub, key=lambda kv: kv[0])
    d.blocks = sorted(db, key=lambda kv: kv[0])
    return d, U


def eigh_split(t: BTensor, split: int):
    """eigh(A, split), sources/btensor_linalg.cpp:369-389."""
    rt = reshape(t, [split])
    d, rU = eigh(rt, True)
    Ushape = concat_shapes(shape_keep(t, list(range(split))), shape_keep(rU, [1]))
    U = reshape_as(rU, Ushape)
    return d, U


# --------------------------------------------------------------------------
# DMRG  (sources/dmrg.cpp)
# --------------------------------------------------------------------------


def compute_2sites_hamil(mpo: List[BTensor]) -> List[BTensor]:
    """compute_2sitesHamil_impl, sources/dmrg.cpp:504-515."""
    return [permute(tensordot(mpo[i], mpo[i + 1], [2], [0]), [0, 1, 3, 4, 2, 5]) for i in range(len(mpo) - 1)]


def hamil2site_times_state(state, hamil, Lenv, Renv) -> BTensor:
    """hamil2site_times_state_impl, sources/dmrg.cpp:521-531."""
    out = tensordot(Lenv, state, [0], [0])
    out = tensordot(out, hamil, [0, 2, 3], [0, 4, 5])
    return tensordot(out, Renv, [1, 4], [0, 1])


def eig2x2(a0: float, a1: float, b: float):
    """eig2x2Mat_impl, sources/dmrg.cpp:544-572 (real scalars)."""
    crit = math.sqrt((a0 - a1) ** 2 + 4 * (b * b))
    E0 = (a0 + a1 - crit) / 2
    delt = E0 - a1
    with np.errstate(all="ignore"):
        o = np.sqrt(np.float64(delt) / np.float64(-crit))
        zero_o = bool((o + E0) == E0) or bool(np.isnan(o))
        n = (b * o) / delt
    if zero_o:
        n = 1.0
        o = 0.0
    if np.isnan(o) or np.isnan(n):
        raise ArithmeticError("nan found in output tensor")
    return float(E0), float(o), float(n)


def one_step_lanczos(state, hamil, Lenv, Renv):
    """one_step_lanczos_impl, sources/dmrg.cpp:585-608."""
    psi = hamil2site_times_state(state, hamil, Lenv, Renv)
    a0 = dot_all(psi, state)
    psi = add_scaled(psi, state, 1.0, -a0)
    b = math.sqrt(dot_all(psi, psi))
    if abs(b) >= 1e-15:
        psi = scale(psi, 1.0 / b)
    a1 = dot_all(psi, hamil2site_times_state(psi, hamil, Lenv, Renv))
    return psi, a0, a1, b


def two_sites_update(state, hamil, Lenv, Renv):
    """two_sites_update_impl, sources/dmrg.cpp:624-638."""
    psi, a0, a1, b = one_step_lanczos(state, hamil, Lenv, Renv)
    E, o, n = eig2x2(a0, a1, b)
    return E, add_scaled(state, psi, o, n)


def compute_left_env(W, A, L):
    """compute_left_env_impl, sources/dmrg.cpp:425-459."""
    out = tensordot(L, A, [0], [0])
    out = tensordot(out, W, [0, 2], [0, 3])
    return tensordot(out, conj(A), [0, 2], [0, 1])


def compute_right_env(W, A, R):
    """compute_right_env_impl, sources/dmrg.cpp:469-493."""
    out = tensordot(R, A, [0], [2])
    out = tensordot(out, W, [0, 3], [2, 3])
    return tensordot(out, conj(A), [3, 0], [1, 2])


def trivial_edge(state_leg: BTensor, mpo_leg: BTensor) -> BTensor:
    """The all-ones rank-3 edge environment (generate_env_impl, sources/dmrg.cpp:371-391;
    edge_shape_prep :335-345) for size-1 edge legs."""
    def leg(t, d):
        return BTensor(t.mods, [t.sbd[d]], t.sec_sizes(d), [q_inv(q, t.mods) for q in t.sec_charges(d)],
                       q_neutral(t.mods), [], t.dtype)
    ls = leg(state_leg[0], state_leg[1])
    lh = leg(mpo_leg[0], mpo_leg[1])
    lsi = inverse_cvals(ls)
    shp = concat_shapes(ls, lh, lsi)
    # selection rule: the sum of the (single-section) edge charges
    q = q_neutral(shp.mods)
    for c in shp.cv:
        q = q_add(q, c, shp.mods)
    shp.sel = q
    return fill(shp, lambda s: np.ones(s))


@dataclass
class DmrgOptions:
    """dmrg_options, include/dmrg_options.h:15-58."""
    cutoff: float = 1e-6
    convergence_criterion: float = 1e-5
    maximum_bond: int = 2**62
    minimum_bond: int = 4
    maximum_iterations: int = 1000


def generate_env(mpo, mps, oc):
    """generate_env_impl, sources/dmrg.cpp:371-409.  Env[-1]..Env[L] stored at i+1."""
    L = len(mpo)
    env: List[Optional[BTensor]] = [None] * (L + 2)
    env[0] = trivial_edge((mps[0], 0), (mpo[0], 0))
    env[L + 1] = trivial_edge((mps[-1], 2), (mpo[-1], 2))
    for i in range(oc):
        env[i + 1] = compute_left_env(mpo[i], mps[i], env[i])
    for i in range(L - 1, oc, -1):
        env[i + 1] = compute_right_env(mpo[i], mps[i], env[i + 2])
    return env


def dmrg_bond_update(mpo, h2, mps, env, oc, forward, opt: DmrgOptions):
    """dmrg_2sites_update::operator(), sources/dmrg.cpp:163-206."""
    theta = tensordot(mps[oc], mps[oc + 1], [2], [0])
    E, theta = two_sites_update(theta, h2[oc], env[oc], env[oc + 3])
    u, d, v = svd_truncated(theta, 2, opt.cutoff, opt.minimum_bond, opt.maximum_bond)
    opt.last_discarded = getattr(d, "discarded_rel", 0.0)
    nrm = math.sqrt(sum(float(np.sum(b ** 2)) for _, b in d.blocks))
    d = scale(d, 1.0 / nrm)
    if forward:
        mps[oc] = u
        mps[oc + 1] = permute(conj(mul_lastleg(v, d)), [2, 0, 1])
        env[oc + 1] = compute_left_env(mpo[oc], mps[oc], env[oc])
    else:
        mps[oc] = mul_lastleg(u, d)
        mps[oc + 1] = permute(conj(v), [2, 0, 1])
        env[oc + 2] = compute_right_env(mpo[oc + 1], mps[oc + 1], env[oc + 3])
    return E


def dmrg(mpo: List[BTensor], mps: List[BTensor], oc: int, opt: DmrgOptions, log=None):
    """details::dmrg_impl (btensor), sources/dmrg.cpp:219-273, with the sweep of
    :128-142.  Mutates ``mps``; returns (E0, oc, per-sweep energies)."""
    L = len(mpo)
    h2 = compute_2sites_hamil(mpo)
    env = generate_env(mpo, mps, oc)
    E0 = 100000.0
    init_pos = oc
    n_step = len(h2) - 1 + (len(h2) == 1)
    step = 1 if oc == 0 else -1
    if len(h2) == 1:
        step = 0
    if oc == L - 1:
        init_pos -= 1
        oc -= 1
    energies = []
    opt.truncated_weights = []
    for it in range(opt.maximum_iterations):
        E = None
        worst = 0.0
        for _ in range(2 * n_step):
            E = dmrg_bond_update(mpo, h2, mps, env, oc, step == 1, opt)
            worst = max(worst, opt.last_discarded)
            oc += step
            if oc == 0 or oc == L - 2:
                step = -step
        energies.append(E)
        opt.truncated_weights.append(worst)
        if log is not None:
            log(it, E, mps)
        prev, E0 = E0, E
        if not (abs((E - prev) / E) > opt.convergence_criterion):
            break
    return E0, oc, energies


# --------------------------------------------------------------------------
# model and state builders (inputs for the parity cases)
# --------------------------------------------------------------------------


def _pauli():
    """pauli(), sources/operators.cpp:52-89."""
    sz = np.array([[1.0, 0.0], [0.0, -1.0]])
    lo = np.array([[0.0, 1.0], [0.0, 0.0]])
    idm = np.eye(2)
    return sz, lo, idm


def heisenberg_dense_w(J: float, delta: float = 1.0) -> np.ndarray:
    """Heisenberg_impl's 5x2x5x2 bulk tensor (sources/models.cpp:38-64) called with
    -J/4 as Heisenberg(J) does (:65-68), so H = -J sum S_i.S_{i+1}; ``delta`` scales
    the S^z S^z channel (XXZ)."""
    Jm = -J / 4.0
    sz, lo, idm = _pauli()
    hi = lo.T
    w = np.zeros((5, 2, 5, 2))
    w[0, :, 0, :] = idm
    w[1, :, 0, :] = lo
    w[2, :, 0, :] = hi
    w[3, :, 0, :] = sz
    w[4, :, 1, :] = 2 * Jm * hi
    w[4, :, 2, :] = 2 * Jm * lo
    w[4, :, 3, :] = Jm * delta * sz
    w[4, :, 4, :] = idm
    return w


def _group_by_charge(q: List[int]):
    """Stable grouping of basis indices by charge: (permutation, [(size, charge)])."""
    order = sorted(range(len(q)), key=lambda i: (q[i], i))
    secs: List[Tuple[int, int]] = []
    for i in order:
        if secs and secs[-1][1] == q[i]:
            secs[-1] = (secs[-1][0] + 1, q[i])
        else:
            secs.append((1, q[i]))
    return order, secs


def dense_mpo_to_block(ws: List[np.ndarray], phys_q: List[int]) -> List[BTensor]:
    """Turn dense MPO tensors W[a, s, b, s'] into U(1) btensors over legs
    (bond, phys, bond^-1, phys^-1).  Bond charges are solved from the nonzero
    entries so that every nonzero element obeys the neutral selection rule, and
    basis states of equal charge are grouped into one section (the section layout
    bMPO::coalesce produces, sources/MPT.cpp:154-168)."""
    bq = [[0] * ws[0].shape[0]]
    for w in ws:
        qa = bq[-1]
        qb: List[Optional[int]] = [None] * w.shape[2]
        for a, s, b, t in zip(*np.nonzero(w)):
            val = qa[a] + phys_q[s] - phys_q[t]
            if qb[b] is None:
                qb[b] = val
            elif qb[b] != val:
                raise ValueError("MPO is not charge conserving")
        bq.append([0 if q is None else q for q in qb])
    porder, psecs = _group_by_charge(phys_q)
    out = []
    for i, w in enumerate(ws):
        lorder, lsecs = _group_by_charge(bq[i])
        rorder, rsecs = _group_by_charge(bq[i + 1])
        wp = w[np.ix_(lorder, porder, rorder, porder)]
        t = btensor([[(n, q) for n, q in lsecs], [(n, q) for n, q in psecs],
                     [(n, -q) for n, q in rsecs], [(n, -q) for n, q in psecs]], [0], (0,))
        offs = [np.concatenate([[0], np.cumsum(t.sec_sizes(d))]).astype(int) for d in range(4)]
        for idx in itertools.product(*[range(n) for n in t.sbd]):
            sl = tuple(slice(offs[d][j], offs[d][j + 1]) for d, j in enumerate(idx))
            blk = wp[sl]
            if np.any(blk != 0.0):
                if not t.allowed(idx):
                    raise ValueError("nonzero MPO element outside the selection rule")
                t.blocks.append((tuple(idx), np.ascontiguousarray(blk)))
        out.append(t)
    return out


def coalesce(mpo: List[BTensor], cutoff: float = 0.0) -> List[BTensor]:
    """bMPO::coalesce, sources/MPT.cpp:154-168: one left-to-right pass of truncating
    SVDs over the right bond of each site, W_i (l, s, r, s') -> (l, s, s', r),
    U d V^H = svd(W_i, 3, cutoff); W_i <- (U d) permuted back, W_(i+1) <- V^H W_(i+1)."""
    out = list(mpo)
    for i in range(len(out) - 1):
        U, d, V = svd_truncated(permute(out[i], [0, 1, 3, 2]), 3, cutoff, 1, 2 ** 62)
        out[i + 1] = tensordot(conj(V), out[i + 1], [0], [0])
        out[i] = permute(mul_lastleg(U, d), [0, 1, 3, 2])
    return out


def mps_overlap(a: List[BTensor], b: List[BTensor]) -> float:
    """contract(bMPS a, bMPS b), sources/MPT.cpp:267-290: a[i] and conj(b[i])
    contracted left to right (real tensors; the edge legs have size one)."""
    env = None
    for x, y in zip(a, b):
        if env is None:
            env = tensordot(x, conj(y), [0, 1], [0, 1])            # (r_a, r_b)
        else:
            t = tensordot(env, x, [0], [0])                         # (r_b, s, r_a)
            env = tensordot(t, conj(y), [0, 1], [0, 1])             # (r_a', r_b')
    return sum(float(np.sum(v)) for _, v in env.blocks)


def heisenberg_mpo(L: int, J: float = -1.0, delta: float = 1.0) -> List[BTensor]:
    """Spin-1/2 Heisenberg (XXZ when delta != 1) chain MPO with U(1) total-2Sz
    charges (physical sections (1, +1), (1, -1) as in tests/DMRG_heisenberg_test.h:25-26)."""
    w = heisenberg_dense_w(J, delta)
    ws = [w[4:5]] + [w] * (L - 2) + [w[:, :, 0:1]]
    return dense_mpo_to_block(ws, [1, -1])


def cap_sectors(mult: Dict[int, int], D: int) -> Dict[int, int]:
    """Cap per-charge multiplicities so that they total at most D: every sector gets
    min(mult, c) for the largest level c that fits, and the remainder goes one by one
    to the sectors that were capped, largest multiplicity first (ties: smaller charge)."""
    if sum(mult.values()) <= D:
        return dict(sorted(mult.items()))
    lo, hi = 0, max(mult.values())
    while lo < hi:
        c = (lo + hi + 1) // 2
        if sum(min(m, c) for m in mult.values()) <= D:
            lo = c
        else:
            hi = c - 1
    dims = {q: min(m, lo) for q, m in mult.items()}
    rem = D - sum(dims.values())
    for q in sorted((q for q, m in mult.items() if m > lo), key=lambda q: (-mult[q], q)):
        if rem == 0:
            break
        dims[q] += 1
        rem -= 1
    return {q: m for q, m in sorted(dims.items()) if m > 0}


def random_mps(L: int, D: int, phys_q: List[int], target: int, rng: np.random.Generator,
               mods=(0,)) -> List[BTensor]:
    """Random normalised U(1) MPS with orthogonality centre at site 0 (oc = 0).

    Bond b (right of site b) carries charges q = target - (sum of physical charges of
    sites <= b) on the right leg of site b and the inverse on the left leg of site
    b+1, the convention of random_bMPS_impl (sources/MPT.cpp:424-462); site 0 holds
    the selection rule.  Sector dimensions are the Hilbert-space multiplicities
    capped so the bond totals at most D (largest sectors trimmed first)."""
    phys_q = list(phys_q)
    # reachable charge multiplicities of the left and right parts
    left = [{0: 1}]
    for i in range(L):
        nxt: Dict[int, int] = {}
        for q, m in left[-1].items():
            for p in phys_q:
                nxt[q + p] = nxt.get(q + p, 0) + m
        left.append(nxt)
    right = [{0: 1}]
    for i in range(L):
        nxt = {}
        for q, m in right[-1].items():
            for p in phys_q:
                nxt[q + p] = nxt.get(q + p, 0) + m
        right.append(nxt)
    bonds = []  # bond b in 0..L-2 : dict partial_sum -> dim
    for b in range(L - 1):
        nl = b + 1
        nr = L - nl
        dims = {}
        for q, m in left[nl].items():
            mr = right[nr].get(target - q, 0)
            if mr:
                dims[q] = min(m, mr)
        bonds.append(cap_sectors(dims, D))
    mps = []
    for i in range(L):
        if i == 0:
            lleg = [(1, 0)]
        else:
            lleg = [(m, q - target) for q, m in bonds[i - 1].items()]
        if i == L - 1:
            rleg = [(1, 0)]
        else:
            rleg = [(m, target - q) for q, m in bonds[i].items()]
        sel = target if i == 0 else 0
        t = btensor([lleg, [(n, q) for n, q in _group_by_charge(phys_q)[1]], rleg], [sel], mods)
        t = randn_like(t, rng)
        nrm = math.sqrt(sum(float(np.sum(b ** 2)) for _, b in t.blocks))
        t = scale(t, 1.0 / nrm)
        mps.append(t)
    return mps


def right_canonicalize(mps: List[BTensor]) -> List[BTensor]:
    """Bring a MPS to right-canonical form with the orthogonality centre on site 0
    and unit norm (what bMPS::move_oc(0) does, sources/MPT.cpp:75-111), with
    untruncated sector SVDs."""
    mps = [m.copy() for m in mps]
    for i in range(len(mps) - 1, 0, -1):
        U, d, V = svd_split(mps[i], 1)
        mps[i] = permute(conj(V), [2, 0, 1])
        mps[i - 1] = tensordot(mps[i - 1], mul_lastleg(U, d), [2], [0])
    nrm = math.sqrt(sum(float(np.sum(b ** 2)) for _, b in mps[0].blocks))
    mps[0] = scale(mps[0], 1.0 / nrm)
    return mps


def mps_norm2(mps: List[BTensor]) -> float:
    """<psi|psi> by contracting the chain from the left (contract(bMPS,bMPS), sources/MPT.cpp:211-290)."""
    env = None
    for A in mps:
        if env is None:
            env = tensordot(A, conj(A), [0, 1], [0, 1])
        else:
            tmp = tensordot(env, A, [0], [0])
            env = tensordot(tmp, conj(A), [0, 1], [0, 1])
    return float(sum(np.sum(b) for _, b in env.blocks))


def mps_energy(mpo: List[BTensor], mps: List[BTensor]) -> float:
    """<psi|H|psi> through the left environments."""
    env = trivial_edge((mps[0], 0), (mpo[0], 0))
    for W, A in zip(mpo, mps):
        env = compute_left_env(W, A, env)
    return float(sum(np.sum(b) for _, b in env.blocks))


# --------------------------------------------------------------------------
# block-list files written by quantit_gb300.serialize (np.savez archives), read
# into oracle tensors so the CPU checks and baselines run on the GPU path's states
# --------------------------------------------------------------------------


def from_arrays(d) -> BTensor:
    """One tensor from its arrays: sbd, ssz, cv [nsec][ncomp], sel, mods, bidx
    [nblocks][rank] (block-list order) and data (the blocks concatenated)."""
    mods = tuple(int(m) for m in np.asarray(d["mods"]).reshape(-1))
    nc = len(mods)

    def charge(vals):
        return tuple((int(v) & 0xFFFF) if m else int(v) for v, m in zip(vals, mods))
    sbd = [int(x) for x in np.asarray(d["sbd"]).reshape(-1)]
    ssz = [int(x) for x in np.asarray(d["ssz"]).reshape(-1)]
    cv = [charge(row) for row in np.asarray(d["cv"]).reshape(-1, nc)] if ssz else []
    t = BTensor(mods, sbd, ssz, cv, charge(np.asarray(d["sel"]).reshape(-1)), [], np.float64)
    bidx = np.asarray(d["bidx"]).reshape(-1, max(len(sbd), 1)) if len(sbd) else np.zeros((0, 0), int)
    data = np.asarray(d["data"], dtype=np.float64) if "data" in d else None
    off = 0
    for row in bidx:
        idx = tuple(int(x) for x in row)
        shp = t.block_shape(idx)
        n = int(np.prod(shp)) if shp else 1
        t.blocks.append((idx, None if data is None else data[off:off + n].reshape(shp).copy()))
        off += n
    return t


def load_npz(path):
    """(kind, tensors, oc) of a file written by quantit_gb300.serialize.save."""
    with np.load(path, allow_pickle=False) as z:
        kind, n, oc = str(z["kind"]), int(z["count"]), int(z["oc"])
        out = []
        for i in range(n):
            pre = f"t{i}_"
            out.append(from_arrays({k[len(pre):]: z[k] for k in z.files if k.startswith(pre)}))
    return kind, out, oc

