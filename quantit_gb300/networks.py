"""MPS / MPO containers and builders feeding the DMRG path.

``bMPO`` / ``bMPS`` are lists of btensor handles (QuantiT's bMPO / bMPS,
include/MPT.h:487-701); ``bMPS.orthogonality_center`` is the centre position.
Builders:
  * ``heisenberg`` / ``xxz``: the 5x2x5x2 Heisenberg_impl MPO (sources/models.cpp:38-68)
    with U(1) total-2Sz charges, H = -J sum S.S (so J=-1 is the antiferromagnet),
    ``delta`` scaling the S^z S^z channel;
  * ``random_bmps``: seeded N(0,1) MPS whose bond sectors are the charge
    multiplicities capped to D;
  * ``bMPS.move_oc``: sector-SVD sweep moving the orthogonality centre
    (bMPS::move_oc, sources/MPT.cpp:75-111), on the GPU.
"""
import itertools
import math

import numpy as np

from . import linalg
from .conserved import Z
from .tensor import btensor, dot_all, from_blocks


class bMPO(list):
    pass


class bMPS(list):
    def __init__(self, tensors=(), orthogonality_center=0):
        super().__init__(tensors)
        self.orthogonality_center = orthogonality_center

    @property
    def oc(self):
        return self.orthogonality_center

    def move_oc(self, pos):
        """Move the orthogonality centre to ``pos`` with untruncated sector SVDs."""
        while self.orthogonality_center > pos:
            i = self.orthogonality_center
            U, d, V = linalg.svd(self[i], 1)                    # A_i = U d V^H
            self[i] = V.conj().permute([2, 0, 1])               # [k, s, r]
            self[i - 1] = self[i - 1].tensordot(U.mul(d), ([2], [0]))
            self.orthogonality_center = i - 1
        while self.orthogonality_center < pos:
            i = self.orthogonality_center
            U, d, V = linalg.svd(self[i], 2)                    # V: [r, k]
            self[i] = U
            dvh = V.mul(d).conj().permute([1, 0])               # [k, r]
            self[i + 1] = dvh.tensordot(self[i + 1], ([1], [0]))
            self.orthogonality_center = i + 1
        return self

    def normalize_center(self):
        c = self.orthogonality_center
        n = math.sqrt(dot_all(self[c], self[c]))
        self[c] = self[c] * (1.0 / n)
        return self


def _group_by_charge(q):
    order = sorted(range(len(q)), key=lambda i: (q[i], i))
    secs = []
    for i in order:
        if secs and secs[-1][1] == q[i]:
            secs[-1] = (secs[-1][0] + 1, q[i])
        else:
            secs.append((1, q[i]))
    return order, secs


def heisenberg_dense(J=-1.0, delta=1.0):
    """Bulk W[a, s, b, s'] of Heisenberg_impl(-J/4) (sources/models.cpp:38-68)."""
    Jm = -J / 4.0
    sz = np.array([[1.0, 0.0], [0.0, -1.0]])
    lo = np.array([[0.0, 1.0], [0.0, 0.0]])
    hi = lo.T
    idm = np.eye(2)
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


def dense_mpo_to_bmpo(ws, phys_q):
    """U(1) block MPO from dense site tensors: bond charges solved from the nonzero
    elements, equal charges grouped into one section (the layout of bMPO::coalesce)."""
    bq = [[0] * ws[0].shape[0]]
    for w in ws:
        qa = bq[-1]
        qb = [None] * w.shape[2]
        for a, s, b, t in zip(*np.nonzero(w)):
            v = qa[a] + phys_q[s] - phys_q[t]
            if qb[b] is None:
                qb[b] = v
            elif qb[b] != v:
                raise ValueError("MPO is not charge conserving")
        bq.append([0 if q is None else q for q in qb])
    porder, psecs = _group_by_charge(phys_q)
    out = bMPO()
    for i, w in enumerate(ws):
        lorder, lsecs = _group_by_charge(bq[i])
        rorder, rsecs = _group_by_charge(bq[i + 1])
        wp = w[np.ix_(lorder, porder, rorder, porder)]
        legs = [[(n, Z(q)) for n, q in lsecs], [(n, Z(q)) for n, q in psecs],
                [(n, Z(-q)) for n, q in rsecs], [(n, Z(-q)) for n, q in psecs]]
        sizes = [[n for n, _ in l] for l in legs]
        charges = [[q.values[0] for _, q in l] for l in legs]
        offs = [np.concatenate([[0], np.cumsum(s)]).astype(int) for s in sizes]
        blocks = []
        for idx in itertools.product(*[range(len(s)) for s in sizes]):
            sl = tuple(slice(offs[d][j], offs[d][j + 1]) for d, j in enumerate(idx))
            blk = wp[sl]
            if np.any(blk != 0.0):
                if sum(charges[d][j] for d, j in enumerate(idx)) != 0:
                    raise ValueError("nonzero MPO element outside the selection rule")
                blocks.append((idx, np.ascontiguousarray(blk)))
        out.append(from_blocks(legs, Z(0), blocks))
    return out


def heisenberg(L, J=-1.0, delta=1.0):
    """Open spin-1/2 Heisenberg (XXZ for delta != 1) chain with U(1) total-2Sz charges."""
    w = heisenberg_dense(J, delta)
    ws = [w[4:5]] + [w] * (L - 2) + [w[:, :, 0:1]]
    return dense_mpo_to_bmpo(ws, [1, -1])


def xxz(L, delta, J=-1.0):
    return heisenberg(L, J=J, delta=delta)


def cap_sectors(mult, D):
    """Cap per-charge multiplicities to a total of at most D (water filling; the
    remainder goes to the largest capped sectors first, ties to the smaller charge)."""
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


def bond_sectors(L, D, phys_q, target):
    """Sector dimensions of every bond: dict partial charge -> dimension."""
    left = [{0: 1}]
    for _ in range(L):
        nxt = {}
        for q, m in left[-1].items():
            for p in phys_q:
                nxt[q + p] = nxt.get(q + p, 0) + m
        left.append(nxt)
    bonds = []
    for b in range(L - 1):
        nl, nr = b + 1, L - b - 1
        dims = {}
        for q, m in left[nl].items():
            mr = left[nr].get(target - q, 0)
            if mr:
                dims[q] = min(m, mr)
        bonds.append(cap_sectors(dims, D))
    return bonds


def random_bmps(L, D, phys_q=(1, -1), target=0, seed=0):
    """Seeded random U(1) MPS in the manner of random_bMPS (sources/MPT.cpp:424-460):
    N(0,1) blocks, every site tensor scaled to unit Frobenius norm, no canonical
    form (so the environments of a long chain shrink geometrically; the FP64 path
    and the mixed path's power-of-two operand scaling both handle that).  The
    orthogonality centre is recorded as the last site, where a sweep starts."""
    rng = np.random.default_rng(seed)
    bonds = bond_sectors(L, D, list(phys_q), target)
    _, psecs = _group_by_charge(list(phys_q))
    mps = bMPS(orthogonality_center=L - 1)
    for i in range(L):
        lleg = [(1, Z(0))] if i == 0 else [(m, Z(q - target)) for q, m in bonds[i - 1].items()]
        rleg = [(1, Z(0))] if i == L - 1 else [(m, Z(target - q)) for q, m in bonds[i].items()]
        legs = [lleg, [(n, Z(q)) for n, q in psecs], rleg]
        sel = target if i == 0 else 0
        blocks = []
        lq = [q.values[0] for _, q in lleg]
        pq = [q for _, q in psecs]
        rq = [q.values[0] for _, q in rleg]
        for a, s, b in itertools.product(range(len(lleg)), range(len(psecs)), range(len(rleg))):
            if lq[a] + pq[s] + rq[b] == sel:
                shp = (lleg[a][0], psecs[s][0], rleg[b][0])
                blocks.append(((a, s, b), rng.standard_normal(shp)))
        nrm = math.sqrt(sum(float(np.sum(v ** 2)) for _, v in blocks))
        blocks = [(k, v / nrm) for k, v in blocks]
        mps.append(from_blocks(legs, Z(sel), blocks))
    return mps
