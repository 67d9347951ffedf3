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
from .conserved import Z, quantity
from .tensor import btensor, dot_all, from_blocks


class bMPO(list):
    def coalesce(self, cutoff=0.0):
        """bMPO::coalesce (sources/MPT.cpp:154-168): one left-to-right pass of
        truncating sector SVDs over each site's right bond, W_i(l, s, r, s') viewed as
        the (l s s') x r matrix, U d V^H = svd(W_i, 3, cutoff); W_i <- U d and the next
        site absorbs V^H.  Linearly dependent MPO channels vanish, so the bond
        dimension drops to the operator's rank seen from the left.  On the GPU."""
        for i in range(len(self) - 1):
            U, d, V = linalg.svd(self[i].permute([0, 1, 3, 2]), 3, float(cutoff))
            self[i + 1] = V.conj().tensordot(self[i + 1], ([0], [0]))
            self[i] = U.mul(d).permute([0, 1, 3, 2])
        return self

    def mirrored(self):
        """The same operator on the reversed chain: site order reversed and each
        W(l, s, r, s') -> W(r, s, l, s')."""
        return bMPO([w.permute([2, 1, 0, 3]) for w in reversed(self)])

    def compress(self, cutoff=1e-13):
        """coalesce in both directions (no counterpart in QuantiT, whose coalesce is
        the left-to-right pass only): the right-to-left pass removes the channels
        that are dependent seen from the right, so each bond dimension drops to the
        operator's Schmidt rank at that cut (35 -> 20 for the 12 x 6 snake cylinder).
        A cutoff > 0 drops the numerically zero singular values the first pass leaves."""
        self.coalesce(cutoff)
        self[:] = self.mirrored().coalesce(cutoff).mirrored()
        return self


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


class _Charges:
    """Charge arithmetic on plain tuples for one group (moduli: 0 = U(1), n = Z(n));
    plain ints are the one-component U(1) case."""

    def __init__(self, mods=(0,)):
        self.mods = tuple(int(m) for m in mods)

    def norm(self, c):
        c = (c,) if isinstance(c, (int, np.integer)) else tuple(c)
        if len(c) != len(self.mods):
            raise ValueError("charge with the wrong number of components")
        return tuple((int(v) % m) if m else int(v) for v, m in zip(c, self.mods))

    def add(self, a, b):
        return self.norm(tuple(x + y for x, y in zip(a, b)))

    def neg(self, a):
        return self.norm(tuple(-x for x in a))

    def zero(self):
        return tuple(0 for _ in self.mods)

    def q(self, c):
        return quantity(c, self.mods)


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


def fermions():
    """(c_up, c_dn, F, id) on the basis {empty, up, down, up+down} (fermions(),
    sources/operators.cpp:21-39; the down operator carries the on-site sign)."""
    c_up = np.zeros((4, 4))
    c_dn = np.zeros((4, 4))
    c_up[0, 1] = 1.0
    c_up[2, 3] = 1.0
    c_dn[0, 2] = 1.0
    c_dn[1, 3] = -1.0
    F = np.diag([1.0, -1.0, -1.0, 1.0])
    return c_up, c_dn, F, np.eye(4)


def hubbard_dense(U, mu):
    """Bulk W[a, s, b, s'] of Hubbard(U, mu, L) (sources/models.cpp:118-148): the
    6x4x6x4 operator matrix with hopping channels c^dg F, F c and the on-site term
    U n_up n_dn - mu (n_up + n_dn)."""
    c_up, c_dn, F, idm = fermions()
    n_up = c_up.T @ c_up
    n_dn = c_dn.T @ c_dn
    w = np.zeros((6, 4, 6, 4))
    w[0, :, 0, :] = idm
    w[1, :, 0, :] = c_up
    w[2, :, 0, :] = c_dn
    w[3, :, 0, :] = c_up.T
    w[4, :, 0, :] = c_dn.T
    w[5, :, 0, :] = U * (n_up @ n_dn) - mu * (n_up + n_dn)
    w[5, :, 1, :] = c_up.T @ F
    w[5, :, 2, :] = c_dn.T @ F
    w[5, :, 3, :] = F @ c_up
    w[5, :, 4, :] = F @ c_dn
    w[5, :, 5, :] = idm
    return w


# physical charges (N, 2 Sz) of the Hubbard basis {empty, up, down, up+down}
HUBBARD_PHYS = [(0, 0), (1, 1), (1, -1), (2, 0)]


def dense_mpo_to_bmpo(ws, phys_q, mods=(0,)):
    """Block MPO from dense site tensors: bond charges solved from the nonzero
    elements, equal charges grouped into one section (the layout of bMPO::coalesce).
    Charges are ints (U(1)) or tuples of the group given by ``mods``."""
    G = _Charges(mods)
    pq = [G.norm(c) for c in phys_q]
    bq = [[G.zero()] * ws[0].shape[0]]
    for w in ws:
        qa = bq[-1]
        qb = [None] * w.shape[2]
        for a, s, b, t in zip(*np.nonzero(w)):
            v = G.add(G.add(qa[a], pq[s]), G.neg(pq[t]))
            if qb[b] is None:
                qb[b] = v
            elif qb[b] != v:
                raise ValueError("MPO is not charge conserving")
        bq.append([G.zero() if q is None else q for q in qb])
    porder, psecs = _group_by_charge(pq)
    out = bMPO()
    for i, w in enumerate(ws):
        lorder, lsecs = _group_by_charge(bq[i])
        rorder, rsecs = _group_by_charge(bq[i + 1])
        wp = w[np.ix_(lorder, porder, rorder, porder)]
        charges = [[q for _, q in lsecs], [q for _, q in psecs], [G.neg(q) for _, q in rsecs],
                   [G.neg(q) for _, q in psecs]]
        sizes = [[n for n, _ in l] for l in (lsecs, psecs, rsecs, psecs)]
        legs = [[(n, G.q(c)) for n, c in zip(sz, ch)] for sz, ch in zip(sizes, charges)]
        offs = [np.concatenate([[0], np.cumsum(sz)]).astype(int) for sz in sizes]
        blocks = []
        for idx in itertools.product(*[range(len(sz)) for sz in sizes]):
            sl = tuple(slice(offs[d][j], offs[d][j + 1]) for d, j in enumerate(idx))
            blk = wp[sl]
            if np.any(blk != 0.0):
                tot = G.zero()
                for d, j in enumerate(idx):
                    tot = G.add(tot, charges[d][j])
                if tot != G.zero():
                    raise ValueError("nonzero MPO element outside the selection rule")
                blocks.append((idx, np.ascontiguousarray(blk)))
        out.append(from_blocks(legs, G.q(G.zero()), blocks))
    return out


def _edge_eye(a, la, b, lb):
    """eye_like(shape_from(a's leg la).inverse_cvals_(), shape_from(b's leg lb)):
    the identity between leg la of a (charges inverted) and leg lb of b, on the
    sections whose charges match (the edges of sources/MPT.cpp:279-290)."""
    def leg(t, d):
        sbd, ssz, cv, _ = t.structure()
        start = sum(sbd[:d])
        return list(ssz[start:start + sbd[d]]), list(cv[start:start + sbd[d]])
    na, qa = leg(a, la)
    nb, qb = leg(b, lb)
    e = btensor([[(n, q.inv()) for n, q in zip(na, qa)], [(n, q) for n, q in zip(nb, qb)]], qb[0].neutral())
    blocks = [((i, j), np.eye(na[i], nb[j])) for i in range(len(na)) for j in range(len(nb)) if qa[i] == qb[j]]
    return e.set_blocks(blocks)


def contract(a, b, left_edge=None, right_edge=None):
    """contract(bMPS a, bMPS b[, left_edge, right_edge]) (include/MPT.h:726-727,
    sources/MPT.cpp:267-290): the scalar sum over a[i] and conj(b[i]) contracted
    left to right through the edges (identities on the outer legs by default), as
    a rank-0 btensor.  On the GPU."""
    if len(a) != len(b):
        raise ValueError("contract needs two MPS of the same length")
    E = left_edge if left_edge is not None else _edge_eye(a[0], 0, b[0], 0)
    R = right_edge if right_edge is not None else _edge_eye(a[-1], 2, b[-1], 2)
    for x, y in zip(a, b):
        E = E.tensordot(x, ([0], [0]))
        E = E.tensordot(y.conj(), ([0, 1], [0, 1]))
    return E.tensordot(R, ([0, 1], [0, 1]))


def random_bMPS(bond_dim, mpo, constraint, seed=0):
    """random_bMPS(bond_dim, mpo, constraint, seed) (include/MPT.h:49-53,
    sources/MPT.cpp:424-462) built on the GPU: physical legs from the MPO, total
    charge ``constraint`` (a quantity of the MPO's group), bond sectors capped to
    ``bond_dim``, N(0, 1) entries from a counter-based generator, unit-norm sites.
    The orthogonality centre is the last site."""
    import ctypes as C
    from . import _lib
    L = len(mpo)
    hs = (C.c_void_p * L)(*[t._h.value for t in mpo])
    vals = constraint.values if hasattr(constraint, "values") else tuple(constraint)
    cq = (C.c_int16 * max(len(vals), 1))(*[((int(v) + 32768) % 65536) - 32768 for v in vals])
    out = (C.c_void_p * L)()
    _lib.call("qtt_random_mps", L, hs, int(bond_dim), cq, C.c_uint64(int(seed) & (2 ** 64 - 1)), out)
    return bMPS([btensor._wrap(C.c_void_p(out[i])) for i in range(L)], L - 1)


def heisenberg(L, J=-1.0, delta=1.0):
    """Open spin-1/2 Heisenberg (XXZ for delta != 1) chain with U(1) total-2Sz charges."""
    w = heisenberg_dense(J, delta)
    ws = [w[4:5]] + [w] * (L - 2) + [w[:, :, 0:1]]
    return dense_mpo_to_bmpo(ws, [1, -1])


def xxz(L, delta, J=-1.0):
    return heisenberg(L, J=J, delta=delta)


def hubbard(L, U, mu=0.0):
    """Open Fermi-Hubbard chain (Hubbard(U, mu, L, shape), sources/models.cpp:118-172)
    with U(1)xU(1) charges (N, 2 Sz) on the physical basis {empty, up, down, up+down}."""
    w = hubbard_dense(U, mu)
    ws = [w[5:6]] + [w] * (L - 2) + [w[:, :, 0:1]]
    return dense_mpo_to_bmpo(ws, HUBBARD_PHYS, mods=(0, 0))


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


def bond_sectors(L, D, phys_q, target, mods=(0,)):
    """Sector dimensions of every bond: dict partial charge -> dimension."""
    G = _Charges(mods)
    pq = [G.norm(c) for c in phys_q]
    tg = G.norm(target)
    left = [{G.zero(): 1}]
    for _ in range(L):
        nxt = {}
        for q, m in left[-1].items():
            for p in pq:
                k = G.add(q, p)
                nxt[k] = nxt.get(k, 0) + m
        left.append(nxt)
    bonds = []
    for b in range(L - 1):
        nl, nr = b + 1, L - b - 1
        dims = {}
        for q, m in left[nl].items():
            mr = left[nr].get(G.add(tg, G.neg(q)), 0)
            if mr:
                dims[q] = min(m, mr)
        capped = cap_sectors(dims, D)
        bonds.append(capped if len(mods) > 1 or mods[0] else {k[0]: v for k, v in capped.items()})
    return bonds


def random_bmps(L, D, phys_q=(1, -1), target=0, seed=0, mods=(0,)):
    """Seeded random MPS in the manner of random_bMPS (sources/MPT.cpp:424-460):
    N(0,1) blocks, every site tensor scaled to unit Frobenius norm, no canonical
    form (so the environments of a long chain shrink geometrically; the FP64 path
    and the mixed path's power-of-two operand scaling both handle that).  The
    orthogonality centre is recorded as the last site, where a sweep starts.
    Charges are ints (U(1)) or tuples of the group given by ``mods``."""
    G = _Charges(mods)
    rng = np.random.default_rng(seed)
    bonds = [{G.norm(k): v for k, v in b.items()} for b in bond_sectors(L, D, phys_q, target, mods)]
    pq = [G.norm(c) for c in phys_q]
    tg = G.norm(target)
    _, psecs = _group_by_charge(pq)
    zero = G.zero()
    mps = bMPS(orthogonality_center=L - 1)
    for i in range(L):
        lq = [zero] if i == 0 else [G.add(q, G.neg(tg)) for q in bonds[i - 1]]
        lm = [1] if i == 0 else list(bonds[i - 1].values())
        rq = [zero] if i == L - 1 else [G.add(tg, G.neg(q)) for q in bonds[i]]
        rm = [1] if i == L - 1 else list(bonds[i].values())
        sel = tg if i == 0 else zero
        legs = [[(m, G.q(c)) for m, c in zip(lm, lq)], [(n, G.q(c)) for n, c in psecs],
                [(m, G.q(c)) for m, c in zip(rm, rq)]]
        blocks = []
        for a, s_, b in itertools.product(range(len(lq)), range(len(psecs)), range(len(rq))):
            if G.add(G.add(lq[a], psecs[s_][1]), rq[b]) == sel:
                shp = (lm[a], psecs[s_][0], rm[b])
                blocks.append(((a, s_, b), rng.standard_normal(shp)))
        nrm = math.sqrt(sum(float(np.sum(v ** 2)) for _, v in blocks))
        blocks = [(k, v / nrm) for k, v in blocks]
        mps.append(from_blocks(legs, G.q(sel), blocks))
    return mps


def gaussian_sections(D, qmax=8, sigma=3.0):
    """Section sizes over charges -qmax..qmax from a Gaussian of width sigma,
    rounded by largest remainders so that they sum to exactly D."""
    qs = np.arange(-qmax, qmax + 1)
    w = np.exp(-qs.astype(float) ** 2 / (2.0 * sigma * sigma))
    raw = D * w / w.sum()
    sizes = np.floor(raw).astype(int)
    for i in np.argsort(-(raw - sizes), kind="stable")[:D - int(sizes.sum())]:
        sizes[i] += 1
    return [(int(n), int(q)) for n, q in zip(sizes, qs) if n > 0]


def theta_pair(D, seed=0, qmax=8, sigma=3.0):
    """The synthetic contraction operands: A[a, s, t, b] and B[b, t', u, c] with
    bond legs of total D over U(1) charges -qmax..qmax (Gaussian section sizes),
    spin-1/2 physical legs and N(0, 1) entries; A's legs (t, b) contract with B's
    (t', b).  Returns (A, B)."""
    rng = np.random.default_rng(seed)
    bond = gaussian_sections(D, qmax, sigma)
    phys = [(1, 1), (1, -1)]

    def make(legs):
        t = btensor([[(n, Z(q)) for n, q in leg] for leg in legs], Z(0))
        charges = [[q for _, q in leg] for leg in legs]
        sizes = [[n for n, _ in leg] for leg in legs]
        blocks = []
        for idx in itertools.product(*[range(len(c)) for c in charges]):
            if sum(charges[d][j] for d, j in enumerate(idx)) == 0:
                shp = tuple(sizes[d][j] for d, j in enumerate(idx))
                blocks.append((idx, rng.standard_normal(shp)))
        t.set_blocks(blocks)
        return t

    A = make([bond, phys, phys, [(n, -q) for n, q in bond]])
    B = make([bond, [(n, -q) for n, q in phys], phys, [(n, -q) for n, q in bond]])
    return A, B


def heisenberg_couplings_dense(L, couplings):
    """Dense site tensors W_i[a, s, b, s'] of H = sum_(i<j) J_ij S_i.S_j for arbitrary
    pair couplings, as a finite-state automaton on the spin-1/2 basis {up, down}
    (the local layout of Heisenberg_impl, sources/models.cpp:38-68: the left edge
    takes the last row, the right edge the first column).  States: 0 = every term
    finished; 1 + 3 (d - 1) + o = operator o in (S+, S-, Sz) placed d sites to the
    left (d = 1 .. the longest coupling); last = nothing placed yet.  A coupling
    J_ij is placed as S_i^o at site i and closed with its partner at site j."""
    pairs = {}
    dmax = 0
    for i, j, J in couplings:
        i, j = int(min(i, j)), int(max(i, j))
        if i == j or not (0 <= i < L and 0 <= j < L):
            raise ValueError("couplings need two different sites of the chain")
        pairs[(i, j)] = pairs.get((i, j), 0.0) + float(J)
        dmax = max(dmax, j - i)
    sp = np.array([[0.0, 1.0], [0.0, 0.0]])   # S+ on (up, down)
    sm = sp.T
    sz = np.diag([0.5, -0.5])
    idm = np.eye(2)
    ops = (sp, sm, sz)
    partner = (0.5 * sm, 0.5 * sp, sz)        # S.S = (S+S- + S-S+)/2 + SzSz
    n = 2 + 3 * dmax
    start = n - 1
    ws = []
    for k in range(L):
        w = np.zeros((n, 2, n, 2))
        w[0, :, 0, :] = idm
        w[start, :, start, :] = idm
        if any(i == k for (i, j) in pairs):
            for o in range(3):
                w[start, :, 1 + o, :] = ops[o]
        for d in range(1, dmax + 1):
            for o in range(3):
                a = 1 + 3 * (d - 1) + o
                if d < dmax:
                    w[a, :, a + 3, :] = idm
                J = pairs.get((k - d, k))
                if J:
                    w[a, :, 0, :] = J * partner[o]
        ws.append(w)
    ws[0] = ws[0][start:start + 1]
    ws[-1] = ws[-1][:, :, 0:1]
    return ws


def heisenberg_couplings(L, couplings):
    """Block MPO (U(1) 2Sz charges) of heisenberg_couplings_dense."""
    return dense_mpo_to_bmpo(heisenberg_couplings_dense(L, couplings), [1, -1])


def cylinder_sites(Lx, Ly, order="snake"):
    """Chain position of lattice site (x, y) of an Lx (open) x Ly (periodic) cylinder:
    column by column, every other column reversed for ``snake``."""
    pos = {}
    for x in range(Lx):
        for y in range(Ly):
            yy = (Ly - 1 - y) if (order == "snake" and x % 2) else y
            pos[(x, y)] = x * Ly + yy
    return pos


def cylinder_couplings(Lx, Ly, J=1.0, order="snake"):
    """Nearest-neighbour pairs of the Lx x Ly cylinder (periodic around Ly) as chain
    couplings (i, j, J)."""
    pos = cylinder_sites(Lx, Ly, order)
    out = set()
    for x in range(Lx):
        for y in range(Ly):
            a = pos[(x, y)]
            nbrs = [(x, (y + 1) % Ly)] + ([(x + 1, y)] if x + 1 < Lx else [])
            for nb in nbrs:
                b = pos[nb]
                if a != b:
                    out.add((min(a, b), max(a, b)))
    return [(i, j, J) for i, j in sorted(out)]


def cylinder_heisenberg(Lx, Ly, J=1.0, order="snake", compress=False):
    """Spin-1/2 Heisenberg model on an Lx x Ly open cylinder, H = J sum_<ij> S_i.S_j.
    With compress, the automaton MPO is compressed in both directions to the
    operator's Schmidt rank (bMPO.compress)."""
    mpo = heisenberg_couplings(Lx * Ly, cylinder_couplings(Lx, Ly, J, order))
    return mpo.compress() if compress else mpo
