"""Model MPO builders on the CPU: the dense Hubbard site tensor (the operator
matrix of sources/models.cpp:118-148 with fermions() of sources/operators.cpp:21-39)
contracted into the full Hamiltonian of a short chain has the spectrum of an
independently built Jordan-Wigner Hubbard Hamiltonian in every (N, 2Sz) sector,
and the product-charge bond sectors respect the target charge."""
import itertools

import numpy as np
import pytest

from quantit_gb300 import networks


def _mpo_matrix(ws):
    """Dense H from W[a, s, b, s'] site tensors (left edge row, right edge column)."""
    T = ws[0][0]  # [s, b, s']
    d = T.shape[0]
    H = T.transpose(1, 0, 2)  # [b, s, s']
    for w in ws[1:]:
        # H[b, S, S'] x w[b, s, c, s'] -> [c, S s, S' s']
        H = np.einsum("bxy,bscz->cxsyz", H, w)
        n = H.shape[1] * H.shape[2]
        H = H.reshape(H.shape[0], n, n)
    assert H.shape[0] == 1
    return H[0]


def _jordan_wigner_hubbard(L, U, mu, t=1.0):
    """H = -t sum_{i,sigma} (a+_{i s} a_{i+1 s} + h.c.) + U sum n_up n_dn - mu N on
    modes ordered (site, up), (site, down), in the site basis {0, up, down, up+down}."""
    nm = 2 * L
    dim = 4 ** L
    # occupation bits of every basis state: site i digit v -> (up = v in (1,3), down = v in (2,3))
    occ = np.zeros((dim, nm), dtype=int)
    for idx in range(dim):
        digits = np.base_repr(idx, 4).zfill(L) if L else ""
        for i, ch in enumerate(digits):
            v = int(ch)
            occ[idx, 2 * i] = 1 if v in (1, 3) else 0
            occ[idx, 2 * i + 1] = 1 if v in (2, 3) else 0
    index = {tuple(o): k for k, o in enumerate(occ)}

    def annihilate(mode):
        A = np.zeros((dim, dim))
        for k in range(dim):
            if occ[k, mode]:
                o = occ[k].copy()
                sign = (-1) ** int(np.sum(o[:mode]))
                o[mode] = 0
                A[index[tuple(o)], k] = sign
        return A

    a = [annihilate(m) for m in range(nm)]
    n = [x.T @ x for x in a]
    H = np.zeros((dim, dim))
    for i in range(L - 1):
        for s in range(2):
            h = a[2 * i + s].T @ a[2 * (i + 1) + s]
            H -= t * (h + h.T)
    for i in range(L):
        H += U * n[2 * i] @ n[2 * i + 1] - mu * (n[2 * i] + n[2 * i + 1])
    N = np.sum(occ, axis=1)
    Sz2 = np.sum(occ[:, 0::2], axis=1) - np.sum(occ[:, 1::2], axis=1)
    return H, N, Sz2


@pytest.mark.parametrize("L, U, mu", [(2, 8.0, 0.0), (3, 4.0, 0.5), (4, 8.0, 0.0)])
def test_hubbard_mpo_spectrum_matches_jordan_wigner(L, U, mu):
    w = networks.hubbard_dense(U, mu)
    ws = [w[5:6]] + [w] * (L - 2) + [w[:, :, 0:1]]
    Hm = _mpo_matrix(ws)
    assert np.allclose(Hm, Hm.T)
    Hj, N, Sz2 = _jordan_wigner_hubbard(L, U, mu)
    # the MPO basis is the product of site digits: same state labels, so compare per sector
    for n in range(0, 2 * L + 1):
        for sz in range(-n, n + 1, 2):
            sel = np.where((N == n) & (Sz2 == sz))[0]
            if sel.size == 0:
                continue
            em = np.linalg.eigvalsh(Hm[np.ix_(sel, sel)])
            ej = np.linalg.eigvalsh(Hj[np.ix_(sel, sel)])
            np.testing.assert_allclose(em, ej, atol=1e-12)
            # the MPO conserves both charges: no element leaves the sector
            out = np.setdiff1d(np.arange(Hm.shape[0]), sel)
            assert np.all(Hm[np.ix_(out, sel)] == 0.0)


def test_two_site_hubbard_ground_state():
    U = 8.0
    w = networks.hubbard_dense(U, 0.0)
    Hm = _mpo_matrix([w[5:6], w[:, :, 0:1]])
    _, N, Sz2 = _jordan_wigner_hubbard(2, U, 0.0)
    sel = np.where((N == 2) & (Sz2 == 0))[0]
    e0 = np.linalg.eigvalsh(Hm[np.ix_(sel, sel)])[0]
    assert e0 == pytest.approx((U - np.sqrt(U * U + 16.0)) / 2.0, abs=1e-12)


def test_product_charge_bond_sectors():
    L, D = 10, 40
    bonds = networks.bond_sectors(L, D, networks.HUBBARD_PHYS, (L, 0), mods=(0, 0))
    assert len(bonds) == L - 1
    for b, sec in enumerate(bonds):
        assert 0 < sum(sec.values()) <= D
        for (n, sz), m in sec.items():
            assert m > 0
            assert 0 <= n <= 2 * (b + 1) and abs(sz) <= n and (n - sz) % 2 == 0
            # the rest of the chain can complete the target (L, 0)
            nr = L - n
            assert 0 <= nr <= 2 * (L - b - 1) and abs(sz) <= nr
    # the U(1) interface is unchanged: integer keys
    assert all(isinstance(k, int) for k in networks.bond_sectors(8, 16, [1, -1], 0)[3])
