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


def _energy_dense(ws, mps):
    env = np.ones((1, 1, 1))
    for W, A in zip(ws, mps):
        env = np.einsum("abc,bsBt,asx,ctz->xBz", env, W, A, A, optimize=True)
    nrm = np.ones((1, 1))
    for A in mps:
        nrm = np.einsum("ac,asx,csz->xz", nrm, A, A)
    return env.reshape(-1)[0] / nrm.reshape(-1)[0]


def test_coupling_mpo_matches_reference_cylinder_fixture():
    """The reference's 4x8 Heisenberg cylinder MPO (tests/2dHeisenberg of the reference,
    converted by tests/golden/make_cylinder_fixture.py) is column-major with columns of
    8 periodic sites and J = 1 on 55 bonds (the last column's wrap bond 24-31 is absent
    from the fixture).  The automaton builder given that coupling list is the same
    operator: equal <psi|H|psi> on random MPS, same bond dimension."""
    import os
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "heisenberg_cylinder_4x8_mpo.npz"))
    fix = [z[f"w{i}"][:, ::-1, :, ::-1] for i in range(32)]  # fixture basis {down, up} -> {up, down}
    cp = [c for c in networks.cylinder_couplings(4, 8, 1.0, "column") if (c[0], c[1]) != (24, 31)]
    assert len(cp) == 55
    ws = networks.heisenberg_couplings_dense(32, cp)
    assert max(w.shape[0] for w in ws) == max(w.shape[0] for w in fix) == 26
    rng = np.random.default_rng(5)
    for _ in range(3):
        dims = [1] + [4] * 31 + [1]
        mps = [rng.standard_normal((dims[i], 2, dims[i + 1])) for i in range(32)]
        assert _energy_dense(ws, mps) == pytest.approx(_energy_dense(fix, mps), rel=1e-12, abs=1e-12)


@pytest.mark.parametrize("Lx, Ly, order", [(2, 3, "snake"), (3, 2, "column"), (2, 4, "snake")])
def test_cylinder_mpo_matches_direct_hamiltonian(Lx, Ly, order):
    L = Lx * Ly
    cp = networks.cylinder_couplings(Lx, Ly, 1.0, order)
    Hm = _mpo_matrix(networks.heisenberg_couplings_dense(L, cp))
    sx = np.array([[0, .5], [.5, 0]])
    sy = np.array([[0, -.5j], [.5j, 0]])
    sz = np.diag([.5, -.5])

    def op(a, i):
        m = np.eye(1)
        for j in range(L):
            m = np.kron(m, a if j == i else np.eye(2))
        return m
    H = sum(J * (op(sx, i) @ op(sx, j) + op(sy, i) @ op(sy, j) + op(sz, i) @ op(sz, j)).real for i, j, J in cp)
    np.testing.assert_allclose(Hm, H, atol=1e-12)
    # geometry: every site has its 3 (or 4) neighbours, the snake keeps columns contiguous
    pos = networks.cylinder_sites(Lx, Ly, order)
    assert sorted(pos.values()) == list(range(L))
