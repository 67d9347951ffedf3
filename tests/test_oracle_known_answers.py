"""The oracle against the known answers of QuantiT's own unit tests (CPU only)."""
import json
import math
import os

import numpy as np
import pytest

from oracle import qtt_oracle as o

HERE = os.path.dirname(os.path.abspath(__file__))
KNOWN = json.load(open(os.path.join(HERE, "golden", "reference_known_answers.json")))
C5 = (5,)


def _mk(legs, sel, blocks, rng, mods=C5, scale=1.0):
    t = o.btensor([[(n, q) for n, q in leg] for leg in legs], [sel], mods)
    for b in blocks:
        t.blocks.append((tuple(b), scale * rng.random(t.block_shape(tuple(b)))))
    t.blocks.sort(key=lambda kv: kv[0])
    assert t.check() == ""
    return t


def test_c5_constructor_and_group_ops():
    k = KNOWN["c5_charges"]
    for v, want in k["ctor"]:
        assert o.make_C(v, k["mod"]) == want
    assert o.q_add((2,), (2,), C5) == (4,)
    assert o.q_inv((3,), C5) == (2,)
    assert o.q_add(o.q_inv((3,), C5), (3,), C5) == (0,)
    assert o.q_inv((3,), (0,)) == (-3,)
    assert o.q_add((1,), (1,), (2,)) == (0,)


def test_tensordot_block_structure_and_values():
    k = KNOWN["tensordot_blocks"]
    rng = np.random.default_rng(0)
    A = _mk(k["A_legs"], k["A_sel"], k["A_blocks"], rng)
    B = _mk(k["B_legs"], k["B_sel"], k["B_blocks"], rng)
    C = o.tensordot(A, B, *k["dims"])
    assert [list(i) for i, _ in C.blocks] == k["C_blocks"]
    Ad, Bd = A.block_dict(), B.block_dict()
    for key, (ia, ib) in k["C_from"].items():
        want = np.tensordot(Ad[tuple(ia)], Bd[tuple(ib)], ([1], [1]))
        got = C.block_dict()[tuple(int(x) for x in key.split(","))]
        np.testing.assert_allclose(got, want, rtol=1e-13)
    # trace of A with its inverse: every block contributes
    tr = o.tensordot(A, o.inverse_cvals(A), [0, 1], [0, 1])
    want = sum(float(np.sum(b * b)) for _, b in A.blocks)
    assert len(tr.blocks) == 1 and tr.blocks[0][0] == ()
    np.testing.assert_allclose(float(tr.blocks[0][1]), want, rtol=1e-13)


def test_tensor_product_via_empty_contraction():
    k = KNOWN["tensordot_blocks"]
    rng = np.random.default_rng(1)
    A = _mk(k["A_legs"], k["A_sel"], k["A_blocks"], rng)
    C = o.tensordot(A, A, [], [])
    assert [list(i) for i, _ in C.blocks] == KNOWN["tensor_product_blocks"]["C_blocks"]
    Ad = A.block_dict()
    np.testing.assert_array_equal(C.block_dict()[(0, 0, 1, 1)], np.multiply.outer(Ad[(0, 0)], Ad[(1, 1)]))


def test_trace_independent_of_leg_order():
    """btensor.h:1551-1580: the full self-contraction is the same for every order."""
    k = KNOWN["tensordot_blocks"]
    rng = np.random.default_rng(2)
    A = _mk(k["A_legs"], k["A_sel"], k["A_blocks"], rng)
    X = o.randn_like(o.concat_shapes(A, o.permute(A, [1, 0])), rng)
    want = sum(float(np.sum(b * b)) for _, b in X.blocks)
    import itertools
    for perm in itertools.permutations(range(4)):
        t = o.tensordot(X, o.conj(X), list(perm), list(perm))
        np.testing.assert_allclose(float(t.blocks[0][1]), want, rtol=1e-12)


def test_reshape_known_answers():
    k = KNOWN["tensordot_blocks"]
    r = KNOWN["reshape_vector"]
    rng = np.random.default_rng(3)
    A = _mk(k["A_legs"], k["A_sel"], k["A_blocks"], rng)
    B = o.reshape(A, [])
    keys = [i for i, _ in B.blocks]
    for p in r["present"]:
        assert (p,) in keys
    for p in r["absent"]:
        assert (p,) not in keys
    for s, q in r["charges"].items():
        assert B.cv[int(s)] == (q,)
    for s, n in r["sizes"].items():
        assert B.ssz[int(s)] == n
    C = o.reshape_as(B, A)
    assert C.check() == ""
    assert [i for i, _ in C.blocks] == [i for i, _ in A.blocks]
    for (_, x), (_, y) in zip(C.blocks, A.blocks):
        np.testing.assert_array_equal(x, y)


def test_sector_order_and_compact_round_trip():
    k = KNOWN["sector_order"]
    rng = np.random.default_rng(4)
    A = _mk(k["A_legs"], k["A_sel"], k["A_blocks"], rng)
    assert [list(i) for i, _ in o.reorder_by_cvals(A)] == k["reorder_rank3"]
    B = o.reshape(A, [1])
    assert [list(i) for i, _ in o.reorder_by_cvals(B)] == k["reorder_after_reshape1"]
    Bd = B.block_dict()
    for sec in o.compact_dense(B):
        for row, ra, rb in sec.rows:
            for col, ca, cb in sec.cols:
                key = sec.other + (row, col)
                blk = sec.mat[..., ra:rb, ca:cb]
                if key in Bd:
                    np.testing.assert_array_equal(blk, Bd[key])
                else:
                    assert not np.any(blk)


def test_heisenberg_L3_matrix():
    h = KNOWN["heisenberg_L3"]
    want = np.zeros((8, 8))
    for i, j, v in h["entries"]:
        want[i, j] = v
    w = o.heisenberg_dense_w(-4.0)   # Heisenberg_impl(J=1) == Heisenberg(J=-4)
    ws = [w[4:5], w, w[:, :, 0:1]]
    c = np.tensordot(ws[0], ws[1], ([2], [0])).transpose(0, 1, 3, 4, 2, 5).reshape(1, 4, 5, 4)
    c = np.tensordot(c, ws[2], ([2], [0])).transpose(0, 1, 3, 4, 2, 5).reshape(8, 8)
    np.testing.assert_array_equal(c, want)
    # the block MPO encodes the same operator
    mpo = o.heisenberg_mpo(3, J=-4.0)
    dense = [o.to_dense(t) for t in mpo]
    assert all(t.check() == "" for t in mpo)
    # undo the charge grouping by comparing spectra of the contracted operator
    c2 = np.tensordot(dense[0], dense[1], ([2], [0])).transpose(0, 1, 3, 4, 2, 5).reshape(1, 4, -1, 4)
    c2 = np.tensordot(c2, dense[2], ([2], [0])).transpose(0, 1, 3, 4, 2, 5).reshape(8, 8)
    np.testing.assert_allclose(np.sort(np.linalg.eigvalsh(c2)), np.sort(np.linalg.eigvalsh(want)), atol=1e-12)


def test_eig2x2():
    """dmrg.h:115-139."""
    rng = np.random.default_rng(5)
    for _ in range(20):
        ang = rng.random() * 2 * math.pi
        E0, E1 = -rng.random(), rng.random()
        p00, p01, p10, p11 = math.cos(ang), math.sin(ang), math.sin(ang), -math.cos(ang)
        a0 = p00 ** 2 * E0 + p10 ** 2 * E1
        a1 = p01 ** 2 * E0 + p11 ** 2 * E1
        b = p01 * p00 * E0 + p11 * p10 * E1
        E, oc, nc = o.eig2x2(a0, a1, b)
        assert E == pytest.approx(E0, abs=1e-12)
        ok = (np.allclose([p00, p01], [oc, nc]) or np.allclose([-p00, -p01], [oc, nc]))
        assert ok


def _ising_mpo():
    w = np.zeros((3, 2, 3, 2))
    w[1, 0, 0, 0] = w[2, 0, 1, 0] = 1
    w[1, 1, 0, 1] = w[2, 1, 1, 1] = -1
    w[0, 0, 0, 0] = w[0, 1, 0, 1] = 1
    w[2, 0, 2, 0] = w[2, 1, 2, 1] = 1
    return o.dense_mpo_to_block([w[2:3], w[:, :, 0:1]], [1, -1])


def test_two_site_mpo_and_lanczos_identities():
    """dmrg.h:141-221 with the Ising MPO: <H> three ways and the one-step Lanczos identities."""
    mpo = _ising_mpo()
    h2 = o.compute_2sites_hamil(mpo)
    mps = o.right_canonicalize(o.random_mps(2, 4, [1, -1], 0, np.random.default_rng(6)))
    theta = o.tensordot(mps[0], mps[1], [2], [0])
    assert o.dot_all(theta, theta) == pytest.approx(1.0)
    H_av = o.mps_energy(mpo, mps)
    L = o.trivial_edge((mps[0], 0), (mpo[0], 0))
    R = o.trivial_edge((mps[1], 2), (mpo[1], 2))
    H_upd = o.dot_all(theta, o.hamil2site_times_state(theta, h2[0], L, R))
    assert H_upd == pytest.approx(H_av, abs=1e-12)
    psi, a0, a1, b = o.one_step_lanczos(theta, h2[0], L, R)
    E, oc, nc = o.eig2x2(a0, a1, b)
    assert oc ** 2 + nc ** 2 == pytest.approx(1.0)
    upd = o.add_scaled(theta, psi, oc, nc)
    assert o.dot_all(upd, upd) == pytest.approx(1.0)
    assert o.dot_all(psi, theta) == pytest.approx(0.0, abs=1e-12)
    assert o.dot_all(psi, psi) == pytest.approx(0.0, abs=1e-12)  # the state is an Ising eigenstate


def test_truncating_svd_error_bound():
    """LinearAlgebra.h:402-567: blocks of A*U*d*V^H differ from A by less than tol."""
    k = KNOWN["sector_order"]
    tole = 1e-5
    rng = np.random.default_rng(8)
    A = _mk(k["A_legs"], k["A_sel"], [], rng)
    scales = {(0, 0, 2): 1, (0, 1, 0): 1, (0, 3, 2): 0.1, (1, 0, 1): 1, (1, 1, 2): 1, (1, 2, 0): 0.1, (1, 3, 1): 1}
    for key, s in scales.items():
        A.blocks.append((key, tole * s * rng.random(A.block_shape(key))))
    A.blocks.sort(key=lambda kv: kv[0])
    for mult in (1.0, 0.3):
        Am = o.scale(A, mult)
        U, d, V = o.svd_truncated(Am, 1, tole, 1, 2 ** 62)
        AA = o.tensordot(o.mul_lastleg(U, d), o.conj(V), [U.rank - 1], [V.rank - 1])
        AAd = AA.block_dict()
        for key, blk in Am.blocks:
            if key in AAd:
                assert np.all(np.abs(blk - AAd[key]) < tole)
            else:
                assert np.all(np.abs(blk) < tole)


def test_untruncated_svd_reconstruction_and_unitarity():
    """LinearAlgebra.h:341-400,447-472."""
    rng = np.random.default_rng(9)
    X = o.btensor([[(2, -2), (2, 0), (2, 2)], [(1, 1), (1, -1)], [(1, 1), (1, -1)], [(2, 2), (2, 0), (2, -2)]],
                  [0], (2,))
    X = o.randn_like(X, rng)
    U, d, V = o.svd_split(X, 2)
    nd = sum(d.ssz)
    assert o.dot_all(U, U) == pytest.approx(nd)
    assert o.dot_all(V, V) == pytest.approx(nd)
    XX = o.tensordot(o.mul_lastleg(U, d), o.conj(V), [2], [2])
    Xd = X.block_dict()
    for key, blk in XX.blocks:
        np.testing.assert_allclose(blk, Xd[key], atol=1e-12)
    assert set(XX.block_dict()) == set(Xd)


def test_dmrg_matches_exact_diagonalisation():
    L = 8
    sx = np.array([[0, .5], [.5, 0]])
    sy = np.array([[0, -.5j], [.5j, 0]])
    sz = np.diag([.5, -.5])

    def op(a, i):
        m = np.eye(1)
        for j in range(L):
            m = np.kron(m, a if j == i else np.eye(2))
        return m
    H = sum((op(sx, i) @ op(sx, i + 1) + op(sy, i) @ op(sy, i + 1) + op(sz, i) @ op(sz, i + 1)).real
            for i in range(L - 1))
    e0 = np.linalg.eigvalsh(H)[0]
    mpo = o.heisenberg_mpo(L)
    mps = o.right_canonicalize(o.random_mps(L, 16, [1, -1], 0, np.random.default_rng(0)))
    E, oc, Es = o.dmrg(mpo, mps, 0, o.DmrgOptions(cutoff=1e-10, convergence_criterion=0.0, maximum_bond=16,
                                                  minimum_bond=4, maximum_iterations=5))
    assert oc == 0
    assert E == pytest.approx(e0, abs=1e-10)
    assert o.mps_energy(mpo, mps) == pytest.approx(e0, abs=1e-10)


def test_tensorgdot_is_addmm():
    """tensorgdot.h:281-320: beta*add + alpha*tensordot."""
    rng = np.random.default_rng(10)
    k = KNOWN["tensordot_blocks"]
    A = _mk(k["A_legs"], k["A_sel"], k["A_blocks"], rng)
    B = _mk(k["B_legs"], k["B_sel"], k["B_blocks"], rng)
    C = o.tensordot(A, B, [1], [1])
    add = o.randn_like(C.empty_like(), rng)
    G = o.tensorgdot(add, A, B, [1], [1], beta=0.5, alpha=2.0)
    want = o.add_scaled(add, C, 0.5, 2.0)
    for (ka, va), (kb, vb) in zip(G.blocks, want.blocks):
        assert ka == kb
        np.testing.assert_allclose(va, vb, rtol=1e-13)


def test_contraction_errors():
    k = KNOWN["tensordot_blocks"]
    rng = np.random.default_rng(11)
    A = _mk(k["A_legs"], k["A_sel"], k["A_blocks"], rng)
    with pytest.raises(o.ContractionError):
        o.tensordot(A, A, [1], [1])          # charges do not cancel
    with pytest.raises(o.ContractionError):
        o.tensordot(A, A, [0, 1], [0])       # dims lists of different length
