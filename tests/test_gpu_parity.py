"""Parity of the CUDA path with the oracle (run on a GB300: pytest -m gpu).

Block structures must be identical; FP64 values agree to 1e-12 relative
(contractions, inner products) and 1e-10 (decompositions, DMRG energies)."""
import os

import numpy as np
import pytest

import quantit_gb300 as q
from oracle import qtt_oracle as o
from tests._convert import same_structure, to_device, to_oracle
from tests.test_library_cpu import _contractible_pair, _random_tensor

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
RTOL = 1e-12


def _assert_same(dev, ora, rtol=RTOL, atol=1e-13):
    assert same_structure(dev, ora)
    got = dev.blocks()
    assert [k for k, _ in got] == [k for k, _ in ora.blocks]
    scale = max([float(np.max(np.abs(v))) for _, v in ora.blocks if v.size] + [1.0])
    for (k, a), (_, b) in zip(got, ora.blocks):
        np.testing.assert_allclose(a, b, rtol=rtol, atol=atol * scale, err_msg=str(k))


@pytest.mark.parametrize("mods", [(0,), (5,), (0, 0)])
def test_tensordot_values(mods):
    rng = np.random.default_rng(11 + len(mods))
    n = 0
    for trial in range(600):
        if n >= 25:
            break
        ra, rb = int(rng.integers(1, 5)), int(rng.integers(1, 5))
        nc = int(rng.integers(0, min(ra, rb) + 1))
        A, B, dA, dB = _contractible_pair(rng, mods, ra, rb, nc)
        if not A.blocks or not B.blocks:
            continue
        want = o.tensordot(A, B, dA, dB)
        got = to_device(A).tensordot(to_device(B), (dA, dB))
        _assert_same(got, want)
        n += 1
    assert n >= 10


def test_tensordot_golden_fixture():
    g = np.load(os.path.join(ROOT, "tests", "golden", "oracle_cases.npz"))
    rng = np.random.default_rng(1234)
    A = o.btensor([[(2, -1), (3, 0), (1, 2)], [(1, -1), (1, 1)], [(1, -1), (1, 1)], [(2, -2), (4, 0), (3, 1)]],
                  [0], (0,))
    A = o.randn_like(A, rng)
    B = o.btensor([[(2, 2), (4, 0), (3, -1)], [(1, 1), (1, -1)], [(1, 1), (1, -1)], [(3, 1), (2, -1)]], [1], (0,))
    B = o.randn_like(B, rng)
    C = to_device(A).tensordot(to_device(B), ([3, 2], [0, 1]))
    assert [list(k) for k in C.block_indices()] == g["C_blocks"].tolist()
    nrm = np.sqrt(sum(float(np.sum(v ** 2)) for _, v in C.blocks()))
    assert nrm == pytest.approx(float(g["C_norm"]), rel=1e-12)


def test_large_contraction_property():
    """A contraction big enough to use many tiles: checked against a dense einsum."""
    rng = np.random.default_rng(5)
    A = o.btensor([[(40, -1), (70, 0), (33, 1)], [(1, -1), (1, 1)], [(1, -1), (1, 1)], [(50, -2), (90, 0), (45, 2)]],
                  [0], (0,))
    A = o.randn_like(A, rng)
    B = o.btensor([[(50, 2), (90, 0), (45, -2)], [(1, 1), (1, -1)], [(65, 1), (80, -1)]], [0], (0,))
    B = o.randn_like(B, rng)
    got = to_device(A).tensordot(to_device(B), ([3, 2], [0, 1]))
    want = np.tensordot(o.to_dense(A), o.to_dense(B), ([3, 2], [0, 1]))
    np.testing.assert_allclose(o.to_dense(to_oracle(got)), want, rtol=1e-11, atol=1e-11)


def test_tensorgdot_and_algebra():
    rng = np.random.default_rng(6)
    A, B, dA, dB = _contractible_pair(rng, (0,), 3, 3, 1)
    while not A.blocks or not B.blocks:
        A, B, dA, dB = _contractible_pair(rng, (0,), 3, 3, 1)
    C = o.tensordot(A, B, dA, dB)
    add = o.randn_like(C.empty_like(), rng)
    got = q.tensorgdot(to_device(add), to_device(A), to_device(B), dA, dB, beta=0.25, alpha=-1.5)
    _assert_same(got, o.tensorgdot(add, A, B, dA, dB, beta=0.25, alpha=-1.5))
    # in place variant
    dadd = to_device(add)
    q.tensorgdot_(dadd, to_device(A), to_device(B), dA, dB, beta=2.0, alpha=0.5)
    _assert_same(dadd, o.tensorgdot(add, A, B, dA, dB, beta=2.0, alpha=0.5))
    X = o.randn_like(C.empty_like(), rng)
    Y = C
    _assert_same(to_device(X).add(to_device(Y), -0.75), o.add_scaled(X, Y, 1.0, -0.75))
    _assert_same(to_device(X) * 3.0, o.scale(X, 3.0))
    assert q.dot_all(to_device(X), to_device(Y)) == pytest.approx(o.dot_all(X, Y), rel=1e-12, abs=1e-12)


def test_permute_reshape_values():
    rng = np.random.default_rng(7)
    for trial in range(20):
        T = _random_tensor(rng, 4, (0,), sizes=(1, 4))
        if not T.blocks:
            continue
        perm = rng.permutation(4).tolist()
        _assert_same(to_device(T).permute(perm), o.permute(T, perm), rtol=0, atol=0)
        _assert_same(to_device(T).reshape([2]), o.reshape(T, [2]), rtol=0, atol=0)


def _theta(rng, D=(3, 5, 4), mods=(0,)):
    a, b, c = D
    T = o.btensor([[(a, -2), (b, 0), (c, 2)], [(1, -1), (1, 1)], [(1, -1), (1, 1)], [(c, 2), (b, 0), (a, -2)]],
                  [0], mods)
    return o.randn_like(T, rng)


def _sorted_values(d):
    return np.sort(np.concatenate([np.ravel(v) for _, v in d.blocks()]))[::-1]


def test_svd_untruncated():
    rng = np.random.default_rng(8)
    T = _theta(rng, (6, 9, 7))
    U, d, V = q.linalg.svd(to_device(T), 2)
    Uo, do, Vo = o.svd_split(T, 2)
    for got, want in ((U, Uo), (d, do), (V, Vo)):
        assert same_structure(got, want)
        assert got.block_indices() == [k for k, _ in want.blocks]
    np.testing.assert_allclose(_sorted_values(d), np.sort(np.concatenate([v for _, v in do.blocks]))[::-1],
                               rtol=1e-12, atol=1e-13)
    # reconstruction and isometry
    R = U.mul(d).tensordot(V.conj(), ([2], [2]))
    _assert_same(R, T, rtol=1e-11, atol=1e-12)
    nd = sum(d.section_sizes)
    assert q.dot_all(U, U) == pytest.approx(nd, rel=1e-12)
    assert q.dot_all(V, V) == pytest.approx(nd, rel=1e-12)


def test_svd_truncated_matches_oracle():
    rng = np.random.default_rng(9)
    for trial in range(6):
        T = _theta(rng, (5, 8, 6))
        for (tol, mn, mx) in ((1e-10, 1, 7), (1e-10, 4, 20), (0.5, 1, 100)):
            U, d, V = q.linalg.svd(to_device(T), 2, tol, min_size=mn, max_size=mx)
            Uo, do, Vo = o.svd_truncated(T, 2, tol, mn, mx)
            for got, want in ((U, Uo), (d, do), (V, Vo)):
                assert same_structure(got, want)
                assert got.block_indices() == [k for k, _ in want.blocks]
            dv = d.blocks()
            for (k, a), (_, b) in zip(dv, do.blocks):
                np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-13)
            R = U.mul(d).tensordot(V.conj(), ([2], [2]))
            Ro = o.tensordot(o.mul_lastleg(Uo, do), o.conj(Vo), [2], [2])
            _assert_same(R, Ro, rtol=1e-10, atol=1e-12)


def test_svd_rank_deficient_sector_stays_isometric():
    rng = np.random.default_rng(10)
    T = _theta(rng, (4, 6, 4))
    # make one sector rank one
    T.blocks = [(k, (np.outer(np.ones(v.shape[0]), np.ones(v.size // v.shape[0])).reshape(v.shape)
                     if k[0] == 1 and k[3] == 1 else v)) for k, v in T.blocks]
    U, d, V = q.linalg.svd(to_device(T), 2)
    nd = sum(d.section_sizes)
    assert q.dot_all(U, U) == pytest.approx(nd, rel=1e-10)
    assert q.dot_all(V, V) == pytest.approx(nd, rel=1e-10)


def test_eigh_matches_oracle():
    rng = np.random.default_rng(12)
    X = _theta(rng, (4, 7, 5))
    H = o.tensordot(X, o.conj(X), [2, 3], [2, 3])      # [a, s, a', s'] hermitian
    d, U = q.linalg.eigh(to_device(H), 2)
    do, Uo = o.eigh_split(H, 2)
    assert same_structure(d, do) and same_structure(U, Uo)
    for (k, a), (_, b) in zip(d.blocks(), do.blocks):
        np.testing.assert_allclose(a, b, rtol=1e-10, atol=1e-10 * float(np.max(np.abs(b))))
    R = U.mul(d).tensordot(U.conj(), ([2], [2]))
    _assert_same(R, H, rtol=1e-9, atol=1e-10)


def _heis_setup(L, D, seed):
    mpo = o.heisenberg_mpo(L)
    mps = o.right_canonicalize(o.random_mps(L, D, [1, -1], 0, np.random.default_rng(seed)))
    return mpo, mps


def test_heff_matvec_and_lanczos():
    L = 8
    mpo, mps = _heis_setup(L, 16, 3)
    env = o.generate_env(mpo, mps, 0)
    # move to bond 3 with oracle sweeps so environments are nontrivial
    h2 = o.compute_2sites_hamil(mpo)
    for oc in range(3):
        o.dmrg_bond_update(mpo, h2, mps, env, oc, True, o.DmrgOptions(cutoff=1e-12, maximum_bond=16))
    oc = 3
    theta = o.tensordot(mps[oc], mps[oc + 1], [2], [0])
    Lenv, Renv = env[oc], env[oc + 3]
    dt, dh, dL, dR = to_device(theta), to_device(h2[oc]), to_device(Lenv), to_device(Renv)
    _assert_same(q.algorithms.hamil2site_times_state(dt, dh, dL, dR), o.hamil2site_times_state(theta, h2[oc], Lenv, Renv),
                 rtol=1e-11, atol=1e-12)
    psi, a0, a1, b = q.algorithms.one_step_lanczos(dt, dh, dL, dR)
    psio, a0o, a1o, bo = o.one_step_lanczos(theta, h2[oc], Lenv, Renv)
    assert a0 == pytest.approx(a0o, rel=1e-12)
    assert b == pytest.approx(bo, rel=1e-10)
    assert a1 == pytest.approx(a1o, rel=1e-10)
    _assert_same(psi, psio, rtol=1e-9, atol=1e-11)
    # environments
    _assert_same(q.algorithms.compute_left_env(to_device(mpo[oc]), to_device(mps[oc]), to_device(env[oc])),
                 o.compute_left_env(mpo[oc], mps[oc], env[oc]), rtol=1e-11, atol=1e-12)
    h2d = q.algorithms.compute_2sites_hamil(to_device(mpo[2]), to_device(mpo[3]))
    _assert_same(h2d, h2[2], rtol=0, atol=0)
    E, oo, nn = q.algorithms.eig2x2(a0o, a1o, bo)
    Eo, ooo, nno = o.eig2x2(a0o, a1o, bo)
    assert (E, oo, nn) == pytest.approx((Eo, ooo, nno), rel=1e-14)


def test_dmrg_energies_match_oracle_and_golden():
    g = np.load(os.path.join(ROOT, "tests", "golden", "oracle_cases.npz"))
    L, D = 10, 16
    mpo = o.heisenberg_mpo(L)
    mps = o.right_canonicalize(o.random_mps(L, D, [1, -1], 0, np.random.default_rng(7)))
    dmpo = q.networks.bMPO([to_device(t) for t in mpo])
    dmps = q.networks.bMPS([to_device(t) for t in mps], 0)
    log = q.algorithms.dmrg_log_sweeptime()
    E = q.algorithms.dmrg(dmpo, dmps, q.algorithms.dmrg_options(cutoff=1e-10, convergence_criterion=0.0, max_bond=D,
                                                                min_bond=4, maximum_iterations=3), log)
    np.testing.assert_allclose(log.energies, g["dmrg_E"], rtol=1e-10)
    assert E == pytest.approx(float(g["dmrg_E"][-1]), rel=1e-10)
    assert dmps.orthogonality_center == 0
    # the state itself: bond structures equal the oracle's run
    E2, oc2, Es2 = o.dmrg(mpo, mps, 0, o.DmrgOptions(cutoff=1e-10, convergence_criterion=0.0, maximum_bond=D,
                                                      minimum_bond=4, maximum_iterations=3))
    for a, b in zip(dmps, mps):
        assert same_structure(a, b)
        assert a.block_indices() == [k for k, _ in b.blocks]


def test_dmrg_exact_energy_L8():
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
    mpo = q.networks.heisenberg(L)
    mps = q.networks.random_bmps(L, 16, seed=1)
    mps.move_oc(0)
    mps.normalize_center()
    E = q.algorithms.dmrg(mpo, mps, q.algorithms.dmrg_options(cutoff=1e-10, convergence_criterion=1e-13,
                                                              max_bond=16, maximum_iterations=20))
    assert E == pytest.approx(e0, abs=1e-9)


@pytest.mark.parametrize("gemm, tol", [("f64", 1e-10), ("tf32x3", 1e-8)])
def test_dmrg_svd_warm_start_is_exact(gemm, tol):
    """Each bond's sector SVD may start from the rotation of its previous decomposition
    in the call: any orthogonal start gives an exact SVD, so the energies agree with
    cold starts (FP64: 1e-10 relative, structures equal; mixed: FP32-level)."""
    L, D = 12, 40
    mpo = o.heisenberg_mpo(L)
    mps = o.right_canonicalize(o.random_mps(L, D, [1, -1], 0, np.random.default_rng(8)))
    dmpo = q.networks.bMPO([to_device(t) for t in mpo])
    out = {}
    for warm in (False, True):
        dmps = q.networks.bMPS([to_device(t) for t in mps], 0)
        log = q.algorithms.dmrg_log_sweeptime()
        q.algorithms.dmrg(dmpo, dmps, q.algorithms.dmrg_options(
            cutoff=1e-10, convergence_criterion=0.0, max_bond=D, min_bond=4, maximum_iterations=4, gemm=gemm,
            svd_warm_start=warm), log)
        e, n2 = q.algorithms.mps_energy(dmpo, dmps)
        out[warm] = (e / n2, dmps)
    assert abs(out[True][0] - out[False][0]) <= tol * abs(out[False][0])
    if gemm == "f64":
        for a, b in zip(out[True][1], out[False][1]):
            assert a.block_indices() == b.block_indices()
