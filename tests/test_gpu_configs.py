"""Parity with the oracle on the benchmark configurations at their stated sizes
(pytest -m gpu).  Each case runs the CUDA path and the oracle from the same seeded
inputs and asks for identical block structures and FP64 values to 1e-12
(contractions) / 1e-10 relative (decompositions, DMRG energies).

* Plain Heisenberg chain L=32, D=64, cutoff 1e-10, 6 sweeps from a seeded N(0,1)
  MPS (right-canonical), and the isolated mid-chain two-site H_eff.theta at
  oc = 15 of the final state (sources/dmrg.cpp:504-531, tests/DMRG_heisenberg_test.h).
* Synthetic theta-pair contraction + truncated sector SVD at D = 512.
* Fermi-Hubbard L=16, D=128, U(1)xU(1), half filling.
* The 4x8 Heisenberg cylinder built from the reference's own MPO fixture
  (tests/2dHeisenberg of the reference)."""
import os

import numpy as np
import pytest

import quantit_gb300 as q
from oracle import qtt_oracle as o
from tests._convert import same_structure, to_device, to_oracle

pytestmark = pytest.mark.gpu
NET = q.networks
HERE = os.path.dirname(os.path.abspath(__file__))


def _assert_same(dev, ora, rtol, atol):
    assert same_structure(dev, ora)
    got = dev.blocks()
    assert [k for k, _ in got] == [k for k, _ in ora.blocks]
    scale = max([float(np.max(np.abs(v))) for _, v in ora.blocks if v.size] + [1.0])
    for (k, a), (_, b) in zip(got, ora.blocks):
        np.testing.assert_allclose(a, b, rtol=rtol, atol=atol * scale, err_msg=str(k))


def _run_both(mpo_o, mps_o, oc, D, sweeps, min_bond):
    """The same DMRG on the GPU (from an upload of the oracle's start state) and in
    the oracle; returns (gpu per-sweep energies, gpu final MPS, oracle energies,
    oracle final MPS)."""
    dmpo = NET.bMPO([to_device(t) for t in mpo_o])
    dmps = NET.bMPS([to_device(t) for t in mps_o], oc)
    log = q.algorithms.dmrg_log_sweeptime()
    q.algorithms.dmrg(dmpo, dmps, q.algorithms.dmrg_options(cutoff=1e-10, convergence_criterion=0.0, max_bond=D,
                                                            min_bond=min_bond, maximum_iterations=sweeps), log)
    mps = [t for t in mps_o]
    _, _, Es = o.dmrg(mpo_o, mps, oc, o.DmrgOptions(cutoff=1e-10, convergence_criterion=0.0, maximum_bond=D,
                                                    minimum_bond=min_bond, maximum_iterations=sweeps))
    return log.energies, dmps, Es, mps


def _same_bonds(dmps, mps):
    for a, b in zip(dmps, mps):
        assert same_structure(a, b)
        assert a.block_indices() == [k for k, _ in b.blocks]


def test_heisenberg_L32_D64_six_sweeps_and_mid_chain_matvec():
    L, D = 32, 64
    mpo = o.heisenberg_mpo(L)
    mps0 = o.right_canonicalize(o.random_mps(L, D, [1, -1], 0, np.random.default_rng(7)))
    Eg, dmps, Eo, mps = _run_both(mpo, mps0, 0, D, 6, 4)
    assert len(Eg) == len(Eo) == 6
    np.testing.assert_allclose(Eg, Eo, rtol=1e-10)
    _same_bonds(dmps, mps)
    # the isolated H_eff.theta at oc = 15 of the oracle's final state, and the
    # environments it needs, computed on both sides from that same state
    oc = 15
    h2 = o.compute_2sites_hamil(mpo)
    left = o.trivial_edge((mps[0], 0), (mpo[0], 0))
    for i in range(oc):
        left = o.compute_left_env(mpo[i], mps[i], left)
    right = o.trivial_edge((mps[-1], 2), (mpo[-1], 2))
    for i in range(L - 1, oc + 1, -1):
        right = o.compute_right_env(mpo[i], mps[i], right)
    theta = o.tensordot(mps[oc], mps[oc + 1], [2], [0])
    want = o.hamil2site_times_state(theta, h2[oc], left, right)
    dl = to_device(o.trivial_edge((mps[0], 0), (mpo[0], 0)))
    for i in range(oc):
        dl = q.algorithms.compute_left_env(to_device(mpo[i]), to_device(mps[i]), dl)
    dr = to_device(o.trivial_edge((mps[-1], 2), (mpo[-1], 2)))
    for i in range(L - 1, oc + 1, -1):
        dr = q.algorithms.compute_right_env(to_device(mpo[i]), to_device(mps[i]), dr)
    _assert_same(dl, left, 1e-11, 1e-12)
    _assert_same(dr, right, 1e-11, 1e-12)
    dh2 = q.algorithms.compute_2sites_hamil(to_device(mpo[oc]), to_device(mpo[oc + 1]))
    got = q.algorithms.hamil2site_times_state(to_device(theta), dh2, dl, dr)
    _assert_same(got, want, 1e-11, 1e-12)


def test_theta_pair_D512_contraction_and_truncation():
    D = 512
    A, B = NET.theta_pair(D, seed=0)
    Ao, Bo = to_oracle(A), to_oracle(B)
    C = A.tensordot(B, ([2, 3], [1, 0]))
    Co = o.tensordot(Ao, Bo, [2, 3], [1, 0])
    _assert_same(C, Co, 1e-12, 1e-13)
    U, d, V = q.linalg.svd(C, 2, 1e-10, min_size=1, max_size=D)
    Uo, do, Vo = o.svd_truncated(Co, 2, 1e-10, 1, D)
    for t, w in ((U, Uo), (d, do), (V, Vo)):
        assert same_structure(t, w)
        assert t.block_indices() == [k for k, _ in w.blocks]
    dmax = max(float(np.max(v)) for _, v in do.blocks)
    for (k, a), (_, b) in zip(d.blocks(), do.blocks):
        np.testing.assert_allclose(a, b, rtol=1e-10, atol=1e-12 * dmax)


def test_hubbard_L16_D128_matches_oracle():
    L, D, U = 16, 128, 8.0
    mpo = NET.hubbard(L, U)
    mps = NET.random_bmps(L, D, NET.HUBBARD_PHYS, (L, 0), seed=4, mods=(0, 0))
    mpo_o = [to_oracle(t) for t in mpo]
    mps_o = [to_oracle(t) for t in mps]
    Eg, dmps, Eo, mps_f = _run_both(mpo_o, mps_o, mps.orthogonality_center, D, 2, 2)
    np.testing.assert_allclose(Eg, Eo, rtol=1e-10)
    _same_bonds(dmps, mps_f)


def test_cylinder_4x8_from_reference_fixture_matches_oracle():
    z = np.load(os.path.join(HERE, "golden", "heisenberg_cylinder_4x8_mpo.npz"))
    ws = [z[f"w{i}"][:, ::-1, :, ::-1] for i in range(32)]  # fixture basis {down, up} -> {up, down}
    mpo = NET.dense_mpo_to_bmpo(ws, [1, -1])
    L, D = 32, 48
    mps = NET.random_bmps(L, D, seed=9)
    mpo_o = [to_oracle(t) for t in mpo]
    mps_o = o.right_canonicalize([to_oracle(t) for t in mps])
    Eg, dmps, Eo, mps_f = _run_both(mpo_o, mps_o, 0, D, 3, 2)
    np.testing.assert_allclose(Eg, Eo, rtol=1e-10)
    _same_bonds(dmps, mps_f)
