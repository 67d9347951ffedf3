"""Fermi-Hubbard chain with U(1)xU(1) (N, 2Sz) charges on the GPU (pytest -m gpu):
DMRG reaches the exact ground state of a short chain, follows the oracle's DMRG
sweep for sweep (energies to 1e-10, identical bond structures), and the mixed
path agrees with FP64."""
import numpy as np
import pytest

import quantit_gb300 as q
from oracle import qtt_oracle as o
from tests._convert import same_structure, to_device, to_oracle
from tests.test_models_cpu import _jordan_wigner_hubbard

pytestmark = pytest.mark.gpu
NET = q.networks


def _hubbard_state(L, D, seed):
    return NET.random_bmps(L, D, NET.HUBBARD_PHYS, (L, 0), seed=seed, mods=(0, 0))


def test_hubbard_dmrg_approaches_exact_L4():
    # QuantiT's update is a single two-vector Krylov step per bond, which converges
    # slowly on Hubbard (the oracle is still 2e-5 above the exact energy after 40
    # sweeps from this start): the energy is variational and close after 40 sweeps
    L, U = 4, 8.0
    H, N, Sz2 = _jordan_wigner_hubbard(L, U, 0.0)
    sel = np.where((N == L) & (Sz2 == 0))[0]
    e0 = np.linalg.eigvalsh(H[np.ix_(sel, sel)])[0]
    mpo = NET.hubbard(L, U)
    mps = _hubbard_state(L, 16, seed=3)
    log = q.algorithms.dmrg_log_sweeptime()
    E = q.algorithms.dmrg(mpo, mps, q.algorithms.dmrg_options(cutoff=1e-12, convergence_criterion=1e-13,
                                                              max_bond=16, min_bond=1, maximum_iterations=40), log)
    assert E > e0 - 1e-10
    assert E - e0 < 1e-4
    assert all(b <= a + 1e-12 for a, b in zip(log.energies[2:], log.energies[3:]))


def test_hubbard_dmrg_matches_oracle():
    L, D, U = 6, 24, 8.0
    mpo = NET.hubbard(L, U)
    mps = _hubbard_state(L, D, seed=4)
    mpo_o = [to_oracle(t) for t in mpo]
    mps_o = [to_oracle(t) for t in mps]
    log = q.algorithms.dmrg_log_sweeptime()
    opts = dict(cutoff=1e-10, convergence_criterion=0.0, max_bond=D, min_bond=2, maximum_iterations=3)
    dmps = NET.bMPS([to_device(t) for t in mps_o], mps.orthogonality_center)
    E = q.algorithms.dmrg(mpo, dmps, q.algorithms.dmrg_options(**opts), log)
    E2, oc2, Es2 = o.dmrg(mpo_o, mps_o, mps.orthogonality_center,
                          o.DmrgOptions(cutoff=1e-10, convergence_criterion=0.0, maximum_bond=D, minimum_bond=2,
                                        maximum_iterations=3))
    np.testing.assert_allclose(log.energies, Es2, rtol=1e-10)
    assert E == pytest.approx(E2, rel=1e-10)
    for a, b in zip(dmps, mps_o):
        assert same_structure(a, b)
        assert a.block_indices() == [k for k, _ in b.blocks]


def test_hubbard_mixed_matches_fp64():
    # the one-step update converges slowly on Hubbard, so compare like the bench:
    # the same sweeps in each precision from one warmed-up state, FP64-evaluated
    L, D, U = 12, 48, 8.0
    mpo = NET.hubbard(L, U)
    mps = _hubbard_state(L, D, seed=5)
    mps.move_oc(0)
    mps.normalize_center()
    base = dict(cutoff=1e-10, convergence_criterion=0.0, max_bond=D, min_bond=1)
    q.algorithms.dmrg(mpo, mps, q.algorithms.dmrg_options(maximum_iterations=40, gemm="f64", **base))
    out = {}
    for gemm in ("f64", "tf32x3", "bf16x3"):
        cur = NET.bMPS(list(mps), mps.orthogonality_center)
        q.algorithms.dmrg(mpo, cur, q.algorithms.dmrg_options(maximum_iterations=3, gemm=gemm, **base))
        e, n2 = q.algorithms.mps_energy(mpo, cur)
        out[gemm] = e / n2
    for gemm in ("tf32x3", "bf16x3"):
        assert abs(out[gemm] - out["f64"]) / L < 1e-8, (gemm, out)


def test_cylinder_dmrg_matches_oracle():
    """Long-range MPO (4x3 snake cylinder, couplings up to distance 5): the GPU DMRG
    follows the oracle sweep for sweep."""
    mpo = NET.cylinder_heisenberg(4, 3, 1.0, "snake")
    L, D = len(mpo), 16
    mps = NET.random_bmps(L, D, seed=6)
    mpo_o = [to_oracle(t) for t in mpo]
    mps_o = [to_oracle(t) for t in mps]
    log = q.algorithms.dmrg_log_sweeptime()
    dmps = NET.bMPS([to_device(t) for t in mps_o], mps.orthogonality_center)
    q.algorithms.dmrg(mpo, dmps, q.algorithms.dmrg_options(cutoff=1e-10, convergence_criterion=0.0, max_bond=D,
                                                           min_bond=2, maximum_iterations=3), log)
    E2, oc2, Es2 = o.dmrg(mpo_o, mps_o, mps.orthogonality_center,
                          o.DmrgOptions(cutoff=1e-10, convergence_criterion=0.0, maximum_bond=D, minimum_bond=2,
                                        maximum_iterations=3))
    np.testing.assert_allclose(log.energies, Es2, rtol=1e-10)
    for a, b in zip(dmps, mps_o):
        assert same_structure(a, b)
        assert a.block_indices() == [k for k, _ in b.blocks]


def test_cylinder_mixed_matches_fp64():
    mpo = NET.cylinder_heisenberg(4, 4, 1.0, "snake")
    L, D = len(mpo), 64
    mps = NET.random_bmps(L, D, seed=7)
    mps.move_oc(0)
    mps.normalize_center()
    base = dict(cutoff=1e-10, convergence_criterion=0.0, max_bond=D, min_bond=1)
    q.algorithms.dmrg(mpo, mps, q.algorithms.dmrg_options(maximum_iterations=8, gemm="f64", **base))
    out = {}
    # config 3: split-TF32 and split-BF16 GEMMs against FP64 from the same state
    for gemm in ("f64", "tf32x3", "bf16x3"):
        cur = NET.bMPS(list(mps), mps.orthogonality_center)
        q.algorithms.dmrg(mpo, cur, q.algorithms.dmrg_options(maximum_iterations=2, gemm=gemm, **base))
        e, n2 = q.algorithms.mps_energy(mpo, cur)
        out[gemm] = e / n2
    for gemm in ("tf32x3", "bf16x3"):
        assert abs(out[gemm] - out["f64"]) / L < 1e-8, (gemm, out)
