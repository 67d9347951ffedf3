"""MPO / MPS container operations on the GPU against the oracle (pytest -m gpu):
bMPO::coalesce (sources/MPT.cpp:154-168), the two-direction compression built on
it, and contract(bMPS, bMPS[, edges]) (sources/MPT.cpp:267-290)."""
import numpy as np
import pytest

import quantit_gb300 as q
from oracle import qtt_oracle as o
from tests._convert import same_structure, to_device, to_oracle

pytestmark = pytest.mark.gpu
NET = q.networks


def _bond_dims(mpo):
    return [int(sum(to_oracle(t, with_data=False).sec_sizes(2))) for t in mpo]


def test_coalesce_matches_oracle():
    """Same block structures and bond dimensions as the oracle's coalesce, and the
    same operator: <psi|H|psi> unchanged on a random MPS (1e-12)."""
    mpo = NET.cylinder_heisenberg(4, 3, 1.0, "snake")
    mpo_o = [to_oracle(t) for t in mpo]
    want = o.coalesce(mpo_o, 1e-13)
    got = NET.bMPO(list(mpo)).coalesce(1e-13)
    for a, b in zip(got, want):
        assert same_structure(a, b)
        assert a.block_indices() == [k for k, _ in b.blocks]
    mps = o.random_mps(len(mpo), 12, [1, -1], 0, np.random.default_rng(3))
    e0 = o.mps_energy(mpo_o, mps) / o.mps_norm2(mps)
    e1, n1 = q.algorithms.mps_energy(got, NET.bMPS([to_device(t) for t in mps], 0))
    e2, _ = q.algorithms.mps_energy(mpo, NET.bMPS([to_device(t) for t in mps], 0))
    assert e1 / n1 == pytest.approx(e0, rel=1e-12)
    assert e2 / n1 == pytest.approx(e0, rel=1e-12)


def test_compress_reaches_the_schmidt_rank_of_the_cylinder():
    """Both directions: the 12 x 6 snake cylinder's automaton MPO (bond dimension 35)
    drops to its operator Schmidt rank, 2 + 3 x 6 = 20, with the operator unchanged."""
    mpo = NET.cylinder_heisenberg(12, 6, 1.0, "snake")
    assert max(_bond_dims(mpo)) == 35
    small = NET.cylinder_heisenberg(12, 6, 1.0, "snake", compress=True)
    assert max(_bond_dims(small)) == 20
    mps = NET.random_bmps(72, 6, seed=4)
    e0, n0 = q.algorithms.mps_energy(mpo, mps)
    e1, n1 = q.algorithms.mps_energy(small, mps)
    assert e1 / n1 == pytest.approx(e0 / n0, rel=1e-11, abs=1e-13 * abs(e0 / n0))


def test_contract_two_mps_matches_oracle():
    L = 10
    rng = np.random.default_rng(5)
    a = o.random_mps(L, 16, [1, -1], 0, rng)
    b = o.random_mps(L, 12, [1, -1], 0, rng)
    want = o.mps_overlap(a, b)
    da = NET.bMPS([to_device(t) for t in a], 0)
    db = NET.bMPS([to_device(t) for t in b], 0)
    got = NET.contract(da, db)
    assert got.dim() == 0
    val = sum(float(np.sum(v)) for _, v in got.blocks())
    assert val == pytest.approx(want, rel=1e-12)
    # <a|a> agrees with the norm of the FP64 energy contraction
    aa = sum(float(np.sum(v)) for _, v in NET.contract(da, da).blocks())
    _, n2 = q.algorithms.mps_energy(q.networks.heisenberg(L), da)
    assert aa == pytest.approx(n2, rel=1e-12)


def test_environments_match_the_oracle():
    L, D = 10, 12
    mpo = o.heisenberg_mpo(L)
    mps = o.random_mps(L, D, [1, -1], 0, np.random.default_rng(6))
    env = o.generate_env(mpo, mps, 0)
    # left environments built up to bond 6, right ones down to bond 3
    dmpo = [to_device(t) for t in mpo]
    dmps = [to_device(t) for t in mps]
    got = q.algorithms.environments(dmpo, dmps, [3, 6])
    wl = o.trivial_edge((mps[0], 0), (mpo[0], 0))
    lefts = [wl]
    for i in range(L):
        lefts.append(o.compute_left_env(mpo[i], mps[i], lefts[-1]))
    wr = o.trivial_edge((mps[-1], 2), (mpo[-1], 2))
    rights = {L - 1: wr}
    for i in range(L - 1, 0, -1):
        rights[i - 1] = o.compute_right_env(mpo[i], mps[i], rights[i])
    for b in (3, 6):
        Lb, Rb = got[b]
        for dev, ora in ((Lb, lefts[b]), (Rb, rights[b + 1])):
            assert same_structure(dev, ora)
            for (k, x), (_, y) in zip(dev.blocks(), ora.blocks):
                np.testing.assert_allclose(x, y, rtol=1e-11, atol=1e-13)
    del env


def _ed_ground_energy(L, couplings):
    """Lowest eigenvalue of sum J S_i.S_j in the Sz=0 sector (sparse Lanczos)."""
    sp = pytest.importorskip("scipy.sparse")
    spl = pytest.importorskip("scipy.sparse.linalg")
    states = np.array([s for s in range(1 << L) if bin(s).count("1") == L // 2], dtype=np.int64)
    index = {int(s): k for k, s in enumerate(states)}
    rows, cols, vals = [], [], []
    diag = np.zeros(len(states))
    for i, j, J in couplings:
        bi = (states >> (L - 1 - i)) & 1
        bj = (states >> (L - 1 - j)) & 1
        diag += J * np.where(bi == bj, 0.25, -0.25)
        flip = states ^ ((1 << (L - 1 - i)) | (1 << (L - 1 - j)))
        for k in np.nonzero(bi != bj)[0]:
            rows.append(index[int(flip[k])])
            cols.append(k)
            vals.append(0.5 * J)
    n = len(states)
    H = sp.csr_matrix((vals, (rows, cols)), shape=(n, n)) + sp.diags(diag)
    return float(spl.eigsh(H, k=1, which="SA")[0][0])


@pytest.mark.parametrize("compress, gemm, ritz_tol, tol", [(False, "f64", 1e-9, 1e-9), (True, "f64", 1e-9, 1e-9),
                                                           (True, "tf32x3", 1e-4, 1e-7)])
def test_cylinder_dmrg_energy_is_the_state_energy_and_exact(compress, gemm, ritz_tol, tol):
    """4 x 4 snake cylinder at a bond dimension that holds the ground state exactly
    (256 = 2^8): the Ritz energy the sweep reports (k-step and one-step Lanczos) equals
    the FP64 <psi|H|psi>/<psi|psi> of the state the sweep leaves, and that the exact
    ground energy, with the automaton MPO and with the compressed one.  On the mixed
    path the state's FP64 energy is still exact to 1e-7; its Ritz values come from
    split-TF32 matvecs and environments, whose FP32 tensor-core accumulation errs by
    ~1e-6 of a contraction's scale, growing with the contracted length and along the
    chain of environment updates, so they are held to 1e-4 only."""
    Lx, Ly = 4, 4
    mpo = NET.cylinder_heisenberg(Lx, Ly, 1.0, "snake", compress=compress)
    L = len(mpo)
    E_ed = _ed_ground_energy(L, NET.cylinder_couplings(Lx, Ly, 1.0, "snake"))
    mps = NET.random_bMPS(32, mpo, q.conserved.Z(0), seed=3)
    mps.move_oc(0)
    mps.normalize_center()
    for D, steps, sweeps in ((32, 4, 2), (256, 4, 4), (256, 1, 2)):
        log = q.algorithms.dmrg_log_sweeptime()
        q.algorithms.dmrg(mpo, mps, q.algorithms.dmrg_options(
            cutoff=1e-14, convergence_criterion=0.0, max_bond=D, min_bond=1, maximum_iterations=sweeps,
            lanczos_steps=steps, final_energy_fp64=False, gemm=gemm), log)
        e, n2 = q.algorithms.mps_energy(mpo, mps)
        assert log.energies[-1] == pytest.approx(e / n2, rel=ritz_tol, abs=ritz_tol), (D, steps, log.energies, e / n2)
    assert e / n2 == pytest.approx(E_ed, rel=tol, abs=tol)
