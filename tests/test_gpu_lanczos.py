"""k-step Lanczos bond update (dmrg_options lanczos_steps > 1; pytest -m gpu).

QuantiT's update is one two-vector Krylov step per bond visit; the optional
k-step Lanczos (full two-pass reorthogonalisation, device scalars, host Ritz
solve) converges each bond in one visit.  It reaches the exact ground states of
short chains, needs fewer sweeps than the one-step update, and its mixed path
agrees with FP64."""
import numpy as np
import pytest

import quantit_gb300 as q
from tests.test_models_cpu import _jordan_wigner_hubbard

pytestmark = pytest.mark.gpu
NET = q.networks


def _heisenberg_ed(L):
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
    return np.linalg.eigvalsh(H)[0]


def _run(mpo, mps, k, sweeps, gemm="f64", conv=1e-13, D=16):
    log = q.algorithms.dmrg_log_sweeptime()
    E = q.algorithms.dmrg(mpo, mps, q.algorithms.dmrg_options(cutoff=1e-12, convergence_criterion=conv, max_bond=D,
                                                              min_bond=1, maximum_iterations=sweeps, gemm=gemm,
                                                              lanczos_steps=k), log)
    return E, log.energies


def test_k_step_lanczos_exact_heisenberg_L8():
    L = 8
    e0 = _heisenberg_ed(L)
    mps = NET.random_bmps(L, 16, seed=1)
    mps.move_oc(0)
    mps.normalize_center()
    E, Es = _run(NET.heisenberg(L), mps, 6, 20)
    assert E == pytest.approx(e0, abs=1e-10)
    assert len(Es) <= 8


def test_k_step_lanczos_exact_hubbard_L4_where_one_step_stalls():
    L, U = 4, 8.0
    H, N, Sz2 = _jordan_wigner_hubbard(L, U, 0.0)
    sel = np.where((N == L) & (Sz2 == 0))[0]
    e0 = np.linalg.eigvalsh(H[np.ix_(sel, sel)])[0]
    mpo = NET.hubbard(L, U)
    mk = NET.random_bmps(L, 16, NET.HUBBARD_PHYS, (L, 0), seed=3, mods=(0, 0))
    E, Es = _run(mpo, mk, 8, 20)
    assert E == pytest.approx(e0, abs=1e-9)
    m1 = NET.random_bmps(L, 16, NET.HUBBARD_PHYS, (L, 0), seed=3, mods=(0, 0))
    E1, Es1 = _run(mpo, m1, 1, 20)
    assert E1 - e0 > 100 * (E - e0 + 1e-15)   # the one-step update is still far away


def test_k_step_mixed_matches_fp64():
    L, D = 20, 48
    mpo = NET.heisenberg(L)
    out = {}
    for gemm in ("f64", "tf32x3"):
        mps = NET.random_bmps(L, D, seed=9)
        mps.move_oc(0)
        mps.normalize_center()
        out[gemm], _ = _run(mpo, mps, 4, 30, gemm=gemm, conv=1e-10, D=D)
    assert abs(out["tf32x3"] - out["f64"]) / L < 1e-8, out


@pytest.mark.parametrize("model", ["heisenberg", "hubbard"])
def test_cuda_graph_replay_is_bit_identical(model):
    """The k-step update with the matvec captured once per bond and replayed from a
    CUDA graph gives exactly the energies of the directly launched matvecs (the
    block-width autotuner is off: while it explores, consecutive decompositions of
    one class run different widths and round differently)."""
    q.set_autotune(False)
    out = {}
    for graphs in (False, True):
        if model == "hubbard":
            L, D = 8, 32
            mpo = NET.hubbard(L, 8.0)
            mps = NET.random_bmps(L, D, NET.HUBBARD_PHYS, (L, 0), seed=4, mods=(0, 0))
        else:
            L, D = 16, 32
            mpo = NET.heisenberg(L)
            mps = NET.random_bmps(L, D, seed=4)
        mps.move_oc(0)
        mps.normalize_center()
        log = q.algorithms.dmrg_log_sweeptime()
        q.algorithms.dmrg(mpo, mps, q.algorithms.dmrg_options(cutoff=1e-10, convergence_criterion=0.0, max_bond=D,
                                                              min_bond=1, maximum_iterations=3, lanczos_steps=6,
                                                              cuda_graphs=graphs), log)
        out[graphs] = log.energies
    q.set_autotune(True)
    assert out[True] == out[False]
