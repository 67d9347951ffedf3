"""random_bMPS on the GPU (sources/MPT.cpp:424-462; pytest -m gpu): bond sectors
equal to the host builder's (charge multiplicities capped to the bond dimension),
unit-norm sites with N(0, 1)-distributed entries, the same tensors for the same seed,
and a state DMRG optimises to the exact ground energy."""
import numpy as np
import pytest

import quantit_gb300 as q
from quantit_gb300.conserved import Z, quantity
from tests._convert import structure_of

pytestmark = pytest.mark.gpu
NET = q.networks


@pytest.mark.parametrize("model", ["heisenberg", "hubbard"])
def test_structure_matches_host_builder(model):
    if model == "heisenberg":
        L, D = 12, 20
        mpo = NET.heisenberg(L)
        dev = NET.random_bMPS(D, mpo, Z(0), seed=3)
        host = NET.random_bmps(L, D, seed=3)
    else:
        L, D = 8, 32
        mpo = NET.hubbard(L, 8.0)
        dev = NET.random_bMPS(D, mpo, quantity((L, 0), (0, 0)), seed=3)
        host = NET.random_bmps(L, D, NET.HUBBARD_PHYS, (L, 0), seed=3, mods=(0, 0))
    assert dev.orthogonality_center == L - 1
    for a, b in zip(dev, host):
        assert structure_of(a) == structure_of(b)
        assert a.block_indices() == b.block_indices()
        assert q.dot_all(a, a) == pytest.approx(1.0, rel=1e-12)


def test_entries_are_normal_and_seeded():
    mpo = NET.heisenberg(16)
    a = NET.random_bMPS(64, mpo, Z(0), seed=11)
    b = NET.random_bMPS(64, mpo, Z(0), seed=11)
    c = NET.random_bMPS(64, mpo, Z(0), seed=12)
    for x, y in zip(a, b):
        for (k1, v1), (k2, v2) in zip(x.blocks(), y.blocks()):
            assert k1 == k2 and np.array_equal(v1, v2)
    vals = np.concatenate([v.ravel() for _, v in a[8].blocks()])
    z = vals / np.sqrt(np.mean(vals ** 2))          # undo the unit-norm scaling
    assert abs(np.mean(z)) < 4.0 / np.sqrt(z.size)
    assert np.mean(z ** 4) == pytest.approx(3.0, abs=0.3)   # Gaussian kurtosis
    assert not np.array_equal(np.concatenate([v.ravel() for _, v in c[8].blocks()]), vals)


def test_dmrg_from_random_bmps_reaches_the_ground_state():
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
    mpo = NET.heisenberg(L)
    mps = NET.random_bMPS(16, mpo, Z(0), seed=5)
    mps.move_oc(0)
    mps.normalize_center()
    E = q.algorithms.dmrg(mpo, mps, q.algorithms.dmrg_options(cutoff=1e-12, convergence_criterion=1e-13,
                                                              max_bond=16, maximum_iterations=30))
    assert E == pytest.approx(e0, abs=1e-9)
