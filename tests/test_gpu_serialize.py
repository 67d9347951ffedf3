"""Checkpoint / resume on the GPU (pytest -m gpu): an MPS and its MPO written to a
block-list file and read back are bit-identical, and a DMRG resumed from the
checkpoint gives exactly the energies of the uninterrupted run."""
import numpy as np
import pytest

import quantit_gb300 as q
from quantit_gb300 import serialize

pytestmark = pytest.mark.gpu


def test_mps_round_trip_bit_exact(tmp_path):
    mps = q.networks.random_bmps(12, 24, q.networks.HUBBARD_PHYS, (12, 0), seed=2, mods=(0, 0))
    serialize.save(tmp_path / "psi.npz", mps)
    back = serialize.load(tmp_path / "psi.npz")
    assert back.orthogonality_center == mps.orthogonality_center
    for a, b in zip(mps, back):
        assert a.structure()[1] == b.structure()[1]
        ba, bb = a.blocks(), b.blocks()
        assert [k for k, _ in ba] == [k for k, _ in bb]
        for (_, x), (_, y) in zip(ba, bb):
            assert np.array_equal(x, y)


def test_dmrg_resumes_from_checkpoint(tmp_path):
    L, D = 16, 32
    mpo = q.networks.heisenberg(L)
    opts = q.algorithms.dmrg_options(cutoff=1e-10, convergence_criterion=0.0, max_bond=D, min_bond=2,
                                     maximum_iterations=2)
    ref = q.networks.random_bmps(L, D, seed=8)
    ref.move_oc(0)
    ref.normalize_center()
    start = q.networks.bMPS(list(ref), ref.orthogonality_center)
    q.algorithms.dmrg(mpo, ref, opts)
    serialize.save(tmp_path / "ckpt.npz", ref)
    serialize.save(tmp_path / "mpo.npz", mpo)
    E1 = q.algorithms.dmrg(mpo, ref, opts)
    resumed = serialize.load(tmp_path / "ckpt.npz")
    mpo2 = serialize.load(tmp_path / "mpo.npz")
    E2 = q.algorithms.dmrg(mpo2, resumed, opts)
    assert E1 == E2
    assert len(start) == L


def test_serving_checkpoint_and_resume(tmp_path):
    from quantit_gb300 import serving
    reqs = [serving.SolveRequest(i, 12, 0.5 + 0.5 * i, 16, seed=20 + i) for i in range(3)]
    eng = serving.ServingEngine(slots=3, checkpoint_dir=str(tmp_path), convergence=1e-9, max_sweeps=30)
    first = eng.run(reqs, realtime=False)
    assert all(r.error is None for r in first)
    again = [serving.SolveRequest(r.rid, r.L, r.delta, r.D, seed=0, resume=str(tmp_path / f"request_{r.rid}.npz"))
             for r in reqs]
    second = serving.ServingEngine(slots=3, convergence=1e-9, max_sweeps=30).run(again, realtime=False)
    for a, b in zip(first, second):
        assert b.error is None
        # resumed from a converged state: converges at once to the same energy
        assert b.sweeps <= a.sweeps
        assert abs(a.energy - b.energy) / a.L < 1e-8
