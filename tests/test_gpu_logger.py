"""The DMRG logger interface (dmrg_logger, include/dmrg_logger.h:27-185) on the GPU
driver (pytest -m gpu): init once before the first sweep, it_log_all after every
sweep with the current state, end_log_all once at the end with the returned energy,
dmrg_log_simple's middle bond dimension, and the per-sweep largest relative
discarded weight of the truncations against the oracle's."""
import numpy as np
import pytest

import quantit_gb300 as q
from oracle import qtt_oracle as o
from tests._convert import to_device

pytestmark = pytest.mark.gpu


class Recorder(q.algorithms.dmrg_logger):
    def __init__(self):
        self.calls = []

    def init(self, options):
        self.calls.append(("init", options.maximum_iterations))

    def log_truncation(self, weight):
        self.calls.append(("trunc", weight))

    def it_log_all(self, step, energy, mps):
        self.calls.append(("it", step, energy, len(mps), mps.orthogonality_center))

    def end_log_all(self, step, energy, mps):
        self.calls.append(("end", step, energy, len(mps)))


def _state(L, D, seed):
    mpo = o.heisenberg_mpo(L)
    mps = o.right_canonicalize(o.random_mps(L, D, [1, -1], 0, np.random.default_rng(seed)))
    return mpo, mps


def test_logger_call_order_and_arguments():
    L, D, sweeps = 10, 16, 3
    mpo, mps = _state(L, D, 7)
    dmpo = q.networks.bMPO([to_device(t) for t in mpo])
    dmps = q.networks.bMPS([to_device(t) for t in mps], 0)
    rec = Recorder()
    E = q.algorithms.dmrg(dmpo, dmps, q.algorithms.dmrg_options(cutoff=1e-10, convergence_criterion=0.0, max_bond=D,
                                                                 min_bond=4, maximum_iterations=sweeps), rec)
    kinds = [c[0] for c in rec.calls]
    assert kinds == ["init"] + ["trunc", "it"] * sweeps + ["end"]
    assert rec.calls[0] == ("init", sweeps)
    its = [c for c in rec.calls if c[0] == "it"]
    assert [c[1] for c in its] == list(range(sweeps))
    assert all(c[3] == L for c in its)
    end = rec.calls[-1]
    # the loop ran to maximum_iterations: end_log_all gets that count (dmrg.cpp:238-270)
    assert end[1] == sweeps and end[2] == pytest.approx(E, rel=1e-15) and end[3] == L
    assert its[-1][2] == pytest.approx(E, rel=1e-15)


def test_sweeptime_and_simple_loggers():
    L, D = 10, 16
    mpo, mps = _state(L, D, 8)
    dmpo = q.networks.bMPO([to_device(t) for t in mpo])
    opts = q.algorithms.dmrg_options(cutoff=1e-10, convergence_criterion=0.0, max_bond=D, min_bond=4,
                                     maximum_iterations=2)
    st = q.algorithms.dmrg_log_sweeptime()
    q.algorithms.dmrg(dmpo, q.networks.bMPS([to_device(t) for t in mps], 0), opts, st)
    assert len(st.time_list) == len(st.bond_list) == len(st.energies) == 2
    assert all(t > 0 for t in st.time_list)
    simple = q.algorithms.dmrg_log_simple()
    dm = q.networks.bMPS([to_device(t) for t in mps], 0)
    q.algorithms.dmrg(dmpo, dm, opts, simple)
    mid = dm[L // 2].sizes()
    assert simple.middle_bond_dim == max(mid[0], mid[2]) == st.bond_list[-1]
    assert simple.it_num == 2


def test_truncated_weight_matches_oracle():
    """A bond dimension below the state's: every sweep truncates.  The per-sweep
    largest relative discarded weight agrees with the oracle's run (FP64 path)."""
    L, D, Dmax = 12, 24, 10
    mpo, mps = _state(L, D, 9)
    dmpo = q.networks.bMPO([to_device(t) for t in mpo])
    dmps = q.networks.bMPS([to_device(t) for t in mps], 0)
    st = q.algorithms.dmrg_log_sweeptime()
    q.algorithms.dmrg(dmpo, dmps, q.algorithms.dmrg_options(cutoff=1e-10, convergence_criterion=0.0,
                                                             max_bond=Dmax, min_bond=4, maximum_iterations=3), st)
    opt = o.DmrgOptions(cutoff=1e-10, convergence_criterion=0.0, maximum_bond=Dmax, minimum_bond=4,
                        maximum_iterations=3)
    o.dmrg(mpo, [t for t in mps], 0, opt)
    assert all(w > 1e-12 for w in st.truncated_weights)
    np.testing.assert_allclose(st.truncated_weights, opt.truncated_weights, rtol=1e-6)


def test_logger_exception_reaches_the_caller():
    L, D = 8, 8
    mpo, mps = _state(L, D, 10)

    class Boom(q.algorithms.dmrg_logger):
        def it_log_all(self, step, energy, mps):
            raise KeyError("from the logger")
    dmpo = q.networks.bMPO([to_device(t) for t in mpo])
    with pytest.raises(KeyError):
        q.algorithms.dmrg(dmpo, q.networks.bMPS([to_device(t) for t in mps], 0),
                          q.algorithms.dmrg_options(cutoff=1e-10, convergence_criterion=0.0, max_bond=D,
                                                    maximum_iterations=1), Boom())
