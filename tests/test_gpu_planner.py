"""The device-side block-sparsity planner (pytest -m gpu).

tensordot's charge check and merge-join (sources/btensor.cpp:783-883,1998-2110) run
on the GPU (csrc/planner.cu) and must emit the host planner's output block list and
pair order bit for bit: the same block list as the oracle, the same values to the
last bit (the pairs are accumulated in the same order), the same errors, and the
same DMRG energies."""
import numpy as np
import pytest

import quantit_gb300 as q
from oracle import qtt_oracle as o
from tests._convert import same_structure, to_device
from tests.test_library_cpu import _contractible_pair

pytestmark = pytest.mark.gpu
NET = q.networks


def _host_and_device(fn):
    """fn() planned on the host, then on the device; the device run's planner counts."""
    try:
        q.set_planner("host")
        h = fn()
        q.planner_stats(reset=True)
        q.set_planner("device")
        d = fn()
        st = q.planner_stats(reset=True)
    finally:
        q.set_planner("host", 3000)
    return h, d, st


def _bit_identical(h, d):
    assert h.block_indices() == d.block_indices()
    for (k1, x), (k2, y) in zip(h.blocks(), d.blocks()):
        assert k1 == k2
        assert np.array_equal(x, y), k1


@pytest.mark.parametrize("mods", [(0,), (5,), (0, 0), (0, 2)])
def test_device_planner_matches_oracle_and_host(mods):
    rng = np.random.default_rng(17 + sum(mods) + len(mods))
    n_dev = 0
    for trial in range(900):
        if n_dev >= 12:
            break
        ra, rb = int(rng.integers(1, 5)), int(rng.integers(1, 5))
        nc = int(rng.integers(0, min(ra, rb) + 1))
        A, B, dA, dB = _contractible_pair(rng, mods, ra, rb, nc)
        if not A.blocks or not B.blocks:
            continue
        want, plan, _, _ = o.tdot_plan(A, B, dA, dB)
        Ad, Bd = to_device(A), to_device(B)
        h, d, st = _host_and_device(lambda: Ad.tensordot(Bd, (dA, dB)))
        assert same_structure(d, want)
        assert d.block_indices() == sorted(oidx for oidx, _ in plan), (trial, dA, dB)
        _bit_identical(h, d)
        if nc > 0:
            assert (st["device_calls"], st["device_fallbacks"], st["host_calls"]) == (1, 0, 0)
            n_dev += 1
    assert n_dev >= 8


@pytest.mark.parametrize("D", [512, 2048])
def test_device_planner_on_the_theta_pair(D):
    """Config-2 operands (17 charge sectors per bond leg, ~10^3 blocks each): planned
    over one and two legs of A against B and over two and three legs of A against its
    conjugate (structure only: the two-leg product has D^4 elements), and computed with
    data where the product is small enough."""
    A, B = NET.theta_pair(D, seed=3)
    sa = A.copy_structure().set_block_structure(A.block_indices())
    sb = B.copy_structure().set_block_structure(B.block_indices())
    sc = sa.conj()
    plans = [lambda: sa.tensordot(sb, ([3], [0])), lambda: sa.tensordot(sb, ([2, 3], [1, 0])),
             lambda: sa.tensordot(sc, ([1, 2], [1, 2])), lambda: sa.tensordot(sc, ([0, 1, 2], [0, 1, 2]))]
    for fn in plans:
        h, d, st = _host_and_device(fn)
        assert h.block_indices() == d.block_indices()
        assert st["device_calls"] == 1 and st["device_fallbacks"] == 0
    Ac = A.conj()
    for fn in (lambda: A.tensordot(B, ([2, 3], [1, 0])), lambda: A.tensordot(Ac, ([0, 1, 2], [0, 1, 2]))):
        h, d, st = _host_and_device(fn)
        _bit_identical(h, d)
        assert st["device_calls"] == 1 and st["device_fallbacks"] == 0


def test_device_planner_structure_only_and_errors():
    """Structure-only operands plan without data; a contracted section pair whose
    charges do not cancel, or whose sizes differ, raises the host planner's error."""
    A, B = NET.theta_pair(256, seed=5)
    sa = A.copy_structure().set_block_structure(A.block_indices())
    sb = B.copy_structure().set_block_structure(B.block_indices())
    h, d, _ = _host_and_device(lambda: sa.tensordot(sb, ([2, 3], [1, 0])))
    assert h.block_indices() == d.block_indices()
    assert not d.has_data()
    # A's leg 1 (spin charges +1, -1) against B's leg 2 (the same charges): no cancellation
    msgs = []
    for mode in ("host", "device"):
        q.set_planner(mode)
        try:
            with pytest.raises(RuntimeError, match="sum to zero") as e:
                sa.tensordot(sb, ([1], [2]))
            msgs.append(str(e.value))
        finally:
            q.set_planner("host", 3000)
    assert msgs[0] == msgs[1]


def test_dmrg_energies_identical_with_either_planner():
    """Hubbard L=8, D=48 (U(1)xU(1) charges, hundreds of blocks per contraction): the
    sweep energies and the final state agree bit for bit between the two planners."""
    L, D = 8, 48
    mpo = NET.hubbard(L, 8.0)
    out = {}
    for mode in ("host", "device"):
        q.set_planner(mode)
        try:
            mps = NET.random_bmps(L, D, NET.HUBBARD_PHYS, (L, 0), seed=2, mods=(0, 0))
            log = q.algorithms.dmrg_log_sweeptime()
            q.planner_stats(reset=True)
            q.algorithms.dmrg(mpo, mps, q.algorithms.dmrg_options(cutoff=1e-10, convergence_criterion=0.0,
                                                                  max_bond=D, min_bond=2, maximum_iterations=3),
                              log)
            out[mode] = (list(log.energies), [t.blocks() for t in mps], q.planner_stats(reset=True))
        finally:
            q.set_planner("host", 3000)
    assert out["host"][0] == out["device"][0]
    for th, td in zip(out["host"][1], out["device"][1]):
        assert [k for k, _ in th] == [k for k, _ in td]
        for (_, x), (_, y) in zip(th, td):
            assert np.array_equal(x, y)
    assert out["device"][2]["device_calls"] > 0
    assert out["host"][2]["device_calls"] == 0
