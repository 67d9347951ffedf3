"""The C-ABI library on a machine without a GPU: it loads, exports every entry
point of include/qtt_gb300.h, and its host planner emits exactly the oracle's
block structures (structure-only btensors never touch the device)."""
import itertools
import json
import os
import re

import numpy as np
import pytest

import quantit_gb300 as q
from oracle import qtt_oracle as o
from tests._convert import same_structure, to_device

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KNOWN = json.load(open(os.path.join(ROOT, "tests", "golden", "reference_known_answers.json")))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "qtt_gb300.h")).read()
    return sorted(set(re.findall(r"\b(qtt_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    L = q.lib()
    names = declared_symbols()
    assert len(names) >= 45
    for n in names:
        assert hasattr(L, n), n
    assert b"sm_103a" in L.qtt_version()


def _random_tensor(rng, rank, mods, nsec=(1, 4), qrange=3, sizes=(1, 3), density=0.7):
    legs = []
    for _ in range(rank):
        ns = int(rng.integers(nsec[0], nsec[1] + 1))
        leg = []
        for _ in range(ns):
            qv = [int(rng.integers(-qrange, qrange + 1)) for _ in mods]
            leg.append((int(rng.integers(sizes[0], sizes[1] + 1)), qv))
        legs.append(leg)
    t = o.btensor(legs, [0] * len(mods), mods)
    allowed = o.allowed_blocks(t)
    if not allowed:
        return t
    # choose a selection rule that some block satisfies
    idx = allowed[int(rng.integers(len(allowed)))] if allowed else None
    t.sel = t.block_charge_sum(idx) if idx else t.sel
    allowed = o.allowed_blocks(t)
    keep = [a for a in allowed if rng.random() < density] or allowed[:1]
    t.blocks = [(k, rng.standard_normal(t.block_shape(k))) for k in keep]
    return t


def _partner(rng, A, dims, rank, mods, density=0.7):
    """A tensor whose legs `dims` contract with A's legs `dimsA`."""
    return None


def _contractible_pair(rng, mods, ra, rb, ncontr):
    A = _random_tensor(rng, ra, mods)
    dA = sorted(rng.choice(ra, size=ncontr, replace=False).tolist())
    rng.shuffle(dA)
    # build B with legs matching A's contracted legs (inverted charges), other legs random
    legs = []
    dB = sorted(rng.choice(rb, size=ncontr, replace=False).tolist())
    rng.shuffle(dB)
    slot = {b: a for a, b in zip(dA, dB)}
    for d in range(rb):
        if d in slot:
            a = slot[d]
            legs.append([(n, list(o.q_inv(c, mods))) for n, c in zip(A.sec_sizes(a), A.sec_charges(a))])
        else:
            ns = int(rng.integers(1, 4))
            legs.append([(int(rng.integers(1, 3)), [int(rng.integers(-3, 4)) for _ in mods]) for _ in range(ns)])
    B = o.btensor(legs, [0] * len(mods), mods)
    allowed = o.allowed_blocks(B)
    if allowed:
        B.sel = B.block_charge_sum(allowed[int(rng.integers(len(allowed)))])
        allowed = o.allowed_blocks(B)
        keep = [a for a in allowed if rng.random() < 0.7] or allowed[:1]
        B.blocks = [(k, rng.standard_normal(B.block_shape(k))) for k in keep]
    return A, B, dA, dB


def test_planner_known_answer_contraction():
    k = KNOWN["tensordot_blocks"]
    A = o.btensor(k["A_legs"], [k["A_sel"]], (5,))
    A.blocks = [(tuple(b), None) for b in k["A_blocks"]]
    B = o.btensor(k["B_legs"], [k["B_sel"]], (5,))
    B.blocks = [(tuple(b), None) for b in k["B_blocks"]]
    C = to_device(A, True).tensordot(to_device(B, True), ([1], [1]))
    assert [list(i) for i in C.block_indices()] == k["C_blocks"]
    assert not C.has_data()


@pytest.mark.parametrize("mods", [(0,), (5,), (0, 0), (0, 2)])
def test_planner_matches_oracle_block_lists(mods):
    rng = np.random.default_rng(hash(mods) % 1000)
    for trial in range(40):
        ra = int(rng.integers(1, 5))
        rb = int(rng.integers(1, 5))
        nc = int(rng.integers(0, min(ra, rb) + 1))
        A, B, dA, dB = _contractible_pair(rng, mods, ra, rb, nc)
        if not A.blocks or not B.blocks:
            continue
        want, plan, _, _ = o.tdot_plan(A, B, dA, dB)
        want_blocks = sorted(oidx for oidx, _ in plan)
        got = to_device(A, True).tensordot(to_device(B, True), (dA, dB))
        assert same_structure(got, want)
        assert got.block_indices() == want_blocks, (trial, dA, dB)


def test_planner_reshape_permute_structures():
    rng = np.random.default_rng(3)
    for trial in range(30):
        mods = [(0,), (3,), (0, 0)][trial % 3]
        r = int(rng.integers(2, 5))
        T = _random_tensor(rng, r, mods)
        if not T.blocks:
            continue
        D = to_device(T, True)
        perm = rng.permutation(r).tolist()
        P = D.permute(perm)
        Po = o.permute(T, perm)
        assert same_structure(P, Po)
        assert P.block_indices() == [k for k, _ in Po.blocks]
        split = int(rng.integers(1, r))
        R = D.reshape([split])
        Ro = o.reshape(T, [split])
        assert same_structure(R, Ro)
        assert R.block_indices() == [k for k, _ in Ro.blocks]
        back = R.reshape_as(D)
        assert back.block_indices() == D.block_indices()


def test_svd_structure_matches_oracle():
    rng = np.random.default_rng(4)
    for trial in range(20):
        mods = [(0,), (4,)][trial % 2]
        T = _random_tensor(rng, 4, mods, nsec=(1, 3))
        if not T.blocks:
            continue
        U, d, V = o.svd_split(T, 2)
        Ud, dd, Vd = q.linalg.svd(to_device(T, True), 2)
        for got, want in ((Ud, U), (dd, d), (Vd, V)):
            assert same_structure(got, want)
            assert got.block_indices() == [k for k, _ in want.blocks]


def test_contraction_errors_map_to_reference_exceptions():
    k = KNOWN["tensordot_blocks"]
    A = o.btensor(k["A_legs"], [k["A_sel"]], (5,))
    A.blocks = [(tuple(b), None) for b in k["A_blocks"]]
    Ad = to_device(A, True)
    with pytest.raises(RuntimeError, match="sum to zero"):
        Ad.tensordot(Ad, ([1], [1]))
    with pytest.raises(RuntimeError, match="same length"):
        Ad.tensordot(Ad, ([0, 1], [0]))
    bad = q.btensor([[(2, q.conserved.C5(0)), (3, q.conserved.C5(1))], [(2, q.conserved.C5(0)), (3, q.conserved.C5(-1))]],
                    q.conserved.C5(0))
    with pytest.raises(ValueError, match="not allowed"):
        bad.set_block_structure([(1, 0)])


def _legs_tensor(legs, mods, sel):
    return o.fill(o.btensor(legs, sel, mods), np.zeros)


@pytest.mark.parametrize("mods", [(0,), (0, 0), (3,)])
def test_reshape_as_acceptance_matches_oracle(mods):
    """reshape_as checks charge and size compatibility at every block position
    (btensor.cpp:2876-2934); the library checks it group by group.  Both must accept
    and reject the same layouts, including offsets that cancel across groups."""
    rng = np.random.default_rng(31 + len(mods) + mods[0])
    nc = len(mods)

    def charge():
        return tuple(int(rng.integers(0, m)) if m else int(rng.integers(-2, 3)) for m in mods)

    def shift(c, s):
        return tuple(((x + s) % m) if m else x + s for x, m in zip(c, mods))

    zero = tuple(0 for _ in mods)
    n = 0
    for trial in range(60):
        r = int(rng.integers(2, 5))
        legs = [[(int(rng.integers(1, 4)), charge()) for _ in range(int(rng.integers(1, 4)))] for _ in range(r)]
        T = _legs_tensor(legs, mods, zero)
        if not T.blocks:
            continue
        split = int(rng.integers(1, r))
        R = o.reshape(T, [split])
        variants = []
        # 1. the original layout (compatible)
        variants.append(legs)
        # 2. per-leg charge offsets that cancel across the split (compatible: every position's total is unchanged)
        s = int(rng.integers(1, 3))
        v = [[(sz, shift(c, s if d == 0 else 0)) for sz, c in leg] for d, leg in enumerate(legs)]
        v[-1] = [(sz, shift(c, -s)) for sz, c in v[-1]]
        variants.append(v)
        # 3. one section's charge changed (incompatible unless the change is invisible)
        v = [list(leg) for leg in legs]
        d = int(rng.integers(0, r))
        j = int(rng.integers(0, len(v[d])))
        v[d][j] = (v[d][j][0], shift(v[d][j][1], 1))
        variants.append(v)
        # 4. two section sizes swapped between legs (sizes move between groups)
        v = [list(leg) for leg in legs]
        if len(v[0]) > 1:
            v[0][0], v[0][1] = (v[0][1][0], v[0][0][1]), (v[0][0][0], v[0][1][1])
        variants.append(v)
        for lv in variants:
            S = o.btensor(lv, zero, mods)
            want = None
            try:
                o.reshape_as(R, S)
            except ValueError as e:
                want = str(e)
            dR = to_device(R, True)
            dS = q.btensor([[(sz, q.conserved.quantity(c, mods)) for sz, c in leg] for leg in lv],
                           q.conserved.quantity(zero, mods))
            got = None
            try:
                dR.reshape_as(dS)
            except ValueError as e:
                got = str(e)
            assert (want is None) == (got is None), (legs, lv, want, got)
            n += 1
    assert n > 50


def test_tuning_switches_and_dmrg_options_round_trip():
    """The tuning switches with no reference counterpart (persistent GEMM, SVD deflation,
    autotuner, Jacobi kernel, planner) are plain host settings: they take effect without a GPU, and
    dmrg_options carries the build's extra fields into the C struct unchanged."""
    import quantit_gb300 as q
    for on in (False, True):
        q.set_persistent_gemm(on)
        q.set_svd_deflation(on)
        q.set_autotune(on)
    q.set_svd_deflation(True)   # the default
    for kernel in ("scalar", "block"):
        q.set_jacobi_kernel(kernel)
    with pytest.raises(ValueError):
        q.set_jacobi_kernel(7)
    # the planner switch: every mode is accepted without a GPU (with no device the
    # host plans), unknown modes and negative thresholds are refused
    for mode in ("host", "device", "auto"):
        q.set_planner(mode, 512)
    with pytest.raises(ValueError):
        q.set_planner("gpu")
    with pytest.raises(ValueError):
        q.set_planner("auto", -1)
    q.set_planner("host", 3000)   # the default
    st = q.planner_stats(reset=True)
    assert set(st) == {"host_calls", "device_calls", "device_fallbacks", "host_s", "device_s"}
    o = q.algorithms.dmrg_options(gemm="bf16x3", lanczos_steps=4, cuda_graphs=False, svd_warm_start=False,
                                  final_energy_fp64=False)._c()
    assert (o.gemm_mode, o.lanczos_steps, o.cuda_graphs, o.svd_warm_start, o.final_energy_fp64) == (2, 4, 0, 0, 0)
    d = q.algorithms.dmrg_options()._c()
    assert (d.gemm_mode, d.lanczos_steps, d.cuda_graphs, d.svd_warm_start, d.final_energy_fp64) == (0, 1, 1, 1, 1)
