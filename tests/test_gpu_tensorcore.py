"""The split-precision tcgen05 grouped GEMMs (pytest -m gpu).

Tolerance: TF32x3 keeps hi*hi + hi*lo + lo*hi, BF16x3 the six products of order <= 2
of the hi / mid / lo bf16 terms; both accumulate in FP32 and reach about FP32
accuracy, so a block product agrees with the FP64 result to 2e-6 relative to the
block's largest magnitude (checked against the oracle)."""
import numpy as np
import pytest

import quantit_gb300 as q
from oracle import qtt_oracle as o
from tests._convert import same_structure, to_device
from tests.test_library_cpu import _contractible_pair

pytestmark = pytest.mark.gpu
TOL = 2e-6


TC_MODES = ("tf32x3", "bf16x3")


@pytest.fixture(params=TC_MODES)
def tc_mode(request):
    q.set_gemm_mode(request.param)
    yield request.param
    q.set_gemm_mode("f64")


def _check(got, want, tol=TOL):
    assert same_structure(got, want)
    blocks = got.blocks()
    assert [k for k, _ in blocks] == [k for k, _ in want.blocks]
    for (k, a), (_, b) in zip(blocks, want.blocks):
        scale = max(float(np.max(np.abs(b))) if b.size else 0.0, 1e-300)
        err = float(np.max(np.abs(a - b))) if b.size else 0.0
        assert err <= tol * scale, (k, err, scale)


def test_tc_gemm_random_layouts(tc_mode):
    rng = np.random.default_rng(21)
    n = 0
    for trial in range(600):
        if n >= 25:
            break
        ra, rb = int(rng.integers(1, 5)), int(rng.integers(1, 5))
        nc = int(rng.integers(0, min(ra, rb) + 1))
        A, B, dA, dB = _contractible_pair(rng, (0,), ra, rb, nc)
        if not A.blocks or not B.blocks:
            continue
        _check(to_device(A).tensordot(to_device(B), (dA, dB)), o.tensordot(A, B, dA, dB))
        n += 1
    assert n >= 10


@pytest.mark.parametrize("sizes", [(40, 70, 33), (130, 257, 129), (300, 190, 200)])
def test_tc_gemm_large_blocks(tc_mode, sizes):
    a, b, c = sizes
    rng = np.random.default_rng(22)
    A = o.btensor([[(a, -1), (b, 0), (c, 1)], [(1, -1), (1, 1)], [(1, -1), (1, 1)], [(c, -2), (b, 0), (a, 2)]],
                  [0], (0,))
    A = o.randn_like(A, rng)
    B = o.btensor([[(c, 2), (b, 0), (a, -2)], [(1, 1), (1, -1)], [(b, 1), (c, -1)]], [0], (0,))
    B = o.randn_like(B, rng)
    for dA, dB in (([3, 2], [0, 1]), ([3], [0]), ([0], [2])):
        try:
            want = o.tensordot(A, B, dA, dB)
        except o.ContractionError:
            continue
        _check(to_device(A).tensordot(to_device(B), (dA, dB)), want, tol=5e-6)


def test_tc_gemm_tensorgdot_epilogue(tc_mode):
    rng = np.random.default_rng(23)
    A, B, dA, dB = _contractible_pair(rng, (0,), 3, 3, 1)
    while not A.blocks or not B.blocks:
        A, B, dA, dB = _contractible_pair(rng, (0,), 3, 3, 1)
    C = o.tensordot(A, B, dA, dB)
    add = o.randn_like(C.empty_like(), rng)
    _check(q.tensorgdot(to_device(add), to_device(A), to_device(B), dA, dB, beta=0.5, alpha=2.0),
           o.tensorgdot(add, A, B, dA, dB, beta=0.5, alpha=2.0), tol=5e-6)


def test_mixed_dmrg_energy_close_to_fp64():
    """Converged runs: the mixed paths (split-TF32 or split-BF16 block GEMMs, FP64-finished sector SVD)
    reports the FP64 variational energy of its final state, which matches the
    plain FP64 path to better than 1e-8 per site.  (Its per-bond Ritz values carry
    ~1e-6 relative noise from FP32 accumulation and are not used for the result.)"""
    for L, D, sweeps in ((10, 64, 10), (16, 64, 12)):
        mpo = o.heisenberg_mpo(L)
        mps = o.right_canonicalize(o.random_mps(L, D, [1, -1], 0, np.random.default_rng(5)))
        dmpo = q.networks.bMPO([to_device(t) for t in mpo])
        res = {}
        for mode in ("f64",) + TC_MODES:
            dmps = q.networks.bMPS([to_device(t) for t in mps], 0)
            res[mode] = q.algorithms.dmrg(dmpo, dmps, q.algorithms.dmrg_options(
                cutoff=1e-10, convergence_criterion=0.0, max_bond=D, min_bond=4, maximum_iterations=sweeps,
                gemm=mode))
            e, n2 = q.algorithms.mps_energy(dmpo, dmps)
            assert abs(n2 - 1.0) < 1e-5
            if mode != "f64":
                assert res[mode] == pytest.approx(e / n2, rel=1e-14)
        for mode in TC_MODES:
            assert abs(res[mode] - res["f64"]) / L < 1e-8, (L, D, mode, res)


@pytest.mark.parametrize("scale_a, scale_b", [(1e-60, 1.0), (1e-30, 1e-30), (1e45, 1e-40), (3e-200, 2e150)])
def test_tc_gemm_operand_magnitudes(tc_mode, scale_a, scale_b):
    # operands far outside the FP32 range: each is scaled by an exact power of two
    # before the split and the product is scaled back in the epilogue
    rng = np.random.default_rng(24)
    A, B, dA, dB = _contractible_pair(rng, (0,), 3, 3, 1)
    while not A.blocks or not B.blocks:
        A, B, dA, dB = _contractible_pair(rng, (0,), 3, 3, 1)
    A = o.scale(A, scale_a)
    B = o.scale(B, scale_b)
    _check(to_device(A).tensordot(to_device(B), (dA, dB)), o.tensordot(A, B, dA, dB))


def test_mixed_dmrg_from_noncanonical_state():
    """random_bmps (like random_bMPS) is not in canonical form: the left environments
    of L=32 shrink to ~1e-60 before the first sweep.  The mixed path must still
    converge to the FP64 path's energy."""
    L, D = 32, 48
    mpo = q.networks.xxz(L, 1.0)
    out = {}
    for gemm in ("f64",) + TC_MODES:
        mps = q.networks.random_bmps(L, D, seed=5)
        opts = q.algorithms.dmrg_options(cutoff=1e-10, convergence_criterion=1e-9, max_bond=D, min_bond=1,
                                         maximum_iterations=20, gemm=gemm, final_energy_fp64=True)
        log = q.algorithms.dmrg_log_sweeptime()
        out[gemm] = q.algorithms.dmrg(mpo, mps, opts, log)
        if gemm != "f64":
            # converged on consecutive FP64 energies before the sweep limit; the returned
            # energy is the state's FP64 energy
            assert len(log.energies) < 20, log.energies
            e, n2 = q.algorithms.mps_energy(mpo, mps)
            assert out[gemm] == pytest.approx(e / n2, rel=1e-12)
            assert log.energies[-1] == out[gemm]
            assert abs(log.energies[-1] - log.energies[-2]) <= 1e-9 * abs(log.energies[-1])
    for gemm in TC_MODES:
        assert np.isfinite(out[gemm])
        assert abs(out[gemm] - out["f64"]) / L < 1e-7, (gemm, out)


@pytest.mark.parametrize("mode", TC_MODES)
def test_persistent_gemm_matches_one_tile_per_cta(mode):
    """Launches of at least two tiles per SM run the persistent kernel (one CTA per SM
    walking the tile list, double-buffered TMEM accumulator).  Each tile's MMA sequence
    is the same as in the one-tile-per-CTA kernel, so the results are identical, and
    they match FP64 products to FP32 accuracy."""
    from quantit_gb300.conserved import Z
    rng = np.random.default_rng(25)
    ns, m, k = 9, 700, 300  # 9 output blocks of 700 x 700: 324 tiles of 128 x 128
    A = q.btensor([[(m, Z(i)) for i in range(ns)], [(k, Z(-i)) for i in range(ns)]], Z(0))
    B = q.btensor([[(k, Z(i)) for i in range(ns)], [(m, Z(-i)) for i in range(ns)]], Z(0))
    a_blocks = [((i, i), rng.standard_normal((m, k))) for i in range(ns)]
    b_blocks = [((i, i), rng.standard_normal((k, m))) for i in range(ns)]
    A.set_blocks(a_blocks)
    B.set_blocks(b_blocks)
    out = {}
    q.set_gemm_mode(mode)
    try:
        for persistent in (False, True):
            q.set_persistent_gemm(persistent)
            out[persistent] = dict(A.tensordot(B, ([1], [0])).blocks())
    finally:
        q.set_persistent_gemm(True)
        q.set_gemm_mode("f64")
    assert out[True].keys() == out[False].keys()
    for key in out[False]:
        np.testing.assert_array_equal(out[True][key], out[False][key])
    for (key, a), (_, b) in zip(a_blocks, b_blocks):
        want = a @ b
        assert float(np.max(np.abs(out[True][key] - want))) <= TOL * float(np.max(np.abs(want))) * 4
