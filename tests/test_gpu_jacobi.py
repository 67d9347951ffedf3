"""Both sector-SVD Jacobi kernels against LAPACK's SVD (pytest -m gpu).

The block-cyclic kernel (column blocks of 16 (FP32) or 8 (FP64) in shared
memory, one CTA per block pair and grid step) is the default; the scalar kernel
(one column pair per warp and grid step) serves sectors with columns too long
for shared memory.  Both must give the same decomposition as numpy's SVD for
sector shapes that exercise ragged last blocks, odd block counts (a phantom
block in the round-robin), sectors narrower than one block, wide sectors
(decomposed as A^T), graded and rank-deficient spectra.  The mixed path (FP32
sweeps, then FP64 sweeps from the FP32 rotation made orthogonal in FP64) is held
to the same FP64 tolerances."""
import numpy as np
import pytest

import quantit_gb300 as q
from oracle import qtt_oracle as o
from quantit_gb300.conserved import Z

pytestmark = pytest.mark.gpu

SHAPES = [(1, 1), (5, 3), (3, 5), (16, 16), (17, 16), (16, 33), (40, 33), (100, 47), (250, 260), (300, 31),
          (129, 140)]


def _matrix(rng, m, n, kind):
    k = min(m, n)
    if kind == "graded":
        s = np.logspace(0, -9, k)
    elif kind == "deficient":
        s = np.concatenate([rng.uniform(0.5, 2.0, max(1, k // 3)), np.zeros(k - max(1, k // 3))])
    else:
        return rng.standard_normal((m, n))
    u, _ = np.linalg.qr(rng.standard_normal((m, k)))
    v, _ = np.linalg.qr(rng.standard_normal((n, k)))
    return (u * s) @ v.T


def _sector_tensor(rng, shapes):
    kinds = ["random", "graded", "deficient"]
    blocks = [((i, i), _matrix(rng, m, n, kinds[i % 3])) for i, (m, n) in enumerate(shapes)]
    legs = [[(m, Z(i)) for i, (m, _) in enumerate(shapes)], [(n, Z(-i)) for i, (_, n) in enumerate(shapes)]]
    t = q.btensor(legs, Z(0))
    t.set_blocks(blocks)
    return t, blocks


def _svd_with(t, kernel, mode):
    q.set_jacobi_kernel(kernel)
    q.set_gemm_mode(mode)
    try:
        return q.linalg.svd(t)
    finally:
        q.set_jacobi_kernel("block")
        q.set_gemm_mode("f64")


def _check(t, blocks, out, mode):
    U, d, V = out
    # LAPACK agreement to 1e-12 of the sector's largest singular value, for the plain
    # FP64 path and the mixed path (whose FP32 sweeps are finished in FP64) alike
    rtol = 1e-12
    dv = dict(d.blocks())
    new_section = {k[0]: k[1] for k, _ in U.blocks()}  # sector (row section) -> section of the new leg
    for i, (_, a) in enumerate(blocks):
        want = np.linalg.svd(a, compute_uv=False)
        got = dv[(new_section[i],)]
        np.testing.assert_allclose(got, want, atol=rtol * max(want[0], 1e-300) * 4, rtol=0, err_msg=str(a.shape))
    R = U.mul(d).tensordot(V.conj(), ([1], [1]))
    got = dict(R.blocks())
    for k, a in blocks:
        np.testing.assert_allclose(got[k], a, atol=10 * rtol * float(np.max(np.abs(a))), rtol=0, err_msg=str(a.shape))
    nd = sum(d.section_sizes)
    iso = 1e-11
    assert q.dot_all(U, U) == pytest.approx(nd, rel=iso)
    assert q.dot_all(V, V) == pytest.approx(nd, rel=iso)


@pytest.mark.parametrize("mode", ["f64", "tf32x3"])
@pytest.mark.parametrize("kernel", ["block", "scalar"])
def test_sector_svd_kernels_match_lapack(kernel, mode):
    rng = np.random.default_rng(77)
    t, blocks = _sector_tensor(rng, SHAPES)
    _check(t, blocks, _svd_with(t, kernel, mode), mode)


@pytest.mark.parametrize("mode", ["f64", "tf32x3"])
def test_sector_svd_block_width_limits(mode):
    # the longest column decides the kernel: 1000 (both block widths), 1600 (FP32
    # block kernel, FP64 falls back to the scalar kernel), 2100 (scalar for both)
    rng = np.random.default_rng(78)
    for p in (1000, 1600, 2100):
        t, blocks = _sector_tensor(rng, [(p, 24), (40, 70), (9, 9)])
        _check(t, blocks, _svd_with(t, "block", mode), mode)


def test_block_and_scalar_kernels_agree():
    rng = np.random.default_rng(79)
    t, _ = _sector_tensor(rng, SHAPES)
    a = _svd_with(t, "block", "f64")
    b = _svd_with(t, "scalar", "f64")
    for x, y in zip(a[1].blocks(), b[1].blocks()):
        np.testing.assert_allclose(x[1], y[1], rtol=0, atol=1e-13 * max(float(np.max(y[1])), 1e-300))


def test_autotuner_times_both_widths_and_results_stay_exact():
    """The block-width autotuner runs each candidate width on the first calls of a
    class of decompositions; every one of those calls is an exact SVD, and the
    class ends up with a decision."""
    q.set_autotune(True)
    rng = np.random.default_rng(80)
    t, blocks = _sector_tensor(rng, [(200, 180), (150, 150), (90, 60), (33, 31)])
    for _ in range(5):
        _check(t, blocks, _svd_with(t, "block", "tf32x3"), "tf32x3")
    rep = q.autotune_report()
    assert "fp32 R=8 " in rep and "tuned" in rep, rep


def _last_sweeps():
    import ctypes as C
    buf = (C.c_int32 * 4096)()
    n = C.c_int32()
    assert q.lib().qtt_last_svd_sweeps(buf, 4096, C.byref(n)) == 0
    return list(buf[:n.value])


def _low_rank_tensor(rng, shapes, ranks):
    blocks = []
    for i, ((m, n), r) in enumerate(zip(shapes, ranks)):
        k = min(m, n)
        # r resolved values over five decades, the rest far below FP32 resolution
        s = np.concatenate([np.logspace(0, -5, r), 1e-10 * rng.uniform(size=k - r)])
        u, _ = np.linalg.qr(rng.standard_normal((m, k)))
        v, _ = np.linalg.qr(rng.standard_normal((n, k)))
        blocks.append(((i, i), (u * s) @ v.T))
    legs = [[(m, Z(i)) for i, (m, _) in enumerate(shapes)], [(n, Z(-i)) for i, (_, n) in enumerate(shapes)]]
    t = q.btensor(legs, Z(0))
    t.set_blocks(blocks)
    return t, blocks


def _isometry_error(F):
    """max |F^H F - I| over the new (last) leg's sectors of a factor."""
    cols = {}
    for k, b in F.blocks():
        cols.setdefault(k[-1], []).append(b.reshape(-1, b.shape[-1]))
    err = 0.0
    for v in cols.values():
        m = np.concatenate(v, axis=0)
        err = max(err, float(np.max(np.abs(m.T @ m - np.eye(m.shape[1])))))
    return err


@pytest.mark.parametrize("defl", [False, True])
@pytest.mark.parametrize("kernel", ["block", "scalar"])
def test_mixed_truncated_svd_is_fp64_accurate(kernel, defl):
    """svd with a cutoff on the mixed path: FP32 sweeps, then FP64 sweeps from the
    FP32 rotation made orthogonal in FP64.  All values, including those far below
    FP32 resolution, match LAPACK to 1e-12 of their sector's largest; the kept
    factors are isometries to FP64 precision; the FP64 stage needs fewer sweeps than
    a plain FP64 decomposition from the identity.  With deflation on, numerically null
    columns leave the sweeps and the FP64 sweeps still resolve everything else."""
    rng = np.random.default_rng(81)
    shapes, ranks = [(150, 130), (90, 80), (40, 40), (12, 9)], [30, 20, 10, 9]
    t, blocks = _low_rank_tensor(rng, shapes, ranks)
    q.set_autotune(False)
    q.set_jacobi_kernel(kernel)
    q.set_svd_deflation(defl)
    try:
        q.linalg.svd(t, 1, 1e-14, min_size=1, max_size=10 ** 6)
        plain_sweeps = _last_sweeps()
        assert q.linalg.last_svd_sweeps(fp32_stage=True) == []
        q.set_gemm_mode("tf32x3")
        U, d, V = q.linalg.svd(t, 1, 1e-14, min_size=1, max_size=10 ** 6)
        fp64_sweeps = _last_sweeps()
        fp32_sweeps = q.linalg.last_svd_sweeps(fp32_stage=True)
    finally:
        q.set_jacobi_kernel("block")
        q.set_gemm_mode("f64")
        q.set_svd_deflation(True)   # the default
        q.set_autotune(True)
    assert len(fp32_sweeps) == len(fp64_sweeps) == len(blocks)
    if not defl:
        assert max(fp64_sweeps) < max(plain_sweeps), (fp64_sweeps, plain_sweeps)
    new_section = {k[0]: k[1] for k, _ in U.blocks()}
    dv = dict(d.blocks())
    for i, (_, a) in enumerate(blocks):
        want = np.linalg.svd(a, compute_uv=False)
        got = dv[(new_section[i],)]
        assert len(got) >= int(np.sum(want > 1e-12 * want[0]))
        np.testing.assert_allclose(got, want[:len(got)], atol=1e-12 * want[0], rtol=0)
    assert _isometry_error(U) < 1e-11
    assert _isometry_error(V) < 1e-11
    R = dict(U.mul(d).tensordot(V.conj(), ([1], [1])).blocks())
    for k, a in blocks:
        np.testing.assert_allclose(R[k], a, atol=1e-12 * float(np.max(np.abs(a))), rtol=0)


@pytest.mark.parametrize("kernel", ["block", "scalar"])
def test_truncation_aware_fp64_stage_keeps_fp64_accuracy(kernel):
    """A truncation to a quarter of the values (max_size), with every sector's spectrum
    spread over 13 decades: the threshold lies far above FP32 resolution, so the mixed
    path's FP64 stage leaves the columns below half its estimate out of the sweeps
    (pairs of two of them in the decoupling sweep, every pair of theirs afterwards).  A
    variant that also skipped pairs of a kept column with a discarded one 2^14 times
    smaller shifted the kept values by up to 7e-12 of the largest: the columns the FP32
    sweeps deflated are not decoupled from the kept ones.  The kept values match LAPACK to
    1e-12 of the largest, the kept singular vectors match LAPACK's to 1e-10, the kept
    factors are isometries to FP64 precision, and the plain FP64 path keeps the same."""
    rng = np.random.default_rng(97)
    shapes = [(160, 140), (120, 100), (90, 90), (40, 30)]
    blocks, ref = [], []
    for i, (m, n) in enumerate(shapes):
        k = min(m, n)
        sv = np.logspace(0, -13, k) * (0.5 + 0.5 * rng.uniform())
        u, _ = np.linalg.qr(rng.standard_normal((m, k)))
        v, _ = np.linalg.qr(rng.standard_normal((n, k)))
        blocks.append(((i, i), (u * sv) @ v.T))
        ref.append(np.linalg.svd(blocks[-1][1]))
    legs = [[(m, Z(i)) for i, (m, _) in enumerate(shapes)], [(n, Z(-i)) for i, (_, n) in enumerate(shapes)]]
    t = q.btensor(legs, Z(0))
    t.set_blocks(blocks)
    keep = sum(min(sh) for sh in shapes) // 4
    pooled = np.sort(np.concatenate([r[1] for r in ref]))[::-1]
    smax = pooled[0]
    q.set_autotune(False)
    q.set_jacobi_kernel(kernel)
    try:
        plain = q.linalg.svd(t, 1, 1e-14, min_size=1, max_size=keep)
        q.set_gemm_mode("tf32x3")
        U, d, V = q.linalg.svd(t, 1, 1e-14, min_size=1, max_size=keep)
    finally:
        q.set_jacobi_kernel("block")
        q.set_gemm_mode("f64")
        q.set_autotune(True)
    assert sum(b.size for _, b in d.blocks()) == keep
    assert plain[1].block_indices() == d.block_indices()
    new_section = {k[0]: k[1] for k, _ in U.blocks()}
    dv = dict(d.blocks())
    Ub = dict(U.blocks())
    for i, (uref, sref, _) in enumerate(ref):
        if i not in new_section:
            assert sref[0] <= pooled[keep - 1]
            continue
        got = dv[(new_section[i],)]
        kk = len(got)
        assert kk == int(np.sum(sref >= pooled[keep - 1]))
        np.testing.assert_allclose(got, sref[:kk], atol=1e-12 * smax, rtol=0)
        ug = Ub[(i, new_section[i])]
        overlap = np.abs(np.sum(ug * uref[:, :kk], axis=0))
        np.testing.assert_allclose(overlap, np.ones(kk), atol=1e-10, rtol=0)
    for (k1, x), (k2, y) in zip(plain[1].blocks(), d.blocks()):
        np.testing.assert_allclose(x, y, atol=1e-12 * smax, rtol=0)
    assert _isometry_error(U) < 1e-11
    assert _isometry_error(V) < 1e-11


def test_truncated_svd_drops_exact_zero_values_like_the_oracle():
    """A truncation keeps only values strictly above its threshold less 2 eps, so an
    exact zero singular value is never kept, whatever min_size asks (the oracle's
    truncate, btensor_linalg.cpp:658-755); null columns are not completed then."""
    rng = np.random.default_rng(83)
    a = np.zeros((30, 24))
    a[:, :10] = rng.standard_normal((30, 10))
    legs = [[(30, Z(0))], [(24, Z(0))]]
    t = q.btensor(legs, Z(0))
    t.set_blocks([((0, 0), a)])
    ot = o.btensor([[(30, 0)], [(24, 0)]], [0], (0,))
    ot.blocks = [((0, 0), a.copy())]
    Uo, do, Vo = o.svd_truncated(ot, 1, 1e-10, 20, 10 ** 6)
    for mode, defl in (("f64", False), ("tf32x3", False), ("tf32x3", True)):
        q.set_gemm_mode(mode)
        q.set_svd_deflation(defl)
        try:
            U, d, V = q.linalg.svd(t, 1, 1e-10, min_size=20, max_size=10 ** 6)
        finally:
            q.set_gemm_mode("f64")
            q.set_svd_deflation(True)   # the default
        assert sum(d.section_sizes) == sum(len(v) for _, v in do.blocks) == 10, mode
        assert _isometry_error(U) < 1e-11
