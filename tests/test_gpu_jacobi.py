"""Both sector-SVD Jacobi kernels against LAPACK's SVD (pytest -m gpu).

The block-cyclic kernel (column blocks of 16 (FP32) or 8 (FP64) in shared
memory, one CTA per block pair and grid step) is the default; the scalar kernel
(one column pair per warp and grid step) serves sectors with columns too long
for shared memory.  Both must give the same decomposition as numpy's SVD for
sector shapes that exercise ragged last blocks, odd block counts (a phantom
block in the round-robin), sectors narrower than one block, wide sectors
(decomposed as A^T), graded and rank-deficient spectra."""
import numpy as np
import pytest

import quantit_gb300 as q
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
    # FP64 work: LAPACK agreement to 1e-12 of the sector's largest singular value;
    # FP32 work (the mixed path): to a few FP32 ulps of it
    rtol = 1e-12 if mode == "f64" else 3e-6
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
    iso = 1e-11 if mode == "f64" else 1e-4
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
