"""The synthetic contraction + truncation microbench on small sizes (pytest -m gpu):
the theta pair's contraction and the truncated sector SVD of the result match the
oracle (block lists exactly, values to 1e-12 / 1e-10), and the mixed path stays
within its FP32-level tolerance."""
import numpy as np
import pytest

import quantit_gb300 as q
from oracle import qtt_oracle as o
from tests._convert import same_structure, to_oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("D", [40, 96])
def test_theta_pair_contraction_and_truncation_match_oracle(D):
    A, B = q.networks.theta_pair(D, seed=0)
    Ao, Bo = to_oracle(A), to_oracle(B)
    C = A.tensordot(B, ([2, 3], [1, 0]))
    Co = o.tensordot(Ao, Bo, [2, 3], [1, 0])
    assert same_structure(C, Co)
    got = C.blocks()
    assert [k for k, _ in got] == [k for k, _ in Co.blocks]
    scale = max(float(np.max(np.abs(v))) for _, v in Co.blocks)
    for (k, a), (_, b) in zip(got, Co.blocks):
        np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-13 * scale)
    kmax = D // 2
    U, d, V = q.linalg.svd(C, 2, 1e-10, min_size=1, max_size=kmax)
    Uo, do, Vo = o.svd_truncated(Co, 2, 1e-10, 1, kmax)
    for t, w in ((U, Uo), (d, do), (V, Vo)):
        assert same_structure(t, w)
        assert t.block_indices() == [k for k, _ in w.blocks]
    for (k, a), (_, b) in zip(d.blocks(), do.blocks):
        np.testing.assert_allclose(a, b, rtol=1e-10, atol=1e-12 * float(np.max(b)))


@pytest.mark.parametrize("mode", ["tf32x3", "bf16x3"])
def test_theta_pair_mixed_precision(mode):
    D = 96
    A, B = q.networks.theta_pair(D, seed=1)
    ref = dict(A.tensordot(B, ([2, 3], [1, 0])).blocks())
    q.set_gemm_mode(mode)
    try:
        C = A.tensordot(B, ([2, 3], [1, 0]))
        U, d, V = q.linalg.svd(C, 2, 1e-10, min_size=1, max_size=D)
    finally:
        q.set_gemm_mode("f64")
    num = sum(float(np.sum((v - ref[k]) ** 2)) for k, v in C.blocks())
    den = sum(float(np.sum(v ** 2)) for v in ref.values())
    assert (num / den) ** 0.5 < 2e-6
    Uf, df, Vf = q.linalg.svd(q.tensordot(A, B, [2, 3], [1, 0]), 2, 1e-10, min_size=1, max_size=D)
    a = np.sort(np.concatenate([v for _, v in d.blocks()]))[::-1]
    b = np.sort(np.concatenate([v for _, v in df.blocks()]))[::-1]
    n = min(len(a), len(b))
    assert np.max(np.abs(a[:n] - b[:n])) < 2e-5 * b[0]
