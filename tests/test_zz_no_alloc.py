"""The allocation-free dense SVD entry point (pytest -m gpu; collected last).

qtt_svd_dense_noalloc serves callers that cannot allocate device memory (a
captured graph region, a fixed memory budget, pre-registered buffers only): it
works in a static device array instead.  Here it is called through the C-ABI
with device buffers owned by the test, twice in a row, and compared with the
library's regular SVD entry point (qtt_svd on a one-block btensor holding the
same matrix) within the FP64 tolerances of the other SVD tests."""
import ctypes as C

import numpy as np
import pytest

import quantit_gb300 as q
from quantit_gb300 import _lib

pytestmark = pytest.mark.gpu


def _regular_svd(a):
    m, n = a.shape
    t = q.btensor([[(m, q.conserved.Z(0))], [(n, q.conserved.Z(0))]], q.conserved.Z(0))
    t.set_blocks([((0, 0), a)])
    U, d, V = q.linalg.svd(t)
    return U.block_at((0, 0)), d.block_at((0,)), V.block_at((0, 0))


def _noalloc_svd(torch, a):
    m, n = a.shape
    k = min(m, n)
    dev = torch.device("cuda", 0)
    da = torch.as_tensor(a, dtype=torch.float64, device=dev).contiguous()
    du = torch.full((m, k), np.nan, dtype=torch.float64, device=dev)
    ds = torch.full((k,), np.nan, dtype=torch.float64, device=dev)
    dv = torch.full((n, k), np.nan, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    _lib.call("qtt_svd_dense_noalloc", C.c_void_p(da.data_ptr()), m, n, C.c_void_p(du.data_ptr()),
              C.c_void_p(ds.data_ptr()), C.c_void_p(dv.data_ptr()), C.c_void_p(stream.cuda_stream))
    torch.cuda.synchronize(dev)
    return du.cpu().numpy(), ds.cpu().numpy(), dv.cpu().numpy()


def _check_same(a, got, want):
    u, s, v = got
    U, S, V = want
    np.testing.assert_allclose(s, S, rtol=1e-12, atol=1e-13 * S[0])
    scale = float(np.max(np.abs(a)))
    np.testing.assert_allclose((u * s) @ v.T, a, atol=1e-11 * scale)
    np.testing.assert_allclose((U * S) @ V.T, (u * s) @ v.T, atol=1e-11 * scale)
    # singular vectors agree up to the sign of each pair of columns
    sign = np.sign(np.sum(u * U, axis=0))
    np.testing.assert_allclose(u * sign, U, atol=1e-9)
    np.testing.assert_allclose(v * sign, V, atol=1e-9)


def test_noalloc_svd_matches_regular_entry_point_twice():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(2024)
    shapes = [(120, 77), (64, 200)]
    for m, n in shapes:   # two calls in a row, the second reusing the scratch of the first
        a = rng.standard_normal((m, n)) * np.exp(-np.arange(n) / 20.0)
        _check_same(a, _noalloc_svd(torch, a), _regular_svd(a))


def test_noalloc_svd_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    big = np.zeros((257, 4))
    with pytest.raises(ValueError, match="exceeds the maximum"):
        _noalloc_svd(torch, big)
