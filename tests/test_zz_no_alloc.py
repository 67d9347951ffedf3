"""The allocation-free dense SVD entry point (pytest -m gpu; collected last).

qtt_svd_dense_noalloc serves callers that cannot allocate device memory: a plug-in
inside a host application that owns all device memory, a solver under a budget fixed
at start-up, or a real-time loop that cannot afford cudaMalloc / cudaFree (they can
synchronise the whole device).  It works in a static device array instead.  Here it
is called through the C-ABI with device buffers owned by the test, twice in a row,
and compared with the library's regular SVD entry point (qtt_svd on a one-block
btensor holding the same matrix) and with LAPACK (numpy) within the FP64
tolerances of the other SVD tests."""
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


def _noalloc_svd(torch, a, stream=None):
    """One call on `stream` (a torch stream; default: the current one), read back
    after that stream alone has been synchronised."""
    m, n = a.shape
    k = min(m, n)
    dev = torch.device("cuda", 0)
    st = stream if stream is not None else torch.cuda.current_stream(dev)
    with torch.cuda.stream(st):
        da = torch.as_tensor(a, dtype=torch.float64, device=dev).contiguous()
        du = torch.full((m, k), np.nan, dtype=torch.float64, device=dev)
        ds = torch.full((k,), np.nan, dtype=torch.float64, device=dev)
        dv = torch.full((n, k), np.nan, dtype=torch.float64, device=dev)
    _lib.call("qtt_svd_dense_noalloc", C.c_void_p(da.data_ptr()), m, n, C.c_void_p(du.data_ptr()),
              C.c_void_p(ds.data_ptr()), C.c_void_p(dv.data_ptr()), C.c_void_p(st.cuda_stream))
    st.synchronize()
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


def _check_lapack(a, got):
    """Independent reference: numpy's LAPACK SVD (values to 1e-12 of the largest;
    factors orthonormal)."""
    u, s, v = got
    ref = np.linalg.svd(a, compute_uv=False)
    np.testing.assert_allclose(s, ref, rtol=0, atol=1e-12 * ref[0])
    k = s.size
    np.testing.assert_allclose(u.T @ u, np.eye(k), atol=1e-12)
    np.testing.assert_allclose(v.T @ v, np.eye(k), atol=1e-12)


def test_noalloc_svd_matches_regular_entry_point_twice():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(2024)
    shapes = [(120, 77), (64, 200)]
    for m, n in shapes:   # two calls in a row, the second reusing the scratch of the first
        a = rng.standard_normal((m, n)) * np.exp(-np.arange(n) / 20.0)
        got = _noalloc_svd(torch, a)
        _check_same(a, got, _regular_svd(a))
        _check_lapack(a, got)


def test_noalloc_svd_on_a_non_default_stream():
    """Two calls on a caller-created stream, each read after that stream's own
    synchronisation."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(77)
    st = torch.cuda.Stream(device=torch.device("cuda", 0))
    for m, n in [(256, 256), (31, 9)]:
        a = rng.standard_normal((m, n))
        got = _noalloc_svd(torch, a, stream=st)
        _check_same(a, got, _regular_svd(a))
        _check_lapack(a, got)


def test_noalloc_svd_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    big = np.zeros((257, 4))
    with pytest.raises(ValueError, match="exceeds the maximum"):
        _noalloc_svd(torch, big)
