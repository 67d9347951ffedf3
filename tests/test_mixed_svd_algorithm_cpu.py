"""The mixed path's truncating sector SVD (linalg.cpp, svd_refine.cu, jacobi.cu),
restated step by step in numpy on small sectors: FP32 one-sided Jacobi sweeps with
deflation at FP32 resolution; two Newton-Schulz steps making the FP32 rotation
orthogonal in FP64; W1 = W V; the discard level tau = t/2 from the FP32 column norms
with truncate's rule; one FP64 decoupling sweep that leaves pairs of two columns below
tau alone; then FP64 sweeps on the kept columns only, gathered with a fresh rotation R
(V's kept columns become V_k R); every sweep stops on quadratic convergence.  The kept
values and vectors must match LAPACK to FP64 accuracy.  This checks the algorithm on
the CPU; the GPU tests check the kernels (test_gpu_jacobi.py)."""
import numpy as np

EPS32, EPS64 = 1.1920929e-07, 2.220446049250313e-16


def _rounds(n):
    m = n + (n & 1)
    out = []
    for k in range(m - 1):
        a, b = [], []
        for slot in range(m // 2):
            x, y = (0, 1 + k) if slot == 0 else (1 + (k + slot) % (m - 1), 1 + (k - slot) % (m - 1))
            if x < n and y < n:
                a.append(x)
                b.append(y)
        out.append((np.array(a, int), np.array(b, int)))
    return out


def _jacobi(W, V, dtype, tol, defl=0.0, skip=None, max_sweeps=80, settle=1e-3):
    """One-sided Jacobi (round-robin), the kernels' acceptance test, deflation of columns
    at or below defl (squared norm) and the quadratic-convergence stop; returns W, V and
    the deflated columns' squared norms."""
    W, V = W.astype(dtype).copy(), V.astype(dtype).copy()
    q = W.shape[1]
    dead = np.zeros(q, bool)
    dn = np.zeros(q)
    for _ in range(max_sweeps):
        nrot, rmax = 0, 0.0
        for a, b in _rounds(q):
            live = ~dead[a] & ~dead[b]
            a, b = a[live], b[live]
            if a.size == 0:
                continue
            x, y = W[:, a], W[:, b]
            al, be, ga = (x * x).sum(0), (y * y).sum(0), (x * y).sum(0)
            do = (ga != 0) & (np.abs(ga) > tol * np.sqrt(al * be))
            if skip is not None:
                do &= ~((al < skip) & (be < skip))
            if do.any():
                nrot += int(do.sum())
                rmax = max(rmax, float(np.max(np.abs(ga[do]) / np.sqrt(al[do] * be[do]))))
                zeta = (be[do] - al[do]) / (2 * ga[do])
                t = np.sign(zeta) / (np.abs(zeta) + np.sqrt(1 + zeta * zeta))
                t = np.where(zeta == 0, 1.0, t).astype(dtype)
                c = (1 / np.sqrt(1 + t * t)).astype(dtype)
                s = (c * t).astype(dtype)
                for M in (W, V):
                    xx, yy = M[:, a[do]].copy(), M[:, b[do]].copy()
                    M[:, a[do]], M[:, b[do]] = c * xx - s * yy, s * xx + c * yy
            if defl > 0:
                for cols in (a, b):
                    nn = (W[:, cols].astype(np.float64) ** 2).sum(0)
                    kill = (nn <= defl) & (nn > 0)
                    dn[cols[kill]], dead[cols[kill]] = nn[kill], True
                    W[:, cols[kill]] = 0
        if nrot == 0 or rmax * rmax <= settle * tol:
            break
    return W, V, dn


def _kept_threshold(vals, keep):
    return np.sort(vals)[::-1][keep - 1]


def mixed_truncated_svd(W, keep):
    """Values and left vectors of the kept columns, the mixed path's way."""
    p, q = W.shape
    F = np.linalg.norm(W)
    W32, V32, _ = _jacobi(W, np.eye(q), np.float32, np.sqrt(p) * EPS32, defl=(EPS32 * F) ** 2)
    t = _kept_threshold(np.linalg.norm(W32.astype(np.float64), axis=0), keep)
    tau = 0.5 * t
    assert tau > 4 * EPS32 * F  # the discard path applies
    V = V32.astype(np.float64)
    I = np.eye(q)
    for _ in range(2):
        V = V @ (1.5 * I - 0.5 * (V.T @ V))
    W1 = W @ V
    null2 = (8 * EPS64 * F) ** 2
    W1, V, dn = _jacobi(W1, V, np.float64, p * EPS64, defl=null2, skip=tau * tau, max_sweeps=1)
    n2 = (W1 ** 2).sum(0)
    kept = np.nonzero(n2 > max(null2, tau * tau))[0]
    Wk, R, _ = _jacobi(W1[:, kept], np.eye(kept.size), np.float64, p * EPS64, defl=null2)
    W1[:, kept] = Wk
    V[:, kept] = V[:, kept] @ R
    s = np.linalg.norm(W1, axis=0)
    order = np.argsort(-s)[:keep]
    return s[order], W1[:, order] / s[order], V[:, order]


def test_mixed_truncated_svd_matches_lapack():
    rng = np.random.default_rng(5)
    for p, q, decades in ((70, 60, 13), (50, 50, 9), (40, 24, 12)):
        sv = np.logspace(0, -decades, q) * (0.5 + rng.uniform())
        u, _ = np.linalg.qr(rng.standard_normal((p, q)))
        v, _ = np.linalg.qr(rng.standard_normal((q, q)))
        W = (u * sv) @ v.T
        keep = q // 3
        s, U, Vk = mixed_truncated_svd(W, keep)
        ur, sr, vrt = np.linalg.svd(W)
        np.testing.assert_allclose(s, sr[:keep], rtol=0, atol=1e-13 * sr[0])
        np.testing.assert_allclose(np.abs(np.sum(U * ur[:, :keep], axis=0)), 1.0, atol=1e-10)
        np.testing.assert_allclose(np.abs(np.sum(Vk * vrt[:keep].T, axis=0)), 1.0, atol=1e-10)
        np.testing.assert_allclose(U.T @ U, np.eye(keep), atol=1e-12)
        np.testing.assert_allclose(Vk.T @ Vk, np.eye(keep), atol=1e-12)
