// Batched per-sector SVD / symmetric eigendecomposition by one-sided (Hestenes)
// Jacobi.  All sectors of a decomposition run in ONE cooperative launch: at
// every step each sector contributes its round-robin set of disjoint column
// pairs, every warp in the grid takes pairs from the combined list, and a grid
// barrier closes the step.  This replaces the per-sector LAPACK calls of
// btensor_linalg.cpp:483 (torch::svd) and :354 (linalg eigh).
//
// The work type T is double for the plain FP64 path and float for the mixed
// path (FP32 runs on GB300's CUDA cores at 64x the FP64 rate; the mixed DMRG
// reports its energy from an FP64 contraction of the final state, which is
// second order in the SVD's orthogonality error).  Outputs are always FP64.
//
// Every loop is bounded: at most max_sweeps sweeps per sector.
#include <cooperative_groups.h>

#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "kernels.h"
#include "qtt_core.h"

namespace cg = cooperative_groups;

namespace qtt {
namespace {
constexpr int JT = 256;   // threads per CTA of the packing kernels
constexpr int JJ = 256;   // threads per CTA of the Jacobi kernel

template <class T>
__device__ __forceinline__ T wsum(T v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <class T>
struct Eps;
template <>
struct Eps<double> {
    // off-orthogonality accepted per column pair: p * eps64
    __device__ static double tol(int p) { return 2.220446049250313e-16 * double(p); }
};
template <>
struct Eps<float> {
    // sqrt(p) * eps32: columns orthogonal to a few 1e-6 relative
    __device__ static float tol(int p) { return 1.1920929e-07f * sqrtf(float(p)); }
};

__device__ __forceinline__ double ldcg(const double *p) { return __ldcg(p); }
__device__ __forceinline__ float ldcg(const float *p) { return __ldcg(p); }

// Plane rotation (c, s) applied in half-angle form with tau = s / (1 + c) = tan(theta/2):
//     x' = x - s (y + tau x) = c x - s y,   y' = y + s (x - tau y) = s x + c y.
// For small angles c rounds to 1 while 1 - c = s tau does not, so the plain form
// c x - s y would scale both columns by sqrt(1 + t^2) at every such rotation; in
// FP32 that bias accumulates to ~1e-5 in the singular values over a few sweeps.
template <class T>
__device__ __forceinline__ void rot_apply(T &x, T &y, T s, T tau) {
    const T u = fma(tau, x, y);
    const T v = fma(-tau, y, x);
    x = fma(-s, u, x);
    y = fma(s, v, y);
}

// Hestenes rotation for column norms al, be and inner product ga: s and tau.
template <class T>
__device__ __forceinline__ void rot_params(T al, T be, T ga, T &s, T &tau, T &t) {
    const T zeta = (be - al) / (T(2) * ga);
    if (fabs(zeta) > T(1e18))
        t = T(0.5) / zeta;
    else
        t = copysign(T(1), zeta) / (fabs(zeta) + sqrt(T(1) + zeta * zeta));
    const T c = T(1) / sqrt(T(1) + t * t);
    s = c * t;
    tau = s / (T(1) + c);
}
template <class T>
__device__ __forceinline__ void rot_params(T al, T be, T ga, T &s, T &tau) {
    T t;
    rot_params(al, be, ga, s, tau, t);
}

// Round-robin (circle method) pairing of qp (even) players at round k in [0, qp-1):
// slot 0 pairs player 0 with 1 + k; slot i > 0 pairs 1 + (k+i) mod (qp-1) with 1 + (k-i) mod (qp-1).
__device__ __forceinline__ void rr_pair(int qp, int k, int slot, int &a, int &b) {
    int r = qp - 1;
    if (slot == 0) {
        a = 0;
        b = 1 + k;
    } else {
        a = 1 + (k + slot) % r;
        b = 1 + ((k - slot) % r + r) % r;
    }
}

template <class T>
__global__ void k_pack(const double *__restrict__ src, T *__restrict__ work, const PackEntry *__restrict__ ents,
                       const Chunk *__restrict__ chunks, const SectorDesc *__restrict__ secs) {
    const Chunk ch = chunks[blockIdx.x];
    const PackEntry e = ents[ch.seg];
    const SectorDesc sd = secs[e.sector];
    for (int i = threadIdx.x; i < ch.len; i += blockDim.x) {
        int64_t k = ch.start + i;
        int r = int(k / e.cols), c = int(k - int64_t(r) * e.cols);
        int ar = e.r0 + r, ac = e.c0 + c;  // position in A (m x n)
        int64_t w = sd.trans ? (int64_t(ac) + int64_t(ar) * sd.p) : (int64_t(ar) + int64_t(ac) * sd.p);
        work[sd.w_off + w] = T(src[e.src_off + k]);
    }
}

__device__ double block_sum_d(double v) {
    __shared__ double red[32];
    v = wsum(v);
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[w] = v;
    __syncthreads();
    int nw = (blockDim.x + 31) >> 5;
    v = (threadIdx.x < nw) ? red[threadIdx.x] : 0.0;
    if (w == 0) v = wsum(v);
    return v;  // valid in thread 0
}

// eigh: symmetrise from one triangle, shift by the Frobenius norm (stored in the descriptor)
template <class T>
__global__ void k_eigh_prepare(T *work, SectorDesc *secs, int upper) {
    SectorDesc &sd = secs[blockIdx.x];
    const int n = sd.p;
    T *W = work + sd.w_off;
    for (int64_t t = threadIdx.x; t < int64_t(n) * n; t += blockDim.x) {
        int i = int(t % n), j = int(t / n);
        if (i == j) continue;
        bool keep = upper ? (i < j) : (i > j);
        if (!keep) continue;
        W[j + int64_t(i) * n] = W[i + int64_t(j) * n];
    }
    __syncthreads();
    double acc = 0.0;
    for (int64_t t = threadIdx.x; t < int64_t(n) * n; t += blockDim.x) acc += double(W[t]) * double(W[t]);
    acc = block_sum_d(acc);
    __shared__ double shift;
    if (threadIdx.x == 0) {
        shift = sqrt(acc);
        if (shift < 1.0e-200) shift = 1.0;
        sd.shift = shift;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) W[i + int64_t(i) * n] += T(shift);
}

template <class T>
struct JacobiParams {
    T *work;
    T *rot;
    const SectorDesc *secs;
    const int *slot_start;  // nsec + 1 prefix sums of pairs per step
    int nsec;
    int max_sweeps;
    int64_t max_steps;
    int *sweeps;   // per sector (written at the end)
    int *rotated;  // nsec * max_sweeps flags, zero on entry: a rotation happened in (sector, sweep)
    const T *defl; // per sector: squared-norm deflation threshold (null: no deflation)
    T *dnorm;      // per column (s_off + column): squared norm when deflated, 0 otherwise
    const T *skip; // per sector (null: none): squared discard level of pair_skipped
};

// Pairs the decoupling FP64 sweep of a truncating mixed-precision SVD leaves alone
// (skip = the squared discard level of the sector, 0: none): both columns below it.
// A pair of one kept and one discarded column is always rotated: the columns the FP32
// sweeps deflated (norm below FP32 resolution) were never decoupled from the kept ones,
// their couplings can be of the order of the product of the norms, and left in place
// they would shift the kept values by ~1e-12 of the largest.  Rotations among the
// discarded columns are the ones skipped: they would shuffle those couplings around
// within the discarded set instead of removing them.
template <class T>
__device__ __forceinline__ bool pair_skipped(T al, T be, T skip) {
    return al < skip && be < skip;
}

// End of a sweep.  The sweep's largest relative coupling |<w_a, w_b>| / (|w_a| |w_b|)
// among the pairs it rotated is kept as the bits of a non-negative float (0: nothing
// rotated; a deflation alone counts as the smallest normal float: zeroing a null
// column removes its couplings and changes no other column).  The sector is done when nothing rotated, or when
// every rotation was so small that the next sweep has nothing left to do: one-sided
// Jacobi converges quadratically near the end, so couplings of at most delta before a
// sweep are of order delta^2 after it, and delta^2 <= 1e-3 tol leaves a margin of 1e3
// for the constant (small relative gaps between the values).  That saves the sweep
// which would only have confirmed convergence, and the sweeps that chase rounding noise
// just above the tolerance.
constexpr double kSettle = 1e-3;
template <class T>
__device__ __forceinline__ bool sweep_converged(int bits, int p) {
    if (bits == 0) return true;
    const double d = double(__int_as_float(bits));
    return d * d <= kSettle * double(Eps<T>::tol(p));
}

// Rotation of one column pair by one warp.  With R > 0 (p <= 32 R) every lane
// first loads its R elements of both columns into registers -- one round trip to
// L2 instead of one per element -- then forms the three inner products, the
// rotation, and writes back from registers; the rotation-matrix columns follow
// the same pattern.  R == 0 streams columns of any length.  A nonzero column whose
// squared norm is at most thr (> 0) is deflated: set to zero, never rotated again.
// Returns whether a column was rotated or deflated.
template <class T, int R>
__device__ __forceinline__ bool rotate_pair(T *__restrict__ wa, T *__restrict__ wb, T *__restrict__ va,
                                            T *__restrict__ vb, int p, int q, int lane, T thr, T *da, T *db,
                                            T skip, float &rel) {
    T al = 0, be = 0, ga = 0;
    T x[R > 0 ? R : 1], y[R > 0 ? R : 1];
    if (R > 0) {
#pragma unroll
        for (int i = 0; i < R; ++i) {
            const int r = lane + 32 * i;
            x[i] = r < p ? ldcg(wa + r) : T(0);
            y[i] = r < p ? ldcg(wb + r) : T(0);
        }
#pragma unroll
        for (int i = 0; i < R; ++i) {
            al = fma(x[i], x[i], al);
            be = fma(y[i], y[i], be);
            ga = fma(x[i], y[i], ga);
        }
    } else {
        for (int r = lane; r < p; r += 32) {
            T xx = ldcg(wa + r), yy = ldcg(wb + r);
            al = fma(xx, xx, al);
            be = fma(yy, yy, be);
            ga = fma(xx, yy, ga);
        }
    }
    al = wsum(al);
    be = wsum(be);
    ga = wsum(ga);
    const bool za = thr > T(0) && al > T(0) && al <= thr, zb = thr > T(0) && be > T(0) && be <= thr;
    if (za || zb) {
        for (int r = lane; r < p; r += 32) {
            if (za) wa[r] = T(0);
            if (zb) wb[r] = T(0);
        }
        if (lane == 0) {
            if (za) *da = al;
            if (zb) *db = be;
        }
        rel = 1.17549435e-38f;  // a deflation removes couplings and adds none: it alone settles
        return true;
    }
    if (pair_skipped(al, be, skip)) return false;
    if (ga == T(0) || fabs(ga) <= Eps<T>::tol(p) * sqrt(al) * sqrt(be)) return false;
    rel = float(fabs(ga) / (sqrt(al) * sqrt(be)));
    T sn, tau;
    rot_params(al, be, ga, sn, tau);
    if (R > 0) {
#pragma unroll
        for (int i = 0; i < R; ++i) {
            const int r = lane + 32 * i;
            if (r < p) {
                T xx = x[i], yy = y[i];
                rot_apply(xx, yy, sn, tau);
                wa[r] = xx;
                wb[r] = yy;
            }
        }
#pragma unroll
        for (int i = 0; i < R; ++i) {
            const int r = lane + 32 * i;
            x[i] = r < q ? ldcg(va + r) : T(0);
            y[i] = r < q ? ldcg(vb + r) : T(0);
        }
#pragma unroll
        for (int i = 0; i < R; ++i) {
            const int r = lane + 32 * i;
            if (r < q) {
                T xx = x[i], yy = y[i];
                rot_apply(xx, yy, sn, tau);
                va[r] = xx;
                vb[r] = yy;
            }
        }
    } else {
        for (int r = lane; r < p; r += 32) {
            T xx = ldcg(wa + r), yy = ldcg(wb + r);
            rot_apply(xx, yy, sn, tau);
            wa[r] = xx;
            wb[r] = yy;
        }
        for (int r = lane; r < q; r += 32) {
            T xx = ldcg(va + r), yy = ldcg(vb + r);
            rot_apply(xx, yy, sn, tau);
            va[r] = xx;
            vb[r] = yy;
        }
    }
    return true;
}

// One grid barrier per step.  Every CTA keeps its own copy of the per-sector
// sweep / done state in shared memory and updates it identically after each
// barrier from the rotation flags, so no second barrier is needed to publish it.
template <class T, int R>
__global__ void __launch_bounds__(JJ) k_jacobi(JacobiParams<T> P) {
    cg::grid_group grid = cg::this_grid();
    extern __shared__ int jsh[];
    const int nsec = P.nsec;
    int *done = jsh;          // nsec
    int *sweep = jsh + nsec;  // nsec
    __shared__ int ndone;
    const int lane = threadIdx.x & 31;
    const int64_t gw = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = (int64_t(gridDim.x) * blockDim.x) >> 5;
    const int64_t gt = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t nt = int64_t(gridDim.x) * blockDim.x;
    const int total_slots = P.slot_start[nsec];

    for (int s = 0; s < nsec; ++s) {
        const SectorDesc sd = P.secs[s];
        const int64_t qq = int64_t(sd.q) * sd.q;
        if (sd.warm) continue;  // rot already holds the warm start V0
        for (int64_t e = gt; e < qq; e += nt) P.rot[sd.rot_off + e] = (e % (sd.q + 1) == 0) ? T(1) : T(0);
    }
    if (threadIdx.x == 0) ndone = 0;
    __syncthreads();
    for (int s = threadIdx.x; s < nsec; s += blockDim.x) {
        done[s] = (P.secs[s].q < 2) ? 1 : 0;
        sweep[s] = 0;
        if (done[s]) atomicAdd(&ndone, 1);
    }
    grid.sync();

    for (int64_t step = 0; step < P.max_steps; ++step) {
        if (ndone >= nsec) break;
        for (int64_t slot = gw; slot < total_slots; slot += nw) {
            int lo = 0, hi = nsec - 1;
            while (lo < hi) {
                int mid = (lo + hi + 1) >> 1;
                if (P.slot_start[mid] <= slot)
                    lo = mid;
                else
                    hi = mid - 1;
            }
            const int s = lo;
            if (done[s]) continue;
            const SectorDesc sd = P.secs[s];
            const int qp = sd.q + (sd.q & 1);
            const int k = int(step % (qp - 1));
            int a, b;
            rr_pair(qp, k, int(slot - P.slot_start[s]), a, b);
            if (a >= sd.q || b >= sd.q) continue;
            if (a > b) {
                int t = a;
                a = b;
                b = t;
            }
            T *wa = P.work + sd.w_off + int64_t(a) * sd.p;
            T *wb = P.work + sd.w_off + int64_t(b) * sd.p;
            T *va = P.rot + sd.rot_off + int64_t(a) * sd.q;
            T *vb = P.rot + sd.rot_off + int64_t(b) * sd.q;
            T *dn = P.dnorm ? P.dnorm + sd.s_off : nullptr;
            float rel = 0.0f;
            if (!rotate_pair<T, R>(wa, wb, va, vb, sd.p, sd.q, lane, P.defl ? P.defl[s] : T(0), dn ? dn + a : nullptr,
                                   dn ? dn + b : nullptr, P.skip ? P.skip[s] : T(0), rel))
                continue;
            if (lane == 0) atomicMax(P.rotated + int64_t(s) * P.max_sweeps + sweep[s], __float_as_int(rel));
        }
        grid.sync();
        for (int s = threadIdx.x; s < nsec; s += blockDim.x) {
            if (done[s]) continue;
            const int q = P.secs[s].q;
            const int qp = q + (q & 1);
            if ((step + 1) % (qp - 1) == 0) {
                const int sw = sweep[s];
                const int bits = ((volatile int *)P.rotated)[int64_t(s) * P.max_sweeps + sw];
                sweep[s] = sw + 1;
                if (sweep_converged<T>(bits, P.secs[s].p) || sw + 1 >= P.max_sweeps) {
                    done[s] = 1;
                    atomicAdd(&ndone, 1);
                }
            }
        }
        __syncthreads();
    }
    if (blockIdx.x == 0)
        for (int s = threadIdx.x; s < nsec; s += blockDim.x) P.sweeps[s] = sweep[s];
}

// ---------------------------------------------------------------------------
// Block-cyclic one-sided Jacobi.  The q columns of a sector are cut into blocks
// of B columns; a grid step pairs the blocks round-robin (nbp - 1 steps per
// sweep, nbp = blocks rounded up to even, a phantom block when odd) and one CTA
// takes one block pair.  The CTA copies the 2B columns into shared memory and
// runs, with CTA barriers only:
//   * on the first step of a sweep, the B - 1 round-robin rounds inside each of
//     the two blocks (every intra-block pair once per sweep);
//   * the B rounds of inter-block pairs (I_k, J_(k+r) mod B): warp k keeps I_k in
//     registers and the J columns move through shared memory.
// Every column pair of the sector is thus visited exactly once per sweep, as in
// the scalar ordering, but a sweep costs ~q/B grid barriers instead of ~q.  The
// rotations of a step are accumulated into a 2B x 2B orthogonal matrix Q (one
// element per lane and column) and applied to the rotation matrix V once at the
// end of the step (V[:, I u J] <- V[:, I u J] Q).
template <class T>
struct BJacobiParams {
    T *work;
    T *rot;
    const SectorDesc *secs;
    int nsec;
    int max_sweeps;
    int64_t max_steps;
    int *sweeps;   // per sector (written at the end)
    int *rotated;  // nsec * max_sweeps flags, zero on entry
    // deferred V updates (null qbuf: each CTA updates V at the end of its block pair)
    T *qbuf;       // 2 x max_jobs rotation matrices (NP x NP), by step parity
    int *jobs;     // 2 x max_jobs x {sector, block a, block b, valid columns a | b << 16}
    int *njobs;    // per step: jobs recorded (zero on entry)
    int *vnext;    // per step: V work units claimed (zero on entry)
    int max_jobs;  // >= block pairs per step
    int upj;       // V work units (row chunks of one CTA width) per job
    int max_q;     // widest sector (columns)
    const T *defl; // per sector: squared-norm deflation threshold (null: no deflation)
    T *dnorm;      // per column (s_off + column): squared norm when deflated, 0 otherwise
    const T *skip; // per sector (null: none): squared discard level of pair_skipped
};

__device__ __forceinline__ int bj_items(int q, int B) {
    if (q < 2) return 0;
    const int nb = (q + B - 1) / B;
    return (nb + (nb & 1)) / 2;
}

// 16-byte shared-memory chunks: lane l holds elements (32 i + l) * V + c of a
// column, V = 16 / sizeof(T); slots are zero-padded to PP, so no bounds checks.
template <class T, int R>
__device__ __forceinline__ void bj_load(T (&x)[R], const T *slot, int lane) {
    if constexpr (sizeof(T) == 4) {
#pragma unroll
        for (int i = 0; i < R / 4; ++i) {
            const float4 v = reinterpret_cast<const float4 *>(slot)[32 * i + lane];
            x[4 * i] = v.x;
            x[4 * i + 1] = v.y;
            x[4 * i + 2] = v.z;
            x[4 * i + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int i = 0; i < R / 2; ++i) {
            const double2 v = reinterpret_cast<const double2 *>(slot)[32 * i + lane];
            x[2 * i] = v.x;
            x[2 * i + 1] = v.y;
        }
    }
}

template <class T, int R>
__device__ __forceinline__ void bj_store(const T (&x)[R], T *slot, int lane) {
    if constexpr (sizeof(T) == 4) {
#pragma unroll
        for (int i = 0; i < R / 4; ++i)
            reinterpret_cast<float4 *>(slot)[32 * i + lane] = make_float4(x[4 * i], x[4 * i + 1], x[4 * i + 2], x[4 * i + 3]);
    } else {
#pragma unroll
        for (int i = 0; i < R / 2; ++i)
            reinterpret_cast<double2 *>(slot)[32 * i + lane] = make_double2(x[2 * i], x[2 * i + 1]);
    }
}

// Per-lane partial sums in NA independent chains (the dot product is on the
// critical path of every round: R dependent FMAs would cost R FMA latencies).
template <class T, int R>
__device__ __forceinline__ T bj_dot(const T (&x)[R], const T (&y)[R]) {
    constexpr int NA = R >= 16 ? 4 : (R >= 4 ? 2 : 1);
    T a[NA];
#pragma unroll
    for (int k = 0; k < NA; ++k) a[k] = T(0);
#pragma unroll
    for (int i = 0; i < R; ++i) a[i % NA] = fma(x[i], y[i], a[i % NA]);
#pragma unroll
    for (int w = NA / 2; w > 0; w >>= 1)
#pragma unroll
        for (int k = 0; k < w; ++k) a[k] += a[k + w];
    return wsum(a[0]);
}

// Rotation parameters from the multi-function unit (FP32 only).  t need not be
// the exact optimum (a near-optimal angle leaves |ga'| ~ 1e-7 |ga|, far under the
// acceptance threshold); s = t / h and tau = t / (1 + h) with h = sqrt(1 + t^2)
// define an orthogonal transformation up to O(s^2 * ulp), so approximate
// reciprocals and square roots cost no accuracy but ~4x less latency than the
// IEEE-rounded divisions and square roots on the critical path of every round.
__device__ __forceinline__ void bj_params_fast(float al, float be, float ga, float &sn, float &tau, float &t) {
    const float zeta = __fdividef(be - al, 2.0f * ga);
    const float az = fabsf(zeta);
    if (az > 1e18f) {
        t = 0.5f / zeta;
    } else {
        const float w = fmaf(zeta, zeta, 1.0f);
        t = copysignf(__fdividef(1.0f, az + w * rsqrtf(w)), zeta);
    }
    const float w2 = fmaf(t, t, 1.0f);
    const float rh = rsqrtf(w2);
    sn = t * rh;
    tau = __fdividef(t, 1.0f + w2 * rh);
}

// Hestenes rotation of two register-resident columns with tracked squared norms
// al, be: only the inner product is formed; after the rotation the norms follow
// from al' = al - t ga, be' = be + t ga (t = tan theta), and are recomputed from
// the columns when that update cancels (norm drops below 1/16).  Same acceptance
// test and rotation as rotate_pair (tol = Eps<T>::tol(p), hoisted by the caller).
// A zero column (norm 0) is skipped without forming the product; with thr > 0 a
// column whose squared norm falls to thr or below after the rotation is deflated
// (set to zero, norm 0; dx / dy receive its squared norm before, else stay 0).
template <class T, int R>
__device__ __forceinline__ bool bj_rotate(T (&x)[R], T (&y)[R], T &al, T &be, T tol, T thr, T &sn, T &tau, T &dx,
                                          T &dy, T skip, float &rmax) {
    if (al == T(0) || be == T(0)) return false;
    if (pair_skipped(al, be, skip)) return false;
    const T ga = bj_dot(x, y);
    if (ga == T(0)) return false;
    T t;
    if constexpr (sizeof(T) == 4) {
        const float rel = fabsf(ga) * rsqrtf(al) * rsqrtf(be);
        if (rel <= tol) return false;
        rmax = fmaxf(rmax, rel);
        bj_params_fast(al, be, ga, sn, tau, t);
    } else {
        const double rel = fabs(ga) / sqrt(al * be);
        if (rel <= tol) return false;
        rmax = fmaxf(rmax, float(rel));
        rot_params(al, be, ga, sn, tau, t);
    }
#pragma unroll
    for (int i = 0; i < R; ++i) rot_apply(x[i], y[i], sn, tau);
    const T a2 = al - t * ga, b2 = be + t * ga;
    al = (a2 > al * T(0.0625)) ? a2 : bj_dot(x, x);
    be = (b2 > be * T(0.0625)) ? b2 : bj_dot(y, y);
    if (thr > T(0)) {
        if (al <= thr) {
#pragma unroll
            for (int i = 0; i < R; ++i) x[i] = T(0);
            dx = al;
            al = T(0);
        }
        if (be <= thr) {
#pragma unroll
            for (int i = 0; i < R; ++i) y[i] = T(0);
            dy = be;
            be = T(0);
        }
    }
    return true;
}

template <class T, int NP>
__device__ __forceinline__ T bj_qdot(const T (&vr)[NP], const T *qcol) {
    T acc0 = 0, acc1 = 0;
    if constexpr (sizeof(T) == 4) {
#pragma unroll
        for (int j = 0; j < NP / 4; ++j) {
            const float4 qv = reinterpret_cast<const float4 *>(qcol)[j];
            acc0 = fma(vr[4 * j], qv.x, acc0);
            acc1 = fma(vr[4 * j + 1], qv.y, acc1);
            acc0 = fma(vr[4 * j + 2], qv.z, acc0);
            acc1 = fma(vr[4 * j + 3], qv.w, acc1);
        }
    } else {
#pragma unroll
        for (int j = 0; j < NP / 2; ++j) {
            const double2 qv = reinterpret_cast<const double2 *>(qcol)[j];
            acc0 = fma(vr[2 * j], qv.x, acc0);
            acc1 = fma(vr[2 * j + 1], qv.y, acc1);
        }
    }
    return acc0 + acc1;
}

// V[r, cols] <- V[r, cols] Q for rows [r0, r1) of the 2B columns of blocks a and b
// (na / nbc valid columns), Q = NP x NP column-major in shared memory.
template <class T, int B>
__device__ __forceinline__ void bj_apply_v(T *V, int q, int a, int b, int na, int nbc, const T *Qs, int r0, int r1,
                                           int tid) {
    constexpr int NP = 2 * B, NT = 32 * B;
    auto valid = [&](int j) { return j < B ? j < na : (j - B) < nbc; };
    auto column = [&](int j) { return j < B ? a * B + j : b * B + (j - B); };
    for (int r = r0 + tid; r < r1; r += NT) {
        T vr[NP];
#pragma unroll
        for (int j = 0; j < NP; ++j) vr[j] = valid(j) ? ldcg(V + int64_t(column(j)) * q + r) : T(0);
#pragma unroll 2
        for (int jp = 0; jp < NP; ++jp) {
            if (!valid(jp)) continue;
            V[int64_t(column(jp)) * q + r] = bj_qdot<T, NP>(vr, Qs + jp * NP);
        }
    }
}

// The deferred V updates of step `st`: CTAs claim (job, row chunk) units from a
// counter until none are left, so CTAs without a block pair take most of them.
template <class T, int B>
__device__ void bj_vwork(const BJacobiParams<T> &P, int64_t st, T *Qs, int *s_unit, int tid) {
    constexpr int NP = 2 * B, NT = 32 * B;
    const int nj = __ldcg(P.njobs + st);
    const int total = nj * P.upj;
    const int par = int(st & 1);
    for (;;) {
        if (tid == 0) *s_unit = atomicAdd(P.vnext + st, 1);
        __syncthreads();
        const int u = *s_unit;
        __syncthreads();
        if (u >= total) break;
        const int jb = u / P.upj, chunk = u - jb * P.upj;
        const int *jr = P.jobs + (int64_t(par) * P.max_jobs + jb) * 4;
        const int s = __ldcg(jr), a = __ldcg(jr + 1), b = __ldcg(jr + 2), nn = __ldcg(jr + 3);
        const SectorDesc sd = P.secs[s];
        const int r0 = chunk * NT;
        if (r0 >= sd.q) continue;
        const T *qsrc = P.qbuf + (int64_t(par) * P.max_jobs + jb) * NP * NP;
        for (int e = tid; e < NP * NP; e += NT) Qs[e] = ldcg(qsrc + e);
        __syncthreads();
        bj_apply_v<T, B>(P.rot + sd.rot_off, sd.q, a, b, nn & 0xFFFF, nn >> 16, Qs, r0, min(sd.q, r0 + NT), tid);
        __syncthreads();
    }
}

template <class T, int B, int R>
__global__ void __launch_bounds__(B * 32) k_bjacobi(BJacobiParams<T> P) {
    constexpr int NP = 2 * B;   // columns (players) of a block pair
    constexpr int PP = 32 * R;  // shared-memory slot per column (zero-padded)
    constexpr int NT = 32 * B;
    cg::grid_group grid = cg::this_grid();
    extern __shared__ __align__(16) unsigned char bsh[];
    T *cols = reinterpret_cast<T *>(bsh);  // NP slots of PP
    T *Qs = cols + NP * PP;                // NP x NP, column-major
    T *nrm = Qs + NP * NP;                 // NP squared column norms
    const int nsec = P.nsec;
    int *done = reinterpret_cast<int *>(nrm + NP);
    int *sweep = done + nsec;
    int *istart = sweep + nsec;  // nsec + 1 prefix sums of block pairs per step
    __shared__ int ndone, any_rot, s_unit, s_rmax;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const bool defer_v = P.qbuf != nullptr;
    const int64_t gt = int64_t(blockIdx.x) * NT + tid;
    const int64_t nt = int64_t(gridDim.x) * NT;

    for (int s = 0; s < nsec; ++s) {
        const SectorDesc sd = P.secs[s];
        const int64_t qq = int64_t(sd.q) * sd.q;
        if (sd.warm) continue;  // rot already holds the warm start V0
        for (int64_t e = gt; e < qq; e += nt) P.rot[sd.rot_off + e] = (e % (sd.q + 1) == 0) ? T(1) : T(0);
    }
    if (tid == 0) {
        ndone = 0;
        istart[0] = 0;
    }
    __syncthreads();
    for (int s = tid; s < nsec; s += NT) {
        const int q = P.secs[s].q;
        done[s] = (q < 2) ? 1 : 0;
        sweep[s] = 0;
        istart[s + 1] = bj_items(q, B);
        if (done[s]) atomicAdd(&ndone, 1);
    }
    __syncthreads();
    if (warp == 0) {
        int carry = 0;
        for (int base = 0; base < nsec; base += 32) {
            const int i = base + lane;
            int v = i < nsec ? istart[i + 1] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                const int u = __shfl_up_sync(0xffffffffu, v, o);
                if (lane >= o) v += u;
            }
            if (i < nsec) istart[i + 1] = v + carry;
            carry += __shfl_sync(0xffffffffu, v, 31);
        }
    }
    __syncthreads();
    const int total = istart[nsec];
    grid.sync();

    int64_t steps_run = 0;
    for (int64_t step = 0; step < P.max_steps; ++step) {
        if (ndone >= nsec) break;
        steps_run = step + 1;
        for (int item = blockIdx.x; item < total; item += gridDim.x) {
            int lo = 0, hi = nsec - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (istart[mid] <= item)
                    lo = mid;
                else
                    hi = mid - 1;
            }
            const int s = lo;
            if (done[s]) continue;
            const SectorDesc sd = P.secs[s];
            const int p = sd.p, q = sd.q;
            const int nb = (q + B - 1) / B, nbp = nb + (nb & 1);
            const int k = int(step % (nbp - 1));
            int a, b;
            rr_pair(nbp, k, item - istart[s], a, b);
            if (a > b) {
                const int t = a;
                a = b;
                b = t;
            }
            const bool has_b = b < nb;  // otherwise b is the phantom block
            if (!has_b && k != 0) continue;
            const int na = min(B, q - a * B), nbc = has_b ? min(B, q - b * B) : 0;
            auto valid = [&](int j) { return j < B ? j < na : (j - B) < nbc; };
            auto column = [&](int j) { return j < B ? a * B + j : b * B + (j - B); };
            T *W = P.work + sd.w_off;
            T *V = P.rot + sd.rot_off;
            const T tol = Eps<T>::tol(p);
            const T thr = P.defl ? P.defl[s] : T(0);
            const T skp = P.skip ? P.skip[s] : T(0);
            bool zeroed = false;

            for (int j = warp; j < NP; j += B) {
                if (!valid(j)) continue;
                const T *src = W + int64_t(column(j)) * p;
                // all R loads of a lane in flight at once (one L2 round trip per column)
                T v[R];
#pragma unroll
                for (int i = 0; i < R; ++i) {
                    const int r = lane + 32 * i;
                    v[i] = r < p ? ldcg(src + r) : T(0);
                }
                T acc = 0;
#pragma unroll
                for (int i = 0; i < R; ++i) {
                    acc = fma(v[i], v[i], acc);
                    cols[j * PP + lane + 32 * i] = v[i];
                }
                acc = wsum(acc);
                if (thr > T(0) && acc > T(0) && acc <= thr) {
                    // a numerically zero column: deflated (zero from here on)
#pragma unroll
                    for (int i = 0; i < R; ++i) cols[j * PP + lane + 32 * i] = T(0);
                    if (lane == 0) P.dnorm[sd.s_off + column(j)] = acc;
                    acc = T(0);
                    zeroed = true;
                }
                if (lane == 0) nrm[j] = acc;
            }
            for (int e = tid; e < NP * NP; e += NT) Qs[e] = (e % (NP + 1) == 0) ? T(1) : T(0);
            if (tid == 0) {
                any_rot = 0;
                s_rmax = 0;
            }
            __syncthreads();
            bool rotated_any = zeroed;
            float rmax = zeroed ? 1.17549435e-38f : 0.0f;  // a deflation removes couplings and adds none
            T x[R], y[R], sn, tau;
            if (k == 0) {
                // intra-block pairs: round-robin over the B columns of each block
                const int half = warp / (B / 2), slot = warp % (B / 2);
                for (int round = 0; round < B - 1; ++round) {
                    int u, v;
                    rr_pair(B, round, slot, u, v);
                    u += half * B;
                    v += half * B;
                    if (valid(u) && valid(v)) {
                        bj_load(x, cols + u * PP, lane);
                        bj_load(y, cols + v * PP, lane);
                        T al = nrm[u], be = nrm[v], dx = T(0), dy = T(0);
                        if (bj_rotate(x, y, al, be, tol, thr, sn, tau, dx, dy, skp, rmax)) {
                            if (lane == 0 && dx > T(0)) P.dnorm[sd.s_off + column(u)] = dx;
                            if (lane == 0 && dy > T(0)) P.dnorm[sd.s_off + column(v)] = dy;
                            bj_store(x, cols + u * PP, lane);
                            bj_store(y, cols + v * PP, lane);
                            if (lane < NP) {
                                T qu = Qs[u * NP + lane], qv = Qs[v * NP + lane];
                                rot_apply(qu, qv, sn, tau);
                                Qs[u * NP + lane] = qu;
                                Qs[v * NP + lane] = qv;
                            }
                            if (lane == 0) {
                                nrm[u] = al;
                                nrm[v] = be;
                            }
                            rotated_any = true;
                        }
                    }
                    __syncthreads();
                }
            }
            if (has_b) {
                // inter-block pairs: warp k keeps I_k, the J columns move through shared memory
                const bool mine = valid(warp);
                T qx = T(0), al = T(0);
                if (mine) {
                    bj_load(x, cols + warp * PP, lane);
                    if (lane < NP) qx = Qs[warp * NP + lane];
                    al = nrm[warp];
                }
                bool mine_rot = false;
                for (int round = 0; round < B; ++round) {
                    const int j = B + (warp + round) % B;
                    if (mine && valid(j)) {
                        bj_load(y, cols + j * PP, lane);
                        T be = nrm[j], dx = T(0), dy = T(0);
                        if (bj_rotate(x, y, al, be, tol, thr, sn, tau, dx, dy, skp, rmax)) {
                            if (lane == 0 && dx > T(0)) P.dnorm[sd.s_off + column(warp)] = dx;
                            if (lane == 0 && dy > T(0)) P.dnorm[sd.s_off + column(j)] = dy;
                            bj_store(y, cols + j * PP, lane);
                            if (lane < NP) {
                                T qy = Qs[j * NP + lane];
                                rot_apply(qx, qy, sn, tau);
                                Qs[j * NP + lane] = qy;
                            }
                            if (lane == 0) nrm[j] = be;
                            mine_rot = true;
                        }
                    }
                    __syncthreads();
                }
                if (mine_rot) {
                    bj_store(x, cols + warp * PP, lane);
                    if (lane < NP) Qs[warp * NP + lane] = qx;
                    rotated_any = true;
                }
            }
            if (rotated_any && lane == 0) {
                any_rot = 1;
                atomicMax(&s_rmax, __float_as_int(rmax > 0.0f ? rmax : 1.17549435e-38f));
            }
            __syncthreads();
            if (any_rot) {
                for (int j = warp; j < NP; j += B) {
                    if (!valid(j)) continue;
                    T *dst = W + int64_t(column(j)) * p;
#pragma unroll
                    for (int i = 0; i < R; ++i) {
                        const int r = lane + 32 * i;
                        if (r < p) dst[r] = cols[j * PP + r];
                    }
                }
                if (defer_v) {
                    // record Q and the job; the V update runs in the next step (bj_vwork)
                    if (tid == 0) s_unit = atomicAdd(P.njobs + step, 1);
                    __syncthreads();
                    const int jb = s_unit;
                    const int par = int(step & 1);
                    T *qd = P.qbuf + (int64_t(par) * P.max_jobs + jb) * NP * NP;
                    for (int e = tid; e < NP * NP; e += NT) qd[e] = Qs[e];
                    if (tid == 0) {
                        int *jr = P.jobs + (int64_t(par) * P.max_jobs + jb) * 4;
                        jr[0] = s;
                        jr[1] = a;
                        jr[2] = b;
                        jr[3] = na | (nbc << 16);
                    }
                } else {
                    bj_apply_v<T, B>(V, q, a, b, na, nbc, Qs, 0, q, tid);
                }
                if (tid == 0) atomicMax(P.rotated + int64_t(s) * P.max_sweeps + sweep[s], s_rmax);
            }
            __syncthreads();
        }
        // the previous step's V updates: their columns are disjoint within that step,
        // and the next step's updates of the same columns come after the next barrier
        if (defer_v && step > 0) bj_vwork<T, B>(P, step - 1, Qs, &s_unit, tid);
        grid.sync();
        for (int s = tid; s < nsec; s += NT) {
            if (done[s]) continue;
            const int nb = (P.secs[s].q + B - 1) / B;
            const int nbp = nb + (nb & 1);
            if ((step + 1) % (nbp - 1) == 0) {
                const int sw = sweep[s];
                const int bits = ((volatile int *)P.rotated)[int64_t(s) * P.max_sweeps + sw];
                sweep[s] = sw + 1;
                if (sweep_converged<T>(bits, P.secs[s].p) || sw + 1 >= P.max_sweeps) {
                    done[s] = 1;
                    atomicAdd(&ndone, 1);
                }
            }
        }
        __syncthreads();
    }
    if (defer_v && steps_run > 0) bj_vwork<T, B>(P, steps_run - 1, Qs, &s_unit, tid);
    if (blockIdx.x == 0)
        for (int s = tid; s < nsec; s += NT) P.sweeps[s] = sweep[s];
}

// Deflation thresholds of the SVD sectors: thr[s] = delta2 * ||W_s||_F^2, summed in
// a fixed order (the value, and so every deflation decision, is deterministic);
// 0 for eigh sectors.
template <class T>
__global__ void __launch_bounds__(256) k_defl_thr(const T *__restrict__ work, const SectorDesc *__restrict__ secs,
                                                  double delta2, T *__restrict__ thr) {
    __shared__ double red[8];
    const SectorDesc sd = secs[blockIdx.x];
    const int64_t n = int64_t(sd.p) * sd.q;
    const T *W = work + sd.w_off;
    double acc = 0.0;
    for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
        const double x = double(W[e]);
        acc = fma(x, x, acc);
    }
    acc = wsum(acc);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int i = 0; i < 8; ++i) t += red[i];
        thr[blockIdx.x] = sd.mode == 0 ? T(delta2 * t) : T(0);
    }
}

// One CTA per sector: column norms, ordering, normalisation, completion.
// scratch: at least p doubles per sector at offset w_off (the candidate vector).
// perm_out (with cap == 0): the CTA only orders the columns (S, perm_out at s_off) and
// k_finish_copy writes the factors with many CTAs per sector.
template <class T>
__global__ void __launch_bounds__(1024) k_finish(const T *__restrict__ work, const T *__restrict__ rot,
                                                 double *__restrict__ U, double *__restrict__ V,
                                                 double *__restrict__ S, const SectorDesc *__restrict__ secs,
                                                 double *__restrict__ scratch, int cap, const T *__restrict__ dnorm,
                                                 int *__restrict__ dpos, int *__restrict__ perm_out) {
    extern __shared__ double sh[];
    const SectorDesc sd = secs[blockIdx.x];
    const int q = sd.q, p = sd.p;
    double *sig = sh;                             // q values
    int *perm = reinterpret_cast<int *>(sh + q);  // q ints
    int *defl = perm + q;                         // q flags: column deflated by the sweeps
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    const T *W = work + sd.w_off;
    const T *R = rot + sd.rot_off;
    for (int j = w; j < q; j += nwarp) {
        double acc = 0.0;
        for (int r = lane; r < p; r += 32) {
            double x = double(W[int64_t(j) * p + r]);
            acc = fma(x, x, acc);
        }
        acc = wsum(acc);
        // a deflated column (dnorm given) keeps the norm it had when it left the sweeps
        const double dn = (dnorm && acc == 0.0) ? double(dnorm[sd.s_off + j]) : 0.0;
        if (lane == 0) {
            sig[j] = dn > 0.0 ? sqrt(dn) : sqrt(acc);
            defl[j] = dn > 0.0 ? 1 : 0;
        }
    }
    __syncthreads();
    for (int j = threadIdx.x; j < q; j += blockDim.x) {
        double v = sig[j];
        int rk = 0;
        for (int i = 0; i < q; ++i) {
            double u = sig[i];
            bool before = sd.mode == 0 ? (u > v || (u == v && i < j)) : (u < v || (u == v && i < j));
            rk += before;
        }
        perm[rk] = j;
    }
    __syncthreads();
    if (perm_out)
        for (int j = threadIdx.x; j < q; j += blockDim.x) perm_out[sd.s_off + j] = perm[j];
    if (sd.mode == 1) {
        const int n = q;
        for (int j = threadIdx.x; j < n; j += blockDim.x) S[sd.s_off + j] = sig[perm[j]] - sd.shift;
        if (perm_out) return;
        for (int64_t e = threadIdx.x; e < int64_t(n) * n; e += blockDim.x) {
            int j = int(e / n), r = int(e % n);
            U[sd.u_off + e] = double(R[int64_t(perm[j]) * n + r]);
        }
        return;
    }
    for (int j = threadIdx.x; j < q; j += blockDim.x) {
        S[sd.s_off + j] = sig[perm[j]];
        // 0: resolved column, 1: deflated (left vector to complete), 2: null column
        if (dpos) dpos[sd.s_off + j] = defl[perm[j]] ? 1 : (sig[perm[j]] > 0.0 ? 0 : 2);
    }
    if (perm_out) return;  // k_finish_copy writes the factors
    // the side built from W (length p): U when !trans, V when trans; the other is R (length q)
    double *Wside = sd.trans ? (V + sd.v_off) : (U + sd.u_off);
    double *Rside = sd.trans ? (U + sd.u_off) : (V + sd.v_off);
    for (int64_t e = threadIdx.x; e < int64_t(q) * p; e += blockDim.x) {
        int j = int(e / p), r = int(e % p);
        double sj = sig[perm[j]];
        Wside[e] = (sj > 0.0 && !defl[perm[j]]) ? double(W[int64_t(perm[j]) * p + r]) / sj : 0.0;
    }
    for (int64_t e = threadIdx.x; e < int64_t(q) * q; e += blockDim.x) {
        int j = int(e / q), r = int(e % q);
        Rside[e] = double(R[int64_t(perm[j]) * q + r]);
    }
    __syncthreads();
    // complete null columns of the W side with unit vectors orthogonalised against
    // every other column (modified Gram-Schmidt, twice), so the factor stays an isometry
    __shared__ double red[32];
    __shared__ double bcast;
    __shared__ int accepted;
    double *cand = scratch + sd.w_off;
    int completed = 0;
    for (int jz = 0; jz < q; ++jz) {
        if (sig[perm[jz]] > 0.0) continue;
        if (cap >= 0 && completed >= cap) break;  // the rest are truncated away by the caller
        ++completed;
        for (int e = 0; e < p; ++e) {
            for (int r = threadIdx.x; r < p; r += blockDim.x) cand[r] = (r == e) ? 1.0 : 0.0;
            __syncthreads();
            for (int pass = 0; pass < 2; ++pass) {
                for (int j = 0; j < q; ++j) {
                    if (j == jz || (sig[perm[j]] <= 0.0 && j > jz)) continue;
                    double acc = 0.0;
                    for (int r = threadIdx.x; r < p; r += blockDim.x) acc = fma(Wside[int64_t(j) * p + r], cand[r], acc);
                    acc = wsum(acc);
                    if (lane == 0) red[w] = acc;
                    __syncthreads();
                    if (threadIdx.x == 0) {
                        double t = 0.0;
                        for (int i = 0; i < nwarp; ++i) t += red[i];
                        bcast = t;
                    }
                    __syncthreads();
                    double dj = bcast;
                    for (int r = threadIdx.x; r < p; r += blockDim.x) cand[r] -= dj * Wside[int64_t(j) * p + r];
                    __syncthreads();
                }
            }
            double acc = 0.0;
            for (int r = threadIdx.x; r < p; r += blockDim.x) acc = fma(cand[r], cand[r], acc);
            acc = wsum(acc);
            if (lane == 0) red[w] = acc;
            __syncthreads();
            if (threadIdx.x == 0) {
                double t = 0.0;
                for (int i = 0; i < nwarp; ++i) t += red[i];
                bcast = sqrt(t);
                accepted = bcast > 0.5;
            }
            __syncthreads();
            if (accepted) {
                double inv = 1.0 / bcast;
                for (int r = threadIdx.x; r < p; r += blockDim.x) Wside[int64_t(jz) * p + r] = cand[r] * inv;
                __syncthreads();
                break;
            }
            __syncthreads();
        }
    }
}


// Warm start: tmp = W V0 per sector in 64 x 64 tiles (256 threads, 4 x 4 outputs each,
// K slabs of 16 through shared memory), then (mode 1) work <- tmp and rot <- V0.
template <class T>
__global__ void __launch_bounds__(256) k_warm_gemm(const T *__restrict__ work, T *__restrict__ tmp,
                                                   const WarmDesc *__restrict__ wd, int nwarm) {
    __shared__ T As[16][64 + 1];
    __shared__ T Bs[16][64 + 1];
    int lo = 0, hi = nwarm - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (wd[mid].tile_start <= int(blockIdx.x))
            lo = mid;
        else
            hi = mid - 1;
    }
    const WarmDesc d = wd[lo];
    const int p = d.p, q = d.q;
    const int tm = (p + 63) / 64;
    const int t = int(blockIdx.x) - d.tile_start;
    const int r0 = (t % tm) * 64, c0 = (t / tm) * 64;
    const T *W = work + d.w_off;
    const T *V0 = static_cast<const T *>(d.v0);
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
    for (int k0 = 0; k0 < q; k0 += 16) {
        for (int e = threadIdx.x; e < 16 * 64; e += 256) {
            const int kk = e / 64, i = e % 64;  // A: rows contiguous
            const int r = r0 + i, k = k0 + kk;
            As[kk][i] = (r < p && k < q) ? W[int64_t(k) * p + r] : T(0);
            const int jj = e / 16, kb = e % 16;  // B: k contiguous within a column of V0
            const int c = c0 + jj, kq = k0 + kb;
            Bs[kb][jj] = (c < q && kq < q) ? V0[int64_t(c) * q + kq] : T(0);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; ++kk) {
            T a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int r = r0 + ty + 16 * i, c = c0 + tx + 16 * j;
            if (r < p && c < q) tmp[d.w_off + int64_t(c) * p + r] = acc[i][j];
        }
}

template <class T>
__global__ void __launch_bounds__(256) k_warm_commit(T *__restrict__ work, T *__restrict__ rot,
                                                     const T *__restrict__ tmp, const WarmDesc *__restrict__ wd) {
    const WarmDesc d = wd[blockIdx.y];
    const int64_t nw = int64_t(d.p) * d.q, nr = int64_t(d.q) * d.q;
    const T *V0 = static_cast<const T *>(d.v0);
    for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < nw; e += int64_t(gridDim.x) * blockDim.x)
        work[d.w_off + e] = tmp[d.w_off + e];
    for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < nr; e += int64_t(gridDim.x) * blockDim.x)
        rot[d.rot_off + e] = V0[e];
}

// The factor writes of k_finish spread over many CTAs per sector (grid: chunks of
// 2048 elements x sectors): the W side W[:, perm[j]] / s_j (zero for null or deflated
// columns), the R side R[:, perm[j]]; for eigh U = R[:, perm[j]].
template <class T>
__global__ void __launch_bounds__(256) k_finish_copy(const T *__restrict__ work, const T *__restrict__ rot,
                                                     double *__restrict__ U, double *__restrict__ V,
                                                     const double *__restrict__ S, const SectorDesc *__restrict__ secs,
                                                     const int *__restrict__ perm, const int *__restrict__ dpos) {
    const SectorDesc sd = secs[blockIdx.y];
    const int q = sd.q, p = sd.p;
    const int64_t nw = sd.mode == 1 ? 0 : int64_t(q) * p, n = nw + int64_t(q) * q;
    const int64_t e0 = int64_t(blockIdx.x) * 2048;
    if (e0 >= n) return;
    const T *W = work + sd.w_off;
    const T *R = rot + sd.rot_off;
    const int *pm = perm + sd.s_off;
    double *Wside = sd.trans ? (V + sd.v_off) : (U + sd.u_off);
    double *Rside = sd.mode == 1 ? (U + sd.u_off) : (sd.trans ? (U + sd.u_off) : (V + sd.v_off));
    const int64_t e1 = min(n, e0 + 2048);
    for (int64_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
        if (e < nw) {
            const int j = int(e / p), r = int(e - int64_t(j) * p);
            const double sj = S[sd.s_off + j];
            const bool zero = !(sj > 0.0) || (dpos && dpos[sd.s_off + j] == 1);
            Wside[e] = zero ? 0.0 : double(W[int64_t(pm[j]) * p + r]) / sj;
        } else {
            const int64_t f = e - nw;
            const int j = int(f / q), r = int(f - int64_t(j) * q);
            Rside[f] = double(R[int64_t(pm[j]) * q + r]);
        }
    }
}

int sm_count() { return device_sm_count(); }

// Cooperative grids are sized to the work (pairs or block pairs per step), not to
// the whole GPU, so that small decompositions on concurrent streams overlap.
template <class T, int R>
void jacobi_launch(const JacobiParams<T> &P, size_t smem, int64_t pairs_bound, cudaStream_t stream) {
    static std::atomic<uint64_t> attr{0};
    once_per_device(attr, [] {
        cuda_check(cudaFuncSetAttribute(k_jacobi<T, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024),
                   "Jacobi smem attribute");
    });
    const int nsm = sm_count();
    int occ = 0;
    cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_jacobi<T, R>, JJ, smem), "occupancy");
    if (occ < 1) fail(ERR_RUNTIME, "the Jacobi kernel cannot be resident on an SM");
    const int64_t want = std::max<int64_t>(1, (pairs_bound + JJ / 32 - 1) / (JJ / 32));
    JacobiParams<T> Pc = P;
    void *args[] = {&Pc};
    dim3 grid(unsigned(std::min<int64_t>(int64_t(nsm) * std::min(occ, 4), want))), block(JJ);
    cuda_check(cudaLaunchCooperativeKernel((void *)k_jacobi<T, R>, grid, block, args, smem, stream),
               "cooperative Jacobi launch");
    count_launch();
}

constexpr size_t BJ_SMEM_MAX = 220 * 1024;  // dynamic shared memory of one block-Jacobi CTA

// false when the columns and the per-CTA sector tables (3 ints per sector) do not
// fit one CTA's shared memory; the scalar kernel runs instead
// Bytes of the deferred-V work area for block width B and element size es:
// rotation matrices and job records for two steps, two counters per step.
size_t bj_vwork_bytes(int B, size_t es, int nsec, int64_t sum_q, int64_t max_steps) {
    const int64_t jobs = sum_q / (2 * B) + nsec;
    const size_t np = size_t(2 * B);
    return 2 * size_t(jobs) * np * np * es + 2 * size_t(jobs) * 4 * sizeof(int) + 2 * size_t(max_steps + 1) * sizeof(int) +
           256;
}

template <class T, int B, int R>
bool bjacobi_launch(const BJacobiParams<T> &P, int max_block_steps, int64_t sum_q, void *vwork, size_t vwork_bytes,
                    cudaStream_t stream) {
    const size_t smem = size_t(2 * B) * (32 * R + 2 * B + 1) * sizeof(T) + size_t(3 * P.nsec + 1) * sizeof(int);
    if (smem > BJ_SMEM_MAX) return false;
    static std::atomic<uint64_t> attr{0};
    once_per_device(attr, [] {
        cuda_check(cudaFuncSetAttribute(k_bjacobi<T, B, R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        int(BJ_SMEM_MAX)),
                   "block Jacobi smem attribute");
    });
    const int nsm = sm_count();
    int occ = 0;
    cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_bjacobi<T, B, R>, 32 * B, smem), "occupancy");
    if (occ < 1) fail(ERR_RUNTIME, "the block Jacobi kernel cannot be resident on an SM");
    BJacobiParams<T> Pc = P;
    Pc.max_steps = int64_t(P.max_sweeps) * std::max(1, max_block_steps) + 1;
    Pc.qbuf = nullptr;
    Pc.jobs = Pc.njobs = Pc.vnext = nullptr;
    Pc.max_jobs = 0;
    Pc.upj = 1;
    const size_t need = bj_vwork_bytes(B, sizeof(T), P.nsec, sum_q, Pc.max_steps);
    if (vwork && vwork_bytes >= need) {
        // carve: counters first (zeroed here), then job records, then rotation matrices
        const int64_t jobs = sum_q / (2 * B) + P.nsec;
        char *w = static_cast<char *>(vwork);
        const size_t cbytes = 2 * size_t(Pc.max_steps + 1) * sizeof(int);
        Pc.njobs = reinterpret_cast<int *>(w);
        Pc.vnext = Pc.njobs + (Pc.max_steps + 1);
        Pc.jobs = reinterpret_cast<int *>(w + cbytes);
        const size_t qoff = (cbytes + 2 * size_t(jobs) * 4 * sizeof(int) + 255) & ~size_t(255);
        Pc.qbuf = reinterpret_cast<T *>(w + qoff);
        Pc.max_jobs = int(jobs);
        Pc.upj = std::max(1, int((P.max_q + 32 * B - 1) / (32 * B)));
        cuda_check(cudaMemsetAsync(w, 0, cbytes, stream), "memset block-Jacobi counters");
    }
    void *args[] = {&Pc};
    // block pairs per step: sum over sectors of ceil(ceil(q / B) / 2) <= sum_q / (2B) + nsec
    const int64_t items = sum_q / (2 * B) + P.nsec;
    dim3 grid(unsigned(std::min<int64_t>(int64_t(nsm) * std::min(occ, 2), std::max<int64_t>(1, items)))),
        block(32 * B);
    cuda_check(cudaLaunchCooperativeKernel((void *)k_bjacobi<T, B, R>, grid, block, args, smem, stream),
               "cooperative block Jacobi launch");
    count_launch();
    return true;
}

// Register slice (elements per lane and column) for columns of at most max_p.
int r_class(int max_p) {
    for (int R : {4, 8, 16, 24, 32, 48, 64})
        if (max_p <= 32 * R) return R;
    return 0;
}

// Block widths the block kernel is built with for (element type, R): FP32 16 (R <= 32)
// and 8 (R <= 64); FP64 8 and 4 (R <= 48).  The first entry is the default.
std::vector<int> block_widths(bool f32, int R) {
    if (R == 0) return {};
    if (f32) return R <= 32 ? std::vector<int>{16, 8} : std::vector<int>{8};
    if (R > 48) return {};
    // FP64: two SMs' worth of block pairs per sector at width 4 against one at 8; the
    // FP64 pipe (2 FMA per clock per SM) rather than the round latency bounds a wide sector
    return std::vector<int>{8, 4};
}

// Block kernel for columns up to 2048 (FP32) / 1536 (FP64) elements, as many
// sectors as the shared-memory tables allow, block width B (one of block_widths);
// returns false when the scalar kernel has to run instead.
template <class T>
bool bjacobi_dispatch(const BJacobiParams<T> &P, int max_steps_per_sweep, int max_p, int64_t sum_q, void *vwork,
                      size_t vwork_bytes, int B, cudaStream_t stream) {
    const int max_qp = max_steps_per_sweep + 1;  // the widest sector's even column count
    auto steps = [&](int b) {
        const int nb = (max_qp + b - 1) / b;
        return nb + (nb & 1) - 1;
    };
    const int R = r_class(max_p);
#define QTT_BJ(BB, RR)                                                                                            \
    if (B == BB && R == RR) return bjacobi_launch<T, BB, RR>(P, steps(BB), sum_q, vwork, vwork_bytes, stream);
    if constexpr (sizeof(T) == 4) {
        QTT_BJ(16, 4) QTT_BJ(16, 8) QTT_BJ(16, 16) QTT_BJ(16, 24) QTT_BJ(16, 32)
        QTT_BJ(8, 4) QTT_BJ(8, 8) QTT_BJ(8, 16) QTT_BJ(8, 24) QTT_BJ(8, 32) QTT_BJ(8, 48) QTT_BJ(8, 64)
    } else {
        QTT_BJ(8, 4) QTT_BJ(8, 8) QTT_BJ(8, 16) QTT_BJ(8, 24) QTT_BJ(8, 32) QTT_BJ(8, 48)
        QTT_BJ(4, 4) QTT_BJ(4, 8) QTT_BJ(4, 16) QTT_BJ(4, 24) QTT_BJ(4, 32) QTT_BJ(4, 48)
    }
#undef QTT_BJ
    return false;
}

// ---------------------------------------------------------------------------
// Autotuner of the block width.  Decompositions are classed by element type, R,
// the widest sector (power-of-two bucket) and the sector count (power-of-two
// bucket) -- the shape of the skewed sector-size distribution that decides whether
// wide blocks (fewer grid steps) or narrow ones (more block pairs in flight, fewer
// rounds per step) win.  The first calls of a class run every candidate width
// twice, timed with CUDA events on the launching stream; the faster width is used
// for the class from then on.  QTT_AUTOTUNE_FILE names a file the decisions are
// read from at first use and appended to.
struct TuneKey {
    int f32, R, qcls, ncls;
    bool operator<(const TuneKey &o) const {
        return std::tie(f32, R, qcls, ncls) < std::tie(o.f32, o.R, o.qcls, o.ncls);
    }
};
struct TuneState {
    int tried[2] = {0, 0};
    float best_ms[2] = {1e30f, 1e30f};
    int winner = -1;  // index into block_widths()
};
std::mutex g_tune_mu;
std::map<TuneKey, TuneState> g_tune;
std::atomic<int> g_autotune{1};
bool g_tune_loaded = false;
constexpr int TUNE_TRIALS = 2;

int ceil_log2(int64_t x) {
    int b = 0;
    while ((int64_t(1) << b) < x) ++b;
    return b;
}

void tune_load_locked() {
    if (g_tune_loaded) return;
    g_tune_loaded = true;
    const char *path = std::getenv("QTT_AUTOTUNE_FILE");
    if (!path) return;
    if (FILE *f = std::fopen(path, "r")) {
        TuneKey k;
        int w;
        while (std::fscanf(f, "%d %d %d %d %d", &k.f32, &k.R, &k.qcls, &k.ncls, &w) == 5) g_tune[k].winner = w;
        std::fclose(f);
    }
}

void tune_save(const TuneKey &k, int w) {
    const char *path = std::getenv("QTT_AUTOTUNE_FILE");
    if (!path) return;
    if (FILE *f = std::fopen(path, "a")) {
        std::fprintf(f, "%d %d %d %d %d\n", k.f32, k.R, k.qcls, k.ncls, w);
        std::fclose(f);
    }
}

template <class T>
void jacobi_impl(T *work, T *rot, const SectorDesc *sec, const int *slot_start, int nsec, int max_steps_per_sweep,
                 int max_sweeps, int *sweeps_out, int *flags, int max_p, int64_t sum_q, void *vwork, size_t vwork_bytes,
                 const T *defl, T *dnorm, cudaStream_t stream, bool tune, const T *skip) {
    if (nsec > 12 * 1024) fail(ERR_INVALID_ARGUMENT, "too many sectors for one decomposition launch");
    const size_t smem = size_t(2 * nsec) * sizeof(int);
    cuda_check(cudaMemsetAsync(flags, 0, size_t(nsec) * max_sweeps * sizeof(int), stream), "memset flags");
    if (jacobi_variant() != 1) {
        BJacobiParams<T> B;
        B.work = work;
        B.rot = rot;
        B.secs = sec;
        B.nsec = nsec;
        B.max_sweeps = max_sweeps;
        B.max_steps = 0;
        B.sweeps = sweeps_out;
        B.rotated = flags;
        B.defl = defl;
        B.dnorm = dnorm;
        B.skip = skip;
        B.max_q = max_steps_per_sweep + 1;  // the widest sector's even column count bounds q
        const bool f32 = sizeof(T) == 4;
        const std::vector<int> cands = block_widths(f32, r_class(max_p));
        if (!cands.empty()) {
            int ci = 0;
            bool timing = false;
            const TuneKey key{f32 ? 1 : 0, r_class(max_p), ceil_log2(max_steps_per_sweep + 1), ceil_log2(nsec)};
            if (g_autotune.load() && cands.size() > 1) {
                std::lock_guard<std::mutex> lk(g_tune_mu);
                tune_load_locked();
                TuneState &st = g_tune[key];
                if (st.winner >= 0 && st.winner < int(cands.size())) {
                    ci = st.winner;
                } else if (tune) {
                    ci = st.tried[1] < st.tried[0] ? 1 : 0;
                    timing = true;
                }
            }
            cudaEvent_t e0 = nullptr, e1 = nullptr;
            if (timing) {
                cuda_check(cudaEventCreate(&e0), "cudaEventCreate");
                cuda_check(cudaEventCreate(&e1), "cudaEventCreate");
                cuda_check(cudaEventRecord(e0, stream), "cudaEventRecord");
            }
            const bool ok = bjacobi_dispatch(B, max_steps_per_sweep, max_p, sum_q, vwork, vwork_bytes, cands[ci], stream);
            if (timing) {
                float ms = 0.f;
                cuda_check(cudaEventRecord(e1, stream), "cudaEventRecord");
                cuda_check(cudaEventSynchronize(e1), "cudaEventSynchronize");
                cuda_check(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
                cudaEventDestroy(e0);
                cudaEventDestroy(e1);
                if (ok) {
                    std::lock_guard<std::mutex> lk(g_tune_mu);
                    TuneState &st = g_tune[key];
                    st.tried[ci] += 1;
                    st.best_ms[ci] = std::min(st.best_ms[ci], ms);
                    // decide after TUNE_TRIALS of each width, or as soon as one trial of each
                    // shows a clear gap (> 1.5x and > 2 ms, beyond any first-launch cost)
                    const float lo = std::min(st.best_ms[0], st.best_ms[1]), hi = std::max(st.best_ms[0], st.best_ms[1]);
                    const bool clear = st.tried[0] >= 1 && st.tried[1] >= 1 && hi > 1.5f * lo && hi - lo > 2.0f;
                    if (st.winner < 0 && (clear || (st.tried[0] >= TUNE_TRIALS && st.tried[1] >= TUNE_TRIALS))) {
                        st.winner = st.best_ms[1] < st.best_ms[0] ? 1 : 0;
                        tune_save(key, st.winner);
                    }
                }
            }
            if (ok) return;
        }
    }
    JacobiParams<T> P;
    P.work = work;
    P.rot = rot;
    P.secs = sec;
    P.slot_start = slot_start;
    P.nsec = nsec;
    P.max_sweeps = max_sweeps;
    P.max_steps = int64_t(max_sweeps) * std::max(1, max_steps_per_sweep) + 1;
    P.sweeps = sweeps_out;
    P.rotated = flags;
    P.defl = defl;
    P.dnorm = dnorm;
    P.skip = skip;
    const int64_t pairs = (sum_q + nsec) / 2 + nsec;  // pairs per step, an upper bound
    // registers per lane: the longest column over the sectors decides
    if (max_p <= 4 * 32)
        jacobi_launch<T, 4>(P, smem, pairs, stream);
    else if (max_p <= 8 * 32)
        jacobi_launch<T, 8>(P, smem, pairs, stream);
    else if (max_p <= 16 * 32)
        jacobi_launch<T, 16>(P, smem, pairs, stream);
    else if (max_p <= 32 * 32)
        jacobi_launch<T, 32>(P, smem, pairs, stream);
    else
        jacobi_launch<T, 0>(P, smem, pairs, stream);
}

template <class T>
void finish_impl(const T *work, const T *rot, double *U, double *V, double *s, const SectorDesc *sec, int nsec,
                 int max_q, double *scratch, int cap, const T *dnorm, int *dpos, int *perm_out, int64_t max_elems,
                 cudaStream_t stream) {
    size_t smem = size_t(max_q) * (sizeof(double) + 2 * sizeof(int)) + 16;
    static std::atomic<uint64_t> attr{0};
    once_per_device(attr, [] {
        cuda_check(cudaFuncSetAttribute(k_finish<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024),
                   "finish smem attribute");
    });
    if (smem > 200 * 1024) fail(ERR_INVALID_ARGUMENT, "sector too large for the SVD finishing kernel");
    // with no null column to complete, the factor writes run on many CTAs per sector
    const bool split = perm_out && cap == 0 && max_elems > 0;
    k_finish<T><<<nsec, 1024, smem, stream>>>(work, rot, U, V, s, sec, scratch, cap, dnorm, dpos,
                                              split ? perm_out : nullptr);
    count_launch();
    cuda_check(cudaGetLastError(), "SVD finishing kernel launch");
    if (split) {
        const dim3 grid(unsigned((max_elems + 2047) / 2048), unsigned(nsec));
        k_finish_copy<T><<<grid, 256, 0, stream>>>(work, rot, U, V, s, sec, perm_out, dpos);
        count_launch();
        cuda_check(cudaGetLastError(), "SVD factor copy kernel launch");
    }
}
}  // namespace

void launch_pack(const double *src, void *work, const PackEntry *e, const Chunk *chunks, int64_t nchunks,
                 const SectorDesc *sec, int f32) {
    if (nchunks <= 0) return;
    if (f32)
        k_pack<float><<<unsigned(nchunks), JT, 0, ctx().stream>>>(src, static_cast<float *>(work), e, chunks, sec);
    else
        k_pack<double><<<unsigned(nchunks), JT, 0, ctx().stream>>>(src, static_cast<double *>(work), e, chunks, sec);
    count_launch();
    cuda_check(cudaGetLastError(), "pack kernel launch");
}

void launch_eigh_prepare(void *work, SectorDesc *sec, int nsec, int upper, int f32) {
    if (nsec <= 0) return;
    if (f32)
        k_eigh_prepare<float><<<nsec, JT, 0, ctx().stream>>>(static_cast<float *>(work), sec, upper);
    else
        k_eigh_prepare<double><<<nsec, JT, 0, ctx().stream>>>(static_cast<double *>(work), sec, upper);
    count_launch();
    cuda_check(cudaGetLastError(), "eigh prepare kernel launch");
}

void launch_jacobi_on(cudaStream_t stream, void *work, void *rot, const SectorDesc *sec, const int *slot_start,
                      int nsec, int max_steps_per_sweep, int max_sweeps, int *sweeps_out, int *flags, int f32,
                      int max_p, int64_t sum_q, void *vwork, size_t vwork_bytes, const void *defl, void *dnorm,
                      bool tune, const void *skip) {
    if (nsec <= 0) return;
    if ((defl == nullptr) != (dnorm == nullptr)) fail(ERR_INVALID_ARGUMENT, "deflation needs thresholds and norms");
    if (f32)
        jacobi_impl(static_cast<float *>(work), static_cast<float *>(rot), sec, slot_start, nsec, max_steps_per_sweep,
                    max_sweeps, sweeps_out, flags, max_p, sum_q, vwork, vwork_bytes,
                    static_cast<const float *>(defl), static_cast<float *>(dnorm), stream, tune,
                    static_cast<const float *>(skip));
    else
        jacobi_impl(static_cast<double *>(work), static_cast<double *>(rot), sec, slot_start, nsec,
                    max_steps_per_sweep, max_sweeps, sweeps_out, flags, max_p, sum_q, vwork, vwork_bytes,
                    static_cast<const double *>(defl), static_cast<double *>(dnorm), stream, tune,
                    static_cast<const double *>(skip));
}

void launch_jacobi(void *work, void *rot, const SectorDesc *sec, const int *slot_start, int nsec,
                   int max_steps_per_sweep, int max_sweeps, int *sweeps_out, int *flags, int f32, int max_p,
                   int64_t sum_q, void *vwork, size_t vwork_bytes, const void *defl, void *dnorm, const void *skip) {
    launch_jacobi_on(ctx().stream, work, rot, sec, slot_start, nsec, max_steps_per_sweep, max_sweeps, sweeps_out, flags,
                     f32, max_p, sum_q, vwork, vwork_bytes, defl, dnorm, true, skip);
}

void launch_warm_apply(void *work, void *rot, void *tmp, const WarmDesc *wd, int nwarm, int ntiles, int f32) {
    if (nwarm <= 0 || ntiles <= 0) return;
    if (f32) {
        k_warm_gemm<float><<<ntiles, 256, 0, ctx().stream>>>(static_cast<const float *>(work),
                                                               static_cast<float *>(tmp), wd, nwarm);
        k_warm_commit<float><<<dim3(64, nwarm), 256, 0, ctx().stream>>>(static_cast<float *>(work),
                                                                        static_cast<float *>(rot),
                                                                        static_cast<const float *>(tmp), wd);
    } else {
        k_warm_gemm<double><<<ntiles, 256, 0, ctx().stream>>>(static_cast<const double *>(work),
                                                                static_cast<double *>(tmp), wd, nwarm);
        k_warm_commit<double><<<dim3(64, nwarm), 256, 0, ctx().stream>>>(static_cast<double *>(work),
                                                                         static_cast<double *>(rot),
                                                                         static_cast<const double *>(tmp), wd);
    }
    count_launch();
    count_launch();
    cuda_check(cudaGetLastError(), "warm-start kernel launch");
}

void launch_deflation_thresholds(const void *work, const SectorDesc *sec, int nsec, double delta, void *thr, int f32) {
    if (nsec <= 0) return;
    if (f32)
        k_defl_thr<float><<<nsec, 256, 0, ctx().stream>>>(static_cast<const float *>(work), sec, delta * delta,
                                                          static_cast<float *>(thr));
    else
        k_defl_thr<double><<<nsec, 256, 0, ctx().stream>>>(static_cast<const double *>(work), sec, delta * delta,
                                                           static_cast<double *>(thr));
    count_launch();
    cuda_check(cudaGetLastError(), "deflation threshold kernel launch");
}

size_t jacobi_vwork_bytes(int nsec, int64_t sum_q, int max_steps_per_sweep, int max_sweeps, int f32) {
    const size_t es = f32 ? 4 : 8;
    size_t best = 0;
    for (int B : {8, 16}) {
        const int nb = (max_steps_per_sweep + 1 + B - 1) / B;
        const int64_t steps = int64_t(max_sweeps) * std::max(1, nb + (nb & 1) - 1) + 1;
        best = std::max(best, bj_vwork_bytes(B, es, nsec, sum_q, steps));
    }
    return best;
}

void launch_finish_on(cudaStream_t stream, const void *work, const void *rot, double *U, double *V, double *s,
                      const SectorDesc *sec, int nsec, int max_q, double *scratch, int f32, int complete_cap,
                      const void *dnorm, int *dpos, int *perm_out, int64_t max_elems) {
    if (nsec <= 0) return;
    if (f32)
        finish_impl(static_cast<const float *>(work), static_cast<const float *>(rot), U, V, s, sec, nsec, max_q,
                    scratch, complete_cap, static_cast<const float *>(dnorm), dpos, perm_out, max_elems, stream);
    else
        finish_impl(static_cast<const double *>(work), static_cast<const double *>(rot), U, V, s, sec, nsec, max_q,
                    scratch, complete_cap, static_cast<const double *>(dnorm), dpos, perm_out, max_elems, stream);
}

void launch_finish(const void *work, const void *rot, double *U, double *V, double *s, const SectorDesc *sec, int nsec,
                   int max_q, double *scratch, int f32, int complete_cap, const void *dnorm, int *dpos, int *perm_out,
                   int64_t max_elems) {
    launch_finish_on(ctx().stream, work, rot, U, V, s, sec, nsec, max_q, scratch, f32, complete_cap, dnorm, dpos,
                     perm_out, max_elems);
}

}  // namespace qtt

namespace qtt {
void set_autotune(int on) { g_autotune = on ? 1 : 0; }
std::string autotune_report() {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    std::string out;
    char line[160];
    for (auto &kv : g_tune) {
        const TuneKey &k = kv.first;
        const TuneState &st = kv.second;
        const std::vector<int> c = block_widths(k.f32 != 0, k.R);
        char t0[32] = "-", t1[32] = "-";
        if (st.tried[0]) std::snprintf(t0, sizeof(t0), "%.3f", st.best_ms[0]);
        if (st.tried[1]) std::snprintf(t1, sizeof(t1), "%.3f", st.best_ms[1]);
        std::snprintf(line, sizeof(line), "%s R=%d max_q<=2^%d nsec<=2^%d: B=%d (%s; B=%d %s ms, B=%d %s ms)\n",
                      k.f32 ? "fp32" : "fp64", k.R, k.qcls, k.ncls,
                      st.winner >= 0 && st.winner < int(c.size()) ? c[st.winner] : (c.empty() ? 0 : c[0]),
                      st.winner >= 0 ? "tuned" : "tuning", c.size() > 0 ? c[0] : 0, t0, c.size() > 1 ? c[1] : 0, t1);
        out += line;
    }
    return out;
}
}  // namespace qtt
