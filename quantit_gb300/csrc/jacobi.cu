// Batched per-sector SVD / symmetric eigendecomposition by one-sided (Hestenes)
// Jacobi in FP64.  All sectors of a decomposition run in ONE cooperative launch:
// at every step each sector contributes its round-robin set of disjoint column
// pairs, every warp in the grid takes pairs from the combined list, and a grid
// barrier closes the step.  This replaces the per-sector LAPACK calls of
// btensor_linalg.cpp:483 (torch::svd) and :354 (linalg eigh).
//
// The loop is bounded: at most max_sweeps sweeps per sector.
#include <cooperative_groups.h>

#include "kernels.h"
#include "qtt_core.h"

namespace cg = cooperative_groups;

namespace qtt {
namespace {
constexpr int JT = 256;  // threads per CTA

__device__ __forceinline__ double wsum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
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

struct JacobiParams {
    double *work;
    double *rot;
    const SectorDesc *secs;
    const int *slot_start;  // nsec + 1 prefix sums of pairs per step
    int nsec;
    int max_sweeps;
    int64_t max_steps;
    int *sweeps;   // per sector (written at the end)
    int *rotated;  // nsec * max_sweeps flags, zero on entry: a rotation happened in (sector, sweep)
};

// One grid barrier per step.  Every CTA keeps its own copy of the per-sector
// sweep / done state in shared memory and updates it identically after each
// barrier from the rotation flags, so no second barrier is needed to publish it.
__global__ void __launch_bounds__(JT) k_jacobi(JacobiParams P) {
    cg::grid_group grid = cg::this_grid();
    extern __shared__ int jsh[];
    const int nsec = P.nsec;
    int *done = jsh;            // nsec
    int *sweep = jsh + nsec;    // nsec
    __shared__ int ndone;
    const int lane = threadIdx.x & 31;
    const int64_t gw = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = (int64_t(gridDim.x) * blockDim.x) >> 5;
    const int64_t gt = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t nt = int64_t(gridDim.x) * blockDim.x;
    const int total_slots = P.slot_start[nsec];

    // rotation matrices start as identity; sectors with < 2 columns are done at once
    for (int s = 0; s < nsec; ++s) {
        const SectorDesc sd = P.secs[s];
        const int64_t qq = int64_t(sd.q) * sd.q;
        for (int64_t e = gt; e < qq; e += nt) P.rot[sd.rot_off + e] = (e % (sd.q + 1) == 0) ? 1.0 : 0.0;
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
            // sector of this slot
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
            double *wa = P.work + sd.w_off + int64_t(a) * sd.p;
            double *wb = P.work + sd.w_off + int64_t(b) * sd.p;
            double al = 0.0, be = 0.0, ga = 0.0;
            for (int r = lane; r < sd.p; r += 32) {
                double x = __ldcg(wa + r), y = __ldcg(wb + r);
                al = fma(x, x, al);
                be = fma(y, y, be);
                ga = fma(x, y, ga);
            }
            al = wsum(al);
            be = wsum(be);
            ga = wsum(ga);
            const double tol = 2.220446049250313e-16 * double(sd.p);
            if (ga == 0.0 || fabs(ga) <= tol * sqrt(al) * sqrt(be)) continue;
            const double zeta = (be - al) / (2.0 * ga);
            double t;
            if (fabs(zeta) > 1e150)
                t = 0.5 / zeta;
            else
                t = copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
            const double c = 1.0 / sqrt(1.0 + t * t);
            const double sn = c * t;
            for (int r = lane; r < sd.p; r += 32) {
                double x = __ldcg(wa + r), y = __ldcg(wb + r);
                wa[r] = c * x - sn * y;
                wb[r] = sn * x + c * y;
            }
            double *va = P.rot + sd.rot_off + int64_t(a) * sd.q;
            double *vb = P.rot + sd.rot_off + int64_t(b) * sd.q;
            for (int r = lane; r < sd.q; r += 32) {
                double x = __ldcg(va + r), y = __ldcg(vb + r);
                va[r] = c * x - sn * y;
                vb[r] = sn * x + c * y;
            }
            if (lane == 0) P.rotated[int64_t(s) * P.max_sweeps + sweep[s]] = 1;
        }
        grid.sync();
        // end-of-sweep bookkeeping, identical in every CTA
        for (int s = threadIdx.x; s < nsec; s += blockDim.x) {
            if (done[s]) continue;
            const int q = P.secs[s].q;
            const int qp = q + (q & 1);
            if ((step + 1) % (qp - 1) == 0) {
                const int sw = sweep[s];
                const bool rot = ((volatile int *)P.rotated)[int64_t(s) * P.max_sweeps + sw] != 0;
                sweep[s] = sw + 1;
                if (!rot || sw + 1 >= P.max_sweeps) {
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

// One CTA per sector: column norms, ordering, normalisation, completion.
__global__ void __launch_bounds__(1024) k_finish(double *__restrict__ work, const double *__restrict__ rot,
                                                 double *__restrict__ U, double *__restrict__ V,
                                                 double *__restrict__ S, const SectorDesc *__restrict__ secs) {
    extern __shared__ double sh[];
    const SectorDesc sd = secs[blockIdx.x];
    const int q = sd.q, p = sd.p;
    double *sig = sh;                                 // q values
    int *perm = reinterpret_cast<int *>(sh + q);      // q ints
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    const double *W = work + sd.w_off;
    const double *R = rot + sd.rot_off;
    for (int j = w; j < q; j += nwarp) {
        double acc = 0.0;
        for (int r = lane; r < p; r += 32) acc = fma(W[int64_t(j) * p + r], W[int64_t(j) * p + r], acc);
        acc = wsum(acc);
        if (lane == 0) sig[j] = sqrt(acc);
    }
    __syncthreads();
    // stable rank sort: svd descending by sigma, eigh ascending
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
    if (sd.mode == 1) {
        // eigh: eigenvalues sigma - shift, eigenvectors are the rotation columns
        const int n = q;
        for (int j = threadIdx.x; j < n; j += blockDim.x) S[sd.s_off + j] = sig[perm[j]] - sd.shift;
        for (int64_t e = threadIdx.x; e < int64_t(n) * n; e += blockDim.x) {
            int j = int(e / n), r = int(e % n);
            U[sd.u_off + e] = R[int64_t(perm[j]) * n + r];
        }
        return;
    }
    for (int j = threadIdx.x; j < q; j += blockDim.x) S[sd.s_off + j] = sig[perm[j]];
    // the side built from W (length p): U when !trans, V when trans; the other is R (length q)
    double *Wside = sd.trans ? (V + sd.v_off) : (U + sd.u_off);
    double *Rside = sd.trans ? (U + sd.u_off) : (V + sd.v_off);
    for (int64_t e = threadIdx.x; e < int64_t(q) * p; e += blockDim.x) {
        int j = int(e / p), r = int(e % p);
        double sj = sig[perm[j]];
        Wside[e] = sj > 0.0 ? W[int64_t(perm[j]) * p + r] / sj : 0.0;
    }
    for (int64_t e = threadIdx.x; e < int64_t(q) * q; e += blockDim.x) {
        int j = int(e / q), r = int(e % q);
        Rside[e] = R[int64_t(perm[j]) * q + r];
    }
    __syncthreads();
    // complete null columns of the W side with unit vectors orthogonalised against
    // every other column (modified Gram-Schmidt, twice), so the factor stays an isometry
    __shared__ double red[32];
    __shared__ double bcast;
    __shared__ int accepted;
    // candidate vector: the sector's work columns are no longer read past this point
    double *cand = work + sd.w_off;
    for (int jz = 0; jz < q; ++jz) {
        if (sig[perm[jz]] > 0.0) continue;
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
}  // namespace

void launch_jacobi(double *work, double *rot, const SectorDesc *sec, const int *slot_start, int nsec,
                   int max_steps_per_sweep, int max_sweeps, int *sweeps_out, int *flags) {
    if (nsec <= 0) return;
    static int nsm = 0;
    if (!nsm) {
        int dev = ctx().device;
        cuda_check(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev), "SM count");
        cuda_check(cudaFuncSetAttribute(k_jacobi, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024),
                   "Jacobi smem attribute");
    }
    if (nsec > 12 * 1024) fail(ERR_INVALID_ARGUMENT, "too many sectors for one decomposition launch");
    const size_t smem = size_t(2 * nsec) * sizeof(int);
    int per_sm = 0;
    cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_jacobi, JT, smem), "occupancy");
    per_sm = std::max(1, std::min(per_sm, 4));
    cuda_check(cudaMemsetAsync(flags, 0, size_t(nsec) * max_sweeps * sizeof(int), ctx().stream), "memset flags");
    JacobiParams P;
    P.work = work;
    P.rot = rot;
    P.secs = sec;
    P.slot_start = slot_start;
    P.nsec = nsec;
    P.max_sweeps = max_sweeps;
    P.max_steps = int64_t(max_sweeps) * std::max(1, max_steps_per_sweep) + 1;
    P.sweeps = sweeps_out;
    P.rotated = flags;
    void *args[] = {&P};
    dim3 grid(nsm * per_sm), block(JT);
    cuda_check(cudaLaunchCooperativeKernel((void *)k_jacobi, grid, block, args, smem, ctx().stream),
               "cooperative Jacobi launch");
    count_launch();
}

void launch_finish(double *work, const double *rot, double *U, double *V, double *s, const SectorDesc *sec,
                   int nsec, int max_q) {
    if (nsec <= 0) return;
    size_t smem = size_t(max_q) * (sizeof(double) + sizeof(int)) + 16;
    static bool attr = false;
    if (!attr) {
        cuda_check(cudaFuncSetAttribute(k_finish, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024),
                   "finish smem attribute");
        attr = true;
    }
    if (smem > 200 * 1024) fail(ERR_INVALID_ARGUMENT, "sector too large for the SVD finishing kernel");
    k_finish<<<nsec, 1024, smem, ctx().stream>>>(work, rot, U, V, s, sec);
    count_launch();
    cuda_check(cudaGetLastError(), "SVD finishing kernel launch");
}

}  // namespace qtt
