// FP64 refinement of the mixed path's sector SVDs.
//
// QuantiT decomposes every sector in FP64 (torch::svd, sources/btensor_linalg.cpp:483).
// The mixed path keeps that accuracy while doing most sweeps in FP32: the one-sided
// Jacobi first runs on an FP32 copy of each sector (FP32 runs at 64x the FP64 rate on
// GB300's CUDA cores), and its accumulated rotation V0 then starts an FP64 Jacobi on
// the FP64 sector matrix:
//
//   1. V0 is orthogonal only to ~1e-6 (FP32 accumulation).  Two Newton-Schulz steps
//      V <- V (3 I - V^T V) / 2 in FP64 make it orthogonal to FP64 precision (each step
//      squares the departure from orthogonality: 1e-6 -> 1e-12 -> 1e-16).
//   2. W1 = W V in FP64 from the FP64 sector matrix W.
//   3. The FP64 Jacobi sweeps run on (W1, V).  Any orthogonal V gives an exact SVD of
//      W (W V = U S Vt^T => W = U S (V Vt)^T), so the factors are an FP64 SVD; from the
//      near-diagonal W1 the columns FP32 resolved converge in a sweep or two.
//
// All three steps are batched FP64 GEMMs over the sectors of one decomposition
// (k_secgemm): 64 x 64 output tiles, 256 threads with 4 x 4 outputs each, K slabs
// of 16 through shared memory.  GB300's FP64 pipe (about 2 FMA per clock per SM)
// bounds them; shared-memory traffic is 8 loads per 16 FMA.
#include "kernels.h"
#include "qtt_core.h"

namespace qtt {
namespace {

// C[M x N] (column-major, ldc) = op(A) B', A = M x K (a_trans: stored K x M), and
// B' = B (K x N) or, with b_ns, 1.5 I - 0.5 B (the Newton-Schulz factor).  sym bit 0: C is
// symmetric (A^T A), only tiles on or above the diagonal are computed; bit 1: B is such a
// matrix, its elements below the diagonal are read from above it.
struct SecGemm {
    int64_t a_off, b_off, c_off;
    int32_t M, N, K, lda, ldb, ldc;
    int32_t a_trans, b_ns, tile_start, sym;
};

template <class TA, class TB>
__global__ void __launch_bounds__(256) k_secgemm(const TA *__restrict__ A, const TB *__restrict__ B,
                                                 double *__restrict__ C, const SecGemm *__restrict__ g, int ng) {
    __shared__ double As[16][64 + 1];
    __shared__ double Bs[16][64 + 1];
    int lo = 0, hi = ng - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (g[mid].tile_start <= int(blockIdx.x))
            lo = mid;
        else
            hi = mid - 1;
    }
    const SecGemm d = g[lo];
    const int tm = (d.M + 63) / 64;
    const int t = int(blockIdx.x) - d.tile_start;
    const int r0 = (t % tm) * 64, c0 = (t / tm) * 64;
    if ((d.sym & 1) && c0 + 63 < r0) return;  // strictly below the diagonal of a symmetric C
    const TA *a = A + d.a_off;
    const TB *b = B + d.b_off;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    double acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
    for (int k0 = 0; k0 < d.K; k0 += 16) {
        for (int e = threadIdx.x; e < 16 * 64; e += 256) {
            // A tile: the stored layout's contiguous index runs fastest across threads
            int i, kk;
            if (d.a_trans) {
                kk = e % 16;
                i = e / 16;
            } else {
                i = e % 64;
                kk = e / 64;
            }
            const int r = r0 + i, k = k0 + kk;
            double av = 0.0;
            if (r < d.M && k < d.K)
                av = double(d.a_trans ? a[int64_t(r) * d.lda + k] : a[int64_t(k) * d.lda + r]);
            As[kk][i] = av;
            // B tile: k contiguous within a column
            const int kb = e % 16, jj = e / 16;
            const int c = c0 + jj, kq = k0 + kb;
            double bv = 0.0;
            if (c < d.N && kq < d.K) {
                const int lo = (d.sym & 2) ? min(kq, c) : kq, hi = (d.sym & 2) ? max(kq, c) : c;
                bv = double(b[int64_t(hi) * d.ldb + lo]);
                if (d.b_ns) bv = (kq == c ? 1.5 : 0.0) - 0.5 * bv;
            }
            Bs[kb][jj] = bv;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; ++kk) {
            double av[4], bv[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) av[i] = As[kk][tx + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) bv[j] = Bs[kk][ty + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(av[i], bv[j], acc[i][j]);
        }
        __syncthreads();
    }
    double *c = C + d.c_off;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int col = c0 + ty + 16 * j;
        if (col >= d.N) continue;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int row = r0 + tx + 16 * i;
            if (row < d.M) c[int64_t(col) * d.ldc + row] = acc[i][j];
        }
    }
}

template <class TA, class TB>
void secgemm(const TA *A, const TB *B, double *C, std::vector<SecGemm> &tasks, cudaStream_t st) {
    int tiles = 0;
    std::vector<SecGemm> live;
    for (SecGemm &t : tasks) {
        if (t.M <= 0 || t.N <= 0 || t.K <= 0) continue;
        t.tile_start = tiles;
        tiles += ((t.M + 63) / 64) * ((t.N + 63) / 64);
        live.push_back(t);
    }
    if (live.empty()) return;
    const SecGemm *dg = upload_vec(live);
    k_secgemm<TA, TB><<<tiles, 256, 0, st>>>(A, B, C, dg, int(live.size()));
    count_launch();
    cuda_check(cudaGetLastError(), "sector GEMM launch");
}

// Squared column norms of every sector matrix (one warp per column).
template <class T>
__global__ void k_col_norms(const T *__restrict__ W, const SectorDesc *__restrict__ secs,
                            double *__restrict__ out) {
    const SectorDesc sd = secs[blockIdx.y];
    const int lane = threadIdx.x & 31;
    const int col = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (col >= sd.q) return;
    const T *w = W + sd.w_off + int64_t(col) * sd.p;
    double acc = 0.0;
    for (int r = lane; r < sd.p; r += 32) acc = fma(double(w[r]), double(w[r]), acc);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) out[sd.s_off + col] = acc;
}

__global__ void __launch_bounds__(256) k_col_copy(const double *__restrict__ src, double *__restrict__ dst,
                                                  const ColCopy *__restrict__ cc, int n) {
    for (int c = blockIdx.x; c < n; c += gridDim.x) {
        const ColCopy e = cc[c];
        for (int r = threadIdx.x; r < e.len; r += blockDim.x) dst[e.dst_off + r] = src[e.src_off + r];
    }
}

}  // namespace

void launch_col_copy(const double *src, double *dst, const std::vector<ColCopy> &cols) {
    if (cols.empty()) return;
    const ColCopy *d = upload_vec(cols);
    const int grid = int(std::min<size_t>(cols.size(), 8192));
    k_col_copy<<<grid, 256, 0, ctx().stream>>>(src, dst, d, int(cols.size()));
    count_launch();
    cuda_check(cudaGetLastError(), "column copy launch");
}

void launch_rot_product(const double *vg, const double *r, double *vn, const std::vector<RotProduct> &t) {
    std::vector<SecGemm> g;
    for (const RotProduct &e : t)
        g.push_back({e.vg_off, e.r_off, e.vn_off, e.vrows, e.k, e.k, e.vrows, e.k, e.vrows, 0, 0, 0, 0});
    secgemm(vg, r, vn, g, ctx().stream);
}

void launch_col_norms(const void *W, const SectorDesc *secs, int nsec, int max_q, double *out, int f32) {
    if (nsec <= 0 || max_q <= 0) return;
    const dim3 grid(unsigned((max_q + 7) / 8), unsigned(nsec));
    if (f32)
        k_col_norms<float><<<grid, 256, 0, ctx().stream>>>(static_cast<const float *>(W), secs, out);
    else
        k_col_norms<double><<<grid, 256, 0, ctx().stream>>>(static_cast<const double *>(W), secs, out);
    count_launch();
    cuda_check(cudaGetLastError(), "column norm launch");
}

void launch_svd_refine(const float *rot32, const double *w64, double *w1, double *va, double *vb, double *g,
                       const std::vector<SectorDesc> &secs) {
    cudaStream_t st = ctx().stream;
    auto gram = [&]() {
        std::vector<SecGemm> t;
        for (const SectorDesc &s : secs)
            t.push_back({s.rot_off, s.rot_off, s.rot_off, s.q, s.q, s.q, s.q, s.q, s.q, 1, 0, 0, 1});
        return t;
    };
    auto ns = [&]() {
        std::vector<SecGemm> t;
        for (const SectorDesc &s : secs)
            t.push_back({s.rot_off, s.rot_off, s.rot_off, s.q, s.q, s.q, s.q, s.q, s.q, 0, 1, 0, 2});
        return t;
    };
    // Newton-Schulz step 1 from the FP32 rotation: G = V0^T V0, va = V0 (1.5 I - 0.5 G)
    {
        auto t = gram();
        secgemm(rot32, rot32, g, t, st);
        auto u = ns();
        secgemm(rot32, static_cast<const double *>(g), va, u, st);
    }
    // step 2 in FP64: G = va^T va, vb = va (1.5 I - 0.5 G)
    {
        auto t = gram();
        secgemm(static_cast<const double *>(va), static_cast<const double *>(va), g, t, st);
        auto u = ns();
        secgemm(static_cast<const double *>(va), static_cast<const double *>(g), vb, u, st);
    }
    // W1 = W vb
    std::vector<SecGemm> t;
    for (const SectorDesc &s : secs)
        t.push_back({s.w_off, s.rot_off, s.w_off, s.p, s.q, s.q, s.p, s.q, s.p, 0, 0, 0, 0});
    secgemm(w64, static_cast<const double *>(vb), w1, t, st);
}

}  // namespace qtt
