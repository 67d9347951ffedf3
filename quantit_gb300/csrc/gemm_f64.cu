// Grouped FP64 block GEMM: every charge-matched block product of one
// contraction in one launch (btensor::tensordot's mm / addmm_ loop,
// sources/btensor.cpp:2057-2114).  One CTA computes a 64x64 tile of one output
// block and accumulates all of that block's matching (A, B) pairs in registers
// before a single store, so no output block is written twice.
//
// FP64 has no tcgen05 kind; on GB300 this path is bound by the FP64 pipe.
#include "kernels.h"
#include "qtt_core.h"

namespace qtt {
namespace {
constexpr int BM = 64, BN = 64, BK = 16, THREADS = 256;

__global__ void __launch_bounds__(THREADS) k_gemm_f64(GemmArgs g) {
    const GemmTile t = g.tiles[blockIdx.x];
    const GemmOut o = g.outs[t.out];
    __shared__ double As[BK][BM + 1];
    __shared__ double Bs[BK][BN + 1];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    double acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;

    for (int p = o.p0; p < o.p1; ++p) {
        const GemmPair pr = g.pairs[p];
        const double *__restrict__ A = g.A + pr.a_off;
        const double *__restrict__ B = g.B + pr.b_off;
        const int K = pr.K;
        for (int k0 = 0; k0 < K; k0 += BK) {
#pragma unroll
            for (int i = 0; i < (BM * BK) / THREADS; ++i) {
                int e = tid + i * THREADS;
                int m, k;
                if (!g.a_t) {
                    k = e % BK;
                    m = e / BK;
                } else {
                    m = e % BM;
                    k = e / BM;
                }
                int gm = t.m0 + m, gk = k0 + k;
                double v = 0.0;
                if (gm < o.M && gk < K) v = g.a_t ? A[int64_t(gk) * o.M + gm] : A[int64_t(gm) * K + gk];
                As[k][m] = v;
            }
#pragma unroll
            for (int i = 0; i < (BN * BK) / THREADS; ++i) {
                int e = tid + i * THREADS;
                int n, k;
                if (!g.b_t) {
                    n = e % BN;
                    k = e / BN;
                } else {
                    k = e % BK;
                    n = e / BK;
                }
                int gn = t.n0 + n, gk = k0 + k;
                double v = 0.0;
                if (gn < o.N && gk < K) v = g.b_t ? B[int64_t(gn) * K + gk] : B[int64_t(gk) * o.N + gn];
                Bs[k][n] = v;
            }
            __syncthreads();
#pragma unroll
            for (int k = 0; k < BK; ++k) {
                double a[4], b[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) a[i] = As[k][ty + 16 * i];
#pragma unroll
                for (int j = 0; j < 4; ++j) b[j] = Bs[k][tx + 16 * j];
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
            }
            __syncthreads();
        }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        int m = t.m0 + ty + 16 * i;
        if (m >= o.M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            int n = t.n0 + tx + 16 * j;
            if (n >= o.N) continue;
            int64_t idx = int64_t(m) * o.N + n;
            double v = g.alpha * acc[i][j];
            if (o.add_off >= 0) v += g.beta * g.Cadd[o.add_off + idx];
            g.C[o.c_off + idx] = v;
        }
    }
}
}  // namespace

void launch_gemm_f64(const GemmArgs &a) {
    if (a.ntiles <= 0) return;
    k_gemm_f64<<<a.ntiles, THREADS, 0, ctx().stream>>>(a);
    count_launch();
    cuda_check(cudaGetLastError(), "grouped FP64 GEMM launch");
}

}  // namespace qtt
