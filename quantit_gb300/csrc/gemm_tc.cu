// Grouped block GEMM on the 5th-generation tensor cores (tcgen05) with
// split-precision TF32 operands: every FP64 operand element x is split into
// hi = tf32(x) and lo = tf32(x - hi), and each output tile accumulates
//     A_hi B_hi + A_hi B_lo + A_lo B_hi
// in FP32 in tensor memory (TMEM).  The dropped A_lo B_lo term and the FP32
// accumulation leave about FP32 accuracy (~1e-7 relative) at a third of the TF32
// tensor throughput -- the "compensated (split-precision) products" of the mixed
// path; everything outside the block GEMMs stays FP64.
//
// CTA = one 128 x 128 tile of one output block (same tile/pair tables as the FP64
// kernel).  All 8 warps produce: they read FP64 A / B from global memory (plain,
// transposed or packed layouts), split, and store hi/lo into a 2-stage shared
// memory ring in the canonical no-swizzle K-major UMMA layout (core matrices of
// 8 rows x 16 bytes).  Thread 0 issues the tcgen05.mma instructions of a stage
// (3 products x 4 k-steps of 8) and commits them to that stage's mbarrier, which
// the producers wait on before refilling the stage.  The epilogue reads the
// accumulator with tcgen05.ld and writes alpha*acc + beta*add in FP64.
//
// Every mbarrier wait is bounded; on timeout the kernel records an error code in
// a device word that the host checks, still waits (bounded) for its MMAs and
// frees its TMEM before returning.
#include <cstdint>

#include "kernels.h"
#include "qtt_core.h"

namespace qtt {
namespace {

constexpr int TBM = 128, TBN = 128, TBK = 32;  // tile and K chunk (elements)
constexpr int TTHREADS = 256;
constexpr int TMEM_COLS = 128;  // FP32 accumulator columns (N)
// one operand copy (rows x TBK tf32) = rows * 128 bytes; core matrix = 8 rows x 16 B
constexpr int A_BYTES = TBM * TBK * 4;  // 16 KB
constexpr int B_BYTES = TBN * TBK * 4;  // 16 KB
constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;  // hi/lo of A and B: 64 KB
constexpr int NSTAGE = 2;
constexpr int SMEM_BYTES = NSTAGE * STAGE_BYTES + 1024;
constexpr uint32_t LBO = 128;               // K-adjacent core matrices
constexpr uint32_t SBO = (TBK * 4 / 16) * 128;  // next 8-row group: 1024 B
constexpr long long WAIT_LIMIT = 1ll << 22;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t make_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= uint64_t((saddr & 0x3FFFF) >> 4);
    d |= uint64_t(LBO >> 4) << 16;
    d |= uint64_t(SBO >> 4) << 32;
    d |= uint64_t(1) << 46;  // descriptor version for tcgen05
    // base offset 0, no swizzle (layout type 0)
    return d;
}

// kind::tf32, D=F32, A=B=TF32, both K-major, N=128, M=128
__host__ __device__ constexpr uint32_t idesc_tf32() {
    return (1u << 4) | (2u << 7) | (2u << 10) | (uint32_t(TBN >> 3) << 17) | (uint32_t(TBM >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    const uint32_t a = smem_u32(bar);
    for (long long it = 0; it < WAIT_LIMIT; ++it) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.b32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(a), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

__device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

// byte offset of element (row r, k) in one operand copy
__device__ __forceinline__ uint32_t kmaj_off(int r, int k) {
    return uint32_t(r >> 3) * SBO + uint32_t(k >> 2) * LBO + uint32_t(r & 7) * 16u + uint32_t(k & 3) * 4u;
}

__device__ __forceinline__ void split_store(char *hi, char *lo, uint32_t off, double x) {
    const uint32_t h = to_tf32(float(x));
    const double rem = x - double(__uint_as_float(h));
    const uint32_t l = to_tf32(float(rem));
    *reinterpret_cast<uint32_t *>(hi + off) = h;
    *reinterpret_cast<uint32_t *>(lo + off) = l;
}

__global__ void __launch_bounds__(TTHREADS, 1) k_gemm_tf32x3(GemmArgs g, int *err) {
    extern __shared__ __align__(1024) char smem_raw[];
    // align the ring to 1024 bytes
    char *smem = reinterpret_cast<char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    __shared__ uint64_t mbar[NSTAGE];
    __shared__ uint32_t tmem_base_sh;
    __shared__ int abort_flag;

    const GemmTile t = g.tiles[blockIdx.x];
    const GemmOut o = g.outs[t.out];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_sh)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        for (int s = 0; s < NSTAGE; ++s) mbar_init(&mbar[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;");
        abort_flag = 0;
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_base_sh;

    // chunk list of this output block: (pair, k0) in pair order
    int nchunk = 0;
    for (int p = o.p0; p < o.p1; ++p) nchunk += (g.pairs[p].K + TBK - 1) / TBK;

    int p = o.p0, k0 = 0;
    uint32_t commits[NSTAGE] = {0, 0};
    for (int c = 0; c < nchunk; ++c) {
        const int s = c % NSTAGE;
        // wait until the MMAs that last read this stage are complete
        if (c >= NSTAGE) {
            if (!mbar_wait(&mbar[s], (commits[s] - 1) & 1)) {
                if (tid == 0) atomicExch(err, 1);
                abort_flag = 1;
            }
        }
        __syncthreads();
        if (abort_flag) break;
        // advance to the chunk's pair
        while (k0 >= g.pairs[p].K) {
            ++p;
            k0 = 0;
        }
        const GemmPair pr = g.pairs[p];
        const int K = pr.K;
        const double *__restrict__ A = g.A + pr.a_off;
        const double *__restrict__ B = g.B + pr.b_off;
        char *st = smem + s * STAGE_BYTES;
        char *ahi = st, *alo = st + A_BYTES, *bhi = st + 2 * A_BYTES, *blo = st + 2 * A_BYTES + B_BYTES;
        // A tile: 128 rows (m) x 32 (k)
#pragma unroll 4
        for (int i = 0; i < (TBM * TBK) / TTHREADS; ++i) {
            const int e = tid + i * TTHREADS;
            int m, k;
            if (!g.a_t) {
                k = e & (TBK - 1);
                m = e / TBK;
            } else {
                m = e & (TBM - 1);
                k = e / TBM;
            }
            const int gm = t.m0 + m, gk = k0 + k;
            double x = 0.0;
            if (gm < o.M && gk < K) x = g.a_t ? A[int64_t(gk) * o.M + gm] : A[int64_t(gm) * K + gk];
            split_store(ahi, alo, kmaj_off(m, k), x);
        }
        // B tile stored N-rows x K (K-major): 128 (n) x 32 (k)
#pragma unroll 4
        for (int i = 0; i < (TBN * TBK) / TTHREADS; ++i) {
            const int e = tid + i * TTHREADS;
            int n, k;
            if (!g.b_t) {
                n = e & (TBN - 1);
                k = e / TBN;
            } else {
                k = e & (TBK - 1);
                n = e / TBK;
            }
            const int gn = t.n0 + n, gk = k0 + k;
            double x = 0.0;
            if (gn < o.N && gk < K) x = g.b_t ? B[int64_t(gn) * K + gk] : B[int64_t(gk) * o.N + gn];
            split_store(bhi, blo, kmaj_off(n, k), x);
        }
        k0 += TBK;
        // make the generic-proxy stores visible to the tensor core
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint32_t idesc = idesc_tf32();
            const uint32_t a_hi = smem_u32(ahi), a_lo = smem_u32(alo), b_hi = smem_u32(bhi), b_lo = smem_u32(blo);
#pragma unroll
            for (int ks = 0; ks < TBK / 8; ++ks) {
                const uint32_t koff = uint32_t(ks) * 2u * LBO;  // 8 tf32 = 2 core matrices along K
                const uint64_t dAh = make_desc(a_hi + koff), dAl = make_desc(a_lo + koff);
                const uint64_t dBh = make_desc(b_hi + koff), dBl = make_desc(b_lo + koff);
                // small terms first, then the leading product
                const uint32_t acc0 = (c > 0 || ks > 0) ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred q;\n setp.ne.b32 q, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, q;\n}\n" ::"r"(tmem),
                    "l"(dAh), "l"(dBl), "r"(idesc), "r"(acc0));
                asm volatile(
                    "{\n .reg .pred q;\n setp.ne.b32 q, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, q;\n}\n" ::"r"(tmem),
                    "l"(dAl), "l"(dBh), "r"(idesc), "r"(1u));
                asm volatile(
                    "{\n .reg .pred q;\n setp.ne.b32 q, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, q;\n}\n" ::"r"(tmem),
                    "l"(dAh), "l"(dBh), "r"(idesc), "r"(1u));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(&mbar[s]))
                         : "memory");
        }
        commits[s] += 1;
    }
    // wait for every outstanding commit before reading the accumulator (or freeing TMEM)
    for (int s = 0; s < NSTAGE; ++s) {
        if (commits[s] == 0) continue;
        if (!mbar_wait(&mbar[s], (commits[s] - 1) & 1)) {
            if (tid == 0) atomicExch(err, 2);
        }
    }
    asm volatile("tcgen05.fence::after_thread_sync;");
    __syncthreads();

    // epilogue: warp w reads TMEM lanes 32*(w%4).., columns 64*(w/4) .. +63
    const int quarter = warp & 3, half = warp >> 2;
    const int row = quarter * 32 + lane;
    const int gm = t.m0 + row;
    const bool have_acc = nchunk > 0 && !abort_flag;
#pragma unroll
    for (int cb = 0; cb < 2; ++cb) {
        const int col0 = half * 64 + cb * 32;
        uint32_t v[32];
        if (have_acc) {
            const uint32_t taddr = tmem + (uint32_t(quarter * 32) << 16) + uint32_t(col0);
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                  "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
                  "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
                  "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        } else {
#pragma unroll
            for (int j = 0; j < 32; ++j) v[j] = 0u;
        }
        if (gm < o.M) {
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                const int gn = t.n0 + col0 + j;
                if (gn < o.N) {
                    const int64_t idx = int64_t(gm) * o.N + gn;
                    double val = g.alpha * double(__uint_as_float(v[j]));
                    if (o.add_off >= 0) val += g.beta * g.Cadd[o.add_off + idx];
                    g.C[o.c_off + idx] = val;
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
    }
}

std::atomic<bool> g_tc_used{false};  // a tensor-core launch happened since the last error check

int *err_word() {
    static int *p = nullptr;
    if (!p) {
        cuda_check(cudaMalloc(&p, sizeof(int)), "cudaMalloc(error word)");
        cuda_check(cudaMemset(p, 0, sizeof(int)), "cudaMemset(error word)");
    }
    return p;
}

}  // namespace

int gemm_tile_m(int) { return TBM; }
int gemm_tile_n(int) { return TBN; }

void launch_gemm_tc(const GemmArgs &a, int mode) {
    if (mode != GEMM_TF32X3) fail(ERR_INVALID_ARGUMENT, "this tensor-core GEMM precision mode is not built");
    if (a.ntiles <= 0) return;
    static bool attr = false;
    if (!attr) {
        cuda_check(cudaFuncSetAttribute(k_gemm_tf32x3, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES),
                   "tcgen05 GEMM smem attribute");
        attr = true;
    }
    k_gemm_tf32x3<<<a.ntiles, TTHREADS, SMEM_BYTES, ctx().stream>>>(a, err_word());
    count_launch();
    g_tc_used = true;
    cuda_check(cudaGetLastError(), "tcgen05 GEMM launch");
}

// Non-zero when a tensor-core kernel hit a bounded wait (read and cleared; synchronises).
int tc_error_check() {
    if (!g_tc_used.exchange(false)) return 0;
    int h = 0;
    cuda_check(cudaStreamSynchronize(ctx().stream), "cudaStreamSynchronize");
    cuda_check(cudaMemcpy(&h, err_word(), sizeof(int), cudaMemcpyDeviceToHost), "read error word");
    if (h) cuda_check(cudaMemset(err_word(), 0, sizeof(int)), "clear error word");
    return h;
}

}  // namespace qtt
