// Grouped block GEMM on the 5th-generation tensor cores (tcgen05) with
// split-precision TF32 operands: every FP64 operand element x is split into
// hi = tf32(x) and lo = tf32(x - hi), and each output tile accumulates
//     A_hi B_lo + A_lo B_hi + A_hi B_hi
// in FP32 in tensor memory (TMEM).  The dropped A_lo B_lo term and the FP32
// accumulation leave about FP32 accuracy (~1e-7 relative) at a third of the TF32
// tensor throughput -- the "compensated (split-precision) products" of the mixed
// path; everything outside the block GEMMs stays FP64.
//
// Two kernels:
//  * k_split_tf32: one pass over the operand blocks writes hi / lo as FP32 bit
//    patterns in matrix form (rows x K4, K contiguous, zero padded to a multiple
//    of 4).  The FP64 -> FP32 conversion uses integer operations only: GB300's FP64
//    pipe is a small fraction of its FP32 / integer rate.
//  * k_gemm_tf32x3: CTA = one 128 x 128 tile of one output block (same tile and
//    pair tables as the FP64 kernel).  All 8 warps copy 16-byte vectors of the
//    split operands into a 3-stage shared-memory ring in the canonical no-swizzle
//    K-major UMMA layout (core matrices of 8 rows x 16 bytes).  Thread 0 issues
//    the tcgen05.mma instructions of a stage (3 products x 4 k-steps of 8) and
//    commits them to that stage's mbarrier, which the producers wait on before
//    refilling the stage.  The epilogue reads the accumulator with tcgen05.ld and
//    writes alpha*acc + beta*add in FP64 (a plain integer widening when alpha = 1
//    and there is no add term).
//
// Every mbarrier wait is bounded; on timeout the kernel records an error code in
// a device word that the host checks, still waits (bounded) for its MMAs and
// frees its TMEM before returning.
#include <cstdint>
#include <mutex>

#include "kernels.h"
#include "qtt_core.h"
#include "tc_common.cuh"

namespace qtt {
namespace {

constexpr int TBM = 128, TBN = 128, TBK = 32;  // tile and K chunk (elements)
constexpr int TTHREADS = 256;
constexpr int TMEM_COLS = 128;  // FP32 accumulator columns (N)
constexpr int A_BYTES = TBM * TBK * 4;  // one operand copy: 16 KB
constexpr int B_BYTES = TBN * TBK * 4;  // 16 KB
constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;  // hi/lo of A and B: 64 KB
constexpr int NSTAGE = 3;
constexpr int SMEM_BYTES = NSTAGE * STAGE_BYTES + 1024;
using tc::LBO;
using tc::SBO;
using tc::smem_u32;
using tc::make_desc;
using tc::mbar_init;
using tc::mbar_wait;
using tc::amax_shift;
using tc::f64_to_f32_int;
using tc::f32_to_f64_int;
using tc::st_shared_v4;
static_assert(SBO == (TBK * 4 / 16) * 128, "the shared layout assumes 128-byte rows per K chunk");

// kind::tf32, D=F32, A=B=TF32, both K-major, N=128, M=128
__host__ __device__ constexpr uint32_t idesc_tf32() {
    return (1u << 4) | (2u << 7) | (2u << 10) | (uint32_t(TBN >> 3) << 17) | (uint32_t(TBM >> 4) << 24);
}

__device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

__global__ void k_amax(const double *__restrict__ x, int64_t n, unsigned long long *amax) {
    unsigned long long m = 0;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        const unsigned long long v = static_cast<unsigned long long>(__double_as_longlong(x[i])) & 0x7FFFFFFFFFFFFFFFull;
        m = v > m ? v : m;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long u = __shfl_xor_sync(0xffffffffu, m, o);
        m = u > m ? u : m;
    }
    if ((threadIdx.x & 31) == 0 && m) atomicMax(amax, m);
}

__global__ void k_split_tf32(const double *__restrict__ src, float *__restrict__ hi, float *__restrict__ lo,
                             const SplitEntry *__restrict__ ents, const Chunk *__restrict__ chunks,
                             const unsigned long long *__restrict__ amax) {
    const Chunk ch = chunks[blockIdx.x];
    const SplitEntry &e = ents[ch.seg];
    const int r = e.rank;
    const int shift = amax_shift(*amax);
    for (int i = threadIdx.x; i < ch.len; i += blockDim.x) {
        const int64_t lin = ch.start + i;
        int64_t rem = lin, so = e.src_off;
        for (int d = r - 1; d >= 0; --d) {
            const int64_t n = e.dims[d];
            const int64_t q = rem / n;
            so += (rem - q * n) * e.stride[d];
            rem = q;
        }
        const float xf = f64_to_f32_int(src[so], shift);
        const uint32_t h = to_tf32(xf);
        const uint32_t l = to_tf32(xf - __uint_as_float(h));
        const int64_t row = lin / e.K, k = lin - row * e.K;
        const int64_t dst = e.dst_off + row * e.K4 + k;
        hi[dst] = __uint_as_float(h);
        lo[dst] = __uint_as_float(l);
    }
}

// byte offset of (row r, k) in one operand copy of the canonical K-major layout
__device__ __forceinline__ uint32_t kmaj_off(int r, int k) {
    return uint32_t(r >> 3) * SBO + uint32_t(k >> 2) * LBO + uint32_t(r & 7) * 16u + uint32_t(k & 3) * 4u;
}

// rows x (TBK / 4) 16-byte vectors of one operand tile (hi and lo) into shared memory
template <int ROWS>
__device__ __forceinline__ void load_tile(const float *__restrict__ hi, const float *__restrict__ lo, int64_t off,
                                          int rows_valid, int row0, int K4, int k0, char *shi, char *slo, int tid) {
#pragma unroll
    for (int i = 0; i < (ROWS * (TBK / 4)) / TTHREADS; ++i) {
        const int e = tid + i * TTHREADS;
        // eight consecutive threads take eight consecutive rows of one core matrix
        // (one contiguous 128-byte store per quarter warp, no bank conflicts)
        const int row = ((e >> 6) << 3) | (e & 7), kc = (e >> 3) & 7;
        const int gr = row0 + row, gk = k0 + kc * 4;
        uint4 vh = make_uint4(0, 0, 0, 0), vl = make_uint4(0, 0, 0, 0);
        if (gr < rows_valid && gk < K4) {
            const int64_t idx = off + int64_t(gr) * K4 + gk;
            vh = __ldg(reinterpret_cast<const uint4 *>(hi + idx));
            vl = __ldg(reinterpret_cast<const uint4 *>(lo + idx));
        }
        const uint32_t so = kmaj_off(row, kc * 4);
        st_shared_v4(shi + so, vh);
        st_shared_v4(slo + so, vl);
    }
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred q;\n setp.ne.b32 q, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, q;\n}\n" ::"r"(tmem),
        "l"(da), "l"(db), "r"(idesc), "r"(acc));
}

__global__ void __launch_bounds__(TTHREADS, 1) k_gemm_tf32x3(TcArgs g, int *err) {
    extern __shared__ __align__(1024) char smem_raw[];
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

    int nchunk = 0;
    for (int p = o.p0; p < o.p1; ++p) nchunk += ((g.pairs[p].K + 3) / 4 * 4 + TBK - 1) / TBK;

    int p = o.p0, k0 = 0;
    uint32_t commits[NSTAGE] = {};
    for (int c = 0; c < nchunk; ++c) {
        const int s = c % NSTAGE;
        if (c >= NSTAGE) {
            if (!mbar_wait(&mbar[s], (commits[s] - 1) & 1)) {
                if (tid == 0) atomicExch(err, 1);
                abort_flag = 1;
            }
        }
        __syncthreads();
        if (abort_flag) break;
        while (k0 >= ((g.pairs[p].K + 3) & ~3)) {
            ++p;
            k0 = 0;
        }
        const GemmPair pr = g.pairs[p];
        const int K4 = (pr.K + 3) & ~3;
        char *st = smem + s * STAGE_BYTES;
        char *ahi = st, *alo = st + A_BYTES, *bhi = st + 2 * A_BYTES, *blo = st + 2 * A_BYTES + B_BYTES;
        load_tile<TBM>(static_cast<const float *>(g.Ahi), static_cast<const float *>(g.Alo), pr.a_off, o.M, t.m0, K4, k0, ahi, alo, tid);
        load_tile<TBN>(static_cast<const float *>(g.Bhi), static_cast<const float *>(g.Blo), pr.b_off, o.N, t.n0, K4, k0, bhi, blo, tid);
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
                const uint32_t acc0 = (c > 0 || ks > 0) ? 1u : 0u;
                // small terms first, then the leading product
                mma_tf32(tmem, make_desc(a_hi + koff), make_desc(b_lo + koff), idesc, acc0);
                mma_tf32(tmem, make_desc(a_lo + koff), make_desc(b_hi + koff), idesc, 1u);
                mma_tf32(tmem, make_desc(a_hi + koff), make_desc(b_hi + koff), idesc, 1u);
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(&mbar[s]))
                         : "memory");
        }
        commits[s] += 1;
    }
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
    const int shift = amax_shift(*g.amax_a) + amax_shift(*g.amax_b);
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
            // GB300's FP64 pipe is narrow: the plain case (alpha = 1, no add term) converts
            // with integer operations only; FP64 arithmetic only for tensorgdot's epilogue
            const bool plain = g.alpha == 1.0 && o.add_off < 0;
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                const int gn = t.n0 + col0 + j;
                if (gn < o.N) {
                    const int64_t idx = int64_t(gm) * o.N + gn;
                    double val = f32_to_f64_int(__uint_as_float(v[j]), shift);
                    if (!plain) {
                        val *= g.alpha;
                        if (o.add_off >= 0) val += g.beta * g.Cadd[o.add_off + idx];
                    }
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

// the calling thread's error word (one per stream context, so concurrent solves
// on different threads see only their own kernels' status)
int *err_word() {
    Ctx &c = ctx();
    if (!c.tc_err) {
        cuda_check(cudaMalloc(&c.tc_err, sizeof(int)), "cudaMalloc(error word)");
        cuda_check(cudaMemset(c.tc_err, 0, sizeof(int)), "cudaMemset(error word)");
    }
    return c.tc_err;
}

}  // namespace

int gemm_tile_m(int) { return TBM; }
int gemm_tile_n(int) { return TBN; }

void launch_split_tf32(const double *src, float *hi, float *lo, const SplitEntry *e, const Chunk *chunks,
                       int64_t nchunks, const unsigned long long *amax) {
    if (nchunks <= 0) return;
    k_split_tf32<<<unsigned(nchunks), 256, 0, ctx().stream>>>(src, hi, lo, e, chunks, amax);
    count_launch();
    cuda_check(cudaGetLastError(), "split kernel launch");
}

void launch_amax(const double *x, int64_t n, unsigned long long *amax) {
    if (n <= 0) return;
    const int64_t blocks = std::min<int64_t>((n + 2047) / 2048, 4 * 152);
    k_amax<<<unsigned(blocks), 256, 0, ctx().stream>>>(x, n, amax);
    count_launch();
    cuda_check(cudaGetLastError(), "amax kernel launch");
}

void launch_gemm_tc(const TcArgs &a, int mode) {
    if (mode != GEMM_TF32X3 && mode != GEMM_BF16X3) fail(ERR_INVALID_ARGUMENT, "unknown tensor-core GEMM mode");
    if (a.ntiles <= 0) return;
    if (mode == GEMM_BF16X3) {
        launch_gemm_bf16x3(a, err_word(), ctx().stream);
        ctx().tc_used = true;
        return;
    }
    static std::once_flag attr;
    std::call_once(attr, [] {
        cuda_check(cudaFuncSetAttribute(k_gemm_tf32x3, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES),
                   "tcgen05 GEMM smem attribute");
    });
    k_gemm_tf32x3<<<a.ntiles, TTHREADS, SMEM_BYTES, ctx().stream>>>(a, err_word());
    count_launch();
    ctx().tc_used = true;
    cuda_check(cudaGetLastError(), "tcgen05 GEMM launch");
}

// Non-zero when a tensor-core kernel hit a bounded wait (read and cleared; synchronises).
int tc_error_check() {
    Ctx &c = ctx();
    if (!c.tc_used) return 0;
    c.tc_used = false;
    int h = 0;
    cuda_check(cudaMemcpyAsync(&h, err_word(), sizeof(int), cudaMemcpyDeviceToHost, c.stream), "read error word");
    cuda_check(cudaStreamSynchronize(c.stream), "cudaStreamSynchronize");
    if (h) cuda_check(cudaMemsetAsync(err_word(), 0, sizeof(int), c.stream), "clear error word");
    return h;
}

}  // namespace qtt
