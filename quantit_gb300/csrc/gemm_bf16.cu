// Grouped block GEMM on the tcgen05 tensor cores with split-BF16 operands: every
// (power-of-two scaled) operand element x is split into three bf16 terms
//     hi = bf16(x), mid = bf16(x - hi), lo = bf16(x - hi - mid)
// carrying 24 significant bits together, and each output tile accumulates the six
// products of order <= 2,
//     A_hi B_lo + A_mid B_mid + A_lo B_hi + A_hi B_mid + A_mid B_hi + A_hi B_hi,
// in FP32 in TMEM (tcgen05.mma kind::f16 with BF16 A and B).  The dropped terms are
// O(2^-24) relative, the FP32 accumulation level: the "split-BF16 with FP32
// accumulation plus compensated correction" precision mode (QTT_GEMM_BF16X3).  Six
// BF16 products cost the tensor time of three TF32 products (BF16 runs at twice the
// TF32 rate) and move 3 x 2 bytes per operand element instead of 2 x 4.
//
// Layout and pipeline follow k_gemm_tf32x3: one 128 x 128 output tile per CTA,
// 8 warps copy 16-byte vectors of the split operands (rows x K8, K contiguous,
// zero padded to a multiple of 8) into the canonical no-swizzle K-major layout
// (128-byte rows per K chunk of 64 bf16), a 2-stage ring of 96 KB stages, thread 0
// issues 6 products x 4 k-steps of 16 per stage and commits them to the stage's
// mbarrier.  Every wait is bounded; on timeout the kernel records an error code,
// still waits (bounded) for its MMAs and frees its TMEM.
#include <cstdint>
#include <mutex>

#include "kernels.h"
#include "qtt_core.h"
#include "tc_common.cuh"

namespace qtt {
namespace {

constexpr int BM = 128, BN = 128, BK = 64;  // tile and K chunk (bf16 elements: 128 bytes per row)
constexpr int BTHREADS = 256;
constexpr int BTMEM_COLS = 128;
constexpr int COPY_BYTES = 128 * BK * 2;           // one operand copy (hi, mid or lo): 16 KB
constexpr int BSTAGE_BYTES = 6 * COPY_BYTES;       // hi/mid/lo of A and B: 96 KB
constexpr int BNSTAGE = 2;
constexpr int BSMEM_BYTES = BNSTAGE * BSTAGE_BYTES + 1024;
using tc::LBO;
using tc::SBO;
static_assert(SBO == (BK * 2 / 16) * 128, "the shared layout assumes 128-byte rows per K chunk");

// kind::f16, D=F32, A=B=BF16, both K-major, N=128, M=128
__host__ __device__ constexpr uint32_t idesc_bf16() {
    return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(BN >> 3) << 17) | (uint32_t(BM >> 4) << 24);
}

__device__ __forceinline__ uint16_t to_bf16(float x) {
    uint16_t r;
    asm("cvt.rn.bf16.f32 %0, %1;" : "=h"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float from_bf16(uint16_t h) { return __uint_as_float(uint32_t(h) << 16); }

__global__ void k_split_bf16x3(const double *__restrict__ src, uint16_t *__restrict__ hi, uint16_t *__restrict__ mid,
                               uint16_t *__restrict__ lo, const SplitEntry *__restrict__ ents,
                               const Chunk *__restrict__ chunks, const unsigned long long *__restrict__ amax) {
    const Chunk ch = chunks[blockIdx.x];
    const SplitEntry &e = ents[ch.seg];
    const int r = e.rank;
    const int shift = tc::amax_shift(*amax);
    for (int i = threadIdx.x; i < ch.len; i += blockDim.x) {
        const int64_t lin = ch.start + i;
        int64_t rem = lin, so = e.src_off;
        for (int d = r - 1; d >= 0; --d) {
            const int64_t n = e.dims[d];
            const int64_t q = rem / n;
            so += (rem - q * n) * e.stride[d];
            rem = q;
        }
        const float x = tc::f64_to_f32_int(src[so], shift);
        const uint16_t h = to_bf16(x);
        const float r1 = x - from_bf16(h);
        const uint16_t m = to_bf16(r1);
        const uint16_t l = to_bf16(r1 - from_bf16(m));
        const int64_t row = lin / e.K, k = lin - row * e.K;
        const int64_t dst = e.dst_off + row * e.K4 + k;
        hi[dst] = h;
        mid[dst] = m;
        lo[dst] = l;
    }
}

// byte offset of (row r, bf16 element k) in one operand copy of the canonical K-major layout
__device__ __forceinline__ uint32_t kmaj_off16(int r, int k) {
    return uint32_t(r >> 3) * SBO + uint32_t(k >> 3) * LBO + uint32_t(r & 7) * 16u + uint32_t(k & 7) * 2u;
}

// ROWS x 8 16-byte vectors (8 bf16 each) of the three copies of one operand tile
template <int ROWS>
__device__ __forceinline__ void load_tile3(const uint16_t *__restrict__ s0, const uint16_t *__restrict__ s1,
                                           const uint16_t *__restrict__ s2, int64_t off, int rows_valid, int row0,
                                           int K8, int k0, char *d0, char *d1, char *d2, int tid) {
#pragma unroll
    for (int i = 0; i < (ROWS * 8) / BTHREADS; ++i) {
        const int e = tid + i * BTHREADS;
        // eight consecutive threads take eight consecutive rows of one core matrix
        const int row = ((e >> 6) << 3) | (e & 7), kc = (e >> 3) & 7;
        const int gr = row0 + row, gk = k0 + kc * 8;
        uint4 v0 = make_uint4(0, 0, 0, 0), v1 = v0, v2 = v0;
        if (gr < rows_valid && gk < K8) {
            const int64_t idx = off + int64_t(gr) * K8 + gk;
            v0 = __ldg(reinterpret_cast<const uint4 *>(s0 + idx));
            v1 = __ldg(reinterpret_cast<const uint4 *>(s1 + idx));
            v2 = __ldg(reinterpret_cast<const uint4 *>(s2 + idx));
        }
        const uint32_t so = kmaj_off16(row, kc * 8);
        tc::st_shared_v4(d0 + so, v0);
        tc::st_shared_v4(d1 + so, v1);
        tc::st_shared_v4(d2 + so, v2);
    }
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred q;\n setp.ne.b32 q, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, q;\n}\n" ::"r"(tmem),
        "l"(da), "l"(db), "r"(idesc), "r"(acc));
}

__global__ void __launch_bounds__(BTHREADS, 1) k_gemm_bf16x3(TcArgs g, int *err) {
    extern __shared__ __align__(1024) char smem_raw[];
    char *smem = reinterpret_cast<char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    __shared__ uint64_t mbar[BNSTAGE];
    __shared__ uint32_t tmem_base_sh;
    __shared__ int abort_flag;

    const GemmTile t = g.tiles[blockIdx.x];
    const GemmOut o = g.outs[t.out];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint16_t *Ah = static_cast<const uint16_t *>(g.Ahi), *Am = static_cast<const uint16_t *>(g.Amid),
                   *Al = static_cast<const uint16_t *>(g.Alo);
    const uint16_t *Bh = static_cast<const uint16_t *>(g.Bhi), *Bm = static_cast<const uint16_t *>(g.Bmid),
                   *Bl = static_cast<const uint16_t *>(g.Blo);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         tc::smem_u32(&tmem_base_sh)),
                     "r"(BTMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        for (int s = 0; s < BNSTAGE; ++s) tc::mbar_init(&mbar[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;");
        abort_flag = 0;
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_base_sh;

    int nchunk = 0;
    for (int p = o.p0; p < o.p1; ++p) nchunk += (((g.pairs[p].K + 7) & ~7) + BK - 1) / BK;

    int p = o.p0, k0 = 0;
    uint32_t commits[BNSTAGE] = {};
    for (int c = 0; c < nchunk; ++c) {
        const int s = c % BNSTAGE;
        if (c >= BNSTAGE) {
            if (!tc::mbar_wait(&mbar[s], (commits[s] - 1) & 1)) {
                if (tid == 0) atomicExch(err, 3);
                abort_flag = 1;
            }
        }
        __syncthreads();
        if (abort_flag) break;
        while (k0 >= ((g.pairs[p].K + 7) & ~7)) {
            ++p;
            k0 = 0;
        }
        const GemmPair pr = g.pairs[p];
        const int K8 = (pr.K + 7) & ~7;
        char *st = smem + s * BSTAGE_BYTES;
        char *ah = st, *am = st + COPY_BYTES, *al = st + 2 * COPY_BYTES;
        char *bh = st + 3 * COPY_BYTES, *bm = st + 4 * COPY_BYTES, *bl = st + 5 * COPY_BYTES;
        load_tile3<BM>(Ah, Am, Al, pr.a_off, o.M, t.m0, K8, k0, ah, am, al, tid);
        load_tile3<BN>(Bh, Bm, Bl, pr.b_off, o.N, t.n0, K8, k0, bh, bm, bl, tid);
        k0 += BK;
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint32_t idesc = idesc_bf16();
            const uint32_t a0 = tc::smem_u32(ah), a1 = tc::smem_u32(am), a2 = tc::smem_u32(al);
            const uint32_t b0 = tc::smem_u32(bh), b1 = tc::smem_u32(bm), b2 = tc::smem_u32(bl);
#pragma unroll
            for (int ks = 0; ks < BK / 16; ++ks) {
                const uint32_t koff = uint32_t(ks) * 2u * LBO;  // 16 bf16 = 2 core matrices along K
                const uint32_t acc0 = (c > 0 || ks > 0) ? 1u : 0u;
                // second-order terms first, then first order, then the leading product
                mma_bf16(tmem, tc::make_desc(a0 + koff), tc::make_desc(b2 + koff), idesc, acc0);
                mma_bf16(tmem, tc::make_desc(a1 + koff), tc::make_desc(b1 + koff), idesc, 1u);
                mma_bf16(tmem, tc::make_desc(a2 + koff), tc::make_desc(b0 + koff), idesc, 1u);
                mma_bf16(tmem, tc::make_desc(a0 + koff), tc::make_desc(b1 + koff), idesc, 1u);
                mma_bf16(tmem, tc::make_desc(a1 + koff), tc::make_desc(b0 + koff), idesc, 1u);
                mma_bf16(tmem, tc::make_desc(a0 + koff), tc::make_desc(b0 + koff), idesc, 1u);
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             tc::smem_u32(&mbar[s]))
                         : "memory");
        }
        commits[s] += 1;
    }
    for (int s = 0; s < BNSTAGE; ++s) {
        if (commits[s] == 0) continue;
        if (!tc::mbar_wait(&mbar[s], (commits[s] - 1) & 1)) {
            if (tid == 0) atomicExch(err, 4);
        }
    }
    asm volatile("tcgen05.fence::after_thread_sync;");
    __syncthreads();

    // epilogue: warp w reads TMEM lanes 32*(w%4).., columns 64*(w/4) .. +63
    const int quarter = warp & 3, half = warp >> 2;
    const int shift = tc::amax_shift(*g.amax_a) + tc::amax_shift(*g.amax_b);
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
            const bool plain = g.alpha == 1.0 && o.add_off < 0;
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                const int gn = t.n0 + col0 + j;
                if (gn < o.N) {
                    const int64_t idx = int64_t(gm) * o.N + gn;
                    double val = tc::f32_to_f64_int(__uint_as_float(v[j]), shift);
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
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BTMEM_COLS));
    }
}

}  // namespace

void launch_split_bf16x3(const double *src, void *hi, void *mid, void *lo, const SplitEntry *e, const Chunk *chunks,
                         int64_t nchunks, const unsigned long long *amax) {
    if (nchunks <= 0) return;
    k_split_bf16x3<<<unsigned(nchunks), 256, 0, ctx().stream>>>(src, static_cast<uint16_t *>(hi),
                                                                 static_cast<uint16_t *>(mid),
                                                                 static_cast<uint16_t *>(lo), e, chunks, amax);
    count_launch();
    cuda_check(cudaGetLastError(), "bf16 split kernel launch");
}

void launch_gemm_bf16x3(const TcArgs &a, int *err, cudaStream_t stream) {
    static std::once_flag attr;
    std::call_once(attr, [] {
        cuda_check(cudaFuncSetAttribute(k_gemm_bf16x3, cudaFuncAttributeMaxDynamicSharedMemorySize, BSMEM_BYTES),
                   "tcgen05 bf16 GEMM smem attribute");
    });
    k_gemm_bf16x3<<<a.ntiles, BTHREADS, BSMEM_BYTES, stream>>>(a, err);
    count_launch();
    cuda_check(cudaGetLastError(), "tcgen05 bf16 GEMM launch");
}

}  // namespace qtt
