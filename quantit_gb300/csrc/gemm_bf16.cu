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
// Layout and pipeline follow k_gemm_tf32x3: the split operands are tiled in core
// matrices of 8 rows x 8 bf16 (128 bytes; rows padded to 8, K to 16), one 128 x 128
// output tile per CTA, a producer warp fills a 2-stage ring (96 KB stages: K chunks
// of 64 bf16, hi / mid / lo of A and B) with one bulk asynchronous copy (1 KB) per
// operand copy and row group, one thread issues 6 products x 4 k-steps of 16 per stage and
// commits them to the stage's "empty" mbarrier.  Every wait is bounded; on timeout
// the kernel records an error code, drains what it issued and frees its TMEM.
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
constexpr uint32_t BSBO = (BK * 2 / 16) * 128;     // next 8-row group: 8 core matrices along K (1 KB)
constexpr int COPY_BYTES = 128 * BK * 2;           // one operand copy (hi, mid or lo): 16 KB
constexpr int BSTAGE_BYTES = 6 * COPY_BYTES;       // hi/mid/lo of A and B: 96 KB
constexpr int bsmem_bytes(int nstage) { return nstage * BSTAGE_BYTES + 1024; }
using tc::LBO;

// no-swizzle K-major descriptor with this kernel's 8-row-group stride
__device__ __forceinline__ uint64_t make_desc_b(uint32_t saddr) {
    uint64_t d = 0;
    d |= uint64_t((saddr & 0x3FFFF) >> 4);
    d |= uint64_t(LBO >> 4) << 16;
    d |= uint64_t(BSBO >> 4) << 32;
    d |= uint64_t(1) << 46;
    return d;
}

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
    const int shift = tc::amax_shift(*amax);
    for (int i = threadIdx.x; i < ch.len; i += blockDim.x) {
        const int64_t lin = ch.start + i;
        const float x = tc::f64_to_f32_int(src[split_src(e, lin)], shift);
        const uint16_t h = to_bf16(x);
        const float r1 = x - from_bf16(h);
        const uint16_t m = to_bf16(r1);
        const uint16_t l = to_bf16(r1 - from_bf16(m));
        int64_t row, k;
        split_rowk(e, lin, row, k);
        const int64_t dst = e.dst_off + ((row >> 3) * (e.K4 >> 3) + (k >> 3)) * 64 + (row & 7) * 8 + (k & 7);
        hi[dst] = h;
        mid[dst] = m;
        lo[dst] = l;
    }
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred q;\n setp.ne.b32 q, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, q;\n}\n" ::"r"(tmem),
        "l"(da), "l"(db), "r"(idesc), "r"(acc));
}

template <int BNSTAGE>
__global__ void __launch_bounds__(BTHREADS, 1) k_gemm_bf16x3(TcArgs g, int *err) {
    extern __shared__ __align__(1024) char smem_raw[];
    char *smem = reinterpret_cast<char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    __shared__ uint64_t full[BNSTAGE], empty[BNSTAGE], done;
    __shared__ uint32_t tmem_base_sh;
    __shared__ int abort_flag, n_issued, n_consumed;

    const GemmTile t = g.tiles[blockIdx.x];
    const GemmOut o = g.outs[t.out];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         tc::smem_u32(&tmem_base_sh)),
                     "r"(BTMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        for (int s = 0; s < BNSTAGE; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        tc::mbar_init(&done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;");
        abort_flag = 0;
        n_issued = 0;
        n_consumed = 0;
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_base_sh;

    int nchunk = 0;
    for (int p = o.p0; p < o.p1; ++p) nchunk += (((g.pairs[p].K + 15) & ~15) + BK - 1) / BK;

    if (warp == 0) {
        // producer: one bulk copy per (operand copy, row group) of each K chunk
        const uint16_t *srcs[6] = {static_cast<const uint16_t *>(g.Ahi), static_cast<const uint16_t *>(g.Amid),
                                   static_cast<const uint16_t *>(g.Alo), static_cast<const uint16_t *>(g.Bhi),
                                   static_cast<const uint16_t *>(g.Bmid), static_cast<const uint16_t *>(g.Blo)};
        const int rga = min(BM / 8, (o.M - t.m0 + 7) / 8), rgb = min(BN / 8, (o.N - t.n0 + 7) / 8);
        int p = o.p0, k0 = 0, c = 0;
        for (; c < nchunk; ++c) {
            const int s = c % BNSTAGE;
            int ok = 1;
            if (lane == 0 && c >= BNSTAGE) ok = tc::mbar_wait(&empty[s], ((c / BNSTAGE) - 1) & 1) ? 1 : 0;
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok) {
                if (lane == 0) {
                    atomicExch(err, 3);
                    atomicExch(&abort_flag, 1);
                }
                break;
            }
            while (k0 >= ((g.pairs[p].K + 15) & ~15)) {
                ++p;
                k0 = 0;
            }
            const GemmPair pr = g.pairs[p];
            const int KP = (pr.K + 15) & ~15, kv = min(BK, KP - k0);
            const uint32_t rg_bytes = uint32_t(kv) * 16u;  // kv / 8 core matrices of 128 bytes
            if (lane == 0) tc::mbar_expect_tx(&full[s], 3u * rg_bytes * uint32_t(rga + rgb));
            __syncwarp();
            char *st = smem + s * BSTAGE_BYTES;
            const int nA = 3 * rga, ncopy = 3 * (rga + rgb);
            for (int i = lane; i < ncopy; i += 32) {
                const bool isA = i < nA;
                const int j = isA ? i : i - nA, which = j % 3, rg = j / 3;
                const int64_t grg = (isA ? t.m0 : t.n0) / 8 + rg;
                const uint16_t *src = srcs[(isA ? 0 : 3) + which] + (isA ? pr.a_off : pr.b_off) +
                                      (grg * (KP / 8) + k0 / 8) * 64;
                char *dst = st + ((isA ? 0 : 3) + which) * COPY_BYTES + rg * int(BSBO);
                tc::bulk_g2s(dst, src, rg_bytes, &full[s]);
            }
            k0 += BK;
        }
        if (lane == 0) n_issued = c;
    } else if (warp == 1 && lane == 0) {
        // MMA issuer
        const uint32_t idesc = idesc_bf16();
        int p = o.p0, k0 = 0, c = 0;
        for (; c < nchunk; ++c) {
            const int s = c % BNSTAGE;
            if (!tc::mbar_wait(&full[s], (c / BNSTAGE) & 1)) {
                atomicExch(err, 4);
                atomicExch(&abort_flag, 1);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
            while (k0 >= ((g.pairs[p].K + 15) & ~15)) {
                ++p;
                k0 = 0;
            }
            const int kv = min(BK, ((g.pairs[p].K + 15) & ~15) - k0);
            const uint32_t base = tc::smem_u32(smem + s * BSTAGE_BYTES);
            const uint32_t a0 = base, a1 = base + COPY_BYTES, a2 = base + 2 * COPY_BYTES;
            const uint32_t b0 = base + 3 * COPY_BYTES, b1 = base + 4 * COPY_BYTES, b2 = base + 5 * COPY_BYTES;
            for (int ks = 0; ks < kv / 16; ++ks) {
                const uint32_t koff = uint32_t(ks) * 2u * LBO;  // 16 bf16 = 2 core matrices along K
                const uint32_t acc0 = (c > 0 || ks > 0) ? 1u : 0u;
                // second-order terms first, then first order, then the leading product
                mma_bf16(tmem, make_desc_b(a0 + koff), make_desc_b(b2 + koff), idesc, acc0);
                mma_bf16(tmem, make_desc_b(a1 + koff), make_desc_b(b1 + koff), idesc, 1u);
                mma_bf16(tmem, make_desc_b(a2 + koff), make_desc_b(b0 + koff), idesc, 1u);
                mma_bf16(tmem, make_desc_b(a0 + koff), make_desc_b(b1 + koff), idesc, 1u);
                mma_bf16(tmem, make_desc_b(a1 + koff), make_desc_b(b0 + koff), idesc, 1u);
                mma_bf16(tmem, make_desc_b(a0 + koff), make_desc_b(b0 + koff), idesc, 1u);
            }
            tc::umma_commit(&empty[s]);
            k0 += BK;
        }
        n_consumed = c;
        tc::umma_commit(&done);
    }
    if (lane == 0 && !tc::mbar_wait(&done, 0)) atomicExch(err, 4);
    __syncwarp();
    __syncthreads();
    if (tid == 0) {
        for (int c = n_consumed; c < n_issued; ++c)
            if (!tc::mbar_wait(&full[c % BNSTAGE], (c / BNSTAGE) & 1)) atomicExch(err, 4);
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

// Persistent variant for launches of many tiles (the structure of
// k_gemm_tf32x3_persistent): one CTA per SM walks the tile list, the producer streams
// the K chunks of consecutive tiles through the ring, the MMA thread alternates two
// TMEM accumulators, and warps 4-7 run one tile's epilogue during the next tile's MMAs.
template <int BNSTAGE>
__global__ void __launch_bounds__(BTHREADS, 1) k_gemm_bf16x3_persistent(TcArgs g, int *err) {
    extern __shared__ __align__(1024) char smem_raw[];
    char *smem = reinterpret_cast<char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    __shared__ uint64_t full[BNSTAGE], empty[BNSTAGE], acc_full[2], acc_empty[2];
    __shared__ uint32_t tmem_base_sh;
    __shared__ int n_issued, n_consumed;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // round r of the longest-first tile list, in boustrophedon order across the CTAs, so
    // that every CTA's tiles add up to about the same work
    auto snake_tile = [&](int r) {
        const int G = int(gridDim.x), b = int(blockIdx.x);
        return r * G + ((r & 1) ? (G - 1 - b) : b);
    };

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         tc::smem_u32(&tmem_base_sh)),
                     "r"(2 * BTMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        for (int s = 0; s < BNSTAGE; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&acc_full[b], 1);
            tc::mbar_init(&acc_empty[b], 4);
        }
        asm volatile("fence.mbarrier_init.release.cluster;");
        n_issued = 0;
        n_consumed = 0;
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_base_sh;
    auto tile_chunks = [&](const GemmOut &o) {
        int n = 0;
        for (int p = o.p0; p < o.p1; ++p) n += (((g.pairs[p].K + 15) & ~15) + BK - 1) / BK;
        return n;
    };

    if (warp == 0) {
        const uint16_t *srcs[6] = {static_cast<const uint16_t *>(g.Ahi), static_cast<const uint16_t *>(g.Amid),
                                   static_cast<const uint16_t *>(g.Alo), static_cast<const uint16_t *>(g.Bhi),
                                   static_cast<const uint16_t *>(g.Bmid), static_cast<const uint16_t *>(g.Blo)};
        int gc = 0;
        bool stop = false;
        for (int r = 0; r * int(gridDim.x) < g.ntiles && !stop; ++r) {
            const int tile = snake_tile(r);
            if (tile >= g.ntiles) continue;
            const GemmTile t = g.tiles[tile];
            const GemmOut o = g.outs[t.out];
            const int rga = min(BM / 8, (o.M - t.m0 + 7) / 8), rgb = min(BN / 8, (o.N - t.n0 + 7) / 8);
            const int nch = tile_chunks(o);
            int p = o.p0, k0 = 0;
            for (int c = 0; c < nch; ++c) {
                const int s = gc % BNSTAGE;
                int ok = 1;
                if (lane == 0 && gc >= BNSTAGE) ok = tc::mbar_wait(&empty[s], ((gc / BNSTAGE) - 1) & 1) ? 1 : 0;
                ok = __shfl_sync(0xffffffffu, ok, 0);
                if (!ok) {
                    if (lane == 0) atomicExch(err, 3);
                    stop = true;
                    break;
                }
                while (k0 >= ((g.pairs[p].K + 15) & ~15)) {
                    ++p;
                    k0 = 0;
                }
                const GemmPair pr = g.pairs[p];
                const int KP = (pr.K + 15) & ~15, kv = min(BK, KP - k0);
                const uint32_t rg_bytes = uint32_t(kv) * 16u;
                if (lane == 0) tc::mbar_expect_tx(&full[s], 3u * rg_bytes * uint32_t(rga + rgb));
                __syncwarp();
                char *st = smem + s * BSTAGE_BYTES;
                const int nA = 3 * rga, ncopy = 3 * (rga + rgb);
                for (int i = lane; i < ncopy; i += 32) {
                    const bool isA = i < nA;
                    const int j = isA ? i : i - nA, which = j % 3, rg = j / 3;
                    const int64_t grg = (isA ? t.m0 : t.n0) / 8 + rg;
                    const uint16_t *src = srcs[(isA ? 0 : 3) + which] + (isA ? pr.a_off : pr.b_off) +
                                          (grg * (KP / 8) + k0 / 8) * 64;
                    char *dst = st + ((isA ? 0 : 3) + which) * COPY_BYTES + rg * int(BSBO);
                    tc::bulk_g2s(dst, src, rg_bytes, &full[s]);
                }
                k0 += BK;
                ++gc;
            }
        }
        if (lane == 0) n_issued = gc;
    } else if (warp == 1 && lane == 0) {
        const uint32_t idesc = idesc_bf16();
        int gc = 0, i = 0;
        bool stop = false;
        for (int r = 0; r * int(gridDim.x) < g.ntiles && !stop; ++r) {
            const int tile = snake_tile(r);
            if (tile >= g.ntiles) continue;
            const GemmOut o = g.outs[g.tiles[tile].out];
            const int b = i & 1;
            if (i >= 2 && !tc::mbar_wait(&acc_empty[b], ((i / 2) - 1) & 1)) {
                atomicExch(err, 4);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint32_t acc_t = tmem + uint32_t(b * BTMEM_COLS);
            const int nch = tile_chunks(o);
            int p = o.p0, k0 = 0;
            for (int c = 0; c < nch; ++c) {
                const int s = gc % BNSTAGE;
                if (!tc::mbar_wait(&full[s], (gc / BNSTAGE) & 1)) {
                    atomicExch(err, 4);
                    stop = true;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;");
                while (k0 >= ((g.pairs[p].K + 15) & ~15)) {
                    ++p;
                    k0 = 0;
                }
                const int kv = min(BK, ((g.pairs[p].K + 15) & ~15) - k0);
                const uint32_t base = tc::smem_u32(smem + s * BSTAGE_BYTES);
                const uint32_t a0 = base, a1 = base + COPY_BYTES, a2 = base + 2 * COPY_BYTES;
                const uint32_t b0 = base + 3 * COPY_BYTES, b1 = base + 4 * COPY_BYTES, b2 = base + 5 * COPY_BYTES;
                for (int ks = 0; ks < kv / 16; ++ks) {
                    const uint32_t koff = uint32_t(ks) * 2u * LBO;
                    const uint32_t acc0 = (c > 0 || ks > 0) ? 1u : 0u;
                    mma_bf16(acc_t, make_desc_b(a0 + koff), make_desc_b(b2 + koff), idesc, acc0);
                    mma_bf16(acc_t, make_desc_b(a1 + koff), make_desc_b(b1 + koff), idesc, 1u);
                    mma_bf16(acc_t, make_desc_b(a2 + koff), make_desc_b(b0 + koff), idesc, 1u);
                    mma_bf16(acc_t, make_desc_b(a0 + koff), make_desc_b(b1 + koff), idesc, 1u);
                    mma_bf16(acc_t, make_desc_b(a1 + koff), make_desc_b(b0 + koff), idesc, 1u);
                    mma_bf16(acc_t, make_desc_b(a0 + koff), make_desc_b(b0 + koff), idesc, 1u);
                }
                tc::umma_commit(&empty[s]);
                k0 += BK;
                ++gc;
            }
            tc::umma_commit(&acc_full[b]);
            ++i;
        }
        n_consumed = gc;
    } else if (warp >= 4) {
        const int quarter = warp - 4;
        const int shift = tc::amax_shift(*g.amax_a) + tc::amax_shift(*g.amax_b);
        const int row = quarter * 32 + lane;
        int i = 0;
        for (int r = 0; r * int(gridDim.x) < g.ntiles; ++r) {
            const int tile = snake_tile(r);
            if (tile >= g.ntiles) continue;
            const GemmTile t = g.tiles[tile];
            const GemmOut o = g.outs[t.out];
            const int b = i & 1;
            int ok = 1;
            if (lane == 0) ok = tc::mbar_wait(&acc_full[b], (i / 2) & 1) ? 1 : 0;
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok) {
                if (lane == 0) atomicExch(err, 4);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
            const bool have_acc = tile_chunks(o) > 0;
            const int gm = t.m0 + row;
            const bool plain = g.alpha == 1.0 && o.add_off < 0;
#pragma unroll 1
            for (int cb = 0; cb < 4; ++cb) {
                const int col0 = cb * 32;
                uint32_t v[32];
                const uint32_t taddr = tmem + (uint32_t(quarter * 32) << 16) + uint32_t(b * BTMEM_COLS + col0);
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
                if (gm < o.M) {
#pragma unroll
                    for (int j = 0; j < 32; ++j) {
                        const int gn = t.n0 + col0 + j;
                        if (gn < o.N) {
                            const int64_t idx = int64_t(gm) * o.N + gn;
                            double val = have_acc ? tc::f32_to_f64_int(__uint_as_float(v[j]), shift) : 0.0;
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
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&acc_empty[b]);
            ++i;
        }
    }
    __syncthreads();
    if (tid == 0) {
        for (int c = n_consumed; c < n_issued; ++c)
            if (!tc::mbar_wait(&full[c % BNSTAGE], (c / BNSTAGE) & 1)) atomicExch(err, 4);
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * BTMEM_COLS));
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

template <int NST>
void launch_bf16x3(const TcArgs &a, int *err, cudaStream_t stream) {
    static std::atomic<uint64_t> attr{0};
    once_per_device(attr, [] {
        cuda_check(cudaFuncSetAttribute(k_gemm_bf16x3<NST>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        bsmem_bytes(NST)),
                   "tcgen05 bf16 GEMM smem attribute");
    });
    k_gemm_bf16x3<NST><<<a.ntiles, BTHREADS, bsmem_bytes(NST), stream>>>(a, err);
}

int bf_sm_count() { return device_sm_count(); }

void launch_gemm_bf16x3(const TcArgs &a, int *err, cudaStream_t stream) {
    if (a.ntiles >= 2 * bf_sm_count() && persistent_gemm()) {
        static std::atomic<uint64_t> attr{0};
        once_per_device(attr, [] {
            cuda_check(cudaFuncSetAttribute(k_gemm_bf16x3_persistent<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            bsmem_bytes(2)),
                       "tcgen05 persistent bf16 GEMM smem attribute");
        });
        k_gemm_bf16x3_persistent<2><<<std::min(a.ntiles, bf_sm_count()), BTHREADS, bsmem_bytes(2), stream>>>(a, err);
    }
    // tiles of one K chunk: one stage (2 CTAs per SM); otherwise a 2-stage ring
    else if (a.max_chunks == 1)
        launch_bf16x3<1>(a, err, stream);
    else
        launch_bf16x3<2>(a, err, stream);
    count_launch();
    cuda_check(cudaGetLastError(), "tcgen05 bf16 GEMM launch");
}

}  // namespace qtt
