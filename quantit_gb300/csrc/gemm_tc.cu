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
//    patterns in the tensor cores' core-matrix tiling: rows padded to 8 and K to 8,
//    each 8-row x 4-element core matrix (128 bytes) contiguous, the core matrices of
//    a row group in K order.  A row group's slice of a K chunk is then one contiguous
//    block of memory.  The FP64 -> FP32 conversion uses integer operations only:
//    GB300's FP64 pipe is a small fraction of its FP32 / integer rate.
//  * k_gemm_tf32x3: CTA = one 128 x 128 tile of one output block (same tile and
//    pair tables as the FP64 kernel), warp-specialised:
//      - warp 0 (producer) fills a 3-stage shared-memory ring with bulk asynchronous
//        copies (cp.async.bulk, one per row group and operand copy), counted in bytes
//        on the stage's "full" mbarrier; the shared layout is the canonical
//        no-swizzle K-major UMMA layout (LBO 128 B, SBO 1024 B);
//      - one thread of warp 1 waits on "full", issues the stage's tcgen05.mma
//        (3 products x up to 4 k-steps of 8) and commits them to the stage's "empty"
//        mbarrier, which the producer waits on before refilling the stage;
//      - after the last stage it commits to "done", and all warps run the epilogue:
//        tcgen05.ld of the accumulator, alpha*acc + beta*add in FP64 (a plain integer
//        widening when alpha = 1 and there is no add term).
//
// Every mbarrier wait is bounded; on timeout the kernel records an error code in
// a device word that the host checks, drains (bounded) the copies and MMAs it
// issued and frees its TMEM before returning.
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
// up to 3 stages; a launch whose tiles need fewer K chunks uses a smaller ring, so that
// 2 or 3 CTAs share an SM and hide each other's fixed per-tile latency
constexpr int smem_bytes(int nstage) { return nstage * STAGE_BYTES + 1024; }
using tc::LBO;
using tc::SBO;
using tc::smem_u32;
using tc::make_desc;
using tc::mbar_init;
using tc::mbar_wait;
using tc::amax_shift;
using tc::f64_to_f32_int;
using tc::f32_to_f64_int;
using tc::mbar_expect_tx;
using tc::bulk_g2s;
using tc::umma_commit;
using tc::mbar_arrive;
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
    const int shift = amax_shift(*amax);
    for (int i = threadIdx.x; i < ch.len; i += blockDim.x) {
        const int64_t lin = ch.start + i;
        const float xf = f64_to_f32_int(src[split_src(e, lin)], shift);
        const uint32_t h = to_tf32(xf);
        const uint32_t l = to_tf32(xf - __uint_as_float(h));
        int64_t row, k;
        split_rowk(e, lin, row, k);
        const int64_t dst = e.dst_off + ((row >> 3) * (e.K4 >> 2) + (k >> 2)) * 32 + (row & 7) * 4 + (k & 3);
        hi[dst] = __uint_as_float(h);
        lo[dst] = __uint_as_float(l);
    }
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred q;\n setp.ne.b32 q, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, q;\n}\n" ::"r"(tmem),
        "l"(da), "l"(db), "r"(idesc), "r"(acc));
}

template <int NSTAGE>
__global__ void __launch_bounds__(TTHREADS, 1) k_gemm_tf32x3(TcArgs g, int *err) {
    extern __shared__ __align__(1024) char smem_raw[];
    char *smem = reinterpret_cast<char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    __shared__ uint64_t full[NSTAGE], empty[NSTAGE], done;
    __shared__ uint32_t tmem_base_sh;
    __shared__ int abort_flag, n_issued, n_consumed;

    const GemmTile t = g.tiles[blockIdx.x];
    const GemmOut o = g.outs[t.out];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_sh)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        for (int s = 0; s < NSTAGE; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(&done, 1);
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
    for (int p = o.p0; p < o.p1; ++p) nchunk += (((g.pairs[p].K + 7) & ~7) + TBK - 1) / TBK;

    if (warp == 0) {
        // producer: one bulk copy per (operand copy, row group) of each K chunk
        const float *srcs[4] = {static_cast<const float *>(g.Ahi), static_cast<const float *>(g.Alo),
                                static_cast<const float *>(g.Bhi), static_cast<const float *>(g.Blo)};
        const int rga = min(TBM / 8, (o.M - t.m0 + 7) / 8), rgb = min(TBN / 8, (o.N - t.n0 + 7) / 8);
        int p = o.p0, k0 = 0, c = 0;
        for (; c < nchunk; ++c) {
            const int s = c % NSTAGE;
            int ok = 1;
            if (lane == 0 && c >= NSTAGE) ok = mbar_wait(&empty[s], ((c / NSTAGE) - 1) & 1) ? 1 : 0;
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok) {
                if (lane == 0) {
                    atomicExch(err, 1);
                    atomicExch(&abort_flag, 1);
                }
                break;
            }
            while (k0 >= ((g.pairs[p].K + 7) & ~7)) {
                ++p;
                k0 = 0;
            }
            const GemmPair pr = g.pairs[p];
            const int KP = (pr.K + 7) & ~7, kv = min(TBK, KP - k0);
            const uint32_t rg_bytes = uint32_t(kv) * 32u;  // kv / 4 core matrices of 128 bytes
            if (lane == 0) mbar_expect_tx(&full[s], 2u * rg_bytes * uint32_t(rga + rgb));
            __syncwarp();
            char *st = smem + s * STAGE_BYTES;
            const int nA = 2 * rga, ncopy = 2 * (rga + rgb);
            for (int i = lane; i < ncopy; i += 32) {
                const bool isA = i < nA;
                const int j = isA ? i : i - nA, which = j & 1, rg = j >> 1;
                const int64_t grg = (isA ? t.m0 : t.n0) / 8 + rg;
                const float *src = srcs[(isA ? 0 : 2) + which] + (isA ? pr.a_off : pr.b_off) +
                                   (grg * (KP / 4) + k0 / 4) * 32;
                char *dst = st + (isA ? 0 : 2 * A_BYTES) + which * (isA ? A_BYTES : B_BYTES) + rg * int(SBO);
                bulk_g2s(dst, src, rg_bytes, &full[s]);
            }
            k0 += TBK;
        }
        if (lane == 0) n_issued = c;
    } else if (warp == 1 && lane == 0) {
        // MMA issuer
        const uint32_t idesc = idesc_tf32();
        int p = o.p0, k0 = 0, c = 0;
        for (; c < nchunk; ++c) {
            const int s = c % NSTAGE;
            if (!mbar_wait(&full[s], (c / NSTAGE) & 1)) {
                atomicExch(err, 2);
                atomicExch(&abort_flag, 1);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
            while (k0 >= ((g.pairs[p].K + 7) & ~7)) {
                ++p;
                k0 = 0;
            }
            const int kv = min(TBK, ((g.pairs[p].K + 7) & ~7) - k0);
            char *st = smem + s * STAGE_BYTES;
            const uint32_t a_hi = smem_u32(st), a_lo = a_hi + A_BYTES, b_hi = a_hi + 2 * A_BYTES, b_lo = b_hi + B_BYTES;
            for (int ks = 0; ks < kv / 8; ++ks) {
                const uint32_t koff = uint32_t(ks) * 2u * LBO;  // 8 tf32 = 2 core matrices along K
                const uint32_t acc0 = (c > 0 || ks > 0) ? 1u : 0u;
                // small terms first, then the leading product
                mma_tf32(tmem, make_desc(a_hi + koff), make_desc(b_lo + koff), idesc, acc0);
                mma_tf32(tmem, make_desc(a_lo + koff), make_desc(b_hi + koff), idesc, 1u);
                mma_tf32(tmem, make_desc(a_hi + koff), make_desc(b_hi + koff), idesc, 1u);
            }
            umma_commit(&empty[s]);
            k0 += TBK;
        }
        n_consumed = c;
        umma_commit(&done);
    }
    // everyone: the accumulator is final once "done" fires
    if (lane == 0 && !mbar_wait(&done, 0)) atomicExch(err, 2);
    __syncwarp();
    __syncthreads();
    if (tid == 0) {
        // copies issued but never consumed (only after a timeout) must land before exit
        for (int c = n_consumed; c < n_issued; ++c)
            if (!mbar_wait(&full[c % NSTAGE], (c / NSTAGE) & 1)) atomicExch(err, 2);
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

// Persistent variant for launches of many tiles: one CTA per SM walks the sorted tile
// list (tiles blockIdx.x, + gridDim.x, ...).  The producer warp streams the K chunks of
// its tiles through the ring without draining it between tiles; the MMA thread
// accumulates tile i in TMEM buffer i % 2 (2 x 128 columns) and commits it to
// acc_full[i % 2]; warps 4-7 (one TMEM lane quarter each) run tile i's epilogue from
// that buffer and release it on acc_empty[i % 2] while the MMAs of tile i + 1 proceed.
template <int NSTAGE>
__global__ void __launch_bounds__(TTHREADS, 1) k_gemm_tf32x3_persistent(TcArgs g, int *err) {
    extern __shared__ __align__(1024) char smem_raw[];
    char *smem = reinterpret_cast<char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    __shared__ uint64_t full[NSTAGE], empty[NSTAGE], acc_full[2], acc_empty[2];
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
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_sh)),
                     "r"(2 * TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        for (int s = 0; s < NSTAGE; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], 4);  // one arrival per epilogue warp
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
        for (int p = o.p0; p < o.p1; ++p) n += (((g.pairs[p].K + 7) & ~7) + TBK - 1) / TBK;
        return n;
    };

    if (warp == 0) {
        const float *srcs[4] = {static_cast<const float *>(g.Ahi), static_cast<const float *>(g.Alo),
                                static_cast<const float *>(g.Bhi), static_cast<const float *>(g.Blo)};
        int gc = 0;
        bool stop = false;
        for (int r = 0; r * int(gridDim.x) < g.ntiles && !stop; ++r) {
            const int tile = snake_tile(r);
            if (tile >= g.ntiles) continue;
            const GemmTile t = g.tiles[tile];
            const GemmOut o = g.outs[t.out];
            const int rga = min(TBM / 8, (o.M - t.m0 + 7) / 8), rgb = min(TBN / 8, (o.N - t.n0 + 7) / 8);
            const int nch = tile_chunks(o);
            int p = o.p0, k0 = 0;
            for (int c = 0; c < nch; ++c) {
                const int s = gc % NSTAGE;
                int ok = 1;
                if (lane == 0 && gc >= NSTAGE) ok = mbar_wait(&empty[s], ((gc / NSTAGE) - 1) & 1) ? 1 : 0;
                ok = __shfl_sync(0xffffffffu, ok, 0);
                if (!ok) {
                    if (lane == 0) atomicExch(err, 1);
                    stop = true;
                    break;
                }
                while (k0 >= ((g.pairs[p].K + 7) & ~7)) {
                    ++p;
                    k0 = 0;
                }
                const GemmPair pr = g.pairs[p];
                const int KP = (pr.K + 7) & ~7, kv = min(TBK, KP - k0);
                const uint32_t rg_bytes = uint32_t(kv) * 32u;
                if (lane == 0) mbar_expect_tx(&full[s], 2u * rg_bytes * uint32_t(rga + rgb));
                __syncwarp();
                char *st = smem + s * STAGE_BYTES;
                const int nA = 2 * rga, ncopy = 2 * (rga + rgb);
                for (int i = lane; i < ncopy; i += 32) {
                    const bool isA = i < nA;
                    const int j = isA ? i : i - nA, which = j & 1, rg = j >> 1;
                    const int64_t grg = (isA ? t.m0 : t.n0) / 8 + rg;
                    const float *src = srcs[(isA ? 0 : 2) + which] + (isA ? pr.a_off : pr.b_off) +
                                       (grg * (KP / 4) + k0 / 4) * 32;
                    char *dst = st + (isA ? 0 : 2 * A_BYTES) + which * (isA ? A_BYTES : B_BYTES) + rg * int(SBO);
                    bulk_g2s(dst, src, rg_bytes, &full[s]);
                }
                k0 += TBK;
                ++gc;
            }
        }
        if (lane == 0) n_issued = gc;
    } else if (warp == 1 && lane == 0) {
        const uint32_t idesc = idesc_tf32();
        int gc = 0, i = 0;
        bool stop = false;
        for (int r = 0; r * int(gridDim.x) < g.ntiles && !stop; ++r) {
            const int tile = snake_tile(r);
            if (tile >= g.ntiles) continue;
            const GemmOut o = g.outs[g.tiles[tile].out];
            const int b = i & 1;
            if (i >= 2 && !mbar_wait(&acc_empty[b], ((i / 2) - 1) & 1)) {
                atomicExch(err, 2);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint32_t acc_t = tmem + uint32_t(b * TMEM_COLS);
            const int nch = tile_chunks(o);
            int p = o.p0, k0 = 0;
            for (int c = 0; c < nch; ++c) {
                const int s = gc % NSTAGE;
                if (!mbar_wait(&full[s], (gc / NSTAGE) & 1)) {
                    atomicExch(err, 2);
                    stop = true;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;");
                while (k0 >= ((g.pairs[p].K + 7) & ~7)) {
                    ++p;
                    k0 = 0;
                }
                const int kv = min(TBK, ((g.pairs[p].K + 7) & ~7) - k0);
                char *st = smem + s * STAGE_BYTES;
                const uint32_t a_hi = smem_u32(st), a_lo = a_hi + A_BYTES, b_hi = a_hi + 2 * A_BYTES,
                               b_lo = b_hi + B_BYTES;
                for (int ks = 0; ks < kv / 8; ++ks) {
                    const uint32_t koff = uint32_t(ks) * 2u * LBO;
                    const uint32_t acc0 = (c > 0 || ks > 0) ? 1u : 0u;
                    mma_tf32(acc_t, make_desc(a_hi + koff), make_desc(b_lo + koff), idesc, acc0);
                    mma_tf32(acc_t, make_desc(a_lo + koff), make_desc(b_hi + koff), idesc, 1u);
                    mma_tf32(acc_t, make_desc(a_hi + koff), make_desc(b_hi + koff), idesc, 1u);
                }
                umma_commit(&empty[s]);
                k0 += TBK;
                ++gc;
            }
            umma_commit(&acc_full[b]);  // this tile's accumulator is final once its MMAs complete
            ++i;
        }
        n_consumed = gc;
    } else if (warp >= 4) {
        // epilogue: warp 4 + q reads TMEM lanes 32 q .. 32 q + 31 (rows), all 128 columns
        const int quarter = warp - 4;
        const int shift = amax_shift(*g.amax_a) + amax_shift(*g.amax_b);
        const int row = quarter * 32 + lane;
        int i = 0;
        for (int r = 0; r * int(gridDim.x) < g.ntiles; ++r) {
            const int tile = snake_tile(r);
            if (tile >= g.ntiles) continue;
            const GemmTile t = g.tiles[tile];
            const GemmOut o = g.outs[t.out];
            const int b = i & 1;
            int ok = 1;
            if (lane == 0) ok = mbar_wait(&acc_full[b], (i / 2) & 1) ? 1 : 0;
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok) {
                if (lane == 0) atomicExch(err, 2);
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
                const uint32_t taddr = tmem + (uint32_t(quarter * 32) << 16) + uint32_t(b * TMEM_COLS + col0);
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
                            double val = have_acc ? f32_to_f64_int(__uint_as_float(v[j]), shift) : 0.0;
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
            if (lane == 0) mbar_arrive(&acc_empty[b]);
            ++i;
        }
    }
    __syncthreads();
    if (tid == 0) {
        // copies issued but never consumed (only after a timeout) must land before exit
        for (int c = n_consumed; c < n_issued; ++c)
            if (!mbar_wait(&full[c % NSTAGE], (c / NSTAGE) & 1)) atomicExch(err, 2);
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * TMEM_COLS));
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

int tc_sm_count() { return device_sm_count(); }

void launch_tf32x3_persistent(const TcArgs &a) {
    static std::atomic<uint64_t> attr{0};
    once_per_device(attr, [] {
        cuda_check(cudaFuncSetAttribute(k_gemm_tf32x3_persistent<3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        smem_bytes(3)),
                   "tcgen05 persistent GEMM smem attribute");
    });
    const int grid = std::min(a.ntiles, tc_sm_count());
    k_gemm_tf32x3_persistent<3><<<grid, TTHREADS, smem_bytes(3), ctx().stream>>>(a, err_word());
}

template <int NST>
void launch_tf32x3(const TcArgs &a) {
    static std::atomic<uint64_t> attr{0};
    once_per_device(attr, [] {
        cuda_check(cudaFuncSetAttribute(k_gemm_tf32x3<NST>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes(NST)),
                   "tcgen05 GEMM smem attribute");
    });
    k_gemm_tf32x3<NST><<<a.ntiles, TTHREADS, smem_bytes(NST), ctx().stream>>>(a, err_word());
}

void launch_gemm_tc(const TcArgs &a, int mode) {
    if (mode != GEMM_TF32X3 && mode != GEMM_BF16X3) fail(ERR_INVALID_ARGUMENT, "unknown tensor-core GEMM mode");
    if (a.ntiles <= 0) return;
    if (mode == GEMM_BF16X3) {
        launch_gemm_bf16x3(a, err_word(), ctx().stream);
        ctx().tc_used = true;
        return;
    }
    const int mc = a.max_chunks;
    if (a.ntiles >= 2 * tc_sm_count() && persistent_gemm())
        launch_tf32x3_persistent(a);
    else if (mc == 1)
        launch_tf32x3<1>(a);
    else if (mc == 2)
        launch_tf32x3<2>(a);
    else
        launch_tf32x3<3>(a);
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
