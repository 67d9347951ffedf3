// Device helpers shared by the tcgen05 grouped-GEMM kernels (split-TF32 and
// split-BF16): shared-memory addresses and UMMA descriptors of the canonical
// no-swizzle K-major layout (rows of 128 bytes per K chunk: core matrices of
// 8 rows x 16 bytes, LBO = 128 B to the next core matrix along K, SBO = 1024 B to
// the next 8-row group), bounded mbarrier waits, mbarrier arrivals and transaction
// counts, bulk asynchronous global -> shared copies, MMA commits, the operands'
// power-of-two scaling and the integer FP64 <-> FP32 conversions.
#pragma once
#include <cstdint>

namespace qtt {
namespace tc {

constexpr uint32_t LBO = 128;    // K-adjacent core matrices
constexpr uint32_t SBO = 1024;   // next 8-row group (8 core matrices of 16 B x 8 rows along K)
constexpr long long WAIT_LIMIT = 1ll << 22;

static __device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

static __device__ __forceinline__ uint64_t make_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= uint64_t((saddr & 0x3FFFF) >> 4);
    d |= uint64_t(LBO >> 4) << 16;
    d |= uint64_t(SBO >> 4) << 32;
    d |= uint64_t(1) << 46;  // descriptor version for tcgen05
    return d;                // base offset 0, no swizzle (layout type 0)
}

static __device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

static __device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
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

// Arrive on an mbarrier and add `bytes` to its expected transaction count.
static __device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// Asynchronous bulk copy global -> this CTA's shared memory (16-byte aligned addresses,
// size a multiple of 16); completion is counted in bytes on `bar`.
static __device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// Plain arrival on an mbarrier.
static __device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Commit the calling thread's prior tcgen05.mma operations to an mbarrier (one arrival
// when they have completed).
static __device__ __forceinline__ void umma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// Exponent of an operand's max |x| (the scale 2^-shift brings it to [1, 2));
// zero, infinite or NaN maxima leave the operand unscaled.
static __device__ __forceinline__ int amax_shift(unsigned long long bits) {
    const int e = int((bits >> 52) & 0x7FF);
    if (e == 0x7FF || bits == 0) return 0;
    return (e == 0 ? 1 : e) - 1023;
}

// FP64 * 2^-shift -> FP32 (round to nearest, ties away) with integer operations only.
// Magnitudes below the FP32 normal range flush to zero.
static __device__ __forceinline__ float f64_to_f32_int(double x, int shift) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
    const uint32_t sign = uint32_t(b >> 63) << 31;
    const int e = int((b >> 52) & 0x7FF);
    const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
    uint32_t f;
    if (e == 0) {
        f = 0;
    } else if (e == 0x7FF) {
        f = 0x7F800000u | (m ? 0x400000u : 0u);
    } else {
        const int fe = e - 1023 + 127 - shift;
        if (fe <= 0) {
            f = 0;
        } else if (fe >= 255) {
            f = 0x7F800000u;
        } else {
            const unsigned long long em = ((unsigned long long)fe << 52 | m) + (1ull << 28);
            f = uint32_t(em >> 29);
            if (f >= 0x7F800000u) f = 0x7F800000u;
        }
    }
    return __uint_as_float(sign | f);
}

// FP32 * 2^shift -> FP64 (exact unless the result leaves the FP64 normal range,
// where it flushes to zero or saturates to infinity) with integer operations only;
// FP32 subnormals flush to zero.
static __device__ __forceinline__ double f32_to_f64_int(float f, int shift) {
    const uint32_t b = __float_as_uint(f);
    const unsigned long long sign = (unsigned long long)(b >> 31) << 63;
    const uint32_t e = (b >> 23) & 0xFF, m = b & 0x7FFFFF;
    unsigned long long d;
    if (e == 0) {
        d = sign;
    } else if (e == 0xFF) {
        d = sign | 0x7FF0000000000000ull | ((unsigned long long)m << 29);
    } else {
        const int de = int(e) - 127 + 1023 + shift;
        if (de <= 0)
            d = sign;
        else if (de >= 0x7FF)
            d = sign | 0x7FF0000000000000ull;
        else
            d = sign | ((unsigned long long)de << 52) | ((unsigned long long)m << 29);
    }
    return __longlong_as_double(static_cast<long long>(d));
}

}  // namespace tc
}  // namespace qtt
