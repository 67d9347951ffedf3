// Memory-bound kernels of the block-sparse path: block permutation, segmented
// axpby / dot / broadcast products, sector packing and scattering, and the
// scalar steps of the one-step Lanczos update.  Every launch covers all blocks
// of an operation at once; work is cut into chunks that never cross a block.
#include <cuda_runtime.h>

#include "kernels.h"
#include "qtt_core.h"

namespace qtt {

namespace {
constexpr int TPB = 256;

inline unsigned grid_for(int64_t n) { return unsigned(n); }

template <class T>
__global__ void k_permute(const T *__restrict__ src, T *__restrict__ dst, const PermEntry *__restrict__ ents,
                          const Chunk *__restrict__ chunks) {
    const Chunk ch = chunks[blockIdx.x];
    const PermEntry &e = ents[ch.seg];
    const int r = e.rank;
    for (int i = threadIdx.x; i < ch.len; i += blockDim.x) {
        int64_t lin = ch.start + i;
        int64_t rem = lin;
        int64_t so = e.src_off;
        for (int d = r - 1; d >= 0; --d) {
            int64_t n = e.dims[d];
            int64_t q = rem / n;
            so += (rem - q * n) * e.stride[d];
            rem = q;
        }
        dst[e.dst_off + lin] = src[so];
    }
}

__device__ __forceinline__ double coef_val(const Coef &c) {
    if (!c.dev) return c.mult;
    double x = *c.dev;
    if (c.invert) x = (fabs(x) >= c.guard) ? 1.0 / x : 1.0;
    return c.mult * x;
}

__global__ void k_axpby(const double *__restrict__ a, const double *__restrict__ b, double *__restrict__ out,
                        const AxpbySeg *__restrict__ segs, const Chunk *__restrict__ chunks, Coef ca, Coef cb) {
    const Chunk ch = chunks[blockIdx.x];
    const AxpbySeg s = segs[ch.seg];
    const double xa = coef_val(ca), xb = coef_val(cb);
    for (int i = threadIdx.x; i < ch.len; i += blockDim.x) {
        int64_t k = ch.start + i;
        double v = 0.0;
        if (s.a_off >= 0) v = xa * a[s.a_off + k];
        if (s.b_off >= 0) v += xb * b[s.b_off + k];
        out[s.out_off + k] = v;
    }
}

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ double block_sum(double v) {
    __shared__ double red[32];
    v = warp_sum(v);
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[w] = v;
    __syncthreads();
    int nw = (blockDim.x + 31) >> 5;
    v = (threadIdx.x < nw) ? red[threadIdx.x] : 0.0;
    if (w == 0) v = warp_sum(v);
    return v;  // valid in thread 0
}

__global__ void k_dot(const double *__restrict__ a, const double *__restrict__ b, const DotSeg *__restrict__ segs,
                      const Chunk *__restrict__ chunks, double *__restrict__ partials) {
    const Chunk ch = chunks[blockIdx.x];
    const DotSeg s = segs[ch.seg];
    double acc = 0.0;
    for (int i = threadIdx.x; i < ch.len; i += blockDim.x) {
        int64_t k = ch.start + i;
        acc = fma(a[s.a_off + k], b[s.b_off + k], acc);
    }
    acc = block_sum(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

__global__ void k_reduce(const double *__restrict__ partials, int64_t n, double *__restrict__ out) {
    double acc = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) acc += partials[i];
    acc = block_sum(acc);
    if (threadIdx.x == 0) *out = acc;
}

__global__ void k_mul_lastleg(const double *__restrict__ u, const double *__restrict__ d, double *__restrict__ out,
                              const LastLegSeg *__restrict__ segs, const Chunk *__restrict__ chunks) {
    const Chunk ch = chunks[blockIdx.x];
    const LastLegSeg s = segs[ch.seg];
    for (int i = threadIdx.x; i < ch.len; i += blockDim.x) {
        int64_t k = ch.start + i;
        out[s.out_off + k] = u[s.u_off + k] * d[s.d_off + (k % s.L)];
    }
}

__global__ void k_normalize(double *x, int64_t n) {
    double acc = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) acc = fma(x[i], x[i], acc);
    acc = block_sum(acc);
    __shared__ double inv;
    if (threadIdx.x == 0) inv = 1.0 / sqrt(acc);
    __syncthreads();
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) x[i] *= inv;
}

__global__ void k_convert(const void *src, void *dst, int64_t n, int sf, int df) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        double v = sf ? static_cast<const double *>(src)[i] : double(static_cast<const float *>(src)[i]);
        if (df)
            static_cast<double *>(dst)[i] = v;
        else
            static_cast<float *>(dst)[i] = float(v);
    }
}

__global__ void k_zero(double *p, int64_t n) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        p[i] = 0.0;
}

__global__ void k_scatter(const double *__restrict__ src, double *__restrict__ dst,
                          const ScatterEntry *__restrict__ ents, const Chunk *__restrict__ chunks) {
    const Chunk ch = chunks[blockIdx.x];
    const ScatterEntry e = ents[ch.seg];
    for (int i = threadIdx.x; i < ch.len; i += blockDim.x) {
        int64_t k = ch.start + i;
        int r = int(k / e.k), c = int(k - int64_t(r) * e.k);
        dst[e.dst_off + k] = src[e.src_off + int64_t(e.r0 + r) + int64_t(c) * e.ld];
    }
}

__global__ void k_sqrt(double *x) { x[0] = sqrt(x[0]); }

// eig2x2Mat_impl (sources/dmrg.cpp:544-572) for real scalars.
__global__ void k_eig2x2(double *s) {
    double a0 = s[0], b = s[1], a1 = s[2];
    double crit = sqrt((a0 - a1) * (a0 - a1) + 4.0 * (b * b));
    double E0 = (a0 + a1 - crit) / 2.0;
    double delt = E0 - a1;
    double o = sqrt(delt / (-crit));
    bool zero_o = ((o + E0) == E0) || isnan(o);
    double n = (b * o) / delt;
    if (zero_o) {
        n = 1.0;
        o = 0.0;
    }
    s[3] = E0;
    s[4] = o;
    s[5] = n;
    s[6] = (isnan(o) || isnan(n)) ? 1.0 : 0.0;
}
}  // namespace

void launch_permute(const void *src, void *dst, const PermEntry *entries, const Chunk *chunks, int64_t nchunks,
                    int elem_bytes) {
    if (nchunks <= 0) return;
    auto s = ctx().stream;
    if (elem_bytes == 8)
        k_permute<double><<<grid_for(nchunks), TPB, 0, s>>>(static_cast<const double *>(src),
                                                            static_cast<double *>(dst), entries, chunks);
    else
        k_permute<float><<<grid_for(nchunks), TPB, 0, s>>>(static_cast<const float *>(src), static_cast<float *>(dst),
                                                           entries, chunks);
    count_launch();
    cuda_check(cudaGetLastError(), "permute kernel launch");
}

void launch_axpby(const double *a, const double *b, double *out, const AxpbySeg *segs, const Chunk *chunks,
                  int64_t nchunks, Coef ca, Coef cb) {
    if (nchunks <= 0) return;
    k_axpby<<<grid_for(nchunks), TPB, 0, ctx().stream>>>(a, b, out, segs, chunks, ca, cb);
    count_launch();
    cuda_check(cudaGetLastError(), "axpby kernel launch");
}

void launch_dot(const double *a, const double *b, const DotSeg *segs, const Chunk *chunks, int64_t nchunks,
                double *partials, double *out) {
    auto s = ctx().stream;
    if (nchunks > 0) {
        k_dot<<<grid_for(nchunks), TPB, 0, s>>>(a, b, segs, chunks, partials);
        count_launch();
    }
    k_reduce<<<1, 1024, 0, s>>>(partials, nchunks, out);
    count_launch();
    cuda_check(cudaGetLastError(), "dot kernel launch");
}

void launch_mul_lastleg(const double *u, const double *d, double *out, const LastLegSeg *segs, const Chunk *chunks,
                        int64_t nchunks) {
    if (nchunks <= 0) return;
    k_mul_lastleg<<<grid_for(nchunks), TPB, 0, ctx().stream>>>(u, d, out, segs, chunks);
    count_launch();
    cuda_check(cudaGetLastError(), "mul_lastleg kernel launch");
}

void launch_normalize(double *x, int64_t n, double *) {
    if (n <= 0) return;
    k_normalize<<<1, 1024, 0, ctx().stream>>>(x, n);
    count_launch();
    cuda_check(cudaGetLastError(), "normalize kernel launch");
}

void launch_convert(const void *src, void *dst, int64_t n, int sf, int df) {
    if (n <= 0) return;
    int64_t g = std::min<int64_t>((n + TPB - 1) / TPB, 152 * 16);
    k_convert<<<unsigned(g), TPB, 0, ctx().stream>>>(src, dst, n, sf, df);
    count_launch();
    cuda_check(cudaGetLastError(), "convert kernel launch");
}

void launch_zero(double *p, int64_t n) {
    if (n <= 0) return;
    int64_t g = std::min<int64_t>((n + TPB - 1) / TPB, 152 * 16);
    k_zero<<<unsigned(g), TPB, 0, ctx().stream>>>(p, n);
    count_launch();
    cuda_check(cudaGetLastError(), "zero kernel launch");
}

void launch_scatter(const double *src, double *dst, const ScatterEntry *e, const Chunk *chunks, int64_t nchunks) {
    if (nchunks <= 0) return;
    k_scatter<<<grid_for(nchunks), TPB, 0, ctx().stream>>>(src, dst, e, chunks);
    count_launch();
    cuda_check(cudaGetLastError(), "scatter kernel launch");
}

void launch_eig2x2(double *s) {
    k_eig2x2<<<1, 1, 0, ctx().stream>>>(s);
    count_launch();
    cuda_check(cudaGetLastError(), "eig2x2 kernel launch");
}

void launch_sqrt(double *x) {
    k_sqrt<<<1, 1, 0, ctx().stream>>>(x);
    count_launch();
    cuda_check(cudaGetLastError(), "sqrt kernel launch");
}

}  // namespace qtt
