// Launch wrappers between the host layer and the CUDA kernels.  All tables are
// device pointers prepared by the host planner (uploaded through the staging
// ring); all launches go to the current context stream.
#pragma once
#include <atomic>
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

namespace qtt {

// Work over many variable-length segments is cut into chunks of at most
// CHUNK elements that never straddle a segment; one CTA handles one chunk.
constexpr int CHUNK = 2048;
struct Chunk {
    int32_t seg;
    int32_t len;
    int64_t start;  // element offset inside the segment
};

// ------------------------------------------------------------ permute / copy
// Segment = one block: dst[dst_off + e] = src[src_off + sum_d idx_d(e) * stride[d]]
// where idx(e) is the row-major multi-index of e over dims[0..rank).
struct PermEntry {
    int64_t src_off, dst_off;
    int32_t rank, pad;
    int64_t dims[8];
    int64_t stride[8];
};
void launch_permute(const void *src, void *dst, const PermEntry *entries, const Chunk *chunks, int64_t nchunks,
                    int elem_bytes);

// ------------------------------------------------------------ grouped GEMM
// Output block o: C[o] (M x N row-major at c_off) = alpha * sum_{p in [p0,p1)} A_p B_p
//                                                   + beta * Cadd (at add_off, when add_off >= 0).
// A_p is M x K: row-major at a_off when a_t == 0, stored K x M row-major when a_t == 1.
// B_p is K x N: row-major at b_off when b_t == 0, stored N x K row-major when b_t == 1.
struct GemmPair {
    int64_t a_off, b_off;
    int32_t K;
    int32_t pad;
};
struct GemmOut {
    int64_t c_off, add_off;
    int32_t M, N;
    int32_t p0, p1;
};
struct GemmTile {
    int32_t out, m0, n0, pad;
};
struct GemmArgs {
    const double *A;
    const double *B;
    double *C;
    const double *Cadd;
    const GemmPair *pairs;
    const GemmOut *outs;
    const GemmTile *tiles;
    int32_t ntiles;
    int32_t a_t, b_t;
    double alpha, beta;
};
void launch_gemm_f64(const GemmArgs &a);

// Split-precision tensor-core variant (tcgen05).  Operands are first converted,
// block by block, into "matrix form" split arrays: hi = tf32(x), lo = tf32(x - hi)
// as FP32 bit patterns, rows x K4 row-major (K contiguous, K4 = K rounded up to 4,
// zero padded), so the GEMM producers only move 16-byte vectors.
// Segment = one operand block; element e of the (rows x K) matrix reads
// src[src_off + sum_d idx_d(e) * stride[d]] with idx(e) the row-major index over dims.
struct SplitEntry {
    int64_t src_off, dst_off;  // dst_off: element offset of the block in the split arrays
    // K4: the padded K (rounded up to 8 for TF32X3, 16 for BF16X3); blocks are tiled in
    // core matrices of 8 rows x 16 bytes (rows padded to 8), a row group's core
    // matrices in K order
    int32_t rank, K, K4;
    int32_t flags;  // SPLIT_SMALL: rows * K < 2^31 (32-bit index math); SPLIT_CONTIG: row-major source
    int64_t dims[8];
    int64_t stride[8];
};
enum : int32_t { SPLIT_SMALL = 1, SPLIT_CONTIG = 2 };
// Source offset of element `lin` (row-major over dims) of a split entry.
__device__ __forceinline__ int64_t split_src(const SplitEntry &e, int64_t lin) {
    if (e.flags & SPLIT_CONTIG) return e.src_off + lin;
    if (e.flags & SPLIT_SMALL) {
        uint32_t rem = uint32_t(lin), off = 0;
        for (int d = e.rank - 1; d >= 0; --d) {
            const uint32_t n = uint32_t(e.dims[d]), q = rem / n;
            off += (rem - q * n) * uint32_t(e.stride[d]);
            rem = q;
        }
        return e.src_off + off;
    }
    int64_t rem = lin, so = e.src_off;
    for (int d = e.rank - 1; d >= 0; --d) {
        const int64_t n = e.dims[d], q = rem / n;
        so += (rem - q * n) * e.stride[d];
        rem = q;
    }
    return so;
}
// (row, k) of element `lin` of a split entry's rows x K matrix.
__device__ __forceinline__ void split_rowk(const SplitEntry &e, int64_t lin, int64_t &row, int64_t &k) {
    if (e.flags & SPLIT_SMALL) {
        const uint32_t r = uint32_t(lin) / uint32_t(e.K);
        row = r;
        k = int64_t(uint32_t(lin) - r * uint32_t(e.K));
    } else {
        row = lin / e.K;
        k = lin - row * e.K;
    }
}
// amax: the bit pattern of max |x| over the operand (launch_amax); every element is
// scaled by the exact power of two 2^-ilogb(amax) before the split, so operands of any
// magnitude use the FP32 range, and the GEMM epilogue undoes the two scales exactly.
void launch_split_tf32(const double *src, float *hi, float *lo, const SplitEntry *e, const Chunk *chunks,
                       int64_t nchunks, const unsigned long long *amax);
// *amax (zeroed by the caller) <- max(*amax, bits of |x|) over n doubles (bit order =
// value order for non-negative doubles, so the maximum is exact and deterministic).
void launch_amax(const double *x, int64_t n, unsigned long long *amax);
// Split-BF16 variant: hi / mid / lo bf16 (uint16) arrays in the same tiling (core
// matrices of 8 rows x 8 elements, K padded to 16); the same amax scaling.
void launch_split_bf16x3(const double *src, void *hi, void *mid, void *lo, const SplitEntry *e, const Chunk *chunks,
                         int64_t nchunks, const unsigned long long *amax);
// A pair's a_off / b_off index the split arrays (core-matrix tiling); A rows = M,
// B rows = N (TF32X3: hi / lo, mid unused; BF16X3: hi / mid / lo).
struct TcArgs {
    const void *Ahi, *Amid, *Alo, *Bhi, *Bmid, *Blo;
    const unsigned long long *amax_a, *amax_b;  // operand scales (see launch_split_tf32)
    double *C;
    const double *Cadd;
    const GemmPair *pairs;
    const GemmOut *outs;
    const GemmTile *tiles;
    int32_t ntiles;
    int32_t max_chunks;  // most K chunks of any tile (sizes the shared-memory ring; 0: unknown)
    double alpha, beta;
};
void launch_gemm_tc(const TcArgs &a, int mode);
// the BF16X3 kernel (called by launch_gemm_tc); err: the context's device error word
void launch_gemm_bf16x3(const TcArgs &a, int *err, cudaStream_t stream);
int gemm_tile_m(int mode);
int gemm_tile_n(int mode);

// ------------------------------------------------------------ elementwise
// A coefficient: mult * (dev ? f(*dev) : 1) with f(x) = x, or f(x) = 1/x when
// invert is set and |x| >= guard (f(x) = 1 below the guard).
struct Coef {
    double mult;
    const double *dev;
    int32_t invert;
    int32_t pad;
    double guard;
};
inline Coef coef_host(double v) { return Coef{v, nullptr, 0, 0, 0.0}; }
// Segment: out[out_off + i] = ca * a[a_off + i] + cb * b[b_off + i]; an offset of -1 reads 0.
struct AxpbySeg {
    int64_t a_off, b_off, out_off;
};
void launch_axpby(const double *a, const double *b, double *out, const AxpbySeg *segs, const Chunk *chunks,
                  int64_t nchunks, Coef ca, Coef cb);
// Segment: sum_i a[a_off + i] * b[b_off + i]; partial sums per chunk then a fixed-order
// reduction into *out (device), so the result is deterministic.
struct DotSeg {
    int64_t a_off, b_off;
};
void launch_dot(const double *a, const double *b, const DotSeg *segs, const Chunk *chunks, int64_t nchunks,
                double *partials, double *out);
// Segment: out[out_off + e] = u[u_off + e] * d[d_off + (e % L)]
struct LastLegSeg {
    int64_t u_off, d_off, out_off, L;
};
void launch_mul_lastleg(const double *u, const double *d, double *out, const LastLegSeg *segs, const Chunk *chunks,
                        int64_t nchunks);
// x[0..n) *= 1/sqrt(sum x^2)   (d /= sqrt(sum(d.pow(2))), sources/dmrg.cpp:188)
void launch_normalize(double *x, int64_t n, double *scratch);
void launch_convert(const void *src, void *dst, int64_t n, int src_f64, int dst_f64);

// ------------------------------------------------------------ sector decompositions
// Sector s: m x n matrix A; the work matrix W (p x q, column-major, p >= q) is A when
// m >= n, A^T otherwise.  Offsets are element offsets into the work, rotation,
// left-vector, right-vector and value buffers.
struct SectorDesc {
    int64_t w_off, rot_off, u_off, v_off, s_off;
    int32_t m, n, p, q;
    int32_t trans;  // 1 when W = A^T
    int32_t mode;   // 0: svd, 1: eigh (symmetric input, shifted to positive definite)
    int32_t warm;   // 1: rot holds an orthogonal start V0 and work holds W V0 (warm start)
    int32_t pad;
    double shift;   // eigh: diagonal shift added before the sweeps
};
// Warm start of one sector SVD: work[w_off ..] (p x q, column-major) <- W V0 with V0 the
// q x q orthogonal matrix at v0 (the work type), and rot[rot_off ..] <- V0.  tmp: scratch
// with the work buffer's offsets.  Tiles of 64 x 64 outputs, tile_start = prefix sums.
struct WarmDesc {
    int64_t w_off, rot_off;
    const void *v0;
    int32_t p, q, tile_start, pad;
};
void launch_warm_apply(void *work, void *rot, void *tmp, const WarmDesc *wd, int nwarm, int ntiles, int f32);
// FP64 refinement of an FP32 sector decomposition (mixed path): from the FP32
// rotations rot32 (at rot_off), vb <- the FP64-orthogonalised rotation (two
// Newton-Schulz steps through va, with g as q x q scratch), w1 <- w64 vb (at w_off).
// The FP64 Jacobi then runs warm on (w1, vb).
void launch_svd_refine(const float *rot32, const double *w64, double *w1, double *va, double *vb, double *g,
                       const std::vector<SectorDesc> &secs);
// out[s_off + j] = squared norm (FP64) of column j of every sector's work matrix (f32:
// FP32 work matrices)
void launch_col_norms(const void *W, const SectorDesc *secs, int nsec, int max_q, double *out, int f32);
// Column copies dst[dst_off + r] = src[src_off + r], r < len (FP64), one task per column:
// the gather and scatter of the kept columns around the restricted FP64 sweeps.
struct ColCopy {
    int64_t src_off, dst_off;
    int32_t len, pad;
};
void launch_col_copy(const double *src, double *dst, const std::vector<ColCopy> &cols);
// Vn = Vg R per sector (FP64): Vg (vrows x k at vg_off, column-major), R (k x k at r_off),
// Vn (vrows x k at vn_off).
struct RotProduct {
    int64_t vg_off, r_off, vn_off;
    int32_t vrows, k;
};
void launch_rot_product(const double *vg, const double *r, double *vn, const std::vector<RotProduct> &t);
// Segment = one input block (rows x cols at src_off) placed at rows [r0, r0+rows),
// cols [c0, c0+cols) of sector `sector`.
struct PackEntry {
    int64_t src_off;
    int32_t sector, rows, cols, r0, c0, pad;
};
void launch_zero(double *p, int64_t n);
// The work / rotation buffers hold float when f32 != 0 (mixed path), else double.
void launch_pack(const double *src, void *work, const PackEntry *e, const Chunk *chunks, int64_t nchunks,
                 const SectorDesc *sec, int f32);
// eigh: symmetrise W from one triangle, then shift the diagonal by the sector's
// Frobenius norm (written back into sec[s].shift) so the matrix is positive definite.
void launch_eigh_prepare(void *work, SectorDesc *sec, int nsec, int upper, int f32);
// Batched one-sided Jacobi over all sectors in one cooperative launch.
// slot_start[nsec+1]: prefix sums of the pairs each sector contributes per step
// ((q + q%2)/2); max_steps_per_sweep = max over sectors of (q + q%2 - 1).
// sweeps_out[s] receives the number of sweeps sector s used; flags holds
// nsec*max_sweeps ints of scratch.
// sum_q: the sectors' total column count (sizes the cooperative grid to the work).
// vwork (optional, jacobi_vwork_bytes): lets the block kernel defer each step's V
// updates to the next step, where CTAs without a block pair run them; without it
// every CTA updates V right after its block pair.
// defl (optional, launch_deflation_thresholds, the work type): per sector, a column
// whose squared norm falls to the threshold or below is set to zero and leaves the
// sweeps (a numerically zero column); null: no deflation.
// skip (optional, the work type): per sector, a pair whose squared column norms are both
// below it is not rotated (columns the caller will discard).
void launch_jacobi(void *work, void *rot, const SectorDesc *sec, const int *slot_start, int nsec,
                   int max_steps_per_sweep, int max_sweeps, int *sweeps_out, int *flags, int f32, int max_p,
                   int64_t sum_q, void *vwork = nullptr, size_t vwork_bytes = 0, const void *defl = nullptr,
                   void *dnorm = nullptr, const void *skip = nullptr);
// thr[s] <- delta^2 ||W_s||_F^2 for every svd sector (0 for eigh), in the work type.
void launch_deflation_thresholds(const void *work, const SectorDesc *sec, int nsec, double delta, void *thr, int f32);
// dnorm (with defl; the work type, sum of q entries at s_off, zero on entry) receives
// the squared norm of every deflated column.
size_t jacobi_vwork_bytes(int nsec, int64_t sum_q, int max_steps_per_sweep, int max_sweeps, int f32);
// Column norms, sort (descending for svd, ascending eigenvalues for eigh),
// normalisation and completion of null columns; writes U (m x k), V (n x k)
// column-major and s (k) per sector in FP64, k = min(m, n).  max_q: largest q;
// scratch: FP64 buffer with the work buffer's element offsets.  complete_cap >= 0
// completes only the first complete_cap null columns of each sector (in value
// order): the caller truncates the others away.  perm_out (sum of q ints at s_off) with
// complete_cap == 0: the factor writes run on many CTAs per sector (max_elems: the
// largest q * (p + q) over the sectors).
void launch_finish(const void *work, const void *rot, double *U, double *V, double *s, const SectorDesc *sec,
                   int nsec, int max_q, double *scratch, int f32, int complete_cap = -1, const void *dnorm = nullptr,
                   int *dpos = nullptr, int *perm_out = nullptr, int64_t max_elems = 0);
// The same two launches on an explicit stream (no library context involved).
// tune == false never times block widths (no host synchronisation): the width the
// autotuner settled on for the class is used if there is one, else the default.
void launch_jacobi_on(cudaStream_t stream, void *work, void *rot, const SectorDesc *sec, const int *slot_start,
                      int nsec, int max_steps_per_sweep, int max_sweeps, int *sweeps_out, int *flags, int f32,
                      int max_p, int64_t sum_q, void *vwork = nullptr, size_t vwork_bytes = 0,
                      const void *defl = nullptr, void *dnorm = nullptr, bool tune = true,
                      const void *skip = nullptr);
void launch_finish_on(cudaStream_t stream, const void *work, const void *rot, double *U, double *V, double *s,
                      const SectorDesc *sec, int nsec, int max_q, double *scratch, int f32, int complete_cap = -1,
                      const void *dnorm = nullptr, int *dpos = nullptr, int *perm_out = nullptr,
                      int64_t max_elems = 0);
// Segment = one output block (rows x k row-major at dst_off) from a column-major
// (ld x *) sector matrix at src_off: dst[i*k + j] = src[src_off + (r0 + i) + j*ld].
struct ScatterEntry {
    int64_t src_off, dst_off;
    int32_t ld, r0, k, pad;
};
void launch_scatter(const double *src, double *dst, const ScatterEntry *e, const Chunk *chunks, int64_t nchunks);

// ------------------------------------------------------------ 2x2 Ritz step on device
// s[0]=a0, s[1]=b, s[2]=a1  ->  s[3]=E, s[4]=o, s[5]=n, s[6]=nan flag
// (eig2x2Mat_impl, sources/dmrg.cpp:544-572)
void launch_eig2x2(double *s);
void launch_sqrt(double *x);

}  // namespace qtt
