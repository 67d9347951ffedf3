// Internal C++ host layer of the GB300 block-sparse tensor library.
//
// A btensor (QuantiT's quantit::btensor, include/blockTensor/btensor.h:105) is
// kept as host-side structure tables (sections, charges, selection rule, block
// list) plus ONE device buffer holding every block, each block a dense row-major
// array at a recorded element offset.  The host tables drive planning (which
// block pairs meet in a contraction, which blocks form an SVD sector); the
// device buffer is only touched by kernels.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <functional>
#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace qtt {

#ifdef __CUDACC__
#define QTT_HD __host__ __device__
#else
#define QTT_HD
#endif

constexpr int MAXC = 4;     // group factors per charge (U(1)xU(1)xZ(n)... up to 4)
constexpr int MAXRANK = 8;  // largest tensor rank handled by the kernels

// ---------------------------------------------------------------- errors
// Status codes returned through the C-ABI; the C++ exception the reference
// throws for the same condition is noted beside each.
enum Status : int {
    OK = 0,
    ERR_INVALID_ARGUMENT = 1,  // std::invalid_argument
    ERR_OUT_OF_RANGE = 2,      // std::out_of_range (block_at on a missing block)
    ERR_DOMAIN = 3,            // std::domain_error (throw_bad_tensor)
    ERR_LOGIC = 4,             // std::logic_error (NaN in the 2x2 solve, item() on many blocks)
    ERR_RUNTIME = 5,           // std::runtime_error
    ERR_CUDA = 6,              // CUDA runtime failure
    ERR_OOM = 7,               // device allocation failure
    ERR_CHECK = 8,             // c10::Error from TORCH_CHECK (contraction compatibility)
    ERR_NO_DATA = 9,           // a structure-only btensor was given to a numeric operation
};

struct Error : std::exception {
    int code;
    std::string msg;
    Error(int c, std::string m) : code(c), msg(std::move(m)) {}
    const char *what() const noexcept override { return msg.c_str(); }
};

[[noreturn]] inline void fail(int code, const std::string &m) { throw Error(code, m); }
inline void cuda_check(cudaError_t e, const char *what) {
    if (e != cudaSuccess) fail(e == cudaErrorMemoryAllocation ? ERR_OOM : ERR_CUDA,
                               std::string(what) + ": " + cudaGetErrorString(e));
}

// Kernel attributes (dynamic shared-memory limits) and device properties belong to
// a device, so set-up done once per process would configure only the first device
// a host thread used.  once_per_device runs f the first time it is reached with
// a given device current (devices 0..63; a repeated f is harmless, so a race
// between two threads costs at most one extra call).
inline int current_device() {
    int dev = 0;
    cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    return dev;
}
template <class F>
void once_per_device(std::atomic<uint64_t> &done, F &&f) {
    const int dev = current_device();
    const uint64_t bit = (dev >= 0 && dev < 64) ? (uint64_t(1) << dev) : 0;
    if (bit && (done.load(std::memory_order_acquire) & bit)) return;
    f();
    if (bit) done.fetch_or(bit, std::memory_order_release);
}
// Streaming multiprocessors of the current device (cached per device).
inline int device_sm_count() {
    static std::atomic<int> cache[64];
    const int dev = current_device();
    if (dev >= 0 && dev < 64) {
        const int c = cache[dev].load(std::memory_order_relaxed);
        if (c > 0) return c;
    }
    int nsm = 0;
    cuda_check(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev), "SM count");
    if (dev >= 0 && dev < 64) cache[dev].store(nsm, std::memory_order_relaxed);
    return nsm;
}

// ---------------------------------------------------------------- charges
// conserved::Z (int16, +) and conserved::C<N> (uint16 in [0,N), + mod N), and
// their tuple products quantity<G...> (include/Conserved/quantity.h,
// Composite/quantity_impl.h).  mod[i] == 0 marks a Z factor.
struct Group {
    int n = 1;
    uint16_t mod[MAXC] = {0, 0, 0, 0};
    bool operator==(const Group &o) const {
        if (n != o.n) return false;
        for (int i = 0; i < n; ++i)
            if (mod[i] != o.mod[i]) return false;
        return true;
    }
};

struct Charge {
    int16_t v[MAXC] = {0, 0, 0, 0};
};

QTT_HD inline Charge qadd(const Charge &a, const Charge &b, const Group &g) {
    Charge r;
    for (int i = 0; i < g.n; ++i) {
        if (g.mod[i]) {
            uint32_t s = uint32_t(uint16_t(a.v[i])) + uint32_t(uint16_t(b.v[i]));
            if (s >= g.mod[i]) s -= g.mod[i];
            r.v[i] = int16_t(uint16_t(s));
        } else {
            r.v[i] = int16_t(a.v[i] + b.v[i]);
        }
    }
    return r;
}
inline Charge qinv(const Charge &a, const Group &g) {
    Charge r;
    for (int i = 0; i < g.n; ++i) {
        if (g.mod[i]) {
            uint16_t x = uint16_t(a.v[i]);
            r.v[i] = int16_t(uint16_t(x ? g.mod[i] - x : 0));
        } else {
            r.v[i] = int16_t(-a.v[i]);
        }
    }
    return r;
}
QTT_HD inline bool qeq(const Charge &a, const Charge &b, const Group &g) {
    for (int i = 0; i < g.n; ++i)
        if (a.v[i] != b.v[i]) return false;
    return true;
}
// tuple-lexicographic order, signed for Z factors and unsigned for C<N> factors
inline bool qless(const Charge &a, const Charge &b, const Group &g) {
    for (int i = 0; i < g.n; ++i) {
        int x = g.mod[i] ? int(uint16_t(a.v[i])) : int(a.v[i]);
        int y = g.mod[i] ? int(uint16_t(b.v[i])) : int(b.v[i]);
        if (x < y) return true;
        if (y < x) return false;
    }
    return false;
}
inline Charge qneutral() { return Charge{}; }

// ---------------------------------------------------------------- device memory
enum DType : int { F64 = 0, F32 = 1 };
inline size_t dsize(DType t) { return t == F64 ? 8 : 4; }

// A stream-ordered device allocation (cudaMallocAsync from the device's default
// memory pool, which keeps freed memory cached for reuse).
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    cudaStream_t stream = nullptr;
    ~DevBuf();
};
using BufPtr = std::shared_ptr<DevBuf>;

// Per-thread execution context: the stream all work is issued on and a pinned
// staging ring used to ship planning tables (task lists, offsets) to the device.
struct Ctx {
    cudaStream_t stream = nullptr;
    int device = 0;
    // staging ring
    char *host_ring = nullptr;
    char *dev_ring = nullptr;
    size_t ring_bytes = 0;
    size_t ring_pos = 0;
    cudaEvent_t half_done[2] = {nullptr, nullptr};
    int cur_half = 0;
    bool half_used[2] = {false, false};
    // error word of this thread's tensor-core launches (bounded waits that expired)
    int *tc_err = nullptr;
    bool tc_used = false;
    // set while a CUDA graph is being captured on this stream: uploads go to
    // dedicated device buffers (constants of the graph) and statistics are off
    bool capturing = false;
    std::vector<void *> *capture_tables = nullptr;
};
Ctx &ctx();
void set_stream(cudaStream_t s);
BufPtr dev_alloc(size_t bytes);
// Copy a host table to device memory valid for work issued afterwards on the
// current stream (ring-buffered; the region is reused after the stream passes it).
void *upload(const void *host, size_t bytes);
template <class T>
T *upload_vec(const std::vector<T> &v) {
    return v.empty() ? nullptr : static_cast<T *>(upload(v.data(), v.size() * sizeof(T)));
}

// ---------------------------------------------------------------- btensor
struct BT {
    Group g;
    int rank = 0;
    std::vector<int64_t> sbd;  // sections_by_dim
    std::vector<int64_t> ssz;  // packed sections_sizes
    std::vector<Charge> cv;    // packed c_vals
    Charge sel;                // selection rule
    DType dt = F64;
    std::vector<int64_t> bidx;  // nblocks * rank block indices, in block-list order
    std::vector<int64_t> boff;  // element offset of each block in buf
    int64_t nnz = 0;            // total elements of all blocks
    BufPtr buf;                 // device data; null for a structure-only btensor
    bool has_data = false;

    int64_t nblocks() const { return int64_t(boff.size()); }
    const int64_t *idx(int64_t b) const { return bidx.data() + b * rank; }
    int64_t addr(int d) const {
        int64_t a = 0;
        for (int i = 0; i < d; ++i) a += sbd[i];
        return a;
    }
    std::vector<int64_t> addrs() const {
        std::vector<int64_t> a(rank + 1, 0);
        for (int i = 0; i < rank; ++i) a[i + 1] = a[i] + sbd[i];
        return a;
    }
    int64_t block_numel(int64_t b) const {
        int64_t n = 1;
        int64_t a = 0;
        const int64_t *ix = idx(b);
        for (int d = 0; d < rank; ++d) {
            n *= ssz[a + ix[d]];
            a += sbd[d];
        }
        return n;
    }
    void block_shape(int64_t b, int64_t *out) const {
        int64_t a = 0;
        const int64_t *ix = idx(b);
        for (int d = 0; d < rank; ++d) {
            out[d] = ssz[a + ix[d]];
            a += sbd[d];
        }
    }
    Charge block_charge(const int64_t *ix) const {
        Charge q;
        int64_t a = 0;
        for (int d = 0; d < rank; ++d) {
            q = qadd(q, cv[a + ix[d]], g);
            a += sbd[d];
        }
        return q;
    }
    bool allowed(const int64_t *ix) const { return qeq(block_charge(ix), sel, g); }
    void *data() const {
        if (!has_data || !buf) fail(ERR_NO_DATA, "this btensor carries structure only (no device data)");
        return buf->p;
    }
    // Copy of the structure without blocks.
    BT shape_only() const {
        BT o;
        o.g = g;
        o.rank = rank;
        o.sbd = sbd;
        o.ssz = ssz;
        o.cv = cv;
        o.sel = sel;
        o.dt = dt;
        return o;
    }
    // Assign compact offsets in block-list order (boff already sized to the block
    // count, which a rank-0 tensor cannot derive from bidx) and recount nnz.
    void compact_offsets() {
        int64_t o = 0;
        for (size_t b = 0; b < boff.size(); ++b) {
            boff[b] = o;
            o += block_numel(int64_t(b));
        }
        nnz = o;
    }
    void alloc_data() {
        buf = dev_alloc(size_t(std::max<int64_t>(nnz, 1)) * dsize(dt));
        has_data = true;
    }
};

std::string check_tensor(const BT &t);  // sources/btensor.cpp:405-467

// lexicographic comparison of block indices
inline bool idx_less(const int64_t *a, const int64_t *b, int r) {
    for (int i = 0; i < r; ++i) {
        if (a[i] < b[i]) return true;
        if (b[i] < a[i]) return false;
    }
    return false;
}
// Reorder the blocks of t into lexicographic order of their indices (the order a
// flat_map keeps, include/blockTensor/flat_map.h:151).
void sort_blocks(BT &t);

// ---------------------------------------------------------------- operations
BT make_tensor(const Group &g, int rank, const int64_t *sbd, const int64_t *ssz, const Charge *cv,
               const Charge &sel, DType dt);
void set_blocks(BT &t, int64_t nb, const int64_t *idx, bool with_data, const void *src, bool src_on_device);
BT permute(const BT &t, const std::vector<int64_t> &perm);
BT reshape(const BT &t, const std::vector<int64_t> &groups);
BT reshape_as(const BT &t, const BT &shape);
BT inverse_cvals(const BT &t);
BT conj(const BT &t);
BT tensordot(const BT &a, const BT &b, const std::vector<int64_t> &da, const std::vector<int64_t> &db);
BT tensorgdot(const BT &add, const BT &a, const BT &b, const std::vector<int64_t> &da,
              const std::vector<int64_t> &db, double beta, double alpha);
BT add_scaled(const BT &a, const BT &b, double ca, double cb);
BT scale(const BT &a, double c);
double dot_all(const BT &a, const BT &b);
BT mul_lastleg(const BT &u, const BT &d);

struct SVDOut {
    BT U, d, V;
    // after a truncation: sum of |s|^pow over the dropped values and over all values
    // (the discarded weight truncate_impl bounds by tol^pow, btensor_linalg.cpp:658-682)
    double discarded = 0.0, total = 0.0;
    double kept_min = -1.0;  // the smallest value the truncation keeps, less its 2 eps slack
};
SVDOut svd(const BT &t);                       // untruncated, rank >= 2, sectors on the last two legs
SVDOut svd_split(const BT &t, int64_t split);  // svd(A, split)
SVDOut truncate(SVDOut &&in, int64_t max_size, int64_t min_size, double tol, double pw, bool has_v = true);
// Orthogonal start matrices for the sector SVDs at one bond: the q-side rotation V of
// each sector of the previous decomposition there, keyed by the sector's orientation
// and q-side sections.  Any orthogonal start V0 gives an exact SVD (W = (W V0) V0^T, and
// the sweeps accumulate into V0); one from an unchanged basis leaves W V0 nearly
// column-orthogonal, and the Jacobi needs a few sweeps instead of tens.
struct WarmStart {
    struct Entry {
        std::vector<int64_t> key;
        BufPtr buf;   // the rotation buffer of that decomposition
        int64_t off;  // element offset of the sector's q x q matrix in buf
        int f32;      // element type: float (mixed path) or double
    };
    std::vector<Entry> entries;
};
// ws (optional): warm starts read from and written back to ws.
SVDOut svd_truncated(const BT &t, int64_t split, double tol, int64_t min_size, int64_t max_size, double pw,
                     WarmStart *ws = nullptr);
struct EighOut {
    BT d, U;
};
// random_bMPS(bond_dim, mpo, constraint, seed) (sources/MPT.cpp:424-462): one rank-3
// site tensor per MPO site, total charge `target`, N(0, 1) entries, unit-norm sites.
std::vector<BT> random_mps(const std::vector<BT> &mpo, int64_t D, const Charge &target, uint64_t seed);
EighOut eigh(const BT &t, bool upper);
EighOut eigh_split(const BT &t, int64_t split);
// Jacobi sweeps per sector of the last decomposition: of the FP64 sweeps that gave the
// factors, or (first_stage) of the mixed path's FP32 sweeps before them (empty otherwise)
std::vector<int> last_svd_sweeps(bool first_stage = false);

// ---------------------------------------------------------------- precision of block GEMMs
enum GemmMode : int {
    GEMM_F64 = 0,        // plain FP64 (the drop-in)
    GEMM_TF32X3 = 1,     // split TF32 on tcgen05, FP32 accumulation, 3 products
    GEMM_BF16X3 = 2,     // split BF16 on tcgen05, FP32 accumulation, 3 products
};
void set_gemm_mode(int mode);  // process-wide default
int gemm_mode();               // the calling thread's override, else the default
// Per-thread override for the duration of a call (a DMRG solve runs its own
// precision without touching other threads' solves).
struct ScopedGemmMode {
    int saved;
    explicit ScopedGemmMode(int mode);
    ~ScopedGemmMode();
};
// Sector-SVD Jacobi kernel: 0 = block-cyclic where it fits (default), 1 = scalar
// (one column pair per warp and grid step).
void set_jacobi_variant(int v);
int jacobi_variant();
// Block-width autotuner of the block-Jacobi kernel (on by default) and its decisions.
void set_autotune(int on);
std::string autotune_report();
// Persistent tensor-core GEMM for launches of at least two tiles per SM (on by default).
void set_persistent_gemm(int on);
int persistent_gemm();
// Block-sparsity planner of tensordot: 0 host merge-join (the default), 1 device
// (planner.cu) wherever its limits allow, 2 device for contractions of at least
// planner_auto_blocks() blocks in the two operands together.
void set_planner(int mode, int64_t auto_blocks);
int planner_mode();
int64_t planner_auto_blocks();
// planner calls and host wall seconds (planning only): [0] host calls, [1] device
// calls, [2] device attempts that fell back to the host; secs[0] host, secs[1] device
void planner_stats(int64_t *calls, double *secs, bool reset);
void planner_account(int which, double secs);
// Deflation of numerically zero columns in the sector SVDs of a truncating svd (on by default).
void set_svd_deflation(int on);
int svd_deflation();
// Non-zero when a tensor-core kernel gave up on a bounded wait since the last
// check (synchronises the device; read and cleared).
int tc_error_check();
inline void tc_error_raise() {
    if (int e = tc_error_check()) fail(ERR_RUNTIME, "tensor-core GEMM: bounded wait expired (code " + std::to_string(e) + ")");
}

// ---------------------------------------------------------------- timing statistics
// Per-kernel-class device time measured with CUDA events on the launching stream,
// plus the algorithmic work each launch did (FLOPs or bytes).
// ST_SVD64: the FP64 stage of the mixed path's sector SVDs (a part of ST_SVD's time).
// ST_JAC32 / ST_JAC64: work only (no time): the FLOPs the sector SVDs' Jacobi sweeps
// performed in FP32 and in FP64 (sweeps x (6 p q^2 + 3 q^3) per p x q sector, the
// one-sided Jacobi count; the FP64 count adds the mixed path's Newton-Schulz and W V
// products, 8 q^3 + 2 p q^2, and counts its sweeps after the decoupling one on the K kept
// columns, plus their V product 2 q K^2).
enum StatKind : int {
    ST_GEMM = 0,
    ST_PERMUTE = 1,
    ST_SVD = 2,
    ST_ELEMWISE = 3,
    ST_PACK = 4,
    ST_SVD64 = 5,
    ST_JAC32 = 6,
    ST_JAC64 = 7,
    ST_COUNT = 8
};
void stats_enable(bool on);
bool stats_enabled();
// Work known only after the kernels ran (e.g. Jacobi sweeps): resolved when read.
void stats_defer_work(int kind, std::function<double()> f);
struct StatScope {
    int kind;
    double work;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    StatScope(int k, double w);
    ~StatScope();
};
void stats_get(int kind, double *ms, double *work, int64_t *launches);
void stats_reset();
int64_t launch_count();
void count_launch(int n = 1);

}  // namespace qtt
