// Runtime support: per-thread stream context, stream-ordered device memory, the
// pinned staging ring for planning tables, kernel timing statistics, and the
// btensor construction / validation helpers.
#include <atomic>
#include <mutex>
#include <numeric>
#include <sstream>

#include "kernels.h"
#include "qtt_core.h"

namespace qtt {

namespace {
thread_local Ctx *tl_ctx = nullptr;
thread_local cudaStream_t tl_user_stream = nullptr;
std::mutex g_ctx_mu;
std::vector<Ctx *> g_ctxs;  // leaked on purpose: contexts live until process exit

constexpr size_t RING_BYTES = size_t(64) << 20;

void init_ring(Ctx &c) {
    if (c.host_ring) return;
    c.ring_bytes = RING_BYTES;
    cuda_check(cudaMallocHost(&c.host_ring, c.ring_bytes), "cudaMallocHost(staging ring)");
    cuda_check(cudaMalloc(&c.dev_ring, c.ring_bytes), "cudaMalloc(staging ring)");
    for (auto &e : c.half_done) cuda_check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
}
}  // namespace

Ctx &ctx() {
    if (!tl_ctx) {
        std::lock_guard<std::mutex> lk(g_ctx_mu);
        auto *c = new Ctx();
        int dev = 0;
        cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
        c->device = dev;
        cuda_check(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "cudaStreamCreate");
        // keep freed pool memory cached instead of returning it to the driver
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            uint64_t thr = ~uint64_t(0);
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
        }
        init_ring(*c);
        g_ctxs.push_back(c);
        tl_ctx = c;
    }
    if (tl_user_stream) tl_ctx->stream = tl_user_stream;
    return *tl_ctx;
}

void set_stream(cudaStream_t s) {
    tl_user_stream = s;
    if (tl_ctx && !s) {
        // restore a library-owned stream
        cuda_check(cudaStreamCreateWithFlags(&tl_ctx->stream, cudaStreamNonBlocking), "cudaStreamCreate");
    }
}

DevBuf::~DevBuf() {
    if (p) cudaFreeAsync(p, stream);
}

BufPtr dev_alloc(size_t bytes) {
    Ctx &c = ctx();
    auto b = std::make_shared<DevBuf>();
    bytes = (bytes + 255) & ~size_t(255);
    cudaError_t e = cudaMallocAsync(&b->p, bytes, c.stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        fail(ERR_OOM, std::string("device allocation of ") + std::to_string(bytes) + " bytes failed: " +
                          cudaGetErrorString(e));
    }
    b->bytes = bytes;
    b->stream = c.stream;
    return b;
}

void *upload(const void *host, size_t bytes) {
    Ctx &c = ctx();
    size_t need = (bytes + 255) & ~size_t(255);
    if (c.capturing) {
        // a captured graph replays its kernels long after this call: its tables live in
        // their own buffers, filled now (relaxed capture mode allows the synchronous copy)
        void *d = nullptr;
        cuda_check(cudaMalloc(&d, std::max<size_t>(need, 256)), "cudaMalloc(graph table)");
        c.capture_tables->push_back(d);
        cuda_check(cudaMemcpy(d, host, bytes, cudaMemcpyHostToDevice), "cudaMemcpy(graph table)");
        return d;
    }
    if (need > c.ring_bytes / 2) fail(ERR_RUNTIME, "planning table larger than the staging ring");
    size_t half = c.ring_bytes / 2;
    size_t half_end = (c.cur_half + 1) * half;
    if (c.ring_pos + need > half_end) {
        // leave the current half: mark where the stream is, then enter the other half
        cuda_check(cudaEventRecord(c.half_done[c.cur_half], c.stream), "cudaEventRecord");
        c.half_used[c.cur_half] = true;
        c.cur_half ^= 1;
        if (c.half_used[c.cur_half]) cuda_check(cudaEventSynchronize(c.half_done[c.cur_half]), "cudaEventSync");
        c.ring_pos = c.cur_half * half;
    }
    std::memcpy(c.host_ring + c.ring_pos, host, bytes);
    void *d = c.dev_ring + c.ring_pos;
    cuda_check(cudaMemcpyAsync(d, c.host_ring + c.ring_pos, bytes, cudaMemcpyHostToDevice, c.stream),
               "cudaMemcpyAsync(plan)");
    c.ring_pos += need;
    return d;
}

// ---------------------------------------------------------------- statistics
namespace {
struct StatAcc {
    double ms = 0, work = 0;
    int64_t launches = 0;
};
bool g_stats_on = false;
StatAcc g_stats[ST_COUNT];
struct Pending {
    int kind;
    double work;
    cudaEvent_t e0, e1;
};
std::vector<Pending> g_pending;
std::mutex g_stats_mu;
std::atomic<int64_t> g_launches{0};

std::vector<std::pair<int, std::function<double()>>> g_deferred;

void drain_pending() {
    for (auto &d : g_deferred) g_stats[d.first].work += d.second();
    g_deferred.clear();
    for (auto &p : g_pending) {
        float ms = 0;
        cudaEventSynchronize(p.e1);
        cudaEventElapsedTime(&ms, p.e0, p.e1);
        g_stats[p.kind].ms += ms;
        g_stats[p.kind].work += p.work;
        g_stats[p.kind].launches += 1;
        cudaEventDestroy(p.e0);
        cudaEventDestroy(p.e1);
    }
    g_pending.clear();
}
}  // namespace

void stats_enable(bool on) { g_stats_on = on; }
void stats_defer_work(int kind, std::function<double()> f) {
    std::lock_guard<std::mutex> lk(g_stats_mu);
    g_deferred.push_back({kind, std::move(f)});
}
bool stats_enabled() { return g_stats_on; }
StatScope::StatScope(int k, double w) : kind(k), work(w) {
    if (!g_stats_on || ctx().capturing) return;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, ctx().stream);
}
StatScope::~StatScope() {
    if (!e0) return;
    cudaEventRecord(e1, ctx().stream);
    std::lock_guard<std::mutex> lk(g_stats_mu);
    g_pending.push_back({kind, work, e0, e1});
    if (g_pending.size() > 4096) drain_pending();
}
void stats_get(int kind, double *ms, double *work, int64_t *launches) {
    std::lock_guard<std::mutex> lk(g_stats_mu);
    drain_pending();
    if (kind < 0 || kind >= ST_COUNT) fail(ERR_INVALID_ARGUMENT, "unknown statistics kind");
    if (ms) *ms = g_stats[kind].ms;
    if (work) *work = g_stats[kind].work;
    if (launches) *launches = g_stats[kind].launches;
}
void stats_reset() {
    std::lock_guard<std::mutex> lk(g_stats_mu);
    drain_pending();
    for (auto &s : g_stats) s = StatAcc();
}
int64_t launch_count() { return g_launches.load(); }
void count_launch(int n) { g_launches += n; }

// ---------------------------------------------------------------- gemm mode
namespace {
std::atomic<int> g_gemm_mode{GEMM_F64};
thread_local int tl_gemm_mode = -1;  // -1: no override on this thread
}
void set_gemm_mode(int m) {
    if (m < GEMM_F64 || m > GEMM_BF16X3) fail(ERR_INVALID_ARGUMENT, "unknown GEMM precision mode");
    g_gemm_mode = m;
}
int gemm_mode() { return tl_gemm_mode >= 0 ? tl_gemm_mode : g_gemm_mode.load(); }
ScopedGemmMode::ScopedGemmMode(int mode) : saved(tl_gemm_mode) {
    if (mode < GEMM_F64 || mode > GEMM_BF16X3) fail(ERR_INVALID_ARGUMENT, "unknown GEMM precision mode");
    tl_gemm_mode = mode;
}
ScopedGemmMode::~ScopedGemmMode() { tl_gemm_mode = saved; }

namespace {
std::atomic<int> g_jacobi_variant{0};
}
void set_jacobi_variant(int v) {
    if (v < 0 || v > 1) fail(ERR_INVALID_ARGUMENT, "unknown Jacobi kernel variant");
    g_jacobi_variant = v;
}
int jacobi_variant() { return g_jacobi_variant; }
namespace {
std::atomic<int> g_svd_deflation{1};
std::atomic<int> g_persistent_gemm{1};
}
void set_persistent_gemm(int on) { g_persistent_gemm = on ? 1 : 0; }
int persistent_gemm() { return g_persistent_gemm; }
void set_svd_deflation(int on) { g_svd_deflation = on ? 1 : 0; }
int svd_deflation() { return g_svd_deflation; }

namespace {
std::atomic<int> g_planner{0};
std::atomic<int64_t> g_planner_auto{3000};
std::mutex g_plan_mu;
int64_t g_plan_calls[3] = {0, 0, 0};
double g_plan_secs[2] = {0.0, 0.0};
}  // namespace
void set_planner(int mode, int64_t auto_blocks) {
    if (mode < 0 || mode > 2) fail(ERR_INVALID_ARGUMENT, "planner mode must be 0 (host), 1 (device) or 2 (auto)");
    if (auto_blocks < 0) fail(ERR_INVALID_ARGUMENT, "the automatic planner threshold must be >= 0");
    g_planner = mode;
    g_planner_auto = auto_blocks;
}
int planner_mode() { return g_planner; }
int64_t planner_auto_blocks() { return g_planner_auto; }
void planner_account(int which, double secs) {
    std::lock_guard<std::mutex> lk(g_plan_mu);
    g_plan_calls[which] += 1;
    if (which < 2) g_plan_secs[which] += secs;
}
void planner_stats(int64_t *calls, double *secs, bool reset) {
    std::lock_guard<std::mutex> lk(g_plan_mu);
    for (int i = 0; i < 3; ++i) calls[i] = g_plan_calls[i];
    for (int i = 0; i < 2; ++i) secs[i] = g_plan_secs[i];
    if (reset) {
        for (auto &c : g_plan_calls) c = 0;
        for (auto &x : g_plan_secs) x = 0.0;
    }
}

// ---------------------------------------------------------------- btensor helpers
std::string check_tensor(const BT &t) {
    std::ostringstream M;
    if (int64_t(t.sbd.size()) != t.rank)
        M << "rank (" << t.rank << ") incoherent with internal sections_by_dim (size " << t.sbd.size() << ")\n";
    int64_t tot = std::accumulate(t.sbd.begin(), t.sbd.end(), int64_t(0));
    if (tot != int64_t(t.ssz.size()) || tot != int64_t(t.cv.size()))
        M << "number of section accross all dimension (" << tot << ") incoherent with number of specified section sizes ("
          << t.ssz.size() << ")\n";
    for (int64_t b = 0; b < t.nblocks(); ++b) {
        const int64_t *ix = t.idx(b);
        bool ok = true;
        for (int d = 0; d < t.rank; ++d)
            if (ix[d] < 0 || ix[d] >= t.sbd[d]) {
                M << "block " << b << " index " << d << " is out of range\n";
                ok = false;
            }
        if (ok && !t.allowed(ix)) M << "block " << b << " incompatible with selection rule\n";
    }
    return M.str();
}

void sort_blocks(BT &t) {
    int64_t nb = t.nblocks();
    std::vector<int64_t> ord(nb);
    std::iota(ord.begin(), ord.end(), 0);
    int r = t.rank;
    std::stable_sort(ord.begin(), ord.end(),
                     [&](int64_t a, int64_t b) { return idx_less(t.idx(a), t.idx(b), r); });
    std::vector<int64_t> bi(t.bidx.size()), bo(nb);
    for (int64_t k = 0; k < nb; ++k) {
        std::copy(t.idx(ord[k]), t.idx(ord[k]) + r, bi.begin() + k * r);
        bo[k] = t.boff[ord[k]];
    }
    t.bidx.swap(bi);
    t.boff.swap(bo);
}

BT make_tensor(const Group &g, int rank, const int64_t *sbd, const int64_t *ssz, const Charge *cv,
               const Charge &sel, DType dt) {
    if (rank < 0 || rank > MAXRANK) fail(ERR_INVALID_ARGUMENT, "rank must be in [0, 8]");
    if (g.n < 1 || g.n > MAXC) fail(ERR_INVALID_ARGUMENT, "a charge has 1 to 4 group factors");
    BT t;
    t.g = g;
    t.rank = rank;
    t.sbd.assign(sbd, sbd + rank);
    int64_t ns = 0;
    for (int d = 0; d < rank; ++d) {
        if (sbd[d] < 1) fail(ERR_INVALID_ARGUMENT, "every leg needs at least one section");
        ns += sbd[d];
    }
    t.ssz.assign(ssz, ssz + ns);
    for (auto s : t.ssz)
        if (s < 0) fail(ERR_INVALID_ARGUMENT, "section sizes must be non-negative");
    t.cv.assign(cv, cv + ns);
    t.sel = sel;
    t.dt = dt;
    return t;
}

void set_blocks(BT &t, int64_t nb, const int64_t *idx, bool with_data, const void *src, bool src_on_device) {
    if (nb < 0) fail(ERR_INVALID_ARGUMENT, "negative block count");
    int r = t.rank;
    std::vector<int64_t> bi(idx, idx + nb * r);
    if (r == 0 && nb > 1) fail(ERR_INVALID_ARGUMENT, "a rank-0 btensor holds at most one block");
    // validate like btensor::block (btensor.cpp:380-395)
    for (int64_t b = 0; b < nb; ++b) {
        const int64_t *ix = bi.data() + b * r;
        for (int d = 0; d < r; ++d)
            if (ix[d] < 0 || ix[d] >= t.sbd[d]) fail(ERR_INVALID_ARGUMENT, "block index out of range");
        if (!t.allowed(ix)) fail(ERR_INVALID_ARGUMENT, "block index not allowed by selection rule");
    }
    t.bidx = bi;
    t.boff.assign(nb, 0);
    // offsets of the caller's order
    std::vector<int64_t> src_off(nb);
    int64_t o = 0;
    for (int64_t b = 0; b < nb; ++b) {
        src_off[b] = o;
        o += t.block_numel(b);
    }
    t.nnz = o;
    t.boff = src_off;
    // reject duplicate indices, sort into flat_map order (data offsets travel along)
    sort_blocks(t);
    for (int64_t b = 1; b < nb; ++b)
        if (!idx_less(t.idx(b - 1), t.idx(b), r)) fail(ERR_INVALID_ARGUMENT, "duplicate block index");
    t.buf.reset();
    t.has_data = false;
    if (!with_data) return;
    t.alloc_data();
    size_t bytes = size_t(t.nnz) * dsize(t.dt);
    Ctx &c = ctx();
    if (!src) {
        cuda_check(cudaMemsetAsync(t.buf->p, 0, bytes, c.stream), "cudaMemsetAsync");
    } else if (src_on_device) {
        cuda_check(cudaMemcpyAsync(t.buf->p, src, bytes, cudaMemcpyDeviceToDevice, c.stream), "cudaMemcpyAsync");
    } else {
        cuda_check(cudaMemcpyAsync(t.buf->p, src, bytes, cudaMemcpyHostToDevice, c.stream), "cudaMemcpyAsync");
        cuda_check(cudaStreamSynchronize(c.stream), "cudaStreamSynchronize");
    }
}

}  // namespace qtt
