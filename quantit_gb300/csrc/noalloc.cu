// Dense SVD without any device allocation: qtt_svd_dense_noalloc.
//
// Some callers cannot call cudaMalloc.  A plug-in loaded into a host application
// that owns all device memory may not allocate behind the host's back; a solver
// running under a memory budget fixed at start-up may not grow; a real-time loop
// sharing the GPU cannot afford cudaMalloc / cudaFree, which can synchronise the
// whole device.  For them this entry point runs the same FP64 one-sided Jacobi as
// the block-sparse SVD on one dense matrix, with all its working storage in a
// file-scope device array instead of allocations.  The caller still passes the
// input and output buffers.
//
// Scratch: g_svd_scratch below, QTT_SVD_NOALLOC_SCRATCH_BYTES (about 2.6 MB),
// enough for m, n <= QTT_SVD_NOALLOC_MAX_DIM (256).  Every GPU that loads the
// library holds it until the process exits.  All calls share it and it keeps the
// last call's contents: two calls whose work overlaps on the GPU (different
// streams, or different host threads without ordering) race on it and corrupt
// each other's results.  Every call writes every scratch element it reads.
//
// Set-up: the first call on a device, with that device current, looks up the
// array's device address (cudaGetSymbolAddress) and the kernels' shared-memory
// attributes for that device; make that first call before any stream capture.
// The block width of the Jacobi kernel is never timed on this path, so a call
// only issues work on the caller's stream and returns without waiting for it.
#include <mutex>
#include <string>

#include "../../include/qtt_gb300.h"
#include "kernels.h"
#include "qtt_core.h"

namespace qtt {
void set_last_error(const std::string &msg);
}

namespace {

constexpr int kMaxDim = QTT_SVD_NOALLOC_MAX_DIM;
constexpr int kMaxSweeps = 80;
constexpr size_t kMat = size_t(kMaxDim) * kMaxDim * sizeof(double);  // one max-size matrix
// layout: work W | rotation | U (col-major) | V (col-major) | finish scratch | tables
constexpr size_t kOffW = 0, kOffRot = kMat, kOffU = 2 * kMat, kOffV = 3 * kMat, kOffScr = 4 * kMat;
constexpr size_t kOffDesc = 5 * kMat;                       // one SectorDesc
constexpr size_t kOffSlots = kOffDesc + 256;                // 2 ints
constexpr size_t kOffSweeps = kOffSlots + 256;              // 1 int
constexpr size_t kOffFlags = kOffSweeps + 256;              // kMaxSweeps ints
constexpr size_t kTotal = kOffFlags + kMaxSweeps * sizeof(int);
static_assert(kTotal <= QTT_SVD_NOALLOC_SCRATCH_BYTES, "scratch layout exceeds the declared size");

static __device__ __align__(256) unsigned char g_svd_scratch[QTT_SVD_NOALLOC_SCRATCH_BYTES];

// Device address of g_svd_scratch on each device (host code may not use the
// symbol itself: on the host it names a stand-in, not device memory).
std::mutex g_mu;
void *g_addr[64] = {nullptr};

void *scratch_for_current_device() {
    int dev = 0;
    qtt::cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= 64) qtt::fail(qtt::ERR_INVALID_ARGUMENT, "device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
        void *p = nullptr;
        qtt::cuda_check(cudaGetSymbolAddress(&p, g_svd_scratch), "cudaGetSymbolAddress(scratch)");
        g_addr[dev] = p;
    }
    return g_addr[dev];
}

__global__ void k_na_init(qtt::SectorDesc d, int slots, qtt::SectorDesc *desc, int *slot_start) {
    *desc = d;
    slot_start[0] = 0;
    slot_start[1] = slots;
}

// W (p x q, column-major) = A when m >= n, A^T otherwise; A is m x n row-major.
__global__ void k_na_pack(const double *__restrict__ a, int m, int n, double *__restrict__ w, int trans) {
    const int64_t total = int64_t(m) * n;
    for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < total; e += int64_t(gridDim.x) * blockDim.x) {
        const int i = int(e / n), j = int(e % n);
        w[trans ? (int64_t(j) + int64_t(i) * n) : (int64_t(i) + int64_t(j) * m)] = a[e];
    }
}

// dst (rows x k, row-major) from src (rows x k, column-major)
__global__ void k_na_rowmajor(const double *__restrict__ src, int rows, int k, double *__restrict__ dst) {
    const int64_t total = int64_t(rows) * k;
    for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < total; e += int64_t(gridDim.x) * blockDim.x) {
        const int i = int(e / k), j = int(e % k);
        dst[e] = src[int64_t(i) + int64_t(j) * rows];
    }
}

void svd_dense_noalloc(const double *a, int64_t m, int64_t n, double *u, double *s, double *v, cudaStream_t st) {
    if (m < 1 || n < 1) qtt::fail(qtt::ERR_INVALID_ARGUMENT, "matrix dimensions must be positive");
    if (m > kMaxDim || n > kMaxDim)
        qtt::fail(qtt::ERR_INVALID_ARGUMENT, "qtt_svd_dense_noalloc: " + std::to_string(m) + " x " + std::to_string(n) +
                                                  " exceeds the maximum of " + std::to_string(kMaxDim) + " x " +
                                                  std::to_string(kMaxDim) + " its static scratch holds");
    if (!a || !u || !s || !v) qtt::fail(qtt::ERR_INVALID_ARGUMENT, "null device pointer");
    char *base = static_cast<char *>(scratch_for_current_device());
    double *W = reinterpret_cast<double *>(base + kOffW);
    double *rot = reinterpret_cast<double *>(base + kOffRot);
    double *Uc = reinterpret_cast<double *>(base + kOffU);
    double *Vc = reinterpret_cast<double *>(base + kOffV);
    double *scr = reinterpret_cast<double *>(base + kOffScr);
    qtt::SectorDesc *desc = reinterpret_cast<qtt::SectorDesc *>(base + kOffDesc);
    int *slots = reinterpret_cast<int *>(base + kOffSlots);
    int *sweeps = reinterpret_cast<int *>(base + kOffSweeps);
    int *flags = reinterpret_cast<int *>(base + kOffFlags);

    qtt::SectorDesc d{};
    d.m = int32_t(m);
    d.n = int32_t(n);
    d.trans = m < n ? 1 : 0;
    d.p = int32_t(std::max(m, n));
    d.q = int32_t(std::min(m, n));
    d.mode = 0;
    const int qp = d.q + (d.q & 1);
    k_na_init<<<1, 1, 0, st>>>(d, qp / 2, desc, slots);
    qtt::cuda_check(cudaGetLastError(), "no-alloc init launch");
    k_na_pack<<<64, 256, 0, st>>>(a, int(m), int(n), W, d.trans);
    qtt::cuda_check(cudaGetLastError(), "no-alloc pack launch");
    // the Jacobi kernel initialises the rotation; the launcher clears the flags
    // tune = false: the block width is never timed here, so the call never waits on the stream
    qtt::launch_jacobi_on(st, W, rot, desc, slots, 1, std::max(1, qp - 1), kMaxSweeps, sweeps, flags, 0, d.p, d.q,
                          nullptr, 0, nullptr, nullptr, false);
    qtt::launch_finish_on(st, W, rot, Uc, Vc, s, desc, 1, d.q, scr, 0);
    k_na_rowmajor<<<64, 256, 0, st>>>(Uc, int(m), d.q, u);
    k_na_rowmajor<<<64, 256, 0, st>>>(Vc, int(n), d.q, v);
    qtt::cuda_check(cudaGetLastError(), "no-alloc layout launch");
    qtt::count_launch(4);  // init, pack, two layout kernels (the Jacobi and finish launchers count theirs)
}

}  // namespace

extern "C" int qtt_svd_dense_noalloc(const double *a, int64_t m, int64_t n, double *u, double *s, double *v,
                                     void *stream) {
    try {
        svd_dense_noalloc(a, m, n, u, s, v, static_cast<cudaStream_t>(stream));
        return QTT_OK;
    } catch (const qtt::Error &e) {
        qtt::set_last_error(e.msg);
        return e.code;
    } catch (const std::exception &e) {
        qtt::set_last_error(e.what());
        return QTT_ERR_RUNTIME;
    }
}
