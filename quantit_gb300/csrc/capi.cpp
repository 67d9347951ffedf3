// extern "C" boundary: opaque btensor handles over the C++ host layer.  Every
// entry point catches the host layer's exceptions and turns them into a status
// code plus a thread-local message (include/qtt_gb300.h).
#include <cstring>
#include <string>

#include "../../include/qtt_gb300.h"
#include "dmrg.h"
#include "ops_util.h"
#include "qtt_core.h"

struct qtt_bt_s {
    qtt::BT t;
};

namespace {
thread_local std::string tl_err;

template <class F>
int guarded(F &&f) {
    try {
        f();
        return QTT_OK;
    } catch (const qtt::Error &e) {
        tl_err = e.msg;
        return e.code;
    } catch (const std::bad_alloc &) {
        tl_err = "host allocation failed";
        return QTT_ERR_OOM;
    } catch (const std::exception &e) {
        tl_err = e.what();
        return QTT_ERR_RUNTIME;
    }
}

}  // namespace

namespace qtt {
void set_last_error(const std::string &msg) { tl_err = msg; }
}  // namespace qtt

namespace {
qtt::BT &T(qtt_bt h) {
    if (!h) qtt::fail(qtt::ERR_INVALID_ARGUMENT, "null btensor handle");
    return h->t;
}
qtt_bt wrap(qtt::BT &&t) {
    auto *h = new qtt_bt_s();
    h->t = std::move(t);
    return h;
}
std::vector<int64_t> vec(const int64_t *p, int64_t n) {
    if (n > 0 && !p) qtt::fail(qtt::ERR_INVALID_ARGUMENT, "null array");
    return std::vector<int64_t>(p, p + std::max<int64_t>(n, 0));
}
void out_check(void *p) {
    if (!p) qtt::fail(qtt::ERR_INVALID_ARGUMENT, "null output pointer");
}
}  // namespace

extern "C" {

const char *qtt_last_error(void) { return tl_err.c_str(); }
const char *qtt_version(void) { return "quantit_gb300 0.1 (sm_103a)"; }

int qtt_init(int device) {
    return guarded([&] {
        qtt::cuda_check(cudaSetDevice(device), "cudaSetDevice");
        qtt::ctx();
    });
}
int qtt_set_stream(void *stream) {
    return guarded([&] { qtt::set_stream(static_cast<cudaStream_t>(stream)); });
}
void *qtt_get_stream(void) {
    void *s = nullptr;
    guarded([&] { s = qtt::ctx().stream; });
    return s;
}
int qtt_synchronize(void) {
    return guarded([&] { qtt::cuda_check(cudaStreamSynchronize(qtt::ctx().stream), "cudaStreamSynchronize"); });
}
int qtt_set_gemm_mode(int mode) {
    return guarded([&] { qtt::set_gemm_mode(mode); });
}
int qtt_get_gemm_mode(void) { return qtt::gemm_mode(); }
int qtt_device_memory(int64_t *free_bytes, int64_t *total_bytes) {
    return guarded([&] {
        if (!free_bytes || !total_bytes) qtt::fail(qtt::ERR_INVALID_ARGUMENT, "null output pointer");
        size_t f = 0, t = 0;
        qtt::cuda_check(cudaMemGetInfo(&f, &t), "cudaMemGetInfo");
        *free_bytes = int64_t(f);
        *total_bytes = int64_t(t);
    });
}
int qtt_set_autotune(int on) {
    return guarded([&] { qtt::set_autotune(on); });
}
int qtt_set_svd_deflation(int on) {
    return guarded([&] { qtt::set_svd_deflation(on); });
}
int qtt_set_planner(int mode, int64_t auto_blocks) {
    return guarded([&] { qtt::set_planner(mode, auto_blocks); });
}
int qtt_planner_stats(int64_t *calls, double *secs, int reset) {
    return guarded([&] {
        if (!calls || !secs) qtt::fail(qtt::ERR_INVALID_ARGUMENT, "null output pointer");
        qtt::planner_stats(calls, secs, reset != 0);
    });
}
int qtt_set_persistent_gemm(int on) {
    return guarded([&] { qtt::set_persistent_gemm(on); });
}
int qtt_autotune_report(char *buf, int64_t cap, int64_t *len) {
    return guarded([&] {
        const std::string r = qtt::autotune_report();
        if (len) *len = int64_t(r.size());
        if (buf && cap > 0) {
            const size_t n = std::min<size_t>(r.size(), size_t(cap - 1));
            std::memcpy(buf, r.data(), n);
            buf[n] = 0;
        }
    });
}
int qtt_set_jacobi_kernel(int which) {
    return guarded([&] { qtt::set_jacobi_variant(which); });
}

int qtt_bt_create(int32_t rank, const int64_t *sbd, const int64_t *ssz, int32_t ncomp, const uint16_t *moduli,
                  const int16_t *c_vals, const int16_t *sel, int32_t dtype, qtt_bt *out) {
    return guarded([&] {
        out_check(out);
        if (ncomp < 1 || ncomp > qtt::MAXC) qtt::fail(qtt::ERR_INVALID_ARGUMENT, "a charge has 1 to 4 factors");
        if (dtype != QTT_F64 && dtype != QTT_F32) qtt::fail(qtt::ERR_INVALID_ARGUMENT, "unknown dtype");
        if (rank < 0 || rank > qtt::MAXRANK) qtt::fail(qtt::ERR_INVALID_ARGUMENT, "rank must be in [0, 8]");
        qtt::Group g;
        g.n = ncomp;
        for (int i = 0; i < ncomp; ++i) g.mod[i] = moduli ? moduli[i] : 0;
        int64_t ns = 0;
        for (int d = 0; d < rank; ++d) ns += sbd[d];
        std::vector<qtt::Charge> cv(ns);
        for (int64_t s = 0; s < ns; ++s)
            for (int i = 0; i < ncomp; ++i) cv[s].v[i] = c_vals[s * ncomp + i];
        qtt::Charge q;
        for (int i = 0; i < ncomp; ++i) q.v[i] = sel ? sel[i] : 0;
        *out = wrap(qtt::make_tensor(g, rank, sbd, ssz, cv.data(), q, qtt::DType(dtype)));
    });
}

int qtt_bt_set_blocks(qtt_bt t, int64_t nb, const int64_t *idx, const void *host_data) {
    return guarded([&] { qtt::set_blocks(T(t), nb, idx, true, host_data, false); });
}
int qtt_bt_set_blocks_device(qtt_bt t, int64_t nb, const int64_t *idx, const void *dev_data) {
    return guarded([&] { qtt::set_blocks(T(t), nb, idx, true, dev_data, true); });
}
int qtt_bt_set_block_structure(qtt_bt t, int64_t nb, const int64_t *idx) {
    return guarded([&] { qtt::set_blocks(T(t), nb, idx, false, nullptr, false); });
}
int qtt_bt_destroy(qtt_bt t) {
    return guarded([&] { delete t; });
}
int qtt_bt_clone(qtt_bt t, qtt_bt *out) {
    return guarded([&] {
        out_check(out);
        qtt::BT c = T(t);
        *out = wrap(std::move(c));
    });
}
int qtt_bt_meta(qtt_bt h, int32_t *rank, int64_t *nsections, int32_t *ncomp, int64_t *nblocks, int64_t *nnz,
                int32_t *dtype, int32_t *has_data) {
    return guarded([&] {
        const qtt::BT &t = T(h);
        if (rank) *rank = t.rank;
        if (nsections) *nsections = int64_t(t.ssz.size());
        if (ncomp) *ncomp = t.g.n;
        if (nblocks) *nblocks = t.nblocks();
        if (nnz) *nnz = t.nnz;
        if (dtype) *dtype = t.dt;
        if (has_data) *has_data = t.has_data ? 1 : 0;
    });
}
int qtt_bt_structure(qtt_bt h, int64_t *sbd, int64_t *ssz, int16_t *c_vals, int16_t *sel, uint16_t *moduli) {
    return guarded([&] {
        const qtt::BT &t = T(h);
        if (sbd) std::copy(t.sbd.begin(), t.sbd.end(), sbd);
        if (ssz) std::copy(t.ssz.begin(), t.ssz.end(), ssz);
        if (c_vals)
            for (size_t s = 0; s < t.cv.size(); ++s)
                for (int i = 0; i < t.g.n; ++i) c_vals[s * t.g.n + i] = t.cv[s].v[i];
        if (sel)
            for (int i = 0; i < t.g.n; ++i) sel[i] = t.sel.v[i];
        if (moduli)
            for (int i = 0; i < t.g.n; ++i) moduli[i] = t.g.mod[i];
    });
}
int qtt_bt_blocks(qtt_bt h, int64_t *block_index, int64_t *block_numel) {
    return guarded([&] {
        const qtt::BT &t = T(h);
        if (block_index) std::copy(t.bidx.begin(), t.bidx.end(), block_index);
        if (block_numel)
            for (int64_t b = 0; b < t.nblocks(); ++b) block_numel[b] = t.block_numel(b);
    });
}
int qtt_bt_download(qtt_bt h, void *host, int64_t nbytes) {
    return guarded([&] {
        const qtt::BT &t = T(h);
        const size_t es = qtt::dsize(t.dt);
        if (nbytes < int64_t(t.nnz * es)) qtt::fail(qtt::ERR_INVALID_ARGUMENT, "host buffer too small");
        if (t.nnz == 0) return;
        auto s = qtt::ctx().stream;
        char *dst = static_cast<char *>(host);
        // blocks in block-list order (offsets may be non-compact)
        bool compact = true;
        int64_t o = 0;
        for (int64_t b = 0; b < t.nblocks(); ++b) {
            if (t.boff[b] != o) compact = false;
            o += t.block_numel(b);
        }
        if (compact) {
            qtt::cuda_check(cudaMemcpyAsync(dst, t.data(), size_t(t.nnz) * es, cudaMemcpyDeviceToHost, s), "download");
        } else {
            o = 0;
            for (int64_t b = 0; b < t.nblocks(); ++b) {
                size_t n = size_t(t.block_numel(b)) * es;
                qtt::cuda_check(cudaMemcpyAsync(dst + o, static_cast<char *>(t.data()) + t.boff[b] * es, n,
                                                cudaMemcpyDeviceToHost, s),
                                "download");
                o += int64_t(n);
            }
        }
        qtt::cuda_check(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    });
}
int qtt_bt_check(qtt_bt h, char *msg, int64_t cap) {
    return guarded([&] {
        std::string m = qtt::check_tensor(T(h));
        if (msg && cap > 0) {
            std::strncpy(msg, m.c_str(), size_t(cap - 1));
            msg[cap - 1] = 0;
        }
    });
}

int qtt_permute(qtt_bt t, const int64_t *perm, qtt_bt *out) {
    return guarded([&] {
        out_check(out);
        *out = wrap(qtt::permute(T(t), vec(perm, T(t).rank)));
    });
}
int qtt_reshape(qtt_bt t, int32_t ng, const int64_t *groups, qtt_bt *out) {
    return guarded([&] {
        out_check(out);
        *out = wrap(qtt::reshape(T(t), vec(groups, ng)));
    });
}
int qtt_reshape_as(qtt_bt t, qtt_bt shape, qtt_bt *out) {
    return guarded([&] {
        out_check(out);
        *out = wrap(qtt::reshape_as(T(t), T(shape)));
    });
}
int qtt_conj(qtt_bt t, qtt_bt *out) {
    return guarded([&] {
        out_check(out);
        *out = wrap(qtt::conj(T(t)));
    });
}
int qtt_inverse_cvals(qtt_bt t, qtt_bt *out) {
    return guarded([&] {
        out_check(out);
        *out = wrap(qtt::inverse_cvals(T(t)));
    });
}

int qtt_tensordot(qtt_bt a, qtt_bt b, int32_t nd, const int64_t *da, const int64_t *db, qtt_bt *out) {
    return guarded([&] {
        out_check(out);
        *out = wrap(qtt::tensordot(T(a), T(b), vec(da, nd), vec(db, nd)));
    });
}
int qtt_tensorgdot(qtt_bt add, qtt_bt a, qtt_bt b, int32_t nd, const int64_t *da, const int64_t *db, double beta,
                   double alpha, qtt_bt *out) {
    return guarded([&] {
        out_check(out);
        *out = wrap(qtt::tensorgdot(T(add), T(a), T(b), vec(da, nd), vec(db, nd), beta, alpha));
    });
}
int qtt_tensorgdot_(qtt_bt add, qtt_bt a, qtt_bt b, int32_t nd, const int64_t *da, const int64_t *db, double beta,
                    double alpha) {
    return guarded([&] { T(add) = qtt::tensorgdot(T(add), T(a), T(b), vec(da, nd), vec(db, nd), beta, alpha); });
}

int qtt_add(qtt_bt a, qtt_bt b, double alpha, qtt_bt *out) {
    return guarded([&] {
        out_check(out);
        *out = wrap(qtt::add_scaled(T(a), T(b), 1.0, alpha));
    });
}
int qtt_mul_scalar(qtt_bt a, double s, qtt_bt *out) {
    return guarded([&] {
        out_check(out);
        *out = wrap(qtt::scale(T(a), s));
    });
}
int qtt_dot_all(qtt_bt a, qtt_bt b, double *out) {
    return guarded([&] {
        out_check(out);
        *out = qtt::dot_all(T(a), T(b));
    });
}
int qtt_mul_lastleg(qtt_bt u, qtt_bt d, qtt_bt *out) {
    return guarded([&] {
        out_check(out);
        *out = wrap(qtt::mul_lastleg(T(u), T(d)));
    });
}

int qtt_svd(qtt_bt t, qtt_bt *U, qtt_bt *d, qtt_bt *V) {
    return guarded([&] {
        out_check(U);
        out_check(d);
        out_check(V);
        auto r = qtt::svd(T(t));
        *U = wrap(std::move(r.U));
        *d = wrap(std::move(r.d));
        *V = wrap(std::move(r.V));
    });
}
int qtt_svd_split(qtt_bt t, int64_t split, qtt_bt *U, qtt_bt *d, qtt_bt *V) {
    return guarded([&] {
        out_check(U);
        out_check(d);
        out_check(V);
        auto r = qtt::svd_split(T(t), split);
        *U = wrap(std::move(r.U));
        *d = wrap(std::move(r.d));
        *V = wrap(std::move(r.V));
    });
}
int qtt_svd_truncate(qtt_bt t, int64_t split, double tol, int64_t min_size, int64_t max_size, double pw, qtt_bt *U,
                     qtt_bt *d, qtt_bt *V) {
    return guarded([&] {
        out_check(U);
        out_check(d);
        out_check(V);
        auto r = qtt::svd_truncated(T(t), split, tol, min_size, max_size, pw);
        *U = wrap(std::move(r.U));
        *d = wrap(std::move(r.d));
        *V = wrap(std::move(r.V));
    });
}
int qtt_truncate(qtt_bt U, qtt_bt d, qtt_bt V, int64_t max_size, int64_t min_size, double tol, double pw,
                 qtt_bt *Uo, qtt_bt *do_, qtt_bt *Vo) {
    return guarded([&] {
        out_check(Uo);
        out_check(do_);
        qtt::SVDOut in;
        in.U = T(U);
        in.d = T(d);
        if (V) in.V = T(V);
        auto r = qtt::truncate(std::move(in), max_size, min_size, tol, pw, V != nullptr);
        *Uo = wrap(std::move(r.U));
        *do_ = wrap(std::move(r.d));
        if (V && Vo) *Vo = wrap(std::move(r.V));
    });
}
int qtt_eigh(qtt_bt t, int32_t upper, qtt_bt *d, qtt_bt *U) {
    return guarded([&] {
        out_check(d);
        out_check(U);
        auto r = qtt::eigh(T(t), upper != 0);
        *d = wrap(std::move(r.d));
        *U = wrap(std::move(r.U));
    });
}
int qtt_eigh_split(qtt_bt t, int64_t split, qtt_bt *d, qtt_bt *U) {
    return guarded([&] {
        out_check(d);
        out_check(U);
        auto r = qtt::eigh_split(T(t), split);
        *d = wrap(std::move(r.d));
        *U = wrap(std::move(r.U));
    });
}

void qtt_dmrg_options_default(qtt_dmrg_options *o) {
    if (!o) return;
    o->cutoff = 1e-6;
    o->convergence_criterion = 1e-5;
    o->maximum_bond = INT64_MAX;
    o->minimum_bond = 4;
    o->maximum_iterations = 1000;
    o->gemm_mode = QTT_GEMM_F64;
    o->final_energy_fp64 = 1;
    o->lanczos_steps = 1;
    o->cuda_graphs = 1;
    o->svd_warm_start = 1;
    o->pad = 0;
}
int qtt_compute_2sites_hamil(qtt_bt wl, qtt_bt wr, qtt_bt *out) {
    return guarded([&] {
        out_check(out);
        *out = wrap(qtt::compute_2sites_hamil(T(wl), T(wr)));
    });
}
int qtt_hamil2site_times_state(qtt_bt state, qtt_bt hamil, qtt_bt L, qtt_bt R, qtt_bt *out) {
    return guarded([&] {
        out_check(out);
        *out = wrap(qtt::hamil2site_times_state(T(state), T(hamil), T(L), T(R)));
    });
}
int qtt_one_step_lanczos(qtt_bt state, qtt_bt hamil, qtt_bt L, qtt_bt R, qtt_bt *psi, double *a0, double *a1,
                         double *b) {
    return guarded([&] {
        out_check(psi);
        auto r = qtt::one_step_lanczos(T(state), T(hamil), T(L), T(R));
        *psi = wrap(std::move(r.psi));
        if (a0) *a0 = r.a0;
        if (a1) *a1 = r.a1;
        if (b) *b = r.b;
    });
}
int qtt_eig2x2(double a0, double a1, double b, double *E, double *o, double *n) {
    return guarded([&] {
        double e, oo, nn;
        qtt::eig2x2(a0, a1, b, e, oo, nn);
        if (E) *E = e;
        if (o) *o = oo;
        if (n) *n = nn;
    });
}
int qtt_compute_left_env(qtt_bt W, qtt_bt A, qtt_bt L, qtt_bt *out) {
    return guarded([&] {
        out_check(out);
        *out = wrap(qtt::compute_left_env(T(W), T(A), T(L)));
    });
}
int qtt_compute_right_env(qtt_bt W, qtt_bt A, qtt_bt R, qtt_bt *out) {
    return guarded([&] {
        out_check(out);
        *out = wrap(qtt::compute_right_env(T(W), T(A), T(R)));
    });
}
namespace {
qtt::DmrgOpts dmrg_opts(const qtt_dmrg_options *opt) {
    qtt::DmrgOpts o;
    if (opt) {
        o.cutoff = opt->cutoff;
        o.convergence_criterion = opt->convergence_criterion;
        o.maximum_bond = opt->maximum_bond;
        o.minimum_bond = opt->minimum_bond;
        o.maximum_iterations = opt->maximum_iterations;
        o.gemm_mode = opt->gemm_mode;
        o.final_energy_fp64 = opt->final_energy_fp64;
        o.lanczos_steps = opt->lanczos_steps > 0 ? opt->lanczos_steps : 1;
        o.cuda_graphs = opt->cuda_graphs;
        o.svd_warm_start = opt->svd_warm_start;
    }
    return o;
}

// The state handed to a logger callback: handles that live for the call only.
struct BorrowedMps {
    std::vector<qtt_bt> h;
    explicit BorrowedMps(const std::vector<qtt::BT> &mps) {
        for (const qtt::BT &t : mps) h.push_back(wrap(qtt::BT(t)));
    }
    ~BorrowedMps() {
        for (qtt_bt x : h) qtt_bt_destroy(x);
    }
};

int run_dmrg(int32_t L, const qtt_bt *mpo, qtt_bt *mps, int64_t *oc, const qtt_dmrg_options *opt,
             const qtt::DmrgHooks &hooks, double *E0) {
    return guarded([&] {
        out_check(oc);
        out_check(E0);
        if (L < 2) qtt::fail(qtt::ERR_INVALID_ARGUMENT, "need at least 2 sites");
        std::vector<qtt::BT> W(L), S(L);
        for (int i = 0; i < L; ++i) {
            W[i] = T(mpo[i]);
            S[i] = T(mps[i]);
        }
        *E0 = qtt::dmrg(W, S, *oc, dmrg_opts(opt), hooks);
        for (int i = 0; i < L; ++i) mps[i] = wrap(std::move(S[i]));
    });
}

struct SimpleLog {
    qtt_dmrg_log_fn fn;
    void *user;
};
struct FullLog {
    const qtt_dmrg_logger *lg;
};
}  // namespace

int qtt_dmrg(int32_t L, const qtt_bt *mpo, qtt_bt *mps, int64_t *oc, const qtt_dmrg_options *opt,
             qtt_dmrg_log_fn log_fn, void *log_user, double *E0) {
    SimpleLog sl{log_fn, log_user};
    qtt::DmrgHooks hk;
    if (log_fn) {
        hk.user = &sl;
        hk.sweep = [](void *u, int64_t it, double E, double secs, double, const std::vector<qtt::BT> &, int64_t) {
            auto *s = static_cast<SimpleLog *>(u);
            s->fn(s->user, it, E, secs);
        };
    }
    return run_dmrg(L, mpo, mps, oc, opt, hk, E0);
}

int qtt_dmrg_logged(int32_t L, const qtt_bt *mpo, qtt_bt *mps, int64_t *oc, const qtt_dmrg_options *opt,
                    const qtt_dmrg_logger *logger, double *E0) {
    FullLog fl{logger};
    qtt::DmrgHooks hk;
    if (logger) {
        if (logger->init) logger->init(logger->user, opt);
        hk.user = &fl;
        hk.sweep = [](void *u, int64_t it, double E, double secs, double trunc, const std::vector<qtt::BT> &m,
                      int64_t c) {
            const qtt_dmrg_logger *lg = static_cast<FullLog *>(u)->lg;
            if (!lg->it_log_all) return;
            BorrowedMps b(m);
            lg->it_log_all(lg->user, it, E, secs, trunc, int32_t(b.h.size()), b.h.data(), c);
        };
        hk.done = [](void *u, int64_t it, double E, const std::vector<qtt::BT> &m, int64_t c) {
            const qtt_dmrg_logger *lg = static_cast<FullLog *>(u)->lg;
            if (!lg->end_log_all) return;
            BorrowedMps b(m);
            lg->end_log_all(lg->user, it, E, int32_t(b.h.size()), b.h.data(), c);
        };
    }
    return run_dmrg(L, mpo, mps, oc, opt, hk, E0);
}

int qtt_trivial_edge(qtt_bt state, int32_t state_leg, qtt_bt mpo, int32_t mpo_leg, qtt_bt *out) {
    return guarded([&] {
        out_check(out);
        const qtt::BT &s = T(state), &w = T(mpo);
        if (state_leg < 0 || state_leg >= s.rank || mpo_leg < 0 || mpo_leg >= w.rank)
            qtt::fail(qtt::ERR_INVALID_ARGUMENT, "edge leg out of range");
        *out = wrap(qtt::trivial_edge(s, state_leg, w, mpo_leg));
    });
}

int qtt_random_mps(int32_t L, const qtt_bt *mpo, int64_t bond_dim, const int16_t *constraint, uint64_t seed,
                   qtt_bt *out) {
    return guarded([&] {
        out_check(out);
        if (L < 1) qtt::fail(qtt::ERR_INVALID_ARGUMENT, "need at least 1 site");
        std::vector<qtt::BT> W(L);
        for (int i = 0; i < L; ++i) W[i] = T(mpo[i]);
        qtt::Charge q;
        for (int i = 0; i < W[0].g.n; ++i) q.v[i] = constraint ? constraint[i] : 0;
        std::vector<qtt::BT> S = qtt::random_mps(W, bond_dim, q, seed);
        for (int i = 0; i < L; ++i) out[i] = wrap(std::move(S[i]));
    });
}

int qtt_mps_energy(int32_t L, const qtt_bt *mpo, const qtt_bt *mps, double *energy, double *norm2) {
    return guarded([&] {
        out_check(energy);
        std::vector<qtt::BT> W(L), S(L);
        for (int i = 0; i < L; ++i) {
            W[i] = T(mpo[i]);
            S[i] = T(mps[i]);
        }
        *energy = qtt::mps_energy(W, S, norm2);
    });
}

int qtt_stats_enable(int on) {
    return guarded([&] { qtt::stats_enable(on != 0); });
}
int qtt_stats_reset(void) {
    return guarded([&] { qtt::stats_reset(); });
}
int qtt_stats_get(int kind, double *ms, double *work, int64_t *launches) {
    return guarded([&] { qtt::stats_get(kind, ms, work, launches); });
}
int64_t qtt_launch_count(void) { return qtt::launch_count(); }
int qtt_last_svd_sweeps(int32_t *out, int32_t cap, int32_t *n) {
    return guarded([&] {
        auto v = qtt::last_svd_sweeps();
        if (n) *n = int32_t(v.size());
        for (int32_t i = 0; i < cap && i < int32_t(v.size()); ++i) out[i] = v[i];
    });
}
int qtt_last_svd_fp32_sweeps(int32_t *out, int32_t cap, int32_t *n) {
    return guarded([&] {
        auto v = qtt::last_svd_sweeps(true);
        if (n) *n = int32_t(v.size());
        for (int32_t i = 0; i < cap && i < int32_t(v.size()); ++i) out[i] = v[i];
    });
}

}  // extern "C"
