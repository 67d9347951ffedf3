// Two-site DMRG on the device (sources/dmrg.cpp).
//
// The bond update keeps every Lanczos scalar on the device: the inner products
// a0, <r|r>, a1 are written by the dot kernels, b = sqrt(<r|r>) and the closed
// form 2x2 Ritz step (eig2x2Mat_impl, :544-572) run in one-thread kernels, and
// the axpby kernels read their coefficients from device memory.  The only host
// synchronisation of a bond update is the read-back of the singular values for
// the truncation threshold, which also brings back the bond energy.
#include <chrono>
#include <cmath>

#include "contract.h"
#include "dmrg.h"
#include "kernels.h"
#include "ops_util.h"
#include "qtt_core.h"

namespace qtt {

BT compute_2sites_hamil(const BT &wl, const BT &wr) {
    return permute(tensordot(wl, wr, {2}, {0}), {0, 1, 3, 4, 2, 5});
}

BT hamil2site_times_state(const BT &state, const BT &hamil, const BT &L, const BT &R) {
    BT out = tensordot(L, state, {0}, {0});
    out = tensordot(out, hamil, {0, 2, 3}, {0, 4, 5});
    return tensordot(out, R, {1, 4}, {0, 1});
}

BT compute_left_env(const BT &W, const BT &A, const BT &L) {
    BT out = tensordot(L, A, {0}, {0});
    out = tensordot(out, W, {0, 2}, {0, 3});
    return tensordot(out, conj(A), {0, 2}, {0, 1});
}

BT compute_right_env(const BT &W, const BT &A, const BT &R) {
    BT out = tensordot(R, A, {0}, {2});
    out = tensordot(out, W, {0, 3}, {2, 3});
    return tensordot(out, conj(A), {3, 0}, {1, 2});
}

void eig2x2(double a0, double a1, double b, double &E, double &o, double &n) {
    double crit = std::sqrt((a0 - a1) * (a0 - a1) + 4.0 * (b * b));
    E = (a0 + a1 - crit) / 2.0;
    double delt = E - a1;
    o = std::sqrt(delt / (-crit));
    bool zero_o = ((o + E) == E) || std::isnan(o);
    n = (b * o) / delt;
    if (zero_o) {
        n = 1.0;
        o = 0.0;
    }
    if (std::isnan(o) || std::isnan(n)) fail(ERR_LOGIC, "nan found in output tensor");
}

namespace {
// Lowest eigenpair of a small dense symmetric matrix (row-major n x n) by cyclic
// Jacobi rotations in FP64 (n is the Krylov dimension, at most a few dozen).
void small_sym_lowest(std::vector<double> A, int n, double &lam, std::vector<double> &vec) {
    std::vector<double> V(size_t(n) * n, 0.0);
    for (int i = 0; i < n; ++i) V[size_t(i) * n + i] = 1.0;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0, tot = 0.0;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                const double x = A[size_t(i) * n + j] * A[size_t(i) * n + j];
                tot += x;
                if (i != j) off += x;
            }
        if (off <= 1e-30 * tot || off == 0.0) break;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double apq = A[size_t(p) * n + q];
                if (apq == 0.0) continue;
                const double app = A[size_t(p) * n + p], aqq = A[size_t(q) * n + q];
                const double th = (aqq - app) / (2.0 * apq);
                const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int r = 0; r < n; ++r) {  // A <- A J (columns p, q)
                    const double x = A[size_t(r) * n + p], y = A[size_t(r) * n + q];
                    A[size_t(r) * n + p] = c * x - s * y;
                    A[size_t(r) * n + q] = s * x + c * y;
                }
                for (int r = 0; r < n; ++r) {  // A <- J^T A (rows p, q)
                    const double x = A[size_t(p) * n + r], y = A[size_t(q) * n + r];
                    A[size_t(p) * n + r] = c * x - s * y;
                    A[size_t(q) * n + r] = s * x + c * y;
                }
                for (int r = 0; r < n; ++r) {
                    const double x = V[size_t(r) * n + p], y = V[size_t(r) * n + q];
                    V[size_t(r) * n + p] = c * x - s * y;
                    V[size_t(r) * n + q] = s * x + c * y;
                }
            }
    }
    int best = 0;
    for (int i = 1; i < n; ++i)
        if (A[size_t(i) * n + i] < A[size_t(best) * n + best]) best = i;
    lam = A[size_t(best) * n + best];
    vec.assign(n, 0.0);
    for (int r = 0; r < n; ++r) vec[r] = V[size_t(r) * n + best];
}
bool same_layout(const BT &a, const BT &b) {
    return a.rank == b.rank && a.dt == b.dt && a.nnz == b.nnz && a.sbd == b.sbd && a.ssz == b.ssz &&
           a.bidx == b.bidx && a.boff == b.boff;
}

// t's structure in a buffer of its own, filled by a device copy of `src` (same layout)
BT copy_layout(const BT &t, const void *src) {
    BT o = t.shape_only();
    o.sel = t.sel;
    o.bidx = t.bidx;
    o.boff = t.boff;
    o.nnz = t.nnz;
    o.alloc_data();
    if (t.nnz)
        cuda_check(cudaMemcpyAsync(o.data(), src, size_t(t.nnz) * dsize(t.dt), cudaMemcpyDeviceToDevice,
                                   ctx().stream),
                   "cudaMemcpyAsync(copy)");
    return o;
}

// The two-site matvec captured once as a CUDA graph and replayed for every Krylov
// vector of the same block layout: the host planning of its three contractions
// (merge-joins, tile and split tables) and their launches are paid once per bond
// instead of once per Lanczos iteration.  The graph reads its input from X and
// writes its output into graph-owned memory (instantiated with auto-free on launch,
// so every launch reuses the same address); run() copies it out.
struct GraphedMatvec {
    cudaGraphExec_t exec = nullptr;
    BT X, Y;
    void *yptr = nullptr;
    bool launched = false;
    int64_t launches = 0;
    std::vector<void *> tables;

    bool capture(const BT &v, const BT &hamil, const BT &L, const BT &R) {
        Ctx &c = ctx();
        X = copy_layout(v, v.data());
        const int64_t l0 = launch_count();
        c.capturing = true;
        c.capture_tables = &tables;
        cudaGraph_t g = nullptr;
        bool ok = cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeRelaxed) == cudaSuccess;
        if (ok) {
            try {
                Y = hamil2site_times_state(X, hamil, L, R);
            } catch (...) {
                ok = false;
            }
            ok = (cudaStreamEndCapture(c.stream, &g) == cudaSuccess) && ok;
        }
        c.capturing = false;
        c.capture_tables = nullptr;
        if (ok) ok = cudaGraphInstantiateWithFlags(&exec, g, cudaGraphInstantiateFlagAutoFreeOnLaunch) == cudaSuccess;
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        if (!ok || !Y.has_data) {
            exec = nullptr;
            Y = BT();
            return false;
        }
        launches = launch_count() - l0;
        // Y's memory belongs to the graph: detach it from the tensor's owner
        yptr = Y.buf->p;
        Y.buf->p = nullptr;
        return true;
    }
    BT run(const BT &v) {
        Ctx &c = ctx();
        if (v.nnz)
            cuda_check(cudaMemcpyAsync(X.data(), v.data(), size_t(v.nnz) * dsize(v.dt), cudaMemcpyDeviceToDevice,
                                       c.stream),
                       "cudaMemcpyAsync(graph input)");
        cuda_check(cudaGraphLaunch(exec, c.stream), "cudaGraphLaunch");
        launched = true;
        count_launch(int(launches));
        return copy_layout(Y, yptr);
    }
    ~GraphedMatvec() {
        Ctx &c = ctx();
        if (launched && yptr) cudaFreeAsync(yptr, c.stream);
        if (exec) {
            cudaStreamSynchronize(c.stream);
            cudaGraphExecDestroy(exec);
        }
        for (void *p : tables) cudaFree(p);
    }
};
}  // namespace

// k-step Lanczos on the two-site effective Hamiltonian.  Not a QuantiT function:
// an optional replacement of its one-step update (dmrg_options lanczos_steps > 1)
// that converges a bond in one visit instead of many sweeps.  Every coefficient
// (alpha, beta, the two-pass Gram-Schmidt projections) stays a device scalar, so
// the k matvecs run without a host synchronisation; one download then feeds the
// k x k tridiagonal Ritz problem, solved on the host in FP64.  A Krylov breakdown
// (beta below 1e-13 of the largest |alpha|) truncates the Ritz problem there.
LanczosKOut lanczos_k(const BT &state, const BT &hamil, const BT &L, const BT &R, int k, bool graphs) {
    if (k < 1) fail(ERR_INVALID_ARGUMENT, "lanczos_steps must be at least 1");
    GraphedMatvec gm;
    bool graph_ok = graphs;
    DevScratch scr;
    double *a = scr.get(size_t(k)), *b = scr.get(size_t(k)), *c = scr.get(1), *n0 = scr.get(1);
    std::vector<BT> V;
    dot_all_dev(state, state, n0, scr);
    launch_sqrt(n0);
    V.push_back(scale_dev(state, Coef{1.0, n0, 1, 0, 1e-300}));
    for (int j = 0; j < k; ++j) {
        BT w;
        if (graph_ok && gm.exec && same_layout(V[j], gm.X)) {
            w = gm.run(V[j]);
        } else if (graph_ok && !gm.exec && j >= 1 && j + 1 < k && same_layout(V[j], V[j - 1])) {
            // the Krylov vectors' layout has settled: capture once, replay from here on
            if (gm.capture(V[j], hamil, L, R))
                w = gm.run(V[j]);
            else {
                graph_ok = false;
                w = hamil2site_times_state(V[j], hamil, L, R);
            }
        } else {
            w = hamil2site_times_state(V[j], hamil, L, R);
        }
        dot_all_dev(V[j], w, a + j, scr);
        w = add_scaled_dev(w, V[j], coef_host(1.0), Coef{-1.0, a + j, 0, 0, 0.0});
        if (j > 0) w = add_scaled_dev(w, V[j - 1], coef_host(1.0), Coef{-1.0, b + j - 1, 0, 0, 0.0});
        for (int pass = 0; pass < 2; ++pass)
            for (int i = 0; i <= j; ++i) {
                dot_all_dev(V[i], w, c, scr);
                w = add_scaled_dev(w, V[i], coef_host(1.0), Coef{-1.0, c, 0, 0, 0.0});
            }
        if (j + 1 == k) break;
        dot_all_dev(w, w, b + j, scr);
        launch_sqrt(b + j);
        V.push_back(scale_dev(w, Coef{1.0, b + j, 1, 0, 1e-300}));
    }
    std::vector<double> ha(k), hb(k);
    cuda_check(cudaMemcpyAsync(ha.data(), a, size_t(k) * 8, cudaMemcpyDeviceToHost, ctx().stream), "Lanczos alpha");
    if (k > 1)
        cuda_check(cudaMemcpyAsync(hb.data(), b, size_t(k - 1) * 8, cudaMemcpyDeviceToHost, ctx().stream),
                   "Lanczos beta");
    cuda_check(cudaStreamSynchronize(ctx().stream), "cudaStreamSynchronize");
    double scale = 0.0;
    for (int j = 0; j < k; ++j) {
        if (std::isnan(ha[j]) || (j + 1 < k && std::isnan(hb[j]))) fail(ERR_LOGIC, "nan found in output tensor");
        scale = std::max(scale, std::fabs(ha[j]));
    }
    int m = k;
    for (int j = 0; j + 1 < k; ++j)
        if (!(hb[j] > 1e-13 * std::max(scale, 1e-300))) {
            m = j + 1;
            break;
        }
    std::vector<double> T(size_t(m) * m, 0.0);
    for (int j = 0; j < m; ++j) {
        T[size_t(j) * m + j] = ha[j];
        if (j + 1 < m) T[size_t(j) * m + j + 1] = T[size_t(j + 1) * m + j] = hb[j];
    }
    LanczosKOut o;
    std::vector<double> y;
    small_sym_lowest(T, m, o.E, y);
    o.psi = scale_dev(V[0], coef_host(y[0]));
    for (int j = 1; j < m; ++j) o.psi = add_scaled_dev(o.psi, V[j], coef_host(1.0), coef_host(y[j]));
    o.dim = m;
    return o;
}

// scal layout: [0] a0, [1] b, [2] a1, [3] E, [4] o, [5] n, [6] nan flag
LanczosOut one_step_lanczos_dev(const BT &state, const BT &hamil, const BT &L, const BT &R, double *scal,
                                DevScratch &scr) {
    BT psi = hamil2site_times_state(state, hamil, L, R);
    dot_all_dev(psi, state, scal + 0, scr);
    psi = add_scaled_dev(psi, state, coef_host(1.0), Coef{-1.0, scal + 0, 0, 0, 0.0});
    dot_all_dev(psi, psi, scal + 1, scr);
    launch_sqrt(scal + 1);
    psi = scale_dev(psi, Coef{1.0, scal + 1, 1, 0, 1e-15});
    BT hpsi = hamil2site_times_state(psi, hamil, L, R);
    dot_all_dev(psi, hpsi, scal + 2, scr);
    LanczosOut o;
    o.psi = psi;
    return o;
}

LanczosHost one_step_lanczos(const BT &state, const BT &hamil, const BT &L, const BT &R) {
    DevScratch scr;
    double *scal = scr.get(8);
    LanczosOut r = one_step_lanczos_dev(state, hamil, L, R, scal, scr);
    double h[3];
    cuda_check(cudaMemcpyAsync(h, scal, 3 * sizeof(double), cudaMemcpyDeviceToHost, ctx().stream), "cudaMemcpyAsync");
    cuda_check(cudaStreamSynchronize(ctx().stream), "cudaStreamSynchronize");
    LanczosHost o;
    o.psi = r.psi;
    o.a0 = h[0];
    o.b = h[1];
    o.a1 = h[2];
    return o;
}

BT trivial_edge(const BT &st, int sleg, const BT &w, int wleg) {
    // all-ones rank-3 edge (generate_env_impl, dmrg.cpp:371-391; edge_shape_prep :335-345)
    BT e;
    e.g = st.g;
    e.dt = F64;
    e.rank = 3;
    auto adS = st.addrs(), adW = w.addrs();
    auto add_leg = [&](const BT &t, const std::vector<int64_t> &ad, int leg, bool inv) {
        e.sbd.push_back(t.sbd[leg]);
        for (int64_t s = 0; s < t.sbd[leg]; ++s) {
            e.ssz.push_back(t.ssz[ad[leg] + s]);
            Charge q = t.cv[ad[leg] + s];
            e.cv.push_back(inv ? qinv(q, t.g) : q);
        }
    };
    add_leg(st, adS, sleg, true);
    add_leg(w, adW, wleg, true);
    add_leg(st, adS, sleg, false);
    Charge q;
    for (auto &c : e.cv) q = qadd(q, c, e.g);
    e.sel = q;
    std::vector<int64_t> idx;
    for (int64_t a = 0; a < e.sbd[0]; ++a)
        for (int64_t b = 0; b < e.sbd[1]; ++b)
            for (int64_t c = 0; c < e.sbd[2]; ++c) {
                int64_t ix[3] = {a, e.sbd[0] + b, e.sbd[0] + e.sbd[1] + c};
                Charge s = qadd(qadd(e.cv[ix[0]], e.cv[ix[1]], e.g), e.cv[ix[2]], e.g);
                if (qeq(s, e.sel, e.g)) {
                    idx.push_back(a);
                    idx.push_back(b);
                    idx.push_back(c);
                }
            }
    set_blocks(e, int64_t(idx.size() / 3), idx.data(), true, nullptr, false);
    // ones
    std::vector<double> ones(e.nnz, 1.0);
    if (e.nnz) {
        cuda_check(cudaMemcpyAsync(e.data(), ones.data(), ones.size() * 8, cudaMemcpyHostToDevice, ctx().stream),
                   "cudaMemcpyAsync(edge)");
        cuda_check(cudaStreamSynchronize(ctx().stream), "cudaStreamSynchronize");
    }
    return e;
}

namespace {
double sum_all(const BT &t) {
    if (t.nnz == 0) return 0.0;
    std::vector<double> h(t.nnz);
    cuda_check(cudaMemcpyAsync(h.data(), t.data(), size_t(t.nnz) * 8, cudaMemcpyDeviceToHost, ctx().stream),
               "cudaMemcpyAsync(scalar)");
    cuda_check(cudaStreamSynchronize(ctx().stream), "cudaStreamSynchronize");
    double s = 0.0;
    for (double x : h) s += x;
    return s;
}
}  // namespace

// <psi|H|psi> and <psi|psi> by contracting the chain from the left in FP64
// (contract(bMPS, bMPS, bMPO) and contract(bMPS, bMPS), sources/MPT.cpp:211-290).
double mps_energy(const std::vector<BT> &mpo, const std::vector<BT> &mps, double *norm2) {
    const int64_t L = int64_t(mpo.size());
    if (L < 1 || int64_t(mps.size()) != L) fail(ERR_INVALID_ARGUMENT, "MPO and MPS need the same length");
    ScopedGemmMode guard(GEMM_F64);
    BT env = trivial_edge(mps[0], 0, mpo[0], 0);
    for (int64_t i = 0; i < L; ++i) env = compute_left_env(mpo[i], mps[i], env);
    const double e = sum_all(env);
    BT n = tensordot(mps[0], conj(mps[0]), {0, 1}, {0, 1});
    for (int64_t i = 1; i < L; ++i) n = tensordot(tensordot(n, mps[i], {0}, {0}), conj(mps[i]), {0, 1}, {0, 1});
    const double nn = sum_all(n);
    if (norm2) *norm2 = nn;
    return e;
}

double dmrg(const std::vector<BT> &mpo, std::vector<BT> &mps, int64_t &oc_io, const DmrgOpts &opt,
            const DmrgHooks &hooks) {
    const int64_t L = int64_t(mpo.size());
    if (L < 2 || int64_t(mps.size()) != L) fail(ERR_INVALID_ARGUMENT, "MPO and MPS need the same length >= 2");
    ScopedGemmMode guard(opt.gemm_mode);
    // compute_2sitesHamil (dmrg.cpp:504-515)
    std::vector<BT> h2(L - 1);
    for (int64_t i = 0; i < L - 1; ++i) h2[i] = compute_2sites_hamil(mpo[i], mpo[i + 1]);
    // generate_env (dmrg.cpp:371-409); env[i+1] holds Env[i]
    int64_t oc = oc_io;
    std::vector<BT> env(L + 2);
    // per bond: the sector rotations of its last decomposition in this call (warm starts)
    std::vector<WarmStart> warm(opt.svd_warm_start ? size_t(std::max<int64_t>(L, 1)) : 0);
    env[0] = trivial_edge(mps[0], 0, mpo[0], 0);
    env[L + 1] = trivial_edge(mps[L - 1], 2, mpo[L - 1], 2);
    for (int64_t i = 0; i < oc; ++i) env[i + 1] = compute_left_env(mpo[i], mps[i], env[i]);
    for (int64_t i = L - 1; i > oc; --i) env[i + 1] = compute_right_env(mpo[i], mps[i], env[i + 2]);
    // dmrg_impl (dmrg.cpp:219-273)
    double E0 = 100000.0;
    const bool fp64_energy = opt.gemm_mode != GEMM_F64 && opt.final_energy_fp64;
    bool last_fp64 = false;  // E0 is the FP64 energy of the current state
    int64_t init_pos = oc;
    const int64_t nh = L - 1;
    const int64_t n_step = nh - 1 + (nh == 1);
    int step = (oc == 0) ? 1 : -1;
    if (nh == 1) step = 0;
    if (oc == L - 1) {
        --init_pos;
        --oc;
    }
    double *hscal = nullptr;
    cuda_check(cudaMallocHost(&hscal, 8 * sizeof(double)), "cudaMallocHost");
    struct HostFree {
        double *p;
        ~HostFree() { cudaFreeHost(p); }
    } hf{hscal};
    int64_t it = 0;
    for (; it < opt.maximum_iterations; ++it) {
        auto t0 = std::chrono::steady_clock::now();
        double E = 0.0;
        double trunc = 0.0;  // the sweep's largest relative discarded weight
        for (int64_t k = 0; k < 2 * n_step; ++k) {
            const bool forward = step == 1;
            DevScratch scr;
            double *scal = scr.get(8);
            BT theta = tensordot(mps[oc], mps[oc + 1], {2}, {0});
            BT upd;
            if (opt.lanczos_steps > 1) {
                LanczosKOut lk = lanczos_k(theta, h2[oc], env[oc], env[oc + 3], opt.lanczos_steps, opt.cuda_graphs != 0);
                upd = lk.psi;
                hscal[3] = lk.E;
                hscal[6] = 0.0;
            } else {
                LanczosOut lz = one_step_lanczos_dev(theta, h2[oc], env[oc], env[oc + 3], scal, scr);
                launch_eig2x2(scal);
                upd = add_scaled_dev(theta, lz.psi, Coef{1.0, scal + 4, 0, 0, 0.0}, Coef{1.0, scal + 5, 0, 0, 0.0});
                cuda_check(cudaMemcpyAsync(hscal, scal, 7 * sizeof(double), cudaMemcpyDeviceToHost, ctx().stream),
                           "cudaMemcpyAsync(scalars)");
            }
            SVDOut f = svd_truncated(upd, 2, opt.cutoff, opt.minimum_bond, opt.maximum_bond, 2.0,
                                     warm.empty() ? nullptr : &warm[size_t(oc)]);  // syncs
            if (hscal[6] != 0.0) fail(ERR_LOGIC, "nan found in output tensor");
            E = hscal[3];
            if (f.total > 0.0) trunc = std::max(trunc, f.discarded / f.total);
            // d /= sqrt(sum(d.pow(2)))  (dmrg.cpp:188)
            launch_normalize(static_cast<double *>(f.d.data()), f.d.nnz, nullptr);
            if (forward) {
                mps[oc] = f.U;
                mps[oc + 1] = permute(conj(mul_lastleg(f.V, f.d)), {2, 0, 1});
                env[oc + 1] = compute_left_env(mpo[oc], mps[oc], env[oc]);
            } else {
                mps[oc] = mul_lastleg(f.U, f.d);
                mps[oc + 1] = permute(conj(f.V), {2, 0, 1});
                env[oc + 2] = compute_right_env(mpo[oc + 1], mps[oc + 1], env[oc + 3]);
            }
            oc += step;
            if (oc == 0 || oc == L - 2) step = -step;
        }
        cuda_check(cudaStreamSynchronize(ctx().stream), "cudaStreamSynchronize");
        tc_error_raise();
        double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (!(fp64_energy && opt.convergence_criterion > 0.0)) {
            if (hooks.sweep) hooks.sweep(hooks.user, it, E, secs, trunc, mps, oc);
            double prev = E0;
            E0 = E;
            if (!(std::fabs((E0 - prev) / E0) > opt.convergence_criterion)) break;
            continue;
        }
        // Mixed path with a criterion: its Ritz values carry the error of the FP32
        // tensor-core accumulation (1e-7 .. 1e-4 relative, growing with the bond dimension
        // and along the chain of environment updates), under which a tight relative
        // criterion never fires; the criterion is tested on the FP64 energy of every
        // sweep's state (a contraction of the whole network in FP64).
        {
            double n2 = 1.0;
            const double e = mps_energy(mpo, mps, &n2);
            E = e / n2;
        }
        last_fp64 = true;
        if (hooks.sweep) hooks.sweep(hooks.user, it, E, secs, trunc, mps, oc);
        const double prev = E0;
        E0 = E;
        if (!(std::fabs((E0 - prev) / E0) > opt.convergence_criterion)) break;
    }
    // `it`: the sweep that met the criterion, or maximum_iterations (dmrg.cpp:238-270)
    if (oc != init_pos) {
        if (oc != init_pos - 1 && init_pos != L - 1)
            fail(ERR_RUNTIME, "the orthogonality center finished somewhere surprising! final oc: " +
                                  std::to_string(oc) + ". original oc: " + std::to_string(init_pos));
    }
    oc_io = oc;
    if (fp64_energy && !last_fp64) {
        // the mixed path's Ritz values carry the FP32-level noise of its block
        // GEMMs; the variational energy of its final state, reduced in FP64, does not
        double n2 = 1.0;
        const double e = mps_energy(mpo, mps, &n2);
        E0 = e / n2;
    }
    if (hooks.done) hooks.done(hooks.user, it, E0, mps, oc_io);
    return E0;
}

}  // namespace qtt
