// Per-charge-sector SVD / eigh and truncation (sources/btensor_linalg.cpp).
//
// The host groups blocks into sectors exactly like reorder_by_cvals +
// compact_dense (:30-255) and builds the U / d / V structures of :390-502; the
// device packs every sector matrix, runs all sector decompositions in one
// cooperative Jacobi launch, and scatters the factors into the output blocks.
// Truncation (:658-755, LinearAlgebra.cpp:57-75) reads the singular values back
// once, picks the global threshold in FP64 on the host, and slices the blocks.
#include <cmath>
#include <numeric>

#include "kernels.h"
#include "ops_util.h"
#include "qtt_core.h"

namespace qtt {

namespace {

struct SecRow {
    int64_t sec, start, size;
};
struct Sector {
    std::vector<int64_t> lead;            // leading block index (rank > 2)
    std::vector<int64_t> lead_shape;      // leading block sizes
    int64_t batch = 1;                    // product of lead_shape
    std::vector<SecRow> rows, cols;       // rows in first-appearance order; cols sorted by section
    std::vector<int64_t> blocks;          // member blocks
    int64_t m = 0, n = 0;
};

// reorder_by_cvals + compact_dense(_single) (btensor_linalg.cpp:30-255)
std::vector<Sector> make_sectors(const BT &t) {
    const int r = t.rank;
    if (r < 2) fail(ERR_INVALID_ARGUMENT, "decompositions need a tensor of rank 2 or more");
    auto ad = t.addrs();
    const Charge *rowq = t.cv.data() + ad[r - 2];
    const Charge *colq = t.cv.data() + ad[r - 1];
    std::vector<int64_t> ord(t.nblocks());
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](int64_t a, int64_t b) {
        const Charge &ra = rowq[t.idx(a)[r - 2]], &rb = rowq[t.idx(b)[r - 2]];
        const Charge &ca = colq[t.idx(a)[r - 1]], &cb = colq[t.idx(b)[r - 1]];
        if (qless(ra, rb, t.g)) return true;
        return qeq(ra, rb, t.g) && qless(ca, cb, t.g);
    });
    std::vector<Sector> out;
    size_t i = 0;
    while (i < ord.size()) {
        size_t j = i + 1;
        const int64_t *k0 = t.idx(ord[i]);
        while (j < ord.size()) {
            const int64_t *k1 = t.idx(ord[j]);
            bool same = std::equal(k0, k0 + r - 2, k1) && qeq(rowq[k1[r - 2]], rowq[k0[r - 2]], t.g) &&
                        qeq(colq[k1[r - 1]], colq[k0[r - 1]], t.g);
            if (!same) break;
            ++j;
        }
        Sector s;
        s.lead.assign(k0, k0 + r - 2);
        int64_t shp[MAXRANK];
        t.block_shape(ord[i], shp);
        s.lead_shape.assign(shp, shp + r - 2);
        for (auto x : s.lead_shape) s.batch *= x;
        int64_t cur_row = k0[r - 2];
        s.rows.push_back({cur_row, 0, shp[r - 2]});
        s.m = shp[r - 2];
        for (size_t k = i; k < j; ++k) {
            const int64_t b = ord[k];
            const int64_t *ix = t.idx(b);
            t.block_shape(b, shp);
            int64_t c = ix[r - 1];
            auto pos = std::lower_bound(s.cols.begin(), s.cols.end(), c,
                                        [](const SecRow &x, int64_t v) { return x.sec < v; });
            if (pos == s.cols.end() || pos->sec != c) {
                s.cols.insert(pos, SecRow{c, s.n, shp[r - 1]});
                s.n += shp[r - 1];
            }
            if (cur_row != ix[r - 2]) {
                cur_row = ix[r - 2];
                s.rows.push_back({cur_row, s.m, shp[r - 2]});
                s.m += shp[r - 2];
            }
            s.blocks.push_back(b);
        }
        out.push_back(std::move(s));
        i = j;
    }
    return out;
}

const SecRow &find_row(const std::vector<SecRow> &v, int64_t sec) {
    for (auto &x : v)
        if (x.sec == sec) return x;
    fail(ERR_RUNTIME, "internal: section missing from sector");
}

// a structure made of t's legs `legs` (optionally with inverted charges), neutral selection rule
BT legs_of(const BT &t, const std::vector<int> &legs, bool invert, bool neutral) {
    BT o;
    o.g = t.g;
    o.dt = t.dt;
    o.rank = int(legs.size());
    auto ad = t.addrs();
    for (int d : legs) {
        o.sbd.push_back(t.sbd[d]);
        for (int64_t s = 0; s < t.sbd[d]; ++s) {
            o.ssz.push_back(t.ssz[ad[d] + s]);
            Charge q = t.cv[ad[d] + s];
            if (neutral) q = Charge{};
            if (invert) q = qinv(q, t.g);
            o.cv.push_back(q);
        }
    }
    return o;
}
BT concat(const BT &a, const BT &b) {
    BT o = a;
    o.rank = a.rank + b.rank;
    o.sbd.insert(o.sbd.end(), b.sbd.begin(), b.sbd.end());
    o.ssz.insert(o.ssz.end(), b.ssz.begin(), b.ssz.end());
    o.cv.insert(o.cv.end(), b.cv.begin(), b.cv.end());
    o.sel = qadd(a.sel, b.sel, a.g);
    o.bidx.clear();
    o.boff.clear();
    o.nnz = 0;
    return o;
}
BT single_leg(const BT &like, const std::vector<int64_t> &sizes, const std::vector<Charge> &q) {
    BT o;
    o.g = like.g;
    o.dt = like.dt;
    o.rank = 1;
    o.sbd = {int64_t(sizes.size())};
    o.ssz = sizes;
    o.cv = q;
    return o;
}

// sweep counts of the most recent decomposition (diagnostics)
struct LastSweeps {
    BufPtr buf;       // sweeps of the stage that produced the factors
    BufPtr pre;       // mixed path: sweeps of the FP32 stage
    int n = 0;
    bool mixed = false;
};
LastSweeps &last_sweeps() {
    thread_local LastSweeps l;  // per host thread, like its stream
    return l;
}

// Set by svd_truncated around the decomposition it runs: its caller keeps only the
// values the truncation selects, and the truncation never keeps a zero value
// (btensor_linalg.cpp:658-755 keeps values strictly above the smallest kept one
// less 2 eps, which is >= 0).  So null columns need no completion, and numerically
// null columns may leave the sweeps (deflation, below).
struct TruncHint {
    bool active = false;
    int64_t min_size = 0;
    WarmStart *ws = nullptr;  // warm starts of the decomposition (svd only)
    // the truncation that follows (tol, max_size, pow), for the mixed path's estimate of
    // its threshold; discard_tau receives the largest column norm that left the FP64
    // sweeps as "below the threshold" (0: none), allow_discard switches that off
    double tol = 0.0, pw = 2.0;
    int64_t max_size = 0;
    bool allow_discard = true;
    double discard_tau = 0.0;
};
TruncHint &trunc_hint() {
    thread_local TruncHint h;
    return h;
}
struct ScopedTruncHint {
    TruncHint saved;
    ScopedTruncHint(const TruncHint &h) : saved(trunc_hint()) { trunc_hint() = h; }
    ~ScopedTruncHint() { trunc_hint() = saved; }
};

// The smallest value truncate_impl keeps (btensor_linalg.cpp:658-682,
// LinearAlgebra.cpp:57-75) among `vals` sorted descending, less the 2 eps slack; -1 when
// there are none.
double kept_threshold(const std::vector<double> &sorted, double tol, double pw, int64_t min_size, int64_t max_size) {
    const int64_t n = int64_t(sorted.size());
    if (n == 0) return -1.0;
    const double toln = std::pow(tol, pw);
    int64_t last = n - 1;
    double trunc = std::pow(std::fabs(sorted[last]), pw);
    // `last_index >= min_size` compares a signed index with an unsigned size
    while (uint64_t(last) >= uint64_t(min_size)) {
        if (trunc > toln && last < max_size) break;
        --last;
        int64_t li = last < 0 ? last + n : last;  // negative indices wrap like tensor.index
        trunc += std::pow(std::fabs(sorted[li]), pw);
    }
    double smallest = sorted[last < 0 ? last + n : last];
    return smallest - 2.0 * smallest * 2.220446049250313e-16;
}
constexpr double kDeflateF32 = 1.1920928955078125e-07;  // FP32 epsilon (2^-23)
constexpr double kDeflateF64 = 8.0 * 2.220446049250313e-16;  // 8 x FP64 epsilon (2^-49)

struct Decomp {
    std::vector<Sector> secs;
    std::vector<SectorDesc> desc;  // one per (sector, batch element)
    std::vector<int64_t> first_desc;
    BufPtr work, rot, U, V, S;
    int64_t total_k = 0;
};

// Pack, Jacobi and finish every sector; mode 0 svd, 1 eigh.
void run_decomp(const BT &t, Decomp &D, int mode, int upper) {
    require_f64(t);
    const int r = t.rank;
    int64_t wtot = 0, rtot = 0, utot = 0, vtot = 0, stot = 0;
    int max_q = 0, max_p = 0, max_steps = 1;
    std::vector<int> slots(1, 0);
    for (size_t g = 0; g < D.secs.size(); ++g) {
        const Sector &s = D.secs[g];
        if (mode == 1 && s.m != s.n) fail(ERR_INVALID_ARGUMENT, "eigh needs square sectors");
        D.first_desc.push_back(int64_t(D.desc.size()));
        for (int64_t e = 0; e < s.batch; ++e) {
            SectorDesc d{};
            d.m = int32_t(s.m);
            d.n = int32_t(s.n);
            d.trans = s.m < s.n ? 1 : 0;
            d.p = int32_t(std::max(s.m, s.n));
            d.q = int32_t(std::min(s.m, s.n));
            d.mode = mode;
            d.w_off = wtot;
            d.rot_off = rtot;
            d.u_off = utot;
            d.v_off = vtot;
            d.s_off = stot;
            wtot += int64_t(d.p) * d.q;
            rtot += int64_t(d.q) * d.q;
            utot += int64_t(d.m) * d.q;
            vtot += int64_t(d.n) * d.q;
            stot += d.q;
            max_q = std::max(max_q, int(d.q));
            max_p = std::max(max_p, int(d.p));
            int qp = d.q + (d.q & 1);
            if (qp >= 2) max_steps = std::max(max_steps, qp - 1);
            slots.push_back(slots.back() + qp / 2);
            D.desc.push_back(d);
        }
    }
    D.total_k = stot;
    const int nsec = int(D.desc.size());
    // The mixed path (split-precision block GEMMs) runs its SVD sweeps in FP32 first and
    // finishes them in FP64 (svd_refine.cu): the result is an FP64 SVD either way.  eigh
    // always runs in FP64.
    const int f32 = (mode == 0 && gemm_mode() != GEMM_F64) ? 1 : 0;
    const size_t es = f32 ? 4 : 8;
    D.work = dev_alloc(size_t(std::max<int64_t>(wtot, 1)) * es);
    D.rot = dev_alloc(size_t(std::max<int64_t>(rtot, 1)) * es);
    D.U = dev_alloc(size_t(std::max<int64_t>(utot, 1)) * 8);
    D.V = dev_alloc(size_t(std::max<int64_t>(vtot, 1)) * 8);
    D.S = dev_alloc(size_t(std::max<int64_t>(stot, 1)) * 8);
    if (nsec == 0) return;
    void *W = D.work->p;
    cuda_check(cudaMemsetAsync(W, 0, size_t(wtot) * es, ctx().stream), "cudaMemsetAsync(work)");
    // pack entries: one per (block, batch element)
    std::vector<PackEntry> pe;
    std::vector<int64_t> lens;
    for (size_t g = 0; g < D.secs.size(); ++g) {
        const Sector &s = D.secs[g];
        for (int64_t b : s.blocks) {
            int64_t shp[MAXRANK];
            t.block_shape(b, shp);
            const int64_t rows = shp[r - 2], cols = shp[r - 1];
            const SecRow &rr = find_row(s.rows, t.idx(b)[r - 2]);
            const SecRow &cc = find_row(s.cols, t.idx(b)[r - 1]);
            for (int64_t e = 0; e < s.batch; ++e) {
                PackEntry x{};
                x.src_off = t.boff[b] + e * rows * cols;
                x.sector = int32_t(D.first_desc[g] + e);
                x.rows = int32_t(rows);
                x.cols = int32_t(cols);
                x.r0 = int32_t(rr.start);
                x.c0 = int32_t(cc.start);
                pe.push_back(x);
                lens.push_back(rows * cols);
            }
        }
    }
    // warm starts: a sector whose key (orientation, batch element, q-side sections) matches
    // an entry of the previous decomposition at this bond starts from that rotation; the
    // long side may differ (W V0 is defined for any number of rows)
    WarmStart *ws = mode == 0 ? trunc_hint().ws : nullptr;
    std::vector<std::vector<int64_t>> keys;
    std::vector<WarmDesc> wdesc;
    int ntiles = 0;
    if (ws) {
        for (size_t g = 0; g < D.secs.size(); ++g) {
            const Sector &s = D.secs[g];
            for (int64_t e = 0; e < s.batch; ++e) {
                SectorDesc &d = D.desc[D.first_desc[g] + e];
                std::vector<int64_t> key = {d.trans, d.q, e};
                key.insert(key.end(), s.lead.begin(), s.lead.end());
                for (const SecRow &sr : (d.trans ? s.rows : s.cols)) {
                    key.push_back(sr.sec);
                    key.push_back(sr.size);
                }
                for (const WarmStart::Entry &en : ws->entries) {
                    if (en.f32 != f32 || en.key != key || d.q < 2) continue;
                    d.warm = 1;
                    WarmDesc w{};
                    w.w_off = d.w_off;
                    w.rot_off = d.rot_off;
                    w.v0 = static_cast<const char *>(en.buf->p) + en.off * int64_t(es);
                    w.p = d.p;
                    w.q = d.q;
                    w.tile_start = ntiles;
                    ntiles += ((d.p + 63) / 64) * ((d.q + 63) / 64);
                    wdesc.push_back(w);
                    break;
                }
                keys.push_back(std::move(key));
            }
        }
    }
    SectorDesc *dsec = static_cast<SectorDesc *>(upload(D.desc.data(), D.desc.size() * sizeof(SectorDesc)));
    const int64_t packed = std::accumulate(lens.begin(), lens.end(), int64_t(0));
    const PackEntry *dpe = upload_vec(pe);
    auto chunks = make_chunks(lens);
    const Chunk *dch = upload_vec(chunks);
    {
        StatScope sc(ST_PACK, 2.0 * 8.0 * double(packed));
        launch_pack(static_cast<const double *>(t.data()), W, dpe, dch, int64_t(chunks.size()), dsec, f32);
    }
    if (mode == 1) launch_eigh_prepare(W, dsec, nsec, upper, f32);
    const int max_sweeps = 80;
    auto ibuf = dev_alloc(size_t(nsec) * (max_sweeps + 1) * sizeof(int));
    int *sweeps = static_cast<int *>(ibuf->p);
    int *flags = sweeps + nsec;
    BufPtr scratch = dev_alloc(size_t(std::max<int64_t>(wtot, 1)) * 8);
    // algorithmic work of the decomposition: the LAPACK-class SVD count per p x q sector,
    // 4 p^2 q + 8 p q^2 + 9 q^3 (eigh: 9 q^3), independent of the method
    double algo = 0;
    for (const SectorDesc &d : D.desc) {
        const double P = d.p, Q = d.q;
        algo += mode == 1 ? 9.0 * Q * Q * Q : 4.0 * P * P * Q + 8.0 * P * Q * Q + 9.0 * Q * Q * Q;
    }
    {
        StatScope sc(ST_SVD, algo);
        const size_t vb = jacobi_vwork_bytes(nsec, stot, max_steps, max_sweeps, f32);
        BufPtr vwork = dev_alloc(vb);
        // a truncation keeps only values above its (non-negative) threshold, never a
        // zero one: null columns need no completion under a truncating svd
        const int cap = (mode == 0 && trunc_hint().active) ? 0 : -1;
        // Under a truncating svd, a column whose norm falls to the working precision's
        // resolution (c eps ||W_s||_F) leaves the sweeps: numerically null columns would
        // otherwise be rotated against each other for many sweeps to no effect.  Its
        // last norm is kept as its value (below any threshold a truncation keeps).
        const bool deflate = cap == 0 && svd_deflation();
        auto deflation = [&](const void *w, int prec32, BufPtr &thr, BufPtr &dn) {
            const size_t e = prec32 ? 4 : 8;
            thr = dev_alloc(size_t(nsec) * e);
            dn = dev_alloc(size_t(std::max<int64_t>(stot, 1)) * e);
            cuda_check(cudaMemsetAsync(dn->p, 0, size_t(std::max<int64_t>(stot, 1)) * e, ctx().stream),
                       "cudaMemsetAsync(dnorm)");
            launch_deflation_thresholds(w, dsec, nsec, prec32 ? kDeflateF32 : kDeflateF64, thr->p, prec32);
        };
        BufPtr thr, dnorm;
        if (deflate) deflation(W, f32, thr, dnorm);
        if (!wdesc.empty()) {
            BufPtr tmp = dev_alloc(size_t(std::max<int64_t>(wtot, 1)) * es);
            launch_warm_apply(W, D.rot->p, tmp->p, upload_vec(wdesc), int(wdesc.size()), ntiles, f32);
        }
        const int *dslots = upload_vec(slots);
        launch_jacobi(W, D.rot->p, dsec, dslots, nsec, max_steps, max_sweeps, sweeps, flags, f32, max_p, stot,
                      vwork->p, vb, deflate ? thr->p : nullptr, deflate ? dnorm->p : nullptr);
        const void *fw = W, *fr = D.rot->p;
        BufPtr w64, w1, va, vbuf, gbuf, ibuf64;
        // The FP32 sweeps resolved every value above FP32 resolution.  When the truncation
        // that follows keeps only values above 8 eps32 ||W_s|| (its threshold estimated from
        // the FP32 column norms with truncate's own rule), the FP64 sweeps may leave the
        // columns below tau = half that threshold unresolved among themselves: they are never
        // kept, and no value above the threshold can hide among them -- a column of norm
        // >= 4 eps32 ||W_s|| carries FP32 rounding noise of at most a quarter of itself.  The
        // truncation is checked against tau all the same (svd_truncated).
        std::vector<double> discard, null2;
        std::vector<int> kept_cols;  // discard path: columns of each sector's compact restricted sweeps
        TruncHint &th = trunc_hint();
        if (f32 && deflate && th.allow_discard && th.max_size > 0) {
            BufPtr cn = dev_alloc(size_t(std::max<int64_t>(stot, 1)) * 8);
            launch_col_norms(W, dsec, nsec, max_q, static_cast<double *>(cn->p), 1);
            std::vector<double> n2(size_t(std::max<int64_t>(stot, 1)));
            cuda_check(cudaMemcpyAsync(n2.data(), cn->p, size_t(stot) * 8, cudaMemcpyDeviceToHost, ctx().stream),
                       "cudaMemcpyAsync(column norms)");
            cuda_check(cudaStreamSynchronize(ctx().stream), "cudaStreamSynchronize");
            std::vector<double> vals(n2.begin(), n2.begin() + stot);
            for (double &x : vals) x = std::sqrt(std::max(x, 0.0));
            std::sort(vals.begin(), vals.end(), std::greater<double>());
            const double t_est = kept_threshold(vals, th.tol, th.pw, th.min_size, th.max_size);
            discard.assign(nsec, 0.0);
            null2.assign(nsec, 0.0);
            double tau_max = 0.0;
            for (int i = 0; i < nsec; ++i) {
                const SectorDesc &d = D.desc[i];
                double f2 = 0.0;
                for (int j = 0; j < d.q; ++j) f2 += n2[d.s_off + j];
                null2[i] = kDeflateF64 * kDeflateF64 * f2;
                const double tau = 0.5 * t_est;
                if (t_est > 0.0 && tau > 4.0 * kDeflateF32 * std::sqrt(f2)) {
                    discard[i] = tau;
                    tau_max = std::max(tau_max, tau);
                }
            }
            if (tau_max > 0.0)
                th.discard_tau = std::max(th.discard_tau, tau_max);
            else
                discard.clear();
        }
        if (f32) {
            StatScope sc64(ST_SVD64, 0.0);
            // FP64 stage: the FP64 sector matrices, the FP32 rotations made orthogonal in
            // FP64, W1 = W V, and FP64 Jacobi sweeps from that warm start
            w64 = dev_alloc(size_t(std::max<int64_t>(wtot, 1)) * 8);
            w1 = dev_alloc(size_t(std::max<int64_t>(wtot, 1)) * 8);
            va = dev_alloc(size_t(std::max<int64_t>(rtot, 1)) * 8);
            vbuf = dev_alloc(size_t(std::max<int64_t>(rtot, 1)) * 8);
            gbuf = dev_alloc(size_t(std::max<int64_t>(rtot, 1)) * 8);
            cuda_check(cudaMemsetAsync(w64->p, 0, size_t(wtot) * 8, ctx().stream), "cudaMemsetAsync(work64)");
            launch_pack(static_cast<const double *>(t.data()), w64->p, dpe, dch, int64_t(chunks.size()), dsec, 0);
            launch_svd_refine(static_cast<const float *>(D.rot->p), static_cast<const double *>(w64->p),
                              static_cast<double *>(w1->p), static_cast<double *>(va->p),
                              static_cast<double *>(vbuf->p), static_cast<double *>(gbuf->p), D.desc);
            std::vector<SectorDesc> d64 = D.desc;
            for (SectorDesc &d : d64) d.warm = 1;
            const SectorDesc *dsec64 = upload_vec(d64);
            ibuf64 = dev_alloc(size_t(nsec) * (max_sweeps + 1) * sizeof(int));
            int *sw64 = static_cast<int *>(ibuf64->p);
            const size_t vb64 = jacobi_vwork_bytes(nsec, stot, max_steps, max_sweeps, 0);
            BufPtr vwork64 = dev_alloc(vb64);
            dsec = const_cast<SectorDesc *>(dsec64);
            BufPtr thr64;
            dnorm.reset();
            if (deflate) deflation(w1->p, 0, thr64, dnorm);
            auto fp64_sweeps = [&](int cap_sweeps, const void *thr, const void *skip) {
                launch_jacobi(w1->p, vbuf->p, dsec64, dslots, nsec, max_steps, cap_sweeps, sw64, sw64 + nsec, 0,
                              max_p, stot, vwork64->p, vb64, deflate ? thr : nullptr, deflate ? dnorm->p : nullptr,
                              skip);
            };
            if (discard.empty()) {
                fp64_sweeps(max_sweeps, thr64 ? thr64->p : nullptr, nullptr);
            } else {
                // one sweep decouples the columns (pairs of two discarded columns stay as they
                // are), then the columns below tau leave the sweeps with the null ones
                std::vector<double> skip2(nsec), thr2(nsec);
                for (int i = 0; i < nsec; ++i) {
                    skip2[i] = discard[i] * discard[i];
                    thr2[i] = std::max(null2[i], skip2[i]);
                }
                const double *dskip = static_cast<const double *>(upload(skip2.data(), skip2.size() * 8));
                fp64_sweeps(1, thr64->p, dskip);
                // The remaining sweeps run on the kept columns only (norm above the discard
                // level after the decoupling sweep), gathered into compact sector matrices
                // W_k (p x K) with a fresh rotation R (K x K): V's kept columns become V_k R
                // afterwards.  The discarded columns keep their decoupled state; they lie
                // below the truncation's threshold, which the caller checks.
                BufPtr cn = dev_alloc(size_t(std::max<int64_t>(stot, 1)) * 8);
                launch_col_norms(w1->p, dsec64, nsec, max_q, static_cast<double *>(cn->p), 0);
                std::vector<double> n2c(size_t(std::max<int64_t>(stot, 1)));
                cuda_check(cudaMemcpyAsync(n2c.data(), cn->p, size_t(stot) * 8, cudaMemcpyDeviceToHost, ctx().stream),
                           "cudaMemcpyAsync(column norms)");
                cuda_check(cudaStreamSynchronize(ctx().stream), "cudaStreamSynchronize");
                std::vector<SectorDesc> dk(nsec);
                std::vector<int> kslots(1, 0);
                std::vector<ColCopy> wgather, vgather, wscatter, vscatter, dscatter;
                std::vector<RotProduct> rp;
                int64_t kw = 0, kr = 0, kv = 0, ks = 0;
                int kmax_steps = 1;
                for (int i = 0; i < nsec; ++i) {
                    const SectorDesc &d = D.desc[i];
                    SectorDesc c{};
                    c.m = d.m;
                    c.n = d.n;
                    c.p = d.p;
                    c.w_off = kw;
                    c.rot_off = kr;
                    c.s_off = ks;
                    int k = 0;
                    for (int j = 0; j < d.q; ++j) {
                        if (!(n2c[size_t(d.s_off + j)] > thr2[i])) continue;
                        wgather.push_back({d.w_off + int64_t(j) * d.p, kw + int64_t(k) * d.p, d.p, 0});
                        vgather.push_back({d.rot_off + int64_t(j) * d.q, kv + int64_t(k) * d.q, d.q, 0});
                        wscatter.push_back({kw + int64_t(k) * d.p, d.w_off + int64_t(j) * d.p, d.p, 0});
                        vscatter.push_back({kv + int64_t(k) * d.q, d.rot_off + int64_t(j) * d.q, d.q, 0});
                        dscatter.push_back({ks + k, d.s_off + j, 1, 0});
                        ++k;
                    }
                    c.q = k;
                    kept_cols.push_back(k);
                    if (k > 0) rp.push_back({kv, kr, kv, d.q, k});
                    kw += int64_t(d.p) * k;
                    kr += int64_t(k) * k;
                    kv += int64_t(d.q) * k;
                    ks += k;
                    const int kp = k + (k & 1);
                    if (kp >= 2) kmax_steps = std::max(kmax_steps, kp - 1);
                    kslots.push_back(kslots.back() + kp / 2);
                    dk[i] = c;
                }
                BufPtr wk = dev_alloc(size_t(std::max<int64_t>(kw, 1)) * 8);
                BufPtr rk = dev_alloc(size_t(std::max<int64_t>(kr, 1)) * 8);
                BufPtr vg = dev_alloc(size_t(std::max<int64_t>(kv, 1)) * 8);
                BufPtr vn = dev_alloc(size_t(std::max<int64_t>(kv, 1)) * 8);
                launch_col_copy(static_cast<const double *>(w1->p), static_cast<double *>(wk->p), wgather);
                launch_col_copy(static_cast<const double *>(vbuf->p), static_cast<double *>(vg->p), vgather);
                const SectorDesc *ddk = upload_vec(dk);
                const int *dkslots = upload_vec(kslots);
                const size_t vbk = jacobi_vwork_bytes(nsec, ks, kmax_steps, max_sweeps, 0);
                BufPtr vworkk = dev_alloc(vbk);
                // numerically null columns (the FP64 null level of each sector) still leave the
                // sweeps; their squared norms land in a compact dnorm and go back to theirs
                BufPtr dnk;
                if (deflate) {
                    dnk = dev_alloc(size_t(std::max<int64_t>(ks, 1)) * 8);
                    cuda_check(cudaMemsetAsync(dnk->p, 0, size_t(std::max<int64_t>(ks, 1)) * 8, ctx().stream),
                               "cudaMemsetAsync(compact dnorm)");
                }
                launch_jacobi(wk->p, rk->p, ddk, dkslots, nsec, kmax_steps, max_sweeps, sw64, sw64 + nsec, 0, max_p, ks,
                              vworkk->p, vbk, deflate ? thr64->p : nullptr, deflate ? dnk->p : nullptr, nullptr);
                launch_rot_product(static_cast<const double *>(vg->p), static_cast<const double *>(rk->p),
                                   static_cast<double *>(vn->p), rp);
                launch_col_copy(static_cast<const double *>(wk->p), static_cast<double *>(w1->p), wscatter);
                launch_col_copy(static_cast<const double *>(vn->p), static_cast<double *>(vbuf->p), vscatter);
                if (deflate) launch_col_copy(static_cast<const double *>(dnk->p), static_cast<double *>(dnorm->p), dscatter);
                // the compact buffers are released in stream order after the copies above
            }
            fw = w1->p;
            fr = vbuf->p;
        }
        last_sweeps() = {f32 ? ibuf64 : ibuf, ibuf, nsec, f32 != 0};
        if (mode == 0 && stats_enabled() && !ctx().capturing) {
            // the sweeps' FLOPs, read from the sweep counters once the statistics are read
            cudaEvent_t raw = nullptr;
            cuda_check(cudaEventCreateWithFlags(&raw, cudaEventDisableTiming), "cudaEventCreate");
            cuda_check(cudaEventRecord(raw, ctx().stream), "cudaEventRecord");
            auto ev = std::shared_ptr<CUevent_st>(raw, [](cudaEvent_t e) { cudaEventDestroy(e); });
            std::vector<std::pair<double, double>> pq;
            for (const SectorDesc &d : D.desc) pq.push_back({double(d.p), double(d.q)});
            // kc (discard path): the recorded sweeps ran on kc[i] kept columns after one
            // decoupling sweep over the whole sector, and V's kept columns took one product
            auto flops = [ev, pq, nsec](const BufPtr &b, bool refine, const std::vector<int> &kc) {
                cudaEventSynchronize(ev.get());
                std::vector<int> sw(size_t(std::max(nsec, 1)), 0);
                cudaMemcpy(sw.data(), b->p, size_t(nsec) * sizeof(int), cudaMemcpyDeviceToHost);
                double f = 0.0;
                for (int i = 0; i < nsec; ++i) {
                    const double P = pq[i].first, Q = pq[i].second;
                    if (kc.empty()) {
                        f += double(sw[i]) * (6.0 * P * Q * Q + 3.0 * Q * Q * Q);
                    } else {
                        const double K = kc[size_t(i)];
                        f += 6.0 * P * Q * Q + 3.0 * Q * Q * Q;
                        f += double(sw[i]) * (6.0 * P * K * K + 3.0 * K * K * K) + 2.0 * Q * K * K;
                    }
                    if (refine) f += 8.0 * Q * Q * Q + 2.0 * P * Q * Q;
                }
                return f;
            };
            if (f32) {
                BufPtr b32 = ibuf, b64 = ibuf64;
                const std::vector<int> none, kc = kept_cols;
                stats_defer_work(ST_JAC32, [flops, b32, none] { return flops(b32, false, none); });
                stats_defer_work(ST_JAC64, [flops, b64, kc] { return flops(b64, true, kc); });
            } else {
                BufPtr b = ibuf;
                const std::vector<int> none;
                stats_defer_work(ST_JAC64, [flops, b, none] { return flops(b, false, none); });
            }
        }
        BufPtr permbuf;
        int64_t max_elems = 0;
        if (cap == 0) {
            permbuf = dev_alloc(size_t(std::max<int64_t>(stot, 1)) * sizeof(int));
            for (const SectorDesc &d : D.desc) max_elems = std::max(max_elems, int64_t(d.q) * (d.p + d.q));
        }
        launch_finish(fw, fr, static_cast<double *>(D.U->p), static_cast<double *>(D.V->p),
                      static_cast<double *>(D.S->p), dsec, nsec, max_q, static_cast<double *>(scratch->p), 0, cap,
                      dnorm ? dnorm->p : nullptr, nullptr, permbuf ? static_cast<int *>(permbuf->p) : nullptr,
                      max_elems);
        if (ws) {
            // this decomposition's rotations (of the first stage) start the next one at the same bond
            std::vector<WarmStart::Entry> next;
            for (int i = 0; i < nsec; ++i)
                next.push_back(WarmStart::Entry{std::move(keys[i]), D.rot, D.desc[i].rot_off, f32});
            ws->entries = std::move(next);
        }
        if (f32) {
            // keep the FP64 stage's buffers alive until the factors are scattered
            D.work = w1;
            D.rot = vbuf;
        }
    }
}

// Write blocks of `out` (its structure already set, offsets compact) from the
// sector factor buffer: out block = (lead..., rows of section, k columns).
void scatter_factor(BT &out, const Decomp &D, const BufPtr &src, bool rows_side_U, const std::vector<int64_t> &blk_sec,
                    const std::vector<int64_t> &blk_kcols) {
    const int r = out.rank;
    std::vector<ScatterEntry> se;
    std::vector<int64_t> lens;
    for (int64_t b = 0; b < out.nblocks(); ++b) {
        const int64_t g = blk_sec[b];
        const Sector &s = D.secs[g];
        const int64_t row_sec = out.idx(b)[r - 2];
        const SecRow &rr = find_row(rows_side_U ? s.rows : s.cols, row_sec);
        const int64_t k = blk_kcols[b];
        for (int64_t e = 0; e < s.batch; ++e) {
            const SectorDesc &d = D.desc[D.first_desc[g] + e];
            ScatterEntry x{};
            x.src_off = rows_side_U ? d.u_off : d.v_off;
            x.dst_off = out.boff[b] + e * rr.size * k;
            x.ld = rows_side_U ? d.m : d.n;
            x.r0 = int32_t(rr.start);
            x.k = int32_t(k);
            se.push_back(x);
            lens.push_back(rr.size * k);
        }
    }
    auto chunks = make_chunks(lens);
    launch_scatter(static_cast<const double *>(src->p), static_cast<double *>(out.data()), upload_vec(se),
                   upload_vec(chunks), int64_t(chunks.size()));
}

void scatter_values(BT &d, const Decomp &D, const std::vector<int64_t> &blk_sec, const std::vector<int64_t> &blk_k) {
    std::vector<ScatterEntry> se;
    std::vector<int64_t> lens;
    for (int64_t b = 0; b < d.nblocks(); ++b) {
        const Sector &s = D.secs[blk_sec[b]];
        for (int64_t e = 0; e < s.batch; ++e) {
            const SectorDesc &x = D.desc[D.first_desc[blk_sec[b]] + e];
            ScatterEntry y{};
            y.src_off = x.s_off;
            y.dst_off = d.boff[b] + e * blk_k[b];
            y.ld = 1;
            y.r0 = 0;
            y.k = int32_t(blk_k[b]);
            se.push_back(y);
            lens.push_back(blk_k[b]);
        }
    }
    auto chunks = make_chunks(lens);
    launch_scatter(static_cast<const double *>(D.S->p), static_cast<double *>(d.data()), upload_vec(se),
                   upload_vec(chunks), int64_t(chunks.size()));
}

}  // namespace

// svd(btensor, some=true), btensor_linalg.cpp:390-502
SVDOut svd(const BT &t) {
    const int r = t.rank;
    Decomp D;
    D.secs = make_sectors(t);
    const int64_t ns = int64_t(D.secs.size());
    auto ad = t.addrs();
    std::vector<int64_t> dsz(ns);
    std::vector<Charge> dq(ns), dqi(ns), neut(ns);
    for (int64_t g = 0; g < ns; ++g) {
        dsz[g] = std::min(D.secs[g].m, D.secs[g].n);
        dq[g] = t.cv[ad[r - 1] + D.secs[g].cols[0].sec];  // :411 right_D_cvals
        dqi[g] = qinv(dq[g], t.g);
    }
    std::vector<int> lead(r - 2);
    std::iota(lead.begin(), lead.end(), 0);
    std::vector<int> lead_row = lead;
    lead_row.push_back(r - 2);
    SVDOut o;
    o.U = concat(legs_of(t, lead_row, false, false), single_leg(t, dsz, dq));
    o.U.sel = t.sel;
    // V: neutral leading legs, inverted column leg, D leg with right_D charges, neutral rule
    o.V = concat(concat(legs_of(t, lead, false, true), legs_of(t, {r - 1}, true, false)), single_leg(t, dsz, dq));
    o.V.sel = Charge{};
    o.d = concat(legs_of(t, lead, false, true), single_leg(t, dsz, neut));
    o.d.sel = Charge{};
    // blocks (sorted: U (lead,row,b), V (lead,col,b), d (lead,b))
    struct B3 {
        std::vector<int64_t> idx;
        int64_t sec, k;
    };
    std::vector<B3> ub, vb, db;
    for (int64_t g = 0; g < ns; ++g) {
        const Sector &s = D.secs[g];
        for (auto &rw : s.rows) {
            auto ix = s.lead;
            ix.push_back(rw.sec);
            ix.push_back(g);
            ub.push_back({ix, g, dsz[g]});
        }
        for (auto &cl : s.cols) {
            auto ix = s.lead;
            ix.push_back(cl.sec);
            ix.push_back(g);
            vb.push_back({ix, g, dsz[g]});
        }
        auto ix = s.lead;
        ix.push_back(g);
        db.push_back({ix, g, dsz[g]});
    }
    auto fill = [](BT &T, std::vector<B3> &v, std::vector<int64_t> &sec, std::vector<int64_t> &kk) {
        std::stable_sort(v.begin(), v.end(), [&](const B3 &a, const B3 &b) { return a.idx < b.idx; });
        T.bidx.clear();
        for (auto &x : v) {
            T.bidx.insert(T.bidx.end(), x.idx.begin(), x.idx.end());
            sec.push_back(x.sec);
            kk.push_back(x.k);
        }
        T.boff.assign(v.size(), 0);
        T.compact_offsets();
    };
    std::vector<int64_t> us, uk, vs, vk, ds, dk;
    fill(o.U, ub, us, uk);
    fill(o.V, vb, vs, vk);
    fill(o.d, db, ds, dk);
    if (!t.has_data) return o;
    run_decomp(t, D, 0, 0);
    o.U.alloc_data();
    o.V.alloc_data();
    o.d.alloc_data();
    scatter_factor(o.U, D, D.U, true, us, uk);
    scatter_factor(o.V, D, D.V, false, vs, vk);
    scatter_values(o.d, D, ds, dk);
    return o;
}

// svd(A, split), btensor_linalg.cpp:503-534
std::vector<int> last_svd_sweeps(bool first_stage) {
    LastSweeps &l = last_sweeps();
    const BufPtr &src = first_stage ? (l.mixed ? l.pre : BufPtr()) : l.buf;
    std::vector<int> out(src ? l.n : 0);
    if (!out.empty()) {
        cuda_check(cudaMemcpyAsync(out.data(), src->p, size_t(l.n) * sizeof(int), cudaMemcpyDeviceToHost,
                                   ctx().stream), "cudaMemcpyAsync(sweeps)");
        cuda_check(cudaStreamSynchronize(ctx().stream), "cudaStreamSynchronize");
    }
    return out;
}

SVDOut svd_split(const BT &t, int64_t split) {
    if (split < 1 || split >= t.rank) fail(ERR_INVALID_ARGUMENT, "split must leave legs on both sides");
    BT rt = reshape(t, {split});
    SVDOut s = svd(rt);
    std::vector<int> left(split), right(t.rank - split);
    std::iota(left.begin(), left.end(), 0);
    std::iota(right.begin(), right.end(), int(split));
    BT ushape = concat(legs_of(t, left, false, false), legs_of(s.U, {1}, false, false));
    BT vshape = concat(legs_of(t, right, true, false), legs_of(s.V, {1}, false, false));
    SVDOut o;
    o.U = reshape_as(s.U, ushape);
    o.V = reshape_as(s.V, vshape);
    o.d = s.d;
    return o;
}

namespace {
// remove_unit_blocks, btensor_linalg.cpp:688-709, restated step by step on a
// list of block positions (including its handling of consecutive matches).
void remove_unit_blocks(std::vector<int64_t> &list, const BT &U, int64_t sector) {
    const int r = U.rank;
    size_t n = list.size(), src = 0, dest = 0;
    while (dest != n) {
        bool m = U.idx(list[dest])[r - 1] == sector;
        dest += m ? 1 : 0;
        if (dest != src && dest != n) std::swap(list[dest], list[src]);
        dest += (dest != n) ? 1 : 0;
        ++src;
    }
    list.resize(n - (dest - src));
}

// Materialise a truncated unitary: blocks `list` of U, the ones on `kcols`
// sectors sliced to their first k columns.
BT materialise(const BT &U, const std::vector<int64_t> &list, const std::vector<int64_t> &new_ssz_last) {
    BT o = U.shape_only();
    const int r = U.rank;
    const int64_t last = U.addr(r - 1);
    for (int64_t s = 0; s < U.sbd[r - 1]; ++s) o.ssz[last + s] = new_ssz_last[s];
    for (auto b : list) o.bidx.insert(o.bidx.end(), U.idx(b), U.idx(b) + r);
    o.boff.assign(list.size(), 0);
    o.compact_offsets();
    if (!U.has_data) return o;
    o.alloc_data();
    std::vector<PermEntry> ents(list.size());
    std::vector<int64_t> lens(list.size());
    for (size_t k = 0; k < list.size(); ++k) {
        const int64_t b = list[k];
        const int64_t kf = U.ssz[last + U.idx(b)[r - 1]];
        const int64_t kn = o.block_numel(int64_t(k));
        const int64_t rows = kf ? U.block_numel(b) / kf : 0;
        const int64_t kk = rows ? kn / rows : 0;
        PermEntry &e = ents[k];
        std::memset(&e, 0, sizeof(e));
        e.src_off = U.boff[b];
        e.dst_off = o.boff[k];
        e.rank = 2;
        e.dims[0] = rows;
        e.dims[1] = kk;
        e.stride[0] = kf;
        e.stride[1] = 1;
        lens[k] = kn;
    }
    auto chunks = make_chunks(lens);
    launch_permute(U.data(), o.data(), upload_vec(ents), upload_vec(chunks), int64_t(chunks.size()), 8);
    return o;
}
}  // namespace

// truncate_impl, btensor_linalg.cpp:658-755 and compute_last_index,
// LinearAlgebra.cpp:57-75.
SVDOut truncate(SVDOut &&in, int64_t max_size, int64_t min_size, double tol, double pw, bool has_v) {
    BT &d = in.d;
    if (d.rank != 1) fail(ERR_INVALID_ARGUMENT, "truncation needs a rank-1 value tensor");
    require_f64(d);
    // gather every value to the host in float64, in d-block order
    std::vector<double> vals(d.nnz);
    if (d.nnz) {
        cuda_check(cudaMemcpyAsync(vals.data(), d.data(), size_t(d.nnz) * 8, cudaMemcpyDeviceToHost, ctx().stream),
                   "cudaMemcpyAsync(d)");
        cuda_check(cudaStreamSynchronize(ctx().stream), "cudaStreamSynchronize");
    }
    tc_error_raise();
    std::vector<double> vd(vals.begin(), vals.end());
    // per-block value ranges in stored order
    std::vector<int64_t> bstart(d.nblocks()), blen(d.nblocks());
    for (int64_t b = 0; b < d.nblocks(); ++b) {
        bstart[b] = d.boff[b];
        blen[b] = d.block_numel(b);
    }
    std::vector<double> sorted;
    for (int64_t b = 0; b < d.nblocks(); ++b) sorted.insert(sorted.end(), vals.begin() + bstart[b], vals.begin() + bstart[b] + blen[b]);
    std::sort(sorted.begin(), sorted.end(), std::greater<double>());
    const int64_t n = int64_t(sorted.size());
    if (n == 0) return std::move(in);
    const double smallest = kept_threshold(sorted, tol, pw, min_size, max_size);
    double dropped = 0.0, total = 0.0;
    for (double v : sorted) {
        const double w = std::pow(std::fabs(v), pw);
        total += w;
        if (!(v > smallest)) dropped += w;
    }
    // walk the d blocks backwards
    BT &U = in.U;
    BT *V = has_v ? &in.V : nullptr;
    std::vector<int64_t> ulist(U.nblocks()), vlist(V ? V->nblocks() : 0), dlist(d.nblocks());
    std::iota(ulist.begin(), ulist.end(), 0);
    std::iota(vlist.begin(), vlist.end(), 0);
    std::iota(dlist.begin(), dlist.end(), 0);
    const int64_t nsec = d.sbd[0];
    std::vector<int64_t> kd(nsec), ku(U.sbd[U.rank - 1]), kv(V ? V->sbd[V->rank - 1] : 0);
    for (int64_t s = 0; s < nsec; ++s) kd[s] = d.ssz[s];
    for (int64_t s = 0; s < int64_t(ku.size()); ++s) ku[s] = U.ssz[U.addr(U.rank - 1) + s];
    for (int64_t s = 0; s < int64_t(kv.size()); ++s) kv[s] = V->ssz[V->addr(V->rank - 1) + s];
    for (int64_t pos = d.nblocks() - 1; pos >= 0; --pos) {
        const int64_t b = dlist[pos];
        const int64_t sector = d.idx(b)[0];
        int64_t k = 0;
        while (k < blen[b] && vals[bstart[b] + k] > smallest) ++k;
        if (k == 0) {
            remove_unit_blocks(ulist, U, sector);
            if (V) remove_unit_blocks(vlist, *V, sector);
            dlist.erase(dlist.begin() + pos);
        } else {
            kd[sector] = k;
            ku[ku.size() - (nsec - sector)] = k;
            if (V) kv[kv.size() - (nsec - sector)] = k;
        }
    }
    SVDOut o;
    o.U = materialise(U, ulist, ku);
    if (V) o.V = materialise(*V, vlist, kv);
    // d: same walk on a rank-1 tensor (its "rows" are a single row)
    BT dd = d.shape_only();
    for (int64_t s = 0; s < nsec; ++s) dd.ssz[s] = kd[s];
    std::sort(dlist.begin(), dlist.end());
    for (auto b : dlist) dd.bidx.push_back(d.idx(b)[0]);
    dd.boff.assign(dlist.size(), 0);
    dd.compact_offsets();
    dd.alloc_data();
    std::vector<PermEntry> ents(dlist.size());
    std::vector<int64_t> lens(dlist.size());
    for (size_t k = 0; k < dlist.size(); ++k) {
        PermEntry &e = ents[k];
        std::memset(&e, 0, sizeof(e));
        e.src_off = d.boff[dlist[k]];
        e.dst_off = dd.boff[k];
        e.rank = 1;
        e.dims[0] = dd.block_numel(int64_t(k));
        e.stride[0] = 1;
        lens[k] = e.dims[0];
    }
    auto chunks = make_chunks(lens);
    launch_permute(d.data(), dd.data(), upload_vec(ents), upload_vec(chunks), int64_t(chunks.size()), 8);
    o.d = dd;
    o.discarded = dropped;
    o.total = total;
    o.kept_min = smallest;
    return o;
}

SVDOut svd_truncated(const BT &t, int64_t split, double tol, int64_t min_size, int64_t max_size, double pw,
                     WarmStart *ws) {
    TruncHint h;
    h.active = tol > 0.0;
    h.min_size = min_size;
    h.ws = ws;
    h.tol = tol;
    h.pw = pw;
    h.max_size = max_size;
    SVDOut full;
    double tau = 0.0;
    {
        ScopedTruncHint hint(h);
        full = svd_split(t, split);
        tau = trunc_hint().discard_tau;
    }
    SVDOut out = truncate(std::move(full), max_size, min_size, tol, pw, true);
    if (tau > 0.0 && !(out.kept_min > tau)) {
        // the truncation reaches down to columns the FP64 sweeps left unresolved as
        // below its estimated threshold: decompose again, resolving every column
        h.allow_discard = false;
        ScopedTruncHint hint(h);
        full = svd_split(t, split);
        out = truncate(std::move(full), max_size, min_size, tol, pw, true);
    }
    return out;
}

// eigh(btensor, upper), btensor_linalg.cpp:294-368 (eigenvalues ascending per sector)
EighOut eigh(const BT &t, bool upper) {
    const int r = t.rank;
    Decomp D;
    D.secs = make_sectors(t);
    const int64_t ns = int64_t(D.secs.size());
    auto ad = t.addrs();
    std::vector<int64_t> dsz(ns);
    std::vector<Charge> dq(ns), neut(ns);
    for (int64_t g = 0; g < ns; ++g) {
        dsz[g] = D.secs[g].n;
        dq[g] = t.cv[ad[r - 1] + D.secs[g].cols[0].sec];
    }
    std::vector<int> lead(r - 2);
    std::iota(lead.begin(), lead.end(), 0);
    std::vector<int> lead_row = lead;
    lead_row.push_back(r - 2);
    EighOut o;
    o.U = concat(legs_of(t, lead_row, false, false), single_leg(t, dsz, dq));
    o.U.sel = t.sel;
    o.d = concat(legs_of(t, lead, false, true), single_leg(t, dsz, neut));
    o.d.sel = Charge{};
    struct B3 {
        std::vector<int64_t> idx;
        int64_t sec, k;
    };
    std::vector<B3> ub, db;
    for (int64_t g = 0; g < ns; ++g) {
        const Sector &s = D.secs[g];
        for (auto &rw : s.rows) {
            auto ix = s.lead;
            ix.push_back(rw.sec);
            ix.push_back(g);
            ub.push_back({ix, g, dsz[g]});
        }
        auto ix = s.lead;
        ix.push_back(g);
        db.push_back({ix, g, dsz[g]});
    }
    auto fill = [](BT &T, std::vector<B3> &v, std::vector<int64_t> &sec, std::vector<int64_t> &kk) {
        std::stable_sort(v.begin(), v.end(), [&](const B3 &a, const B3 &b) { return a.idx < b.idx; });
        for (auto &x : v) {
            T.bidx.insert(T.bidx.end(), x.idx.begin(), x.idx.end());
            sec.push_back(x.sec);
            kk.push_back(x.k);
        }
        T.boff.assign(v.size(), 0);
        T.compact_offsets();
    };
    std::vector<int64_t> us, uk, ds, dk;
    fill(o.U, ub, us, uk);
    fill(o.d, db, ds, dk);
    if (!t.has_data) return o;
    run_decomp(t, D, 1, upper ? 1 : 0);
    o.U.alloc_data();
    o.d.alloc_data();
    scatter_factor(o.U, D, D.U, true, us, uk);
    scatter_values(o.d, D, ds, dk);
    return o;
}

// eigh(A, split), btensor_linalg.cpp:369-389
EighOut eigh_split(const BT &t, int64_t split) {
    if (split < 1 || split >= t.rank) fail(ERR_INVALID_ARGUMENT, "split must leave legs on both sides");
    BT rt = reshape(t, {split});
    EighOut s = eigh(rt, true);
    std::vector<int> left(split);
    std::iota(left.begin(), left.end(), 0);
    BT ushape = concat(legs_of(t, left, false, false), legs_of(s.U, {1}, false, false));
    EighOut o;
    o.U = reshape_as(s.U, ushape);
    o.d = s.d;
    return o;
}

}  // namespace qtt
