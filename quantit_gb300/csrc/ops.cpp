// Structure operations (permute, reshape, reshape_as, conj) and the blockwise
// algebra (a*x + b*y over the union of blocks, full inner products, broadcast
// products on the last leg).  The planning runs on the host tables; every data
// movement is one kernel launch over all blocks.
#include <numeric>

#include "kernels.h"
#include "ops_util.h"
#include "qtt_core.h"

namespace qtt {

// ---------------------------------------------------------------- permute
// btensor::permute, sources/btensor.cpp:1754-1804: the block index, the section
// tables and the block data are permuted; the block list is re-sorted.
BT permute(const BT &t, const std::vector<int64_t> &perm_in) {
    const int r = t.rank;
    if (int(perm_in.size()) != r) fail(ERR_INVALID_ARGUMENT, "permutation length differs from the rank");
    std::vector<int64_t> perm(r);
    std::vector<char> seen(r, 0);
    for (int i = 0; i < r; ++i) {
        int64_t p = perm_in[i] < 0 ? perm_in[i] + r : perm_in[i];
        if (p < 0 || p >= r || seen[p]) fail(ERR_INVALID_ARGUMENT, "invalid permutation");
        seen[p] = 1;
        perm[i] = p;
    }
    BT o = t.shape_only();
    auto ad = t.addrs();
    o.ssz.clear();
    o.cv.clear();
    for (int i = 0; i < r; ++i) {
        int64_t p = perm[i];
        o.sbd[i] = t.sbd[p];
        for (int64_t s = 0; s < t.sbd[p]; ++s) {
            o.ssz.push_back(t.ssz[ad[p] + s]);
            o.cv.push_back(t.cv[ad[p] + s]);
        }
    }
    const int64_t nb = t.nblocks();
    o.bidx.resize(nb * r);
    for (int64_t b = 0; b < nb; ++b)
        for (int i = 0; i < r; ++i) o.bidx[b * r + i] = t.idx(b)[perm[i]];
    // sort, remembering where each output block comes from
    std::vector<int64_t> ord(nb);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](int64_t a, int64_t b) {
        return idx_less(o.bidx.data() + a * r, o.bidx.data() + b * r, r);
    });
    std::vector<int64_t> sorted(nb * r);
    for (int64_t k = 0; k < nb; ++k)
        std::copy(o.bidx.begin() + ord[k] * r, o.bidx.begin() + (ord[k] + 1) * r, sorted.begin() + k * r);
    o.bidx.swap(sorted);
    o.boff.assign(nb, 0);
    o.compact_offsets();
    if (!t.has_data) return o;
    o.alloc_data();
    std::vector<PermEntry> ents(nb);
    std::vector<int64_t> lens(nb);
    for (int64_t k = 0; k < nb; ++k) {
        const int64_t b = ord[k];
        int64_t shp[MAXRANK], str[MAXRANK];
        t.block_shape(b, shp);
        int64_t s = 1;
        for (int d = r - 1; d >= 0; --d) {
            str[d] = s;
            s *= shp[d];
        }
        PermEntry &e = ents[k];
        std::memset(&e, 0, sizeof(e));
        e.src_off = t.boff[b];
        e.dst_off = o.boff[k];
        e.rank = r;
        for (int i = 0; i < r; ++i) {
            e.dims[i] = shp[perm[i]];
            e.stride[i] = str[perm[i]];
        }
        lens[k] = t.block_numel(b);
    }
    auto chunks = make_chunks(lens);
    StatScope sc(ST_PERMUTE, 2.0 * double(t.nnz) * double(dsize(t.dt)));
    launch_permute(t.data(), o.data(), upload_vec(ents), upload_vec(chunks), int64_t(chunks.size()),
                   int(dsize(t.dt)));
    return o;
}

// ---------------------------------------------------------------- reshape
// btensor::reshape(index_groups), sources/btensor.cpp:2986-3026 with
// reshape_helpers (:2762-2985).  New sections are the right-major Cartesian
// product of the grouped legs' sections (charges combined, sizes multiplied).
// Row-major block data needs no movement: the result shares the buffer.
BT reshape(const BT &t, const std::vector<int64_t> &groups) {
    const int r = t.rank;
    std::vector<int64_t> m;
    m.push_back(0);
    for (auto gidx : groups) m.push_back(gidx);
    m.push_back(r);
    for (size_t i = 1; i < m.size(); ++i)
        if (m[i] < m[i - 1] || m[i] > r) fail(ERR_INVALID_ARGUMENT, "index groups must be increasing and within the rank");
    const int orank = int(m.size()) - 1;
    if (orank > MAXRANK) fail(ERR_INVALID_ARGUMENT, "rank too large");
    auto ad = t.addrs();
    BT o;
    o.g = t.g;
    o.rank = orank;
    o.sel = t.sel;
    o.dt = t.dt;
    o.sbd.resize(orank);
    for (int gi = 0; gi < orank; ++gi) {
        int64_t n = 1;
        for (int64_t d = m[gi]; d < m[gi + 1]; ++d) n *= t.sbd[d];
        o.sbd[gi] = n;
        // enumerate combos right-major (last leg fastest)
        std::vector<int64_t> j(m[gi + 1] - m[gi], 0);
        for (int64_t c = 0; c < n; ++c) {
            int64_t sz = 1;
            Charge q;
            for (size_t k = 0; k < j.size(); ++k) {
                int64_t d = m[gi] + int64_t(k);
                sz *= t.ssz[ad[d] + j[k]];
                q = qadd(q, t.cv[ad[d] + j[k]], t.g);
            }
            o.ssz.push_back(sz);
            o.cv.push_back(q);
            for (int64_t k = int64_t(j.size()) - 1; k >= 0; --k) {
                if (++j[k] < t.sbd[m[gi] + k]) break;
                j[k] = 0;
            }
        }
    }
    const int64_t nb = t.nblocks();
    o.bidx.resize(nb * orank);
    for (int64_t b = 0; b < nb; ++b) {
        const int64_t *ix = t.idx(b);
        for (int gi = 0; gi < orank; ++gi) {
            int64_t f = 0;
            for (int64_t d = m[gi]; d < m[gi + 1]; ++d) f = f * t.sbd[d] + ix[d];
            o.bidx[b * orank + gi] = f;
        }
    }
    o.boff = t.boff;
    o.nnz = t.nnz;
    o.buf = t.buf;
    o.has_data = t.has_data;
    return o;
}

namespace {
int64_t flat_index(const int64_t *ix, const std::vector<int64_t> &sbd) {
    int64_t f = 0;
    for (size_t d = 0; d < sbd.size(); ++d) f = f * sbd[d] + ix[d];
    return f;
}
void unflat_index(int64_t f, const std::vector<int64_t> &sbd, int64_t *out) {
    for (int64_t d = int64_t(sbd.size()) - 1; d >= 0; --d) {
        out[d] = f % sbd[d];
        f /= sbd[d];
    }
}
}  // namespace

// btensor::reshape_as<dims_only>, sources/btensor.cpp:3027-3087
BT reshape_as(const BT &t, const BT &shape) {
    int64_t n1 = 1, n2 = 1;
    for (auto s : t.sbd) n1 *= s;
    for (auto s : shape.sbd) n2 *= s;
    if (n1 != n2) fail(ERR_INVALID_ARGUMENT, "incompatible sections layouts");
    // compatible_c_vals and compatible_block_size over every block position
    // (:2876-2934).  Both layouts flatten right-major, so wherever their leading
    // section counts have equal products the flat index splits into independent
    // groups of legs.  Per position, charge(t) - charge(shape) and size(t) / size(shape)
    // are then sums / products of per-group terms; they vanish / equal one at every
    // position exactly when each group's term is constant over the group's positions
    // and the constants cancel.  Checking that visits sum-of-groups positions instead
    // of every position (millions for a sector-rich factor).
    if (n1 > 0) {
        auto adt = t.addrs(), ads = shape.addrs();
        bool zero_size = false;
        for (auto x : t.ssz) zero_size |= x == 0;
        for (auto x : shape.ssz) zero_size |= x == 0;
        Charge dsum{};
        __int128 num = 1, den = 1;
        int k = 0, l = 0;
        while (k < t.rank || l < shape.rank) {
            const int k0 = k, l0 = l;
            int64_t pt = 1, ps = 1;
            do {  // extend the group until the two section-count products meet
                if ((pt <= ps && k < t.rank) || l >= shape.rank)
                    pt *= t.sbd[k++];
                else
                    ps *= shape.sbd[l++];
            } while (pt != ps && (k < t.rank || l < shape.rank));
            if (pt != ps) fail(ERR_INVALID_ARGUMENT, "incompatible sections layouts");
            std::vector<int64_t> jt(k - k0), js(l - l0);
            Charge d0{};
            int64_t t0 = 1, s0 = 1;
            for (int64_t f = 0; f < pt; ++f) {
                int64_t rem = f;
                for (int d = k - 1; d >= k0; --d) {
                    jt[d - k0] = rem % t.sbd[d];
                    rem /= t.sbd[d];
                }
                rem = f;
                for (int d = l - 1; d >= l0; --d) {
                    js[d - l0] = rem % shape.sbd[d];
                    rem /= shape.sbd[d];
                }
                Charge ct{}, cs{};
                int64_t st = 1, ss = 1;
                for (int d = k0; d < k; ++d) {
                    ct = qadd(ct, t.cv[adt[d] + jt[d - k0]], t.g);
                    st *= t.ssz[adt[d] + jt[d - k0]];
                }
                for (int d = l0; d < l; ++d) {
                    cs = qadd(cs, shape.cv[ads[d] + js[d - l0]], t.g);
                    ss *= shape.ssz[ads[d] + js[d - l0]];
                }
                const Charge dq = qadd(ct, qinv(cs, t.g), t.g);
                if (f == 0) {
                    d0 = dq;
                    t0 = st;
                    s0 = ss;
                } else {
                    if (!qeq(dq, d0, t.g)) fail(ERR_INVALID_ARGUMENT, "incompatible conserved quantities");
                    if (!zero_size && __int128(st) * s0 != __int128(ss) * t0)
                        fail(ERR_INVALID_ARGUMENT, "incompatible block dimensions");
                }
            }
            dsum = qadd(dsum, d0, t.g);
            num *= t0;
            den *= s0;
        }
        if (!qeq(dsum, Charge{}, t.g)) fail(ERR_INVALID_ARGUMENT, "incompatible conserved quantities");
        if (zero_size) {
            // degenerate empty sections: the per-position product test, as stated
            std::vector<int64_t> ia(std::max(t.rank, 1)), ib(std::max(shape.rank, 1));
            for (int64_t f = 0; f < n1; ++f) {
                unflat_index(f, t.sbd, ia.data());
                unflat_index(f, shape.sbd, ib.data());
                int64_t s1 = 1, s2 = 1;
                for (int d = 0; d < t.rank; ++d) s1 *= t.ssz[adt[d] + ia[d]];
                for (int d = 0; d < shape.rank; ++d) s2 *= shape.ssz[ads[d] + ib[d]];
                if (s1 != s2) fail(ERR_INVALID_ARGUMENT, "incompatible block dimensions");
            }
        } else if (num != den) {
            fail(ERR_INVALID_ARGUMENT, "incompatible block dimensions");
        }
    }
    BT o = shape.shape_only();
    o.sel = t.sel;
    o.dt = t.dt;
    const int64_t nb = t.nblocks();
    o.bidx.resize(nb * o.rank);
    for (int64_t b = 0; b < nb; ++b) unflat_index(flat_index(t.idx(b), t.sbd), o.sbd, o.bidx.data() + b * o.rank);
    o.boff = t.boff;
    o.nnz = t.nnz;
    o.buf = t.buf;
    o.has_data = t.has_data;
    return o;
}

// inverse_cvals_, sources/btensor.cpp:2163-2172 (shares the data)
BT inverse_cvals(const BT &t) {
    BT o = t;
    for (auto &q : o.cv) q = qinv(q, t.g);
    o.sel = qinv(t.sel, t.g);
    return o;
}
// btensor::conj = conj_only().inverse_cvals_() (sources/btensor.cpp:2156); real data
BT conj(const BT &t) { return inverse_cvals(t); }

// ---------------------------------------------------------------- algebra
bool same_shape(const BT &a, const BT &b) {
    if (!(a.g == b.g) || a.rank != b.rank || a.sbd != b.sbd || a.ssz != b.ssz) return false;
    for (size_t i = 0; i < a.cv.size(); ++i)
        if (!qeq(a.cv[i], b.cv[i], a.g)) return false;
    return qeq(a.sel, b.sel, a.g);
}

std::vector<int64_t> sorted_order(const BT &t) {
    std::vector<int64_t> ord(t.nblocks());
    std::iota(ord.begin(), ord.end(), 0);
    const int r = t.rank;
    std::stable_sort(ord.begin(), ord.end(), [&](int64_t a, int64_t b) { return idx_less(t.idx(a), t.idx(b), r); });
    return ord;
}

UnionPlan union_plan(const BT &a, const BT &b) {
    UnionPlan u;
    auto oa = sorted_order(a), ob = sorted_order(b);
    const int r = a.rank;
    size_t i = 0, j = 0;
    while (i < oa.size() || j < ob.size()) {
        int64_t ba = i < oa.size() ? oa[i] : -1, bb = j < ob.size() ? ob[j] : -1;
        int which;  // 0 both, 1 a only, 2 b only
        if (ba < 0)
            which = 2;
        else if (bb < 0)
            which = 1;
        else if (idx_less(a.idx(ba), b.idx(bb), r))
            which = 1;
        else if (idx_less(b.idx(bb), a.idx(ba), r))
            which = 2;
        else
            which = 0;
        const int64_t *ix = which == 2 ? b.idx(bb) : a.idx(ba);
        u.idx.insert(u.idx.end(), ix, ix + r);
        u.a.push_back(which == 2 ? -1 : ba);
        u.b.push_back(which == 1 ? -1 : bb);
        if (which != 2) ++i;
        if (which != 1) ++j;
    }
    return u;
}

namespace {
BT axpby_impl(const BT &a, const BT &b, Coef ca, Coef cb) {
    if (!same_shape(a, b)) fail(ERR_INVALID_ARGUMENT, "incompatible btensors for addition");
    auto u = union_plan(a, b);
    BT o = a.shape_only();
    o.bidx = u.idx;
    o.boff.assign(u.a.size(), 0);
    o.compact_offsets();
    if (!a.has_data && !b.has_data) return o;
    if (a.nblocks() && !a.has_data) a.data();
    if (b.nblocks() && !b.has_data) b.data();
    o.alloc_data();
    std::vector<AxpbySeg> segs(u.a.size());
    std::vector<int64_t> lens(u.a.size());
    for (size_t k = 0; k < u.a.size(); ++k) {
        segs[k].a_off = u.a[k] >= 0 ? a.boff[u.a[k]] : -1;
        segs[k].b_off = u.b[k] >= 0 ? b.boff[u.b[k]] : -1;
        segs[k].out_off = o.boff[k];
        lens[k] = o.block_numel(int64_t(k));
    }
    auto chunks = make_chunks(lens);
    StatScope sc(ST_ELEMWISE, 3.0 * double(o.nnz) * 8.0);
    launch_axpby(a.has_data ? static_cast<const double *>(a.data()) : nullptr,
                 b.has_data ? static_cast<const double *>(b.data()) : nullptr, static_cast<double *>(o.data()),
                 upload_vec(segs), upload_vec(chunks), int64_t(chunks.size()), ca, cb);
    return o;
}
}  // namespace

BT add_scaled(const BT &a, const BT &b, double ca, double cb) {
    require_f64(a);
    require_f64(b);
    return axpby_impl(a, b, coef_host(ca), coef_host(cb));
}
BT add_scaled_dev(const BT &a, const BT &b, Coef ca, Coef cb) {
    require_f64(a);
    require_f64(b);
    return axpby_impl(a, b, ca, cb);
}

BT scale(const BT &a, double c) { return scale_dev(a, coef_host(c)); }
BT scale_dev(const BT &a, Coef c) {
    require_f64(a);
    BT o = a.shape_only();
    o.bidx = a.bidx;
    o.boff.assign(a.nblocks(), 0);
    o.compact_offsets();
    if (!a.has_data) return o;
    o.alloc_data();
    std::vector<AxpbySeg> segs(a.nblocks());
    std::vector<int64_t> lens(a.nblocks());
    for (int64_t k = 0; k < a.nblocks(); ++k) {
        segs[k] = AxpbySeg{a.boff[k], -1, o.boff[k]};
        lens[k] = a.block_numel(k);
    }
    auto chunks = make_chunks(lens);
    StatScope sc(ST_ELEMWISE, 2.0 * double(o.nnz) * 8.0);
    launch_axpby(static_cast<const double *>(a.data()), nullptr, static_cast<double *>(o.data()), upload_vec(segs),
                 upload_vec(chunks), int64_t(chunks.size()), c, coef_host(0.0));
    return o;
}

void dot_all_dev(const BT &a, const BT &b, double *dev_out, DevScratch &scr) {
    require_f64(a);
    require_f64(b);
    if (!(a.g == b.g) || a.rank != b.rank || a.sbd != b.sbd || a.ssz != b.ssz)
        fail(ERR_CHECK, "full contraction needs tensors of the same shape");
    for (size_t i = 0; i < a.cv.size(); ++i)
        if (!qeq(a.cv[i], b.cv[i], a.g))
            fail(ERR_CHECK, "contracted conserved numbers need to sum to zero (conjugate) on every leg");
    auto u = union_plan(a, b);
    std::vector<DotSeg> segs;
    std::vector<int64_t> lens;
    for (size_t k = 0; k < u.a.size(); ++k) {
        if (u.a[k] < 0 || u.b[k] < 0) continue;
        segs.push_back(DotSeg{a.boff[u.a[k]], b.boff[u.b[k]]});
        lens.push_back(a.block_numel(u.a[k]));
    }
    auto chunks = make_chunks(lens);
    double *partials = scr.get(chunks.size() + 1);
    StatScope sc(ST_ELEMWISE, 2.0 * 8.0 * double(std::accumulate(lens.begin(), lens.end(), int64_t(0))));
    launch_dot(segs.empty() ? nullptr : static_cast<const double *>(a.data()),
               segs.empty() ? nullptr : static_cast<const double *>(b.data()), upload_vec(segs), upload_vec(chunks),
               int64_t(chunks.size()), partials, dev_out);
}

double dot_all(const BT &a, const BT &b) {
    DevScratch scr;
    double *out = scr.get_result();
    dot_all_dev(a, b, out, scr);
    double h = 0;
    cuda_check(cudaMemcpyAsync(&h, out, sizeof(double), cudaMemcpyDeviceToHost, ctx().stream), "cudaMemcpyAsync");
    cuda_check(cudaStreamSynchronize(ctx().stream), "cudaStreamSynchronize");
    tc_error_raise();
    return h;
}

// u.mul(d) for a rank-1 d on u's last leg (broadcast_operation,
// sources/btensor.cpp:1205-1290): blocks whose last section has no d block vanish.
BT mul_lastleg(const BT &u, const BT &d) {
    if (d.rank != 1) fail(ERR_INVALID_ARGUMENT, "the scaling tensor must have rank 1");
    if (u.rank < 1 || u.sbd.back() != d.sbd[0]) fail(ERR_INVALID_ARGUMENT, "incompatible broadcast dimension");
    require_f64(u);
    require_f64(d);
    const int64_t last = u.addr(u.rank - 1);
    for (int64_t s = 0; s < d.sbd[0]; ++s)
        if (u.ssz[last + s] != d.ssz[s] && d.ssz[s] != 1 && u.ssz[last + s] != 1)
            fail(ERR_INVALID_ARGUMENT, "incompatible broadcast section sizes");
    BT o = u.shape_only();
    for (int64_t s = 0; s < d.sbd[0]; ++s) o.cv[last + s] = qadd(u.cv[last + s], d.cv[s], u.g);
    o.sel = qadd(u.sel, d.sel, u.g);
    std::vector<int64_t> dblock(d.sbd[0], -1);
    for (int64_t b = 0; b < d.nblocks(); ++b) dblock[d.idx(b)[0]] = b;
    std::vector<int64_t> src;
    const int r = u.rank;
    for (int64_t b = 0; b < u.nblocks(); ++b) {
        int64_t s = u.idx(b)[r - 1];
        if (dblock[s] < 0) continue;
        o.bidx.insert(o.bidx.end(), u.idx(b), u.idx(b) + r);
        src.push_back(b);
    }
    o.boff.assign(src.size(), 0);
    o.compact_offsets();
    if (!u.has_data) return o;
    o.alloc_data();
    std::vector<LastLegSeg> segs(src.size());
    std::vector<int64_t> lens(src.size());
    for (size_t k = 0; k < src.size(); ++k) {
        int64_t b = src[k];
        int64_t s = u.idx(b)[r - 1];
        segs[k] = LastLegSeg{u.boff[b], d.boff[dblock[s]], o.boff[k], u.ssz[last + s]};
        lens[k] = u.block_numel(b);
    }
    auto chunks = make_chunks(lens);
    StatScope sc(ST_ELEMWISE, 2.0 * double(o.nnz) * 8.0);
    launch_mul_lastleg(static_cast<const double *>(u.data()), static_cast<const double *>(d.data()),
                       static_cast<double *>(o.data()), upload_vec(segs), upload_vec(chunks), int64_t(chunks.size()));
    return o;
}

// ---------------------------------------------------------------- helpers
std::vector<Chunk> make_chunks(const std::vector<int64_t> &lens) {
    std::vector<Chunk> out;
    for (size_t s = 0; s < lens.size(); ++s)
        for (int64_t st = 0; st < lens[s]; st += CHUNK)
            out.push_back(Chunk{int32_t(s), int32_t(std::min<int64_t>(CHUNK, lens[s] - st)), st});
    return out;
}

void require_f64(const BT &t) {
    if (t.dt != F64) fail(ERR_INVALID_ARGUMENT, "this operation supports float64 blocks only");
}

double *DevScratch::get(size_t n) {
    bufs.push_back(dev_alloc(std::max<size_t>(n, 1) * sizeof(double)));
    return static_cast<double *>(bufs.back()->p);
}
double *DevScratch::get_result() { return get(1); }

}  // namespace qtt
