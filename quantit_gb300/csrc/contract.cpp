// Block-sparse contraction: the planner and the grouped-GEMM dispatch.
//
// btensor::tensordot (sources/btensor.cpp:1971-2119) permutes every block of
// both operands into matrix form (permute_bl :1843-1894), merge-joins the two
// sorted block lists on the contracted block-index suffix and, per output block,
// runs torch::mm on the first matching pair and addmm_ on the others.  Here the
// merge-join produces the same output block list (bit-exact, same order) plus a
// pair table; the block products of the whole contraction then run as one
// grouped GEMM launch.  Operands whose natural row-major layout already is the
// (free x contracted) or (contracted x free) matrix are read in place (plain or
// transposed access); only a genuinely scattered leg order is packed first.
#include <chrono>
#include <numeric>

#include "contract.h"
#include "kernels.h"
#include "ops_util.h"
#include "qtt_core.h"

namespace qtt {

namespace {
std::vector<int64_t> norm_dims(const std::vector<int64_t> &d, int r) {
    std::vector<int64_t> o(d.size());
    for (size_t i = 0; i < d.size(); ++i) {
        int64_t x = d[i] < 0 ? d[i] + r : d[i];
        if (x < 0 || x >= r) fail(ERR_CHECK, "dimension out of range");
        o[i] = x;
    }
    std::vector<int64_t> s = o;
    std::sort(s.begin(), s.end());
    if (std::adjacent_find(s.begin(), s.end()) != s.end()) fail(ERR_CHECK, "repeated dimension in contraction");
    return o;
}

struct Keyed {
    std::vector<int64_t> key;  // all keys, nblocks x rank
    std::vector<int64_t> id;   // original block of each sorted entry
    int r;
    const int64_t *k(size_t i) const { return key.data() + i * r; }
};

Keyed permuted_sorted(const BT &t, const std::vector<int64_t> &perm) {
    Keyed K;
    K.r = t.rank;
    const int64_t nb = t.nblocks();
    std::vector<int64_t> raw(nb * K.r);
    for (int64_t b = 0; b < nb; ++b)
        for (int i = 0; i < K.r; ++i) raw[b * K.r + i] = t.idx(b)[perm[i]];
    std::vector<int64_t> ord(nb);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(),
                     [&](int64_t a, int64_t b) { return idx_less(raw.data() + a * K.r, raw.data() + b * K.r, K.r); });
    K.key.resize(nb * K.r);
    for (int64_t k = 0; k < nb; ++k) std::copy(raw.begin() + ord[k] * K.r, raw.begin() + (ord[k] + 1) * K.r, K.key.begin() + k * K.r);
    K.id = ord;
    return K;
}

// runs of equal prefix (length nf); with no contracted leg every block is its own run
std::vector<std::pair<size_t, size_t>> runs(const Keyed &K, int nf, bool singletons) {
    std::vector<std::pair<size_t, size_t>> out;
    size_t n = K.id.size(), i = 0;
    while (i < n) {
        size_t j = i + 1;
        if (!singletons)
            while (j < n && std::equal(K.k(j), K.k(j) + nf, K.k(i))) ++j;
        out.push_back({i, j});
        i = j;
    }
    return out;
}

bool is_identity(const std::vector<int64_t> &p) {
    for (size_t i = 0; i < p.size(); ++i)
        if (p[i] != int64_t(i)) return false;
    return true;
}
}  // namespace

namespace {
void host_join(ContractPlan &P, const BT &A, const BT &B, int dl);
void set_operand_modes(ContractPlan &P);

bool device_present() {
    static const bool present = [] {
        int n = 0;
        return cudaGetDeviceCount(&n) == cudaSuccess && n > 0;
    }();
    return present;
}

[[noreturn]] void fail_sections(const ContractPlan &P, int i, bool size) {
    const std::string a = std::to_string(P.dA[i]), b = std::to_string(P.dB[i]);
    if (size)
        fail(ERR_CHECK, "contracted section sizes differ between dim " + a + " of the left tensor and dim " + b +
                            " of the right tensor");
    fail(ERR_CHECK, "contracted conserved numbers need to sum to zero, but there is a violation when contracting dim " +
                        a + " of the left tensor with dim " + b + " of the right tensor");
}
}  // namespace

ContractPlan plan_contraction(const BT &A, const BT &B, const std::vector<int64_t> &dA_in,
                              const std::vector<int64_t> &dB_in) {
    const auto t_start = std::chrono::steady_clock::now();
    // compute_tdot_shape / check_product_compat (btensor.cpp:783-883)
    if (dA_in.size() != dB_in.size()) fail(ERR_CHECK, "both dimension lists should have the same length.");
    if (!(A.g == B.g)) fail(ERR_CHECK, "the two tensors have different type of conserved quantities");
    ContractPlan P;
    P.dA = norm_dims(dA_in, A.rank);
    P.dB = norm_dims(dB_in, B.rank);
    const int dl = int(P.dA.size());
    auto adA = A.addrs(), adB = B.addrs();
    // dimension by dimension: the section count, then every section's charges and size
    auto host_check = [&]() {
        for (int i = 0; i < dl; ++i) {
            int64_t a = P.dA[i], b = P.dB[i];
            if (A.sbd[a] != B.sbd[b])
                fail(ERR_CHECK, "contracted dimensions need to match, but first has " + std::to_string(A.sbd[a]) +
                                    " sections along dim " + std::to_string(a) + "  and second has " +
                                    std::to_string(B.sbd[b]) + " sections along dim " + std::to_string(b));
            for (int64_t s = 0; s < A.sbd[a]; ++s) {
                if (!qeq(qadd(A.cv[adA[a] + s], B.cv[adB[b] + s], A.g), Charge{}, A.g)) fail_sections(P, i, false);
                if (A.ssz[adA[a] + s] != B.ssz[adB[b] + s]) fail_sections(P, i, true);
            }
        }
    };
    bool counts_match = true;
    for (int i = 0; i < dl; ++i) counts_match = counts_match && A.sbd[P.dA[i]] == B.sbd[P.dB[i]];
    const int mode = planner_mode();
    const int64_t nbl = A.nblocks() + B.nblocks();
    // the device planner checks the section charges itself; graph capture (no
    // synchronisation allowed) and machines without a device plan on the host
    const bool want_dev = mode != 0 && dl > 0 && counts_match && A.nblocks() > 0 && B.nblocks() > 0 &&
                          (mode == 1 || nbl >= planner_auto_blocks()) && device_present() && !ctx().capturing;
    if (!want_dev) host_check();
    std::vector<char> cA(A.rank, 0), cB(B.rank, 0);
    for (auto d : P.dA) cA[d] = 1;
    for (auto d : P.dB) cB[d] = 1;
    for (int i = 0; i < A.rank; ++i)
        if (!cA[i]) P.freeA.push_back(i);
    for (int i = 0; i < B.rank; ++i)
        if (!cB[i]) P.freeB.push_back(i);
    std::vector<int64_t> p1 = P.freeA, p2 = P.dB, p2p = P.freeB;
    p1.insert(p1.end(), P.dA.begin(), P.dA.end());
    p2.insert(p2.end(), P.freeB.begin(), P.freeB.end());
    p2p.insert(p2p.end(), P.dB.begin(), P.dB.end());
    P.p1 = p1;
    P.p2p = p2p;
    P.p2 = p2;
    // output structure (compute_tdot_cval_sectSize :1908-1935)
    BT &o = P.out;
    o.g = A.g;
    o.rank = int(P.freeA.size() + P.freeB.size());
    if (o.rank > MAXRANK) fail(ERR_CHECK, "contraction result rank exceeds 8");
    o.dt = (A.dt == F64 || B.dt == F64) ? F64 : F32;
    o.sel = qadd(A.sel, B.sel, A.g);
    for (auto d : P.freeA) {
        o.sbd.push_back(A.sbd[d]);
        for (int64_t s = 0; s < A.sbd[d]; ++s) {
            o.ssz.push_back(A.ssz[adA[d] + s]);
            o.cv.push_back(A.cv[adA[d] + s]);
        }
    }
    for (auto d : P.freeB) {
        o.sbd.push_back(B.sbd[d]);
        for (int64_t s = 0; s < B.sbd[d]; ++s) {
            o.ssz.push_back(B.ssz[adB[d] + s]);
            o.cv.push_back(B.cv[adB[d] + s]);
        }
    }
    int on_device = 0;
    if (want_dev) {
        int bad_dim = 0;
        bool bad_size = false;
        on_device = plan_join_device(P, A, B, &bad_dim, &bad_size);
        if (on_device < 0) fail_sections(P, bad_dim, bad_size);
        if (!on_device) {
            planner_account(2, 0.0);
            host_check();
        }
    }
    if (!on_device) host_join(P, A, B, dl);
    o.boff.assign(P.out_p0.size(), 0);
    o.compact_offsets();
    set_operand_modes(P);
    planner_account(on_device ? 1 : 0,
                    std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count());
    return P;
}

namespace {
void host_join(ContractPlan &P, const BT &A, const BT &B, int dl) {
    BT &o = P.out;
    // merge-join (btensor.cpp:1998-2114): for every run of A (equal free prefix) and
    // every run of B, in that nested order, the pairs with equal contracted suffix.
    // Only the runs of B that share a suffix with the run of A can produce pairs, so
    // they are found through a sorted (suffix, run) index of B instead of trying
    // every run pair: the same output block list and pair order, in
    // O(n log n + pairs) instead of O(runs_A x runs_B).
    Keyed t1 = permuted_sorted(A, P.p1), t2 = permuted_sorted(B, P.p2p);
    const int nfa = A.rank - dl, nfb = B.rank - dl;
    auto r1 = runs(t1, nfa, dl == 0), r2 = runs(t2, nfb, dl == 0);
    auto join = [&](const std::pair<size_t, size_t> &ra, const std::pair<size_t, size_t> &rb) {
        size_t ia = ra.first, ib = rb.first;
        size_t first_pair = P.pair_a.size();
        while (ia < ra.second && ib < rb.second) {
            const int64_t *sa = t1.k(ia) + nfa, *sb = t2.k(ib) + nfb;
            if (idx_less(sa, sb, dl))
                ++ia;
            else if (idx_less(sb, sa, dl))
                ++ib;
            else {
                P.pair_a.push_back(t1.id[ia]);
                P.pair_b.push_back(t2.id[ib]);
                ++ia;
                ++ib;
            }
        }
        if (P.pair_a.size() > first_pair) {
            o.bidx.insert(o.bidx.end(), t1.k(ra.first), t1.k(ra.first) + nfa);
            o.bidx.insert(o.bidx.end(), t2.k(rb.first), t2.k(rb.first) + nfb);
            P.out_p0.push_back(int64_t(first_pair));
            P.out_p1.push_back(int64_t(P.pair_a.size()));
        }
    };
    if (dl == 0) {
        for (auto &ra : r1)
            for (auto &rb : r2) join(ra, rb);
    } else {
        // (suffix, run of B) for every block of B, sorted by suffix then run
        std::vector<std::pair<size_t, int32_t>> sidx;  // (entry of t2, run)
        sidx.reserve(t2.id.size());
        for (size_t r = 0; r < r2.size(); ++r)
            for (size_t i = r2[r].first; i < r2[r].second; ++i) sidx.push_back({i, int32_t(r)});
        auto suf2 = [&](size_t i) { return t2.k(i) + nfb; };
        std::sort(sidx.begin(), sidx.end(), [&](const auto &x, const auto &y) {
            if (idx_less(suf2(x.first), suf2(y.first), dl)) return true;
            if (idx_less(suf2(y.first), suf2(x.first), dl)) return false;
            return x.second < y.second;
        });
        std::vector<int32_t> cand;
        for (auto &ra : r1) {
            cand.clear();
            for (size_t ia = ra.first; ia < ra.second; ++ia) {
                const int64_t *s = t1.k(ia) + nfa;
                auto lo = std::lower_bound(sidx.begin(), sidx.end(), s,
                                           [&](const auto &x, const int64_t *key) { return idx_less(suf2(x.first), key, dl); });
                for (auto it = lo; it != sidx.end() && !idx_less(s, suf2(it->first), dl); ++it) cand.push_back(it->second);
            }
            std::sort(cand.begin(), cand.end());
            cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
            for (int32_t rb : cand) join(ra, r2[rb]);
        }
    }
}

void set_operand_modes(ContractPlan &P) {
    // operand layouts
    const std::vector<int64_t> &p1 = P.p1, &p2 = P.p2;
    P.a_mode = is_identity(p1) ? 0 : -1;
    if (P.a_mode < 0) {
        // rotation: contracted legs leading in dims order, free legs trailing in order
        std::vector<int64_t> rot = P.dA;
        rot.insert(rot.end(), P.freeA.begin(), P.freeA.end());
        P.a_mode = is_identity(rot) ? 1 : 2;
    }
    P.b_mode = is_identity(p2) ? 0 : -1;
    if (P.b_mode < 0) {
        std::vector<int64_t> rot = P.freeB;
        rot.insert(rot.end(), P.dB.begin(), P.dB.end());
        P.b_mode = is_identity(rot) ? 1 : 2;
    }
}
}  // namespace

namespace {
// permuted copy of every block of t with permutation perm (compact, block-list order)
BufPtr pack_operand(const BT &t, const std::vector<int64_t> &perm, std::vector<int64_t> &offs) {
    const int r = t.rank;
    const int64_t nb = t.nblocks();
    offs.assign(nb, 0);
    std::vector<PermEntry> ents(nb);
    std::vector<int64_t> lens(nb);
    int64_t o = 0;
    for (int64_t b = 0; b < nb; ++b) {
        int64_t shp[MAXRANK], str[MAXRANK];
        t.block_shape(b, shp);
        int64_t s = 1;
        for (int d = r - 1; d >= 0; --d) {
            str[d] = s;
            s *= shp[d];
        }
        PermEntry &e = ents[b];
        std::memset(&e, 0, sizeof(e));
        e.src_off = t.boff[b];
        e.dst_off = o;
        e.rank = r;
        for (int i = 0; i < r; ++i) {
            e.dims[i] = shp[perm[i]];
            e.stride[i] = str[perm[i]];
        }
        offs[b] = o;
        lens[b] = t.block_numel(b);
        o += lens[b];
    }
    auto buf = dev_alloc(size_t(std::max<int64_t>(o, 1)) * 8);
    auto chunks = make_chunks(lens);
    StatScope sc(ST_PERMUTE, 2.0 * 8.0 * double(o));
    launch_permute(t.data(), buf->p, upload_vec(ents), upload_vec(chunks), int64_t(chunks.size()), 8);
    return buf;
}

int64_t prod_sizes(const BT &t, int64_t b, const std::vector<int64_t> &dims) {
    int64_t shp[MAXRANK];
    t.block_shape(b, shp);
    int64_t p = 1;
    for (auto d : dims) p *= shp[d];
    return p;
}
}  // namespace

namespace {
// Split every block of t (legs permuted by perm; the first nrow legs form the
// rows, the rest the contracted K) into hi / lo TF32 arrays (TF32X3) or hi / mid / lo
// BF16 arrays (BF16X3), tiled in the tensor cores' core matrices (8 rows x 16 bytes),
// rows zero padded to 8 and K to the MMA's K step (8 TF32 / 16 BF16).
void split_operand(const BT &t, const std::vector<int64_t> &perm, int nrow, std::vector<int64_t> &offs, BufPtr &hi,
                   BufPtr &mid, BufPtr &lo, unsigned long long *amax, int mode) {
    const bool bf16 = mode == GEMM_BF16X3;
    const int64_t gran = bf16 ? 16 : 8;
    const int r = t.rank;
    const int64_t nb = t.nblocks();
    offs.assign(nb, 0);
    std::vector<SplitEntry> ents(nb);
    std::vector<int64_t> lens(nb);
    int64_t o = 0;
    for (int64_t b = 0; b < nb; ++b) {
        int64_t shp[MAXRANK], str[MAXRANK];
        t.block_shape(b, shp);
        int64_t s = 1;
        for (int d = r - 1; d >= 0; --d) {
            str[d] = s;
            s *= shp[d];
        }
        SplitEntry &e = ents[b];
        std::memset(&e, 0, sizeof(e));
        int64_t rows = 1, K = 1;
        for (int i = 0; i < r; ++i) {
            e.dims[i] = shp[perm[i]];
            e.stride[i] = str[perm[i]];
            (i < nrow ? rows : K) *= shp[perm[i]];
        }
        if (K > INT32_MAX) fail(ERR_INVALID_ARGUMENT, "contracted dimension too large");
        const int64_t K4 = (K + gran - 1) & ~(gran - 1);
        e.src_off = t.boff[b];
        e.dst_off = o;
        e.rank = r;
        e.K = int32_t(K);
        e.K4 = int32_t(K4);
        // index-math fast paths of the split kernels
        bool contig = true;
        int64_t sfx = 1;
        for (int i = r - 1; i >= 0; --i) {
            if (e.stride[i] != sfx && e.dims[i] != 1) contig = false;
            sfx *= e.dims[i];
        }
        e.flags = (rows * K < int64_t(INT32_MAX) ? SPLIT_SMALL : 0) | (contig ? SPLIT_CONTIG : 0);
        offs[b] = o;
        lens[b] = rows * K;
        o += ((rows + 7) & ~int64_t(7)) * K4;
    }
    const size_t bytes = size_t(std::max<int64_t>(o, 8)) * (bf16 ? sizeof(uint16_t) : sizeof(float));
    std::vector<BufPtr *> parts = {&hi, &lo};
    if (bf16) parts.push_back(&mid);
    for (BufPtr *b : parts) {
        *b = dev_alloc(bytes);
        cuda_check(cudaMemsetAsync((*b)->p, 0, bytes, ctx().stream), "cudaMemsetAsync(split)");
    }
    auto chunks = make_chunks(lens);
    const double nel = double(std::accumulate(lens.begin(), lens.end(), int64_t(0)));
    StatScope sc(ST_PACK, (bf16 ? 14.0 : 16.0) * nel);
    launch_amax(static_cast<const double *>(t.data()), t.nnz, amax);
    if (bf16)
        launch_split_bf16x3(static_cast<const double *>(t.data()), hi->p, mid->p, lo->p, upload_vec(ents),
                            upload_vec(chunks), int64_t(chunks.size()), amax);
    else
        launch_split_tf32(static_cast<const double *>(t.data()), static_cast<float *>(hi->p),
                          static_cast<float *>(lo->p), upload_vec(ents), upload_vec(chunks), int64_t(chunks.size()),
                          amax);
}
}  // namespace

void run_contraction(const ContractPlan &P, const BT &A, const BT &B, BT &out, const BT *add, double beta,
                     double alpha, const std::vector<int64_t> *add_block) {
    require_f64(A);
    require_f64(B);
    const int64_t nout = int64_t(P.out_p0.size());
    if (nout == 0) return;
    const int mode = gemm_mode();
    const bool tc = mode != GEMM_F64;
    // operand buffers
    BufPtr pa, pb, ahi, amid, alo, bhi, bmid, blo, amax;
    std::vector<int64_t> offa, offb;
    const double *Ap = static_cast<const double *>(A.data());
    const double *Bp = static_cast<const double *>(B.data());
    const std::vector<int64_t> *oa = &A.boff, *ob = &B.boff;
    int a_t = 0, b_t = 0;
    if (tc) {
        amax = dev_alloc(2 * sizeof(unsigned long long));
        cuda_check(cudaMemsetAsync(amax->p, 0, 2 * sizeof(unsigned long long), ctx().stream), "cudaMemsetAsync(amax)");
        auto *am = static_cast<unsigned long long *>(amax->p);
        split_operand(A, P.p1, int(P.freeA.size()), offa, ahi, amid, alo, am, mode);
        split_operand(B, P.p2p, int(P.freeB.size()), offb, bhi, bmid, blo, am + 1, mode);
        oa = &offa;
        ob = &offb;
    } else {
        if (P.a_mode == 1) a_t = 1;
        if (P.a_mode == 2) {
            pa = pack_operand(A, P.p1, offa);
            Ap = static_cast<const double *>(pa->p);
            oa = &offa;
        }
        if (P.b_mode == 1) b_t = 1;
        if (P.b_mode == 2) {
            pb = pack_operand(B, P.p2, offb);
            Bp = static_cast<const double *>(pb->p);
            ob = &offb;
        }
    }
    const int TM = tc ? gemm_tile_m(mode) : 64;
    const int TN = tc ? gemm_tile_n(mode) : 64;
    std::vector<GemmPair> pairs(P.pair_a.size());
    std::vector<GemmOut> outs(nout);
    std::vector<GemmTile> tiles;
    double flops = 0;
    for (int64_t k = 0; k < int64_t(P.pair_a.size()); ++k) {
        int64_t ia = P.pair_a[k], ib = P.pair_b[k];
        pairs[k].a_off = (*oa)[ia];
        pairs[k].b_off = (*ob)[ib];
        pairs[k].K = int32_t(prod_sizes(A, ia, P.dA));
        pairs[k].pad = 0;
    }
    std::vector<std::pair<double, GemmTile>> wt;
    int64_t max_chunks = 0;
    for (int64_t o = 0; o < nout; ++o) {
        int64_t ia = P.pair_a[P.out_p0[o]], ib = P.pair_b[P.out_p0[o]];
        int64_t M = prod_sizes(A, ia, P.freeA), N = prod_sizes(B, ib, P.freeB);
        if (M > INT32_MAX || N > INT32_MAX) fail(ERR_INVALID_ARGUMENT, "block too large");
        outs[o].c_off = out.boff[o];
        outs[o].add_off = (add && add_block && (*add_block)[o] >= 0) ? add->boff[(*add_block)[o]] : -1;
        outs[o].M = int32_t(M);
        outs[o].N = int32_t(N);
        outs[o].p0 = int32_t(P.out_p0[o]);
        outs[o].p1 = int32_t(P.out_p1[o]);
        double ksum = 0;
        int64_t chunks = 0;
        for (int64_t p = P.out_p0[o]; p < P.out_p1[o]; ++p) {
            ksum += pairs[p].K;
            // K chunks of the tensor-core kernels: 32 TF32 (K padded to 8) / 64 BF16 (to 16)
            chunks += mode == GEMM_BF16X3 ? (((pairs[p].K + 15) & ~15) + 63) / 64 : (((pairs[p].K + 7) & ~7) + 31) / 32;
        }
        max_chunks = std::max(max_chunks, chunks);
        flops += 2.0 * double(M) * double(N) * ksum;
        for (int64_t m0 = 0; m0 < M; m0 += TM)
            for (int64_t n0 = 0; n0 < N; n0 += TN)
                wt.push_back({ksum, GemmTile{int32_t(o), int32_t(m0), int32_t(n0), 0}});
    }
    // longest tiles first: the tail of the grid is made of the cheap ones
    std::stable_sort(wt.begin(), wt.end(), [](const auto &x, const auto &y) { return x.first > y.first; });
    tiles.reserve(wt.size());
    for (auto &w : wt) tiles.push_back(w.second);
    const GemmPair *dpairs = upload_vec(pairs);
    const GemmOut *douts = upload_vec(outs);
    const GemmTile *dtiles = upload_vec(tiles);
    StatScope sc(ST_GEMM, flops);
    if (!tc) {
        GemmArgs g;
        g.A = Ap;
        g.B = Bp;
        g.C = static_cast<double *>(out.data());
        g.Cadd = add ? static_cast<const double *>(add->data()) : nullptr;
        g.pairs = dpairs;
        g.outs = douts;
        g.tiles = dtiles;
        g.ntiles = int32_t(tiles.size());
        g.a_t = a_t;
        g.b_t = b_t;
        g.alpha = alpha;
        g.beta = beta;
        launch_gemm_f64(g);
    } else {
        TcArgs g;
        g.Ahi = ahi->p;
        g.Amid = amid ? amid->p : nullptr;
        g.Alo = alo->p;
        g.Bhi = bhi->p;
        g.Bmid = bmid ? bmid->p : nullptr;
        g.Blo = blo->p;
        g.amax_a = static_cast<const unsigned long long *>(amax->p);
        g.amax_b = g.amax_a + 1;
        g.C = static_cast<double *>(out.data());
        g.Cadd = add ? static_cast<const double *>(add->data()) : nullptr;
        g.pairs = dpairs;
        g.outs = douts;
        g.tiles = dtiles;
        g.ntiles = int32_t(tiles.size());
        g.max_chunks = int32_t(std::min<int64_t>(max_chunks, INT32_MAX));
        g.alpha = alpha;
        g.beta = beta;
        launch_gemm_tc(g, mode);
    }
}

BT tensordot(const BT &a, const BT &b, const std::vector<int64_t> &da, const std::vector<int64_t> &db) {
    ContractPlan P = plan_contraction(a, b, da, db);
    BT out = P.out;
    if (!a.has_data || !b.has_data) {
        if (a.has_data != b.has_data && a.nblocks() && b.nblocks()) fail(ERR_NO_DATA, "mixing structure-only and data btensors");
        return out;
    }
    out.alloc_data();
    run_contraction(P, a, b, out, nullptr, 0.0, 1.0, nullptr);
    return out;
}

// beta*add + alpha*tensordot(a, b): blocks of the product that also exist in add
// take the add term in the GEMM epilogue; blocks only in add are scaled copies.
BT tensorgdot(const BT &add, const BT &a, const BT &b, const std::vector<int64_t> &da, const std::vector<int64_t> &db,
              double beta, double alpha) {
    ContractPlan P = plan_contraction(a, b, da, db);
    if (!same_shape(P.out, add)) fail(ERR_INVALID_ARGUMENT, "the add tensor's shape differs from the contraction's output");
    // union of add's blocks and the product's blocks
    BT prod = P.out;
    auto u = union_plan(add, prod);
    BT out = add.shape_only();
    out.bidx = u.idx;
    out.boff.assign(u.a.size(), 0);
    out.compact_offsets();
    if (!a.has_data || !b.has_data || (!add.has_data && add.nblocks())) return out;
    require_f64(add);
    out.alloc_data();
    // product blocks write at the union positions
    std::vector<int64_t> prod_pos(prod.nblocks(), -1), add_of_prod(prod.nblocks(), -1);
    std::vector<AxpbySeg> segs;
    std::vector<int64_t> lens;
    for (size_t k = 0; k < u.a.size(); ++k) {
        if (u.b[k] >= 0) {
            prod_pos[u.b[k]] = int64_t(k);
            add_of_prod[u.b[k]] = u.a[k];
        } else {
            segs.push_back(AxpbySeg{add.boff[u.a[k]], -1, out.boff[k]});
            lens.push_back(out.block_numel(int64_t(k)));
        }
    }
    BT target = prod;  // product structure with offsets into out's buffer
    for (int64_t o = 0; o < prod.nblocks(); ++o) target.boff[o] = out.boff[prod_pos[o]];
    target.buf = out.buf;
    target.has_data = true;
    run_contraction(P, a, b, target, &add, beta, alpha, &add_of_prod);
    if (!segs.empty()) {
        auto chunks = make_chunks(lens);
        launch_axpby(static_cast<const double *>(add.data()), nullptr, static_cast<double *>(out.data()),
                     upload_vec(segs), upload_vec(chunks), int64_t(chunks.size()), coef_host(beta), coef_host(0.0));
    }
    return out;
}

}  // namespace qtt
