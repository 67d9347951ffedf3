// Device-side block-sparsity planner: the charge check and the merge-join of a
// contraction, on the GPU.
//
// btensor::tensordot (sources/btensor.cpp:1971-2119) checks that the contracted
// sections carry opposite charges and equal sizes (check_product_compat,
// :783-883), sorts the block lists of both operands with their legs permuted to
// (free, contracted) order, cuts them into runs of equal free prefix, and for every
// run of A and every run of B, in that nested order, pairs the blocks whose
// contracted suffixes are equal (:1998-2110).  Each (run of A, run of B) pair with
// at least one match is an output block; its pairs, in suffix order, are the
// products accumulated into it.  The host planner (contract.cpp) restates that
// order with a sorted suffix index; this file computes the same lists on the device
// in ONE cooperative launch:
//
//   0. charge check of every contracted section (qadd(cA, cB) == 0, sizes equal);
//      block indices packed into 64-bit keys, legs most significant first, so that
//      integer order is the reference's lexicographic order of index tuples;
//   1. rank sort of both key lists (a block's position = the number of smaller
//      keys; keys are unique because block indices are), shared-memory tiles;
//   2. runs of equal free prefix (one CTA scans the head flags);
//   3. the suffix index of B: keys (suffix, run of B), rank sorted;
//   4. for every block of A, its range of equal suffix in that index (binary
//      search) and a scan of the range lengths: the pair offset of every block;
//   5. every pair finds its rank inside its run of A from the sorted ranges of the
//      run's other blocks: (number of pairs with a smaller run of B) + (pairs with
//      the same run of B from an earlier block); the first of each run of B is the
//      head of a new output block;
//   6. a scan of the head flags numbers the output blocks.
// The host reads back the pair and output-block tables (two small copies) and
// builds the output block indices from the first pair of each output block.
//
// Limits (the caller plans on the host beyond them): at most 16384 blocks per
// operand, packed keys within 63 bits, at least one contracted leg, and a bounded
// pair-ranking cost.
#include <cooperative_groups.h>

#include "contract.h"
#include "kernels.h"
#include "qtt_core.h"

namespace qtt {
namespace {
namespace cg = cooperative_groups;

constexpr int PT = 256;      // threads per CTA
constexpr int TILE = 1024;   // keys per shared-memory tile of the rank sort
constexpr int64_t MAX_BLOCKS = 16384;
constexpr int64_t MAX_COST = int64_t(1) << 28;  // pair-ranking steps (pairs x run length)

// error word values
enum : int64_t { PE_NONE = 0, PE_CAPACITY = 1, PE_COST = 2, PE_CHARGE = 3, PE_SIZE = 4 };

struct PlanArgs {
    // inputs: block indices (block-list order) and the leg layout of the keys
    const int32_t *abidx, *bbidx;
    int nA, nB, rA, rB;
    int keyA_leg[MAXRANK], keyB_leg[MAXRANK];  // legs in (free, contracted) order
    int shA[MAXRANK], shB[MAXRANK];            // bit shift of each key position
    int sufbits, runbits;
    // charge check: every contracted section (A leg dA[i], B leg dB[i], section s)
    int nchk;
    const Charge *chkA, *chkB;
    const int64_t *chkSzA, *chkSzB;
    Group g;
    // scratch
    uint64_t *akey, *bkey, *t3;
    int32_t *aid, *bid, *t3j, *runA, *runB, *firstA, *lo, *cnt;
    int64_t *off;
    // outputs
    int32_t *pa, *pb, *head, *p0;
    int64_t cap;
    int64_t *ctr;  // [0] pairs [1] output blocks [2] error [3] runs of A [4] runs of B [5] cost [6] bad check
                   // [7] a pair rank outside its run (an internal error)
};

__device__ uint64_t pack_key(const int32_t *ix, const int *leg, const int *sh, int r) {
    uint64_t k = 0;
    for (int i = 0; i < r; ++i) k |= uint64_t(uint32_t(ix[leg[i]])) << sh[i];
    return k;
}

// out[rank(i)] = (key[i], id[i]), rank(i) = #{k : key[k] < key[i]}; keys unique.
__device__ void rank_sort(const uint64_t *key, const int32_t *id, int n, uint64_t *okey, int32_t *oid,
                          uint64_t *tile) {
    const int stride = gridDim.x * PT;
    for (int base = blockIdx.x * PT; base < n; base += stride) {
        const int i = base + threadIdx.x;
        const uint64_t my = i < n ? key[i] : ~uint64_t(0);
        int rank = 0;
        for (int t0 = 0; t0 < n; t0 += TILE) {
            const int m = min(TILE, n - t0);
            for (int e = threadIdx.x; e < m; e += PT) tile[e] = key[t0 + e];
            __syncthreads();
            for (int e = 0; e < m; ++e) rank += tile[e] < my;
            __syncthreads();
        }
        if (i < n) {
            okey[rank] = my;
            oid[rank] = id ? id[i] : i;
        }
    }
}

// Exclusive scan of x[0..n) (int32 flags or counts) into out[0..n], out[n] = total;
// run by one CTA.
template <class TI, class TO>
__device__ void cta_scan(const TI *x, int64_t n, TO *out, int64_t *sh) {
    const int64_t per = (n + PT - 1) / PT;
    const int64_t b = threadIdx.x * per, e = (b + per < n) ? b + per : n;
    int64_t s = 0;
    for (int64_t i = b; i < e; ++i) s += int64_t(x[i]);
    sh[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t acc = 0;
        for (int t = 0; t < PT; ++t) {
            const int64_t v = sh[t];
            sh[t] = acc;
            acc += v;
        }
        sh[PT] = acc;
    }
    __syncthreads();
    int64_t acc = sh[threadIdx.x];
    for (int64_t i = b; i < e; ++i) {
        const int64_t v = int64_t(x[i]);
        out[i] = TO(acc);
        acc += v;
    }
    if (threadIdx.x == 0) out[n] = TO(sh[PT]);
    __syncthreads();
}

// first position in t3[lo, hi) whose run bits are >= rb (the keys share their suffix)
__device__ int lower_run(const uint64_t *t3, int lo, int hi, uint64_t rb, uint64_t rmask) {
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if ((t3[mid] & rmask) < rb)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

__global__ void __launch_bounds__(PT) k_plan(PlanArgs a) {
    cg::grid_group grid = cg::this_grid();
    __shared__ uint64_t tile[TILE];
    __shared__ int64_t scan_sh[PT + 1];
    const int gt = blockIdx.x * PT + threadIdx.x, gs = gridDim.x * PT;
    const int nfA = a.rA, nfB = a.rB;
    // 0. charge check and keys (unsorted, block-list order)
    for (int i = gt; i < a.nchk; i += gs) {
        const bool ok = qeq(qadd(a.chkA[i], a.chkB[i], a.g), Charge{}, a.g);
        if (!ok || a.chkSzA[i] != a.chkSzB[i])
            atomicMin(reinterpret_cast<unsigned long long *>(&a.ctr[6]),
                      (unsigned long long)(int64_t(i) * 2 + (ok ? 1 : 0)));
    }
    for (int i = gt; i < a.nA; i += gs) a.t3[i] = pack_key(a.abidx + int64_t(i) * a.rA, a.keyA_leg, a.shA, nfA);
    for (int i = gt; i < a.nB; i += gs)
        reinterpret_cast<uint64_t *>(a.off)[i] = pack_key(a.bbidx + int64_t(i) * a.rB, a.keyB_leg, a.shB, nfB);
    grid.sync();
    if (a.ctr[6] != INT64_MAX) {
        if (gt == 0) a.ctr[2] = (a.ctr[6] & 1) ? PE_SIZE : PE_CHARGE;
        return;  // uniform: every thread read the same word after the barrier
    }
    // 1. sort both lists (A's raw keys sit in t3, B's in off, both free again after)
    rank_sort(a.t3, nullptr, a.nA, a.akey, a.aid, tile);
    rank_sort(reinterpret_cast<const uint64_t *>(a.off), nullptr, a.nB, a.bkey, a.bid, tile);
    grid.sync();
    // 2. runs of equal free prefix
    for (int i = gt; i < a.nA; i += gs)
        a.lo[i] = (i == 0 || (a.akey[i] >> a.sufbits) != (a.akey[i - 1] >> a.sufbits)) ? 1 : 0;
    for (int i = gt; i < a.nB; i += gs)
        a.cnt[i] = (i == 0 || (a.bkey[i] >> a.sufbits) != (a.bkey[i - 1] >> a.sufbits)) ? 1 : 0;
    grid.sync();
    if (blockIdx.x == 0) {
        cta_scan(a.lo, a.nA, a.runA, scan_sh);  // runA[i] = heads before i; runA[nA] = runs
        cta_scan(a.cnt, a.nB, a.runB, scan_sh);
        if (threadIdx.x == 0) {
            a.ctr[3] = a.runA[a.nA];
            a.ctr[4] = a.runB[a.nB];
        }
    }
    grid.sync();
    // run ids (inclusive count - 1) and the first block of every run of A
    for (int i = gt; i < a.nA; i += gs) {
        const int r = a.runA[i] + a.lo[i] - 1;
        if (a.lo[i]) a.firstA[r] = i;
    }
    if (gt == 0) a.firstA[a.ctr[3]] = a.nA;
    grid.sync();
    for (int i = gt; i < a.nA; i += gs) a.runA[i] = a.runA[i] + a.lo[i] - 1;
    for (int i = gt; i < a.nB; i += gs) a.runB[i] = a.runB[i] + a.cnt[i] - 1;
    const uint64_t smask = a.sufbits ? (~uint64_t(0) >> (64 - a.sufbits)) : 0;
    const uint64_t rmask = a.runbits ? (~uint64_t(0) >> (64 - a.runbits)) : 0;
    grid.sync();
    // 3. suffix index of B: (suffix, run), value = position in sorted B
    for (int i = gt; i < a.nB; i += gs)
        reinterpret_cast<uint64_t *>(a.off)[i] = ((a.bkey[i] & smask) << a.runbits) | uint64_t(a.runB[i]);
    grid.sync();
    rank_sort(reinterpret_cast<const uint64_t *>(a.off), nullptr, a.nB, a.t3, a.t3j, tile);
    grid.sync();
    // 4. the range of equal suffix of every sorted block of A
    for (int i = gt; i < a.nA; i += gs) {
        const uint64_t s = (a.akey[i] & smask) << a.runbits;
        int lo = 0, hi = a.nB;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (a.t3[mid] < s)
                lo = mid + 1;
            else
                hi = mid;
        }
        int e = lo, h2 = a.nB;
        const uint64_t s1 = s + (rmask + 1);
        while (e < h2) {
            const int mid = (e + h2) >> 1;
            if (a.t3[mid] < s1)
                e = mid + 1;
            else
                h2 = mid;
        }
        a.lo[i] = lo;
        a.cnt[i] = e - lo;
        const int r = a.runA[i];
        const int64_t len = a.firstA[r + 1] - a.firstA[r];
        if (e > lo) atomicAdd(reinterpret_cast<unsigned long long *>(&a.ctr[5]), (unsigned long long)((e - lo) * len));
    }
    grid.sync();
    if (blockIdx.x == 0) {
        cta_scan(a.cnt, a.nA, a.off, scan_sh);
        if (threadIdx.x == 0) {
            a.ctr[0] = a.off[a.nA];
            if (a.off[a.nA] > a.cap)
                a.ctr[2] = PE_CAPACITY;
            else if (a.ctr[5] > MAX_COST)
                a.ctr[2] = PE_COST;
        }
    }
    grid.sync();
    if (a.ctr[2] != PE_NONE) return;
    const int64_t P = a.ctr[0];
    // 5. every pair: its rank inside its run of A, and whether it opens an output block
    for (int64_t q = gt; q < P; q += gs) {
        int lo = 0, hi = a.nA - 1;  // last i with off[i] <= q
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (a.off[mid] <= q)
                lo = mid;
            else
                hi = mid - 1;
        }
        const int i = lo;
        const int t = int(q - a.off[i]);
        const int e3 = a.lo[i] + t;
        const uint64_t rb = a.t3[e3] & rmask;
        const int r = a.runA[i];
        const int f = a.firstA[r], fe = a.firstA[r + 1];
        int64_t pos = 0;
        int head = 1;
        for (int j = f; j < fe; ++j) {
            const int l = a.lo[j], c = a.cnt[j];
            const int lb = lower_run(a.t3, l, l + c, rb, rmask);
            pos += lb - l;
            if (j < i && lb < l + c && (a.t3[lb] & rmask) == rb) {
                head = 0;
                ++pos;
            }
        }
        pos += a.off[f];
        if (pos < 0 || pos >= P) {  // cannot happen: the ranks of a run are a permutation
            a.ctr[7] = 1;
            continue;
        }
        a.pa[pos] = a.aid[i];
        a.pb[pos] = a.bid[a.t3j[e3]];
        a.head[pos] = head;
    }
    grid.sync();
    if (a.ctr[7]) return;
    // 6. number the output blocks
    if (blockIdx.x == 0) {
        cta_scan(a.head, P, a.lo, scan_sh);  // lo is free again; P <= cap <= its length
        if (threadIdx.x == 0) a.ctr[1] = a.lo[P];
    }
    grid.sync();
    for (int64_t q = gt; q < P; q += gs)
        if (a.head[q]) a.p0[a.lo[q]] = int32_t(q);
}

int bits_for(int64_t n) {  // bits holding 0 .. n-1
    int b = 0;
    while (b < 63 && (int64_t(1) << b) < n) ++b;
    return b;
}

struct PlanWs {
    BufPtr buf;
    size_t bytes = 0;
    int64_t *host_ctr = nullptr;
};
thread_local PlanWs tl_ws;

}  // namespace

int plan_join_device(ContractPlan &P, const BT &A, const BT &B, int *bad_dim, bool *bad_size) {
    const int64_t nA = A.nblocks(), nB = B.nblocks();
    const int dl = int(P.dA.size());
    if (dl == 0 || nA < 1 || nB < 1 || nA > MAX_BLOCKS || nB > MAX_BLOCKS) return 0;
    if (A.rank > MAXRANK || B.rank > MAXRANK) return 0;
    PlanArgs a{};
    a.nA = int(nA);
    a.nB = int(nB);
    a.rA = A.rank;
    a.rB = B.rank;
    // key layout: positions in (free, contracted) order, first position most significant
    auto layout = [](const BT &t, const std::vector<int64_t> &order, int *leg, int *sh, int *total) {
        int bits[MAXRANK];
        int tot = 0;
        for (size_t i = 0; i < order.size(); ++i) {
            leg[i] = int(order[i]);
            bits[i] = bits_for(t.sbd[order[i]]);
            tot += bits[i];
        }
        int s = tot;
        for (size_t i = 0; i < order.size(); ++i) {
            s -= bits[i];
            sh[i] = s;
        }
        *total = tot;
    };
    int totA = 0, totB = 0;
    layout(A, P.p1, a.keyA_leg, a.shA, &totA);
    layout(B, P.p2p, a.keyB_leg, a.shB, &totB);
    int suf = 0;
    for (int i = 0; i < dl; ++i) suf += bits_for(A.sbd[P.dA[i]]);
    a.sufbits = suf;
    a.runbits = bits_for(nB + 1);
    if (totA > 63 || totB > 63 || suf + a.runbits > 62) return 0;
    // host tables: block indices as int32 and the contracted sections
    std::vector<int32_t> ab(size_t(nA) * A.rank), bb(size_t(nB) * B.rank);
    for (size_t i = 0; i < ab.size(); ++i) ab[i] = int32_t(A.bidx[i]);
    for (size_t i = 0; i < bb.size(); ++i) bb[i] = int32_t(B.bidx[i]);
    std::vector<Charge> ca, cb;
    std::vector<int64_t> za, zb;
    std::vector<int32_t> cd;
    auto adA = A.addrs(), adB = B.addrs();
    for (int i = 0; i < dl; ++i)
        for (int64_t s = 0; s < A.sbd[P.dA[i]]; ++s) {
            ca.push_back(A.cv[adA[P.dA[i]] + s]);
            cb.push_back(B.cv[adB[P.dB[i]] + s]);
            za.push_back(A.ssz[adA[P.dA[i]] + s]);
            zb.push_back(B.ssz[adB[P.dB[i]] + s]);
            cd.push_back(i);
        }
    a.nchk = int(ca.size());
    a.g = A.g;
    a.abidx = upload_vec(ab);
    a.bbidx = upload_vec(bb);
    a.chkA = upload_vec(ca);
    a.chkB = upload_vec(cb);
    a.chkSzA = upload_vec(za);
    a.chkSzB = upload_vec(zb);
    const int64_t nmax = std::max(nA, nB);
    int64_t cap = std::max<int64_t>(4096, 4 * (nA + nB));
    Ctx &c = ctx();
    static int occ = 0;
    static int sms = 0;
    if (!occ) {
        cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_plan, PT, 0), "occupancy");
        sms = device_sm_count();
    }
    PlanWs &ws = tl_ws;
    if (!ws.host_ctr) cuda_check(cudaMallocHost(&ws.host_ctr, 8 * sizeof(int64_t)), "cudaMallocHost(planner)");
    for (int attempt = 0; attempt < 2; ++attempt) {
        // scratch: 3 key arrays, 9 int32 arrays of nmax (+1), off (nA + 1 int64, also
        // holds nB raw keys), 3 pair arrays and p0 of cap (+1), counters
        const int64_t n1 = nmax + 1, c1 = std::max<int64_t>(cap, nmax) + 1;
        size_t need = 0;
        auto take = [&](size_t b) {
            size_t o = need;
            need += (b + 255) & ~size_t(255);
            return o;
        };
        const size_t o_akey = take(8 * n1), o_bkey = take(8 * n1), o_t3 = take(8 * n1);
        const size_t o_aid = take(4 * n1), o_bid = take(4 * n1), o_t3j = take(4 * n1), o_runA = take(4 * n1),
                     o_runB = take(4 * n1), o_first = take(4 * n1), o_lo = take(4 * c1), o_cnt = take(4 * n1);
        const size_t o_off = take(8 * n1);
        const size_t o_pa = take(4 * c1), o_pb = take(4 * c1), o_head = take(4 * c1), o_p0 = take(4 * c1);
        const size_t o_ctr = take(8 * 8);
        if (!ws.buf || ws.bytes < need) {
            ws.buf = dev_alloc(need);
            ws.bytes = need;
        }
        char *base = static_cast<char *>(ws.buf->p);
        a.akey = reinterpret_cast<uint64_t *>(base + o_akey);
        a.bkey = reinterpret_cast<uint64_t *>(base + o_bkey);
        a.t3 = reinterpret_cast<uint64_t *>(base + o_t3);
        a.aid = reinterpret_cast<int32_t *>(base + o_aid);
        a.bid = reinterpret_cast<int32_t *>(base + o_bid);
        a.t3j = reinterpret_cast<int32_t *>(base + o_t3j);
        a.runA = reinterpret_cast<int32_t *>(base + o_runA);
        a.runB = reinterpret_cast<int32_t *>(base + o_runB);
        a.firstA = reinterpret_cast<int32_t *>(base + o_first);
        a.lo = reinterpret_cast<int32_t *>(base + o_lo);
        a.cnt = reinterpret_cast<int32_t *>(base + o_cnt);
        a.off = reinterpret_cast<int64_t *>(base + o_off);
        a.pa = reinterpret_cast<int32_t *>(base + o_pa);
        a.pb = reinterpret_cast<int32_t *>(base + o_pb);
        a.head = reinterpret_cast<int32_t *>(base + o_head);
        a.p0 = reinterpret_cast<int32_t *>(base + o_p0);
        a.ctr = reinterpret_cast<int64_t *>(base + o_ctr);
        a.cap = cap;
        const int64_t init[8] = {0, 0, 0, 0, 0, 0, INT64_MAX, 0};
        std::memcpy(ws.host_ctr, init, sizeof(init));
        cuda_check(cudaMemcpyAsync(a.ctr, ws.host_ctr, sizeof(init), cudaMemcpyHostToDevice, c.stream),
                   "cudaMemcpyAsync(planner counters)");
        const int64_t work = std::max<int64_t>(nmax, cap / 4);
        const int grid = int(std::max<int64_t>(1, std::min<int64_t>(int64_t(occ) * sms, (work + PT - 1) / PT)));
        void *args[] = {&a};
        cuda_check(cudaLaunchCooperativeKernel((void *)k_plan, dim3(grid), dim3(PT), args, 0, c.stream),
                   "cooperative planner launch");
        count_launch();
        cuda_check(cudaMemcpyAsync(ws.host_ctr, a.ctr, 8 * sizeof(int64_t), cudaMemcpyDeviceToHost, c.stream),
                   "cudaMemcpyAsync(planner counters)");
        cuda_check(cudaStreamSynchronize(c.stream), "cudaStreamSynchronize(planner)");
        const int64_t *h = ws.host_ctr;
        if (h[2] == PE_CHARGE || h[2] == PE_SIZE) {
            const int64_t k = h[6] / 2;
            *bad_dim = cd[size_t(k)];
            *bad_size = h[2] == PE_SIZE;
            return -1;
        }
        if (h[2] == PE_COST) return 0;
        if (h[2] == PE_CAPACITY) {
            cap = h[0];
            continue;
        }
        if (h[7]) fail(ERR_RUNTIME, "device planner: a pair rank fell outside its run");
        const int64_t np = h[0], nout = h[1];
        std::vector<int32_t> pa(np), pb(np), p0(nout);
        if (np) {
            cuda_check(cudaMemcpyAsync(pa.data(), a.pa, np * 4, cudaMemcpyDeviceToHost, c.stream), "planner pairs");
            cuda_check(cudaMemcpyAsync(pb.data(), a.pb, np * 4, cudaMemcpyDeviceToHost, c.stream), "planner pairs");
        }
        if (nout)
            cuda_check(cudaMemcpyAsync(p0.data(), a.p0, nout * 4, cudaMemcpyDeviceToHost, c.stream), "planner blocks");
        cuda_check(cudaStreamSynchronize(c.stream), "cudaStreamSynchronize(planner)");
        P.pair_a.assign(pa.begin(), pa.end());
        P.pair_b.assign(pb.begin(), pb.end());
        P.out_p0.resize(nout);
        P.out_p1.resize(nout);
        BT &o = P.out;
        o.bidx.clear();
        o.bidx.reserve(size_t(nout) * o.rank);
        for (int64_t k = 0; k < np; ++k)
            if (pa[k] < 0 || pa[k] >= nA || pb[k] < 0 || pb[k] >= nB)
                fail(ERR_RUNTIME, "device planner: pair table out of range");
        for (int64_t k = 0; k < nout; ++k) {
            if (p0[k] < 0 || p0[k] >= np || (k > 0 && p0[k] <= p0[k - 1]))
                fail(ERR_RUNTIME, "device planner: output block table out of order");
            P.out_p0[k] = p0[k];
            P.out_p1[k] = k + 1 < nout ? p0[k + 1] : np;
            const int64_t *ia = A.idx(pa[p0[k]]), *ib = B.idx(pb[p0[k]]);
            for (auto d : P.freeA) o.bidx.push_back(ia[d]);
            for (auto d : P.freeB) o.bidx.push_back(ib[d]);
        }
        return 1;
    }
    return 0;
}

}  // namespace qtt
