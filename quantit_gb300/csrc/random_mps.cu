// random_bMPS on the GPU (sources/MPT.cpp:424-462): a random MPS that can be
// contracted with a given MPO, with total charge `constraint`.
//
// Structure (host): the physical leg of site i is the MPO's leg 1 (sections and
// charges).  The charges a bond can carry are the partial sums of physical charges
// reachable from the left that can still reach the constraint from the right; each
// charge's dimension is the smaller of its left and right multiplicities, and the
// dimensions are capped to a total of bond_dim (water filling: every charge gets
// min(multiplicity, c) for the largest c that fits, the remainder one by one to the
// largest capped charges, ties to the smaller charge).  The reference draws random
// basis strings to pick its sectors instead (generate_random_string); both give
// allowed bond sectors of total dimension <= bond_dim.
//
// Data (device): every element N(0, 1) from a counter-based generator keyed by
// (seed, site, element) -- the same values on any GPU and stream -- then each site is
// scaled to unit Frobenius norm, as MPT.cpp:450 does.  (The reference fills with
// uniform [0, 1) from torch's global generator, MPT.cpp:449, which is not seedable
// per call; N(0, 1) entries are what the benchmark configurations specify.)
#include <map>

#include "kernels.h"
#include "qtt_core.h"

namespace qtt {
namespace {

// splitmix64 finaliser (Steele, Lea & Flood, "Fast splittable pseudorandom number
// generators", OOPSLA 2014): a bijective 64-bit mix of a counter.
__host__ __device__ inline uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// N(0, 1) by the Box-Muller transform of two uniforms drawn from the counter.
__global__ void k_fill_normal(double *x, int64_t n, uint64_t key) {
    for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < n; e += int64_t(gridDim.x) * blockDim.x) {
        const uint64_t a = mix64(key ^ mix64(uint64_t(2 * e)));
        const uint64_t b = mix64(key ^ mix64(uint64_t(2 * e + 1)));
        const double u1 = (double(a >> 11) + 1.0) * 0x1.0p-53;  // (0, 1]
        const double u2 = double(b >> 11) * 0x1.0p-53;          // [0, 1)
        x[e] = sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
    }
}

struct ChargeLess {
    Group g;
    bool operator()(const Charge &a, const Charge &b) const { return qless(a, b, g); }
};
using Mult = std::map<Charge, int64_t, ChargeLess>;

Mult cap(const Mult &m, int64_t D, const Group &g) {
    int64_t tot = 0, mx = 0;
    for (auto &kv : m) {
        tot += kv.second;
        mx = std::max(mx, kv.second);
    }
    if (tot <= D) return m;
    int64_t lo = 0, hi = mx;
    while (lo < hi) {
        const int64_t c = (lo + hi + 1) / 2;
        int64_t s = 0;
        for (auto &kv : m) s += std::min(kv.second, c);
        if (s <= D)
            lo = c;
        else
            hi = c - 1;
    }
    Mult out(ChargeLess{g});
    int64_t used = 0;
    for (auto &kv : m) {
        out[kv.first] = std::min(kv.second, lo);
        used += out[kv.first];
    }
    std::vector<std::pair<Charge, int64_t>> over;
    for (auto &kv : m)
        if (kv.second > lo) over.push_back(kv);
    std::stable_sort(over.begin(), over.end(),
                     [](const std::pair<Charge, int64_t> &a, const std::pair<Charge, int64_t> &b) {
                         return a.second > b.second;
                     });
    for (auto &kv : over) {
        if (used >= D) break;
        out[kv.first] += 1;
        ++used;
    }
    for (auto it = out.begin(); it != out.end();) it = it->second > 0 ? std::next(it) : out.erase(it);
    return out;
}

}  // namespace

std::vector<BT> random_mps(const std::vector<BT> &mpo, int64_t D, const Charge &target, uint64_t seed) {
    const int64_t L = int64_t(mpo.size());
    if (L < 1) fail(ERR_INVALID_ARGUMENT, "random_bMPS needs at least one site");
    if (D < 1) fail(ERR_INVALID_ARGUMENT, "random_bMPS needs a positive bond dimension");
    const Group g = mpo[0].g;
    ChargeLess lessq{g};
    // physical sections of each site: the MPO's leg 1
    std::vector<std::vector<std::pair<int64_t, Charge>>> phys(L);
    for (int64_t i = 0; i < L; ++i) {
        const BT &w = mpo[i];
        if (w.rank != 4) fail(ERR_INVALID_ARGUMENT, "random_bMPS needs rank-4 MPO tensors");
        if (!(w.g == g)) fail(ERR_INVALID_ARGUMENT, "MPO tensors of different groups");
        const int64_t a = w.addr(1);
        for (int64_t s = 0; s < w.sbd[1]; ++s) phys[i].push_back({w.ssz[a + s], w.cv[a + s]});
    }
    // left[n]: charge -> number of basis strings of the first n sites; right[n] likewise
    // for the last n sites
    std::vector<Mult> left(L + 1, Mult(lessq)), right(L + 1, Mult(lessq));
    left[0][Charge{}] = 1;
    right[0][Charge{}] = 1;
    auto grow = [&](const Mult &m, const std::vector<std::pair<int64_t, Charge>> &ph) {
        Mult o(lessq);
        for (auto &kv : m)
            for (auto &p : ph) {
                int64_t &x = o[qadd(kv.first, p.second, g)];
                x = std::min<int64_t>(x + kv.second * p.first, int64_t(1) << 40);
            }
        return o;
    };
    for (int64_t n = 1; n <= L; ++n) {
        left[n] = grow(left[n - 1], phys[n - 1]);
        right[n] = grow(right[n - 1], phys[L - n]);
    }
    if (!left[L].count(target)) fail(ERR_INVALID_ARGUMENT, "no basis state of the MPO's sites has the requested charge");
    // bond b (between sites b and b+1): partial charge q of the first b+1 sites
    std::vector<Mult> bonds;
    for (int64_t b = 0; b + 1 < L; ++b) {
        Mult dims(lessq);
        for (auto &kv : left[b + 1]) {
            auto it = right[L - b - 1].find(qadd(target, qinv(kv.first, g), g));
            if (it != right[L - b - 1].end()) dims[kv.first] = std::min(kv.second, it->second);
        }
        bonds.push_back(cap(dims, D, g));
    }
    std::vector<BT> out;
    const Charge zero{};
    const Charge tinv = qinv(target, g);
    for (int64_t i = 0; i < L; ++i) {
        std::vector<int64_t> sbd, ssz;
        std::vector<Charge> cv;
        // left leg: partial charges shifted by the inverse target (site 0: one neutral
        // section); right leg: the target less the partial charge (last site: neutral)
        std::vector<std::pair<int64_t, Charge>> lq, rq;
        if (i == 0)
            lq.push_back({1, zero});
        else
            for (auto &kv : bonds[i - 1]) lq.push_back({kv.second, qadd(kv.first, tinv, g)});
        if (i == L - 1)
            rq.push_back({1, zero});
        else
            for (auto &kv : bonds[i]) rq.push_back({kv.second, qadd(target, qinv(kv.first, g), g)});
        for (auto *leg : {&lq, &phys[i], &rq}) {
            sbd.push_back(int64_t(leg->size()));
            for (auto &x : *leg) {
                ssz.push_back(x.first);
                cv.push_back(x.second);
            }
        }
        const Charge sel = i == 0 ? target : zero;
        BT t = make_tensor(g, 3, sbd.data(), ssz.data(), cv.data(), sel, F64);
        std::vector<int64_t> idx;
        int64_t nb = 0;
        for (int64_t a = 0; a < sbd[0]; ++a)
            for (int64_t s = 0; s < sbd[1]; ++s)
                for (int64_t b = 0; b < sbd[2]; ++b) {
                    const int64_t ix[3] = {a, sbd[0] + s, sbd[0] + sbd[1] + b};
                    const Charge q = qadd(qadd(cv[ix[0]], cv[ix[1]], g), cv[ix[2]], g);
                    if (qeq(q, sel, g)) {
                        idx.push_back(a);
                        idx.push_back(s);
                        idx.push_back(b);
                        ++nb;
                    }
                }
        set_blocks(t, nb, idx.data(), false, nullptr, false);
        t.alloc_data();
        if (t.nnz > 0) {
            const int64_t blocks = std::min<int64_t>((t.nnz + 255) / 256, 4096);
            k_fill_normal<<<unsigned(blocks), 256, 0, ctx().stream>>>(static_cast<double *>(t.data()), t.nnz,
                                                                      mix64(seed) ^ mix64(uint64_t(i) + 0x51ED27ull));
            count_launch();
            cuda_check(cudaGetLastError(), "random fill launch");
            const double n2 = dot_all(t, t);
            t = scale(t, 1.0 / std::sqrt(n2));
        }
        out.push_back(std::move(t));
    }
    return out;
}

}  // namespace qtt
