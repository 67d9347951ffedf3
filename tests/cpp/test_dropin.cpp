// C++ drop-in layer test (include/quantit_gb300.hpp), built with g++ by
// tests/test_cpp_dropin.py.  `structure` runs without a GPU: the planner on
// structure-only tensors and the exception types QuantiT throws.  `numeric` needs
// the GPU: contraction values, an SVD reconstruction, and the two dmrg overloads
// with a logger on an L = 8 Heisenberg chain (the energy is printed for the caller
// to check against exact diagonalisation).
#include <cmath>
#include <cstdio>
#include <string>

#include "quantit_gb300.hpp"

namespace quantit = quantit_gb300;
using quantit::btensor;
using quantit::conserved::Z;

static int failures = 0;
#define EXPECT(cond)                                              \
    do {                                                          \
        if (!(cond)) {                                            \
            std::printf("FAILED line %d: %s\n", __LINE__, #cond); \
            ++failures;                                           \
        }                                                         \
    } while (0)

template <class E, class F>
static bool throws(F &&f) {
    try {
        f();
    } catch (const E &) {
        return true;
    } catch (...) {
        return false;
    }
    return false;
}

static void structure_cases() {
    // btensor::block on a disallowed index throws std::invalid_argument (btensor.cpp:380-395)
    btensor a({{{2, Z(0)}, {3, Z(1)}}, {{2, Z(0)}, {3, Z(-1)}}}, Z(0));
    EXPECT(throws<std::invalid_argument>([&] { a.set_block_structure({{0, 1}}); }));
    a.set_block_structure({{0, 0}, {1, 1}});
    EXPECT(a.block_indices().size() == 2);
    EXPECT(a.dim() == 2 && a.sizes() == (std::vector<int64_t>{5, 5}));
    // block_at on a missing block: std::out_of_range
    EXPECT(throws<std::out_of_range>([&] { a.block_at({0, 1}); }));
    // contractions QuantiT rejects with TORCH_CHECK
    btensor b({{{4, Z(0)}}, {{1, Z(0)}}}, Z(0));
    b.set_block_structure({{0, 0}});
    EXPECT(throws<quantit::torch_check_error>([&] { a.tensordot(b, {1, 0}, {0}); }));
    EXPECT(throws<std::exception>([&] { a.tensordot(b, {1}, {0}); }));
    // a valid structure-only contraction: the block list of the product
    btensor c({{{2, Z(0)}, {3, Z(1)}}, {{4, Z(0)}, {3, Z(-1)}}}, Z(0));
    c.set_block_structure({{0, 0}, {1, 1}});
    btensor ct({{{4, Z(0)}, {3, Z(1)}}, {{2, Z(0)}}}, Z(0));
    ct.set_block_structure({{0, 0}});
    btensor p = c.tensordot(ct, {1}, {0});
    EXPECT(p.block_indices() == (std::vector<btensor::index_list>{{0, 0}}));
    // item() of a tensor with many elements: std::logic_error (btensor.cpp:326-331)
    EXPECT(throws<std::logic_error>([&] { c.item(); }));
    // conserved quantities
    EXPECT((Z(3) * Z(-5)) == Z(-2));
    EXPECT(quantit::conserved::C<5>(-2) == quantit::conserved::C<5>(3));
    EXPECT((quantit::conserved::ZZ(1, 2) * quantit::conserved::ZZ(1, 2).inverse()) == quantit::conserved::ZZ(0, 0));
}

// Heisenberg_impl's 5 x 2 x 5 x 2 site tensor (sources/models.cpp:38-68) as blocks:
// H = sum S.S (the reference's J = -1).  Channels 0..4 = {done, S- placed, S+ placed,
// Sz placed, nothing placed}; the left edge is channel 4, the right edge channel 0.
static quantit::bMPO heisenberg(int L) {
    double W[5][2][5][2] = {};  // W[a][s][b][t], basis {up, down}
    auto set = [&](int a, int b, const double m[2][2]) {
        for (int s = 0; s < 2; ++s)
            for (int t = 0; t < 2; ++t) W[a][s][b][t] = m[s][t];
    };
    const double I[2][2] = {{1, 0}, {0, 1}}, Sp[2][2] = {{0, 1}, {0, 0}}, Sm[2][2] = {{0, 0}, {1, 0}},
                 Sz[2][2] = {{0.5, 0}, {0, -0.5}}, hSp[2][2] = {{0, 0.5}, {0, 0}}, hSm[2][2] = {{0, 0}, {0.5, 0}};
    set(0, 0, I);
    set(1, 0, Sm);
    set(2, 0, Sp);
    set(3, 0, Sz);
    set(4, 1, hSp);
    set(4, 2, hSm);
    set(4, 3, Sz);
    set(4, 4, I);
    // channel charges (2Sz): 1 -> +2, 2 -> -2, the others 0; sections in ascending charge
    const int order[5] = {2, 0, 3, 4, 1};
    const int qsec[3] = {-2, 0, 2}, nsec[3] = {1, 3, 1}, first[3] = {0, 1, 4};
    // physical sections in ascending charge: 2Sz = -1 (down, basis 1), +1 (up, basis 0)
    const int phys_state[2] = {1, 0}, phys_q[2] = {-1, 1};
    quantit::bMPO mpo;
    for (int i = 0; i < L; ++i) {
        const bool first_site = i == 0, last_site = i == L - 1;
        std::vector<std::vector<btensor::section>> legs(4);
        if (first_site)
            legs[0] = {{1, Z(0)}};
        else
            for (int s = 0; s < 3; ++s) legs[0].push_back({nsec[s], Z(qsec[s])});
        legs[1] = {{1, Z(phys_q[0])}, {1, Z(phys_q[1])}};
        if (last_site)
            legs[2] = {{1, Z(0)}};
        else
            for (int s = 0; s < 3; ++s) legs[2].push_back({nsec[s], Z(-qsec[s])});
        legs[3] = {{1, Z(-phys_q[0])}, {1, Z(-phys_q[1])}};
        btensor w(legs, Z(0));
        std::vector<std::pair<btensor::index_list, std::vector<double>>> blocks;
        const int nl = first_site ? 1 : 3, nr = last_site ? 1 : 3;
        for (int ls = 0; ls < nl; ++ls)
            for (int ps = 0; ps < 2; ++ps)
                for (int rs = 0; rs < nr; ++rs)
                    for (int ts = 0; ts < 2; ++ts) {
                        const int ql = first_site ? 0 : qsec[ls], qr = last_site ? 0 : -qsec[rs];
                        if (ql + phys_q[ps] + qr - phys_q[ts] != 0) continue;
                        const int a0 = first_site ? 3 : first[ls], a1 = first_site ? 4 : first[ls] + nsec[ls];
                        const int b0 = last_site ? 1 : first[rs], b1 = last_site ? 2 : first[rs] + nsec[rs];
                        std::vector<double> v;
                        bool nz = false;
                        for (int a = a0; a < a1; ++a)
                            for (int b = b0; b < b1; ++b) {
                                v.push_back(W[order[a]][phys_state[ps]][order[b]][phys_state[ts]]);
                                nz = nz || v.back() != 0.0;
                            }
                        if (nz) blocks.push_back({{ls, ps, rs, ts}, v});
                    }
        w.set_blocks(blocks);
        mpo.push_back(w);
    }
    return mpo;
}

struct CountingLogger : quantit::dmrg_default_logger {
    int inits = 0, its = 0, ends = 0;
    double last_E = 0.0;
    void init(const quantit::dmrg_options &) override { ++inits; }
    void it_log_all(size_t, const btensor &E, const quantit::bMPS &s) override {
        ++its;
        last_E = E.item();
        EXPECT(s.size() == 8);
    }
    void end_log_all(size_t, const btensor &E, const quantit::bMPS &) override {
        ++ends;
        last_E = E.item();
    }
};

static void numeric_cases() {
    // contraction values: C = A B of two single-block matrices
    btensor A({{{2, Z(0)}}, {{3, Z(0)}}}, Z(0));
    A.set_blocks({{{0, 0}, {1, 2, 3, 4, 5, 6}}});
    btensor B({{{3, Z(0)}}, {{2, Z(0)}}}, Z(0));
    B.set_blocks({{{0, 0}, {1, 0, 0, 1, 1, 1}}});
    btensor C = quantit::tensordot(A, B, {1}, {0});
    std::vector<double> c = C.block_at({0, 0});
    EXPECT(c.size() == 4 && std::fabs(c[0] - 4) < 1e-14 && std::fabs(c[1] - 5) < 1e-14 &&
           std::fabs(c[2] - 10) < 1e-14 && std::fabs(c[3] - 11) < 1e-14);
    // tensorgdot: 0.5 C + 2 A B = 2.5 C
    btensor G = quantit::tensorgdot(C, A, B, {1}, {0}, 0.5, 2.0);
    EXPECT(std::fabs(G.block_at({0, 0})[3] - 27.5) < 1e-13);
    // svd: U d V^T reconstructs A
    auto [U, d, V] = quantit::svd(A, size_t(1));
    std::vector<double> r = U.mul(d).tensordot(V.conj(), {1}, {1}).block_at({0, 0});
    for (int i = 0; i < 6; ++i) EXPECT(std::fabs(r[i] - (i + 1)) < 1e-12);
    // dmrg on the L = 8 Heisenberg chain, both overloads, with loggers
    quantit::bMPO H = heisenberg(8);
    quantit::dmrg_options opt(1e-12, 1e-13, 16, 4, 30);
    CountingLogger lg;
    auto [E, state] = quantit::dmrg(H, Z(0), opt, lg);
    EXPECT(lg.inits == 1 && lg.ends == 1 && lg.its >= 2);
    EXPECT(std::fabs(lg.last_E - E.item()) < 1e-12);
    quantit::dmrg_log_sweeptime st;
    quantit::bMPS s2 = state;
    btensor E2 = quantit::dmrg(H, s2, quantit::dmrg_options(1e-12, 0.0, 16, 4, 2), st);
    EXPECT(st.time_list.size() == 2 && st.bond_list[1] > 0);
    // a logger's exception reaches the caller after the driver returns
    struct Throwing : quantit::dmrg_default_logger {
        void it_log_all(size_t, const btensor &, const quantit::bMPS &) override {
            throw std::domain_error("from the logger");
        }
    } th;
    quantit::bMPS s3 = state;
    EXPECT(throws<std::domain_error>([&] { quantit::dmrg(H, s3, quantit::dmrg_options(1e-12, 0.0, 16, 4, 1), th); }));
    std::printf("ENERGY %.15f %.15f\n", E.item(), E2.item());
}

int main(int argc, char **argv) {
    const std::string mode = argc > 1 ? argv[1] : "structure";
    if (mode == "structure") {
        structure_cases();
    } else if (mode == "numeric") {
        quantit::check(qtt_init(0));
        numeric_cases();
    } else {
        std::printf("usage: test_dropin structure|numeric\n");
        return 2;
    }
    std::printf("%s: %d failure(s)\n", mode.c_str(), failures);
    return failures ? 1 : 0;
}
