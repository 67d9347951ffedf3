// quantit_gb300.hpp -- C++ drop-in layer over the C-ABI of libqtt_gb300.so.
//
// Mirrors QuantiT's C++ API for the block-sparse DMRG path, with the same argument
// meaning and the same exception types, so that code written against
//   quantit::btensor, quantit::tensordot / tensorgdot      (include/blockTensor/btensor.h)
//   quantit::svd / eigh / truncate                          (include/blockTensor/LinearAlgebra.h)
//   quantit::bMPS / bMPO, random_bMPS, coalesce             (include/MPT.h)
//   quantit::dmrg, dmrg_options, dmrg_logger                (include/dmrg.h, dmrg_options.h,
//                                                            dmrg_logger.h)
// compiles against this header with `namespace quantit = quantit_gb300;`.  Header only:
// link the program with -lqtt_gb300.  Block data lives on the GPU; host data crosses
// the boundary only through set_blocks / block_at / item.
//
// Exceptions (the C-ABI status codes name them): std::invalid_argument (bad shape,
// charge or disallowed block, btensor.cpp:380-395), std::out_of_range (block_at on a
// missing block), std::domain_error (throw_bad_tensor, btensor.cpp:399-404),
// std::logic_error (NaN in the 2x2 Ritz solve, dmrg.cpp:566-569; item() of a tensor
// with many elements, btensor.cpp:326-331), std::runtime_error (CUDA failures and the
// rest), and quantit_gb300::torch_check_error for the conditions QuantiT reports with
// TORCH_CHECK (c10::Error there; this layer does not depend on libtorch).
#ifndef QUANTIT_GB300_HPP
#define QUANTIT_GB300_HPP

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <exception>
#include <initializer_list>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "qtt_gb300.h"

namespace quantit_gb300 {

// ------------------------------------------------------------------ errors
// Stands in for c10::Error (TORCH_CHECK failures in the reference's tensordot checks).
struct torch_check_error : std::runtime_error {
    using std::runtime_error::runtime_error;
};

inline void check(int status) {
    if (status == QTT_OK) return;
    const std::string m = qtt_last_error();
    switch (status) {
    case QTT_ERR_INVALID_ARGUMENT: throw std::invalid_argument(m);
    case QTT_ERR_OUT_OF_RANGE: throw std::out_of_range(m);
    case QTT_ERR_DOMAIN: throw std::domain_error(m);
    case QTT_ERR_LOGIC: throw std::logic_error(m);
    case QTT_ERR_CHECK: throw torch_check_error(m);
    default: throw std::runtime_error(m);
    }
}

// ------------------------------------------------------------------ conserved quantities
// any_quantity: a product of U(1) factors (conserved::Z, int16, +) and Z(N) factors
// (conserved::C<N>, uint16 in [0, N), + mod N) -- quantity<G...> of
// include/Conserved/Composite/quantity_impl.h.  QuantiT writes the group operation as *.
class any_quantity {
  public:
    std::vector<int16_t> values;
    std::vector<uint16_t> mods;  // 0: U(1) factor, N: Z(N) factor

    any_quantity() = default;
    any_quantity(std::vector<int16_t> v, std::vector<uint16_t> m) : values(std::move(v)), mods(std::move(m)) {
        if (values.size() != mods.size() || values.empty() || values.size() > 4)
            throw std::invalid_argument("a conserved quantity has 1 to 4 factors");
    }
    any_quantity neutral() const { return any_quantity(std::vector<int16_t>(values.size(), 0), mods); }
    any_quantity inverse() const {
        any_quantity o = *this;
        for (size_t i = 0; i < values.size(); ++i)
            o.values[i] = mods[i] ? int16_t(values[i] ? mods[i] - uint16_t(values[i]) : 0) : int16_t(-values[i]);
        return o;
    }
    any_quantity operator*(const any_quantity &b) const {
        if (mods != b.mods) throw std::invalid_argument("conserved quantities of different groups");
        any_quantity o = *this;
        for (size_t i = 0; i < values.size(); ++i) {
            if (mods[i])
                o.values[i] = int16_t((uint32_t(uint16_t(values[i])) + uint16_t(b.values[i])) % mods[i]);
            else
                o.values[i] = int16_t(values[i] + b.values[i]);
        }
        return o;
    }
    bool operator==(const any_quantity &b) const { return values == b.values && mods == b.mods; }
    bool operator!=(const any_quantity &b) const { return !(*this == b); }
};
using any_quantity_cref = const any_quantity &;

namespace conserved {
inline any_quantity Z(int v) { return any_quantity({int16_t(v)}, {0}); }
// conserved::C<N>(int16) (include/Conserved/quantity.h:96): v mod N in [0, N)
template <uint16_t N>
inline any_quantity C(int v) {
    const int r = (v % int(N) + int(N)) % int(N);
    return any_quantity({int16_t(r)}, {N});
}
// quantity<A, B, ...>: the factors side by side
inline any_quantity product(std::initializer_list<any_quantity> factors) {
    any_quantity o;
    for (const any_quantity &f : factors) {
        o.values.insert(o.values.end(), f.values.begin(), f.values.end());
        o.mods.insert(o.mods.end(), f.mods.begin(), f.mods.end());
    }
    if (o.values.empty() || o.values.size() > 4) throw std::invalid_argument("a conserved quantity has 1 to 4 factors");
    return o;
}
inline any_quantity ZZ(int a, int b) { return product({Z(a), Z(b)}); }
}  // namespace conserved

// ------------------------------------------------------------------ btensor
class btensor {
  public:
    using Scalar = double;
    using index_list = std::vector<int64_t>;
    struct section {
        int64_t size;
        any_quantity charge;
    };

    btensor() = default;
    // An empty block list over the given legs (btensor(init list, selection_rule),
    // include/blockTensor/btensor.h:134-150): legs[d] = the sections of leg d.
    btensor(const std::vector<std::vector<section>> &legs, any_quantity_cref selection_rule) {
        std::vector<int64_t> sbd, ssz;
        std::vector<int16_t> cv;
        for (const auto &leg : legs) {
            sbd.push_back(int64_t(leg.size()));
            for (const section &s : leg) {
                if (s.charge.mods != selection_rule.mods)
                    throw std::invalid_argument("section charge of another group than the selection rule");
                ssz.push_back(s.size);
                cv.insert(cv.end(), s.charge.values.begin(), s.charge.values.end());
            }
        }
        qtt_bt h = nullptr;
        check(qtt_bt_create(int32_t(legs.size()), sbd.data(), ssz.data(), int32_t(selection_rule.mods.size()),
                            selection_rule.mods.data(), cv.data(), selection_rule.values.data(), QTT_F64, &h));
        h_ = own(h);
    }
    // Adopt a handle returned by the C-ABI.
    explicit btensor(qtt_bt h) : h_(own(h)) {}

    qtt_bt get() const {
        if (!h_) throw std::invalid_argument("empty btensor");
        return h_.get();
    }
    explicit operator bool() const { return bool(h_); }

    // ---- structure
    int64_t dim() const { return meta().rank; }
    std::vector<int64_t> sizes() const {
        Meta m = meta();
        std::vector<int64_t> sbd(std::max(m.rank, 1)), ssz(std::max<int64_t>(m.nsec, 1));
        std::vector<int16_t> cv(std::max<int64_t>(m.nsec * m.ncomp, 1)), sel(m.ncomp);
        std::vector<uint16_t> mods(m.ncomp);
        check(qtt_bt_structure(get(), sbd.data(), ssz.data(), cv.data(), sel.data(), mods.data()));
        std::vector<int64_t> out;
        int64_t a = 0;
        for (int d = 0; d < m.rank; ++d) {
            int64_t n = 0;
            for (int64_t s = 0; s < sbd[d]; ++s) n += ssz[a + s];
            a += sbd[d];
            out.push_back(n);
        }
        return out;
    }
    std::vector<index_list> block_indices() const {
        Meta m = meta();
        std::vector<int64_t> idx(std::max<int64_t>(m.nblocks * m.rank, 1)), numel(std::max<int64_t>(m.nblocks, 1));
        check(qtt_bt_blocks(get(), idx.data(), numel.data()));
        std::vector<index_list> out;
        for (int64_t b = 0; b < m.nblocks; ++b)
            out.emplace_back(idx.begin() + b * m.rank, idx.begin() + (b + 1) * m.rank);
        return out;
    }
    // ---- data
    // Set the block list from host data (row-major blocks), as repeated
    // btensor::block(index) = tensor would; a disallowed block throws
    // std::invalid_argument (btensor.cpp:380-395).
    btensor &set_blocks(const std::vector<std::pair<index_list, std::vector<Scalar>>> &blocks) {
        std::vector<int64_t> idx;
        std::vector<Scalar> data;
        for (const auto &b : blocks) {
            idx.insert(idx.end(), b.first.begin(), b.first.end());
            data.insert(data.end(), b.second.begin(), b.second.end());
        }
        // the sizes are checked before any data crosses to the device
        check(qtt_bt_set_block_structure(get(), int64_t(blocks.size()), idx.data()));
        if (int64_t(data.size()) != meta().nnz)
            throw std::invalid_argument("block data sizes do not match the block shapes");
        check(qtt_bt_set_blocks(get(), int64_t(blocks.size()), idx.data(), data.empty() ? nullptr : data.data()));
        return *this;
    }
    // A block list without data: the planner runs on it without a GPU.
    btensor &set_block_structure(const std::vector<index_list> &blocks) {
        std::vector<int64_t> idx;
        for (const auto &b : blocks) idx.insert(idx.end(), b.begin(), b.end());
        check(qtt_bt_set_block_structure(get(), int64_t(blocks.size()), idx.data()));
        return *this;
    }
    // The block's data (host copy); std::out_of_range when the block is absent
    // (flat_map::at, include/blockTensor/flat_map.h).
    std::vector<Scalar> block_at(const index_list &index) const {
        Meta m = meta();
        std::vector<int64_t> idx(std::max<int64_t>(m.nblocks * m.rank, 1)), numel(std::max<int64_t>(m.nblocks, 1));
        check(qtt_bt_blocks(get(), idx.data(), numel.data()));
        int64_t off = 0;
        for (int64_t b = 0; b < m.nblocks; ++b) {
            if (index_list(idx.begin() + b * m.rank, idx.begin() + (b + 1) * m.rank) == index) {
                std::vector<Scalar> all = download(m.nnz);
                return std::vector<Scalar>(all.begin() + off, all.begin() + off + numel[b]);
            }
            off += numel[b];
        }
        throw std::out_of_range("block not found in the block list");
    }
    // btensor::item (btensor.cpp:326-331): the value of a one-element tensor.
    Scalar item() const {
        Meta m = meta();
        if (m.nnz > 1 || m.nblocks > 1)
            throw std::logic_error("Only simgle block and single element tensors can be converted to scalar");
        if (m.nnz == 0) return 0.0;
        return download(1)[0];
    }

    // ---- operations (btensor.h:555-669)
    btensor tensordot(const btensor &other, const index_list &dims_self, const index_list &dims_other) const {
        if (dims_self.size() != dims_other.size())
            throw torch_check_error("both dimension lists must have the same length");
        qtt_bt o = nullptr;
        check(qtt_tensordot(get(), other.get(), int32_t(dims_self.size()), dims_self.data(), dims_other.data(), &o));
        return btensor(o);
    }
    btensor permute(const index_list &perm) const {
        if (int64_t(perm.size()) != dim()) throw std::invalid_argument("permutation of the wrong length");
        return unary([&](qtt_bt *o) { return qtt_permute(get(), perm.data(), o); });
    }
    btensor reshape(const index_list &index_groups) const {
        return unary(
            [&](qtt_bt *o) { return qtt_reshape(get(), int32_t(index_groups.size()), index_groups.data(), o); });
    }
    btensor reshape_as(const btensor &shape) const {
        return unary([&](qtt_bt *o) { return qtt_reshape_as(get(), shape.get(), o); });
    }
    btensor conj() const { return unary([&](qtt_bt *o) { return qtt_conj(get(), o); }); }
    btensor inverse_cvals() const { return unary([&](qtt_bt *o) { return qtt_inverse_cvals(get(), o); }); }
    btensor add(const btensor &other, Scalar alpha = 1) const {
        return unary([&](qtt_bt *o) { return qtt_add(get(), other.get(), alpha, o); });
    }
    btensor mul(Scalar s) const { return unary([&](qtt_bt *o) { return qtt_mul_scalar(get(), s, o); }); }
    // u.mul(d) with d the rank-1 value tensor of an svd, broadcast on the last leg
    btensor mul(const btensor &d) const {
        return unary([&](qtt_bt *o) { return qtt_mul_lastleg(get(), d.get(), o); });
    }
    // tensorgdot_ (btensor.h:626,1264): *this <- beta * *this + alpha * mul1.mul2
    btensor &tensorgdot_(const btensor &mul1, const btensor &mul2, const index_list &dims1, const index_list &dims2,
                         Scalar beta = 1, Scalar alpha = 1) {
        if (dims1.size() != dims2.size()) throw torch_check_error("both dimension lists must have the same length");
        check(qtt_tensorgdot_(get(), mul1.get(), mul2.get(), int32_t(dims1.size()), dims1.data(), dims2.data(), beta,
                              alpha));
        return *this;
    }
    btensor operator+(const btensor &o) const { return add(o); }
    btensor operator-(const btensor &o) const { return add(o, -1.0); }
    btensor operator*(Scalar s) const { return mul(s); }

  private:
    struct Deleter {
        void operator()(qtt_bt_s *h) const { qtt_bt_destroy(h); }
    };
    std::shared_ptr<qtt_bt_s> h_;
    static std::shared_ptr<qtt_bt_s> own(qtt_bt h) { return std::shared_ptr<qtt_bt_s>(h, Deleter()); }
    struct Meta {
        int32_t rank, ncomp, dtype, has_data;
        int64_t nsec, nblocks, nnz;
    };
    Meta meta() const {
        Meta m{};
        check(qtt_bt_meta(get(), &m.rank, &m.nsec, &m.ncomp, &m.nblocks, &m.nnz, &m.dtype, &m.has_data));
        return m;
    }
    std::vector<Scalar> download(int64_t n) const {
        std::vector<Scalar> v(std::max<int64_t>(n, 1));
        check(qtt_bt_download(get(), v.data(), int64_t(v.size() * sizeof(Scalar))));
        v.resize(n);
        return v;
    }
    template <class F>
    btensor unary(F &&f) const {
        qtt_bt o = nullptr;
        check(f(&o));
        return btensor(o);
    }
};

inline btensor tensordot(const btensor &a, const btensor &b, const btensor::index_list &dims_a,
                         const btensor::index_list &dims_b) {
    return a.tensordot(b, dims_a, dims_b);
}
// tensorgdot(add, mul1, mul2, dims1, dims2, beta, alpha) = beta add + alpha mul1.mul2
// (declared at btensor.h:624-627,1247-1268; addmm semantics of tensorgdot.cpp:102-117)
inline btensor tensorgdot(const btensor &add, const btensor &mul1, const btensor &mul2,
                          const btensor::index_list &dims1, const btensor::index_list &dims2,
                          btensor::Scalar beta = 1, btensor::Scalar alpha = 1) {
    if (dims1.size() != dims2.size()) throw torch_check_error("both dimension lists must have the same length");
    qtt_bt o = nullptr;
    check(qtt_tensorgdot(add.get(), mul1.get(), mul2.get(), int32_t(dims1.size()), dims1.data(), dims2.data(), beta,
                         alpha, &o));
    return btensor(o);
}

// ------------------------------------------------------------------ linear algebra
// (include/blockTensor/LinearAlgebra.h:74-247)
using svd_t = std::tuple<btensor, btensor, btensor>;
namespace detail {
inline svd_t svd_out(int status, qtt_bt U, qtt_bt d, qtt_bt V) {
    check(status);
    return svd_t(btensor(U), btensor(d), btensor(V));
}
inline int64_t clamp_size(size_t n) {
    return n > size_t(std::numeric_limits<int64_t>::max()) ? std::numeric_limits<int64_t>::max() : int64_t(n);
}
}  // namespace detail
// svd(tensor, some = true): sectors on the last two legs
inline svd_t svd(const btensor &tensor, bool some = true) {
    if (!some) throw std::invalid_argument("only the thin decomposition (some = true) is provided");
    qtt_bt U, d, V;
    return detail::svd_out(qtt_svd(tensor.get(), &U, &d, &V), U, d, V);
}
inline svd_t svd(const btensor &tensor, size_t split) {
    qtt_bt U, d, V;
    return detail::svd_out(qtt_svd_split(tensor.get(), int64_t(split), &U, &d, &V), U, d, V);
}
inline svd_t svd(const btensor &tensor, int split) { return svd(tensor, size_t(split)); }
inline svd_t svd(const btensor &A, size_t split, btensor::Scalar tol, size_t min_size, size_t max_size,
                 btensor::Scalar pow = 2) {
    qtt_bt U, d, V;
    return detail::svd_out(qtt_svd_truncate(A.get(), int64_t(split), tol, int64_t(min_size),
                                            detail::clamp_size(max_size), pow, &U, &d, &V),
                           U, d, V);
}
inline svd_t svd(const btensor &A, int split, btensor::Scalar tol, size_t min_size, size_t max_size,
                 btensor::Scalar pow = 2) {
    return svd(A, size_t(split), tol, min_size, max_size, pow);
}
// svd(A, split, tol, pow): min_size 1, no maximum (btensor_linalg.cpp:810-815)
inline svd_t svd(const btensor &A, size_t split, btensor::Scalar tol, btensor::Scalar pow = 2) {
    return svd(A, split, tol, 1, std::numeric_limits<size_t>::max(), pow);
}
inline svd_t svd(const btensor &A, int split, btensor::Scalar tol, btensor::Scalar pow = 2) {
    return svd(A, size_t(split), tol, pow);
}
inline std::tuple<btensor, btensor> eigh(const btensor &tensor, bool upper = false) {
    qtt_bt d, U;
    check(qtt_eigh(tensor.get(), upper ? 1 : 0, &d, &U));
    return {btensor(d), btensor(U)};
}
inline std::tuple<btensor, btensor> eigh(const btensor &tensor, size_t split) {
    qtt_bt d, U;
    check(qtt_eigh_split(tensor.get(), int64_t(split), &d, &U));
    return {btensor(d), btensor(U)};
}
inline svd_t truncate(const btensor &U, const btensor &d, const btensor &V, size_t max_size, size_t min_size,
                      btensor::Scalar tol, btensor::Scalar pow) {
    qtt_bt Uo, dn, Vo;
    return detail::svd_out(qtt_truncate(U.get(), d.get(), V.get(), detail::clamp_size(max_size), int64_t(min_size),
                                        tol, pow, &Uo, &dn, &Vo),
                           Uo, dn, Vo);
}

// ------------------------------------------------------------------ networks (include/MPT.h)
class bMPS : public std::vector<btensor> {
  public:
    size_t orthogonality_center = 0;
    using std::vector<btensor>::vector;
};
class bMPO : public std::vector<btensor> {
  public:
    using std::vector<btensor>::vector;
    // bMPO::coalesce (sources/MPT.cpp:154-168)
    bMPO &coalesce(btensor::Scalar cutoff = 0) {
        for (size_t i = 0; i + 1 < size(); ++i) {
            auto [U, d, V] = svd((*this)[i].permute({0, 1, 3, 2}), size_t(3), cutoff);
            (*this)[i + 1] = tensordot(V.conj(), (*this)[i + 1], {0}, {0});
            (*this)[i] = U.mul(d).permute({0, 1, 3, 2});
        }
        return *this;
    }
};

namespace detail {
inline std::vector<qtt_bt> handles(const std::vector<btensor> &v) {
    std::vector<qtt_bt> h;
    for (const btensor &t : v) h.push_back(t.get());
    return h;
}
inline btensor scalar_tensor(const any_quantity &neutral, double value) {
    btensor e(std::vector<std::vector<btensor::section>>{}, neutral);
    e.set_blocks({{{}, {value}}});
    return e;
}
// the group of a tensor (a neutral quantity of it)
inline any_quantity group_of(const btensor &t) {
    qtt_bt h = t.get();
    int32_t rank, ncomp, dtype, hd;
    int64_t nsec, nb, nnz;
    check(qtt_bt_meta(h, &rank, &nsec, &ncomp, &nb, &nnz, &dtype, &hd));
    std::vector<int64_t> sbd(std::max(rank, 1)), ssz(std::max<int64_t>(nsec, 1));
    std::vector<int16_t> cv(std::max<int64_t>(nsec * ncomp, 1)), sel(ncomp);
    std::vector<uint16_t> mods(ncomp);
    check(qtt_bt_structure(h, sbd.data(), ssz.data(), cv.data(), sel.data(), mods.data()));
    return any_quantity(std::vector<int16_t>(ncomp, 0), mods);
}
}  // namespace detail

// random_bMPS(bond_dim, mpo, constraint, seed) (include/MPT.h:49-53): N(0, 1) entries
inline bMPS random_bMPS(size_t bond_dim, const bMPO &mpo, any_quantity_cref constraint, uint64_t seed = 0) {
    std::vector<qtt_bt> in = detail::handles(mpo), out(mpo.size());
    check(qtt_random_mps(int32_t(mpo.size()), in.data(), int64_t(bond_dim), constraint.values.data(), seed,
                         out.data()));
    bMPS s;
    for (qtt_bt h : out) s.emplace_back(h);
    s.orthogonality_center = s.empty() ? 0 : s.size() - 1;
    return s;
}

// ------------------------------------------------------------------ DMRG (include/dmrg.h)
// dmrg_options (include/dmrg_options.h:15-58), plus this library's switches.
struct dmrg_options {
    btensor::Scalar cutoff = 1e-6;
    btensor::Scalar convergence_criterion = 1e-5;
    size_t maximum_bond = size_t(std::numeric_limits<int64_t>::max());
    size_t minimum_bond = 4;
    size_t maximum_iterations = 1000;
    int gemm_mode = QTT_GEMM_F64;  // QTT_GEMM_TF32X3 / QTT_GEMM_BF16X3: the mixed path
    bool final_energy_fp64 = true;
    int lanczos_steps = 1;
    bool cuda_graphs = true;
    bool svd_warm_start = true;
    dmrg_options() = default;
    dmrg_options(btensor::Scalar cut, btensor::Scalar conv, size_t max_bond, size_t min_bond, size_t max_it)
        : cutoff(cut), convergence_criterion(conv), maximum_bond(max_bond), minimum_bond(min_bond),
          maximum_iterations(max_it) {}
    qtt_dmrg_options c() const {
        qtt_dmrg_options o;
        qtt_dmrg_options_default(&o);
        o.cutoff = cutoff;
        o.convergence_criterion = convergence_criterion;
        o.maximum_bond = detail::clamp_size(maximum_bond);
        o.minimum_bond = int64_t(minimum_bond);
        o.maximum_iterations = int64_t(maximum_iterations);
        o.gemm_mode = gemm_mode;
        o.final_energy_fp64 = final_energy_fp64 ? 1 : 0;
        o.lanczos_steps = lanczos_steps;
        o.cuda_graphs = cuda_graphs ? 1 : 0;
        o.svd_warm_start = svd_warm_start ? 1 : 0;
        return o;
    }
};

// dmrg_logger (include/dmrg_logger.h:27-99); the energy is a rank-0 btensor as in
// QuantiT.  log_truncation (no reference counterpart) receives each sweep's largest
// relative discarded weight before it_log_all.
class dmrg_logger {
  public:
    virtual void log_step(size_t) = 0;
    virtual void log_energy(const btensor &) = 0;
    virtual void log_bond_dims(const bMPS &) = 0;
    virtual void log_truncation(double) {}
    virtual void init(const dmrg_options &) {}
    virtual void it_log_all(size_t step_num, const btensor &E, const bMPS &state) { log_all(step_num, E, state); }
    virtual void end_log_all(size_t step_num, const btensor &E, const bMPS &state) { log_all(step_num, E, state); }
    virtual void log_all(size_t step_num, const btensor &E, const bMPS &state) {
        log_step(step_num);
        log_energy(E);
        log_bond_dims(state);
    }
    virtual ~dmrg_logger() {}
};
class dmrg_default_logger : public dmrg_logger {
  public:
    void log_step(size_t) override {}
    void log_energy(const btensor &) override {}
    void log_bond_dims(const bMPS &) override {}
};
// the larger outer leg of the middle site (dmrg_logger.h:122-126)
inline size_t middle_bond_dim(const bMPS &mps) {
    auto s = mps[mps.size() / 2].sizes();
    return size_t(std::max(s[0], s[2]));
}
// dmrg_log_simple and dmrg_log_sweeptime (dmrg_logger.h:109-185)
class dmrg_log_simple final : public dmrg_default_logger {
  public:
    size_t it_num = 0;
    size_t middle_bond_dim = 0;
    void log_step(size_t it) override { it_num = it; }
    void log_bond_dims(const bMPS &mps) override { middle_bond_dim = quantit_gb300::middle_bond_dim(mps); }
    void it_log_all(size_t, const btensor &, const bMPS &) override {}
};
class dmrg_log_sweeptime final : public dmrg_default_logger {
  public:
    size_t it_num = 0;
    size_t middle_bond_dim = 0;
    std::chrono::steady_clock::time_point then;
    std::vector<double> time_list;
    std::vector<size_t> bond_list;
    std::vector<double> truncated_weights;
    double pending_truncation = 0.0;

    void log_step(size_t it) override { it_num = it; }
    void log_truncation(double w) override { pending_truncation = w; }
    void init(const dmrg_options &opt) override {
        then = std::chrono::steady_clock::now();
        time_list = std::vector<double>(opt.maximum_iterations);
        bond_list = std::vector<size_t>(opt.maximum_iterations);
        truncated_weights = std::vector<double>(opt.maximum_iterations);
    }
    void log_bond_dims(const bMPS &mps) override { middle_bond_dim = quantit_gb300::middle_bond_dim(mps); }
    void it_log_all(size_t it, const btensor &E0, const bMPS &mps) override {
        auto now = std::chrono::steady_clock::now();
        std::chrono::duration<double> elapsed = now - then;
        then = now;
        log_bond_dims(mps);
        if (it < bond_list.size()) {
            bond_list[it] = middle_bond_dim;
            time_list[it] = elapsed.count();
            truncated_weights[it] = pending_truncation;
        }
        log_step(it);
        log_energy(E0);
    }
};

namespace detail {
struct LogBridge {
    dmrg_logger *logger;
    const dmrg_options *options;
    any_quantity neutral;
    std::exception_ptr error;
    static bMPS state(int32_t L, const qtt_bt *mps, int64_t oc) {
        bMPS s;
        for (int32_t i = 0; i < L; ++i) {
            qtt_bt h = nullptr;
            check(qtt_bt_clone(mps[i], &h));
            s.emplace_back(h);
        }
        s.orthogonality_center = size_t(oc);
        return s;
    }
    // exceptions may not cross the C-ABI: the first one is kept and rethrown by dmrg
    template <class F>
    void guarded(F &&f) {
        if (error) return;
        try {
            f();
        } catch (...) {
            error = std::current_exception();
        }
    }
    static void init(void *u, const qtt_dmrg_options *) {
        auto *b = static_cast<LogBridge *>(u);
        b->guarded([&] { b->logger->init(*b->options); });
    }
    static void it(void *u, int64_t step, double E, double, double trunc, int32_t L, const qtt_bt *mps, int64_t oc) {
        auto *b = static_cast<LogBridge *>(u);
        b->guarded([&] {
            b->logger->log_truncation(trunc);
            b->logger->it_log_all(size_t(step), scalar_tensor(b->neutral, E), state(L, mps, oc));
        });
    }
    static void end(void *u, int64_t step, double E, int32_t L, const qtt_bt *mps, int64_t oc) {
        auto *b = static_cast<LogBridge *>(u);
        b->guarded([&] { b->logger->end_log_all(size_t(step), scalar_tensor(b->neutral, E), state(L, mps, oc)); });
    }
};
}  // namespace detail

// dmrg(bMPO&, bMPS&, const dmrg_options&, dmrg_logger&) (include/dmrg.h:39; sources/dmrg.cpp:92-100,
// 219-273): optimises the state in place, returns the energy as a rank-0 btensor.
// An exception thrown by the logger is rethrown when the driver returns.
inline btensor dmrg(bMPO &hamiltonian, bMPS &in_out_state, const dmrg_options &options, dmrg_logger &logger) {
    if (hamiltonian.size() != in_out_state.size()) throw std::invalid_argument("MPO and MPS lengths differ");
    std::vector<qtt_bt> w = detail::handles(hamiltonian), s = detail::handles(in_out_state);
    qtt_dmrg_options o = options.c();
    detail::LogBridge bridge{&logger, &options, detail::group_of(hamiltonian[0]), nullptr};
    qtt_dmrg_logger lg{&bridge, &detail::LogBridge::init, &detail::LogBridge::it, &detail::LogBridge::end};
    int64_t oc = int64_t(in_out_state.orthogonality_center);
    double E = 0.0;
    check(qtt_dmrg_logged(int32_t(w.size()), w.data(), s.data(), &oc, &o, &lg, &E));
    for (size_t i = 0; i < s.size(); ++i) in_out_state[i] = btensor(s[i]);
    in_out_state.orthogonality_center = size_t(oc);
    if (bridge.error) std::rethrow_exception(bridge.error);
    return detail::scalar_tensor(bridge.neutral, E);
}
inline btensor dmrg(bMPO &hamiltonian, bMPS &in_out_state, const dmrg_options &options) {
    dmrg_default_logger logger;
    return dmrg(hamiltonian, in_out_state, options, logger);
}
// dmrg(bMPO&, any_quantity_cref, const dmrg_options&, dmrg_logger&) (include/dmrg.h:49-50):
// from a random state of total charge `constraint` (random_bMPS at the options'
// minimum bond dimension, canonicalised at site 0), returns (energy, state).
inline std::tuple<btensor, bMPS> dmrg(bMPO &hamiltonian, any_quantity_cref constraint, const dmrg_options &options,
                                      dmrg_logger &logger, uint64_t seed = 0) {
    bMPS state = random_bMPS(std::max<size_t>(options.minimum_bond, 1), hamiltonian, constraint, seed);
    // bring the centre to site 0 (bMPS::move_oc) with untruncated sector SVDs
    while (state.orthogonality_center > 0) {
        const size_t i = state.orthogonality_center;
        auto [U, d, V] = svd(state[i], size_t(1));
        state[i] = V.conj().permute({2, 0, 1});
        state[i - 1] = tensordot(state[i - 1], U.mul(d), {2}, {0});
        state.orthogonality_center = i - 1;
    }
    btensor E = dmrg(hamiltonian, state, options, logger);
    return {E, state};
}
inline std::tuple<btensor, bMPS> dmrg(bMPO &hamiltonian, any_quantity_cref constraint, const dmrg_options &options) {
    dmrg_default_logger logger;
    return dmrg(hamiltonian, constraint, options, logger);
}

}  // namespace quantit_gb300

#endif  // QUANTIT_GB300_HPP
