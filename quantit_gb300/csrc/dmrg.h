// DMRG building blocks and driver.
#pragma once
#include <vector>

#include "ops_util.h"
#include "qtt_core.h"

namespace qtt {

struct DmrgOpts {
    double cutoff = 1e-6;
    double convergence_criterion = 1e-5;
    int64_t maximum_bond = INT64_MAX;
    int64_t minimum_bond = 4;
    int64_t maximum_iterations = 1000;
    int gemm_mode = GEMM_F64;
    int final_energy_fp64 = 1;  // mixed modes: return the FP64 <psi|H|psi>/<psi|psi> of the final state
    int lanczos_steps = 1;      // 1: QuantiT's one-step update; k > 1: k-step Lanczos (lanczos_k)
    int cuda_graphs = 1;        // k-step Lanczos: replay the matvec from a captured CUDA graph
    int svd_warm_start = 1;     // start each bond's sector SVD from its previous rotation (this call)
};
// k-step Lanczos with full reorthogonalisation: the lowest Ritz value and its
// (normalised) Ritz vector of the two-site effective Hamiltonian.
struct LanczosKOut {
    BT psi;
    double E = 0.0;
    int dim = 0;  // Krylov dimension used (smaller than k after a breakdown)
};
LanczosKOut lanczos_k(const BT &state, const BT &hamil, const BT &L, const BT &R, int k, bool graphs = true);
// Sweep hooks of the driver (dmrg_logger, include/dmrg_logger.h:27-99): `sweep` after
// every sweep (it_log_all) with the sweep's largest relative discarded weight
// (sum of dropped s^2 / sum of all s^2 over its bonds' truncations), `done` once when
// the driver stops (end_log_all).  mps is the current state, oc its centre.
struct DmrgHooks {
    void *user = nullptr;
    void (*sweep)(void *user, int64_t it, double E, double seconds, double trunc, const std::vector<BT> &mps,
                  int64_t oc) = nullptr;
    void (*done)(void *user, int64_t it, double E, const std::vector<BT> &mps, int64_t oc) = nullptr;
};

struct LanczosOut {
    BT psi;
};
struct LanczosHost {
    BT psi;
    double a0 = 0, a1 = 0, b = 0;
};

BT compute_2sites_hamil(const BT &wl, const BT &wr);
BT hamil2site_times_state(const BT &state, const BT &hamil, const BT &L, const BT &R);
BT compute_left_env(const BT &W, const BT &A, const BT &L);
BT compute_right_env(const BT &W, const BT &A, const BT &R);
void eig2x2(double a0, double a1, double b, double &E, double &o, double &n);
LanczosOut one_step_lanczos_dev(const BT &state, const BT &hamil, const BT &L, const BT &R, double *scal,
                                DevScratch &scr);
LanczosHost one_step_lanczos(const BT &state, const BT &hamil, const BT &L, const BT &R);
double dmrg(const std::vector<BT> &mpo, std::vector<BT> &mps, int64_t &oc, const DmrgOpts &opt,
            const DmrgHooks &hooks = DmrgHooks());
// the all-ones rank-3 edge environment over leg sleg of st and leg wleg of w
// (generate_env_impl, dmrg.cpp:371-391; edge_shape_prep :335-345)
BT trivial_edge(const BT &st, int sleg, const BT &w, int wleg);
double mps_energy(const std::vector<BT> &mpo, const std::vector<BT> &mps, double *norm2);

}  // namespace qtt
