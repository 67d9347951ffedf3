// Contraction planner interface.
#pragma once
#include <vector>

#include "qtt_core.h"

namespace qtt {

// Everything tensordot needs besides the data: output structure (bit-exact block
// list of btensor::tensordot), the matched pairs per output block in
// accumulation order, and how each operand is read.
struct ContractPlan {
    std::vector<int64_t> dA, dB, freeA, freeB, p1, p2;
    std::vector<int64_t> p2p;  // B legs as (free, contracted): B blocks in (N x K) matrix form
    BT out;                               // structure and compact offsets
    std::vector<int64_t> pair_a, pair_b;  // source blocks of each matched pair
    std::vector<int64_t> out_p0, out_p1;  // pair range of each output block
    int a_mode = 0;  // 0: A block is (free x contracted) row-major, 1: stored transposed, 2: packed
    int b_mode = 0;  // 0: B block is (contracted x free) row-major, 1: stored transposed, 2: packed
};

// The merge-join on the device (planner.cu): fills the pair tables and the output
// block list of P, whose legs, permutations and output sections are set.  Returns 1
// when done, 0 when the inputs exceed the device planner's limits (nothing filled),
// -1 when a contracted section pair fails the charge (or, with *bad_size, the size)
// check, at contracted dimension *bad_dim.
int plan_join_device(ContractPlan &P, const BT &A, const BT &B, int *bad_dim, bool *bad_size);

ContractPlan plan_contraction(const BT &A, const BT &B, const std::vector<int64_t> &dA,
                              const std::vector<int64_t> &dB);
// Run the grouped GEMM of a plan into out (whose offsets index out's buffer).
// add / add_block: optional beta*add term per output block (-1: none).
void run_contraction(const ContractPlan &P, const BT &A, const BT &B, BT &out, const BT *add, double beta,
                     double alpha, const std::vector<int64_t> *add_block);

}  // namespace qtt
