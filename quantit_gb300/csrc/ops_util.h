// Helpers shared by the host-layer translation units.
#pragma once
#include <vector>

#include "kernels.h"
#include "qtt_core.h"

namespace qtt {

std::vector<Chunk> make_chunks(const std::vector<int64_t> &lens);
void require_f64(const BT &t);
bool same_shape(const BT &a, const BT &b);
std::vector<int64_t> sorted_order(const BT &t);

// Union of two block lists in lexicographic order: for each output block, the
// source block in a and in b (-1 when absent).
struct UnionPlan {
    std::vector<int64_t> idx;
    std::vector<int64_t> a, b;
};
UnionPlan union_plan(const BT &a, const BT &b);

// Short-lived device scratch buffers released (stream-ordered) with the object.
struct DevScratch {
    std::vector<BufPtr> bufs;
    double *get(size_t n);
    double *get_result();
};

// Device-scalar variants used by the DMRG pipeline (no host synchronisation).
BT add_scaled_dev(const BT &a, const BT &b, Coef ca, Coef cb);
BT scale_dev(const BT &a, Coef c);
void dot_all_dev(const BT &a, const BT &b, double *dev_out, DevScratch &scr);

}  // namespace qtt
