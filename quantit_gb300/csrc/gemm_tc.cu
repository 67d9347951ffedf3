// Split-precision grouped block GEMM on tcgen05 tensor cores (placeholder until
// the kernel lands: the call fails loudly, it never falls back).
#include "kernels.h"
#include "qtt_core.h"

namespace qtt {
int gemm_tile_m(int) { return 128; }
int gemm_tile_n(int) { return 64; }
void launch_gemm_tc(const GemmArgs &, int) { fail(ERR_RUNTIME, "the tensor-core GEMM path is not built"); }
}  // namespace qtt
