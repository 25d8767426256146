// blocks_tc.cu -- tensor-core (tcgen05) block engine.  Placeholder until the
// split-BF16x3 kernel lands: reports no support, so AUTO uses the SIMT engine.
#include "common.cuh"

namespace qcs {

bool tc_supported(const qcs_cuda_state *, int) { return false; }

int apply_block_tc(qcs_cuda_state *, int, const int *, const double *) {
  return set_error(QCS_CUDA_EUNSUP, "tensor-core block engine not built");
}

}  // namespace qcs
