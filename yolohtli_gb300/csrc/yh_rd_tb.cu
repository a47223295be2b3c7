// Temporally blocked reaction-diffusion step (several steps per launch).
#include "yh_kernels.cuh"

namespace yh {

int rd_tb_max_steps() { return 1; }

cudaError_t launch_rd_tb(const StepCoeffs<float> &, const Fld<float> &,
                         const Fld<float> &, const uint8_t *, int,
                         cudaStream_t) {
  return cudaErrorNotSupported;
}

}  // namespace yh
