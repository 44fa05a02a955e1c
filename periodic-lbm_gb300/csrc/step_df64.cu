// step_df64.cu -- binary64-storage step with double-float arithmetic.
#include "plbm_launch.h"

namespace plbm {
cudaError_t step_pull_df64(int kind, const Sweep& s, const CollParams& p) {
  (void)kind; (void)s; (void)p;
  return cudaErrorNotSupported;
}
}  // namespace plbm
