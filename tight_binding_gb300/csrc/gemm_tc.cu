// gemm_tc.cu — mu_nm on the tensor cores (placeholder until the tcgen05 kernel lands).
#include "tbk_internal.h"

namespace tbk {
int mu_gemm_tc(const float2*, const float2*, int32_t, int64_t, int64_t, double*, cudaStream_t) {
  return fail(TBK_ERR_UNSUPPORTED, "tensor-core mu_nm GEMM not available in this build");
}
}  // namespace tbk
