// Tensor-core rotation (placeholder until the tcgen05 kernel lands).
#include "mk_common.cuh"
#include "mk_rot.cuh"

namespace mk {
bool rot_tc_supported(int64_t) { return false; }
int rot_tc_f32(const float *, const float *, int64_t, float *, int64_t, int64_t, int64_t,
               cudaStream_t) {
  set_error("tensor-core rotation is not available in this build");
  return MK_ERR_ARG;
}
}  // namespace mk
