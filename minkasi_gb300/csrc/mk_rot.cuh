// Detector-space rotation R = A . X on the tensor cores (FP32 in/out,
// 3xTF32 split products, FP32 accumulation).  A is (nrow x nrow), X is
// (nrow x ncol) with leading dimension ldx, R has leading dimension ldr; all
// row-major.  Used by apply_noise for the v / vT rotations.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace mk {
// true when the tensor-core kernel handles this detector count
bool rot_tc_supported(int64_t nrow);
int rot_tc_f32(const float *A, const float *X, int64_t ldx, float *R, int64_t ldr, int64_t nrow,
               int64_t ncol, cudaStream_t st);
}  // namespace mk
