// FP64 detector rotation by exact integer slices on the bf16 tensor cores
// (see mk_ozaki.cu).  R (nrow x ncol, ld ldr) = A (nrow x nrow) . X (nrow x
// ncol, ld ldx), all row-major FP64.
#pragma once
#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace mk {
constexpr int64_t OZ_BLOCK = 65536;  // sample columns per block of slices
// true when the slice products of nrow-long sums stay exact in FP32
bool ozaki_supported(int64_t nrow);
// scratch bytes of one call (any ncol: columns go in blocks of OZ_BLOCK)
size_t ozaki_ws_bytes(int64_t nrow);
// stream-ordered on st; uses the cuBLAS handle h (the caller serialises it)
int ozaki_rotate_f64(cublasHandle_t h, const double *A, const double *X, int64_t ldx, double *R, int64_t ldr,
                     int64_t nrow, int64_t ncol, void *ws, size_t ws_bytes, cudaStream_t st);
}  // namespace mk
