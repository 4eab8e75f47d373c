// Detector-space rotation R = A . X on the tensor cores (FP32 in/out,
// 3xTF32 split products, FP32 accumulation).  A is (nrow x nrow), X is
// (nrow x ncol) with leading dimension ldx, R has leading dimension ldr; all
// row-major.  Used by apply_noise for the v / vT rotations.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace mk {
// true when the tensor-core kernel handles this detector count
bool rot_tc_supported(int64_t nrow);
// bytes of the operand image the kernel stages A from (16-byte aligned buffer)
size_t rot_tc_bimg_bytes(int64_t nrow);
// `err` is a device int set to 1 if a bounded wait inside the kernel timed out.
// mirror_n > 0 (= 2(ncol-1), with ldr >= mirror_n) also writes the even
// extension R[., mirror_n - j] = R[., j], 1 <= j <= ncol-2, for a DCT-I.
// x_stride 2 reads X[r][j] at X + r*ldx + 2j (the real parts of an
// interleaved complex array); halve_ends scales columns 0 and ncol-1 by 1/2.
int rot_tc_f32(const float *A, const float *X, int64_t ldx, float *R, int64_t ldr, int64_t nrow,
               int64_t ncol, void *bimg, int *err, cudaStream_t st, int64_t mirror_n = 0,
               int64_t x_stride = 1, int halve_ends = 0);

// One TOD of a grouped rotation: R = A . X with A given by its operand image
// bimg (rot_tc_bprep); tile0 = the first of its ceil(ncol / 128) tiles in the
// launch (jobs sorted by tile0, contiguous).  R may equal X (in place): the
// kernel reads all of a tile's inputs before it writes that tile.
struct RotJob {
  const float *X;
  float *R;
  const char *bimg;
  int64_t ldx, ldr, ncol, tile0;
};
// the operand image of A (rot_tc_bimg_bytes(nrow) bytes)
int rot_tc_bprep(const float *A, int64_t nrow, void *bimg, cudaStream_t st);
// every job of the (device) table in one launch; all jobs have nrow detectors
int rot_tc_group(const RotJob *jobs_dev, int njobs, int64_t ntile, int64_t nrow, int *err, cudaStream_t st);
}  // namespace mk
