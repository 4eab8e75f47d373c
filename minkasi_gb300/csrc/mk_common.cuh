// Shared helpers for libmkgpu: status handling, dtype dispatch, launch sizing.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/mkgpu.h"

namespace mk {

// Last error message of the calling host thread (mk_last_error()).
void set_error(const char *fmt, ...);

// SM count of the current device, cached per device.
int sm_count();

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// CTAs of `kernel` that fit on one SM at `block` threads and `smem` bytes of
// dynamic shared memory (occupancy calculator; cached, the same on every
// device of one architecture).
int resident_ctas(const void *kernel, int block, size_t smem);

// Status of the last launch on this thread, folded into an MK status.
int launch_status(const char *what);

}  // namespace mk

#define MK_CHECK_ARG(cond, ...)        \
  do {                                 \
    if (!(cond)) {                     \
      mk::set_error(__VA_ARGS__);      \
      return MK_ERR_ARG;               \
    }                                  \
  } while (0)

#define MK_CUDA(call)                                                          \
  do {                                                                         \
    cudaError_t _e = (call);                                                   \
    if (_e != cudaSuccess) {                                                   \
      mk::set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(_e),    \
                    __FILE__, __LINE__);                                       \
      return MK_ERR_CUDA;                                                      \
    }                                                                          \
  } while (0)

#define MK_DTYPE_OK(dt) ((dt) == MK_F64 || (dt) == MK_F32)

// Grid size for a grid-stride kernel: enough CTAs to fill every SM `per_sm`
// times, capped by the work available.
inline unsigned mk_grid(int64_t work_items, int block, int per_sm) {
  int64_t need = (work_items + block - 1) / block;
  int64_t cap = (int64_t)mk::sm_count() * per_sm;
  if (need < 1) need = 1;
  return (unsigned)(need < cap ? need : cap);
}

// Grid size for a grid-stride kernel: exactly one wave of resident CTAs
// (registers and shared memory decide how many fit per SM), so that no CTA
// waits for a second wave and runs in a tail at low occupancy.
template <typename Kern>
inline unsigned mk_grid_fit(Kern *kernel, int64_t work_items, int block, size_t smem = 0) {
  return mk_grid(work_items, block, mk::resident_ctas((const void *)kernel, block, smem));
}
