// Status strings, device properties and the library version.
#include <stdarg.h>
#include <string.h>

#include <map>
#include <mutex>
#include <utility>

#include "mk_common.cuh"

namespace mk {

static thread_local char g_err[512] = "no error";

void set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int sm_count() {
  static int cached[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
  if (cached[dev] == 0) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
      n = 152;
    cached[dev] = n;
  }
  return cached[dev];
}

int resident_ctas(const void *kernel, int block, size_t smem) {
  static std::mutex mu;
  static std::map<std::pair<const void *, long long>, int> cache;
  const long long key2 = ((long long)block << 32) | (long long)smem;
  std::lock_guard<std::mutex> lock(mu);
  auto it = cache.find({kernel, key2});
  if (it != cache.end()) return it->second;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, block, smem) != cudaSuccess || n < 1) {
    cudaGetLastError();
    n = 1;
  }
  cache[{kernel, key2}] = n;
  return n;
}

int launch_status(const char *what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("%s: kernel launch failed: %s", what, cudaGetErrorString(e));
    return MK_ERR_CUDA;
  }
  return MK_OK;
}

}  // namespace mk

extern "C" const char *mk_last_error(void) { return mk::g_err; }

extern "C" int mk_version(void) { return 1; }
