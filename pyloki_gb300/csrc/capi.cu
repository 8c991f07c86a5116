// Library-level C ABI: version and per-thread error reporting.
#include <stdarg.h>
#include <stdio.h>

#include <map>
#include <mutex>
#include <utility>

#include "loki_common.cuh"

namespace loki {

static thread_local char g_last_error[512] = "";
static thread_local long long g_launches = 0;

void note_launch() { ++g_launches; }

int set_error(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return code;
}

// Largest dynamic shared-memory limit set so far per (device, kernel). The
// limit is only ever raised, under one lock, so a host thread launching a
// kernel with a smaller tile can never lower it below what another thread's
// launch of the same kernel needs. The attribute is set on every call (a
// context created after a device reset starts from the default again).
static std::mutex g_smem_mu;
static std::map<std::pair<int, const void*>, int> g_smem_limit;

cudaError_t raise_smem_limit(const void* func, int bytes) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(g_smem_mu);
  int& cur = g_smem_limit[{dev, func}];
  if (bytes > cur) cur = bytes;
  return cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, cur);
}

int check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return LOKI_OK;
}

}  // namespace loki

extern "C" int loki_version(void) { return 1; }

extern "C" const char* loki_last_error(void) { return loki::g_last_error; }

extern "C" int64_t loki_launch_count(void) { return loki::g_launches; }
