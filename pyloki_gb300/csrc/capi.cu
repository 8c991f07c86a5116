// Library-level C ABI: version and per-thread error reporting.
#include <stdarg.h>
#include <stdio.h>

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
