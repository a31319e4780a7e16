// Library-wide C ABI pieces: version, thread-local error message.
#include <stdarg.h>
#include <stdio.h>

#include "hermes_common.cuh"

namespace hermes {

static thread_local char g_last_error[1024] = "";

int fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(HERMES_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e),
              cudaGetErrorString(e));
}

}  // namespace hermes

extern "C" const char* hermes_version(void) { return "hermes_gb300 0.1.0 (sm_103a)"; }

extern "C" const char* hermes_last_error(void) { return hermes::g_last_error; }
