// Shared helpers for the hermes_gb300 CUDA library: status/error reporting,
// launch checks and small device utilities.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/hermes_gb300.h"

namespace hermes {

// Records a printf-style message for hermes_last_error() and returns `code`.
int fail(int code, const char* fmt, ...);
// Records a CUDA error (with the failing expression) and returns HERMES_ERR_CUDA.
int cuda_fail(cudaError_t e, const char* what);

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Carves aligned sub-buffers out of a caller-owned workspace.
struct Carver {
  char* base;
  size_t used;
  size_t cap;
  explicit Carver(void* p, size_t c) : base(static_cast<char*>(p)), used(0), cap(c) {}
  template <typename T>
  T* take(size_t count, size_t align = 256) {
    used = align_up(used, align);
    T* out = reinterpret_cast<T*>(base ? base + used : nullptr);
    used += count * sizeof(T);
    return out;
  }
  bool ok() const { return used <= cap; }
};

}  // namespace hermes

#define HERMES_CUDA_TRY(expr)                                   \
  do {                                                          \
    cudaError_t _hermes_e = (expr);                             \
    if (_hermes_e != cudaSuccess) return hermes::cuda_fail(_hermes_e, #expr); \
  } while (0)

#define HERMES_LAUNCH_CHECK(what)                               \
  do {                                                          \
    cudaError_t _hermes_e = cudaGetLastError();                 \
    if (_hermes_e != cudaSuccess) return hermes::cuda_fail(_hermes_e, what); \
  } while (0)

// ---- device helpers --------------------------------------------------------
__device__ __forceinline__ int wrap_mod(int v, int L) {  // L is a power of two
  return v & (L - 1);
}
