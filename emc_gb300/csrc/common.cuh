// Internal definitions shared by the CUDA translation units of libemc_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>
#include <string>

#include "../../include/emc_gb300.h"

struct emc_ctx {
  int device = 0;
  int sm_count = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  long long launches = 0;
  // Small reusable device scratch owned by the context (reductions).
  void* scratch = nullptr;
  size_t scratch_bytes = 0;
  // Pinned host staging for synchronous scalar results.
  void* host_pinned = nullptr;
  std::string last_error = "ok";
};

namespace emc {

// Records an error message on the context and returns `code`.
inline int fail(emc_ctx* ctx, int code, const char* fmt, ...) {
  if (ctx) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    ctx->last_error = buf;
  }
  return code;
}

inline int cuda_fail(emc_ctx* ctx, cudaError_t e, const char* where) {
  return fail(ctx, EMC_ERR_CUDA, "%s: %s", where, cudaGetErrorString(e));
}

// Checks the launch that was just queued and counts it.
inline int after_launch(emc_ctx* ctx, const char* name) {
  ctx->launches++;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(ctx, e, name);
  return EMC_OK;
}

// Grows the context scratch to at least `bytes` (synchronises on growth).
int ensure_scratch(emc_ctx* ctx, size_t bytes);

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

}  // namespace emc

#define EMC_CHECK_CTX(ctx) \
  do {                     \
    if (!(ctx)) return EMC_ERR_INVALID; \
  } while (0)

#define EMC_REQUIRE(ctx, cond, ...)                              \
  do {                                                           \
    if (!(cond)) return emc::fail((ctx), EMC_ERR_INVALID, __VA_ARGS__); \
  } while (0)

#define EMC_CUDA(ctx, call)                                   \
  do {                                                        \
    cudaError_t _e = (call);                                  \
    if (_e != cudaSuccess) return emc::cuda_fail((ctx), _e, #call); \
  } while (0)
