// Per-pattern log-sum-exp normalisation of the responsibilities (rows A7-A9).
//
// Reference: cuda_calculate_max_vectors_kernel (emc_cuda.cu:1041-1056),
// cuda_respons_max_expf_kernel (:1175-1217), cuda_norm_respons_sumexpf_kernel
// (:1253-1272) and the host step lse = log(sum) + max (main.cpp:384-391,
// emc_helper.cpp:579-587).  The reference gives each pattern one block that
// walks a column of the rotation-major [r*N + i] matrix (stride N: one
// 4-byte load per 128-byte line) and allocates an R x N temporary per call.
// Here a thread owns one pattern and a block row owns a range of rotations,
// so each warp reads 128 contiguous bytes per rotation; the partial results of
// the rotation ranges (one float per range and pattern) are folded by a
// second small kernel in range order.  Nothing is allocated per call: the
// partials live in the context scratch.
//
// Results: the max is identical to the reference's (max is order free; NaN
// entries are skipped by the same "<" test, -1e10 is the floor).  The sums
// use a different order than the reference's 512-way tree and so agree to
// float rounding.
#include <algorithm>
#include <mutex>

#include "common.cuh"

namespace emc {

constexpr int kLseThreads = 256;

__host__ __device__ inline int lse_range_rows(int n_slices) {
  int rc = 64;
  while ((n_slices + rc - 1) / rc > 65535) rc *= 2;
  return rc;
}

__global__ void __launch_bounds__(kLseThreads) max_partial_kernel(
    const float* __restrict__ respons, int n_images, int n_slices, int rc,
    float* __restrict__ part) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_images) return;
  const int r0 = blockIdx.y * rc;
  const int r1 = min(n_slices, r0 + rc);
  float m = -1.0e10f;
  for (int r = r0; r < r1; ++r) {
    const float v = __ldg(respons + (size_t)r * n_images + i);
    if (m < v) m = v;
  }
  part[(size_t)blockIdx.y * n_images + i] = m;
}

__global__ void __launch_bounds__(kLseThreads) max_final_kernel(const float* __restrict__ part,
                                                                int n_images, int nb,
                                                                float* __restrict__ maxr) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_images) return;
  float m = -1.0e10f;
  for (int b = 0; b < nb; ++b) {
    const float v = part[(size_t)b * n_images + i];
    if (m < v) m = v;
  }
  maxr[i] = m;
}

__global__ void __launch_bounds__(kLseThreads) sumexp_partial_kernel(
    const float* __restrict__ respons, const float* __restrict__ maxv, int n_images,
    int n_slices, int rc, float* __restrict__ part) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_images) return;
  const int r0 = blockIdx.y * rc;
  const int r1 = min(n_slices, r0 + rc);
  const float m = __ldg(maxv + i);
  float s = 0.0f;
  for (int r = r0; r < r1; ++r) {
    const float d = __fsub_rn(__ldg(respons + (size_t)r * n_images + i), m);
    if (d > -1.0e10f) s = __fadd_rn(s, expf(d));
  }
  part[(size_t)blockIdx.y * n_images + i] = s;
}

__global__ void __launch_bounds__(kLseThreads) sum_final_kernel(const float* __restrict__ part,
                                                                int n_images, int nb,
                                                                float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_images) return;
  float s = 0.0f;
  for (int b = 0; b < nb; ++b) s = __fadd_rn(s, part[(size_t)b * n_images + i]);
  out[i] = s;
}

__global__ void norm_kernel(float* __restrict__ respons, const float* __restrict__ lse,
                            int n_images, long long total) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += stride) {
    const int i = (int)(e % n_images);
    respons[e] = expf(__fsub_rn(respons[e], __ldg(lse + i)));
  }
}

__global__ void log_sum_max_kernel(const float* __restrict__ sum, const float* __restrict__ maxv,
                                   float* __restrict__ lse, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) lse[i] = __fadd_rn(logf(sum[i]), maxv[i]);
}

}  // namespace emc

extern "C" int emc_max_vector(emc_ctx* ctx, const float* d_respons, int N_images, int n_slices,
                              float* d_maxr) {
  EMC_CHECK_CTX(ctx);
  EMC_REQUIRE(ctx, d_respons && d_maxr, "max_vector: null pointer");
  EMC_REQUIRE(ctx, N_images >= 0 && n_slices >= 0, "max_vector: bad sizes");
  if (N_images == 0) return EMC_OK;
  const int rc = emc::lse_range_rows(n_slices);
  const int nb = n_slices > 0 ? emc::ceil_div(n_slices, rc) : 0;
  const int gx = emc::ceil_div(N_images, emc::kLseThreads);
  if (nb > 0) {
    int rcode = emc::ensure_scratch(ctx, sizeof(float) * (size_t)nb * N_images);
    if (rcode) return rcode;
    float* part = (float*)ctx->scratch;
    emc::max_partial_kernel<<<dim3(gx, nb), emc::kLseThreads, 0, ctx->stream>>>(
        d_respons, N_images, n_slices, rc, part);
    if ((rcode = emc::after_launch(ctx, "max_partial_kernel"))) return rcode;
    emc::max_final_kernel<<<gx, emc::kLseThreads, 0, ctx->stream>>>(part, N_images, nb, d_maxr);
  } else {
    emc::max_final_kernel<<<gx, emc::kLseThreads, 0, ctx->stream>>>(nullptr, N_images, 0, d_maxr);
  }
  return emc::after_launch(ctx, "max_final_kernel");
}

extern "C" int emc_respons_max_expf(emc_ctx* ctx, const float* d_respons, const float* d_max,
                                    int N_images, int n_slices, float* d_sum) {
  EMC_CHECK_CTX(ctx);
  EMC_REQUIRE(ctx, d_respons && d_max && d_sum, "respons_max_expf: null pointer");
  EMC_REQUIRE(ctx, N_images >= 0 && n_slices >= 0, "respons_max_expf: bad sizes");
  if (N_images == 0) return EMC_OK;
  const int rc = emc::lse_range_rows(n_slices);
  const int nb = n_slices > 0 ? emc::ceil_div(n_slices, rc) : 0;
  const int gx = emc::ceil_div(N_images, emc::kLseThreads);
  float* part = nullptr;
  int rcode;
  if (nb > 0) {
    if ((rcode = emc::ensure_scratch(ctx, sizeof(float) * (size_t)nb * N_images))) return rcode;
    part = (float*)ctx->scratch;
    emc::sumexp_partial_kernel<<<dim3(gx, nb), emc::kLseThreads, 0, ctx->stream>>>(
        d_respons, d_max, N_images, n_slices, rc, part);
    if ((rcode = emc::after_launch(ctx, "sumexp_partial_kernel"))) return rcode;
  }
  emc::sum_final_kernel<<<gx, emc::kLseThreads, 0, ctx->stream>>>(part, N_images, nb, d_sum);
  return emc::after_launch(ctx, "sum_final_kernel");
}

extern "C" int emc_norm_respons_sumexpf(emc_ctx* ctx, float* d_respons, const float* d_sum,
                                        const float* d_max, int N_images, int n_slices) {
  EMC_CHECK_CTX(ctx);
  (void)d_max;  // unused by the reference kernel as well (emc_cuda.cu:1253-1260)
  EMC_REQUIRE(ctx, d_respons && d_sum, "norm_respons_sumexpf: null pointer");
  EMC_REQUIRE(ctx, N_images >= 0 && n_slices >= 0, "norm_respons_sumexpf: bad sizes");
  const long long total = (long long)N_images * n_slices;
  if (total == 0) return EMC_OK;
  const int blocks = (int)std::min<long long>(emc::ceil_div(total, 256), (long long)ctx->sm_count * 16);
  emc::norm_kernel<<<blocks, 256, 0, ctx->stream>>>(d_respons, d_sum, N_images, total);
  return emc::after_launch(ctx, "norm_kernel");
}

extern "C" int emc_log_sum_max(emc_ctx* ctx, const float* d_sum, const float* d_max,
                               float* d_lse, int N_images) {
  EMC_CHECK_CTX(ctx);
  EMC_REQUIRE(ctx, d_sum && d_max && d_lse && N_images >= 0, "log_sum_max: bad arguments");
  if (N_images == 0) return EMC_OK;
  emc::log_sum_max_kernel<<<emc::ceil_div(N_images, 256), 256, 0, ctx->stream>>>(d_sum, d_max,
                                                                                d_lse, N_images);
  return emc::after_launch(ctx, "log_sum_max_kernel");
}

// ---- allocation-free variant of emc_respons_max_expf ---------------------
// For callers that must not allocate device memory at the time of the call:
// code running inside CUDA stream capture, callbacks and real-time loops
// where cudaMalloc would synchronise the device or is forbidden, and hosts
// that hand the library a fixed memory budget.  The per-range partial sums
// live in one file-scope device array of EMC_NOALLOC_PARTIALS floats (4 MiB),
// which every GPU that loads this library keeps until the process exits.
// Host code never dereferences the array's name (on the host it is only a
// stand-in symbol): its device address is looked up with
// cudaGetSymbolAddress on the first call made on each device, with that
// device current, and cached; that first call therefore does the set-up and
// should come before any stream capture.  No cudaMalloc, cudaFree or
// allocating library routine is called.  Every call on a device shares the
// array and each call overwrites every slot it reads, so nothing has to be
// cleared; calls whose kernels overlap on the GPU (e.g. on two streams) race
// on the array and must be serialised by the caller.
static __device__ __align__(256) float g_noalloc_partials[EMC_NOALLOC_PARTIALS];

static int noalloc_partials(float** out) {
  static std::mutex mu;
  static float* addr[64] = {};
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return EMC_ERR_CUDA;
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_partials) != cudaSuccess || !p) return EMC_ERR_CUDA;
    addr[dev] = (float*)p;
  }
  *out = addr[dev];
  return EMC_OK;
}

extern "C" int emc_respons_max_expf_noalloc(const float* d_respons, const float* d_max,
                                            int N_images, int n_slices, float* d_sum,
                                            void* cuda_stream) {
  if (!d_respons || !d_max || !d_sum || N_images < 0 || n_slices < 0) return EMC_ERR_INVALID;
  if (N_images > EMC_NOALLOC_PARTIALS) return EMC_ERR_INVALID;  // not even one range fits
  if (N_images == 0) return EMC_OK;
  cudaStream_t stream = (cudaStream_t)cuda_stream;
  float* part = nullptr;
  const int max_ranges = std::min(EMC_NOALLOC_PARTIALS / N_images, 65535);
  int rc = 64, nb = 0;
  if (n_slices > 0) {
    rc = std::max(64, (n_slices + max_ranges - 1) / max_ranges);
    nb = (n_slices + rc - 1) / rc;
    const int e = noalloc_partials(&part);
    if (e) return e;
  }
  const int gx = emc::ceil_div(N_images, emc::kLseThreads);
  // cudaLaunchKernel returns this launch's own status, so an earlier,
  // unrelated error pending on the thread is neither reported as this call's
  // failure nor consumed; a failed launch's error is cleared after reading.
  if (nb > 0) {
    void* a[] = {(void*)&d_respons, (void*)&d_max, (void*)&N_images, (void*)&n_slices,
                 (void*)&rc, (void*)&part};
    if (cudaLaunchKernel((const void*)emc::sumexp_partial_kernel, dim3(gx, nb),
                         dim3(emc::kLseThreads), a, 0, stream) != cudaSuccess) {
      cudaGetLastError();
      return EMC_ERR_CUDA;
    }
  }
  const float* cpart = part;
  void* b[] = {(void*)&cpart, (void*)&N_images, (void*)&nb, (void*)&d_sum};
  if (cudaLaunchKernel((const void*)emc::sum_final_kernel, dim3(gx), dim3(emc::kLseThreads), b, 0,
                       stream) != cudaSuccess) {
    cudaGetLastError();
    return EMC_ERR_CUDA;
  }
  return EMC_OK;
}
