// Model operations after insertion (rows A13, A14, A15) and diagnostics.
//
// Reference: cuda_divide_model_kernel / cuda_mask_out_model_kernel
// (emc_cuda.cu:758-786), model_average_kernel + cuda_normalize_model
// (:639-671, 788-798), cuda_model_max (:629-637) and the unfinished
// cuda_blur_model (:1404-1492).
//
// The reference averages the positive voxels with ONE block of 512 threads
// and a float accumulator.  Here the average is a grid-wide reduction with an
// FP64 accumulator (per-block partials folded in block order, so the result is
// deterministic); the scale factor is then formed like the reference's,
// 1.0f / (float)mean.  The blur is the reference's intent -- multiply the
// spectrum by exp(-2 pi^2 sigma^2 |k|^2 / s^2) with folded frequencies --
// computed as three circular 1D convolutions whose taps are the exact inverse
// DFT of the separable 1D factor, so no FFT is needed and the result equals
// the FFT form up to float rounding.
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"

namespace emc {

constexpr int kRedThreads = 256;
constexpr int kRedBlocksMax = 1024;

__global__ void divide_by_weight_kernel(float* __restrict__ model, const float* __restrict__ weight,
                                        long long n) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const float w = weight[i];
    model[i] = w > 0.0f ? __fdiv_rn(model[i], w) : -1.0f;
  }
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Per-block FP64 partial sum and count of x > 0.
__global__ void __launch_bounds__(kRedThreads) positive_partial_kernel(const float* __restrict__ x,
                                                                       long long n,
                                                                       double* __restrict__ part) {
  double s = 0.0, c = 0.0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const float v = x[i];
    if (v > 0.0f) {
      s += (double)v;
      c += 1.0;
    }
  }
  __shared__ double ss[kRedThreads / 32], sc[kRedThreads / 32];
  s = warp_sum_d(s);
  c = warp_sum_d(c);
  if ((threadIdx.x & 31) == 0) {
    ss[threadIdx.x >> 5] = s;
    sc[threadIdx.x >> 5] = c;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double ts = 0.0, tc = 0.0;
    for (int w = 0; w < kRedThreads / 32; ++w) {
      ts += ss[w];
      tc += sc[w];
    }
    part[2 * blockIdx.x] = ts;
    part[2 * blockIdx.x + 1] = tc;
  }
}

__global__ void positive_final_kernel(const double* __restrict__ part, int nb,
                                      double* __restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0.0, c = 0.0;
  for (int b = 0; b < nb; ++b) {
    s += part[2 * b];
    c += part[2 * b + 1];
  }
  out[0] = s;
  out[1] = c;
}

__global__ void scale_by_inverse_mean_kernel(float* __restrict__ x, long long n,
                                             const double* __restrict__ stats) {
  const double c = stats[1];
  const float mean = c > 0.0 ? (float)(stats[0] / c) : 0.0f;
  const float inv = 1.0f / mean;  // the reference's constant factor (Inf when mean == 0)
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    x[i] = __fmul_rn(x[i], inv);
}

__global__ void max_partial_f_kernel(const float* __restrict__ x, long long n,
                                     float* __restrict__ part) {
  float m = 0.0f;  // thrust::reduce(..., real(0), maximum) starts at 0
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    m = fmaxf(m, x[i]);
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
  __shared__ float sm[32];
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmaxf(m, sm[w]);
    part[blockIdx.x] = m;
  }
}

static int reduce_blocks(emc_ctx* ctx, long long n) {
  return (int)std::max<long long>(1, std::min<long long>(ceil_div(n, kRedThreads * 4),
                                                         std::min(kRedBlocksMax, ctx->sm_count * 4)));
}

int launch_positive_mean(emc_ctx* ctx, const float* x, long long n, double* out) {
  // out[0..1] = {sum, count}; partials follow at out + 2.
  const int nb = reduce_blocks(ctx, n);
  double* part = out + 2;
  positive_partial_kernel<<<nb, kRedThreads, 0, ctx->stream>>>(x, n, part);
  int rc = after_launch(ctx, "positive_partial_kernel");
  if (rc) return rc;
  positive_final_kernel<<<1, 32, 0, ctx->stream>>>(part, nb, out);
  return after_launch(ctx, "positive_final_kernel");
}

int launch_scale_by_inverse_mean(emc_ctx* ctx, float* x, long long n, const double* stats) {
  const int nb = (int)std::min<long long>(ceil_div(n, 256), (long long)ctx->sm_count * 8);
  scale_by_inverse_mean_kernel<<<nb, 256, 0, ctx->stream>>>(x, n, stats);
  return after_launch(ctx, "scale_by_inverse_mean_kernel");
}

int launch_divide_by_weight(emc_ctx* ctx, float* model, const float* weight, long long n) {
  const int nb = (int)std::min<long long>(ceil_div(n, 256), (long long)ctx->sm_count * 8);
  divide_by_weight_kernel<<<nb, 256, 0, ctx->stream>>>(model, weight, n);
  return after_launch(ctx, "divide_by_weight_kernel");
}

// ---------------------------------------------------------------- blur ----
// Circular 1D convolution with symmetric taps g[d], d = -h..h (h < side/2),
// or the full circle when the kernel is wide.
constexpr int kMaxSide = 1024;

struct BlurTaps {
  int h_lo, h_hi;  // offsets -h_lo .. h_hi
};

// Row pass along x.  First pass: negative voxels are masked (value 0) and
// the mask is recorded; out-of-place into `dst`.
__global__ void blur_rows_kernel(const float* __restrict__ src, float* __restrict__ dst,
                                 unsigned char* __restrict__ keep, const float* __restrict__ g,
                                 int side, BlurTaps t, int first) {
  extern __shared__ float row[];
  const size_t base = (size_t)blockIdx.x * side;
  for (int x = threadIdx.x; x < side; x += blockDim.x) {
    float v = src[base + x];
    if (first) {
      const bool k = !(v < 0.0f);
      keep[base + x] = k;
      if (!k) v = 0.0f;
    }
    row[x] = v;
  }
  __syncthreads();
  for (int x = threadIdx.x; x < side; x += blockDim.x) {
    float acc = 0.0f;
    for (int d = -t.h_lo; d <= t.h_hi; ++d) {
      int xs = x - d;
      xs += (xs < 0) ? side : 0;
      xs -= (xs >= side) ? side : 0;
      acc = __fmaf_rn(g[d < 0 ? d + side : d], row[xs], acc);
    }
    dst[base + x] = acc;
  }
}

// Column pass along an axis with element stride `astride` (side for y,
// side*side for z).  A block owns 32 consecutive x of one line bundle.
__global__ void blur_cols_kernel(const float* __restrict__ src, float* __restrict__ dst,
                                 const unsigned char* __restrict__ keep,
                                 const float* __restrict__ g, int side, long long astride,
                                 long long bstride, BlurTaps t, int last) {
  extern __shared__ float tile[];  // [side][33]
  const int x0 = blockIdx.x * 32;
  const long long base = (long long)blockIdx.y * bstride + x0;
  const int lx = threadIdx.x & 31;
  const int ly = threadIdx.x >> 5;
  const int ny = blockDim.x >> 5;
  const bool xin = x0 + lx < side;
  for (int a = ly; a < side; a += ny) tile[a * 33 + lx] = xin ? src[base + a * astride + lx] : 0.0f;
  __syncthreads();
  if (!xin) return;
  for (int a = ly; a < side; a += ny) {
    float acc = 0.0f;
    for (int d = -t.h_lo; d <= t.h_hi; ++d) {
      int as = a - d;
      as += (as < 0) ? side : 0;
      as -= (as >= side) ? side : 0;
      acc = __fmaf_rn(g[d < 0 ? d + side : d], tile[as * 33 + lx], acc);
    }
    const long long o = base + a * astride + lx;
    if (last && !keep[o]) acc = -1.0f;
    dst[o] = acc;
  }
}

// Taps g[n] = (1/s) sum_k exp(-2 pi^2 sigma^2 kf^2 / s^2) cos(2 pi k n / s),
// kf = min(k, s - k): the inverse DFT of the reference's per-axis factor.
static BlurTaps blur_taps(int side, double sigma, std::vector<float>& g) {
  g.assign(side, 0.0f);
  std::vector<double> gd(side);
  for (int n = 0; n < side; ++n) {
    double acc = 0.0;
    for (int k = 0; k < side; ++k) {
      const double kf = (double)std::min(k, side - k);
      const double m = std::exp(-2.0 * M_PI * M_PI * sigma * sigma * kf * kf / ((double)side * side));
      acc += m * std::cos(2.0 * M_PI * (double)k * (double)n / (double)side);
    }
    gd[n] = acc / (double)side;
  }
  for (int n = 0; n < side; ++n) g[n] = (float)gd[n];
  int h = 0;
  const double tol = 1e-9 * std::fabs(gd[0]);
  for (int n = 1; n <= side / 2; ++n)  // offset side/2 is its own mirror for even sides
    if (std::fabs(gd[n]) > tol) h = n;
  BlurTaps t;
  if (2 * h + 1 >= side) {  // the whole circle: offsets -(side-1)/2 .. side/2
    t.h_lo = (side - 1) / 2;
    t.h_hi = side / 2;
  } else {
    t.h_lo = h;
    t.h_hi = h;
  }
  return t;
}

int blur_prepare(emc_ctx* ctx, int side, float sigma, float* a, float* b, float* g,
                 unsigned char* keep, BlurWork* w) {
  std::vector<float> taps;
  const BlurTaps t = blur_taps(side, (double)sigma, taps);
  // Pageable source: the call returns once `taps` has been staged.
  EMC_CUDA(ctx, cudaMemcpyAsync(g, taps.data(), sizeof(float) * side, cudaMemcpyHostToDevice,
                                ctx->stream));
  const size_t csm = sizeof(float) * side * 33;
  if (csm > 48 * 1024) {
    EMC_CUDA(ctx, cudaFuncSetAttribute(blur_cols_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)csm));
  }
  w->a = a;
  w->b = b;
  w->g = g;
  w->keep = keep;
  w->side = side;
  w->h_lo = t.h_lo;
  w->h_hi = t.h_hi;
  return EMC_OK;
}

size_t blur_work_bytes(int side) {
  const long long n3 = (long long)side * side * side;
  return sizeof(float) * (2 * n3 + side) + n3 + 256;
}

// Enqueues the three passes only: no allocation, no host copy (capturable).
int blur_run(emc_ctx* ctx, float* model, const BlurWork& w) {
  const int side = w.side;
  BlurTaps t;
  t.h_lo = w.h_lo;
  t.h_hi = w.h_hi;
  int rc;
  const int rthreads = std::min(256, ((side + 31) / 32) * 32);
  blur_rows_kernel<<<side * side, rthreads, sizeof(float) * side, ctx->stream>>>(
      model, w.a, w.keep, w.g, side, t, 1);
  if ((rc = after_launch(ctx, "blur_rows_kernel"))) return rc;
  const size_t csm = sizeof(float) * side * 33;
  dim3 grid(ceil_div(side, 32), side);
  // y pass: lines along y, bundles indexed by z.
  blur_cols_kernel<<<grid, 256, csm, ctx->stream>>>(w.a, w.b, w.keep, w.g, side, side,
                                                    (long long)side * side, t, 0);
  if ((rc = after_launch(ctx, "blur_cols_kernel"))) return rc;
  // z pass: lines along z, bundles indexed by y.
  blur_cols_kernel<<<grid, 256, csm, ctx->stream>>>(w.b, model, w.keep, w.g, side,
                                                    (long long)side * side, side, t, 1);
  return after_launch(ctx, "blur_cols_kernel");
}

int launch_blur(emc_ctx* ctx, float* model, int side, float sigma) {
  const long long n3 = (long long)side * side * side;
  int rc = ensure_scratch(ctx, blur_work_bytes(side));
  if (rc) return rc;
  float* a = (float*)ctx->scratch;
  float* b = a + n3;
  float* g = b + n3;
  unsigned char* keep = (unsigned char*)(g + side);
  BlurWork w;
  if ((rc = blur_prepare(ctx, side, sigma, a, b, g, keep, &w))) return rc;
  return blur_run(ctx, model, w);
}

}  // namespace emc

extern "C" int emc_divide_model_by_weight(emc_ctx* ctx, int side, float* d_model,
                                          const float* d_weight) {
  EMC_CHECK_CTX(ctx);
  EMC_REQUIRE(ctx, side > 0 && d_model && d_weight, "divide_model_by_weight: bad arguments");
  return emc::launch_divide_by_weight(ctx, d_model, d_weight, (long long)side * side * side);
}

static int positive_stats(emc_ctx* ctx, const float* d_model, long long n, double* h_stats) {
  const int nb = emc::kRedBlocksMax;
  int rc = emc::ensure_scratch(ctx, sizeof(double) * (2 + 2 * nb));
  if (rc) return rc;
  double* stats = (double*)ctx->scratch;
  if ((rc = emc::launch_positive_mean(ctx, d_model, n, stats))) return rc;
  if (h_stats) {
    EMC_CUDA(ctx, cudaMemcpyAsync(ctx->host_pinned, stats, 2 * sizeof(double),
                                  cudaMemcpyDeviceToHost, ctx->stream));
    EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    h_stats[0] = ((double*)ctx->host_pinned)[0];
    h_stats[1] = ((double*)ctx->host_pinned)[1];
  }
  return EMC_OK;
}

extern "C" int emc_normalize_model(emc_ctx* ctx, int side, float* d_model, float* h_mean) {
  EMC_CHECK_CTX(ctx);
  EMC_REQUIRE(ctx, side > 0 && d_model, "normalize_model: bad arguments");
  const long long n = (long long)side * side * side;
  double hs[2];
  int rc = positive_stats(ctx, d_model, n, h_mean ? hs : nullptr);
  if (rc) return rc;
  if (h_mean) *h_mean = hs[1] > 0 ? (float)(hs[0] / hs[1]) : 0.0f;
  return emc::launch_scale_by_inverse_mean(ctx, d_model, n, (const double*)ctx->scratch);
}

extern "C" int emc_model_average(emc_ctx* ctx, const float* d_model, int n, float* h_out) {
  EMC_CHECK_CTX(ctx);
  EMC_REQUIRE(ctx, d_model && n >= 0 && h_out, "model_average: bad arguments");
  double hs[2];
  int rc = positive_stats(ctx, d_model, n, hs);
  if (rc) return rc;
  *h_out = hs[1] > 0 ? (float)(hs[0] / hs[1]) : 0.0f;
  return EMC_OK;
}

extern "C" int emc_model_max(emc_ctx* ctx, const float* d_model, int n, float* h_out) {
  EMC_CHECK_CTX(ctx);
  EMC_REQUIRE(ctx, d_model && n >= 0 && h_out, "model_max: bad arguments");
  const int nb = std::max(1, std::min(emc::ceil_div(n, 1024), 512));
  int rc = emc::ensure_scratch(ctx, sizeof(float) * nb);
  if (rc) return rc;
  float* part = (float*)ctx->scratch;
  emc::max_partial_f_kernel<<<nb, 256, 0, ctx->stream>>>(d_model, n, part);
  if ((rc = emc::after_launch(ctx, "max_partial_f_kernel"))) return rc;
  std::vector<float> h(nb);
  EMC_CUDA(ctx, cudaMemcpyAsync(h.data(), part, sizeof(float) * nb, cudaMemcpyDeviceToHost, ctx->stream));
  EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  float m = 0.0f;
  for (float v : h) m = std::max(m, v);
  *h_out = m;
  return EMC_OK;
}

extern "C" int emc_blur_model(emc_ctx* ctx, float* d_model, int side, float sigma) {
  EMC_CHECK_CTX(ctx);
  EMC_REQUIRE(ctx, d_model && side > 1 && side <= emc::kMaxSide, "blur_model: bad arguments");
  EMC_REQUIRE(ctx, sigma >= 0.0f && std::isfinite(sigma), "blur_model: bad sigma");
  return emc::launch_blur(ctx, d_model, side, sigma);
}
