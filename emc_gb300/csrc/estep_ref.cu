// Scaling (row A5) and likelihood (row A6) with the reference's arithmetic.
//
// Reference: update_scaling_full_kernel + calculate_scaling_absolute
// (emc_cuda.cu:438-454, 516-539) and calculate_responsabilities_kernel with
// its per-diff device functions (emc_cuda.cu:159-295).  The reference runs one
// 512-thread block per (image, rotation) pair.  Its result depends on the
// order of the float additions: thread t sums pixels t, t+512, ... and the 512
// partials are then folded by a halving tree.  These kernels keep exactly that
// per-pair order (so the host oracle can check them to the last bit where no
// transcendental function is involved) but give each block one image and
// eight rotations, so every image pixel is read once per eight pairs instead
// of once per pair.  They are the drop-in (quirk-exact) path; the fused
// iteration uses the tiled kernels of the plan instead.
//
// Quirks kept on purpose:
//  * the scaling denominator accumulates in an int: every partial add is
//    truncated toward zero (emc_cuda.cu:439, 446);
//  * the scaling masks compare against the double literal 1e-10;
//  * the POISSON term is evaluated in FP64 per pixel (double literal 0.02,
//    emc_cuda.cu:205) and rounded into a float running sum;
//  * count == 0 or den == 0 give the reference's NaN / Inf.
#include "common.cuh"

namespace emc {

constexpr int kVT = 512;       // virtual threads per pair (the reference's TNUM)
constexpr int kRotPerCta = 8;  // rotations that share one image read

// Folds SLOTS independent 512-wide partial vectors with the reference's tree:
// data[t] += data[t + s] for s = 256, 128, ..., 1.  Steps with s < 32 run as
// warp shuffles, which add exactly the same pairs.  Result valid in thread 0.
template <typename T, int SLOTS>
__device__ __forceinline__ void tree_reduce(T (&v)[SLOTS], T* smem) {
  const int t = threadIdx.x;
#pragma unroll
  for (int j = 0; j < SLOTS; ++j) smem[j * kVT + t] = v[j];
  __syncthreads();
#pragma unroll
  for (int s = kVT / 2; s >= 32; s >>= 1) {
    if (t < s) {
#pragma unroll
      for (int j = 0; j < SLOTS; ++j) smem[j * kVT + t] = smem[j * kVT + t] + smem[j * kVT + t + s];
    }
    __syncthreads();
  }
  if (t < 32) {
#pragma unroll
    for (int j = 0; j < SLOTS; ++j) {
      T r = smem[j * kVT + t];
#pragma unroll
      for (int s = 16; s >= 1; s >>= 1) r = r + __shfl_down_sync(0xffffffffu, r, s);
      v[j] = r;
    }
  }
}

__global__ void __launch_bounds__(kVT) scaling_ref_kernel(
    const float* __restrict__ images, const float* __restrict__ slices,
    const int* __restrict__ mask, float* __restrict__ scaling, int n_2d, int n_images,
    int slice_start, int chunk) {
  __shared__ float s_num[kRotPerCta * kVT];
  __shared__ int s_den[kRotPerCta * kVT];
  const int i = blockIdx.x;
  const int r0 = blockIdx.y * kRotPerCta;
  const int nr = min(kRotPerCta, chunk - r0);
  const float* img = images + (size_t)i * n_2d;
  float num[kRotPerCta];
  int den[kRotPerCta];
#pragma unroll
  for (int j = 0; j < kRotPerCta; ++j) {
    num[j] = 0.0f;
    den[j] = 0;
  }
  for (int p = threadIdx.x; p < n_2d; p += kVT) {
    const float k = __ldg(img + p);
    if (__ldg(mask + p) > 0 && (double)k > 1e-10) {
#pragma unroll
      for (int j = 0; j < kRotPerCta; ++j) {
        if (j < nr) {
          const float s = __ldg(slices + (size_t)(r0 + j) * n_2d + p);
          if ((double)s > 1e-10) {
            num[j] = __fmaf_rn(k, k, num[j]);
            den[j] = __float2int_rz(__fmaf_rn(k, s, __int2float_rn(den[j])));
          }
        }
      }
    }
  }
  tree_reduce<float, kRotPerCta>(num, s_num);
  __syncthreads();
  tree_reduce<int, kRotPerCta>(den, s_den);
  if (threadIdx.x == 0) {
    for (int j = 0; j < nr; ++j)
      scaling[(size_t)(slice_start + r0 + j) * n_images + i] = __fdiv_rn(num[j], __int2float_rn(den[j]));
  }
}

template <int DIFF>
__global__ void __launch_bounds__(kVT) respons_ref_kernel(
    const float* __restrict__ slices, const float* __restrict__ images,
    const int* __restrict__ mask, float sigma, const float* __restrict__ scaling,
    float* __restrict__ respons, const float* __restrict__ weights, int n_2d, int n_images,
    int slice_start, int chunk) {
  __shared__ float s_sum[kRotPerCta * kVT];
  __shared__ int s_cnt[kRotPerCta * kVT];
  const int i = blockIdx.x;
  const int r0 = blockIdx.y * kRotPerCta;
  const int nr = min(kRotPerCta, chunk - r0);
  const float* img = images + (size_t)i * n_2d;
  float phi[kRotPerCta], sum[kRotPerCta];
  int cnt[kRotPerCta];
#pragma unroll
  for (int j = 0; j < kRotPerCta; ++j) {
    phi[j] = j < nr ? __ldg(scaling + (size_t)(slice_start + r0 + j) * n_images + i) : 1.0f;
    sum[j] = 0.0f;
    cnt[j] = 0;
  }
  for (int p = threadIdx.x; p < n_2d; p += kVT) {
    if (__ldg(mask + p) == 0) continue;
    const float k = __ldg(img + p);
#pragma unroll
    for (int j = 0; j < kRotPerCta; ++j) {
      if (j < nr) {
        const float s = __ldg(slices + (size_t)(r0 + j) * n_2d + p);
        if (s > 0.0f) {
          const float d = __fsub_rn(s, __fdiv_rn(k, phi[j]));
          if (DIFF == EMC_DIFF_POISSON) {
            const double t = (double)d / sqrt((double)s + 0.02);
            sum[j] = (float)((double)sum[j] + t * t);
          } else if (DIFF == EMC_DIFF_ABSOLUTE) {
            sum[j] = __fmaf_rn(d, d, sum[j]);
          } else {  // EMC_DIFF_RELATIVE
            const float q = __fdiv_rn(d, s);
            sum[j] = __fmaf_rn(q, q, sum[j]);
          }
          cnt[j] += 1;
        }
      }
    }
  }
  tree_reduce<float, kRotPerCta>(sum, s_sum);
  __syncthreads();
  tree_reduce<int, kRotPerCta>(cnt, s_cnt);
  if (threadIdx.x == 0) {
    const double sig2 = (double)__fmul_rn(sigma, sigma);
    for (int j = 0; j < nr; ++j) {
      const int r = slice_start + r0 + j;
      const double lw = (double)logf(__ldg(weights + r));
      const double v = (double)sum[j] / 2.0 / (double)__int2float_rn(cnt[j]) / sig2;
      respons[(size_t)r * n_images + i] = (float)(lw - v);
    }
  }
}

}  // namespace emc

extern "C" int emc_update_scaling_full(emc_ctx* ctx, const float* d_images,
                                       const float* d_slices, const int* d_mask,
                                       float* d_scaling, int N_2d, int N_images,
                                       int slice_start, int slice_chunk, int diff) {
  EMC_CHECK_CTX(ctx);
  (void)diff;  // the reference ignores diff here and always uses the absolute form
  EMC_REQUIRE(ctx, d_images && d_slices && d_mask && d_scaling, "update_scaling_full: null pointer");
  EMC_REQUIRE(ctx, N_2d > 0 && N_images >= 0 && slice_start >= 0 && slice_chunk >= 0,
              "update_scaling_full: bad sizes");
  if (N_images == 0 || slice_chunk == 0) return EMC_OK;
  const int gy = emc::ceil_div(slice_chunk, emc::kRotPerCta);
  EMC_REQUIRE(ctx, gy <= 65535, "update_scaling_full: chunk too large");
  dim3 grid(N_images, gy);
  emc::scaling_ref_kernel<<<grid, emc::kVT, 0, ctx->stream>>>(
      d_images, d_slices, d_mask, d_scaling, N_2d, N_images, slice_start, slice_chunk);
  return emc::after_launch(ctx, "scaling_ref_kernel");
}

extern "C" int emc_calculate_responsabilities(emc_ctx* ctx, const float* d_slices,
                                              const float* d_images, const int* d_mask,
                                              float sigma, const float* d_scaling,
                                              float* d_respons, const float* d_weights, int N_2d,
                                              int N_images, int slice_start, int slice_chunk,
                                              int diff) {
  EMC_CHECK_CTX(ctx);
  EMC_REQUIRE(ctx, d_images && d_slices && d_mask && d_scaling && d_respons && d_weights,
              "calculate_responsabilities: null pointer");
  EMC_REQUIRE(ctx, N_2d > 0 && N_images >= 0 && slice_start >= 0 && slice_chunk >= 0,
              "calculate_responsabilities: bad sizes");
  EMC_REQUIRE(ctx, diff == EMC_DIFF_ABSOLUTE || diff == EMC_DIFF_POISSON || diff == EMC_DIFF_RELATIVE,
              "calculate_responsabilities: diff %d is not a reference diff type", diff);
  if (N_images == 0 || slice_chunk == 0) return EMC_OK;
  const int gy = emc::ceil_div(slice_chunk, emc::kRotPerCta);
  EMC_REQUIRE(ctx, gy <= 65535, "calculate_responsabilities: chunk too large");
  dim3 grid(N_images, gy);
#define EMC_LAUNCH_RESP(D)                                                                    \
  emc::respons_ref_kernel<D><<<grid, emc::kVT, 0, ctx->stream>>>(                             \
      d_slices, d_images, d_mask, sigma, d_scaling, d_respons, d_weights, N_2d, N_images,     \
      slice_start, slice_chunk)
  if (diff == EMC_DIFF_POISSON)
    EMC_LAUNCH_RESP(EMC_DIFF_POISSON);
  else if (diff == EMC_DIFF_ABSOLUTE)
    EMC_LAUNCH_RESP(EMC_DIFF_ABSOLUTE);
  else
    EMC_LAUNCH_RESP(EMC_DIFF_RELATIVE);
#undef EMC_LAUNCH_RESP
  return emc::after_launch(ctx, "respons_ref_kernel");
}
