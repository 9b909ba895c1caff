// Pattern-side preprocessing and model initialisation on the GPU: the steps
// the reference's host runs before the first iteration (main.cpp:92-108).
//   emc_bin_images            read_images binning       emc_helper.cpp:226-243
//   emc_normalize_images      normalize_images_central_part / _individual_mask
//                                                        emc_helper.cpp:389-438
//   emc_mask_images           mask_model                emc_helper.cpp:567-575
//   emc_model_init_radial     model_init, model_input 3 emc_helper.cpp:458-502
//   emc_model_init_orientations  model_init, model_input 1 emc_helper.cpp:503-518
//                                (insert_slice, emc_helper.cpp:81-135)
// The arithmetic follows the reference's types operation by operation
// (float where it computes in `real`, double where a double literal
// promotes), with explicit rounding intrinsics so nothing is contracted.
// Pixel p of a pattern is y*side + x; voxel v of the model z*side^2 + y*side + x.
#include <cmath>
#include <vector>

#include "common.cuh"
#include "emc_gb300.h"

namespace emc {

// Source coordinate of output pixel o along one axis, emc_helper.cpp:232:
// (int)(stride * ((real)(o - side/2) + 0.5) + raw/2 - 0.5), in double.
__device__ __forceinline__ int bin_source(int o, int side, int stride, int raw) {
  const double c = __dadd_rn(__dadd_rn(__dmul_rn((double)stride,
                                                 __dadd_rn((double)(float)(o - side / 2), 0.5)),
                                       (double)(raw / 2)),
                             -0.5);
  return (int)c;  // truncation toward zero, as the C cast
}

// images[i][p] = sum |raw| / sum mask over the stride x stride source block
// (float sum, xb outer and yb inner as the reference); masks[i][p] = sum > 1.
// Source pixels outside the raw frame count as value 0, mask 0 (the
// reference reads them unchecked).
__global__ void bin_images_kernel(const float* __restrict__ raw, const int* __restrict__ raw_mask,
                                  int raw_w, int raw_h, int side, int stride,
                                  float* __restrict__ images, int* __restrict__ masks) {
  const int i = blockIdx.y;
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  const int n2 = side * side;
  if (o >= n2) return;
  const int x = o % side, y = o / side;
  const int sx0 = bin_source(x, side, stride, raw_w);
  const int sy0 = bin_source(y, side, stride, raw_h);
  const size_t base = (size_t)i * raw_w * raw_h;
  float psum = 0.0f;
  int msum = 0;
  for (int xb = 0; xb < stride; ++xb) {
    for (int yb = 0; yb < stride; ++yb) {
      const int sx = sx0 + xb, sy = sy0 + yb;
      if (sx < 0 || sx >= raw_w || sy < 0 || sy >= raw_h) continue;
      const size_t e = base + (size_t)sy * raw_w + sx;
      psum = __fadd_rn(psum, fabsf(__ldg(raw + e)));
      msum += __ldg(raw_mask + e);
    }
  }
  images[(size_t)i * n2 + o] = __fdiv_rn(psum, (float)msum);
  masks[(size_t)i * n2 + o] = msum > 1 ? 1 : 0;
}

// c_i = (real)N_2d / (sequential float sum of the pixels whose mask is 1);
// the common mask, or pattern i's own mask when masks != nullptr.  One
// thread per pattern keeps the reference's order of additions.
__global__ void image_norm_factor_kernel(const float* __restrict__ images,
                                         const int* __restrict__ mask,
                                         const int* __restrict__ masks, int n2, int n_images,
                                         float* __restrict__ factor) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_images) return;
  const float* img = images + (size_t)i * n2;
  const int* m = masks ? masks + (size_t)i * n2 : mask;
  float s = 0.0f;
  for (int p = 0; p < n2; ++p)
    if (__ldg(m + p) == 1) s = __fadd_rn(s, __ldg(img + p));
  factor[i] = __fdiv_rn((float)n2, s);
}

__global__ void scale_images_kernel(float* __restrict__ images, const float* __restrict__ factor,
                                    int n2, size_t n) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride)
    images[e] = __fmul_rn(images[e], __ldg(factor + e / n2));
}

__global__ void mask_images_kernel(float* __restrict__ images, const int* __restrict__ masks,
                                   size_t n) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride)
    if (masks[e] == 0) images[e] = -1.0f;
}

// Column sums over the patterns, FP64: col[p] = sum_i images[i][p].
__global__ void pixel_sums_kernel(const float* __restrict__ images, int n2, int n_images,
                                  double* __restrict__ col) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n2) return;
  double s = 0.0;
  for (int i = 0; i < n_images; ++i) s += (double)__ldg(images + (size_t)i * n2 + p);
  col[p] = s;
}

// Radius of voxel/pixel centre (a - side/2.0 + 0.5 per axis), in double as
// the reference's pow/sqrt of double arguments.
__host__ __device__ inline double centre_radius3(int x, int y, int z, int side) {
  const double h = (double)side / 2.0;
  const double dx = (double)(float)x - h + 0.5, dy = (double)(float)y - h + 0.5,
               dz = (double)(float)z - h + 0.5;
#ifdef __CUDA_ARCH__
  return sqrt(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
#else
  return std::sqrt(dx * dx + dy * dy + dz * dz);
#endif
}

// model = radavg[r] (1 - (rad - r)) + radavg[r+1] (rad - r) for r = (int)rad
// < side/2, else -1, with the reference's types (emc_helper.cpp:487-496): rad
// is a float (the double root rounded), rad - r a float difference, the first
// product double (1.0 is a double literal), the second a float product.
// radavg has side/2 + 1 entries; the last is 0 (the reference reads one past
// its array there).
__global__ void radial_model_kernel(const float* __restrict__ radavg, int side,
                                    float* __restrict__ model) {
  const long long n3 = (long long)side * side * side;
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n3) return;
  const int x = (int)(v % side), y = (int)((v / side) % side), z = (int)(v / ((long long)side * side));
  const float rad = (float)centre_radius3(x, y, z, side);
  const int r = (int)rad;
  float out = -1.0f;
  if ((double)r < (double)side / 2.0) {
    const float f = __fsub_rn(rad, (float)r);
    out = (float)__dadd_rn(__dmul_rn((double)radavg[r], __dsub_rn(1.0, (double)f)),
                           (double)__fmul_rn(radavg[r + 1], f));
  }
  model[v] = out;
}

// insert_slice (emc_helper.cpp:81-135) of pattern i at quaternion rot[i]
// with weight 1: the rotation's diagonal terms are float, the off-diagonal
// terms double (a double literal 2.0), each coordinate sum double stored to
// float, the voxel round(side/2.0 + 0.5 + c) with bounds [0, side).
__global__ void orient_insert_kernel(const float* __restrict__ images, const int* __restrict__ mask,
                                     const float* __restrict__ rot, const float* __restrict__ xc,
                                     const float* __restrict__ yc, const float* __restrict__ zc,
                                     int side, float* __restrict__ model,
                                     float* __restrict__ weight) {
  const int i = blockIdx.y;
  const int n2 = side * side;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n2 || __ldg(mask + p) != 1) return;
  const float* q = rot + 4 * (size_t)i;
  const float q0 = q[0], q1 = q[1], q2 = q[2], q3 = q[3];
  const float x = __ldg(xc + p), y = __ldg(yc + p), z = __ldg(zc + p);
  const double dq0 = q0, dq1 = q1, dq2 = q2, dq3 = q3;
  auto two = [](double a, double b) { return __dmul_rn(__dmul_rn(2.0, a), b); };
  // float diagonal terms, left to right
  const float d0 = __fsub_rn(__fsub_rn(__fadd_rn(__fmul_rn(q0, q0), __fmul_rn(q1, q1)),
                                       __fmul_rn(q2, q2)), __fmul_rn(q3, q3));
  const float d1 = __fsub_rn(__fadd_rn(__fsub_rn(__fmul_rn(q0, q0), __fmul_rn(q1, q1)),
                                       __fmul_rn(q2, q2)), __fmul_rn(q3, q3));
  const float d2 = __fadd_rn(__fsub_rn(__fsub_rn(__fmul_rn(q0, q0), __fmul_rn(q1, q1)),
                                       __fmul_rn(q2, q2)), __fmul_rn(q3, q3));
  const double a01 = __dsub_rn(two(dq1, dq2), two(dq0, dq3));
  const double a02 = __dadd_rn(two(dq1, dq3), two(dq0, dq2));
  const double a10 = __dadd_rn(two(dq1, dq2), two(dq0, dq3));
  const double a12 = __dsub_rn(two(dq2, dq3), two(dq0, dq1));
  const double a20 = __dsub_rn(two(dq1, dq3), two(dq0, dq2));
  const double a21 = __dadd_rn(two(dq2, dq3), two(dq0, dq1));
  const float nx = (float)__dadd_rn(__dadd_rn((double)__fmul_rn(d0, x), __dmul_rn(a01, (double)y)),
                                    __dmul_rn(a02, (double)z));
  const float ny = (float)__dadd_rn(__dadd_rn(__dmul_rn(a10, (double)x), (double)__fmul_rn(d1, y)),
                                    __dmul_rn(a12, (double)z));
  const float nz = (float)__dadd_rn(__dadd_rn(__dmul_rn(a20, (double)x), __dmul_rn(a21, (double)y)),
                                    (double)__fmul_rn(d2, z));
  const double off = __dadd_rn((double)(float)side / 2.0, 0.5);
  const int rx = (int)round(__dadd_rn(off, (double)nx));
  const int ry = (int)round(__dadd_rn(off, (double)ny));
  const int rz = (int)round(__dadd_rn(off, (double)nz));
  if (rx < 0 || rx >= side || ry < 0 || ry >= side || rz < 0 || rz >= side) return;
  const size_t v = ((size_t)rz * side + ry) * side + rx;
  atomicAdd(model + v, __ldg(images + (size_t)i * n2 + p));  // w * slice with w = 1
  atomicAdd(weight + v, 1.0f);
}

// model = model / weight where weight > 0, else 0 (emc_helper.cpp:512-518).
__global__ void orient_divide_kernel(float* __restrict__ model, const float* __restrict__ weight,
                                     long long n) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  const float w = weight[v];
  model[v] = w > 0.0f ? __fdiv_rn(model[v], w) : 0.0f;
}

static int grid_for(emc_ctx* ctx, size_t n) {
  return (int)std::min<size_t>((n + 255) / 256, (size_t)ctx->sm_count * 16);
}

}  // namespace emc

using namespace emc;

extern "C" int emc_bin_images(emc_ctx* ctx, const float* d_raw, const int* d_raw_mask, int raw_w,
                              int raw_h, int n_images, int side, int stride, float* d_images,
                              int* d_masks) {
  EMC_CHECK_CTX(ctx);
  EMC_REQUIRE(ctx, d_raw && d_raw_mask && d_images && d_masks, "bin_images: null pointer");
  EMC_REQUIRE(ctx, raw_w > 0 && raw_h > 0 && side > 0 && stride > 0 && n_images >= 0,
              "bin_images: bad sizes");
  EMC_REQUIRE(ctx, n_images <= 65535, "bin_images: more than 65535 patterns per call");
  if (n_images == 0) return EMC_OK;
  dim3 grid(ceil_div(side * side, 256), n_images);
  bin_images_kernel<<<grid, 256, 0, ctx->stream>>>(d_raw, d_raw_mask, raw_w, raw_h, side, stride,
                                                   d_images, d_masks);
  return after_launch(ctx, "bin_images_kernel");
}

extern "C" int emc_normalize_images(emc_ctx* ctx, float* d_images, const int* d_mask,
                                    const int* d_masks, int N_2d, int n_images) {
  EMC_CHECK_CTX(ctx);
  EMC_REQUIRE(ctx, d_images && (d_mask || d_masks), "normalize_images: null pointer");
  EMC_REQUIRE(ctx, N_2d > 0 && n_images >= 0, "normalize_images: bad sizes");
  if (n_images == 0) return EMC_OK;
  int rc = ensure_scratch(ctx, sizeof(float) * (size_t)n_images);
  if (rc) return rc;
  float* factor = (float*)ctx->scratch;
  image_norm_factor_kernel<<<ceil_div(n_images, 128), 128, 0, ctx->stream>>>(
      d_images, d_mask, d_masks, N_2d, n_images, factor);
  if ((rc = after_launch(ctx, "image_norm_factor_kernel"))) return rc;
  const size_t n = (size_t)N_2d * n_images;
  scale_images_kernel<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(d_images, factor, N_2d, n);
  return after_launch(ctx, "scale_images_kernel");
}

extern "C" int emc_mask_images(emc_ctx* ctx, float* d_images, const int* d_masks, int N_2d,
                               int n_images) {
  EMC_CHECK_CTX(ctx);
  EMC_REQUIRE(ctx, d_images && d_masks, "mask_images: null pointer");
  EMC_REQUIRE(ctx, N_2d > 0 && n_images >= 0, "mask_images: bad sizes");
  const size_t n = (size_t)N_2d * n_images;
  if (n == 0) return EMC_OK;
  mask_images_kernel<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(d_images, d_masks, n);
  return after_launch(ctx, "mask_images_kernel");
}

extern "C" int emc_model_init_radial(emc_ctx* ctx, const float* d_images, int n_images, int side,
                                     float* d_model) {
  EMC_CHECK_CTX(ctx);
  EMC_REQUIRE(ctx, d_images && d_model, "model_init_radial: null pointer");
  EMC_REQUIRE(ctx, side > 1 && side <= 1024 && n_images >= 0, "model_init_radial: bad sizes");
  const int n2 = side * side, nr = side / 2;
  int rc = ensure_scratch(ctx, sizeof(double) * n2 + sizeof(float) * (nr + 1) + 256);
  if (rc) return rc;
  double* col = (double*)ctx->scratch;
  float* d_radavg = (float*)(col + n2);
  pixel_sums_kernel<<<ceil_div(n2, 256), 256, 0, ctx->stream>>>(d_images, n2, n_images, col);
  if ((rc = after_launch(ctx, "pixel_sums_kernel"))) return rc;
  std::vector<double> hcol(n2);
  EMC_CUDA(ctx, cudaMemcpyAsync(hcol.data(), col, sizeof(double) * n2, cudaMemcpyDeviceToHost,
                                ctx->stream));
  EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  // rings r = (int)radius of the pixel centre, r < side/2 (emc_helper.cpp:468-475)
  std::vector<double> sum(nr + 1, 0.0);
  std::vector<long long> cnt(nr + 1, 0);
  for (int x = 0; x < side; ++x)
    for (int y = 0; y < side; ++y) {
      const double h = (double)side / 2.0;
      const double dx = (double)(float)x - h + 0.5, dy = (double)(float)y - h + 0.5;
      const int r = (int)std::sqrt(dx * dx + dy * dy);
      if ((double)r < h) {
        sum[r] += hcol[(size_t)y * side + x];
        cnt[r] += n_images;
      }
    }
  std::vector<float> radavg(nr + 1, 0.0f);
  for (int r = 0; r < nr; ++r) radavg[r] = cnt[r] > 0 ? (float)sum[r] / (float)cnt[r] : 0.0f;
  EMC_CUDA(ctx, cudaMemcpyAsync(d_radavg, radavg.data(), sizeof(float) * (nr + 1),
                                cudaMemcpyHostToDevice, ctx->stream));
  const long long n3 = (long long)n2 * side;
  radial_model_kernel<<<ceil_div(n3, 256), 256, 0, ctx->stream>>>(d_radavg, side, d_model);
  if ((rc = after_launch(ctx, "radial_model_kernel"))) return rc;
  EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));  // radavg is host memory
  return EMC_OK;
}

extern "C" int emc_model_init_orientations(emc_ctx* ctx, const float* d_images, const int* d_mask,
                                           int n_images, int side, const float* d_rot,
                                           const float* d_x, const float* d_y, const float* d_z,
                                           float* d_model, float* d_weight) {
  EMC_CHECK_CTX(ctx);
  EMC_REQUIRE(ctx, d_images && d_mask && d_rot && d_x && d_y && d_z && d_model && d_weight,
              "model_init_orientations: null pointer");
  EMC_REQUIRE(ctx, side > 1 && side <= 1024 && n_images >= 0 && n_images <= 65535,
              "model_init_orientations: bad sizes");
  const long long n3 = (long long)side * side * side;
  EMC_CUDA(ctx, cudaMemsetAsync(d_model, 0, sizeof(float) * n3, ctx->stream));
  EMC_CUDA(ctx, cudaMemsetAsync(d_weight, 0, sizeof(float) * n3, ctx->stream));
  int rc;
  if (n_images > 0) {
    dim3 grid(ceil_div(side * side, 256), n_images);
    orient_insert_kernel<<<grid, 256, 0, ctx->stream>>>(d_images, d_mask, d_rot, d_x, d_y, d_z,
                                                        side, d_model, d_weight);
    if ((rc = after_launch(ctx, "orient_insert_kernel"))) return rc;
  }
  orient_divide_kernel<<<ceil_div(n3, 256), 256, 0, ctx->stream>>>(d_model, d_weight, n3);
  return after_launch(ctx, "orient_divide_kernel");
}
