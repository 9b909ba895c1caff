// M-step slice update and insertion with the reference's arithmetic
// (rows A10, A11).
//
// Reference: cuda_update_slices (emc_cuda.cu:562-594), update_slices_kernel
// (emc_atomic.cu:88-132), insert_slices_kernel + cuda_insert_slice
// (emc_atomic.cu:33-85, 183-200).  The reference gives each rotation one block
// that streams every pattern (N x N_2d floats per rotation).  Here a block owns
// 256 pixels x 8 rotations and reads each pattern pixel once for the eight
// rotations; the per-(rotation, pixel) sum still runs over the patterns in
// index order with the reference's ((k * resp) / scaling) term, so the result
// is the reference's to the last bit.  The rotation totals T_r are summed in
// pattern order by one thread per rotation, as every reference thread does.
//
// Insertion: pixel p of rotation r with mask == 1 and slice >= 0 is added to
// the nearest voxel (bounds >= 0, unlike the slicing's > 0) with weight T_r.
// Float atomics make the rounding of model/weight order dependent, exactly
// as in the reference.
#include "common.cuh"
#include "geometry.cuh"
#include "kernels.cuh"

namespace emc {

constexpr int kUpdRot = 8;
constexpr int kUpdImg = 32;
constexpr int kUpdThreads = 256;

__global__ void rotation_totals_kernel(const float* __restrict__ respons,
                                       const int* __restrict__ active, int n_images,
                                       int slice_start, int chunk, float* __restrict__ totals) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= chunk) return;
  const float* row = respons + (size_t)(slice_start + r) * n_images;
  float t = 0.0f;
  for (int i = 0; i < n_images; ++i)
    if (__ldg(active + i) > 0) t = __fadd_rn(t, __ldg(row + i));
  totals[r] = t;
}

__global__ void __launch_bounds__(kUpdThreads) update_slices_ref_kernel(
    const float* __restrict__ images, float* __restrict__ slices, const int* __restrict__ mask,
    const float* __restrict__ respons, const float* __restrict__ scaling,
    const int* __restrict__ active, const float* __restrict__ totals, int n_images,
    int slice_start, int chunk, int n_2d) {
  __shared__ float s_resp[kUpdRot][kUpdImg];
  __shared__ float s_scal[kUpdRot][kUpdImg];
  __shared__ int s_act[kUpdImg];
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int r0 = blockIdx.y * kUpdRot;
  const int nr = min(kUpdRot, chunk - r0);
  const bool in = p < n_2d && __ldg(mask + p) != 0;
  float sum[kUpdRot];
#pragma unroll
  for (int j = 0; j < kUpdRot; ++j) sum[j] = 0.0f;
  for (int i0 = 0; i0 < n_images; i0 += kUpdImg) {
    const int ni = min(kUpdImg, n_images - i0);
    __syncthreads();
    for (int e = threadIdx.x; e < kUpdRot * kUpdImg; e += blockDim.x) {
      const int j = e / kUpdImg, ii = e % kUpdImg;
      const bool ok = j < nr && ii < ni;
      const size_t off = (size_t)(slice_start + r0 + j) * n_images + i0 + ii;
      s_resp[j][ii] = ok ? __ldg(respons + off) : 0.0f;
      s_scal[j][ii] = ok ? __ldg(scaling + off) : 1.0f;
    }
    if (threadIdx.x < kUpdImg) s_act[threadIdx.x] = threadIdx.x < ni ? __ldg(active + i0 + threadIdx.x) : 0;
    __syncthreads();
    if (!in) continue;
    for (int ii = 0; ii < ni; ++ii) {
      if (s_act[ii] <= 0) continue;
      const float k = __ldg(images + (size_t)(i0 + ii) * n_2d + p);
#pragma unroll
      for (int j = 0; j < kUpdRot; ++j)
        sum[j] = __fadd_rn(sum[j], __fdiv_rn(__fmul_rn(k, s_resp[j][ii]), s_scal[j][ii]));
    }
  }
  if (p >= n_2d) return;
  for (int j = 0; j < nr; ++j) {
    float v = -1.0f;
    if (in) {
      v = sum[j];
      const float t = totals[r0 + j];
      if (t > 1e-10f) v = __fdiv_rn(v, t);
    }
    slices[(size_t)(r0 + j) * n_2d + p] = v;
  }
}

__global__ void insert_nearest_kernel(const float* __restrict__ slices,
                                      const int* __restrict__ mask,
                                      const float* __restrict__ totals,
                                      const float* __restrict__ rot, const float* __restrict__ xc,
                                      const float* __restrict__ yc, const float* __restrict__ zc,
                                      int side, int n_2d, float* __restrict__ model,
                                      float* __restrict__ weight) {
  const int r = blockIdx.y;
  const float w = __ldg(totals + r);
  if (!(w > 1e-10f)) return;
  __shared__ RotMat sR;
  if (threadIdx.x == 0) sR = quat_to_matrix(rot + 4 * (size_t)r);
  __syncthreads();
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n_2d) return;
  const float s = __ldg(slices + (size_t)r * n_2d + p);
  if (__ldg(mask + p) != 1 || !(s >= 0.0f)) return;
  const RotMat R = sR;
  const float x = __ldg(xc + p), y = __ldg(yc + p), z = __ldg(zc + p);
  const long ix = voxel_round(voxel_coord(side, rotate_row(R, 0, x, y, z)));
  const long iy = voxel_round(voxel_coord(side, rotate_row(R, 1, x, y, z)));
  const long iz = voxel_round(voxel_coord(side, rotate_row(R, 2, x, y, z)));
  if (ix < 0 || ix >= side || iy < 0 || iy >= side || iz < 0 || iz >= side) return;
  const size_t v = ((size_t)iz * side + iy) * side + ix;
  atomicAdd(model + v, __fmul_rn(w, s));
  atomicAdd(weight + v, w);
}

int launch_insert_nearest(emc_ctx* ctx, const float* slices, const int* mask, const float* totals,
                          const float* rot, const float* x, const float* y, const float* z,
                          int side, int n_rot, float* model, float* weight) {
  const int n_2d = side * side;
  dim3 grid(ceil_div(n_2d, 256), n_rot);
  insert_nearest_kernel<<<grid, 256, 0, ctx->stream>>>(slices, mask, totals, rot, x, y, z, side,
                                                       n_2d, model, weight);
  return after_launch(ctx, "insert_nearest_kernel");
}

}  // namespace emc

extern "C" int emc_update_slices(emc_ctx* ctx, const float* d_images, float* d_slices,
                                 const int* d_mask, const float* d_respons,
                                 const float* d_scaling, const int* d_active_images, int N_images,
                                 int slice_start, int slice_chunk, int N_2d, int side,
                                 float* d_model, const float* d_x, const float* d_y,
                                 const float* d_z, const float* d_rot, float* d_weight) {
  EMC_CHECK_CTX(ctx);
  EMC_REQUIRE(ctx, d_images && d_slices && d_mask && d_respons && d_scaling && d_active_images &&
                       d_model && d_x && d_y && d_z && d_rot && d_weight,
              "update_slices: null pointer");
  EMC_REQUIRE(ctx, side > 1 && N_2d == side * side, "update_slices: N_2d %d != side^2", N_2d);
  EMC_REQUIRE(ctx, N_images >= 0 && slice_start >= 0 && slice_chunk >= 0, "update_slices: bad sizes");
  EMC_REQUIRE(ctx, slice_chunk <= 65535, "update_slices: chunk %d > 65535", slice_chunk);
  if (slice_chunk == 0) return EMC_OK;
  int rc = emc::ensure_scratch(ctx, sizeof(float) * (size_t)slice_chunk);
  if (rc) return rc;
  float* totals = (float*)ctx->scratch;
  emc::rotation_totals_kernel<<<emc::ceil_div(slice_chunk, 128), 128, 0, ctx->stream>>>(
      d_respons, d_active_images, N_images, slice_start, slice_chunk, totals);
  if ((rc = emc::after_launch(ctx, "rotation_totals_kernel"))) return rc;
  dim3 grid(emc::ceil_div(N_2d, emc::kUpdThreads), emc::ceil_div(slice_chunk, emc::kUpdRot));
  emc::update_slices_ref_kernel<<<grid, emc::kUpdThreads, 0, ctx->stream>>>(
      d_images, d_slices, d_mask, d_respons, d_scaling, d_active_images, totals, N_images,
      slice_start, slice_chunk, N_2d);
  if ((rc = emc::after_launch(ctx, "update_slices_ref_kernel"))) return rc;
  return emc::launch_insert_nearest(ctx, d_slices, d_mask, totals, d_rot, d_x, d_y, d_z, side,
                                    slice_chunk, d_model, d_weight);
}
