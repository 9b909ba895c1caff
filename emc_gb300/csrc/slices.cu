// Expand step: rotated slices of the 3D model (row A4).
//
// Reference: cuda_get_slice / get_slices_kernel / cuda_get_slices,
// emc_cuda.cu:102-157, 542-560.  There one 512-thread block walks one slice
// with a serial loop over x and a stride over y, so stores are strided by
// `side`.  Here every thread owns four consecutive pixels of one slice, the
// rotation matrix is built once per block in shared memory, the 8 MB model
// (128^3 float) stays resident in L2 between rotations, and a slice row is
// written with one 128-bit store per thread.
#include "common.cuh"
#include "geometry.cuh"
#include "kernels.cuh"

namespace emc {

// Nearest-voxel sample with the reference's bounds: an index of 0 counts as
// outside (emc_cuda.cu:132-134), everything outside gives -1.
__device__ __forceinline__ float sample_nearest(const float* __restrict__ model, int side,
                                                const RotMat& R, float x, float y, float z) {
  const long ix = voxel_round(voxel_coord(side, rotate_row(R, 0, x, y, z)));
  const long iy = voxel_round(voxel_coord(side, rotate_row(R, 1, x, y, z)));
  const long iz = voxel_round(voxel_coord(side, rotate_row(R, 2, x, y, z)));
  if (ix > 0 && ix < side && iy > 0 && iy < side && iz > 0 && iz < side)
    return __ldg(model + ((size_t)iz * side + iy) * side + ix);
  return -1.0f;
}

// Trilinear sample over the known (>= 0) corner voxels, renormalised by the
// weight of the corners used; -1 when no known corner has weight.
__device__ __forceinline__ float sample_trilinear(const float* __restrict__ model, int side,
                                                  const RotMat& R, float x, float y, float z) {
  const float cx = voxel_coord(side, rotate_row(R, 0, x, y, z));
  const float cy = voxel_coord(side, rotate_row(R, 1, x, y, z));
  const float cz = voxel_coord(side, rotate_row(R, 2, x, y, z));
  const float fx0 = floorf(cx), fy0 = floorf(cy), fz0 = floorf(cz);
  const int x0 = (int)fx0, y0 = (int)fy0, z0 = (int)fz0;
  const float tx = cx - fx0, ty = cy - fy0, tz = cz - fz0;
  float acc = 0.0f, wsum = 0.0f;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int xi = x0 + (c & 1), yi = y0 + ((c >> 1) & 1), zi = z0 + (c >> 2);
    if (xi < 0 || xi >= side || yi < 0 || yi >= side || zi < 0 || zi >= side) continue;
    const float w = ((c & 1) ? tx : 1.0f - tx) * (((c >> 1) & 1) ? ty : 1.0f - ty) *
                    ((c >> 2) ? tz : 1.0f - tz);
    const float v = __ldg(model + ((size_t)zi * side + yi) * side + xi);
    if (v < 0.0f || w <= 0.0f) continue;
    acc = __fmaf_rn(w, v, acc);
    wsum += w;
  }
  return wsum > 1e-6f ? acc / wsum : -1.0f;
}

template <int INTERP>
__global__ void __launch_bounds__(256) slice_kernel(const float* __restrict__ model, int side,
                                                    float* __restrict__ slices,
                                                    const float* __restrict__ rot,
                                                    const float* __restrict__ xc,
                                                    const float* __restrict__ yc,
                                                    const float* __restrict__ zc, int n_2d,
                                                    int vec4) {
  __shared__ RotMat sR;
  const int r = blockIdx.y;
  if (threadIdx.x == 0) sR = quat_to_matrix(rot + 4 * (size_t)r);
  __syncthreads();
  const RotMat R = sR;
  float* out = slices + (size_t)r * n_2d;
  const int p0 = 4 * (blockIdx.x * blockDim.x + threadIdx.x);
  if (p0 >= n_2d) return;
  float v[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int p = p0 + k;
    if (p < n_2d) {
      const float x = __ldg(xc + p), y = __ldg(yc + p), z = __ldg(zc + p);
      v[k] = INTERP == EMC_INTERP_NEAREST ? sample_nearest(model, side, R, x, y, z)
                                          : sample_trilinear(model, side, R, x, y, z);
    }
  }
  if (vec4 && p0 + 3 < n_2d) {
    *reinterpret_cast<float4*>(out + p0) = make_float4(v[0], v[1], v[2], v[3]);
  } else {
    for (int k = 0; k < 4 && p0 + k < n_2d; ++k) out[p0 + k] = v[k];
  }
}

int launch_slices(emc_ctx* ctx, const float* model, int side, float* slices, const float* rot,
                  const float* x, const float* y, const float* z, int n_rot, int interp) {
  const int n_2d = side * side;
  const int threads = 256;
  dim3 grid(ceil_div(n_2d, 4 * threads), n_rot);
  const int vec4 = (n_2d % 4 == 0) && (((uintptr_t)slices & 15) == 0);
  if (interp == EMC_INTERP_NEAREST)
    slice_kernel<EMC_INTERP_NEAREST>
        <<<grid, threads, 0, ctx->stream>>>(model, side, slices, rot, x, y, z, n_2d, vec4);
  else
    slice_kernel<EMC_INTERP_TRILINEAR>
        <<<grid, threads, 0, ctx->stream>>>(model, side, slices, rot, x, y, z, n_2d, vec4);
  return after_launch(ctx, "slice_kernel");
}

}  // namespace emc

extern "C" int emc_get_slices(emc_ctx* ctx, const float* d_model, int side, float* d_slices,
                              const float* d_rot, const float* d_x, const float* d_y,
                              const float* d_z, int start_slice, int slice_chunk, int interp) {
  EMC_CHECK_CTX(ctx);
  EMC_REQUIRE(ctx, side > 1 && side <= 1024, "get_slices: side %d out of range", side);
  EMC_REQUIRE(ctx, d_model && d_slices && d_rot && d_x && d_y && d_z, "get_slices: null pointer");
  EMC_REQUIRE(ctx, start_slice >= 0 && slice_chunk >= 0, "get_slices: bad range");
  EMC_REQUIRE(ctx, slice_chunk <= 65535, "get_slices: chunk %d > 65535", slice_chunk);
  EMC_REQUIRE(ctx, interp == EMC_INTERP_NEAREST || interp == EMC_INTERP_TRILINEAR,
              "get_slices: bad interp %d", interp);
  if (slice_chunk == 0) return EMC_OK;
  return emc::launch_slices(ctx, d_model, side, d_slices, d_rot + 4 * (size_t)start_slice, d_x,
                            d_y, d_z, slice_chunk, interp);
}
