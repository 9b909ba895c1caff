// Rotation and voxel-index arithmetic shared by the slicing, insertion and
// fused kernels.  The order of every multiply-add is fixed with explicit
// __fmaf_rn / __fmul_rn so that the FP32 voxel indices are reproducible on
// the host (the oracle mirrors the same sequence with C99 fmaf); nvcc's
// implicit contraction of the reference source (emc_cuda.cu:113-131) is
// believed to produce this same sequence.
#pragma once
#include <cuda_runtime.h>

namespace emc {

struct RotMat {
  float m[9];
};

// Quaternion (w, x, y, z) -> rotation matrix, emc_cuda.cu:113-121.
__host__ __device__ inline RotMat quat_to_matrix(const float* q) {
#ifdef __CUDA_ARCH__
#define EMC_FMA(a, b, c) __fmaf_rn((a), (b), (c))
#define EMC_MUL(a, b) __fmul_rn((a), (b))
#else
#define EMC_FMA(a, b, c) fmaf((a), (b), (c))
#define EMC_MUL(a, b) ((a) * (b))
#endif
  const float a = q[0], b = q[1], c = q[2], d = q[3];
  const float a2 = EMC_MUL(2.0f, a), b2 = EMC_MUL(2.0f, b), c2 = EMC_MUL(2.0f, c);
  RotMat r;
  r.m[0] = EMC_FMA(-d, d, EMC_FMA(-c, c, EMC_FMA(b, b, EMC_MUL(a, a))));
  r.m[1] = EMC_FMA(-a2, d, EMC_MUL(b2, c));
  r.m[2] = EMC_FMA(a2, c, EMC_MUL(b2, d));
  r.m[3] = EMC_FMA(a2, d, EMC_MUL(b2, c));
  r.m[4] = EMC_FMA(-d, d, EMC_FMA(c, c, EMC_FMA(-b, b, EMC_MUL(a, a))));
  r.m[5] = EMC_FMA(-a2, b, EMC_MUL(c2, d));
  r.m[6] = EMC_FMA(-a2, c, EMC_MUL(b2, d));
  r.m[7] = EMC_FMA(a2, b, EMC_MUL(c2, d));
  r.m[8] = EMC_FMA(d, d, EMC_FMA(-c, c, EMC_FMA(-b, b, EMC_MUL(a, a))));
  return r;
}

// Rotated pixel coordinate along row `row` of the matrix.
__host__ __device__ inline float rotate_row(const RotMat& r, int row, float x, float y, float z) {
  return EMC_FMA(r.m[3 * row + 2], z, EMC_FMA(r.m[3 * row + 1], y, EMC_MUL(r.m[3 * row], x)));
}
#undef EMC_FMA
#undef EMC_MUL

// Fractional voxel index of a rotated coordinate: side/2 - 0.5 + c.
__host__ __device__ inline float voxel_coord(int side, float c) {
  const float off = (float)side / 2.0f - 0.5f;
  return off + c;
}

// Nearest voxel index of a fractional index, halfway cases away from zero
// (C's round / lroundf, as the reference rounds): roundf is exact and its
// integral result converts to a 32-bit int exactly (|v| < 2^31 here), which
// avoids lroundf's 64-bit float-to-integer conversion -- a slow instruction,
// three per pixel in the expand and the insertion.
__host__ __device__ inline int voxel_round(float v) { return (int)roundf(v); }

}  // namespace emc
