// The fused EMC iteration (emc_plan_* / emc_iterate) and its FP32 kernels.
//
// One iteration restates main.cpp:239-480 for one process on one GPU:
//   expand        slice the model at every rotation, compacted to the
//                 P_eff pixels with mask != 0                       (A4)
//   scaling +     one tiled kernel per 128x128 (rotation, pattern) tile:
//   likelihood    pass 1 accumulates phi = sum k^2 / sum k s, pass 2 the
//                 per-pixel difference sum, the epilogue writes L and phi
//                 and a per-tile (max, sum exp) pair for every pattern (A5, A6)
//   normalise     FP64 log-sum-exp over the tile partials -> lse_i,
//                 P = exp(L - lse), Q = P / phi, T_r = sum_i P      (A7-A9)
//   M-step        tiled GEMM U = Q K over the compacted pixels; its epilogue
//                 inserts T_r * (U / T_r) into the model and T_r into the
//                 weight (nearest or trilinear; float or fixed-point
//                 atomics)                                           (A10, A11)
//   finish        divide by weight, normalise to mean 1 (FP64), blur (A13-A15)
// The MPI exchanges of the reference (main.cpp:367-392, 467-480) have no
// counterpart: the normaliser and the model sums are device reductions.
//
// Semantics of the fused path (the "intended" forms, stated because they
// differ from the drop-in kernels): the scaling denominator is a float sum
// (the reference truncates it to int), the per-pixel term is FP32, pairs with
// no overlap (count_r == 0) or undefined scaling (num or den <= 0) get
// L = -inf and phi = 1, a pattern whose pairs are all invalid gets zero
// responsibility, and the normaliser is FP64.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include <cuda_fp16.h>

#include "geometry.cuh"
#include "kernels.cuh"
#include "plan.cuh"

namespace emc {

int plan_alloc(emc_plan* p, void** ptr, size_t bytes) {
  if (bytes == 0) bytes = 256;
  cudaError_t e = cudaMalloc(ptr, bytes);
  if (e != cudaSuccess)
    return fail(p->ctx, EMC_ERR_NOMEM, "plan alloc of %zu bytes: %s", bytes, cudaGetErrorString(e));
  p->allocs.push_back(*ptr);
  p->bytes += bytes;
  return EMC_OK;
}

template <typename T>
static int alloc_n(emc_plan* p, T** ptr, size_t n) {
  return plan_alloc(p, (void**)ptr, n * sizeof(T));
}

// ------------------------------------------------------------- bind ------
__global__ void gather_coords_kernel(const int* __restrict__ pix, const float* __restrict__ x,
                                     const float* __restrict__ y, const float* __restrict__ z,
                                     float* cx, float* cy, float* cz, int Kp) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= Kp) return;
  const int p = pix[q];
  cx[q] = p >= 0 ? x[p] : 0.0f;
  cy[q] = p >= 0 ? y[p] : 0.0f;
  cz[q] = p >= 0 ? z[p] : 0.0f;
}

// Per-pattern factor of the reference's image normalisation
// (emc_helper.cpp:389-418): c_i = N_2d / (float sum over mask == 1 pixels).
// Pattern position i of the plan holds input pattern perm[i] (perm == nullptr:
// the identity) in this and the other pattern-side kernels.
__global__ void pattern_norm_kernel(const float* __restrict__ images, const int* __restrict__ mask,
                                    int n2, int N, int normalize, float* __restrict__ cnorm,
                                    const int* __restrict__ perm) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  float c = 1.0f;
  if (normalize) {
    const float* img = images + (size_t)(perm ? perm[i] : i) * n2;
    float s = 0.0f;
    for (int p = 0; p < n2; ++p)
      if (__ldg(mask + p) == 1) s = __fadd_rn(s, __ldg(img + p));
    c = __fdiv_rn((float)n2, s);
  }
  cnorm[i] = c;
}

// Compacted pattern operands.  flags[0] bit 0: non-finite input; bit 1: a
// count that is not an integer in [0, 65504] (no FP16 form); bit 3: an
// integer count above 2048 (FP16 rounds it); flags[8]: the largest integer
// count.  One block per (pattern, 256 compacted pixels), pixel blocks the
// fast index so that a pattern's row stays in L2 while its blocks run; flags
// and part[i][block] (the block's sum of k, FP64, fixed order) reduced by
// warp shuffles and one barrier.  Kraw / Kt / K2 (FP32 path) may be null;
// with Kh non-null the kernel also writes the tensor path's FP16 operands
// (the same values as tc_pattern_ops_kernel with scale k2_scale).
__global__ void pattern_ops_kernel(const float* __restrict__ images, const int* __restrict__ pix,
                                   const float* __restrict__ cnorm, int n2, int N, int Kp,
                                   float* __restrict__ Kraw, float* __restrict__ Kt,
                                   float* __restrict__ K2, int* __restrict__ flags,
                                   const int* __restrict__ perm, double* __restrict__ part,
                                   __half* __restrict__ Kh, __half* __restrict__ K2h,
                                   __half* __restrict__ K2l, float k2_scale) {
  const int nqb = (Kp + 255) / 256;
  const int i = (int)(blockIdx.x / nqb);
  const int q = (int)(blockIdx.x % nqb) * 256 + threadIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const bool in = q < Kp;
  const int p = in ? pix[q] : -1;
  float v = 0.0f, k = 0.0f;
  int bits = 0, vmax = 0;
  if (p >= 0) {
    v = __ldg(images + (size_t)(perm ? perm[i] : i) * n2 + p);
    if (!isfinite(v)) bits |= 1;
    if (!(v >= 0.0f && v <= 65504.0f && v == rintf(v))) {
      bits |= 2;
    } else {
      if (v > 2048.0f) bits |= 8;
      vmax = (int)v;
    }
    k = __fmul_rn(v, __ldg(cnorm + i));
  }
  // FP32 warp tree (exact for integer counts; FP64 throughput is scarce), FP64 after
  float fsum = k;
  for (int o = 16; o > 0; o >>= 1) fsum += __shfl_down_sync(0xffffffffu, fsum, o);
  const double sum = (double)fsum;
  bits = __reduce_or_sync(0xffffffffu, (unsigned)bits);
  vmax = __reduce_max_sync(0xffffffffu, vmax);
  __shared__ double wsum[8];
  __shared__ int wbits[8], wmax[8];
  if (lane == 0) {
    wsum[warp] = sum;
    wbits[warp] = bits;
    wmax[warp] = vmax;
  }
  if (in) {
    const size_t o = (size_t)i * Kp + q;
    if (Kraw) Kraw[o] = k;
    const float kt = k >= 1e-10f ? k : 0.0f;  // the reference's (double)k > 1e-10
    if (Kt) Kt[o] = kt;
    if (K2) K2[o] = __fmul_rn(kt, kt);
    if (Kh) {
      const __half kh = __float2half_rn(v);
      const float kr = __half2float(kh);
      const float k2 = kr * kr * k2_scale;
      const __half hi = __float2half_rn(k2);
      Kh[o] = kh;
      if (K2h) {
        K2h[o] = hi;
        K2l[o] = __float2half_rn(k2 - __half2float(hi));
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    int b = 0, m = 0;
    for (int j = 0; j < 8; ++j) {
      t += wsum[j];
      b |= wbits[j];
      m = max(m, wmax[j]);
    }
    part[blockIdx.x] = t;
    if (b) atomicOr(flags, b);
    // the maximum settles early: skip the atomic when this block cannot raise it
    if (m > flags[8]) atomicMax(flags + 8, m);
  }
}

// The same operands, sums and flags as pattern_ops_kernel with one block per
// pattern: the pattern's row is first staged in shared memory with coalesced
// 16-byte loads, then the compacted values are gathered from there in the
// pixel list's (radius) order -- the list scatters over the whole row, and
// gathering it from global memory, one load per thread in flight, took 3.5 ms
// of a 4.2 ms bind at 128^3 x 20,000 patterns.  For rows that fit shared
// memory (pattern_row_smem <= kRowSmemMax).  Ksum[i] is written directly: a
// warp-shuffle tree per 64 pixels in FP32 (exact for integer counts, whose
// sums stay below 2^24; FP64 arithmetic runs at a small fraction of the FP32
// rate on this GPU, and an FP64 tree per pixel took as long as the rest of
// the bind), then the warp sums in pixel order in FP64.
constexpr int kRowThreads = 512;
constexpr int kRowSmemMax = 200 * 1024;

__host__ __device__ inline size_t pattern_row_smem(int n2, int Kp) {
  return (size_t)n2 * sizeof(float) + (size_t)((Kp + 255) / 256) * 8 * sizeof(double);
}

__global__ void __launch_bounds__(kRowThreads) pattern_row_kernel(
    const float* __restrict__ images, const int* __restrict__ pix, const float* __restrict__ cnorm,
    int n2, int N, int Kp, float* __restrict__ Kraw, float* __restrict__ Kt,
    float* __restrict__ K2, int* __restrict__ flags, const int* __restrict__ perm,
    float* __restrict__ Ksum, __half* __restrict__ Kh, __half* __restrict__ K2h,
    __half* __restrict__ K2l, float k2_scale) {
  extern __shared__ __align__(16) unsigned char row_smem[];
  float* srow = reinterpret_cast<float*>(row_smem);
  double* wsum = reinterpret_cast<double*>(row_smem + (size_t)n2 * sizeof(float));
  const int i = blockIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const float* img = images + (size_t)(perm ? perm[i] : i) * n2;
  if ((n2 & 3) == 0 && ((uintptr_t)img & 15) == 0) {
    const float4* s4 = reinterpret_cast<const float4*>(img);
    float4* d4 = reinterpret_cast<float4*>(srow);
    for (int j = threadIdx.x; j < n2 / 4; j += blockDim.x) d4[j] = __ldg(s4 + j);
  } else {
    for (int j = threadIdx.x; j < n2; j += blockDim.x) srow[j] = __ldg(img + j);
  }
  __syncthreads();
  const float ci = __ldg(cnorm + i);
  int bits = 0, vmax = 0;
  // two neighbouring pixels per thread (Kp is a multiple of 128): the
  // compacted operands go out as 8-byte (float2) and 4-byte (half2) stores
  for (int q = 2 * threadIdx.x; q < Kp; q += 2 * blockDim.x) {
    const int2 pp = __ldg(reinterpret_cast<const int2*>(pix + q));
    const int pv[2] = {pp.x, pp.y};
    float v[2], k[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      v[u] = 0.0f;
      k[u] = 0.0f;
      if (pv[u] >= 0) {
        v[u] = srow[pv[u]];
        if (!isfinite(v[u])) bits |= 1;
        if (!(v[u] >= 0.0f && v[u] <= 65504.0f && v[u] == rintf(v[u]))) {
          bits |= 2;
        } else {
          if (v[u] > 2048.0f) bits |= 8;
          vmax = max(vmax, (int)v[u]);
        }
        k[u] = __fmul_rn(v[u], ci);
      }
    }
    float sum = k[0] + k[1];
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
    if (lane == 0) wsum[(q - 2 * lane) / 64] = (double)sum;
    const size_t o = (size_t)i * Kp + q;
    if (Kraw) *reinterpret_cast<float2*>(Kraw + o) = make_float2(k[0], k[1]);
    const float kt0 = k[0] >= 1e-10f ? k[0] : 0.0f;  // the reference's (double)k > 1e-10
    const float kt1 = k[1] >= 1e-10f ? k[1] : 0.0f;
    if (Kt) *reinterpret_cast<float2*>(Kt + o) = make_float2(kt0, kt1);
    if (K2) *reinterpret_cast<float2*>(K2 + o) = make_float2(__fmul_rn(kt0, kt0), __fmul_rn(kt1, kt1));
    if (Kh) {
      __half kh[2], hi[2], lw[2];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        kh[u] = __float2half_rn(v[u]);
        const float kr = __half2float(kh[u]);
        const float k2 = kr * kr * k2_scale;
        hi[u] = __float2half_rn(k2);
        lw[u] = __float2half_rn(k2 - __half2float(hi[u]));
      }
      *reinterpret_cast<__half2*>(Kh + o) = __halves2half2(kh[0], kh[1]);
      if (K2h) {
        *reinterpret_cast<__half2*>(K2h + o) = __halves2half2(hi[0], hi[1]);
        *reinterpret_cast<__half2*>(K2l + o) = __halves2half2(lw[0], lw[1]);
      }
    }
  }
  bits = (int)__reduce_or_sync(0xffffffffu, (unsigned)bits);
  vmax = (int)__reduce_max_sync(0xffffffffu, (unsigned)vmax);
  __shared__ int sbits[kRowThreads / 32], smax[kRowThreads / 32];
  if (lane == 0) {
    sbits[warp] = bits;
    smax[warp] = vmax;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < Kp / 64; ++w) s += wsum[w];
    Ksum[i] = (float)s;
    int bb = 0, m = 0;
    for (int w = 0; w < (int)(blockDim.x / 32); ++w) {
      bb |= sbits[w];
      m = max(m, smax[w]);
    }
    if (bb) atomicOr(flags, bb);
    if (m > flags[8]) atomicMax(flags + 8, m);
  }
}

// Ksum[i] = the sum of pattern i's block partials (in block order).
__global__ void pattern_sums_kernel(const double* __restrict__ part, int N, int nqb,
                                    float* __restrict__ Ksum) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  double s = 0.0;
  for (int b = 0; b < nqb; ++b) s += part[(size_t)i * nqb + b];
  Ksum[i] = (float)s;
}

// ------------------------------------------------------------ expand -----
constexpr float kPoisC = 0.02f;       // emc_cuda.cu:205
constexpr float kSliceFloor = 1e-6f;  // true-Poisson floor for unknown voxels

template <int INTERP>
__device__ __forceinline__ float plan_sample(const float* __restrict__ model, int side,
                                             const RotMat& R, float x, float y, float z);

template <>
__device__ __forceinline__ float plan_sample<EMC_INTERP_NEAREST>(const float* __restrict__ model,
                                                                  int side, const RotMat& R,
                                                                  float x, float y, float z) {
  const long ix = voxel_round(voxel_coord(side, rotate_row(R, 0, x, y, z)));
  const long iy = voxel_round(voxel_coord(side, rotate_row(R, 1, x, y, z)));
  const long iz = voxel_round(voxel_coord(side, rotate_row(R, 2, x, y, z)));
  if (ix > 0 && ix < side && iy > 0 && iy < side && iz > 0 && iz < side)
    return __ldg(model + ((size_t)iz * side + iy) * side + ix);
  return -1.0f;
}

template <>
__device__ __forceinline__ float plan_sample<EMC_INTERP_TRILINEAR>(const float* __restrict__ model,
                                                                    int side, const RotMat& R,
                                                                    float x, float y, float z) {
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

// The compacted slice rows S[r][0..Kp) (or their FP16 operands) of
// kSliceRows rotations per block and the per-rotation sums: count_r (s > 0),
// A_r = sum s^2/(s+c) and the floored slice sum of the true-Poisson
// likelihood.
// rotations per expand block: four with nearest sampling, two with the
// eight-voxel trilinear gather (registers)
template <int INTERP>
__host__ __device__ constexpr int slice_rows_per_block() { return INTERP == EMC_INTERP_NEAREST ? 4 : 2; }

template <int INTERP>
__global__ void __launch_bounds__(256) slice_rows_kernel(
    const float* __restrict__ model, int side, const float* __restrict__ rot,
    const int* __restrict__ pix, const float* __restrict__ cx, const float* __restrict__ cy,
    const float* __restrict__ cz, int R, int Kp, float* __restrict__ S,
    float* __restrict__ rot_cnt, float* __restrict__ rot_A, float* __restrict__ rot_ssum,
    RotOps ops) {
  // kSliceRows rotations per block: each thread loads the coordinates of four
  // neighbouring compacted pixels once (16-byte loads) and samples them for
  // every rotation of the block, so coordinate traffic is shared and the
  // model gathers of several rotations are in flight together; the operands
  // go out as 8-byte stores (Kp is a multiple of 128)
  constexpr int kSliceRows = slice_rows_per_block<INTERP>();
  const int r0 = blockIdx.x * kSliceRows;
  const int gl_end = ops.gl_end ? 32 * __ldg(ops.gl_end) : Kp;  // G lo pixels
  const int nr = min(kSliceRows, R - r0);
  __shared__ RotMat sR[kSliceRows];
  if (threadIdx.x < nr) sR[threadIdx.x] = quat_to_matrix(rot + 4 * (size_t)(r0 + threadIdx.x));
  __syncthreads();
  // per-thread FP32 partials (FP64 arithmetic is scarce on this GPU), block sums in FP64
  float cnt[kSliceRows], A[kSliceRows], ss[kSliceRows];
#pragma unroll
  for (int k = 0; k < kSliceRows; ++k) cnt[k] = A[k] = ss[k] = 0.0f;
  for (int q = 4 * threadIdx.x; q < Kp; q += 4 * blockDim.x) {
    const int4 pp = __ldg(reinterpret_cast<const int4*>(pix + q));
    const float4 X = __ldg(reinterpret_cast<const float4*>(cx + q));
    const float4 Y = __ldg(reinterpret_cast<const float4*>(cy + q));
    const float4 Z = __ldg(reinterpret_cast<const float4*>(cz + q));
    const int pv[4] = {pp.x, pp.y, pp.z, pp.w};
    const float xv[4] = {X.x, X.y, X.z, X.w}, yv[4] = {Y.x, Y.y, Y.z, Y.w},
                zv[4] = {Z.x, Z.y, Z.z, Z.w};
#pragma unroll
    for (int k = 0; k < kSliceRows; ++k) {
      if (k >= nr) break;  // uniform over the block
      const RotMat Rm = sR[k];
      float sv[4], hv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u)
        sv[u] = pv[u] >= 0 ? plan_sample<INTERP>(model, side, Rm, xv[u], yv[u], zv[u]) : 0.0f;
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        // one division per pixel: h = 1 / (s + c) serves A = s^2 h and the operands
        hv[u] = sv[u] > 0.0f ? 1.0f / (sv[u] + kPoisC) : 0.0f;
        if (pv[u] >= 0) {
          if (sv[u] > 0.0f) {
            cnt[k] += 1.0f;
            A[k] += sv[u] * sv[u] * hv[u];
          }
          ss[k] += fmaxf(sv[u], kSliceFloor);
        }
      }
      // the tensor path takes its FP16 operands straight from s; the FP32
      // path keeps the slices
      const size_t e = (size_t)(r0 + k) * Kp + q;
      if (ops.Gh)
        rot_ops_store4(ops, e, sv, hv, q < gl_end);
      else
        *reinterpret_cast<float4*>(S + e) = make_float4(sv[0], sv[1], sv[2], sv[3]);
    }
  }
  // per row: FP32 warp sums, then FP64 over the warps
  __shared__ double wsum[3][kSliceRows][8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < kSliceRows; ++k) {
    float a = cnt[k], b = A[k], c = ss[k];
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, o);
      b += __shfl_down_sync(0xffffffffu, b, o);
      c += __shfl_down_sync(0xffffffffu, c, o);
    }
    if (lane == 0) {
      wsum[0][k][warp] = (double)a;
      wsum[1][k][warp] = (double)b;
      wsum[2][k][warp] = (double)c;
    }
  }
  __syncthreads();
  if (threadIdx.x < nr) {
    const int k = threadIdx.x;
    double a = 0.0, b = 0.0, c = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      a += wsum[0][k][w];
      b += wsum[1][k][w];
      c += wsum[2][k][w];
    }
    rot_cnt[r0 + k] = (float)a;
    rot_A[r0 + k] = (float)b;
    rot_ssum[r0 + k] = (float)c;
  }
}

// --------------------------------------------------- FP32 E-step tile ----
constexpr int BM = 128, BN = 128, BK = 16, TPB = 256, SP = BM + 4;

// Loads a [128 rows][16 cols] tile of a row-major matrix (leading dim ld,
// ld % 4 == 0) into two float4 per thread; rows >= nrows read as zero.
__device__ __forceinline__ void ld_tile(const float* __restrict__ src, size_t ld, int row0,
                                        int nrows, int k0, float4 (&v)[2]) {
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int f = threadIdx.x + u * TPB;
    const int row = f >> 2, quad = f & 3;
    v[u] = row0 + row < nrows
               ? __ldg(reinterpret_cast<const float4*>(src + (size_t)(row0 + row) * ld + k0) + quad)
               : make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

// Transposed store of a loaded tile: dst[k][row] = op(v).
template <typename Op>
__device__ __forceinline__ void st_tile_t(float (*dst)[SP], const float4 (&v)[2], Op op) {
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int f = threadIdx.x + u * TPB;
    const int row = f >> 2, quad = f & 3;
    dst[quad * 4 + 0][row] = op(v[u].x);
    dst[quad * 4 + 1][row] = op(v[u].y);
    dst[quad * 4 + 2][row] = op(v[u].z);
    dst[quad * 4 + 3][row] = op(v[u].w);
  }
}

__device__ __forceinline__ void ld8(const float (*s)[SP], int k, int base, float (&o)[8]) {
  const float4 a = *reinterpret_cast<const float4*>(&s[k][base]);
  const float4 b = *reinterpret_cast<const float4*>(&s[k][64 + base]);
  o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w;
  o[4] = b.x; o[5] = b.y; o[6] = b.z; o[7] = b.w;
}

__device__ __forceinline__ int micro_idx(int t4, int i) { return (i < 4 ? 0 : 64) + t4 + (i & 3); }

struct EstepArgs {
  const float* S;      // [Rp][Kp]
  const float* Kraw;   // [N][Kp]
  const float* Kt;
  const float* K2;
  const float* Ksum;   // [N]
  const float* rot_cnt;
  const float* rot_ssum;
  const float* rotw;   // [R]
  float* L;            // [R][N]
  float* PHI;          // [R][N]
  float2* part;        // [n_rt][N]
  int* bad;            // invalid pair counter
  int R, N, Kp;
  const float* sigma;  // [1] annealing width (device memory)
  int known_intensity;
};

// Writes L/phi of the micro-tile and the tile's (max, sum exp) per pattern.
__device__ void estep_epilogue(const EstepArgs& a, float (&Lv)[8][8], float (&phi)[8][8],
                               float* sred /* [16][128] */, float* scol /* [128] */) {
  const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;
  const int r0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int ty4 = ty * 4, tx4 = tx * 4;
  // stores
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int r = r0 + micro_idx(ty4, i);
    if (r >= a.R) continue;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int n = n0 + h * 64 + tx4;
      float* lp = a.L + (size_t)r * a.N + n;
      float* pp = a.PHI + (size_t)r * a.N + n;
      if (n + 3 < a.N && ((a.N & 3) == 0)) {
        *reinterpret_cast<float4*>(lp) =
            make_float4(Lv[i][4 * h], Lv[i][4 * h + 1], Lv[i][4 * h + 2], Lv[i][4 * h + 3]);
        *reinterpret_cast<float4*>(pp) =
            make_float4(phi[i][4 * h], phi[i][4 * h + 1], phi[i][4 * h + 2], phi[i][4 * h + 3]);
      } else {
        for (int c = 0; c < 4; ++c)
          if (n + c < a.N) {
            lp[c] = Lv[i][4 * h + c];
            pp[c] = phi[i][4 * h + c];
          }
      }
    }
  }
  // per-pattern max over the tile's rotations
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    float m = -INFINITY;
#pragma unroll
    for (int i = 0; i < 8; ++i) m = fmaxf(m, Lv[i][j]);
    sred[ty * BN + micro_idx(tx4, j)] = m;
  }
  __syncthreads();
  if (threadIdx.x < BN) {
    float m = -INFINITY;
    for (int t = 0; t < 16; ++t) m = fmaxf(m, sred[t * BN + threadIdx.x]);
    scol[threadIdx.x] = m;
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float m = scol[micro_idx(tx4, j)];
    float s = 0.0f;
    if (m > -INFINITY) {
#pragma unroll
      for (int i = 0; i < 8; ++i) s += expf(Lv[i][j] - m);
    }
    sred[ty * BN + micro_idx(tx4, j)] = s;
  }
  __syncthreads();
  if (threadIdx.x < BN) {
    const int n = n0 + threadIdx.x;
    float s = 0.0f;
    for (int t = 0; t < 16; ++t) s += sred[t * BN + threadIdx.x];
    if (n < a.N) a.part[(size_t)blockIdx.y * a.N + n] = make_float2(scol[threadIdx.x], s);
  }
}

// Reference-"poisson" likelihood with per-pair scaling, two pixel passes.
__global__ void __launch_bounds__(TPB, 1) estep_fp32_kernel(EstepArgs a) {
  __shared__ __align__(16) float s0[BK][SP];
  __shared__ __align__(16) float s1[BK][SP];
  __shared__ __align__(16) float s2[BK][SP];
  __shared__ __align__(16) float s3[BK][SP];
  const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;
  const int ty4 = ty * 4, tx4 = tx * 4;
  const int r0 = blockIdx.y * BM, n0 = blockIdx.x * BN;

  float num[8][8], den[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) num[i][j] = den[i][j] = 0.0f;

  float4 vr[2], vk2[2], vkt[2];
  const int nk = a.Kp / BK;
  if (!a.known_intensity) {
    // ---- pass 1: num = sum Kt^2 [s > 1e-10], den = sum Kt s [s > 1e-10]
    ld_tile(a.S, a.Kp, r0, a.R, 0, vr);
    ld_tile(a.K2, a.Kp, n0, a.N, 0, vk2);
    ld_tile(a.Kt, a.Kp, n0, a.N, 0, vkt);
    for (int kb = 0; kb < nk; ++kb) {
      // s >= 1e-10f is the reference's (double)s > 1e-10 for every float s
      st_tile_t(s0, vr, [](float s) { return s >= 1e-10f ? 1.0f : 0.0f; });
      st_tile_t(s1, vr, [](float s) { return s >= 1e-10f ? s : 0.0f; });
      st_tile_t(s2, vk2, [](float v) { return v; });
      st_tile_t(s3, vkt, [](float v) { return v; });
      __syncthreads();
      if (kb + 1 < nk) {
        ld_tile(a.S, a.Kp, r0, a.R, (kb + 1) * BK, vr);
        ld_tile(a.K2, a.Kp, n0, a.N, (kb + 1) * BK, vk2);
        ld_tile(a.Kt, a.Kp, n0, a.N, (kb + 1) * BK, vkt);
      }
#pragma unroll 4
      for (int k = 0; k < BK; ++k) {
        float ra[8], rb[8], pk2[8], pkt[8];
        ld8(s0, k, ty4, ra);
        ld8(s1, k, ty4, rb);
        ld8(s2, k, tx4, pk2);
        ld8(s3, k, tx4, pkt);
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            num[i][j] = __fmaf_rn(pk2[j], ra[i], num[i][j]);
            den[i][j] = __fmaf_rn(pkt[j], rb[i], den[i][j]);
          }
      }
      __syncthreads();
    }
  }
  // 1/phi into num, phi into den (phi = 1 when known or undefined)
  int nbad = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      float phi = 1.0f, iphi = 1.0f;
      if (!a.known_intensity) {
        const bool ok = num[i][j] > 0.0f && den[i][j] > 0.0f;
        phi = ok ? __fdiv_rn(num[i][j], den[i][j]) : 1.0f;
        iphi = ok ? __fdiv_rn(den[i][j], num[i][j]) : -1.0f;  // -1 marks invalid
      }
      num[i][j] = iphi;
      den[i][j] = phi;
    }
  // ---- pass 2: acc = sum (s - k/phi)^2 / (s + c) over s > 0
  float acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;
  ld_tile(a.S, a.Kp, r0, a.R, 0, vr);
  ld_tile(a.Kraw, a.Kp, n0, a.N, 0, vk2);
  for (int kb = 0; kb < nk; ++kb) {
    st_tile_t(s0, vr, [](float s) { return s; });
    st_tile_t(s1, vr, [](float s) { return s > 0.0f ? __frcp_rn(s + kPoisC) : 0.0f; });
    st_tile_t(s2, vk2, [](float v) { return v; });
    __syncthreads();
    if (kb + 1 < nk) {
      ld_tile(a.S, a.Kp, r0, a.R, (kb + 1) * BK, vr);
      ld_tile(a.Kraw, a.Kp, n0, a.N, (kb + 1) * BK, vk2);
    }
#pragma unroll 4
    for (int k = 0; k < BK; ++k) {
      float rs[8], rg[8], pk[8];
      ld8(s0, k, ty4, rs);
      ld8(s1, k, ty4, rg);
      ld8(s2, k, tx4, pk);
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const float d = __fmaf_rn(-pk[j], num[i][j], rs[i]);
          const float t = __fmul_rn(d, rg[i]);
          acc[i][j] = __fmaf_rn(t, d, acc[i][j]);
        }
    }
    __syncthreads();
  }
  // ---- epilogue
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int r = r0 + micro_idx(ty4, i);
    const bool rok = r < a.R;
    const float cnt = rok ? __ldg(a.rot_cnt + r) : 0.0f;
    const float lw = rok ? logf(__ldg(a.rotw + r)) : 0.0f;
    const float sg = *a.sigma;
    const float scale = cnt > 0.0f ? (1.0f / (2.0f * sg * sg)) / cnt : 0.0f;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int n = n0 + micro_idx(tx4, j);
      const bool ok = rok && n < a.N && cnt > 0.0f && num[i][j] > 0.0f;
      if (rok && n < a.N && !ok) nbad++;
      acc[i][j] = ok ? lw - acc[i][j] * scale : -INFINITY;
    }
  }
  if (nbad) atomicAdd(a.bad, nbad);
  float* sred = &s0[0][0];  // 16 x 128 floats fit in s0..s3 (4 x 16 x 132)
  float* scol = &s3[0][0];
  estep_epilogue(a, acc, den, sred, scol);
}

// True-Poisson likelihood: L = log w + sum k log s + K log(K/S_r) - K.
__global__ void __launch_bounds__(TPB, 1) estep_pois_fp32_kernel(EstepArgs a) {
  __shared__ __align__(16) float s0[BK][SP];
  __shared__ __align__(16) float s2[BK][SP];
  __shared__ __align__(16) float s4[BK][SP];
  const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;
  const int ty4 = ty * 4, tx4 = tx * 4;
  const int r0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  float acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;
  float4 vr[2], vk[2];
  const int nk = a.Kp / BK;
  ld_tile(a.S, a.Kp, r0, a.R, 0, vr);
  ld_tile(a.Kraw, a.Kp, n0, a.N, 0, vk);
  for (int kb = 0; kb < nk; ++kb) {
    st_tile_t(s0, vr, [](float s) { return logf(fmaxf(s, kSliceFloor)); });
    st_tile_t(s2, vk, [](float v) { return v; });
    __syncthreads();
    if (kb + 1 < nk) {
      ld_tile(a.S, a.Kp, r0, a.R, (kb + 1) * BK, vr);
      ld_tile(a.Kraw, a.Kp, n0, a.N, (kb + 1) * BK, vk);
    }
#pragma unroll 4
    for (int k = 0; k < BK; ++k) {
      float rl[8], pk[8];
      ld8(s0, k, ty4, rl);
      ld8(s2, k, tx4, pk);
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = __fmaf_rn(pk[j], rl[i], acc[i][j]);
    }
    __syncthreads();
  }
  float phi[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int r = r0 + micro_idx(ty4, i);
    const bool rok = r < a.R;
    const float lw = rok ? logf(__ldg(a.rotw + r)) : 0.0f;
    const float Sr = rok ? __ldg(a.rot_ssum + r) : 1.0f;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int n = n0 + micro_idx(tx4, j);
      const float Ki = n < a.N ? __ldg(a.Ksum + n) : 0.0f;
      float l, f;
      if (a.known_intensity) {
        f = 1.0f;
        l = lw + acc[i][j] - Sr;
      } else if (Ki > 0.0f) {
        f = Ki / Sr;
        l = lw + acc[i][j] + Ki * logf(f) - Ki;
      } else {
        f = 0.0f;
        l = lw;
      }
      acc[i][j] = rok && n < a.N ? l : -INFINITY;
      phi[i][j] = f;
    }
  }
  float* sred = &s0[0][0];
  float* scol = &s4[0][0];
  estep_epilogue(a, acc, phi, sred, scol);
}

// ------------------------------------------------------- normalise -------
// lse_i = M + log(sum_t s_t exp(m_t - M)) over the rotation tiles, FP64,
// also as two floats hi + lo (hi = fl(lse), lo = fl(lse - hi)) so that
// consumers form L - lse in FP32 to the same accuracy.  Patterns with no
// valid pair get lse = +inf (all responsibilities 0).
__global__ void lse_combine_kernel(const float2* __restrict__ part, int n_rt, int N,
                                   double* __restrict__ lse, float2* __restrict__ lse2) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float M = -INFINITY;
  for (int t = 0; t < n_rt; ++t) M = fmaxf(M, part[(size_t)t * N + n].x);
  double l = INFINITY;
  if (M > -INFINITY) {
    double s = 0.0;
    for (int t = 0; t < n_rt; ++t) {
      const float2 v = part[(size_t)t * N + n];
      if (v.x > -INFINITY) s += (double)v.y * exp((double)v.x - (double)M);
    }
    l = (double)M + log(s);
  }
  lse[n] = l;
  const float hi = (float)l;
  lse2[n] = make_float2(hi, isfinite(l) ? (float)(l - (double)hi) : 0.0f);
}

__global__ void fill_part_kernel(float2* __restrict__ part, size_t n) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride)
    part[e] = make_float2(-INFINITY, 0.0f);
}

// Deterministic FP64 sum of the finite entries of x[0..n) into out[0]
// (one block; the order of additions is fixed).
__global__ void finite_sum_kernel(const double* __restrict__ x, int n, double* __restrict__ out) {
  __shared__ double sh[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x)
    if (isfinite(x[i])) s += x[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = sh[0];
}

// One block per rotation row: P = exp(L - lse) (in place), Q = P / phi,
// T_r = sum_i P, the row's captured mass and the inserted-mass bound
// sum_i Q_ri K_i.  Element math is FP32 (L - lse with lse as float hi + lo,
// since FP64 arithmetic is scarce on this GPU); per-thread sums are FP32 and
// the block sums FP64.
//   FP32 M-step: Q [R][ldq] (zero padded).
//   Tensor M-step (Qh != nullptr): Q' = P c_i / phi (phi holds c_i num/den,
//   the tensor M-step multiplies raw counts) as FP16 hi [R][ldq] (and lo,
//   when Ql != nullptr), each row scaled by 2^e_r so its largest entry sits
//   near 2^14 (qscale_r = 2^-e_r); with stage, the row is kept in shared
//   memory between the two passes, else the second pass re-reads it.
constexpr int kMprepThreads = 512;  // two blocks per SM (at most 64 registers per thread)
constexpr int kMprepStageMax = 30720;  // patterns whose row of Q fits shared memory (120 KB)

__global__ void __launch_bounds__(kMprepThreads, 2) mprep_kernel(
    float* __restrict__ L, const float* __restrict__ PHI, const float2* __restrict__ lse2,
    const float* __restrict__ Ksum, const float* __restrict__ cnorm, int R, int N,
    float* __restrict__ Q, __half* __restrict__ Qh, __half* __restrict__ Ql,
    float* __restrict__ qscale, int ldq, float* __restrict__ T, double* __restrict__ row_mass,
    double* __restrict__ row_bound, int stage, const unsigned char* __restrict__ tstate,
    int n_rt, double* __restrict__ row_margin, int write_p) {
  extern __shared__ float qrow[];  // [N] when stage: the row's P c_i / phi
  const int r = blockIdx.x;
  // pruned iteration: tstate[pattern tile][rotation tile] = 0 not evaluated
  // (P = 0), 1 evaluated, 2 evaluated margin tile (its mass is summed)
  const unsigned char* ts = tstate ? tstate + (r >> 7) : nullptr;
  float t = 0.0f, b = 0.0f, qmax = 0.0f, mg = 0.0f;
  const bool fast = Qh != nullptr && Ql == nullptr;  // M-step operand FP16 hi only
  // one element: P = exp(L - lse) (0 outside the evaluated tiles), q = P / phi
  // (x c_i for the FP16 operand); returns q and stores P
  auto elem = [&](int i, int st, float l, float f, float2 li, float ks, float cn) -> float {
    float P = 0.0f;
    if (st) {
      // an M-step operand of FP16 hi only takes P through an 11-bit rounding:
      // the hardware exponential (2^-21 relative) serves it; Q hi + lo and the
      // FP32 path keep expf
      if (isfinite(li.x) && l > -INFINITY) {
        const float x = (l - li.x) - li.y;
        P = fast ? __expf(x) : expf(x);
      }
      if (st == 2) mg += P;
    } else {
      f = 0.0f;
    }
    // q = P / phi correctly rounded, except for an FP16 hi-only operand, which
    // a 2-ulp quotient changes at most in rare ties of its rounding
    float q = f > 0.0f ? (fast ? __fdividef(P, f) : __fdiv_rn(P, f)) : 0.0f;
    t += P;
    b = __fmaf_rn(q, ks, b);
    if (Qh) q = __fmul_rn(q, cn);
    qmax = fmaxf(qmax, q);
    if (Q) Q[(size_t)r * ldq + i] = q;
    if (stage) qrow[i] = q;
    return P;
  };
  if ((N & 3) == 0) {
    // 16-byte rows: four elements per load keep enough bytes in flight to
    // approach HBM bandwidth (4-tuples never straddle a 128-pattern tile)
    float4* L4 = reinterpret_cast<float4*>(L + (size_t)r * N);
    const float4* F4 = reinterpret_cast<const float4*>(PHI + (size_t)r * N);
    const float4* S4 = reinterpret_cast<const float4*>(lse2);
    const float4* K4 = reinterpret_cast<const float4*>(Ksum);
    const float4* C4 = reinterpret_cast<const float4*>(cnorm);
    // two 4-tuples per thread and pass (j and j + blockDim, in that order, as
    // one tuple per pass would take them): both tuples' row loads are in
    // flight together
    const int n4 = N / 4, bd = (int)blockDim.x;
    auto tuple = [&](int j, int st, const float4& l, const float4& f) {
      const int i = 4 * j;
      const float4 s01 = S4[2 * j], s23 = S4[2 * j + 1];
      const float4 ks = __ldg(K4 + j), cn = __ldg(C4 + j);
      float4 P;
      P.x = elem(i, st, l.x, f.x, make_float2(s01.x, s01.y), ks.x, cn.x);
      P.y = elem(i + 1, st, l.y, f.y, make_float2(s01.z, s01.w), ks.y, cn.y);
      P.z = elem(i + 2, st, l.z, f.z, make_float2(s23.x, s23.y), ks.z, cn.z);
      P.w = elem(i + 3, st, l.w, f.w, make_float2(s23.z, s23.w), ks.w, cn.w);
      if (write_p) L4[j] = P;
    };
    const float4 z4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    for (int j = threadIdx.x; j < n4; j += 2 * bd) {
      const int j2 = j + bd;
      const bool two = j2 < n4;
      const int st = ts ? ts[(size_t)((4 * j) >> 7) * n_rt] : 1;
      const int st2 = two ? (ts ? ts[(size_t)((4 * j2) >> 7) * n_rt] : 1) : 0;
      const float4 l = L4[j];
      const float4 f = st ? F4[j] : z4;
      const float4 l2 = two ? L4[j2] : z4;
      const float4 f2 = st2 ? F4[j2] : z4;
      tuple(j, st, l, f);
      if (two) tuple(j2, st2, l2, f2);
    }
  } else {
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
      const size_t e = (size_t)r * N + i;
      const int st = ts ? ts[(size_t)(i >> 7) * n_rt] : 1;
      const float l = L[e];
      const float f = st ? PHI[e] : 0.0f;
      const float P = elem(i, st, l, f, lse2[i], __ldg(Ksum + i), __ldg(cnorm + i));
      if (write_p) L[e] = P;
    }
  }
  if (Q)
    for (int i = N + threadIdx.x; i < ldq; i += blockDim.x) Q[(size_t)r * ldq + i] = 0.0f;
  // row sums and maximum: FP32 warp shuffles over the threads' FP32
  // partials, then the 32 warp sums in FP64 on warp 0 -- a block tree over
  // 1,024 shared FP64 slots took 28 KB of shared memory (one block per SM
  // with the staged row) and ten block barriers, and FP64 shuffles in every
  // warp cost more than they saved (FP64 runs at a small fraction of the
  // FP32 rate on this GPU)
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float f0 = t, f1 = b, f2 = mg, rmx = qmax;
  for (int o = 16; o > 0; o >>= 1) {
    f0 += __shfl_down_sync(0xffffffffu, f0, o);
    f1 += __shfl_down_sync(0xffffffffu, f1, o);
    f2 += __shfl_down_sync(0xffffffffu, f2, o);
    rmx = fmaxf(rmx, __shfl_down_sync(0xffffffffu, rmx, o));
  }
  double r0s = (double)f0, r1s = (double)f1, r2s = (double)f2;
  __shared__ double wsum[3][kMprepThreads / 32];
  __shared__ float wmax[kMprepThreads / 32];
  __shared__ float row_max;
  if (lane == 0) {
    wsum[0][warp] = r0s;
    wsum[1][warp] = r1s;
    wsum[2][warp] = r2s;
    wmax[warp] = rmx;
  }
  __syncthreads();
  if (warp == 0) {
    const int nw = (int)(blockDim.x >> 5);
    r0s = lane < nw ? wsum[0][lane] : 0.0;
    r1s = lane < nw ? wsum[1][lane] : 0.0;
    r2s = lane < nw ? wsum[2][lane] : 0.0;
    rmx = lane < nw ? wmax[lane] : 0.0f;
    for (int o = 16; o > 0; o >>= 1) {
      r0s += __shfl_down_sync(0xffffffffu, r0s, o);
      r1s += __shfl_down_sync(0xffffffffu, r1s, o);
      r2s += __shfl_down_sync(0xffffffffu, r2s, o);
      rmx = fmaxf(rmx, __shfl_down_sync(0xffffffffu, rmx, o));
    }
    if (lane == 0) {
      T[r] = (float)r0s;
      row_mass[r] = r0s;
      row_bound[r] = r1s;
      if (row_margin) row_margin[r] = r2s;
      row_max = rmx;
    }
  }
  if (!Qh) return;
  __syncthreads();
  const float mx = row_max;
  int ex = mx > 0.0f ? 14 - ilogbf(mx) - 1 : 0;
  ex = max(-100, min(100, ex));
  const float up = ldexpf(1.0f, ex);
  auto qval = [&](int i) -> float {
    if (i >= N) return 0.0f;
    if (stage) return __fmul_rn(qrow[i], up);
    // re-read the row (L now holds P)
    const size_t e = (size_t)r * N + i;
    const float f = PHI[e];
    return f > 0.0f ? __fmul_rn(__fmul_rn(__fdiv_rn(L[e], f), __ldg(cnorm + i)), up) : 0.0f;
  };
  // ldq is a multiple of 128: four FP16 values (8 bytes) per store
  for (int j = threadIdx.x; j < ldq / 4; j += blockDim.x) {
    const int i = 4 * j;
    union Pack4 {
      __half h[4];
      uint2 u;
    } hi, lo;
    for (int c = 0; c < 4; ++c) {
      const float q = qval(i + c);
      hi.h[c] = __float2half_rn(q);
      lo.h[c] = __float2half_rn(q - __half2float(hi.h[c]));
    }
    *reinterpret_cast<uint2*>(Qh + (size_t)r * ldq + i) = hi.u;
    if (Ql) *reinterpret_cast<uint2*>(Ql + (size_t)r * ldq + i) = lo.u;
  }
  if (threadIdx.x == 0) qscale[r] = ldexpf(1.0f, -ex);
}

// P = exp(L - lse) in place over the plan's [R][N] rows, with mprep's own
// expression for an evaluated pair (bit-identical to an eagerly written P).
__global__ void respons_from_loglik_kernel(float* __restrict__ L, const float2* __restrict__ lse2,
                                           int N, long long total) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += stride) {
    const int i = (int)(e % N);
    const float l = L[e];
    const float2 li = lse2[i];
    float P = 0.0f;
    if (isfinite(li.x) && l > -INFINITY) P = expf((l - li.x) - li.y);
    L[e] = P;
  }
}

int plan_respons_ready(emc_plan* p) {
  if (p->p_written) return EMC_OK;
  emc_ctx* ctx = p->ctx;
  const long long total = (long long)p->d.n_rot * p->d.n_images;
  respons_from_loglik_kernel<<<ctx->sm_count * 8, 256, 0, ctx->stream>>>(p->L, p->lse2,
                                                                        p->d.n_images, total);
  const int rc = after_launch(ctx, "respons_from_loglik_kernel");
  if (!rc) p->p_written = true;
  return rc;
}

// ---------------------------------------------------------- insert -------
struct InsertCtx {
  float* model;
  float* weight;
  unsigned long long* fix_m;
  unsigned long long* fix_w;
  float2* acc2;          // interleaved (model, weight) sums: one 8-byte atomic per point
  const float2* fix_scale;  // {model, weight} fixed-point scales (deterministic mode)
  float* u;              // sorted mode: pair values [P_eff][ldu] instead of insertion
  int ldu;
  int side;
  int interp;
  int deterministic;
};

__device__ __forceinline__ void add_voxel(const InsertCtx& c, size_t v, float val, float w) {
  if (c.deterministic) {
    const float2 sc = __ldg(c.fix_scale);
    atomicAdd(c.fix_m + v, (unsigned long long)fixed_from_float(__fmul_rn(val, sc.x)));
    atomicAdd(c.fix_w + v, (unsigned long long)fixed_from_float(__fmul_rn(w, sc.y)));
  } else {
    atomicAdd(c.acc2 + v, make_float2(val, w));
  }
}

// Inserts value `val` with weight `w` at the detector point (x, y, z) rotated
// by R: nearest voxel with the reference's insertion bounds (>= 0,
// emc_atomic.cu:67-69) or a trilinear splat.
__device__ __forceinline__ void insert_point(const InsertCtx& c, const RotMat& R, float x, float y,
                                             float z, float val, float w) {
  const int side = c.side;
  if (c.interp == EMC_INTERP_NEAREST) {
    const long ix = voxel_round(voxel_coord(side, rotate_row(R, 0, x, y, z)));
    const long iy = voxel_round(voxel_coord(side, rotate_row(R, 1, x, y, z)));
    const long iz = voxel_round(voxel_coord(side, rotate_row(R, 2, x, y, z)));
    if (ix < 0 || ix >= side || iy < 0 || iy >= side || iz < 0 || iz >= side) return;
    add_voxel(c, ((size_t)iz * side + iy) * side + ix, val, w);
  } else {
    const float cx = voxel_coord(side, rotate_row(R, 0, x, y, z));
    const float cy = voxel_coord(side, rotate_row(R, 1, x, y, z));
    const float cz = voxel_coord(side, rotate_row(R, 2, x, y, z));
    const float fx0 = floorf(cx), fy0 = floorf(cy), fz0 = floorf(cz);
    const int x0 = (int)fx0, y0 = (int)fy0, z0 = (int)fz0;
    const float tx = cx - fx0, ty = cy - fy0, tz = cz - fz0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const int xi = x0 + (k & 1), yi = y0 + ((k >> 1) & 1), zi = z0 + (k >> 2);
      if (xi < 0 || xi >= side || yi < 0 || yi >= side || zi < 0 || zi >= side) continue;
      const float f = ((k & 1) ? tx : 1.0f - tx) * (((k >> 1) & 1) ? ty : 1.0f - ty) *
                      ((k >> 2) ? tz : 1.0f - tz);
      if (f <= 0.0f) continue;
      add_voxel(c, ((size_t)zi * side + yi) * side + xi, val * f, w * f);
    }
  }
}

// ---------------------------------------------------- FP32 M-step --------
struct MstepArgs {
  const float* Q;     // [R][ldq]
  const float* Kraw;  // [N][Kp]
  const float* T;     // [R]
  const float* rot;   // [4R]
  const float *cx, *cy, *cz;  // [Kp]
  int R, N, Kp, ldq, P_eff;
  InsertCtx ins;
};

// U = Q K for a 128-rotation x 128-pixel tile, inserted in the epilogue.
__global__ void __launch_bounds__(TPB, 1) mstep_fp32_kernel(MstepArgs a) {
  __shared__ __align__(16) float sq[BK][SP];
  __shared__ __align__(16) float sk[BK][SP];
  __shared__ RotMat sR[BM];
  const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;
  const int ty4 = ty * 4, tx4 = tx * 4;
  const int r0 = blockIdx.y * BM, q0 = blockIdx.x * BN;
  if (threadIdx.x < BM) {
    const int r = r0 + threadIdx.x;
    if (r < a.R) sR[threadIdx.x] = quat_to_matrix(a.rot + 4 * (size_t)r);
  }
  float acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;
  float4 vq[2], vk[2];
  const int nk = (a.N + BK - 1) / BK;
  auto ld_k = [&](int kb) {
    // [16 pattern rows][128 pixels]: 512 float4, thread t: f = t, t + 256
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int f = threadIdx.x + u * TPB;
      const int row = f >> 5, c4 = f & 31;
      const int i = kb * BK + row;
      vk[u] = i < a.N ? __ldg(reinterpret_cast<const float4*>(a.Kraw + (size_t)i * a.Kp + q0) + c4)
                      : make_float4(0.f, 0.f, 0.f, 0.f);
    }
  };
  auto st_k = [&]() {
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int f = threadIdx.x + u * TPB;
      const int row = f >> 5, c4 = f & 31;
      *reinterpret_cast<float4*>(&sk[row][c4 * 4]) = vk[u];
    }
  };
  ld_tile(a.Q, a.ldq, r0, a.R, 0, vq);
  ld_k(0);
  for (int kb = 0; kb < nk; ++kb) {
    st_tile_t(sq, vq, [](float v) { return v; });
    st_k();
    __syncthreads();
    if (kb + 1 < nk) {
      ld_tile(a.Q, a.ldq, r0, a.R, (kb + 1) * BK, vq);
      ld_k(kb + 1);
    }
#pragma unroll 4
    for (int k = 0; k < BK; ++k) {
      float rq[8], pk[8];
      ld8(sq, k, ty4, rq);
      ld8(sk, k, tx4, pk);
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = __fmaf_rn(rq[i], pk[j], acc[i][j]);
    }
    __syncthreads();
  }
  // ---- epilogue: slice = U / T_r, insert T_r * slice with weight T_r
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int rl = micro_idx(ty4, i);
    const int r = r0 + rl;
    if (r >= a.R) continue;
    const float t = __ldg(a.T + r);
    if (a.ins.u) {  // sorted mode: the pair values, 0 where the rotation inserts nothing
      const bool live = t > 1e-10f;
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int q = q0 + micro_idx(tx4, j);
        if (q < a.P_eff)
          a.ins.u[(size_t)q * a.ins.ldu + r] = live ? __fmul_rn(t, __fdiv_rn(acc[i][j], t)) : 0.0f;
      }
      continue;
    }
    if (!(t > 1e-10f)) continue;
    const RotMat R = sR[rl];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int q = q0 + micro_idx(tx4, j);
      if (q >= a.P_eff) continue;
      const float slice = __fdiv_rn(acc[i][j], t);
      insert_point(a.ins, R, __ldg(a.cx + q), __ldg(a.cy + q), __ldg(a.cz + q),
                   __fmul_rn(t, slice), t);
    }
  }
}

// ------------------------------------------------------- finishing -------
// Upper bounds of the inserted model and weight mass (deterministic mode):
// 1.25 * sum_r sum_i Q_ri K_i and 1.25 * P_eff * sum_r T_r, FP64, fixed order,
// and the fixed-point scales they give.
__global__ void insert_bounds_kernel(const double* __restrict__ row_mass,
                                     const double* __restrict__ row_bound, int R, int P_eff,
                                     double* __restrict__ out, float2* __restrict__ scale) {
  __shared__ double sm[256], sw[256];
  double m = 0.0, w = 0.0;
  for (int r = threadIdx.x; r < R; r += blockDim.x) {
    m += row_bound[r];
    w += row_mass[r];
  }
  sm[threadIdx.x] = m;
  sw[threadIdx.x] = w;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      sm[threadIdx.x] += sm[threadIdx.x + o];
      sw[threadIdx.x] += sw[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = 1.25 * sm[0] + 1e-30;
    out[1] = 1.25 * sw[0] * (double)P_eff + 1e-30;
    *scale = make_float2(fix_scale_pow2(out[0]), fix_scale_pow2(out[1]));
  }
}

// Inserted sums -> weight and model / weight (-1 where the weight is 0,
// emc_cuda.cu:758-768), from the fixed-point (deterministic) or the
// interleaved float accumulators.
__global__ void finish_insert_kernel(const unsigned long long* __restrict__ fm,
                                     const unsigned long long* __restrict__ fw,
                                     const float2* __restrict__ fix_scale,
                                     const float2* __restrict__ acc2, float* __restrict__ model,
                                     float* __restrict__ weight, long long n) {
  const float2 sc = fm ? *fix_scale : make_float2(1.0f, 1.0f);
  const double inv_m = 1.0 / (double)sc.x, inv_w = 1.0 / (double)sc.y;  // powers of two
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += stride) {
    float m, w;
    if (fm) {
      m = (float)((double)(long long)fm[v] * inv_m);
      w = (float)((double)(long long)fw[v] * inv_w);
    } else {
      const float2 a = acc2[v];
      m = a.x;
      w = a.y;
    }
    weight[v] = w;
    model[v] = w > 0.0f ? __fdiv_rn(m, w) : -1.0f;
  }
}

// ---- one rank of a rotation split --------------------------------------
// Per pattern, over this plan's rotations: the largest log-likelihood and the
// sum of exp(L - max) (FP64), from the per-tile partials.
__global__ void rank_partial_kernel(const float2* __restrict__ part, int n_rt, int N,
                                    float* __restrict__ out_max, double* __restrict__ out_sum) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float M = -INFINITY;
  for (int t = 0; t < n_rt; ++t) M = fmaxf(M, part[(size_t)t * N + n].x);
  double sum = 0.0;
  if (M > -INFINITY)
    for (int t = 0; t < n_rt; ++t) {
      const float2 v = part[(size_t)t * N + n];
      if (v.x > -INFINITY) sum += (double)v.y * exp((double)v.x - (double)M);
    }
  out_max[n] = M;
  out_sum[n] = sum;
}

// The normaliser combined over all ranks, in the plan's own form (FP64 and
// float hi + lo).
__global__ void lse_from_global_kernel(const double* __restrict__ lse_in, int N,
                                       double* __restrict__ lse, float2* __restrict__ lse2) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const double l = lse_in[n];
  lse[n] = l;
  const float hi = (float)l;
  lse2[n] = make_float2(hi, isfinite(l) ? (float)(l - (double)hi) : 0.0f);
}

// The inserted sums as floats (model sum of T_r x slice, weight sum of T_r),
// exactly as finish_insert_kernel reads them.
__global__ void sums_out_kernel(const unsigned long long* __restrict__ fm,
                                const unsigned long long* __restrict__ fw,
                                const float2* __restrict__ fix_scale,
                                const float2* __restrict__ acc2,
                                float* __restrict__ msum, float* __restrict__ wsum, long long n) {
  const float2 sc = fm ? *fix_scale : make_float2(1.0f, 1.0f);
  const double inv_m = 1.0 / (double)sc.x, inv_w = 1.0 / (double)sc.y;  // powers of two
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += stride) {
    if (fm) {
      msum[v] = (float)((double)(long long)fm[v] * inv_m);
      wsum[v] = (float)((double)(long long)fw[v] * inv_w);
    } else {
      const float2 a = acc2[v];
      msum[v] = a.x;
      wsum[v] = a.y;
    }
  }
}

// main.cpp:467-476 after the all-reduce: both sums divided by the number of
// ranks (devide_part), then model / weight (-1 where the weight is 0).
__global__ void model_from_sums_kernel(const float* __restrict__ msum,
                                       const float* __restrict__ wsum, float n_ranks,
                                       float* __restrict__ model, float* __restrict__ weight,
                                       long long n) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += stride) {
    const float m = __fdiv_rn(msum[v], n_ranks), w = __fdiv_rn(wsum[v], n_ranks);
    weight[v] = w;
    model[v] = w > 0.0f ? __fdiv_rn(m, w) : -1.0f;
  }
}

}  // namespace emc

using namespace emc;

// ======================================================= C ABI ===========
extern "C" int emc_plan_create(emc_ctx* ctx, const emc_plan_desc* desc, emc_plan** out) {
  EMC_CHECK_CTX(ctx);
  EMC_REQUIRE(ctx, desc && out, "plan_create: null argument");
  *out = nullptr;
  const emc_plan_desc& d = *desc;
  EMC_REQUIRE(ctx, d.side > 1 && d.side <= 1024, "plan_create: side %d out of range", d.side);
  EMC_REQUIRE(ctx, d.n_images > 0 && d.n_rot > 0, "plan_create: empty problem");
  EMC_REQUIRE(ctx, d.n_rot <= 65535 * EMC_RT && (long long)d.n_rot * d.n_images < (1LL << 40),
              "plan_create: problem too large");
  EMC_REQUIRE(ctx, d.diff == EMC_DIFF_POISSON || d.diff == EMC_DIFF_TRUE_POISSON,
              "plan_create: diff %d not supported by the fused path", d.diff);
  EMC_REQUIRE(ctx, d.interp == EMC_INTERP_NEAREST || d.interp == EMC_INTERP_TRILINEAR,
              "plan_create: bad interp");
  EMC_REQUIRE(ctx, d.precision == EMC_PREC_FP32 || d.precision == EMC_PREC_MIXED,
              "plan_create: bad precision");
  EMC_REQUIRE(ctx,
              d.insert_mode == EMC_INSERT_ATOMIC || d.insert_mode == EMC_INSERT_DETERMINISTIC ||
                  d.insert_mode == EMC_INSERT_SORTED,
              "plan_create: bad insert mode");
  EMC_REQUIRE(ctx, d.blur_sigma >= 0.0f && std::isfinite(d.blur_sigma), "plan_create: bad blur");
  emc_plan* p = new emc_plan();
  p->ctx = ctx;
  p->d = d;
  p->n2 = d.side * d.side;
  p->Np = ceil_div(d.n_images, 128) * 128;  // whole 128-pattern tiles (and 64-pattern k-blocks)
  p->Rp = ceil_div(d.n_rot, 128) * 128;
  p->n_rt = ceil_div(d.n_rot, EMC_RT);
  const size_t RN = (size_t)d.n_rot * d.n_images;
  const size_t n3 = (size_t)d.side * d.side * d.side;
  int rc = EMC_OK;
  if (!rc) rc = alloc_n(p, &p->L, RN);
  if (!rc) rc = alloc_n(p, &p->PHI, RN);
  if (!rc) rc = alloc_n(p, &p->part, (size_t)p->n_rt * d.n_images);
  if (!rc) rc = alloc_n(p, &p->lse, d.n_images);
  if (!rc) rc = alloc_n(p, &p->lse2, d.n_images);
  if (!rc) {
    cudaError_t e = cudaFuncSetAttribute(mprep_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(sizeof(float) * kMprepStageMax));
    if (e != cudaSuccess) rc = cuda_fail(ctx, e, "plan_create: mprep smem");
  }
  if (!rc) {
    cudaError_t e = cudaFuncSetAttribute(pattern_row_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, kRowSmemMax);
    if (e != cudaSuccess) rc = cuda_fail(ctx, e, "plan_create: pattern row smem");
  }
  if (!rc) rc = alloc_n(p, &p->T, p->Rp);
  if (!rc) rc = alloc_n(p, &p->rot_cnt, p->Rp);
  if (!rc) rc = alloc_n(p, &p->rot_A, p->Rp);
  if (!rc) rc = alloc_n(p, &p->rot_ssum, p->Rp);
  if (!rc) rc = alloc_n(p, &p->red, (size_t)kRedSlots + 2 * (size_t)p->Rp + 2 * 1024 + 2);
  if (!rc) rc = alloc_n(p, &p->cnorm, d.n_images);
  if (!rc) rc = alloc_n(p, &p->Ksum, d.n_images);
  if (!rc) rc = alloc_n(p, &p->flags, 16);
  if (!rc) rc = alloc_n(p, &p->sigma_dev, 1);
  if (!rc && d.blur_sigma > 0.0f) {
    const size_t n3b = (size_t)d.side * d.side * d.side;
    float *ba = nullptr, *bb = nullptr, *bg = nullptr;
    unsigned char* bk = nullptr;
    rc = alloc_n(p, &ba, n3b);
    if (!rc) rc = alloc_n(p, &bb, n3b);
    if (!rc) rc = alloc_n(p, &bg, (size_t)d.side);
    if (!rc) rc = plan_alloc(p, (void**)&bk, n3b);
    if (!rc) rc = blur_prepare(ctx, d.side, d.blur_sigma, ba, bb, bg, bk, &p->blur);
  }
  if (!rc) {
    cudaError_t e = cudaMemsetAsync(p->flags, 0, 16 * sizeof(int), ctx->stream);
    if (e != cudaSuccess) rc = cuda_fail(ctx, e, "plan_create");
  }
  if (!rc && d.precision == EMC_PREC_FP32) rc = alloc_n(p, &p->Q, (size_t)d.n_rot * p->Np);
  if (!rc && d.insert_mode == EMC_INSERT_DETERMINISTIC) {
    rc = alloc_n(p, &p->fix_m, n3);
    if (!rc) rc = alloc_n(p, &p->fix_w, n3);
  }
  if (!rc && d.insert_mode != EMC_INSERT_DETERMINISTIC) rc = alloc_n(p, &p->acc2, n3);
  if (rc) {
    emc_plan_destroy(p);
    return rc;
  }
  *out = p;
  return EMC_OK;
}

extern "C" int emc_plan_destroy(emc_plan* p) {
  if (!p) return EMC_OK;
  if (p->ctx) cudaStreamSynchronize(p->ctx->stream);
  prune_free(p);
  sorted_free(p);
  if (p->graph_exec) cudaGraphExecDestroy(p->graph_exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  for (auto& e : p->ev)
    if (e) cudaEventDestroy(e);
  if (p->tc) tc_free(p);
  for (void* a : p->allocs) cudaFree(a);
  delete p;
  return EMC_OK;
}

extern "C" size_t emc_plan_workspace_bytes(const emc_plan* p) { return p ? p->bytes : 0; }

// The pattern-side operands (per-pattern factor, compacted counts, their
// sums, and the tensor-core forms once those exist) for the pattern order
// perm (device [N]: position -> input pattern; nullptr: input order).
int emc::pattern_side(emc_plan* p, const int* d_perm, bool with_tc) {
  emc_ctx* ctx = p->ctx;
  const int n2 = p->n2, N = p->d.n_images;
  int rc;
  pattern_norm_kernel<<<ceil_div(N, 128), 128, 0, ctx->stream>>>(
      p->images, p->mask, n2, N, p->d.normalize_images, p->cnorm, d_perm);
  if ((rc = after_launch(ctx, "pattern_norm_kernel"))) return rc;
  // Kt / K2 exist only for the FP32 path (null: not written).
  const int nqb = ceil_div(p->Kp, 256);
  // once the tensor-core operands exist, their FP16 counts come from the same
  // pass at the current K^2 scale (bind re-runs them if the new counts need
  // another scale)
  const bool fused = p->tc != nullptr && p->Kh != nullptr;
  p->fused_k2_scale = fused ? p->k2_scale : 0.0f;
  const size_t row_smem = pattern_row_smem(n2, p->Kp);
  if (row_smem <= (size_t)kRowSmemMax) {
    pattern_row_kernel<<<N, kRowThreads, row_smem, ctx->stream>>>(
        p->images, p->pix, p->cnorm, n2, N, p->Kp, p->Kraw, p->Kt, p->K2, p->flags, d_perm,
        p->Ksum, fused ? p->Kh : nullptr, fused ? p->K2hi : nullptr, fused ? p->K2lo : nullptr,
        p->k2_scale);
    if ((rc = after_launch(ctx, "pattern_row_kernel"))) return rc;
    if (with_tc && p->tc) return tc_pattern_side(p, d_perm, fused);
    return EMC_OK;
  }
  pattern_ops_kernel<<<(unsigned)N * (unsigned)nqb, 256, 0, ctx->stream>>>(
      p->images, p->pix, p->cnorm, n2, N, p->Kp, p->Kraw, p->Kt, p->K2, p->flags, d_perm,
      p->ksum_part, fused ? p->Kh : nullptr, fused ? p->K2hi : nullptr, fused ? p->K2lo : nullptr,
      p->k2_scale);
  if ((rc = after_launch(ctx, "pattern_ops_kernel"))) return rc;
  pattern_sums_kernel<<<ceil_div(N, 256), 256, 0, ctx->stream>>>(p->ksum_part, N, nqb, p->Ksum);
  if ((rc = after_launch(ctx, "pattern_sums_kernel"))) return rc;
  if (with_tc && p->tc) return tc_pattern_side(p, d_perm, fused);
  return EMC_OK;
}

extern "C" int emc_plan_bind(emc_plan* p, const float* d_images, const int* d_mask,
                             const float* d_x, const float* d_y, const float* d_z,
                             const float* d_rot, const float* d_rot_weights) {
  if (!p) return EMC_ERR_INVALID;
  emc_ctx* ctx = p->ctx;
  EMC_REQUIRE(ctx, d_images && d_mask && d_x && d_y && d_z && d_rot && d_rot_weights,
              "plan_bind: null pointer");
  const int n2 = p->n2, N = p->d.n_images;
  const int prev_P = p->P_eff;
  // Mask -> compacted pixel list (host; once per plan).
  std::vector<int> hmask(n2);
  EMC_CUDA(ctx, cudaMemcpyAsync(hmask.data(), d_mask, sizeof(int) * n2, cudaMemcpyDeviceToHost,
                                ctx->stream));
  EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  // a re-bind with the same mask keeps the compacted pixel list
  const bool same_mask = prev_P != 0 && hmask == p->h_mask;
  std::vector<int> pix;
  if (same_mask) {
    pix = p->h_pix;
  } else {
    for (int q = 0; q < n2; ++q) {
      EMC_REQUIRE(ctx, hmask[q] == 0 || hmask[q] == 1, "plan_bind: mask values must be 0 or 1");
      if (hmask[q]) pix.push_back(q);
    }
    EMC_REQUIRE(ctx, !pix.empty(), "plan_bind: mask is empty");
    // Compacted pixels in one-pixel bands of detector radius, each band in
    // order of angle.  By radius: the bright low-q pixels, the only ones whose
    // k^2 needs a second FP16 term, share a few k-blocks of the tensor-core
    // E-step, and the dim outer blocks form the count tail where the G lo
    // term is dropped.  By angle within a band: the 32 pixels of a warp are
    // neighbours on the ring, so the expand's model gathers of a warp touch
    // neighbouring voxels.  (The order is otherwise free: every compacted
    // array uses it consistently.)
    const int side = p->d.side;
    std::vector<std::pair<long long, double>> key(n2);
    for (int q : pix) {
      const double dx = (double)(q % side) - side / 2 + 0.5, dy = (double)(q / side) - side / 2 + 0.5;
      key[q] = {(long long)std::floor(std::sqrt(dx * dx + dy * dy)), std::atan2(dy, dx)};
    }
    std::stable_sort(pix.begin(), pix.end(), [&](int a, int b) { return key[a] < key[b]; });
  }
  EMC_REQUIRE(ctx, prev_P == 0 || prev_P == (int)pix.size(),
              "plan_bind: a re-bind must keep the mask's pixel count (%d != %d)", (int)pix.size(),
              prev_P);
  p->bound = false;
  p->P_eff = (int)pix.size();
  p->Kp = ceil_div(p->P_eff, 128) * 128;  // whole 128-pixel M-step tiles
  pix.resize(p->Kp, -1);
  int rc = EMC_OK;
  if (prev_P == 0) {
  if (!rc) rc = alloc_n(p, &p->pix, p->Kp);
  if (!rc) rc = alloc_n(p, &p->cx, p->Kp);
  if (!rc) rc = alloc_n(p, &p->cy, p->Kp);
  if (!rc) rc = alloc_n(p, &p->cz, p->Kp);
  if (!rc) rc = alloc_n(p, &p->ksum_part, (size_t)N * ceil_div(p->Kp, 256));
  if (!rc && p->d.precision == EMC_PREC_FP32) rc = alloc_n(p, &p->Kraw, (size_t)N * p->Kp);
  if (!rc && p->d.precision == EMC_PREC_FP32) rc = alloc_n(p, &p->S, (size_t)p->Rp * p->Kp);
  if (!rc && p->d.precision == EMC_PREC_FP32) {
    rc = alloc_n(p, &p->Kt, (size_t)N * p->Kp);
    if (!rc) rc = alloc_n(p, &p->K2, (size_t)N * p->Kp);
  }
  // rows R..Rp of the slices stay zero: the expand writes rows < R only
  if (!rc && p->S) {
    const cudaError_t e =
        cudaMemsetAsync(p->S, 0, sizeof(float) * (size_t)p->Rp * p->Kp, ctx->stream);
    if (e != cudaSuccess) rc = cuda_fail(ctx, e, "plan_bind");
  }
  }
  if (rc) return rc;
  if (!same_mask) {
    p->h_mask = hmask;
    p->h_pix.assign(pix.begin(), pix.begin() + p->P_eff);
    // pageable source: staged before the call returns
    EMC_CUDA(ctx, cudaMemcpyAsync(p->pix, pix.data(), sizeof(int) * p->Kp,
                                  cudaMemcpyHostToDevice, ctx->stream));
  }
  EMC_CUDA(ctx, cudaMemsetAsync(p->flags, 0, 16 * sizeof(int), ctx->stream));
  gather_coords_kernel<<<ceil_div(p->Kp, 256), 256, 0, ctx->stream>>>(p->pix, d_x, d_y, d_z, p->cx,
                                                                      p->cy, p->cz, p->Kp);
  if ((rc = after_launch(ctx, "gather_coords_kernel"))) return rc;
  p->images = d_images;
  p->mask = d_mask;
  if ((rc = pattern_side(p, nullptr, false))) return rc;
  int hflags[16];
  EMC_CUDA(ctx, cudaMemcpyAsync(hflags, p->flags, sizeof(hflags), cudaMemcpyDeviceToHost, ctx->stream));
  EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (hflags[0] & 1) return fail(ctx, EMC_ERR_NONFINITE, "plan_bind: images contain NaN/Inf");
  p->counts_fp16_exact = !(hflags[0] & 2) && !(hflags[0] & 8);
  p->counts_integer = !(hflags[0] & 2);
  p->count_max = hflags[8];
  p->images = d_images;
  p->mask = d_mask;
  p->x = d_x;
  p->y = d_y;
  p->z = d_z;
  p->rot = d_rot;
  p->rotw = d_rot_weights;
  if (p->d.precision == EMC_PREC_MIXED) {
    if ((rc = tc_bind(p))) return rc;
  }
  // with pruning on, a new binding starts from the input pattern order, the
  // coherent order of its own rotations and a full scan
  if ((rc = prune_reset(p))) return rc;
  p->bound = true;
  // sorted insertion: the voxel map of this binding's rotations and pixels
  if ((rc = sorted_ensure(p))) {
    p->bound = false;
    return rc;
  }
  return EMC_OK;
}

static int plan_expand(emc_plan* p, const float* model) {
  emc_ctx* ctx = p->ctx;
  const RotOps ops = tc_rot_ops(p);
  if (p->d.interp == EMC_INTERP_NEAREST)
    slice_rows_kernel<EMC_INTERP_NEAREST>
        <<<ceil_div(p->d.n_rot, slice_rows_per_block<EMC_INTERP_NEAREST>()), 256, 0, ctx->stream>>>(
        model, p->d.side, p->rot, p->pix, p->cx, p->cy, p->cz, p->d.n_rot, p->Kp, p->S,
        p->rot_cnt, p->rot_A, p->rot_ssum, ops);
  else
    slice_rows_kernel<EMC_INTERP_TRILINEAR>
        <<<ceil_div(p->d.n_rot, slice_rows_per_block<EMC_INTERP_TRILINEAR>()), 256, 0, ctx->stream>>>(
        model, p->d.side, p->rot, p->pix, p->cx, p->cy, p->cz, p->d.n_rot, p->Kp, p->S,
        p->rot_cnt, p->rot_A, p->rot_ssum, ops);
  return after_launch(ctx, "slice_rows_kernel");
}

static int plan_estep_fp32(emc_plan* p) {
  emc_ctx* ctx = p->ctx;
  EstepArgs a;
  a.S = p->S;
  a.Kraw = p->Kraw;
  a.Kt = p->Kt;
  a.K2 = p->K2;
  a.Ksum = p->Ksum;
  a.rot_cnt = p->rot_cnt;
  a.rot_ssum = p->rot_ssum;
  a.rotw = p->rotw;
  a.L = p->L;
  a.PHI = p->PHI;
  a.part = p->part;
  a.bad = p->flags + 4;
  a.R = p->d.n_rot;
  a.N = p->d.n_images;
  a.Kp = p->Kp;
  a.sigma = p->sigma_dev;
  a.known_intensity = p->d.known_intensity;
  dim3 grid(ceil_div(a.N, BN), ceil_div(a.R, BM));
  if (p->d.diff == EMC_DIFF_POISSON)
    estep_fp32_kernel<<<grid, TPB, 0, ctx->stream>>>(a);
  else
    estep_pois_fp32_kernel<<<grid, TPB, 0, ctx->stream>>>(a);
  return after_launch(ctx, "estep_fp32_kernel");
}

static InsertCtx make_insert_ctx(emc_plan* p, float* model, float* weight) {
  InsertCtx c;
  c.model = model;
  c.weight = weight;
  c.fix_m = p->fix_m;
  c.fix_w = p->fix_w;
  c.acc2 = p->acc2;
  c.fix_scale = reinterpret_cast<const float2*>(p->red + kRedFixScale);
  c.u = p->d.insert_mode == EMC_INSERT_SORTED ? p->ins_u : nullptr;
  c.ldu = p->ins_ldu;
  c.side = p->d.side;
  c.interp = p->d.interp;
  c.deterministic = p->d.insert_mode == EMC_INSERT_DETERMINISTIC;
  return c;
}


static int plan_mstep_fp32(emc_plan* p, float* model, float* weight, const InsertCtx& ins) {
  emc_ctx* ctx = p->ctx;
  MstepArgs a;
  a.Q = p->Q;
  a.Kraw = p->Kraw;
  a.T = p->T;
  a.rot = p->rot;
  a.cx = p->cx;
  a.cy = p->cy;
  a.cz = p->cz;
  a.R = p->d.n_rot;
  a.N = p->d.n_images;
  a.Kp = p->Kp;
  a.ldq = p->Np;
  a.P_eff = p->P_eff;
  a.ins = ins;
  (void)model;
  (void)weight;
  dim3 grid(ceil_div(p->P_eff, BN), ceil_div(a.R, BM));
  mstep_fp32_kernel<<<grid, TPB, 0, ctx->stream>>>(a);
  return after_launch(ctx, "mstep_fp32_kernel");
}

// The stages of one iteration, each enqueued on the context stream: kernels,
// device-to-device copies and memsets only (no allocation, no host copy, no
// synchronisation), so the sequence can be captured in a CUDA graph.  The
// E-step reads sigma from p->sigma_dev.  A full iteration runs them in order;
// one rank of a rotation split (emc_rank_*) runs the E-step, exports its
// per-pattern partials, and resumes at the M-step with the global normaliser.
static int enqueue_normalise(emc_plan* p, float* d_model);

static int mark_phase(emc_plan* p, int i) {
  emc_ctx* ctx = p->ctx;
  if (p->profiling) EMC_CUDA(ctx, cudaEventRecord(p->ev[i], ctx->stream));
  return EMC_OK;
}

// expand + scaling + likelihood + per-tile (max, sum exp) partials
static int enqueue_estep(emc_plan* p, float* d_model) {
  emc_ctx* ctx = p->ctx;
  const int N = p->d.n_images;
  int rc;
  if ((rc = mark_phase(p, 0))) return rc;
  EMC_CUDA(ctx, cudaMemsetAsync(p->flags + 4, 0, sizeof(int), ctx->stream));
  if (p->prune_tiles) {  // skipped tiles contribute (max, sum exp) = (-inf, 0)
    fill_part_kernel<<<ctx->sm_count * 4, 256, 0, ctx->stream>>>(p->part,
                                                                (size_t)p->n_rt * N);
    if ((rc = after_launch(ctx, "fill_part_kernel"))) return rc;
  }
  if ((rc = plan_expand(p, d_model))) return rc;
  if ((rc = mark_phase(p, 1))) return rc;
  if (p->d.precision == EMC_PREC_MIXED)
    rc = tc_estep(p);
  else
    rc = plan_estep_fp32(p);
  if (rc) return rc;
  return mark_phase(p, 2);
}

// the normaliser lse_i from the per-tile partials, and the total log-likelihood
static int enqueue_lse(emc_plan* p) {
  emc_ctx* ctx = p->ctx;
  const int N = p->d.n_images;
  int rc;
  lse_combine_kernel<<<ceil_div(N, 256), 256, 0, ctx->stream>>>(p->part, p->n_rt, N, p->lse,
                                                                p->lse2);
  if ((rc = after_launch(ctx, "lse_combine_kernel"))) return rc;
  finite_sum_kernel<<<1, 256, 0, ctx->stream>>>(p->lse, N, p->red + kRedLL);
  if ((rc = after_launch(ctx, "finite_sum_kernel"))) return rc;
  return mark_phase(p, 3);
}

// responsibilities (mprep) and the M-step with insertion into the zeroed
// accumulators (acc2, or fix_m / fix_w when deterministic); model / weight
// are the buffers the insertion context names (not written here)
static int enqueue_mstep(emc_plan* p, float* d_model, float* d_weight) {
  emc_ctx* ctx = p->ctx;
  const int R = p->d.n_rot, N = p->d.n_images;
  const long long n3 = (long long)p->d.side * p->d.side * p->d.side;
  int rc;
  double* row_mass = p->red + kRedSlots;
  double* row_bound = row_mass + p->Rp;
  const bool tcm = p->d.precision == EMC_PREC_MIXED;
  const int stage = tcm && N <= kMprepStageMax;
  // P is written over L only where it is read back: by the pruning of the
  // next iteration, or by mprep's own second pass when the row of Q does not
  // fit shared memory.  Otherwise the responsibilities are formed on request
  // (emc_plan_results, emc_plan_best_quaternions: plan_respons_ready).
  const int write_p = (p->prune != nullptr || (tcm && !stage)) ? 1 : 0;
  mprep_kernel<<<R, kMprepThreads, stage ? sizeof(float) * N : 0, ctx->stream>>>(
      p->L, p->PHI, p->lse2, p->Ksum, p->cnorm, R, N, tcm ? nullptr : p->Q,
      tcm ? p->Qh : nullptr, tcm && p->mstep_q_lo ? p->Ql : nullptr, p->qscale, p->Np, p->T,
      row_mass, row_bound,
      stage, p->prune_tiles ? p->prune_state : nullptr, p->n_rt, p->prune_margin, write_p);
  p->p_written = write_p != 0;
  if ((rc = after_launch(ctx, "mprep_kernel"))) return rc;
  if ((rc = mark_phase(p, 4))) return rc;
  const bool det = p->d.insert_mode == EMC_INSERT_DETERMINISTIC;
  if (det) {
    insert_bounds_kernel<<<1, 256, 0, ctx->stream>>>(
        row_mass, row_bound, R, p->P_eff, p->red + kRedBoundM,
        reinterpret_cast<float2*>(p->red + kRedFixScale));
    if ((rc = after_launch(ctx, "insert_bounds_kernel"))) return rc;
    EMC_CUDA(ctx, cudaMemsetAsync(p->fix_m, 0, sizeof(unsigned long long) * n3, ctx->stream));
    EMC_CUDA(ctx, cudaMemsetAsync(p->fix_w, 0, sizeof(unsigned long long) * n3, ctx->stream));
  } else if (p->d.insert_mode == EMC_INSERT_ATOMIC) {
    EMC_CUDA(ctx, cudaMemsetAsync(p->acc2, 0, sizeof(float2) * n3, ctx->stream));
  }  // sorted: the reduction writes every voxel of acc2
  InsertCtx ins = make_insert_ctx(p, d_model, d_weight);
  if (tcm)
    rc = tc_mstep(p, d_model, d_weight);
  else
    rc = plan_mstep_fp32(p, d_model, d_weight, ins);
  if (!rc && p->d.insert_mode == EMC_INSERT_SORTED) rc = sorted_reduce(p);
  return rc;
}

// model = inserted sums / weight, normalised to a positive mean of 1, blurred
static int enqueue_finish(emc_plan* p, float* d_model, float* d_weight) {
  emc_ctx* ctx = p->ctx;
  const long long n3 = (long long)p->d.side * p->d.side * p->d.side;
  const bool det = p->d.insert_mode == EMC_INSERT_DETERMINISTIC;
  int rc;
  {
    const int nb = (int)std::min<long long>(ceil_div(n3, 256), (long long)ctx->sm_count * 8);
    finish_insert_kernel<<<nb, 256, 0, ctx->stream>>>(det ? p->fix_m : nullptr, p->fix_w,
                                                       reinterpret_cast<const float2*>(p->red + kRedFixScale),
                                                       p->acc2, d_model,
                                                       d_weight, n3);
    if ((rc = after_launch(ctx, "finish_insert_kernel"))) return rc;
  }
  if ((rc = mark_phase(p, 5))) return rc;
  return enqueue_normalise(p, d_model);
}

// model / positive mean (the reference's normalize_model), then the blur
static int enqueue_normalise(emc_plan* p, float* d_model) {
  emc_ctx* ctx = p->ctx;
  const long long n3 = (long long)p->d.side * p->d.side * p->d.side;
  int rc;
  double* mean_stats = p->red + kRedMean;
  // launch_positive_mean writes {sum, count} then its partials after them;
  // kRedMean + 2 + 2*1024 fits in the reduction buffer tail.
  double* tail = p->red + kRedSlots + 2 * (size_t)p->Rp;
  if ((rc = launch_positive_mean(ctx, d_model, n3, tail))) return rc;
  EMC_CUDA(ctx, cudaMemcpyAsync(mean_stats, tail, 2 * sizeof(double), cudaMemcpyDeviceToDevice,
                                ctx->stream));
  if ((rc = launch_scale_by_inverse_mean(ctx, d_model, n3, tail))) return rc;
  if (p->d.blur_sigma > 0.0f) {
    if ((rc = blur_run(ctx, d_model, p->blur))) return rc;
  }
  return mark_phase(p, 6);
}

static int iterate_enqueue(emc_plan* p, float* d_model, float* d_weight) {
  int rc;
  if ((rc = enqueue_estep(p, d_model))) return rc;
  if ((rc = enqueue_lse(p))) return rc;
  if ((rc = enqueue_mstep(p, d_model, d_weight))) return rc;
  return enqueue_finish(p, d_model, d_weight);
}

// Writes one float on a stream with a kernel rather than a host-to-device
// copy: a copy would queue on the copy engine behind any bulk host copy that
// another stream has issued (the next patterns, uploaded while this iteration
// runs) and hold the iteration back until that copy ends.
__global__ void set_float_kernel(float* __restrict__ dst, float v) { *dst = v; }

static int set_sigma(emc_plan* p, float sigma) {
  emc_ctx* ctx = p->ctx;
  EMC_REQUIRE(ctx, sigma > 0.0f && std::isfinite(sigma), "iterate: bad sigma");
  set_float_kernel<<<1, 1, 0, ctx->stream>>>(p->sigma_dev, sigma);
  return after_launch(ctx, "set_float_kernel");
}

extern "C" int emc_iterate_async(emc_plan* p, float* d_model, float* d_weight, float sigma) {
  if (!p) return EMC_ERR_INVALID;
  emc_ctx* ctx = p->ctx;
  EMC_REQUIRE(ctx, p->bound, "iterate: plan not bound");
  EMC_REQUIRE(ctx, d_model && d_weight, "iterate: null model/weight");
  int rc = set_sigma(p, sigma);
  if (rc) return rc;
  return iterate_enqueue(p, d_model, d_weight);
}

// Synchronises, then reports what the device recorded since the last wait:
// a pipeline wait that timed out, slice values outside the FP16 operand
// range; fills stats (of the last iteration) and clears the status words.
extern "C" int emc_plan_wait(emc_plan* p, emc_iter_stats* stats) {
  if (!p) return EMC_ERR_INVALID;
  emc_ctx* ctx = p->ctx;
  const int R = p->d.n_rot, N = p->d.n_images;
  int hflags[8] = {0};
  int tcs = 0;
  int* dtc = tc_status(p);
  double h[kRedSlots];
  std::vector<double> mass(stats ? R : 0);
  EMC_CUDA(ctx, cudaMemcpyAsync(hflags, p->flags, sizeof(hflags), cudaMemcpyDeviceToHost,
                                ctx->stream));
  if (dtc)
    EMC_CUDA(ctx, cudaMemcpyAsync(&tcs, dtc, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  if (stats) {
    EMC_CUDA(ctx, cudaMemcpyAsync(h, p->red, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    EMC_CUDA(ctx, cudaMemcpyAsync(mass.data(), p->red + kRedSlots, sizeof(double) * R,
                                  cudaMemcpyDeviceToHost, ctx->stream));
  }
  EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (dtc && tcs) EMC_CUDA(ctx, cudaMemsetAsync(dtc, 0, sizeof(int), ctx->stream));
  if (hflags[0] & 4) EMC_CUDA(ctx, cudaMemsetAsync(p->flags, 0, sizeof(int), ctx->stream));
  if (tcs)
    return fail(ctx, EMC_ERR_TIMEOUT, "iterate: tensor-core pipeline wait timed out (status 0x%x)",
                tcs);
  if (hflags[0] & 4)
    return fail(ctx, EMC_ERR_UNSUPPORTED, "iterate: slice values exceed the FP16 operand range");
  if (stats) {
    double m = 0.0;
    for (double v : mass) m += v;
    stats->total_loglik = h[kRedLL];
    stats->model_mean_before = h[kRedMean + 1] > 0 ? h[kRedMean] / h[kRedMean + 1] : 0.0;
    stats->captured_mass = m / (double)N;
    stats->bad_pairs = hflags[4];
    stats->reserved = 0;
  }
  return EMC_OK;
}

extern "C" int emc_iterate(emc_plan* p, float* d_model, float* d_weight, float sigma,
                           emc_iter_stats* stats) {
  if (p && p->prune) {
    bool handled = false;
    const int prc = prune_iterate(p, d_model, d_weight, sigma, stats, &handled);
    if (handled || prc) return prc;
  }
  int rc = emc_iterate_async(p, d_model, d_weight, sigma);
  if (rc) return rc;
  return emc_plan_wait(p, stats);
}

extern "C" int emc_plan_capture(emc_plan* p, float* d_model, float* d_weight) {
  if (!p) return EMC_ERR_INVALID;
  emc_ctx* ctx = p->ctx;
  EMC_REQUIRE(ctx, p->bound, "plan_capture: plan not bound");
  EMC_REQUIRE(ctx, d_model && d_weight, "plan_capture: null model/weight");
  EMC_REQUIRE(ctx, ctx->stream != nullptr,
              "plan_capture: the legacy default stream cannot be captured; use emc_set_stream");
  if (p->graph_exec) {
    EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    cudaGraphExecDestroy(p->graph_exec);
    p->graph_exec = nullptr;
  }
  if (p->graph) {
    cudaGraphDestroy(p->graph);
    p->graph = nullptr;
  }
  const bool prof = p->profiling;
  p->profiling = false;  // no event records inside the graph
  EMC_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  const int rc = iterate_enqueue(p, d_model, d_weight);
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
  p->profiling = prof;
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return cuda_fail(ctx, e, "plan_capture: end capture");
  const cudaError_t ei = cudaGraphInstantiate(&p->graph_exec, g, 0);
  if (ei != cudaSuccess) {
    cudaGraphDestroy(g);
    return cuda_fail(ctx, ei, "plan_capture: instantiate");
  }
  p->graph = g;
  return EMC_OK;
}

extern "C" int emc_plan_replay(emc_plan* p, float sigma) {
  if (!p) return EMC_ERR_INVALID;
  emc_ctx* ctx = p->ctx;
  EMC_REQUIRE(ctx, p->graph_exec, "plan_replay: no captured iteration");
  int rc = set_sigma(p, sigma);
  if (rc) return rc;
  EMC_CUDA(ctx, cudaGraphLaunch(p->graph_exec, ctx->stream));
  return EMC_OK;
}

// ---------------------------------------------------------------- batch --
// Several independent reconstructions in one graph launch: each plan's
// captured iteration becomes a child graph of one parent graph with no edges
// between them, so the GPU runs them concurrently.
struct emc_batch {
  std::vector<emc_plan*> plans;
  emc_ctx* ctx = nullptr;  // stream of the launches (the first plan's context)
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

extern "C" int emc_batch_create(emc_plan** plans, float** d_models, float** d_weights, int n,
                                emc_batch** out) {
  if (!plans || !d_models || !d_weights || n <= 0 || !out || !plans[0]) return EMC_ERR_INVALID;
  emc_ctx* ctx = plans[0]->ctx;
  for (int k = 0; k < n; ++k) {
    EMC_REQUIRE(ctx, plans[k] && d_models[k] && d_weights[k], "batch_create: null entry %d", k);
    EMC_REQUIRE(ctx, plans[k]->ctx->device == ctx->device, "batch_create: plans on two devices");
    const int rc = emc_plan_capture(plans[k], d_models[k], d_weights[k]);
    if (rc) return fail(ctx, rc, "batch_create: plan %d: %s", k, emc_last_error(plans[k]->ctx));
  }
  emc_batch* b = new emc_batch();
  b->plans.assign(plans, plans + n);
  b->ctx = ctx;
  cudaError_t e = cudaGraphCreate(&b->graph, 0);
  for (int k = 0; k < n && e == cudaSuccess; ++k) {
    cudaGraphNode_t node;
    e = cudaGraphAddChildGraphNode(&node, b->graph, nullptr, 0, plans[k]->graph);
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
  if (e != cudaSuccess) {
    emc_batch_destroy(b);
    return cuda_fail(ctx, e, "batch_create");
  }
  *out = b;
  return EMC_OK;
}

extern "C" int emc_batch_run(emc_batch* b, const float* sigmas) {
  if (!b || !sigmas) return EMC_ERR_INVALID;
  emc_ctx* ctx = b->ctx;
  for (size_t k = 0; k < b->plans.size(); ++k) {
    const float sg = sigmas[k];
    EMC_REQUIRE(ctx, sg > 0.0f && std::isfinite(sg), "batch_run: bad sigma %zu", k);
    set_float_kernel<<<1, 1, 0, ctx->stream>>>(b->plans[k]->sigma_dev, sg);
    int rc = after_launch(ctx, "set_float_kernel");
    if (rc) return rc;
  }
  EMC_CUDA(ctx, cudaGraphLaunch(b->exec, ctx->stream));
  return EMC_OK;
}

extern "C" int emc_batch_wait(emc_batch* b, emc_iter_stats* stats) {
  if (!b) return EMC_ERR_INVALID;
  emc_ctx* ctx = b->ctx;
  EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  int first = EMC_OK;
  for (size_t k = 0; k < b->plans.size(); ++k) {
    emc_plan* p = b->plans[k];
    const int rc = emc_plan_wait(p, stats ? stats + k : nullptr);
    if (rc && !first) first = fail(ctx, rc, "batch: plan %zu: %s", k, emc_last_error(p->ctx));
    // the status resets of emc_plan_wait run on the plan's own stream
    cudaStreamSynchronize(p->ctx->stream);
  }
  return first;
}

extern "C" int emc_batch_destroy(emc_batch* b) {
  if (!b) return EMC_OK;
  if (b->ctx) cudaStreamSynchronize(b->ctx->stream);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  delete b;
  return EMC_OK;
}

extern "C" int emc_plan_get_option(const emc_plan* p, int option, int* value) {
  if (!p || !value) return EMC_ERR_INVALID;
  emc_ctx* ctx = p->ctx;
  switch (option) {
    case EMC_OPT_MSTEP_QLO: *value = p->mstep_q_lo; return EMC_OK;
    case EMC_OPT_ESTEP_GHLO: *value = p->estep_gh_lo; return EMC_OK;
    case EMC_OPT_MSTEP_AGGREGATE: *value = p->mstep_aggregate; return EMC_OK;
    case EMC_OPT_COUNTS_ROUND: *value = p->counts_round; return EMC_OK;
    case EMC_OPT_ESTEP_RASTER: *value = p->estep_raster; return EMC_OK;
    case EMC_OPT_ESTEP_PAIR: *value = p->estep_pair; return EMC_OK;
    case EMC_OPT_MSTEP_RASTER: *value = p->mstep_raster; return EMC_OK;
    case EMC_OPT_DEBUG_SPIN: *value = (int)p->debug_spin; return EMC_OK;
    case EMC_OPT_MSTEP_PAIR: *value = p->mstep_pair; return EMC_OK;
    case EMC_OPT_GLO_TAIL: *value = p->glo_tail_ppm; return EMC_OK;
    default: return fail(ctx, EMC_ERR_INVALID, "plan_get_option: unknown option %d", option);
  }
}

extern "C" int emc_plan_set_option(emc_plan* p, int option, int value) {
  if (!p) return EMC_ERR_INVALID;
  emc_ctx* ctx = p->ctx;
  if (option == EMC_OPT_ESTEP_GHLO) {
    EMC_REQUIRE(ctx, value >= -1 && value <= 3, "plan_set_option: gh_lo %d", value);
    p->estep_gh_lo = value;
    return EMC_OK;
  }
  if (option == EMC_OPT_ESTEP_RASTER) {
    EMC_REQUIRE(ctx, value != 0 && value >= -4096 && value <= 4096,
                "plan_set_option: raster %d", value);
    p->estep_raster = value;
    return EMC_OK;
  }
  if (option == EMC_OPT_MSTEP_RASTER) {
    EMC_REQUIRE(ctx, value != 0 && value >= -4096 && value <= 4096,
                "plan_set_option: M-step raster %d", value);
    p->mstep_raster = value;
    return EMC_OK;
  }
  if (option == EMC_OPT_ESTEP_PAIR) {
    EMC_REQUIRE(ctx, value == 0 || value == 1, "plan_set_option: pair %d", value);
    p->estep_pair = value;
    return EMC_OK;
  }
  if (option == EMC_OPT_MSTEP_PAIR) {
    EMC_REQUIRE(ctx, value == 0 || value == 1, "plan_set_option: M-step pair %d", value);
    p->mstep_pair = value;
    return EMC_OK;
  }
  if (option == EMC_OPT_DEBUG_SPIN) {
    EMC_REQUIRE(ctx, value >= 0, "plan_set_option: debug spin %d", value);
    p->debug_spin = (unsigned)value;
    return EMC_OK;
  }
  if (option == EMC_OPT_MSTEP_AGGREGATE) {
    EMC_REQUIRE(ctx, value == 0 || value == 1, "plan_set_option: aggregate %d", value);
    p->mstep_aggregate = value;
    return EMC_OK;
  }
  if (option == EMC_OPT_COUNTS_ROUND) {
    EMC_REQUIRE(ctx, value == 0 || value == 1, "plan_set_option: counts_round %d", value);
    EMC_REQUIRE(ctx, !p->tc, "plan_set_option: set EMC_OPT_COUNTS_ROUND before bind");
    p->counts_round = value;
    return EMC_OK;
  }
  if (option == EMC_OPT_GLO_TAIL) {
    EMC_REQUIRE(ctx, value >= 0 && value <= 1000000, "plan_set_option: G lo tail %d", value);
    p->glo_tail_ppm = value;
    return p->tc ? tc_glo_extent(p) : EMC_OK;
  }
  if (option == EMC_OPT_MSTEP_QLO) {
    EMC_REQUIRE(ctx, value == 0 || value == 1, "plan_set_option: q_lo %d", value);
    p->mstep_q_lo = value;
    return value ? tc_ensure_qlo(p) : EMC_OK;
  }
  return fail(ctx, EMC_ERR_INVALID, "plan_set_option: unknown option %d", option);
}

extern "C" int emc_plan_autotune(emc_plan* p, const float* d_model, float sigma, int* h_raster,
                                 float* h_ms) {
  if (!p) return EMC_ERR_INVALID;
  emc_ctx* ctx = p->ctx;
  EMC_REQUIRE(ctx, p->bound, "autotune: plan not bound");
  EMC_REQUIRE(ctx, d_model, "autotune: null model");
  if (p->d.precision != EMC_PREC_MIXED) {  // the FP32 path has no tile order to tune
    if (h_raster) *h_raster = 0;
    if (h_ms) *h_ms = 0.0f;
    return EMC_OK;
  }
  int rc = set_sigma(p, sigma);
  if (!rc) rc = plan_expand(p, d_model);
  if (!rc) rc = tc_autotune(p, 256, h_raster, h_ms);
  // the timed launches count non-finite pairs of partial grids: not an iteration's
  if (!rc) EMC_CUDA(ctx, cudaMemsetAsync(p->flags + 4, 0, sizeof(int), ctx->stream));
  if (!rc) EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return rc;
}

extern "C" int emc_plan_time_likelihood(emc_plan* p, const float* d_model, float sigma,
                                        int raster, int first_tile, int n_tiles, float* h_ms,
                                        int* h_total_tiles) {
  if (!p) return EMC_ERR_INVALID;
  emc_ctx* ctx = p->ctx;
  EMC_REQUIRE(ctx, p->bound, "time_likelihood: plan not bound");
  EMC_REQUIRE(ctx, p->d.precision == EMC_PREC_MIXED, "time_likelihood: tensor-core plans only");
  EMC_REQUIRE(ctx, raster != 0 && raster >= -4096 && raster <= 4096 && first_tile >= 0 &&
                       n_tiles > 0 && h_ms, "time_likelihood: bad arguments");
  int rc = EMC_OK;
  if (d_model) {
    rc = set_sigma(p, sigma);
    if (!rc) rc = plan_expand(p, d_model);
  }
  if (!rc) rc = tc_time_estep(p, raster, first_tile, n_tiles, h_ms);
  if (!rc && h_total_tiles) *h_total_tiles = tc_estep_tiles(p);
  if (!rc) EMC_CUDA(ctx, cudaMemsetAsync(p->flags + 4, 0, sizeof(int), ctx->stream));
  return rc;
}

extern "C" int emc_plan_set_profiling(emc_plan* p, int on) {
  if (!p) return EMC_ERR_INVALID;
  emc_ctx* ctx = p->ctx;
  if (on && !p->ev[0]) {
    for (auto& e : p->ev) EMC_CUDA(ctx, cudaEventCreate(&e));
  }
  p->profiling = on != 0;
  return EMC_OK;
}

extern "C" int emc_plan_phase_ms(emc_plan* p, float* ms, int n) {
  if (!p || !ms || n < 0) return EMC_ERR_INVALID;
  emc_ctx* ctx = p->ctx;
  EMC_REQUIRE(ctx, p->profiling, "plan_phase_ms: profiling is off");
  EMC_CUDA(ctx, cudaEventSynchronize(p->ev[emc_plan::kPhases]));
  for (int i = 0; i < n && i < emc_plan::kPhases; ++i)
    EMC_CUDA(ctx, cudaEventElapsedTime(ms + i, p->ev[i], p->ev[i + 1]));
  return EMC_OK;
}

extern "C" int emc_plan_results(emc_plan* p, const float** d_respons, const float** d_scaling,
                                const double** d_lse) {
  if (!p) return EMC_ERR_INVALID;
  if (d_respons) {
    const int rc = plan_respons_ready(p);
    if (rc) return rc;
  }
  if (d_respons) *d_respons = p->L;
  if (d_scaling) *d_scaling = p->PHI;
  if (d_lse) *d_lse = p->lse;
  return EMC_OK;
}

// ---- one rank of the reference's rotation split (main.cpp:141-154) -------
extern "C" int emc_rank_estep(emc_plan* p, float* d_model, float sigma, float* d_max,
                              double* d_sumexp) {
  if (!p) return EMC_ERR_INVALID;
  emc_ctx* ctx = p->ctx;
  EMC_REQUIRE(ctx, p->bound, "rank_estep: plan not bound");
  EMC_REQUIRE(ctx, d_model && d_max && d_sumexp, "rank_estep: null argument");
  EMC_REQUIRE(ctx, !p->prune, "rank_estep: pruning is not supported on a rotation split");
  int rc = set_sigma(p, sigma);
  if (rc) return rc;
  if ((rc = enqueue_estep(p, d_model))) return rc;
  const int N = p->d.n_images;
  rank_partial_kernel<<<ceil_div(N, 256), 256, 0, ctx->stream>>>(p->part, p->n_rt, N, d_max,
                                                                 d_sumexp);
  return after_launch(ctx, "rank_partial_kernel");
}

extern "C" int emc_rank_mstep(emc_plan* p, const double* d_lse, float* d_model_sum,
                              float* d_weight_sum) {
  if (!p) return EMC_ERR_INVALID;
  emc_ctx* ctx = p->ctx;
  EMC_REQUIRE(ctx, p->bound, "rank_mstep: plan not bound");
  EMC_REQUIRE(ctx, d_lse && d_model_sum && d_weight_sum, "rank_mstep: null argument");
  EMC_REQUIRE(ctx, !p->prune, "rank_mstep: pruning is not supported on a rotation split");
  const int N = p->d.n_images;
  const long long n3 = (long long)p->d.side * p->d.side * p->d.side;
  lse_from_global_kernel<<<ceil_div(N, 256), 256, 0, ctx->stream>>>(d_lse, N, p->lse, p->lse2);
  int rc = after_launch(ctx, "lse_from_global_kernel");
  if (rc) return rc;
  finite_sum_kernel<<<1, 256, 0, ctx->stream>>>(p->lse, N, p->red + kRedLL);
  if ((rc = after_launch(ctx, "finite_sum_kernel"))) return rc;
  if ((rc = mark_phase(p, 3))) return rc;
  if ((rc = enqueue_mstep(p, d_model_sum, d_weight_sum))) return rc;
  const bool det = p->d.insert_mode == EMC_INSERT_DETERMINISTIC;
  const int nb = (int)std::min<long long>(ceil_div(n3, 256), (long long)ctx->sm_count * 8);
  sums_out_kernel<<<nb, 256, 0, ctx->stream>>>(det ? p->fix_m : nullptr, p->fix_w,
                                                reinterpret_cast<const float2*>(p->red + kRedFixScale),
                                                p->acc2, d_model_sum,
                                                d_weight_sum, n3);
  return after_launch(ctx, "sums_out_kernel");
}

extern "C" int emc_model_from_sums(emc_plan* p, const float* d_model_sum,
                                   const float* d_weight_sum, int n_ranks, float* d_model,
                                   float* d_weight) {
  if (!p) return EMC_ERR_INVALID;
  emc_ctx* ctx = p->ctx;
  EMC_REQUIRE(ctx, d_model_sum && d_weight_sum && d_model && d_weight && n_ranks >= 1,
              "model_from_sums: bad argument");
  const long long n3 = (long long)p->d.side * p->d.side * p->d.side;
  const int nb = (int)std::min<long long>(ceil_div(n3, 256), (long long)ctx->sm_count * 8);
  model_from_sums_kernel<<<nb, 256, 0, ctx->stream>>>(d_model_sum, d_weight_sum, (float)n_ranks,
                                                       d_model, d_weight, n3);
  int rc = after_launch(ctx, "model_from_sums_kernel");
  if (rc) return rc;
  if ((rc = mark_phase(p, 5))) return rc;
  return enqueue_normalise(p, d_model);
}
