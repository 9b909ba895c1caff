// Learned rotation proposal: a small convolutional network that maps a
// diffraction pattern to a rotation, trained on the GPU (forward, backward
// and Adam kernels below) on the most probable rotations of EMC's own
// responsibilities, and used to seed pruned iterations
// (emc_plan_set_proposals) for patterns that have no responsibilities yet.
// The reference has no counterpart; the network follows the
// rotation-proposal design of the EMC iteration's pruning: 4 convolutions
// (3x3, stride 2, 64 channels, ReLU) over the pattern binned to 64 x 64
// pixels, one linear layer to a 6D rotation (the first two columns of the
// rotation matrix, made orthonormal by Gram-Schmidt).
//
// Friedel symmetry makes a pattern at rotation M nearly identical to the one
// at M diag(-1, -1, 1) (a half turn about the beam axis; they differ only
// through the Ewald sphere's curvature), whose 6D form is exactly the
// negative.  The loss is therefore min(|o - t|^2, |o + t|^2) per pattern,
// and a prediction proposes both rotations.
//
// Arithmetic is FP32 SIMT: one forward pass is 26 MFLOP per pattern,
// under 1 % of a 128^3 iteration's E-step per pattern, so the tensor cores
// stay with the iteration's contractions.  Every reduction has a fixed order
// (no atomics), so training is reproducible for a given seed.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "emc_gb300.h"
#include "geometry.cuh"
#include "plan.cuh"

namespace emc {
namespace pn {
constexpr int D = 64;              // input side
constexpr int CH = 64;             // channels of every convolution
constexpr int NCONV = 4;
constexpr int FC_IN = CH * 4 * 4;  // 1024
constexpr int OUT = 6;
constexpr int TILE = 64;           // GEMM tile (rows x columns) of the convolution kernels
constexpr int KCH = 32;            // reduction chunk of the convolution kernels
constexpr int WG_COLS = 1024;      // columns per partial of the weight-gradient kernel

__host__ __device__ constexpr int cin(int l) { return l == 0 ? 1 : CH; }
__host__ __device__ constexpr int hin(int l) { return D >> l; }  // 64, 32, 16, 8
}  // namespace pn

struct ProposalNet {
  emc_ctx* ctx = nullptr;
  size_t off_w[pn::NCONV], off_b[pn::NCONV], off_fw = 0, off_fb = 0, n_params = 0;
  float *params = nullptr, *grads = nullptr, *adam_m = nullptr, *adam_v = nullptr;
  long long adam_t = 0;
  // inputs
  float* X = nullptr;  // [n][64*64]
  int n_data = 0;
  float* stats = nullptr;  // [2][4096]: per-input-pixel mean and 1 / spread of the training data
  bool have_stats = false;
  // per-batch workspace (capacity cap samples)
  int cap = 0;
  float* act[pn::NCONV + 1] = {};  // act[0] = gathered inputs, act[l+1] = output of conv l
  float* out = nullptr;            // [cap][6]
  float *g0 = nullptr, *g1 = nullptr;  // ping-pong activation gradients (largest layer)
  float* gout = nullptr;               // [cap][6]
  float* wpart = nullptr;              // weight-gradient partials
  size_t wpart_cap = 0;
  float* loss = nullptr;               // [cap]
  int* idx = nullptr;                  // [cap] sample -> data row
  int* quarter = nullptr;              // [cap] in-plane quarter turns of the sample
  float* labels6 = nullptr;            // [cap][6]
};

// ------------------------------------------------------------ inputs -----
// X[j] = log1p(v * 4096 / max(sum v, 1)), v = the pattern's counts summed
// over b x b pixel blocks (b = side / 64) inside the mask (negative counts,
// the per-pattern masked pixels, count 0); then standardised per input pixel
// with the training data's mean and spread (the radial falloff that every
// pattern shares carries no orientation).
__global__ void proposal_inputs_kernel(const float* __restrict__ images,
                                       const int* __restrict__ mask, int side, int n,
                                       float* __restrict__ X) {
  const int i = blockIdx.x;
  if (i >= n) return;
  const int b = side / pn::D;
  const float* im = images + (size_t)i * side * side;
  float v[16];
  float s = 0.0f;
  for (int u = 0; u < 16; ++u) {
    const int o = threadIdx.x + u * 256;  // output pixel 0..4095
    const int oy = o / pn::D, ox = o % pn::D;
    float a = 0.0f;
    for (int dy = 0; dy < b; ++dy)
      for (int dx = 0; dx < b; ++dx) {
        const int p = (oy * b + dy) * side + ox * b + dx;
        const float k = im[p];
        if (mask[p] > 0 && k > 0.0f) a += k;
      }
    v[u] = a;
    s += a;
  }
  __shared__ float red[256];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  const float scale = 4096.0f / fmaxf(red[0], 1.0f);
  for (int u = 0; u < 16; ++u)
    X[(size_t)i * 4096 + threadIdx.x + u * 256] = log1pf(v[u] * scale);
}

// Batch inputs: row idx[j] of X turned in-plane by quarter[j] x 90 degrees
// (nullptr: not turned).  A turn by +90 degrees, X'(u, v) = X(v, -u) in
// centred coordinates, is the pattern of rotation M Rz(-90 deg): exact on
// the 64 x 64 grid, whose mask and pixel heights are symmetric under it.
// stats[0][c] = mean over rows of X[.][c], stats[1][c] = 1 / sqrt(var + 1e-4)
// (FP64 sums in row order); one thread per input pixel.
__global__ void input_stats_kernel(const float* __restrict__ X, int n, float* __restrict__ stats) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= 4096) return;
  double s = 0.0, s2 = 0.0;
  for (int i = 0; i < n; ++i) {
    const double v = X[(size_t)i * 4096 + c];
    s += v;
    s2 += v * v;
  }
  const double m = s / n;
  const double var = fmax(s2 / n - m * m, 0.0);
  stats[c] = (float)m;
  stats[4096 + c] = (float)(1.0 / sqrt(var + 1e-4));
}

// X[i][c] = (X[i][c] - mean[c]) * inv[c].
__global__ void standardize_kernel(float* __restrict__ X, size_t n, const float* __restrict__ stats) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * 4096) return;
  const int c = (int)(e % 4096);
  X[e] = (X[e] - stats[c]) * stats[4096 + c];
}

__global__ void gather_rows_kernel(const float* __restrict__ X, const int* __restrict__ idx,
                                   const int* __restrict__ quarter, int rows,
                                   float* __restrict__ out) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)rows * 4096) return;
  const int j = (int)(e / 4096), c = (int)(e % 4096);
  int oy = c / pn::D, ox = c % pn::D;
  const int k = quarter ? (quarter[j] & 3) : 0;
  for (int t = 0; t < k; ++t) {  // source of one +90 degree turn: (63 - ox, oy) as (row, col)
    const int ny = pn::D - 1 - ox, nx = oy;
    oy = ny;
    ox = nx;
  }
  out[e] = X[(size_t)idx[j] * 4096 + oy * pn::D + ox];
}

// ------------------------------------------------------- convolutions ----
// Forward: out[b][co][p] = relu(bias[co] + sum_{ci,t} W[co][ci*9+t] in[b][ci][tap(p,t)])
// as a GEMM of W (64 x Cin*9) by the implicit column matrix (Cin*9 x B*Ho*Ho).
// Block: 64 output channels x 64 columns, 256 threads with 4 x 4 outputs each.
__global__ void __launch_bounds__(256) conv_fwd_kernel(const float* __restrict__ in,
                                                       const float* __restrict__ W,
                                                       const float* __restrict__ bias,
                                                       float* __restrict__ out, int B, int Cin,
                                                       int Hin) {
  const int Ho = Hin / 2, npx = Ho * Ho, ncol = B * npx, K = Cin * 9;
  const int n0 = blockIdx.x * pn::TILE;
  __shared__ float sW[pn::KCH][pn::TILE + 4];  // [k][co]
  __shared__ float sX[pn::KCH][pn::TILE + 4];  // [k][column]
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += pn::KCH) {
    for (int e = threadIdx.x; e < pn::KCH * pn::TILE; e += 256) {
      const int kk = e / pn::TILE, c = e % pn::TILE;  // c: co for sW, column for sX
      const int k = k0 + kk;
      sW[kk][c] = k < K ? W[(size_t)c * K + k] : 0.0f;
      float v = 0.0f;
      const int n = n0 + c;
      if (k < K && n < ncol) {
        const int b = n / npx, p = n % npx;
        const int ci = k / 9, t = k % 9;
        const int yi = 2 * (p / Ho) + t / 3 - 1, xi = 2 * (p % Ho) + t % 3 - 1;
        if (yi >= 0 && yi < Hin && xi >= 0 && xi < Hin)
          v = in[(((size_t)b * Cin + ci) * Hin + yi) * Hin + xi];
      }
      sX[kk][c] = v;
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < pn::KCH; ++kk) {
      float a[4], x[4];
      for (int i = 0; i < 4; ++i) a[i] = sW[kk][ty * 4 + i];
      for (int j = 0; j < 4; ++j) x[j] = sX[kk][tx * 4 + j];
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], x[j], acc[i][j]);
    }
    __syncthreads();
  }
  for (int j = 0; j < 4; ++j) {
    const int n = n0 + tx * 4 + j;
    if (n >= ncol) continue;
    const int b = n / npx, p = n % npx;
    for (int i = 0; i < 4; ++i) {
      const int co = ty * 4 + i;
      out[((size_t)b * pn::CH + co) * npx + p] = fmaxf(acc[i][j] + bias[co], 0.0f);
    }
  }
}

// Backward through ReLU and the convolution to its input:
// gin[b][ci][q] = sum_{co,t} W[co][ci*9+t] d[b][co][p(q,t)], d = gout * (out > 0),
// over the output pixels p whose tap t reads input pixel q.  GEMM of W^T
// (Cin x 64*9) by the gathered d (64*9 x B*Hin*Hin).
__global__ void __launch_bounds__(256) conv_bwd_data_kernel(const float* __restrict__ gout,
                                                            const float* __restrict__ out,
                                                            const float* __restrict__ W,
                                                            float* __restrict__ gin, int B,
                                                            int Cin, int Hin) {
  const int Ho = Hin / 2, npx = Ho * Ho, nin = Hin * Hin, ncol = B * nin, K = pn::CH * 9;
  const int n0 = blockIdx.x * pn::TILE, c0 = blockIdx.y * pn::TILE;
  __shared__ float sW[pn::KCH][pn::TILE + 4];  // [k = co*9 + t][ci]
  __shared__ float sG[pn::KCH][pn::TILE + 4];  // [k][column]
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += pn::KCH) {
    for (int e = threadIdx.x; e < pn::KCH * pn::TILE; e += 256) {
      const int kk = e / pn::TILE, c = e % pn::TILE;
      const int k = k0 + kk, co = k / 9, t = k % 9;
      const int ci = c0 + c;
      sW[kk][c] = ci < Cin ? W[(size_t)co * Cin * 9 + ci * 9 + t] : 0.0f;
      float v = 0.0f;
      const int n = n0 + c;
      if (n < ncol) {
        const int b = n / nin, q = n % nin;
        const int ty2 = q / Hin + 1 - t / 3, tx2 = q % Hin + 1 - t % 3;  // 2y, 2x
        if (ty2 >= 0 && tx2 >= 0 && !(ty2 & 1) && !(tx2 & 1) && ty2 / 2 < Ho && tx2 / 2 < Ho) {
          const size_t o = ((size_t)b * pn::CH + co) * npx + (ty2 / 2) * Ho + tx2 / 2;
          v = out[o] > 0.0f ? gout[o] : 0.0f;
        }
      }
      sG[kk][c] = v;
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < pn::KCH; ++kk) {
      float a[4], x[4];
      for (int i = 0; i < 4; ++i) a[i] = sW[kk][ty * 4 + i];
      for (int j = 0; j < 4; ++j) x[j] = sG[kk][tx * 4 + j];
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], x[j], acc[i][j]);
    }
    __syncthreads();
  }
  for (int j = 0; j < 4; ++j) {
    const int n = n0 + tx * 4 + j;
    if (n >= ncol) continue;
    const int b = n / nin, q = n % nin;
    for (int i = 0; i < 4; ++i) {
      const int ci = c0 + ty * 4 + i;
      if (ci < Cin) gin[((size_t)b * Cin + ci) * nin + q] = acc[i][j];
    }
  }
}

// Weight gradient partials: part[s][co][k] = sum over columns n of chunk s of
// d[co][n] col[k][n] (d = gout * (out > 0), col the implicit input columns);
// chunk s covers columns [s * WG_COLS, (s + 1) * WG_COLS).  Block: 64 co x 64
// k for one chunk.
__global__ void __launch_bounds__(256) conv_wgrad_kernel(const float* __restrict__ gout,
                                                         const float* __restrict__ out,
                                                         const float* __restrict__ in,
                                                         float* __restrict__ part, int B, int Cin,
                                                         int Hin) {
  const int Ho = Hin / 2, npx = Ho * Ho, ncol = B * npx, K = Cin * 9;
  const int k0 = blockIdx.x * pn::TILE, s = blockIdx.y;
  const int nb = s * pn::WG_COLS, ne = min(ncol, nb + pn::WG_COLS);
  __shared__ float sD[pn::KCH][pn::TILE + 4];  // [n][co]
  __shared__ float sC[pn::KCH][pn::TILE + 4];  // [n][k]
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  float acc[4][4] = {};
  for (int c0 = nb; c0 < ne; c0 += pn::KCH) {
    for (int e = threadIdx.x; e < pn::KCH * pn::TILE; e += 256) {
      const int nn = e / pn::TILE, c = e % pn::TILE;
      const int n = c0 + nn;
      float dv = 0.0f, cv = 0.0f;
      if (n < ne) {
        const int b = n / npx, p = n % npx;
        const size_t o = ((size_t)b * pn::CH + c) * npx + p;
        dv = out[o] > 0.0f ? gout[o] : 0.0f;
        const int k = k0 + c;
        if (k < K) {
          const int ci = k / 9, t = k % 9;
          const int yi = 2 * (p / Ho) + t / 3 - 1, xi = 2 * (p % Ho) + t % 3 - 1;
          if (yi >= 0 && yi < Hin && xi >= 0 && xi < Hin)
            cv = in[(((size_t)b * Cin + ci) * Hin + yi) * Hin + xi];
        }
      }
      sD[nn][c] = dv;
      sC[nn][c] = cv;
    }
    __syncthreads();
#pragma unroll 8
    for (int nn = 0; nn < pn::KCH; ++nn) {
      float a[4], x[4];
      for (int i = 0; i < 4; ++i) a[i] = sD[nn][ty * 4 + i];
      for (int j = 0; j < 4; ++j) x[j] = sC[nn][tx * 4 + j];
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], x[j], acc[i][j]);
    }
    __syncthreads();
  }
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      const int co = ty * 4 + i, k = k0 + tx * 4 + j;
      if (k < K) part[((size_t)s * pn::CH + co) * K + k] = acc[i][j];
    }
}

// grad[e] = sum_s part[s][e] (fixed order), e < n.
__global__ void sum_parts_kernel(const float* __restrict__ part, int S, int n,
                                 float* __restrict__ grad) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  float a = 0.0f;
  for (int s = 0; s < S; ++s) a += part[(size_t)s * n + e];
  grad[e] = a;
}

// gbias[co] = sum_{b,p} gout * (out > 0); one block per channel.
__global__ void conv_bgrad_kernel(const float* __restrict__ gout, const float* __restrict__ out,
                                  int B, int npx, float* __restrict__ gbias) {
  const int co = blockIdx.x;
  float a = 0.0f;
  for (int n = threadIdx.x; n < B * npx; n += 256) {
    const size_t o = ((size_t)(n / npx) * pn::CH + co) * npx + n % npx;
    if (out[o] > 0.0f) a += gout[o];
  }
  __shared__ float red[256];
  red[threadIdx.x] = a;
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) gbias[co] = red[0];
}

// ---------------------------------------------------------- linear head --
// o[b][j] = fb[j] + sum_k fw[j][k] h[b][k]; one block per sample.
__global__ void fc_fwd_kernel(const float* __restrict__ h, const float* __restrict__ fw,
                              const float* __restrict__ fb, float* __restrict__ o) {
  const int b = blockIdx.x;
  __shared__ float red[pn::OUT][256];
  for (int j = 0; j < pn::OUT; ++j) {
    float a = 0.0f;
    for (int k = threadIdx.x; k < pn::FC_IN; k += 256)
      a = fmaf(fw[j * pn::FC_IN + k], h[(size_t)b * pn::FC_IN + k], a);
    red[j][threadIdx.x] = a;
  }
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      for (int j = 0; j < pn::OUT; ++j) red[j][threadIdx.x] += red[j][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x < pn::OUT) o[b * pn::OUT + threadIdx.x] = red[threadIdx.x][0] + fb[threadIdx.x];
}

// gh[b][k] = sum_j fw[j][k] go[b][j]; gfw[j][k] = sum_b go[b][j] h[b][k];
// gfb[j] = sum_b go[b][j].  One thread per k (all samples).
__global__ void fc_bwd_kernel(const float* __restrict__ h, const float* __restrict__ fw,
                              const float* __restrict__ go, int B, float* __restrict__ gh,
                              float* __restrict__ gfw, float* __restrict__ gfb) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < pn::FC_IN) {
    float g[pn::OUT] = {};
    for (int b = 0; b < B; ++b) {
      const float hv = h[(size_t)b * pn::FC_IN + k];
      float a = 0.0f;
      for (int j = 0; j < pn::OUT; ++j) {
        const float gj = go[b * pn::OUT + j];
        g[j] = fmaf(gj, hv, g[j]);
        a = fmaf(fw[j * pn::FC_IN + k], gj, a);
      }
      gh[(size_t)b * pn::FC_IN + k] = a;
    }
    for (int j = 0; j < pn::OUT; ++j) gfw[j * pn::FC_IN + k] = g[j];
  }
  if (blockIdx.x == 0 && threadIdx.x < pn::OUT) {
    float a = 0.0f;
    for (int b = 0; b < B; ++b) a += go[b * pn::OUT + threadIdx.x];
    gfb[threadIdx.x] = a;
  }
}

// ------------------------------------------------------------ rotations --
// 6D form of a rotation: the first two columns of its matrix (as used by the
// slicing kernels: rotated = M p).
__device__ __forceinline__ void quat_to_6d(const float* q, float* t) {
  const RotMat m = quat_to_matrix(q);
  t[0] = m.m[0]; t[1] = m.m[3]; t[2] = m.m[6];
  t[3] = m.m[1]; t[4] = m.m[4]; t[5] = m.m[7];
}

// labels6[j] = 6D form of quats[idx[j]] composed with Rz(-90 deg) quarter[j]
// times: (c1, c2) -> (-c2, c1) per turn.
__global__ void labels_kernel(const float* __restrict__ quats, const int* __restrict__ idx,
                              const int* __restrict__ quarter, int B,
                              float* __restrict__ labels6) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= B) return;
  float t[6];
  quat_to_6d(quats + 4 * (size_t)idx[j], t);
  const int k = quarter ? (quarter[j] & 3) : 0;
  for (int u = 0; u < k; ++u) {
    const float a0 = t[0], a1 = t[1], a2 = t[2];
    t[0] = -t[3]; t[1] = -t[4]; t[2] = -t[5];
    t[3] = a0; t[4] = a1; t[5] = a2;
  }
  for (int c = 0; c < 6; ++c) labels6[6 * j + c] = t[c];
}

// loss[j] = min(|o - t|^2, |o + t|^2); go = (2 / B)(o -+ t) of the smaller.
__global__ void loss_kernel(const float* __restrict__ o, const float* __restrict__ t, int B,
                            float* __restrict__ loss, float* __restrict__ go) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= B) return;
  float dp = 0.0f, dm = 0.0f;
  for (int c = 0; c < pn::OUT; ++c) {
    const float a = o[6 * j + c], b = t[6 * j + c];
    dp += (a - b) * (a - b);
    dm += (a + b) * (a + b);
  }
  const float s = dp <= dm ? 1.0f : -1.0f;
  loss[j] = fminf(dp, dm);
  const float f = 2.0f / (float)B;
  for (int c = 0; c < pn::OUT; ++c) go[6 * j + c] = f * (o[6 * j + c] - s * t[6 * j + c]);
}

// Gram-Schmidt of the 6D output to a rotation matrix, then its quaternion
// (Shepperd's method: the largest of 1 + trace and the 1 + 2 m_ii - trace
// picks the stable formula), canonical with w >= 0.
__device__ void six_d_to_quat(const float* o, float* q) {
  float a[3] = {o[0], o[1], o[2]}, b[3] = {o[3], o[4], o[5]};
  float na = sqrtf(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  if (!(na > 1e-20f)) {
    a[0] = 1.0f; a[1] = 0.0f; a[2] = 0.0f;
    na = 1.0f;
  }
  for (int c = 0; c < 3; ++c) a[c] /= na;
  const float d = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
  for (int c = 0; c < 3; ++c) b[c] -= d * a[c];
  float nb = sqrtf(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
  if (!(nb > 1e-20f)) {  // any unit vector orthogonal to a
    const int ax = fabsf(a[0]) < 0.9f ? 0 : 1;
    float e[3] = {0.0f, 0.0f, 0.0f};
    e[ax] = 1.0f;
    const float de = a[ax];
    for (int c = 0; c < 3; ++c) b[c] = e[c] - de * a[c];
    nb = sqrtf(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
  }
  for (int c = 0; c < 3; ++c) b[c] /= nb;
  const float r3[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2],
                       a[0] * b[1] - a[1] * b[0]};
  // row-major m with columns a, b, r3
  const float m0 = a[0], m1 = b[0], m2 = r3[0];
  const float m3 = a[1], m4 = b[1], m5 = r3[1];
  const float m6 = a[2], m7 = b[2], m8 = r3[2];
  const float tr = m0 + m4 + m8;
  float w, x, y, z;
  if (tr > 0.0f) {
    const float S = sqrtf(tr + 1.0f) * 2.0f;
    w = 0.25f * S; x = (m7 - m5) / S; y = (m2 - m6) / S; z = (m3 - m1) / S;
  } else if (m0 > m4 && m0 > m8) {
    const float S = sqrtf(1.0f + m0 - m4 - m8) * 2.0f;
    w = (m7 - m5) / S; x = 0.25f * S; y = (m1 + m3) / S; z = (m2 + m6) / S;
  } else if (m4 > m8) {
    const float S = sqrtf(1.0f + m4 - m0 - m8) * 2.0f;
    w = (m2 - m6) / S; x = (m1 + m3) / S; y = 0.25f * S; z = (m5 + m7) / S;
  } else {
    const float S = sqrtf(1.0f + m8 - m0 - m4) * 2.0f;
    w = (m3 - m1) / S; x = (m2 + m6) / S; y = (m5 + m7) / S; z = 0.25f * S;
  }
  const float n = sqrtf(w * w + x * x + y * y + z * z);
  const float sg = w < 0.0f ? -1.0f / n : 1.0f / n;
  q[0] = w * sg; q[1] = x * sg; q[2] = y * sg; q[3] = z * sg;
}

// quats[row][0] = the predicted rotation, quats[row][1] = its Friedel mate
// q (x) (0, 0, 0, 1) = (-z, y, -x, w), both with w >= 0.
__global__ void predict_quats_kernel(const float* __restrict__ o, const int* __restrict__ idx,
                                     int B, float* __restrict__ quats) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= B) return;
  float q[4];
  six_d_to_quat(o + 6 * j, q);
  float* d = quats + 8 * (size_t)idx[j];
  for (int c = 0; c < 4; ++c) d[c] = q[c];
  float m[4] = {-q[3], q[2], -q[1], q[0]};
  const float sg = m[0] < 0.0f ? -1.0f : 1.0f;
  for (int c = 0; c < 4; ++c) d[4 + c] = sg * m[c];
}

__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g,
                            float* __restrict__ m, float* __restrict__ v, size_t n, float lr_t,
                            float b1, float b2, float eps) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const float ge = g[e];
  const float me = b1 * m[e] + (1.0f - b1) * ge;
  const float ve = b2 * v[e] + (1.0f - b2) * ge * ge;
  m[e] = me;
  v[e] = ve;
  p[e] -= lr_t * me / (sqrtf(ve) + eps);
}

// ------------------------------------------------------------------ host -

static int ensure_cap(ProposalNet* n, int B) {
  emc_ctx* ctx = n->ctx;
  if (B <= n->cap) return EMC_OK;
  for (float** a : {&n->out, &n->g0, &n->g1, &n->gout, &n->loss, &n->labels6}) {
    cudaFree(*a);
    *a = nullptr;
  }
  cudaFree(n->idx);
  n->idx = nullptr;
  cudaFree(n->quarter);
  n->quarter = nullptr;
  for (auto& a : n->act) {
    cudaFree(a);
    a = nullptr;
  }
  n->cap = 0;
  size_t biggest = 0;
  for (int l = 0; l <= pn::NCONV; ++l) {
    const size_t sz = l == 0 ? (size_t)pn::D * pn::D
                             : (size_t)pn::CH * (pn::hin(l - 1) / 2) * (pn::hin(l - 1) / 2);
    EMC_CUDA(ctx, cudaMalloc(&n->act[l], sizeof(float) * sz * B));
    biggest = std::max(biggest, sz);
  }
  EMC_CUDA(ctx, cudaMalloc(&n->out, sizeof(float) * pn::OUT * B));
  EMC_CUDA(ctx, cudaMalloc(&n->gout, sizeof(float) * pn::OUT * B));
  EMC_CUDA(ctx, cudaMalloc(&n->g0, sizeof(float) * biggest * B));
  EMC_CUDA(ctx, cudaMalloc(&n->g1, sizeof(float) * biggest * B));
  EMC_CUDA(ctx, cudaMalloc(&n->loss, sizeof(float) * B));
  EMC_CUDA(ctx, cudaMalloc(&n->idx, sizeof(int) * B));
  EMC_CUDA(ctx, cudaMalloc(&n->quarter, sizeof(int) * B));
  EMC_CUDA(ctx, cudaMalloc(&n->labels6, sizeof(float) * 6 * B));
  n->cap = B;
  return EMC_OK;
}

// Forward pass of the B samples whose data rows are in n->idx (turned by
// n->quarter when `turned`).
static int forward(ProposalNet* n, int B, bool turned) {
  emc_ctx* ctx = n->ctx;
  int rc;
  const size_t e0 = (size_t)B * 4096;
  gather_rows_kernel<<<(unsigned)((e0 + 255) / 256), 256, 0, ctx->stream>>>(
      n->X, n->idx, turned ? n->quarter : nullptr, B, n->act[0]);
  if ((rc = after_launch(ctx, "gather_rows_kernel"))) return rc;
  for (int l = 0; l < pn::NCONV; ++l) {
    const int Hin = pn::hin(l), Ho = Hin / 2, ncol = B * Ho * Ho;
    conv_fwd_kernel<<<ceil_div(ncol, pn::TILE), 256, 0, ctx->stream>>>(
        n->act[l], n->params + n->off_w[l], n->params + n->off_b[l], n->act[l + 1], B, pn::cin(l),
        Hin);
    if ((rc = after_launch(ctx, "conv_fwd_kernel"))) return rc;
  }
  fc_fwd_kernel<<<B, 256, 0, ctx->stream>>>(n->act[pn::NCONV], n->params + n->off_fw,
                                            n->params + n->off_fb, n->out);
  return after_launch(ctx, "fc_fwd_kernel");
}

// Backward pass from n->gout (d loss / d output) into n->grads.
static int backward(ProposalNet* n, int B) {
  emc_ctx* ctx = n->ctx;
  int rc;
  float* gcur = n->g0;  // gradient of act[l + 1] (post-ReLU output of conv l)
  float* gnext = n->g1;
  fc_bwd_kernel<<<ceil_div(pn::FC_IN, 256), 256, 0, ctx->stream>>>(
      n->act[pn::NCONV], n->params + n->off_fw, n->gout, B, gcur, n->grads + n->off_fw,
      n->grads + n->off_fb);
  if ((rc = after_launch(ctx, "fc_bwd_kernel"))) return rc;
  for (int l = pn::NCONV - 1; l >= 0; --l) {
    const int Hin = pn::hin(l), Ho = Hin / 2, Cin = pn::cin(l), K = Cin * 9;
    const int ncol = B * Ho * Ho, S = ceil_div(ncol, pn::WG_COLS);
    const size_t need = (size_t)S * pn::CH * K;
    if (need > n->wpart_cap) {
      cudaFree(n->wpart);
      n->wpart = nullptr;
      n->wpart_cap = 0;
      EMC_CUDA(ctx, cudaMalloc(&n->wpart, sizeof(float) * need));
      n->wpart_cap = need;
    }
    conv_wgrad_kernel<<<dim3(ceil_div(K, pn::TILE), S), 256, 0, ctx->stream>>>(
        gcur, n->act[l + 1], n->act[l], n->wpart, B, Cin, Hin);
    if ((rc = after_launch(ctx, "conv_wgrad_kernel"))) return rc;
    sum_parts_kernel<<<ceil_div(pn::CH * K, 256), 256, 0, ctx->stream>>>(
        n->wpart, S, pn::CH * K, n->grads + n->off_w[l]);
    if ((rc = after_launch(ctx, "sum_parts_kernel"))) return rc;
    conv_bgrad_kernel<<<pn::CH, 256, 0, ctx->stream>>>(gcur, n->act[l + 1], B, Ho * Ho,
                                                        n->grads + n->off_b[l]);
    if ((rc = after_launch(ctx, "conv_bgrad_kernel"))) return rc;
    if (l > 0) {
      const int nin = B * Hin * Hin;
      conv_bwd_data_kernel<<<dim3(ceil_div(nin, pn::TILE), ceil_div(Cin, pn::TILE)), 256, 0,
                             ctx->stream>>>(gcur, n->act[l + 1], n->params + n->off_w[l], gnext,
                                            B, Cin, Hin);
      if ((rc = after_launch(ctx, "conv_bwd_data_kernel"))) return rc;
      std::swap(gcur, gnext);
    }
  }
  return EMC_OK;
}

// Loss of the batch in n->idx against labels (quaternions, data rows) and
// its gradient in n->grads; *h_loss = mean loss.
static int loss_and_grads(ProposalNet* n, int B, const float* d_quats, float* h_loss,
                          bool turned) {
  emc_ctx* ctx = n->ctx;
  int rc;
  if ((rc = forward(n, B, turned))) return rc;
  labels_kernel<<<ceil_div(B, 128), 128, 0, ctx->stream>>>(d_quats, n->idx,
                                                            turned ? n->quarter : nullptr, B,
                                                            n->labels6);
  if ((rc = after_launch(ctx, "labels_kernel"))) return rc;
  loss_kernel<<<ceil_div(B, 128), 128, 0, ctx->stream>>>(n->out, n->labels6, B, n->loss,
                                                          n->gout);
  if ((rc = after_launch(ctx, "loss_kernel"))) return rc;
  if ((rc = backward(n, B))) return rc;
  if (h_loss) {
    std::vector<float> l(B);
    EMC_CUDA(ctx, cudaMemcpyAsync(l.data(), n->loss, sizeof(float) * B, cudaMemcpyDeviceToHost,
                                  ctx->stream));
    EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    double s = 0.0;
    for (float v : l) s += v;
    *h_loss = (float)(s / B);
  }
  return EMC_OK;
}

// splitmix64 stream for weight initialisation and shuffles.
struct Mix64 {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

}  // namespace emc

using namespace emc;

struct emc_proposal : ProposalNet {};

extern "C" int emc_proposal_create(emc_ctx* ctx, unsigned long long seed, emc_proposal** out) {
  if (!ctx || !out) return EMC_ERR_INVALID;
  emc_proposal* n = new emc_proposal();
  n->ctx = ctx;
  size_t o = 0;
  for (int l = 0; l < pn::NCONV; ++l) {
    n->off_w[l] = o;
    o += (size_t)pn::CH * pn::cin(l) * 9;
    n->off_b[l] = o;
    o += pn::CH;
  }
  n->off_fw = o;
  o += (size_t)pn::OUT * pn::FC_IN;
  n->off_fb = o;
  o += pn::OUT;
  n->n_params = o;
  // He-uniform weights (bound sqrt(6 / fan_in)), zero biases
  std::vector<float> h(o, 0.0f);
  Mix64 rng{seed ^ 0x5851f42d4c957f2dULL};
  for (int l = 0; l < pn::NCONV; ++l) {
    const double bound = std::sqrt(6.0 / (pn::cin(l) * 9.0));
    for (size_t e = 0; e < (size_t)pn::CH * pn::cin(l) * 9; ++e)
      h[n->off_w[l] + e] = (float)((2.0 * rng.uniform() - 1.0) * bound);
  }
  const double fb = std::sqrt(3.0 / pn::FC_IN);
  for (size_t e = 0; e < (size_t)pn::OUT * pn::FC_IN; ++e)
    h[n->off_fw + e] = (float)((2.0 * rng.uniform() - 1.0) * fb);
  cudaError_t e = cudaMalloc(&n->params, sizeof(float) * o);
  if (e == cudaSuccess) e = cudaMalloc(&n->grads, sizeof(float) * o);
  if (e == cudaSuccess) e = cudaMalloc(&n->adam_m, sizeof(float) * o);
  if (e == cudaSuccess) e = cudaMalloc(&n->adam_v, sizeof(float) * o);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(n->params, h.data(), sizeof(float) * o, cudaMemcpyHostToDevice,
                        ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(n->adam_m, 0, sizeof(float) * o, ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(n->adam_v, 0, sizeof(float) * o, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    const int rc = cuda_fail(ctx, e, "proposal_create");
    emc_proposal_destroy(n);
    return rc;
  }
  *out = n;
  return EMC_OK;
}

extern "C" int emc_proposal_destroy(emc_proposal* n) {
  if (!n) return EMC_OK;
  if (n->ctx) cudaStreamSynchronize(n->ctx->stream);
  for (float* a : {n->params, n->grads, n->adam_m, n->adam_v, n->X, n->out, n->g0, n->g1,
                   n->gout, n->wpart, n->loss, n->labels6, n->stats})
    cudaFree(a);
  for (auto& a : n->act) cudaFree(a);
  cudaFree(n->idx);
  cudaFree(n->quarter);
  delete n;
  return EMC_OK;
}

extern "C" int emc_proposal_param_count(const emc_proposal* n) {
  return n ? (int)n->n_params : 0;
}

extern "C" int emc_proposal_params(emc_proposal* n, float* h_params, int get) {
  if (!n || !h_params) return EMC_ERR_INVALID;
  emc_ctx* ctx = n->ctx;
  const size_t bytes = sizeof(float) * n->n_params;
  if (get) {
    EMC_CUDA(ctx, cudaMemcpyAsync(h_params, n->params, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  } else {
    EMC_CUDA(ctx, cudaMemcpyAsync(n->params, h_params, bytes, cudaMemcpyHostToDevice, ctx->stream));
    EMC_CUDA(ctx, cudaMemsetAsync(n->adam_m, 0, bytes, ctx->stream));
    EMC_CUDA(ctx, cudaMemsetAsync(n->adam_v, 0, bytes, ctx->stream));
    n->adam_t = 0;
  }
  EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return EMC_OK;
}

extern "C" int emc_proposal_set_data(emc_proposal* n, const float* d_images, const int* d_mask,
                                     int side, int n_images, int fit_stats) {
  if (!n) return EMC_ERR_INVALID;
  emc_ctx* ctx = n->ctx;
  EMC_REQUIRE(ctx, d_images && d_mask && n_images > 0, "proposal_set_data: bad arguments");
  EMC_REQUIRE(ctx, fit_stats || n->have_stats,
              "proposal_set_data: no input statistics yet (fit them on the training data)");
  EMC_REQUIRE(ctx, side >= pn::D && side % pn::D == 0,
              "proposal_set_data: side %d is not a multiple of 64", side);
  if (n_images > n->n_data) {
    cudaFree(n->X);
    n->X = nullptr;
    n->n_data = 0;
    EMC_CUDA(ctx, cudaMalloc(&n->X, sizeof(float) * 4096 * (size_t)n_images));
  }
  n->n_data = n_images;
  proposal_inputs_kernel<<<n_images, 256, 0, ctx->stream>>>(d_images, d_mask, side, n_images,
                                                             n->X);
  int rc = after_launch(ctx, "proposal_inputs_kernel");
  if (rc) return rc;
  if (!n->stats) EMC_CUDA(ctx, cudaMalloc(&n->stats, sizeof(float) * 2 * 4096));
  if (fit_stats) {
    input_stats_kernel<<<16, 256, 0, ctx->stream>>>(n->X, n_images, n->stats);
    if ((rc = after_launch(ctx, "input_stats_kernel"))) return rc;
    n->have_stats = true;
  }
  const size_t e = (size_t)n_images * 4096;
  standardize_kernel<<<(unsigned)((e + 255) / 256), 256, 0, ctx->stream>>>(n->X, n_images,
                                                                          n->stats);
  return after_launch(ctx, "standardize_kernel");
}

extern "C" int emc_proposal_stats(emc_proposal* n, float* h_stats, int get) {
  if (!n || !h_stats) return EMC_ERR_INVALID;
  emc_ctx* ctx = n->ctx;
  if (!n->stats) EMC_CUDA(ctx, cudaMalloc(&n->stats, sizeof(float) * 2 * 4096));
  if (get) {
    EMC_REQUIRE(ctx, n->have_stats, "proposal_stats: none fitted");
    EMC_CUDA(ctx, cudaMemcpyAsync(h_stats, n->stats, sizeof(float) * 8192, cudaMemcpyDeviceToHost,
                                  ctx->stream));
  } else {
    EMC_CUDA(ctx, cudaMemcpyAsync(n->stats, h_stats, sizeof(float) * 8192, cudaMemcpyHostToDevice,
                                  ctx->stream));
    n->have_stats = true;
  }
  EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return EMC_OK;
}

extern "C" int emc_proposal_inputs(emc_proposal* n, int first, int count, float* h_out) {
  if (!n || !h_out) return EMC_ERR_INVALID;
  emc_ctx* ctx = n->ctx;
  EMC_REQUIRE(ctx, first >= 0 && count >= 0 && first + count <= n->n_data,
              "proposal_inputs: rows out of range");
  EMC_CUDA(ctx, cudaMemcpyAsync(h_out, n->X + (size_t)first * 4096, sizeof(float) * 4096 * count,
                                cudaMemcpyDeviceToHost, ctx->stream));
  EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return EMC_OK;
}

extern "C" int emc_proposal_loss_grad(emc_proposal* n, const int* h_rows, int B,
                                      const float* d_quats, float* h_loss, float* h_grads) {
  if (!n) return EMC_ERR_INVALID;
  emc_ctx* ctx = n->ctx;
  EMC_REQUIRE(ctx, h_rows && B > 0 && d_quats && n->X, "proposal_loss_grad: bad arguments");
  for (int j = 0; j < B; ++j)
    EMC_REQUIRE(ctx, h_rows[j] >= 0 && h_rows[j] < n->n_data, "proposal_loss_grad: bad row");
  int rc = ensure_cap(n, B);
  if (rc) return rc;
  EMC_CUDA(ctx, cudaMemcpyAsync(n->idx, h_rows, sizeof(int) * B, cudaMemcpyHostToDevice,
                                ctx->stream));
  if ((rc = loss_and_grads(n, B, d_quats, h_loss, false))) return rc;
  if (h_grads)
    EMC_CUDA(ctx, cudaMemcpyAsync(h_grads, n->grads, sizeof(float) * n->n_params,
                                  cudaMemcpyDeviceToHost, ctx->stream));
  EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return EMC_OK;
}

extern "C" int emc_proposal_train(emc_proposal* n, const float* d_quats, const int* h_rows,
                                  int n_rows, int epochs, int batch, float lr,
                                  unsigned long long seed, int augment, float* h_epoch_loss) {
  if (!n) return EMC_ERR_INVALID;
  emc_ctx* ctx = n->ctx;
  EMC_REQUIRE(ctx, d_quats && n->X && epochs >= 0 && batch > 0 && lr > 0.0f,
              "proposal_train: bad arguments");
  std::vector<int> rows;
  if (h_rows) {
    rows.assign(h_rows, h_rows + n_rows);
    for (int r : rows)
      EMC_REQUIRE(ctx, r >= 0 && r < n->n_data, "proposal_train: row %d out of range", r);
  } else {
    rows.resize(n->n_data);
    for (int j = 0; j < n->n_data; ++j) rows[j] = j;
  }
  EMC_REQUIRE(ctx, !rows.empty(), "proposal_train: no rows");
  int rc = ensure_cap(n, batch);
  if (rc) return rc;
  Mix64 rng{seed};
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  std::vector<int> stage(batch), quarter(batch);
  const long long total_steps = (long long)epochs * (long long)ceil_div((int)rows.size(), batch);
  long long step = 0;
  for (int ep = 0; ep < epochs; ++ep) {
    for (size_t j = rows.size(); j > 1; --j) {  // Fisher-Yates
      const size_t k = (size_t)(rng.next() % j);
      std::swap(rows[j - 1], rows[k]);
    }
    double sum = 0.0;
    size_t seen = 0;
    for (size_t s0 = 0; s0 < rows.size(); s0 += batch) {
      const int B = (int)std::min<size_t>(batch, rows.size() - s0);
      std::copy(rows.begin() + s0, rows.begin() + s0 + B, stage.begin());
      for (int j = 0; j < B; ++j) quarter[j] = augment ? (int)(rng.next() >> 62) : 0;
      EMC_CUDA(ctx, cudaMemcpyAsync(n->idx, stage.data(), sizeof(int) * B, cudaMemcpyHostToDevice,
                                    ctx->stream));
      EMC_CUDA(ctx, cudaMemcpyAsync(n->quarter, quarter.data(), sizeof(int) * B,
                                    cudaMemcpyHostToDevice, ctx->stream));
      // pageable sources are staged before the calls return; the next batch
      // overwrites them only after that
      float l = 0.0f;
      if ((rc = loss_and_grads(n, B, d_quats, h_epoch_loss ? &l : nullptr, true))) return rc;
      sum += (double)l * B;
      seen += B;
      ++n->adam_t;
      const double c1 = 1.0 - std::pow((double)b1, (double)n->adam_t);
      const double c2 = 1.0 - std::pow((double)b2, (double)n->adam_t);
      // cosine decay of the step size over this call, to 5 % at its end
      const double prog = (double)(step++) / (double)std::max<long long>(1, total_steps - 1);
      const double sched = 0.05 + 0.95 * 0.5 * (1.0 + std::cos(M_PI * prog));
      const float lr_t = (float)(lr * sched * std::sqrt(c2) / c1);
      adam_kernel<<<(unsigned)((n->n_params + 255) / 256), 256, 0, ctx->stream>>>(
          n->params, n->grads, n->adam_m, n->adam_v, n->n_params, lr_t, b1, b2, eps);
      if ((rc = after_launch(ctx, "adam_kernel"))) return rc;
    }
    if (h_epoch_loss) h_epoch_loss[ep] = (float)(sum / (double)seen);
  }
  EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return EMC_OK;
}

extern "C" int emc_proposal_predict(emc_proposal* n, float* d_quats_out) {
  if (!n) return EMC_ERR_INVALID;
  emc_ctx* ctx = n->ctx;
  EMC_REQUIRE(ctx, d_quats_out && n->X, "proposal_predict: bad arguments");
  const int B = 1024;
  int rc = ensure_cap(n, B);
  if (rc) return rc;
  std::vector<int> stage(B);
  for (int s0 = 0; s0 < n->n_data; s0 += B) {
    const int cnt = std::min(B, n->n_data - s0);
    for (int j = 0; j < cnt; ++j) stage[j] = s0 + j;
    EMC_CUDA(ctx, cudaMemcpyAsync(n->idx, stage.data(), sizeof(int) * cnt, cudaMemcpyHostToDevice,
                                  ctx->stream));
    if ((rc = forward(n, cnt, false))) return rc;
    predict_quats_kernel<<<ceil_div(cnt, 128), 128, 0, ctx->stream>>>(n->out, n->idx, cnt,
                                                                      d_quats_out);
    if ((rc = after_launch(ctx, "predict_quats_kernel"))) return rc;
    EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));  // `stage` is reused
  }
  return EMC_OK;
}
