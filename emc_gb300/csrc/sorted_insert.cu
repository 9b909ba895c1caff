// Deterministic insertion by sorted voxels (EMC_INSERT_SORTED).
//
// The reference inserts every (rotation, pixel) value with float atomics
// (emc_atomic.cu:72-73, insert_slices_kernel emc_atomic.cu:183-200), so the
// order of the additions into a voxel, and with it the rounding, changes from
// run to run.  Here the insertion is a segmented reduction in a fixed order.
// At bind time every pair of the bound geometry -- rotation r, compacted pixel
// q and, for trilinear splats, the corner k -- is keyed by the voxel it inserts
// into, with the same voxel arithmetic as the atomic insertion, and the pairs
// are sorted by that key with a stable LSD radix sort: each voxel's segment
// lists its pairs in ascending (q, r, k).  Each iteration the M-step epilogue
// stores the value of every pair, T_r x slice (0 where T_r <= 1e-10), in
// U [q][r] instead of adding it; one warp per piece of at most kPiece
// consecutive entries sums its values (lane-strided FP32, then a fixed
// butterfly), and one thread per voxel adds its pieces in order in FP64.  The
// sums depend on the geometry and the values only: reruns, re-binds and other
// processes give the same bits, without the fixed-point mode's global bound.
//
// Memory (128^3 model, 25,680 rotations, 12,780 pixels, nearest): U 1.3 GB
// and the sorted pair codes 1.3 GB stay resident; the sort takes 5.3 GB more
// while the plan is bound.  A pair code is q << (rb + cb) | r << cb | k in 32
// bits, which bounds the rotations x pixels (x 8 corners) a plan can sort.
#include <algorithm>
#include <cstring>
#include <vector>

#include "geometry.cuh"
#include "plan.cuh"

namespace emc {
namespace {

constexpr int kThreads = 256;
constexpr int kItems = 16;
constexpr int kTile = kThreads * kItems;  // entries per radix-sort tile
constexpr int kWarps = kThreads / 32;
constexpr int kWarpItems = kTile / kWarps;  // 512 consecutive entries per warp
constexpr int kDigitBits = 8;
constexpr int kDigits = 1 << kDigitBits;
static_assert(kDigits == kThreads, "one digit per thread in the radix kernels");
constexpr int kScanItems = 8;
constexpr int kScanBlock = kThreads * kScanItems;  // elements per scan block
constexpr int kPiece = 256;                        // entries per reduction piece

// Bits needed to hold v (0 for v == 0).
int bits_for(unsigned long long v) {
  int b = 0;
  while (b < 64 && (1ull << b) <= v) ++b;
  return b;
}

struct SortedInsert {
  const float* rot = nullptr;  // the rotations the map was built for
  uint32_t* ent = nullptr;     // [n] pair codes, sorted by voxel (sentinels last)
  uint32_t* piece_off = nullptr;  // [n3 + 1] first piece of each voxel
  uint2* piece = nullptr;      // [n_pieces] entry range [x, y) of each piece
  float2* part = nullptr;      // [n_pieces] (model, weight) sum of each piece
  long long n = 0, n_valid = 0, n_pieces = 0;
  int rb = 0, cb = 0;
  size_t bytes = 0;     // device bytes held (counted in the plan's workspace once built)
  bool counted = false;
  bool built = false;
  std::vector<float> h_geom;  // the rotations and pixel coordinates it was built from
};

SortedInsert* sstate(emc_plan* p) { return (SortedInsert*)p->sorted; }

void release(emc_plan* p, SortedInsert* s) {
  cudaFree(s->ent);
  cudaFree(s->piece_off);
  cudaFree(s->piece);
  cudaFree(s->part);
  s->ent = nullptr;
  s->piece_off = nullptr;
  s->piece = nullptr;
  s->part = nullptr;
  if (s->counted) p->bytes -= s->bytes;
  s->counted = false;
  s->bytes = 0;
  s->n = s->n_valid = s->n_pieces = 0;
}

template <typename T>
int dev_alloc(emc_ctx* ctx, T** ptr, size_t n, size_t* bytes) {
  const cudaError_t e = cudaMalloc((void**)ptr, sizeof(T) * std::max<size_t>(n, 1));
  if (e != cudaSuccess) {
    *ptr = nullptr;
    cudaGetLastError();
    return fail(ctx, EMC_ERR_NOMEM, "sorted insertion: %zu bytes: %s", sizeof(T) * n,
                cudaGetErrorString(e));
  }
  if (bytes) *bytes += sizeof(T) * std::max<size_t>(n, 1);
  return EMC_OK;
}

// Trilinear corner k of a fractional voxel position: the voxel and its weight,
// with the expression order of the atomic insertion's splat.
__device__ __forceinline__ bool tri_corner(int side, float cx, float cy, float cz, int k,
                                           uint32_t* vox, float* f) {
  const float fx0 = floorf(cx), fy0 = floorf(cy), fz0 = floorf(cz);
  const int xi = (int)fx0 + (k & 1), yi = (int)fy0 + ((k >> 1) & 1), zi = (int)fz0 + (k >> 2);
  const float tx = cx - fx0, ty = cy - fy0, tz = cz - fz0;
  *f = ((k & 1) ? tx : 1.0f - tx) * (((k >> 1) & 1) ? ty : 1.0f - ty) *
       ((k >> 2) ? tz : 1.0f - tz);
  if (xi < 0 || xi >= side || yi < 0 || yi >= side || zi < 0 || zi >= side) return false;
  *vox = ((uint32_t)zi * side + yi) * side + xi;
  return true;
}

// Keys (voxel, or the sentinel n3) and pair codes of every pair, in ascending
// code order: entry ((q R) + r) C + k.
__global__ void sv_keys_kernel(const float* __restrict__ rot, const float* __restrict__ cx,
                               const float* __restrict__ cy, const float* __restrict__ cz, int R,
                               int P, int side, int tri, int rb, int cb, uint32_t sentinel,
                               uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= R) return;
  const RotMat M = quat_to_matrix(rot + 4 * (size_t)r);
  const int C = tri ? 8 : 1;
  for (int q = blockIdx.y; q < P; q += gridDim.y) {
    const float x = cx[q], y = cy[q], z = cz[q];
    const size_t e = ((size_t)q * R + r) * C;
    const uint32_t code = ((uint32_t)q << (rb + cb)) | ((uint32_t)r << cb);
    if (!tri) {
      const int ix = voxel_round(voxel_coord(side, rotate_row(M, 0, x, y, z)));
      const int iy = voxel_round(voxel_coord(side, rotate_row(M, 1, x, y, z)));
      const int iz = voxel_round(voxel_coord(side, rotate_row(M, 2, x, y, z)));
      const bool in = ix >= 0 && ix < side && iy >= 0 && iy < side && iz >= 0 && iz < side;
      keys[e] = in ? ((uint32_t)iz * side + iy) * side + ix : sentinel;
      vals[e] = code;
    } else {
      const float fx = voxel_coord(side, rotate_row(M, 0, x, y, z));
      const float fy = voxel_coord(side, rotate_row(M, 1, x, y, z));
      const float fz = voxel_coord(side, rotate_row(M, 2, x, y, z));
      for (int k = 0; k < 8; ++k) {
        uint32_t v;
        float f;
        const bool ok = tri_corner(side, fx, fy, fz, k, &v, &f) && f > 0.0f;
        keys[e + k] = ok ? v : sentinel;
        vals[e + k] = code | (uint32_t)k;
      }
    }
  }
}

// ---- stable LSD radix sort of (key, value) pairs, 8 bits per pass --------
// Digit counts of each tile, stored digit-major: hist[d * n_tiles + tile].
__global__ void __launch_bounds__(kThreads) sv_hist_kernel(const uint32_t* __restrict__ keys,
                                                           long long n, int shift,
                                                           uint32_t* __restrict__ hist,
                                                           int n_tiles) {
  __shared__ uint32_t cnt[kDigits];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  const long long base = (long long)blockIdx.x * kTile;
  for (int j = 0; j < kItems; ++j) {
    const long long e = base + (long long)j * kThreads + threadIdx.x;
    if (e < n) atomicAdd(&cnt[(keys[e] >> shift) & (kDigits - 1)], 1u);
  }
  __syncthreads();
  hist[(size_t)threadIdx.x * n_tiles + blockIdx.x] = cnt[threadIdx.x];
}

// Exclusive scan of one block's kThreads values (one per thread); returns the
// thread's exclusive prefix and writes the block total to *total.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total) {
  __shared__ uint32_t wsum[kWarps];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) wsum[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < kWarps ? wsum[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += t;
    }
    if (lane < kWarps) wsum[lane] = w;  // inclusive over warps
  }
  __syncthreads();
  const uint32_t before = warp ? wsum[warp - 1] : 0u;
  *total = wsum[kWarps - 1];
  __syncthreads();  // wsum is reused by the next call
  return before + inc - v;
}

// Exclusive scan, in place, of x[0..n) (uint32, total < 2^32): block sums,
// one block over the sums, then each block with its offset.
__global__ void __launch_bounds__(kThreads) scan_sums_kernel(const uint32_t* __restrict__ x,
                                                             long long n,
                                                             uint32_t* __restrict__ sums) {
  const long long base = (long long)blockIdx.x * kScanBlock + (long long)threadIdx.x * kScanItems;
  uint32_t s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i)
    if (base + i < n) s += x[base + i];
  uint32_t total;
  block_exclusive_scan(s, &total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kThreads) scan_block_offsets_kernel(uint32_t* __restrict__ sums,
                                                                      int nb) {
  uint32_t carry = 0;
  for (int b0 = 0; b0 < nb; b0 += kThreads) {
    const int b = b0 + threadIdx.x;
    const uint32_t v = b < nb ? sums[b] : 0u;
    uint32_t total;
    const uint32_t ex = block_exclusive_scan(v, &total);
    if (b < nb) sums[b] = carry + ex;
    carry += total;
  }
}

__global__ void __launch_bounds__(kThreads) scan_apply_kernel(uint32_t* __restrict__ x,
                                                              long long n,
                                                              const uint32_t* __restrict__ sums) {
  const long long base = (long long)blockIdx.x * kScanBlock + (long long)threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  uint32_t s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    v[i] = base + i < n ? x[base + i] : 0u;
    s += v[i];
  }
  uint32_t total;
  uint32_t run = sums[blockIdx.x] + block_exclusive_scan(s, &total);
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    if (base + i < n) x[base + i] = run;
    run += v[i];
  }
}

// Stable scatter of one tile by the digit at `shift`.  Warp w takes the tile's
// entries [w 512, (w + 1) 512) in rounds of 32, so the tile order is (warp,
// round, lane); within a round, lanes with equal digits rank by lane.
__global__ void __launch_bounds__(kThreads) sv_scatter_kernel(
    const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in, long long n,
    int shift, const uint32_t* __restrict__ offs, int n_tiles, uint32_t* __restrict__ keys_out,
    uint32_t* __restrict__ vals_out) {
  __shared__ uint32_t wcnt[kWarps][kDigits];
  __shared__ uint32_t gbase[kDigits];
  for (int i = threadIdx.x; i < kWarps * kDigits; i += kThreads) (&wcnt[0][0])[i] = 0u;
  gbase[threadIdx.x] = offs[(size_t)threadIdx.x * n_tiles + blockIdx.x];
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  const long long base = (long long)blockIdx.x * kTile + (long long)w * kWarpItems;
  uint32_t key[kItems], val[kItems], loc[kItems];
#pragma unroll
  for (int j = 0; j < kItems; ++j) {
    const long long e = base + j * 32 + lane;
    const bool valid = e < n;
    key[j] = valid ? keys_in[e] : 0u;
    val[j] = valid ? vals_in[e] : 0u;
    const uint32_t d = (key[j] >> shift) & (kDigits - 1);
    const unsigned peers = __match_any_sync(0xffffffffu, valid ? d : (uint32_t)kDigits);
    const uint32_t cur = valid ? wcnt[w][d] : 0u;
    __syncwarp();
    if (valid && (peers & lt) == 0) wcnt[w][d] = cur + (uint32_t)__popc(peers);
    __syncwarp();
    loc[j] = cur + (uint32_t)__popc(peers & lt);
  }
  __syncthreads();
  {
    uint32_t run = 0;
    for (int v = 0; v < kWarps; ++v) {
      const uint32_t c = wcnt[v][threadIdx.x];
      wcnt[v][threadIdx.x] = run;
      run += c;
    }
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kItems; ++j) {
    const long long e = base + j * 32 + lane;
    if (e < n) {
      const uint32_t d = (key[j] >> shift) & (kDigits - 1);
      const uint32_t pos = gbase[d] + wcnt[w][d] + loc[j];
      keys_out[pos] = key[j];
      vals_out[pos] = val[j];
    }
  }
}

// seg[v] = first entry of voxel v in the sorted keys (v = 0..n3; seg[n3] is
// the first sentinel, i.e. the number of valid entries).
__global__ void sv_segments_kernel(const uint32_t* __restrict__ keys, long long n, uint32_t n3,
                                   uint32_t* __restrict__ seg) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const long long k = keys[i];
    const long long kp = i ? (long long)keys[i - 1] : -1;
    for (long long v = kp + 1; v <= k && v <= (long long)n3; ++v) seg[v] = (uint32_t)i;
    if (i == n - 1)
      for (long long v = k + 1; v <= (long long)n3; ++v) seg[v] = (uint32_t)n;
  }
}

__global__ void sv_piece_count_kernel(const uint32_t* __restrict__ seg, uint32_t n3,
                                      uint32_t* __restrict__ cnt) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v <= (long long)n3;
       v += stride)
    cnt[v] = v < (long long)n3 ? (seg[v + 1] - seg[v] + kPiece - 1) / kPiece : 0u;
}

__global__ void sv_piece_fill_kernel(const uint32_t* __restrict__ seg,
                                     const uint32_t* __restrict__ off, uint32_t n3,
                                     uint2* __restrict__ piece) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < (long long)n3;
       v += stride) {
    const uint32_t s0 = seg[v], s1 = seg[v + 1];
    uint32_t o = off[v];
    for (unsigned long long s = s0; s < s1; s += kPiece, ++o)
      piece[o] = make_uint2((uint32_t)s, (uint32_t)min(s + kPiece, (unsigned long long)s1));
  }
}

// ---- per iteration -------------------------------------------------------
// One warp per piece: the (model, weight) sum of its entries.  A piece holds
// at most kPiece = 8 x 32 entries, so every lane issues its (up to) eight code
// loads, then its eight value gathers, before it adds anything: the gathers
// from U are independent and in flight together.  Lane l adds the piece's
// entries l, l + 32, ... in that order, then the butterfly combines the lanes.
__global__ void __launch_bounds__(256, 4) sv_reduce_kernel(
    const uint32_t* __restrict__ ent, const uint2* __restrict__ piece, long long n_pieces,
    const float* __restrict__ U, int ldu, const float* __restrict__ T, int rb, int cb,
    const float* __restrict__ rot, const float* __restrict__ cx, const float* __restrict__ cy,
    const float* __restrict__ cz, int side, float2* __restrict__ part) {
  constexpr int kPer = kPiece / 32;
  const int lane = threadIdx.x & 31;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  const uint32_t rmask = (1u << rb) - 1u;
  for (long long pc = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; pc < n_pieces;
       pc += nw) {
    const uint2 rg = piece[pc];
    uint32_t code[kPer];
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
      const uint32_t e = rg.x + lane + 32 * i;
      code[i] = e < rg.y ? __ldg(ent + e) : 0u;
    }
    float val[kPer], wt[kPer];
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
      const bool on = rg.x + lane + 32 * i < rg.y;
      const uint32_t r = (code[i] >> cb) & rmask, q = code[i] >> (rb + cb);
      const float t = on ? __ldg(T + r) : 0.0f;
      val[i] = on ? __ldg(U + (size_t)q * ldu + r) : 0.0f;  // 0 where T_r <= 1e-10
      wt[i] = t > 1e-10f ? t : 0.0f;
    }
    float m = 0.0f, w = 0.0f;
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
      if (rg.x + lane + 32 * i >= rg.y) break;
      float v = val[i], x = wt[i];
      if (cb) {
        const uint32_t r = (code[i] >> cb) & rmask, q = code[i] >> (rb + cb);
        const RotMat M = quat_to_matrix(rot + 4 * (size_t)r);
        const float px = __ldg(cx + q), py = __ldg(cy + q), pz = __ldg(cz + q);
        uint32_t vox;
        float f;
        tri_corner(side, voxel_coord(side, rotate_row(M, 0, px, py, pz)),
                   voxel_coord(side, rotate_row(M, 1, px, py, pz)),
                   voxel_coord(side, rotate_row(M, 2, px, py, pz)), (int)(code[i] & 7u), &vox,
                   &f);
        v = v * f;
        x = x * f;
      }
      m = __fadd_rn(m, v);
      w = __fadd_rn(w, x);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      m = __fadd_rn(m, __shfl_xor_sync(0xffffffffu, m, o));
      w = __fadd_rn(w, __shfl_xor_sync(0xffffffffu, w, o));
    }
    if (lane == 0) part[pc] = make_float2(m, w);
  }
}

// One thread per voxel: its pieces in order, in FP64.
__global__ void sv_combine_kernel(const uint32_t* __restrict__ off,
                                  const float2* __restrict__ part, long long n3,
                                  float2* __restrict__ acc2) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n3; v += stride) {
    double m = 0.0, w = 0.0;
    for (uint32_t pc = off[v]; pc < off[v + 1]; ++pc) {
      const float2 a = part[pc];
      m += (double)a.x;
      w += (double)a.y;
    }
    acc2[v] = make_float2((float)m, (float)w);
  }
}

// In-place exclusive scan of x[0..n) on the context stream; sums: scratch of
// ceil(n / kScanBlock) entries.
int scan_exclusive(emc_ctx* ctx, uint32_t* x, long long n, uint32_t* sums) {
  const int nb = ceil_div(n, kScanBlock);
  int rc;
  scan_sums_kernel<<<nb, kThreads, 0, ctx->stream>>>(x, n, sums);
  if ((rc = after_launch(ctx, "scan_sums_kernel"))) return rc;
  scan_block_offsets_kernel<<<1, kThreads, 0, ctx->stream>>>(sums, nb);
  if ((rc = after_launch(ctx, "scan_block_offsets_kernel"))) return rc;
  scan_apply_kernel<<<nb, kThreads, 0, ctx->stream>>>(x, n, sums);
  return after_launch(ctx, "scan_apply_kernel");
}

int build(emc_plan* p, SortedInsert* s) {
  emc_ctx* ctx = p->ctx;
  const int R = p->d.n_rot, P = p->P_eff, side = p->d.side;
  const bool tri = p->d.interp == EMC_INTERP_TRILINEAR;
  const int C = tri ? 8 : 1;
  const int rb = std::max(1, bits_for((unsigned long long)(R - 1)));
  const int pb = std::max(1, bits_for((unsigned long long)(P - 1)));
  const int cb = tri ? 3 : 0;
  const long long n = (long long)R * P * C;
  // entry indices stay 32-bit with room for a piece past the last entry
  if (rb + pb + cb > 32 || n >= (1LL << 32) - 1024)
    return fail(ctx, EMC_ERR_UNSUPPORTED,
                "sorted insertion: %d rotations x %d pixels%s do not fit 32-bit pair codes", R, P,
                tri ? " x 8 corners" : "");
  const uint32_t n3 = (uint32_t)side * side * side;
  const int key_bits = bits_for(n3);  // keys 0..n3 (n3: out of the model)
  const int passes = (key_bits + kDigitBits - 1) / kDigitBits;
  release(p, s);
  s->rb = rb;
  s->cb = cb;
  s->n = n;
  if (!p->ins_u) {
    int rc = plan_alloc(p, (void**)&p->ins_u, sizeof(float) * (size_t)P * p->Rp);
    if (rc) return rc;
    p->ins_ldu = p->Rp;
  }
  // transient buffers of the sort
  const int n_tiles = ceil_div(n, kTile);
  const long long n_hist = (long long)kDigits * n_tiles;
  const long long n_scan = std::max<long long>(n_hist, (long long)n3 + 1);
  uint32_t *k0 = nullptr, *k1 = nullptr, *v0 = nullptr, *v1 = nullptr, *hist = nullptr,
           *sums = nullptr, *seg = nullptr;
  auto cleanup = [&]() {
    cudaFree(k0);
    cudaFree(k1);
    cudaFree(v0);
    cudaFree(v1);
    cudaFree(hist);
    cudaFree(sums);
    cudaFree(seg);
  };
  int rc = dev_alloc(ctx, &k0, n, nullptr);
  if (!rc) rc = dev_alloc(ctx, &k1, n, nullptr);
  if (!rc) rc = dev_alloc(ctx, &v0, n, nullptr);
  if (!rc) rc = dev_alloc(ctx, &v1, n, nullptr);
  if (!rc) rc = dev_alloc(ctx, &hist, n_scan, nullptr);
  if (!rc) rc = dev_alloc(ctx, &sums, ceil_div(n_scan, kScanBlock), nullptr);
  if (!rc) rc = dev_alloc(ctx, &seg, (size_t)n3 + 1, nullptr);
  if (!rc) {
    dim3 grid(ceil_div(R, 128), std::min(P, 65535));
    sv_keys_kernel<<<grid, 128, 0, ctx->stream>>>(p->rot, p->cx, p->cy, p->cz, R, P, side,
                                                  tri ? 1 : 0, rb, cb, n3, k0, v0);
    rc = after_launch(ctx, "sv_keys_kernel");
  }
  for (int pass = 0; !rc && pass < passes; ++pass) {
    const int shift = pass * kDigitBits;
    sv_hist_kernel<<<n_tiles, kThreads, 0, ctx->stream>>>(k0, n, shift, hist, n_tiles);
    rc = after_launch(ctx, "sv_hist_kernel");
    if (!rc) rc = scan_exclusive(ctx, hist, n_hist, sums);
    if (!rc) {
      sv_scatter_kernel<<<n_tiles, kThreads, 0, ctx->stream>>>(k0, v0, n, shift, hist, n_tiles,
                                                               k1, v1);
      rc = after_launch(ctx, "sv_scatter_kernel");
    }
    std::swap(k0, k1);
    std::swap(v0, v1);
  }
  const int nb = ctx->sm_count * 8;
  if (!rc) {
    sv_segments_kernel<<<nb, 256, 0, ctx->stream>>>(k0, n, n3, seg);
    rc = after_launch(ctx, "sv_segments_kernel");
  }
  uint32_t* cnt = hist;  // reused: n3 + 1 piece counts, scanned to offsets
  if (!rc) {
    sv_piece_count_kernel<<<nb, 256, 0, ctx->stream>>>(seg, n3, cnt);
    rc = after_launch(ctx, "sv_piece_count_kernel");
  }
  if (!rc) rc = scan_exclusive(ctx, cnt, (long long)n3 + 1, sums);
  uint32_t h_last[2] = {0, 0};
  if (!rc) {
    const cudaError_t e1 = cudaMemcpyAsync(&h_last[0], cnt + n3, sizeof(uint32_t),
                                           cudaMemcpyDeviceToHost, ctx->stream);
    const cudaError_t e2 = cudaMemcpyAsync(&h_last[1], seg + n3, sizeof(uint32_t),
                                           cudaMemcpyDeviceToHost, ctx->stream);
    const cudaError_t e3 = cudaStreamSynchronize(ctx->stream);
    if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess)
      rc = cuda_fail(ctx, e1 != cudaSuccess ? e1 : (e2 != cudaSuccess ? e2 : e3),
                     "sorted insertion: piece count");
  }
  if (!rc) {
    s->n_pieces = h_last[0];
    s->n_valid = h_last[1];
    rc = dev_alloc(ctx, &s->piece_off, (size_t)n3 + 1, &s->bytes);
  }
  if (!rc) rc = dev_alloc(ctx, &s->piece, (size_t)s->n_pieces, &s->bytes);
  if (!rc) rc = dev_alloc(ctx, &s->part, (size_t)s->n_pieces, &s->bytes);
  if (!rc) {
    const cudaError_t e = cudaMemcpyAsync(s->piece_off, cnt, sizeof(uint32_t) * ((size_t)n3 + 1),
                                          cudaMemcpyDeviceToDevice, ctx->stream);
    if (e != cudaSuccess) rc = cuda_fail(ctx, e, "sorted insertion: offsets");
  }
  if (!rc) {
    sv_piece_fill_kernel<<<nb, 256, 0, ctx->stream>>>(seg, s->piece_off, n3, s->piece);
    rc = after_launch(ctx, "sv_piece_fill_kernel");
  }
  if (!rc) {
    const cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) rc = cuda_fail(ctx, e, "sorted insertion: build");
  }
  if (!rc) {
    s->ent = v0;  // the sorted codes stay; every other sort buffer goes
    v0 = nullptr;
    s->bytes += sizeof(uint32_t) * (size_t)n;
    p->bytes += s->bytes;
    s->counted = true;
    s->rot = p->rot;
    s->built = true;
  }
  cleanup();
  if (rc) release(p, s);
  return rc;
}

}  // namespace

int sorted_ensure(emc_plan* p) {
  if (p->d.insert_mode != EMC_INSERT_SORTED || !p->bound) return EMC_OK;
  emc_ctx* ctx = p->ctx;
  SortedInsert* s = sstate(p);
  if (!s) {
    s = new SortedInsert();
    p->sorted = s;
  }
  // The map depends on the rotations (in the plan's order) and the compacted
  // pixel coordinates only: a re-bind with the same geometry keeps it.
  const size_t nr = 4 * (size_t)p->d.n_rot, np = (size_t)p->P_eff;
  std::vector<float> g(nr + 3 * np);
  EMC_CUDA(ctx, cudaMemcpyAsync(g.data(), p->rot, sizeof(float) * nr, cudaMemcpyDeviceToHost,
                                ctx->stream));
  EMC_CUDA(ctx, cudaMemcpyAsync(g.data() + nr, p->cx, sizeof(float) * np, cudaMemcpyDeviceToHost,
                                ctx->stream));
  EMC_CUDA(ctx, cudaMemcpyAsync(g.data() + nr + np, p->cy, sizeof(float) * np,
                                cudaMemcpyDeviceToHost, ctx->stream));
  EMC_CUDA(ctx, cudaMemcpyAsync(g.data() + nr + 2 * np, p->cz, sizeof(float) * np,
                                cudaMemcpyDeviceToHost, ctx->stream));
  EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (s->built && s->rot == p->rot && g.size() == s->h_geom.size() &&
      std::memcmp(g.data(), s->h_geom.data(), sizeof(float) * g.size()) == 0)
    return EMC_OK;
  s->built = false;
  const int rc = build(p, s);
  if (!rc) s->h_geom.swap(g);
  return rc;
}

int sorted_reduce(emc_plan* p) {
  emc_ctx* ctx = p->ctx;
  SortedInsert* s = sstate(p);
  if (!s || !s->built || s->rot != p->rot || !p->ins_u)
    return fail(ctx, EMC_ERR_INTERNAL, "sorted insertion: the voxel map is not built for the "
                                       "bound rotations");
  const long long n3 = (long long)p->d.side * p->d.side * p->d.side;
  int rc;
  if (s->n_pieces > 0) {
    const int nb = ctx->sm_count * 8;
    sv_reduce_kernel<<<nb, 256, 0, ctx->stream>>>(s->ent, s->piece, s->n_pieces, p->ins_u,
                                                  p->ins_ldu, p->T, s->rb, s->cb, p->rot, p->cx,
                                                  p->cy, p->cz, p->d.side, s->part);
    if ((rc = after_launch(ctx, "sv_reduce_kernel"))) return rc;
  }
  const int nb = (int)std::min<long long>(ceil_div(n3, 256), (long long)ctx->sm_count * 8);
  sv_combine_kernel<<<nb, 256, 0, ctx->stream>>>(s->piece_off, s->part, n3, p->acc2);
  return after_launch(ctx, "sv_combine_kernel");
}

void sorted_free(emc_plan* p) {
  if (SortedInsert* s = sstate(p)) {
    release(p, s);
    delete s;
  }
  p->sorted = nullptr;
}

}  // namespace emc
