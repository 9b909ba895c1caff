// Tensor-core (tcgen05 + TMA) E-step and M-step of the fused iteration.
//
// E-step.  For a tile of 128 patterns (M, one TMEM lane each) x 128
// rotations (N) the reference's "poisson" likelihood with per-pair scaling
// (emc_cuda.cu:196-216, 438-454) is expanded into four contractions over the
// compacted pixels, accumulated in TMEM (FP32, 4 x 128 columns = all 512):
//   num = sum k^2 [s > 1e-10]             (K^2 hi + lo)  x  M'         exact
//   den = sum k s [s > 1e-10]             K              x  (M' S) hi
//   B   = sum k s/(s+c) [s > 0]           K              x  (G hi + lo)
//   C   = sum k^2 /(s+c) [s > 0]          (K^2 hi + lo)  x  (H hi + lo)
// so that with 1/phi = den/num:  S_ri = A_r - 2 B/phi + C/phi^2  and
// L_ri = log w_r - S_ri / (2 count_r sigma^2).  Counts are integers <= 2048,
// exact in FP16; K^2 * 2^-7 is split exactly into two FP16 terms; the
// rotation-side factors are split hi + lo (the lo x lo products are dropped,
// relative size 2^-22).  The epilogue (4 warps, one pattern row per thread)
// forms L and phi, stores them coalesced along patterns, and keeps a running
// (max, sum exp) per pattern over the tile's rotations: the per-tile LSE
// partials that the FP64 normaliser combines.
//
// M-step.  U = Q K^T over the patterns for a tile of 128 rotations x 256
// pixels, Q = P / phi split hi + lo in FP16 with a per-rotation power-of-two
// scale, K the exact FP16 counts; the epilogue inserts T_r * (U / T_r) at
// the rotated pixel (nearest or trilinear) with weight T_r -- the slice never
// reaches HBM (emc_atomic.cu:88-132, 183-200).
//
// Pipeline: warp 0 issues TMA loads into a ring of shared-memory stages
// (mbarrier full/empty handshake), warp 1 owns TMEM and issues tcgen05.mma
// from one lane, warps 2-5 run the epilogue.  Every wait is bounded and
// reports through a device status word (EMC_ERR_TIMEOUT on the host).
#include <cuda.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

#include "geometry.cuh"
#include "plan.cuh"
#include "ptx.cuh"

namespace emc {

// ------------------------------------------------------- tensor maps -----
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  }
  return fn;
}

// Row-major FP16 matrix [rows][cols] (cols contiguous), tiles of
// box_rows x box_cols, 64B or 128B swizzle (box_cols * 2 == swizzle span).
static int make_map(emc_ctx* ctx, CUtensorMap* map, const void* base, uint64_t rows,
                    uint64_t cols, uint32_t box_rows, uint32_t box_cols) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return fail(ctx, EMC_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  if (((uintptr_t)base & 15) || ((cols * 2) & 15))
    return fail(ctx, EMC_ERR_INTERNAL, "tensor map: misaligned base or pitch");
  cuuint64_t dims[2] = {cols, rows};
  cuuint64_t strides[1] = {cols * 2};
  cuuint32_t box[2] = {box_cols, box_rows};
  cuuint32_t estr[2] = {1, 1};
  const CUtensorMapSwizzle sw =
      box_cols * 2 == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B;
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void*>(base), dims, strides,
                  box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(ctx, EMC_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return EMC_OK;
}

// ---------------------------------------------------- pattern operands ---

// Counts -> FP16 operands, rows of Kp (patterns padded to Np with zeros):
// Kh = fp16(k) (k itself up to 2048; larger counts rounded to 11 significant
// bits), K2h + K2l = Kh^2 * k2_scale exactly (Kh^2 has at most 22 significant
// bits, and k2_scale keeps the largest below 2^15 and every value a multiple
// of 2^-24) (K2h == nullptr: Kh only).
__global__ void tc_pattern_ops_kernel(const float* __restrict__ images, const int* __restrict__ pix,
                                      int n2, int N, int Kp, __half* __restrict__ Kh,
                                      __half* __restrict__ K2h, __half* __restrict__ K2l,
                                      const int* __restrict__ perm, float k2_scale) {
  // one block per (pattern row, 256 pixels), pixel blocks the fast index
  const int nqb = (Kp + 255) / 256;
  const int i = (int)(blockIdx.x / nqb);
  const int q = (int)(blockIdx.x % nqb) * 256 + threadIdx.x;
  if (q >= Kp) return;
  float k = 0.0f;
  if (i < N) {
    const int p = pix[q];
    if (p >= 0) k = __ldg(images + (size_t)(perm ? perm[i] : i) * n2 + p);
  }
  const __half kh = __float2half_rn(k);
  const float kr = __half2float(kh);
  const float k2 = kr * kr * k2_scale;  // exact in FP32: 22 significant bits
  const __half hi = __float2half_rn(k2);
  const __half lo = __float2half_rn(k2 - __half2float(hi));
  const size_t o = (size_t)i * Kp + q;
  Kh[o] = kh;
  if (K2h) {
    K2h[o] = hi;
    K2l[o] = lo;
  }
}

// flags[pt][kb] = any K2l != 0 in rows pt*128..+127, cols kb*32..+31.
__global__ void tc_k2lo_flags_kernel(const __half* __restrict__ K2l, int Kp,
                                     unsigned char* __restrict__ flags, int nkb) {
  const int pt = blockIdx.y, kb = blockIdx.x;
  int any = 0;
  for (int e = threadIdx.x; e < 128 * 32; e += blockDim.x) {
    const int r = pt * 128 + e / 32, c = kb * 32 + e % 32;
    if (__half2float(K2l[(size_t)r * Kp + c]) != 0.0f) any = 1;
  }
  any = __syncthreads_or(any);
  if (threadIdx.x == 0) flags[(size_t)pt * nkb + kb] = (unsigned char)any;
}

// The sum of one 32-pixel block of an FP16 count row (64 bytes, 16-byte aligned).
__device__ __forceinline__ float count_block_sum(const __half* k) {
  const uint4* v = reinterpret_cast<const uint4*>(k);
  float s = 0.0f;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const uint4 u = v[j];
    const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
    for (int h = 0; h < 4; ++h) {
      const float2 f = __half22float2(*reinterpret_cast<const __half2*>(&w[h]));
      s += f.x + f.y;
    }
  }
  return s;
}

// One warp per pattern row n: the last 32-pixel block b whose suffix (blocks
// b ..) still holds more than eps of the row's counts; glo_kb[n / 128] (zeroed
// before) becomes the largest b + 1 over the tile's rows, and glo_kb[n_pt]
// the largest over all tiles (the expand writes G lo below it).  Lane l takes a
// contiguous run of blocks: run sums, a warp prefix scan, then a second walk
// over its run.  Integer counts below 2^24 in total sum exactly in FP32.
__global__ void __launch_bounds__(256) tc_glo_extent_kernel(const __half* __restrict__ Kh, int Kp,
                                                            int nkb, int N, float eps,
                                                            int* __restrict__ glo_kb) {
  const int n = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (n >= N) return;  // whole warps
  const __half* k = Kh + (size_t)n * Kp;
  const int per = (nkb + 31) / 32;
  const int b0 = min(lane * per, nkb), b1 = min(b0 + per, nkb);
  float c = 0.0f;
  for (int b = b0; b < b1; ++b) c += count_block_sum(k + 32 * (size_t)b);
  float inc = c;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const float t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  const float total = __shfl_sync(0xffffffffu, inc, 31);
  const float lim = eps * total;
  float pre = inc - c;  // the counts of the blocks before b0
  int last = -1;
  for (int b = b0; b < b1; ++b) {
    if (total - pre > lim) last = b;  // the suffix from b
    pre += count_block_sum(k + 32 * (size_t)b);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) last = max(last, __shfl_xor_sync(0xffffffffu, last, o));
  if (lane == 0 && last >= 0) {
    atomicMax(glo_kb + n / 128, last + 1);
    atomicMax(glo_kb + (N + 127) / 128, last + 1);
  }
}

// [rows][cols] -> [cols][rows], FP16: 64 x 64 tiles, moved with 4-byte
// (half2) loads and stores where two neighbouring elements are in range.
__global__ void transpose_h_kernel(const __half* __restrict__ in, int rows, int cols,
                                   __half* __restrict__ out) {
  __shared__ __half t[64][66];
  const int c0 = blockIdx.x * 64, r0 = blockIdx.y * 64;
  const int x2 = 2 * threadIdx.x;
  for (int y = threadIdx.y; y < 64; y += blockDim.y) {
    const int r = r0 + y, c = c0 + x2;
    __half a = __float2half_rn(0.f), b = a;
    if (r < rows) {
      if (c + 1 < cols && (cols & 1) == 0) {
        const __half2 v = *reinterpret_cast<const __half2*>(in + (size_t)r * cols + c);
        a = __low2half(v);
        b = __high2half(v);
      } else {
        if (c < cols) a = in[(size_t)r * cols + c];
        if (c + 1 < cols) b = in[(size_t)r * cols + c + 1];
      }
    }
    t[y][x2] = a;
    t[y][x2 + 1] = b;
  }
  __syncthreads();
  for (int y = threadIdx.y; y < 64; y += blockDim.y) {
    const int c = c0 + y, r = r0 + x2;
    if (c >= cols) continue;
    if (r + 1 < rows && (rows & 1) == 0) {
      *reinterpret_cast<__half2*>(out + (size_t)c * rows + r) = __halves2half2(t[x2][y], t[x2 + 1][y]);
    } else {
      if (r < rows) out[(size_t)c * rows + r] = t[x2][y];
      if (r + 1 < rows) out[(size_t)c * rows + r + 1] = t[x2 + 1][y];
    }
  }
}

// ------------------------------------------------------------ E-step -----
// One CTA owns 128 patterns x 128 rotations and all four contractions:
//   B = K . G^T,  den = K . (M'S)^T,  C = K^2 . H^T,  num = K^2 . M'^T.
// Operands that multiply the same pattern-side tile are stored next to each
// other in shared memory ([G | M'S] and [H | M']), so each pair is one
// 128 x 256 MMA: the pattern-side tile is read once per pair, which lowers
// the shared-memory operand traffic per FLOP that bounds 128 x 128 MMAs.
// TMEM columns: B 0-127, den 128-255, C 256-383, num 384-511.
namespace es {
constexpr int BM = 128;        // patterns per tile (TMEM lanes)
constexpr int BN = 128;        // rotations per tile
constexpr int BK = 32;         // pixels per stage (64 B rows, 64B swizzle)
constexpr int STAGES = 3;
constexpr int TILE_BYTES = 128 * BK * 2;  // 8 KB, both operand sides
// stage slots: pattern side, then the two N=256 pairs, then the lo terms
enum Slot { sK = 0, sK2h, sK2l, sGh, sMS, sHh, sMp, sGl, sHl, kSlots };
constexpr int STAGE_BYTES = kSlots * TILE_BYTES;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 8192 + 1024;  // barriers, row data, parts
constexpr int EPI_WARPS = 16;  // four per TMEM lane quarter, 32 columns each
constexpr int EPI_PARTS = EPI_WARPS / 4;
constexpr int THREADS = 64 + 32 * EPI_WARPS;
}  // namespace es

// Tile of CTA b in a grouped raster over n_pt pattern tiles x n_rt rotation
// tiles.  raster > 0: groups of `raster` rotation tiles, each group visiting
// the pattern tiles in turn (the group's rotation panels are read by
// consecutive CTAs); raster < 0: groups of -raster pattern tiles visiting the
// rotation tiles in turn.
__device__ __forceinline__ void raster_tile(int b, int raster, int n_pt, int n_rt, int& pt,
                                            int& rt) {
  if (raster > 0) {
    const int per_group = raster * n_pt;
    const int g = b / per_group, within = b % per_group;
    const int rt0 = g * raster;
    const int gsz = min(raster, n_rt - rt0);
    rt = rt0 + within % gsz;
    pt = within / gsz;
  } else {
    const int G = -raster;
    const int per_group = G * n_rt;
    const int g = b / per_group, within = b % per_group;
    const int pt0 = g * G;
    const int gsz = min(G, n_pt - pt0);
    pt = pt0 + within % gsz;
    rt = within / gsz;
  }
}

struct TcEstepArgs {
  int N, R, Kp, n_pt, n_rt, nkb;
  int raster;                     // tile order (raster_tile)
  int tile0;                      // CTA b runs tile tile0 + b of the order
  int gh_lo;                      // lo terms: bit 0 G, bit 1 H (3: both, 0: hi only)
  const int2* tiles;              // pruned iteration: (pattern tile, rotation tile) per CTA
  const unsigned char* k2lo_any;  // [n_pt][nkb]
  const int* glo_kb;              // [n_pt] G lo runs on k-blocks below glo_kb[pt]
  const float* rot_cnt;
  const float* rot_A;
  const float* rotw;
  const float* cnorm;   // c_i (phi is stored as c_i num/den)
  float k2_inv;         // 1 / k2_scale of the K^2 operand
  const float* sigma;   // [1] annealing width (device memory)
  int known_intensity;
  float* L;
  float* PHI;
  float2* part;
  int* bad;
  int* status;
  uint32_t spin;  // polls per pipeline wait (ptx::kSpinLimit unless a debug option lowers it)
};

// Epilogue of the likelihood kernels (warps 2 .. 2 + EPI_WARPS - 1): EPI_PARTS
// warps per TMEM lane quarter, each on a part of the 128 columns, so that
// the expf / divide latency of one hides behind another.  Reads B, den, C and
// num of this CTA's 128 patterns x 128 rotations from TMEM, writes L and
// phi and the tile's (max, sum exp) per pattern.
__device__ __forceinline__ void estep_epilogue(const TcEstepArgs& a, uint32_t tmem, uint64_t* accum,
                                               const float* s_A, const float* s_scale,
                                               const float* s_lw, float2* s_half, int warp,
                                               int lane, int n0, int r0, int rt) {
  using namespace es;
  // EPI_PARTS warps per TMEM lane quarter, each on a part of the 128
  // columns, so that the expf / divide latency of one hides behind another
  const int quarter = warp & 3;  // TMEM lanes this warp may access
  const int half = (warp - 2) >> 2;  // column part
  const int row = quarter * 32 + lane;
  const int n = n0 + row;
  const bool nok = n < a.N;
  const float ci = nok ? a.cnorm[n] : 1.0f;
  float m = -INFINITY, ssum = 0.0f;
  int nbad = 0;
  if (ptx::mbar_wait_sleep(accum, 0, a.status, 2, 256, a.spin)) {
    ptx::tc_fence_after();
    const uint32_t lane_addr = tmem + ((uint32_t)(quarter * 32) << 16);
    for (int c0 = half * (BN / EPI_PARTS); c0 < (half + 1) * (BN / EPI_PARTS); c0 += 16) {
      float vn[16], vd[16], vb[16], vc[16];
      ptx::tmem_ld16(lane_addr + 0 + c0, vb);
      ptx::tmem_ld16(lane_addr + 128 + c0, vd);
      ptx::tmem_ld16(lane_addr + 256 + c0, vc);
      ptx::tmem_ld16(lane_addr + 384 + c0, vn);
      ptx::tmem_wait_ld();
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const int cl = c0 + j;
        const int r = r0 + cl;
        const float num = vn[j] * a.k2_inv, den = vd[j] * 256.0f;
        const float B = vb[j], Cc = vc[j] * a.k2_inv;
        const float sc = s_scale[cl];
        bool ok = nok && r < a.R && sc > 0.0f;
        float iphi = 1.0f, phi = 1.0f;
        if (!a.known_intensity) {
          ok = ok && num > 0.0f && den > 0.0f;
          iphi = den / num;
          phi = ci * num / den;
        }
        const float Sig = s_A[cl] - 2.0f * B * iphi + Cc * iphi * iphi;
        const float L = ok ? s_lw[cl] - Sig * sc : -INFINITY;
        if (nok && r < a.R) {
          if (!ok) nbad++;
          a.L[(size_t)r * a.N + n] = L;
          a.PHI[(size_t)r * a.N + n] = ok ? phi : 1.0f;
        }
        if (L > m) {
          ssum = ssum * expf(m - L) + 1.0f;
          m = L;
        } else if (L > -INFINITY) {
          ssum += expf(L - m);
        }
      }
    }
  }
  // combine the parts' (max, sum exp) of each row
  if (half > 0) s_half[(half - 1) * BM + row] = make_float2(m, ssum);
  asm volatile("bar.sync 1, %0;" ::"n"(EPI_WARPS * 32) : "memory");  // epilogue warps only
  if (half == 0) {
    float M = m;
    for (int q = 1; q < EPI_PARTS; ++q) M = fmaxf(M, s_half[(q - 1) * BM + row].x);
    float S = 0.0f;
    if (M > -INFINITY) {
      S = ssum * expf(m - M);
      for (int q = 1; q < EPI_PARTS; ++q) {
        const float2 o = s_half[(q - 1) * BM + row];
        S += o.y * expf(o.x - M);
      }
    }
    if (nok) a.part[(size_t)rt * a.N + n] = make_float2(M, S);
  }
  if (nbad) atomicAdd(a.bad, nbad);
}

__global__ void __launch_bounds__(es::THREADS, 1)
    tc_estep_kernel(const __grid_constant__ CUtensorMap mK, const __grid_constant__ CUtensorMap mK2h,
                    const __grid_constant__ CUtensorMap mK2l, const __grid_constant__ CUtensorMap mMp,
                    const __grid_constant__ CUtensorMap mMS, const __grid_constant__ CUtensorMap mGh,
                    const __grid_constant__ CUtensorMap mGl, const __grid_constant__ CUtensorMap mHh,
                    const __grid_constant__ CUtensorMap mHl, TcEstepArgs a) {
  using namespace es;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + STAGES * STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* accum = empty + STAGES;
  uint64_t* drain = accum + 1;  // the MMA issuer's own completion wait before TMEM is freed
  uint32_t* tmem_slot = (uint32_t*)(drain + 1);
  float* s_A = (float*)(smem + STAGES * STAGE_BYTES + 256);
  float* s_scale = s_A + BN;
  float* s_lw = s_scale + BN;
  float2* s_half = (float2*)(s_lw + BN);  // [EPI_PARTS-1][BM] (max, sum exp) of column parts 1..

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const float sg = *a.sigma;
  const float inv2s2 = 1.0f / (2.0f * sg * sg);
  int pt, rt;
  if (a.tiles) {  // pruned: the listed tiles only
    const int2 t = a.tiles[blockIdx.x];
    pt = t.x;
    rt = t.y;
  } else {
    raster_tile(blockIdx.x + a.tile0, a.raster, a.n_pt, a.n_rt, pt, rt);
  }
  const int n0 = pt * BM, r0 = rt * BN;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      ptx::mbar_init(&full[s], 1);
      ptx::mbar_init(&empty[s], 1);
    }
    ptx::mbar_init(accum, 1);
    ptx::mbar_init(drain, 1);
    ptx::fence_mbar_init();
  }
  if (threadIdx.x < BN) {
    const int r = r0 + threadIdx.x;
    const float cnt = r < a.R ? a.rot_cnt[r] : 0.0f;
    s_A[threadIdx.x] = r < a.R ? a.rot_A[r] : 0.0f;
    s_scale[threadIdx.x] = cnt > 0.0f ? inv2s2 / cnt : -1.0f;  // < 0: invalid rotation
    s_lw[threadIdx.x] = r < a.R ? logf(a.rotw[r]) : 0.0f;
  }
  if (warp == 1) {
    ptx::tmem_alloc(tmem_slot, 512);
    ptx::tmem_relinquish();
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const unsigned char* flags = a.k2lo_any + (size_t)pt * a.nkb;
  const bool hlo = (a.gh_lo & 2) != 0;
  const int glo_end = (a.gh_lo & 1) ? a.glo_kb[pt] : 0;  // G lo on k-blocks below it

  if (warp == 0) {
    // ------------------------------------------------ TMA producer
    if (lane == 0) {
      const CUtensorMap* maps[kSlots] = {&mK, &mK2h, &mK2l, &mGh, &mMS, &mHh, &mMp, &mGl, &mHl};
      int kb = 0;
      for (; kb < a.nkb; ++kb) {
        const int s = kb % STAGES;
        const uint32_t ph = (kb / STAGES) & 1;
        if (!ptx::mbar_wait(&empty[s], ph ^ 1, a.status, 0, a.spin)) break;
        const bool lo = flags[kb] != 0;
        const bool glo = kb < glo_end;
        const int ntiles = kSlots - (lo ? 0 : 1) - (glo ? 0 : 1) - (hlo ? 0 : 1);
        ptx::mbar_arrive_expect_tx(&full[s], ntiles * TILE_BYTES);
        unsigned char* st = smem + s * STAGE_BYTES;
        for (int j = 0; j < kSlots; ++j) {
          if (j == sK2l && !lo) continue;
          if ((j == sGl && !glo) || (j == sHl && !hlo)) continue;
          ptx::tma_load_2d(st + j * TILE_BYTES, maps[j], kb * BK, j < sGh ? n0 : r0, &full[s]);
        }
      }
      // no copy may still be landing in shared memory when the CTA exits
      // (after a normal run the MMAs have consumed them all: no wait)
      ptx::drain_loads(full, STAGES, (uint32_t)kb, a.status, 11);
    }
  } else if (warp == 1) {
    // ------------------------------------------------ MMA issuer
    if (lane == 0) {
      constexpr uint32_t idesc2 = ptx::idesc_f16(BM, 2 * BN);  // the N = 256 pairs
      constexpr uint32_t idesc1 = ptx::idesc_f16(BM, BN);
      for (int kb = 0; kb < a.nkb; ++kb) {
        const int s = kb % STAGES;
        const uint32_t ph = (kb / STAGES) & 1;
        if (!ptx::mbar_wait(&full[s], ph, a.status, 1, a.spin)) break;
        ptx::tc_fence_after();
        const bool lo = flags[kb] != 0;
        const bool glo = kb < glo_end;
        const uint32_t base = ptx::smem_u32(smem + s * STAGE_BYTES);
#pragma unroll
        for (int ks = 0; ks < BK / 16; ++ks) {
          // 8-row core-matrix groups 512 B apart: a 256-row operand runs
          // through two adjacent 128-row slots
          auto d = [&](int j) { return ptx::smem_desc(base + j * TILE_BYTES + ks * 32, 512, 4); };
          const uint32_t acc = (kb | ks) ? 1u : 0u;
          ptx::mma_f16(tmem + 0, d(sK), d(sGh), idesc2, acc);      // B hi | den
          ptx::mma_f16(tmem + 256, d(sK2h), d(sHh), idesc2, acc);  // C hi | num
          if (glo) ptx::mma_f16(tmem + 0, d(sK), d(sGl), idesc1, 1u);     // B lo
          if (hlo) ptx::mma_f16(tmem + 256, d(sK2h), d(sHl), idesc1, 1u); // C lo
          if (lo) ptx::mma_f16(tmem + 256, d(sK2l), d(sHh), idesc2, 1u);  // K^2 lo: C | num
        }
        ptx::mma_commit(&empty[s]);
      }
      // fires when every MMA issued above has completed; after a timeout the
      // epilogue's own bounded wait reports it
      ptx::mma_commit(accum);
      // TMEM is freed only after every MMA issued here has completed, also
      // when the epilogue stopped waiting
      ptx::mma_commit(drain);
      ptx::mbar_wait(drain, 0, a.status, 12);
    }
  } else {
    // ------------------------------------------------ epilogue (warps 2-17)
    estep_epilogue(a, tmem, accum, s_A, s_scale, s_lw, s_half, warp, lane, n0, r0, rt);
  }
  ptx::tc_fence_before();
  __syncthreads();
  if (threadIdx.x == 32) ptx::settle_after_timeout(a.status);
  __syncthreads();
  if (warp == 1) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc(tmem, 512);
  }
}

// ------------------------------------------------ E-step on CTA pairs -----
// The same contractions over 256 patterns x 128 rotations per cluster of two
// CTAs, with 256-row MMAs (cta_group::2) issued by rank 0.  Each CTA keeps
// its own 128 patterns' tiles (K, K^2 hi, K^2 lo) and one half of every
// rotation-side operand: rank 0 the G and H columns of the [G | M'S] and
// [H | M'] pairs, rank 1 the M'S and M' columns, and 64 of the 128 G lo rows
// each.  Per 32-pixel stage a CTA loads 36 KB (44 KB with K^2 lo) instead of
// 56-64 KB for the same MMA work, and five stages fit in shared memory: the
// loads in flight cover more of the L2 / HBM latency that stalls the MMAs.  Both CTAs' loads complete
// on rank 0's `full` barriers; rank 0's commits arrive on both CTAs' `empty`
// and `accum` barriers.  The epilogue is the single-CTA kernel's, per CTA.
namespace es2 {
constexpr int STAGES = 5;
constexpr int TILE = 128 * es::BK * 2;  // 8 KB: 128 rows of one operand
constexpr int HALF = TILE / 2;          // 64 rows (G lo half)
constexpr int oK = 0, oK2h = TILE, oK2l = 2 * TILE, oB1 = 3 * TILE, oB2 = 4 * TILE,
              oGl = 5 * TILE;
constexpr int STAGE_BYTES = 5 * TILE + HALF;  // 44 KB; no H lo (known intensity runs single CTAs)
// barriers (256 B), per-rotation rows (3 x 128 floats), epilogue parts
constexpr int EXTRA = 256 + 3 * es::BN * 4 + (es::EPI_PARTS - 1) * es::BM * 8;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + EXTRA + 1024;
static_assert(SMEM_BYTES <= 232448, "shared memory of the pair kernel");
}  // namespace es2

__global__ void __launch_bounds__(es::THREADS, 1)
    tc_estep_pair_kernel(const __grid_constant__ CUtensorMap mK,
                         const __grid_constant__ CUtensorMap mK2h,
                         const __grid_constant__ CUtensorMap mK2l,
                         const __grid_constant__ CUtensorMap mMp,
                         const __grid_constant__ CUtensorMap mMS,
                         const __grid_constant__ CUtensorMap mGh,
                         const __grid_constant__ CUtensorMap mGl64,
                         const __grid_constant__ CUtensorMap mHh, TcEstepArgs a) {
  using namespace es;
  using es2::STAGES;
  using es2::STAGE_BYTES;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + STAGES * STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* accum = empty + STAGES;
  uint64_t* drain = accum + 1;  // rank 0's MMA issuer waits on it before TMEM is freed
  uint32_t* tmem_slot = (uint32_t*)(drain + 1);
  float* s_A = (float*)(smem + STAGES * STAGE_BYTES + 256);
  float* s_scale = s_A + BN;
  float* s_lw = s_scale + BN;
  float2* s_half = (float2*)(s_lw + BN);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t rank = ptx::cluster_ctarank();
  const float sg = *a.sigma;
  const float inv2s2 = 1.0f / (2.0f * sg * sg);
  const int n_ptp = (a.n_pt + 1) / 2;
  int ptp, rt;
  raster_tile((int)(blockIdx.x >> 1) + a.tile0, a.raster, n_ptp, a.n_rt, ptp, rt);
  const int pt = 2 * ptp + (int)rank;  // may be n_pt (no patterns) when n_pt is odd
  const int n0 = pt * BM, r0 = rt * BN;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      ptx::mbar_init(&full[s], 1);
      ptx::mbar_init(&empty[s], 1);
    }
    ptx::mbar_init(accum, 1);
    ptx::mbar_init(drain, 1);
    ptx::fence_mbar_init();
  }
  if (threadIdx.x < BN) {
    const int r = r0 + threadIdx.x;
    const float cnt = r < a.R ? a.rot_cnt[r] : 0.0f;
    s_A[threadIdx.x] = r < a.R ? a.rot_A[r] : 0.0f;
    s_scale[threadIdx.x] = cnt > 0.0f ? inv2s2 / cnt : -1.0f;
    s_lw[threadIdx.x] = r < a.R ? logf(a.rotw[r]) : 0.0f;
  }
  if (warp == 1) {
    ptx::tmem_alloc_pair(tmem_slot, 512);
    ptx::tmem_relinquish_pair();
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::cluster_sync();  // both CTAs' barriers initialised and TMEM allocated
  ptx::tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  // the K^2 lo MMA runs for a k-block when either pattern tile needs it
  const int pt0 = 2 * ptp, pt1 = 2 * ptp + 1;
  const unsigned char* flags0 = a.k2lo_any + (size_t)pt0 * a.nkb;
  const unsigned char* flags1 = pt1 < a.n_pt ? a.k2lo_any + (size_t)pt1 * a.nkb : nullptr;
  // G lo on the k-blocks either pattern tile needs (H lo, gh_lo bit 1, runs on single CTAs)
  const int glo_end =
      (a.gh_lo & 1) ? max(a.glo_kb[pt0], pt1 < a.n_pt ? a.glo_kb[pt1] : 0) : 0;

  if (warp == 0) {
    // ------------------------------------------------ TMA producer (both CTAs)
    if (lane == 0) {
      const CUtensorMap* mb1 = rank ? &mMS : &mGh;
      const CUtensorMap* mb2 = rank ? &mMp : &mHh;
      int kb = 0;
      for (; kb < a.nkb; ++kb) {
        const int s = kb % STAGES;
        const uint32_t ph = (kb / STAGES) & 1;
        if (!ptx::mbar_wait(&empty[s], ph ^ 1, a.status, 0, a.spin)) break;
        const bool lo = flags0[kb] != 0 || (flags1 && flags1[kb] != 0);
        const bool glo = kb < glo_end;
        const uint32_t bytes = (lo ? 5 : 4) * es2::TILE + (glo ? es2::HALF : 0);
        if (rank == 0) ptx::mbar_arrive_expect_tx(&full[s], 2 * bytes);  // both CTAs' loads
        const uint32_t fb = ptx::mapa_shared(ptx::smem_u32(&full[s]), 0);
        unsigned char* st = smem + s * STAGE_BYTES;
        const int x = kb * BK;
        ptx::tma_load_2d_pair(st + es2::oK, &mK, x, n0, fb);
        ptx::tma_load_2d_pair(st + es2::oK2h, &mK2h, x, n0, fb);
        if (lo) ptx::tma_load_2d_pair(st + es2::oK2l, &mK2l, x, n0, fb);
        ptx::tma_load_2d_pair(st + es2::oB1, mb1, x, r0, fb);
        ptx::tma_load_2d_pair(st + es2::oB2, mb2, x, r0, fb);
        if (glo) ptx::tma_load_2d_pair(st + es2::oGl, &mGl64, x, r0 + 64 * (int)rank, fb);
      }
      // rank 0's barriers count both CTAs' bytes of the stages it armed
      if (rank == 0) ptx::drain_loads(full, STAGES, (uint32_t)kb, a.status, 11);
    }
  } else if (warp == 1) {
    // ------------------------------------------------ MMA issuer (rank 0)
    if (rank == 0 && lane == 0) {
      constexpr uint32_t idesc2 = ptx::idesc_f16(2 * BM, 2 * BN);  // 256 x 256 pairs
      constexpr uint32_t idesc1 = ptx::idesc_f16(2 * BM, BN);      // 256 x 128 lo terms
      for (int kb = 0; kb < a.nkb; ++kb) {
        const int s = kb % STAGES;
        const uint32_t ph = (kb / STAGES) & 1;
        if (!ptx::mbar_wait(&full[s], ph, a.status, 1, a.spin)) break;
        ptx::tc_fence_after();
        const bool lo = flags0[kb] != 0 || (flags1 && flags1[kb] != 0);
        const bool glo = kb < glo_end;
        const uint32_t base = ptx::smem_u32(smem + s * STAGE_BYTES);
#pragma unroll
        for (int ks = 0; ks < BK / 16; ++ks) {
          auto d = [&](int off) { return ptx::smem_desc(base + off + ks * 32, 512, 4); };
          const uint32_t acc = (kb | ks) ? 1u : 0u;
          ptx::mma_f16_pair(tmem + 0, d(es2::oK), d(es2::oB1), idesc2, acc);      // B hi | den
          ptx::mma_f16_pair(tmem + 256, d(es2::oK2h), d(es2::oB2), idesc2, acc);  // C hi | num
          if (glo) ptx::mma_f16_pair(tmem + 0, d(es2::oK), d(es2::oGl), idesc1, 1u);
          if (lo) ptx::mma_f16_pair(tmem + 256, d(es2::oK2l), d(es2::oB2), idesc2, 1u);
        }
        ptx::mma_commit_pair(&empty[s], 0x3);
      }
      ptx::mma_commit_pair(accum, 0x3);
      ptx::mma_commit_pair(drain, 0x1);  // both CTAs' TMEM is written by these MMAs
      ptx::mbar_wait(drain, 0, a.status, 12);
    }
  } else {
    // ------------------------------------------------ epilogue (warps 2-17)
    estep_epilogue(a, tmem, accum, s_A, s_scale, s_lw, s_half, warp, lane, n0, r0, rt);
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::cluster_sync();  // the pair's MMAs and barrier traffic are over in both CTAs
  if (threadIdx.x == 32) ptx::settle_after_timeout(a.status);
  __syncthreads();
  if (warp == 1) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc_pair(tmem, 512);
  }
}

// ------------------------------------------------ E-step, true Poisson -----
// L_ri = log w_r + c_i sum_p k_ip log s~_rp + K_i log(K_i / S_r) - K_i,
// s~ = max(s, floor), K_i = c_i sum_p k_ip, S_r = sum_p s~_rp, phi = K_i / S_r
// (known intensity: phi = 1, L = log w_r + c_i sum k log s~ - S_r), as the
// FP32 path.  One contraction K . (log S~)^T with log S~ as FP16 hi + lo;
// one CTA owns 128 patterns x 256 rotations (TMEM columns 0-255) and writes
// one (max, sum exp) partial per 128-rotation half.
namespace ep {
constexpr int BM = 128;   // patterns per tile (TMEM lanes)
constexpr int BN = 256;   // rotations per tile
constexpr int BK = 32;    // pixels per stage (64 B rows, 64B swizzle)
constexpr int STAGES = 4;
constexpr int A_BYTES = BM * BK * 2;  // 8 KB
constexpr int B_BYTES = BN * BK * 2;  // 16 KB
constexpr int STAGE_BYTES = A_BYTES + 2 * B_BYTES;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 256 + 2 * BN * 4 + 1024;
constexpr int EPI_WARPS = 8;  // two per TMEM lane quarter, one per 128-column half
constexpr int THREADS = 64 + 32 * EPI_WARPS;
}  // namespace ep

struct TcEstepPoisArgs {
  int N, R, n_pt, n_rt, nkb;
  int raster;             // tile order (raster_tile)
  int tile0;              // CTA b runs tile tile0 + b of the order
  const int2* tiles;      // pruned iteration: (pattern tile, 256-rotation tile) per CTA
  int n_part;             // 128-rotation partial tiles
  const float* rot_ssum;  // S_r
  const float* rotw;
  const float* Ksum;      // K_i (normalised counts)
  const float* cnorm;     // c_i
  int known_intensity;
  float* L;
  float* PHI;
  float2* part;
  int* status;
  uint32_t spin;  // polls per pipeline wait
};

__global__ void __launch_bounds__(ep::THREADS, 1)
    tc_estep_pois_kernel(const __grid_constant__ CUtensorMap mK,
                         const __grid_constant__ CUtensorMap mLh,
                         const __grid_constant__ CUtensorMap mLl, TcEstepPoisArgs a) {
  using namespace ep;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + STAGES * STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* accum = empty + STAGES;
  uint64_t* drain = accum + 1;  // the MMA issuer's own completion wait before TMEM is freed
  uint32_t* tmem_slot = (uint32_t*)(drain + 1);
  float* s_ss = (float*)(smem + STAGES * STAGE_BYTES + 256);
  float* s_lw = s_ss + BN;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int pt, rt;
  if (a.tiles) {  // pruned: the listed tiles only
    const int2 t = a.tiles[blockIdx.x];
    pt = t.x;
    rt = t.y;
  } else {
    raster_tile(blockIdx.x + a.tile0, a.raster, a.n_pt, a.n_rt, pt, rt);
  }
  const int n0 = pt * BM, r0 = rt * BN;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      ptx::mbar_init(&full[s], 1);
      ptx::mbar_init(&empty[s], 1);
    }
    ptx::mbar_init(accum, 1);
    ptx::mbar_init(drain, 1);
    ptx::fence_mbar_init();
  }
  for (int c = threadIdx.x; c < BN; c += blockDim.x) {
    const int r = r0 + c;
    s_ss[c] = r < a.R ? a.rot_ssum[r] : 1.0f;
    s_lw[c] = r < a.R ? logf(a.rotw[r]) : 0.0f;
  }
  if (warp == 1) {
    ptx::tmem_alloc(tmem_slot, BN);
    ptx::tmem_relinquish();
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ------------------------------------------------ TMA producer
    if (lane == 0) {
      int kb = 0;
      for (; kb < a.nkb; ++kb) {
        const int s = kb % STAGES;
        const uint32_t ph = (kb / STAGES) & 1;
        if (!ptx::mbar_wait(&empty[s], ph ^ 1, a.status, 8, a.spin)) break;
        ptx::mbar_arrive_expect_tx(&full[s], STAGE_BYTES);
        unsigned char* st = smem + s * STAGE_BYTES;
        ptx::tma_load_2d(st, &mK, kb * BK, n0, &full[s]);
        ptx::tma_load_2d(st + A_BYTES, &mLh, kb * BK, r0, &full[s]);
        ptx::tma_load_2d(st + A_BYTES + B_BYTES, &mLl, kb * BK, r0, &full[s]);
      }
      ptx::drain_loads(full, STAGES, (uint32_t)kb, a.status, 11);  // none in flight at exit
    }
  } else if (warp == 1) {
    // ------------------------------------------------ MMA issuer
    if (lane == 0) {
      constexpr uint32_t idesc = ptx::idesc_f16(BM, BN);
      for (int kb = 0; kb < a.nkb; ++kb) {
        const int s = kb % STAGES;
        const uint32_t ph = (kb / STAGES) & 1;
        if (!ptx::mbar_wait(&full[s], ph, a.status, 9, a.spin)) break;
        ptx::tc_fence_after();
        const uint32_t base = ptx::smem_u32(smem + s * STAGE_BYTES);
#pragma unroll
        for (int ks = 0; ks < BK / 16; ++ks) {
          const uint64_t aK = ptx::smem_desc(base + ks * 32, 512, 4);
          const uint64_t bh = ptx::smem_desc(base + A_BYTES + ks * 32, 512, 4);
          const uint64_t bl = ptx::smem_desc(base + A_BYTES + B_BYTES + ks * 32, 512, 4);
          ptx::mma_f16(tmem, aK, bh, idesc, (kb | ks) ? 1u : 0u);
          ptx::mma_f16(tmem, aK, bl, idesc, 1u);
        }
        ptx::mma_commit(&empty[s]);
      }
      ptx::mma_commit(accum);
      ptx::mma_commit(drain);  // TMEM is freed only after these MMAs have completed
      ptx::mbar_wait(drain, 0, a.status, 12);
    }
  } else {
    // ------------------------------------------------ epilogue (warps 2-9)
    const int quarter = warp & 3;
    const int row = quarter * 32 + lane;
    const int n = n0 + row;
    const bool nok = n < a.N;
    const float ci = nok ? a.cnorm[n] : 1.0f;
    const float Ki = nok ? a.Ksum[n] : 0.0f;
    const bool waited = ptx::mbar_wait_sleep(accum, 0, a.status, 10, 256, a.spin);
    if (waited) ptx::tc_fence_after();
    const uint32_t lane_addr = tmem + ((uint32_t)(quarter * 32) << 16);
    {
      const int h = (warp - 2) >> 2;  // the 128-rotation half this warp evaluates
      float m = -INFINITY, ssum = 0.0f;
      for (int c0 = h * 128; waited && c0 < h * 128 + 128; c0 += 16) {
        float v[16];
        ptx::tmem_ld16(lane_addr + c0, v);
        ptx::tmem_wait_ld();
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int cl = c0 + j;
          const int r = r0 + cl;
          const float acc = ci * v[j];
          float l, f;
          if (a.known_intensity) {
            f = 1.0f;
            l = s_lw[cl] + acc - s_ss[cl];
          } else if (Ki > 0.0f) {
            f = Ki / s_ss[cl];
            l = s_lw[cl] + acc + Ki * logf(f) - Ki;
          } else {
            f = 0.0f;
            l = s_lw[cl];
          }
          const bool ok = nok && r < a.R;
          if (ok) {
            a.L[(size_t)r * a.N + n] = l;
            a.PHI[(size_t)r * a.N + n] = f;
          }
          const float L = ok ? l : -INFINITY;
          if (L > m) {
            ssum = ssum * expf(m - L) + 1.0f;
            m = L;
          } else if (L > -INFINITY) {
            ssum += expf(L - m);
          }
        }
      }
      const int t = 2 * rt + h;
      if (nok && t < a.n_part) a.part[(size_t)t * a.N + n] = make_float2(m, ssum);
    }
  }
  ptx::tc_fence_before();
  __syncthreads();
  if (threadIdx.x == 32) ptx::settle_after_timeout(a.status);
  __syncthreads();
  if (warp == 1) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc(tmem, BN);
  }
}

// ------------------------------------------------------------ M-step -----
namespace ms {
constexpr int BM = 128;   // rotations per tile (TMEM lanes)
constexpr int BN = 256;   // pixels per tile
constexpr int BK = 64;    // patterns per stage (128 B rows, 128B swizzle)
constexpr int A_BYTES = BM * BK * 2;  // 16 KB
constexpr int B_BYTES = BN * BK * 2;  // 32 KB
constexpr int EPI_WARPS = 8;          // two per TMEM lane quarter, 128 columns each
constexpr int THREADS = 64 + 32 * EPI_WARPS;
}  // namespace ms

struct TcMstepArgs {
  int R, Kp, Np, P_eff, n_qt, n_rt, nkb, n_tiles;
  int raster;  // tile order (raster_tile over pixel tiles x rotation tiles)
  const float* T;
  const float* qscale;  // [R] 2^-e_r
  const float* rot;
  const float *cx, *cy, *cz;
  int side, interp, deterministic;
  int aggregate;  // 1: lanes hitting the same voxel combine before one atomic
  float* model;
  float* weight;
  unsigned long long* fix_m;
  unsigned long long* fix_w;
  float2* acc2;
  const float2* fix_scale;  // {model, weight} fixed-point scales (deterministic mode)
  float* u;                 // sorted mode: pair values [P_eff][ldu] instead of insertion
  int ldu;
  int q_lo;  // 1: Q hi + lo, 0: Q hi only
  // pruned iteration: the pattern k-blocks of rotation tile rt are
  // kb_list[kb_off[rt] .. kb_off[rt+1]) (Q is zero elsewhere); nullptr: all
  const int* kb_off;
  const int* kb_list;
  int* status;
  uint32_t spin;  // polls per pipeline wait
};

// The k-blocks of rotation tile rt: count, and the j-th of them.
__device__ __forceinline__ int ms_nkb(const TcMstepArgs& a, int rt) {
  return a.kb_off ? a.kb_off[rt + 1] - a.kb_off[rt] : a.nkb;
}
__device__ __forceinline__ int ms_kb(const TcMstepArgs& a, int rt, int j) {
  return a.kb_off ? a.kb_list[a.kb_off[rt] + j] : j;
}

__device__ __forceinline__ void tc_add(const TcMstepArgs& a, size_t v, float val, float w) {
  if (a.deterministic) {
    const float2 sc = __ldg(a.fix_scale);
    atomicAdd(a.fix_m + v, (unsigned long long)fixed_from_float(__fmul_rn(val, sc.x)));
    atomicAdd(a.fix_w + v, (unsigned long long)fixed_from_float(__fmul_rn(w, sc.y)));
  } else {
    atomicAdd(a.acc2 + v, make_float2(val, w));  // model and weight in one 8-byte atomic
  }
}

// Nearest-voxel insertion of one value per lane.  With aggregation (float
// atomics only), lanes of the warp whose voxels coincide -- neighbouring
// rotations at the same small-radius pixel -- add their values in registers
// and their lowest lane issues one atomic.  Called by all 32 lanes.
__device__ __forceinline__ void tc_insert_nearest(const TcMstepArgs& a, bool on, long long v,
                                                  float val, float w) {
  if (a.aggregate && !a.deterministic) {
    const unsigned act = __ballot_sync(0xffffffffu, on);
    if (!on) return;
    const unsigned peers = __match_any_sync(act, v);
    const int me = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    // every lane of a peer group runs the same sequence of shuffles
    for (unsigned m = peers & (peers - 1); m; m &= m - 1) {
      const int src = __ffs(m) - 1;
      const float pv = __shfl_sync(peers, val, src);
      const float pw = __shfl_sync(peers, w, src);
      if (me == leader) {
        val += pv;
        w += pw;
      }
    }
    if (me == leader) atomicAdd(a.acc2 + v, make_float2(val, w));
    return;
  }
  if (on) tc_add(a, (size_t)v, val, w);
}

__device__ __forceinline__ void tc_insert(const TcMstepArgs& a, const RotMat& R, bool on, float x,
                                          float y, float z, float val, float w) {
  const int side = a.side;
  if (a.interp == EMC_INTERP_NEAREST) {
    const long ix = voxel_round(voxel_coord(side, rotate_row(R, 0, x, y, z)));
    const long iy = voxel_round(voxel_coord(side, rotate_row(R, 1, x, y, z)));
    const long iz = voxel_round(voxel_coord(side, rotate_row(R, 2, x, y, z)));
    const bool in = on && ix >= 0 && ix < side && iy >= 0 && iy < side && iz >= 0 && iz < side;
    tc_insert_nearest(a, in, in ? ((long long)iz * side + iy) * side + ix : -1, val, w);
  } else {
    if (!on) return;
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
      tc_add(a, ((size_t)zi * side + yi) * side + xi, val * f, w * f);
    }
  }
}

// Tile t of the grouped raster (raster_tile over pixel tiles x rotation
// tiles; the default -16: groups of 16 pixel tiles run through all rotation
// tiles, 5-6 % faster than groups of 8 rotation tiles at 128^3 and 256^3).
__device__ __forceinline__ void ms_tile(const TcMstepArgs& a, int t, int& r0, int& q0) {
  int qt, rt;
  raster_tile(t, a.raster, a.n_qt, a.n_rt, qt, rt);
  r0 = rt * ms::BM;
  q0 = qt * ms::BN;
}

// Persistent: CTA b takes tiles b, b + grid, ...  The k-block ring runs on
// across tiles, and the accumulator is double-buffered in TMEM (columns
// 0-255 and 256-511), so the insertion epilogue of one tile overlaps the
// MMAs of the next.
// Stage ring of the single-CTA M-step: Q hi (+ Q lo) and the 256 K^T rows of
// a 64-pattern k-block.  Without the Q lo slot a stage is 48 KB and four fit
// where three of 64 KB do: a third more bytes in flight for the same ring.
template <int QLO>
struct MsRing {
  static constexpr int kStageBytes = (QLO ? 2 : 1) * ms::A_BYTES + ms::B_BYTES;
  static constexpr int kStages = QLO ? 3 : 4;
  static constexpr int kOffK = (QLO ? 2 : 1) * ms::A_BYTES;  // K^T tile in a stage
  static constexpr int kSmem = kStages * kStageBytes + 256 + 1024;
  static_assert(kSmem <= 232448, "shared memory of the M-step ring");
};

template <int QLO>
__global__ void __launch_bounds__(ms::THREADS, 1)
    tc_mstep_kernel(const __grid_constant__ CUtensorMap mQh, const __grid_constant__ CUtensorMap mQl,
                    const __grid_constant__ CUtensorMap mKt, TcMstepArgs a) {
  using namespace ms;
  using Ring = MsRing<QLO>;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + Ring::kStages * Ring::kStageBytes);
  uint64_t* empty = full + Ring::kStages;
  uint64_t* tfull = empty + Ring::kStages;  // [2] accumulator ready
  uint64_t* tempty = tfull + 2;      // [2] accumulator drained (one arrival per epilogue warp)
  uint64_t* drain = tempty + 2;      // the MMA issuer's own completion wait before TMEM is freed
  uint32_t* tmem_slot = (uint32_t*)(drain + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < Ring::kStages; ++s) {
      ptx::mbar_init(&full[s], 1);
      ptx::mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      ptx::mbar_init(&tfull[b], 1);
      ptx::mbar_init(&tempty[b], EPI_WARPS);
    }
    ptx::mbar_init(drain, 1);
    ptx::fence_mbar_init();
  }
  if (warp == 1) {
    ptx::tmem_alloc(tmem_slot, 512);
    ptx::tmem_relinquish();
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ------------------------------------------------ TMA producer
    if (lane == 0) {
      uint32_t it = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < a.n_tiles && ok; t += gridDim.x) {
        int r0, q0;
        ms_tile(a, t, r0, q0);
        const int nk = ms_nkb(a, r0 / BM);
        for (int j = 0; j < nk; ++j, ++it) {
          const int kb = ms_kb(a, r0 / BM, j);
          const int s = it % Ring::kStages;
          const uint32_t ph = (it / Ring::kStages) & 1;
          if (!ptx::mbar_wait(&empty[s], ph ^ 1, a.status, 4, a.spin)) {
            ok = false;
            break;
          }
          ptx::mbar_arrive_expect_tx(&full[s], Ring::kStageBytes);
          unsigned char* st = smem + s * Ring::kStageBytes;
          ptx::tma_load_2d(st, &mQh, kb * BK, r0, &full[s]);
          if (QLO) ptx::tma_load_2d(st + A_BYTES, &mQl, kb * BK, r0, &full[s]);
          ptx::tma_load_2d(st + Ring::kOffK, &mKt, kb * BK, q0, &full[s]);
        }
      }
      ptx::drain_loads(full, Ring::kStages, it, a.status, 11);  // none in flight at exit
    }
  } else if (warp == 1) {
    // ------------------------------------------------ MMA issuer
    if (lane == 0) {
      constexpr uint32_t idesc = ptx::idesc_f16(BM, BN);
      uint32_t it = 0;
      bool ok = true;
      int j = 0;
      for (int t = blockIdx.x; t < a.n_tiles && ok; t += gridDim.x, ++j) {
        const int b = j & 1;
        const uint32_t d = tmem + (uint32_t)(b * BN);
        if (!ptx::mbar_wait(&tempty[b], ((j >> 1) & 1) ^ 1, a.status, 7, a.spin)) break;
        ptx::tc_fence_after();
        int r0t, q0t;
        ms_tile(a, t, r0t, q0t);
        // a tile with no k-block leaves the buffer as it was: its rotations
        // have no responsibility (T_r = 0), so the epilogue inserts nothing
        const int nk = ms_nkb(a, r0t / BM);
        for (int kb = 0; kb < nk; ++kb, ++it) {
          const int s = it % Ring::kStages;
          const uint32_t ph = (it / Ring::kStages) & 1;
          if (!ptx::mbar_wait(&full[s], ph, a.status, 5, a.spin)) {
            ok = false;
            break;
          }
          ptx::tc_fence_after();
          const uint32_t base = ptx::smem_u32(smem + s * Ring::kStageBytes);
#pragma unroll
          for (int ks = 0; ks < BK / 16; ++ks) {
            const uint64_t dQh = ptx::smem_desc(base + ks * 32, 1024, 2);
            const uint64_t dQl = ptx::smem_desc(base + A_BYTES + ks * 32, 1024, 2);
            const uint64_t dK = ptx::smem_desc(base + Ring::kOffK + ks * 32, 1024, 2);
            ptx::mma_f16(d, dQh, dK, idesc, (kb | ks) ? 1u : 0u);
            if (QLO) ptx::mma_f16(d, dQl, dK, idesc, 1u);
          }
          ptx::mma_commit(&empty[s]);
        }
        ptx::mma_commit(&tfull[b]);  // fires when this tile's MMAs have completed
      }
      ptx::mma_commit(drain);  // TMEM is freed only after every MMA issued here has completed
      ptx::mbar_wait(drain, 0, a.status, 12);
    }
  } else {
    // ------------------------------------------------ insertion epilogue (warps 2-9)
    const int quarter = warp & 3;       // TMEM lanes this warp may access
    const int half = (warp - 2) >> 2;   // which 128 of the tile's 256 columns
    const int rl = quarter * 32 + lane;
    int j = 0;
    for (int t = blockIdx.x; t < a.n_tiles; t += gridDim.x, ++j) {
      const int b = j & 1;
      int r0, q0;
      ms_tile(a, t, r0, q0);
      const int r = r0 + rl;
      const bool rok = r < a.R;
      const float Tr = rok ? a.T[r] : 0.0f;
      const float qs = rok ? a.qscale[r] : 0.0f;
      const bool live = rok && Tr > 1e-10f;
      RotMat Rm = {};
      if (rok) Rm = quat_to_matrix(a.rot + 4 * (size_t)r);
      if (!ptx::mbar_wait_sleep(&tfull[b], (j >> 1) & 1, a.status, 6, 128, a.spin)) break;
      ptx::tc_fence_after();
      const uint32_t lane_addr = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(b * BN);
      for (int c0 = half * 128; c0 < half * 128 + 128; c0 += 16) {
        float u[16];
        ptx::tmem_ld16(lane_addr + c0, u);
        ptx::tmem_wait_ld();
        if (q0 + c0 >= a.P_eff) continue;  // padding columns (uniform over the warp)
#pragma unroll
        for (int jj = 0; jj < 16; ++jj) {  // fully unrolled: u[] stays in registers
          const int q = q0 + c0 + jj;
          if (q < a.P_eff) {  // uniform over the warp
            const float U = u[jj] * qs;
            const float slice = live ? U / Tr : 0.0f;
            if (a.u) {  // sorted mode: a coalesced store per column (lanes: rotations)
              if (rok) a.u[(size_t)q * a.ldu + r] = Tr * slice;
            } else {
              tc_insert(a, Rm, live, __ldg(a.cx + q), __ldg(a.cy + q), __ldg(a.cz + q),
                        Tr * slice, Tr);
            }
          }
        }
      }
      // this warp's reads of buffer b are complete: hand it back to the MMA warp
      ptx::tc_fence_before();
      __syncwarp();
      if (lane == 0) ptx::mbar_arrive(&tempty[b]);
    }
  }
  ptx::tc_fence_before();
  __syncthreads();
  if (threadIdx.x == 32) ptx::settle_after_timeout(a.status);
  __syncthreads();
  if (warp == 1) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc(tmem, 512);
  }
}

// ------------------------------------------------- M-step on CTA pairs -----
// The M-step's tiles as 256 rotations x 256 pixels per cluster of two CTAs:
// 256-row MMAs (cta_group::2) issued by rank 0, each CTA holding the Q rows
// of its own 128 rotations and 128 of the tile's 256 pixel rows of K^T.  Per
// 64-pattern stage a CTA loads 32 KB instead of 48 KB for the same MMA work
// and its tensor core reads half of the pixel-side operand.  Persistent over
// the cluster's tiles; each CTA's TMEM holds its 128 rotations x 256 pixels,
// double-buffered (2 x 256 columns), so the insertion epilogue of one tile
// overlaps the MMAs of the next.  Both CTAs' loads complete on rank 0's
// `full` barriers; rank 0's commits multicast to both CTAs' `empty` and
// `tfull`; the epilogue warps of both CTAs hand a buffer back on rank 0's
// `tempty`.  Full scans only (a pruned M-step runs single CTAs).
namespace ms2 {
constexpr int A_BYTES = ms::BM * ms::BK * 2;  // 16 KB: 128 rotations x 64 patterns
constexpr int B_BYTES = 128 * ms::BK * 2;     // 16 KB: 128 pixels x 64 patterns
// stage: Q hi (+ Q lo) and the CTA's half of K^T; six 32 KB stages without
// the Q lo slot, four of 48 KB with it
template <int QLO>
struct Ring {
  static constexpr int kStageBytes = (QLO ? 2 : 1) * A_BYTES + B_BYTES;
  static constexpr int kStages = QLO ? 4 : 6;
  static constexpr int kOffK = (QLO ? 2 : 1) * A_BYTES;
  static constexpr int kSmem = kStages * kStageBytes + 256 + 1024;
  static_assert(kSmem <= 232448, "shared memory of the pair M-step");
};
}  // namespace ms2

template <int QLO>
__global__ void __launch_bounds__(ms::THREADS, 1)
    tc_mstep_pair_kernel(const __grid_constant__ CUtensorMap mQh,
                         const __grid_constant__ CUtensorMap mQl,
                         const __grid_constant__ CUtensorMap mKt128, TcMstepArgs a) {
  using namespace ms;
  constexpr int STAGES = ms2::Ring<QLO>::kStages;
  constexpr int STAGE_BYTES = ms2::Ring<QLO>::kStageBytes;
  constexpr int OFF_K = ms2::Ring<QLO>::kOffK;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + STAGES * STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* tfull = empty + STAGES;  // [2] accumulator ready (both CTAs)
  uint64_t* tempty = tfull + 2;      // [2] rank 0: accumulator drained by both CTAs
  uint64_t* drain = tempty + 2;      // rank 0's MMA issuer waits on it before TMEM is freed
  uint32_t* tmem_slot = (uint32_t*)(drain + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t rank = ptx::cluster_ctarank();
  const int cl = (int)(blockIdx.x >> 1), ncl = (int)(gridDim.x >> 1);
  const int n_rp = (a.n_rt + 1) / 2;  // rotation-tile pairs
  const int n_tiles = n_rp * a.n_qt;
  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      ptx::mbar_init(&full[s], 1);
      ptx::mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      ptx::mbar_init(&tfull[b], 1);
      ptx::mbar_init(&tempty[b], 2 * EPI_WARPS);
    }
    ptx::mbar_init(drain, 1);
    ptx::fence_mbar_init();
  }
  if (warp == 1) {
    ptx::tmem_alloc_pair(tmem_slot, 512);
    ptx::tmem_relinquish_pair();
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::cluster_sync();  // both CTAs' barriers initialised and TMEM allocated
  ptx::tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ------------------------------------------------ TMA producer (both CTAs)
    if (lane == 0) {
      uint32_t it = 0;
      bool ok = true;
      const uint32_t bytes = STAGE_BYTES;
      for (int t = cl; t < n_tiles && ok; t += ncl) {
        int qt, rp;
        raster_tile(t, a.raster, a.n_qt, n_rp, qt, rp);
        const int r0 = (2 * rp + (int)rank) * BM, q0 = qt * BN + 128 * (int)rank;
        for (int kb = 0; kb < a.nkb; ++kb, ++it) {
          const int s = it % STAGES;
          const uint32_t ph = (it / STAGES) & 1;
          if (!ptx::mbar_wait(&empty[s], ph ^ 1, a.status, 4, a.spin)) {
            ok = false;
            break;
          }
          if (rank == 0) ptx::mbar_arrive_expect_tx(&full[s], 2 * bytes);  // both CTAs' loads
          const uint32_t fb = ptx::mapa_shared(ptx::smem_u32(&full[s]), 0);
          unsigned char* st = smem + s * STAGE_BYTES;
          ptx::tma_load_2d_pair(st, &mQh, kb * BK, r0, fb);
          if (QLO) ptx::tma_load_2d_pair(st + ms2::A_BYTES, &mQl, kb * BK, r0, fb);
          ptx::tma_load_2d_pair(st + OFF_K, &mKt128, kb * BK, q0, fb);
        }
      }
      // rank 0's barriers count both CTAs' bytes of the stages it armed
      if (rank == 0) ptx::drain_loads(full, STAGES, it, a.status, 11);
    }
  } else if (warp == 1) {
    // ------------------------------------------------ MMA issuer (rank 0)
    if (rank == 0 && lane == 0) {
      constexpr uint32_t idesc = ptx::idesc_f16(2 * BM, BN);  // 256 x 256
      uint32_t it = 0;
      bool ok = true;
      int j = 0;
      for (int t = cl; t < n_tiles && ok; t += ncl, ++j) {
        const int b = j & 1;
        const uint32_t d = tmem + (uint32_t)(b * BN);
        if (!ptx::mbar_wait_cluster(&tempty[b], ((j >> 1) & 1) ^ 1, a.status, 7, a.spin)) break;
        ptx::tc_fence_after();
        for (int kb = 0; kb < a.nkb; ++kb, ++it) {
          const int s = it % STAGES;
          const uint32_t ph = (it / STAGES) & 1;
          if (!ptx::mbar_wait(&full[s], ph, a.status, 5, a.spin)) {
            ok = false;
            break;
          }
          ptx::tc_fence_after();
          const uint32_t base = ptx::smem_u32(smem + s * STAGE_BYTES);
#pragma unroll
          for (int ks = 0; ks < BK / 16; ++ks) {
            const uint64_t dQh = ptx::smem_desc(base + ks * 32, 1024, 2);
            const uint64_t dQl = ptx::smem_desc(base + ms2::A_BYTES + ks * 32, 1024, 2);
            const uint64_t dK = ptx::smem_desc(base + OFF_K + ks * 32, 1024, 2);
            ptx::mma_f16_pair(d, dQh, dK, idesc, (kb | ks) ? 1u : 0u);
            if (QLO) ptx::mma_f16_pair(d, dQl, dK, idesc, 1u);
          }
          ptx::mma_commit_pair(&empty[s], 0x3);
        }
        ptx::mma_commit_pair(&tfull[b], 0x3);  // fires when this tile's MMAs have completed
      }
      ptx::mma_commit_pair(drain, 0x1);  // both CTAs' TMEM is written by these MMAs
      ptx::mbar_wait(drain, 0, a.status, 12);
    }
  } else {
    // ------------------------------------------------ insertion epilogue (warps 2-9)
    const int quarter = warp & 3;      // TMEM lanes this warp may access
    const int half = (warp - 2) >> 2;  // which 128 of the tile's 256 columns
    const int rl = quarter * 32 + lane;
    const uint32_t back = rank == 0 ? 0u : 1u;
    int j = 0;
    for (int t = cl; t < n_tiles; t += ncl, ++j) {
      const int b = j & 1;
      int qt, rp;
      raster_tile(t, a.raster, a.n_qt, n_rp, qt, rp);
      const int r0 = (2 * rp + (int)rank) * BM, q0 = qt * BN;  // TMEM column c: pixel q0 + c
      const int r = r0 + rl;
      const bool rok = r < a.R;
      const float Tr = rok ? a.T[r] : 0.0f;
      const float qs = rok ? a.qscale[r] : 0.0f;
      const bool live = rok && Tr > 1e-10f;
      RotMat Rm = {};
      if (rok) Rm = quat_to_matrix(a.rot + 4 * (size_t)r);
      if (!ptx::mbar_wait_sleep(&tfull[b], (j >> 1) & 1, a.status, 6, 128, a.spin)) break;
      ptx::tc_fence_after();
      const uint32_t lane_addr = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(b * BN);
      for (int c0 = half * 128; c0 < half * 128 + 128; c0 += 16) {
        float u[16];
        ptx::tmem_ld16(lane_addr + c0, u);
        ptx::tmem_wait_ld();
        if (q0 + c0 >= a.P_eff) continue;  // padding columns (uniform over the warp)
#pragma unroll
        for (int jj = 0; jj < 16; ++jj) {
          const int q = q0 + c0 + jj;
          if (q < a.P_eff) {
            const float U = u[jj] * qs;
            const float slice = live ? U / Tr : 0.0f;
            if (a.u) {  // sorted mode: a coalesced store per column (lanes: rotations)
              if (rok) a.u[(size_t)q * a.ldu + r] = Tr * slice;
            } else {
              tc_insert(a, Rm, live, __ldg(a.cx + q), __ldg(a.cy + q), __ldg(a.cz + q),
                        Tr * slice, Tr);
            }
          }
        }
      }
      // this warp's reads of buffer b are complete: hand it back to rank 0's MMA warp
      ptx::tc_fence_before();
      __syncwarp();
      if (lane == 0) {
        if (back)
          ptx::mbar_arrive_cluster(ptx::mapa_shared(ptx::smem_u32(&tempty[b]), 0));
        else
          ptx::mbar_arrive(&tempty[b]);
      }
    }
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::cluster_sync();  // the pair's MMAs and barrier traffic are over in both CTAs
  if (threadIdx.x == 32) ptx::settle_after_timeout(a.status);
  __syncthreads();
  if (warp == 1) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc_pair(tmem, 512);
  }
}

// ------------------------------------------------------------ host -------
struct TcState {
  CUtensorMap mK, mK2h, mK2l, mQh, mQl, mKt;
  CUtensorMap mKt128;  // K^T in 128-row boxes (pair M-step halves)
  CUtensorMap rot[6];    // M', MS, Gh, Gl, Hh, Hl: 128-row boxes
  CUtensorMap gl64;        // G lo: 64-row boxes (CTA-pair halves)
  CUtensorMap mLh, mLl;  // true Poisson: log-slices hi / lo (in Gh, Gl), 256-row boxes
  __half *Mp, *MSh, *Gh, *Gl, *Hh, *Hl;
  int* status;
};

static TcState* state(emc_plan* p) { return (TcState*)p->tc; }

int tc_bind(emc_plan* p) {
  emc_ctx* ctx = p->ctx;
  if (!p->counts_integer || (!p->counts_fp16_exact && !p->counts_round))
    return fail(ctx, EMC_ERR_UNSUPPORTED,
                "mixed precision needs integer counts in [0, 2048] (exact in FP16), or in [0, "
                "65504] with EMC_OPT_COUNTS_ROUND (largest count here %d)", p->count_max);
  {
    // K^2 scale: the largest FP16 count squared times k2_scale stays below 2^15
    const float km = __half2float(__float2half_rn((float)p->count_max));
    int e = 7;
    while (km * km * std::ldexp(1.0f, -e) > 32768.0f) ++e;
    p->k2_scale = std::ldexp(1.0f, -e);
  }
  if (p->d.diff != EMC_DIFF_POISSON && p->d.diff != EMC_DIFF_TRUE_POISSON)
    return fail(ctx, EMC_ERR_UNSUPPORTED,
                "mixed precision implements the poisson and true-poisson likelihoods");
  const bool pois = p->d.diff == EMC_DIFF_TRUE_POISSON;
  const int N = p->d.n_images, Np = p->Np, Kp = p->Kp, Rp = p->Rp;
  int rc = EMC_OK;
  if (!p->tc) {
    TcState* st = new TcState();
    std::memset(st, 0, sizeof(*st));
    p->tc = st;
    const size_t pk = (size_t)Np * Kp, rk = (size_t)Rp * Kp;
    if (!rc) rc = plan_alloc(p, (void**)&p->Kh, pk * 2);
    if (!rc) rc = plan_alloc(p, (void**)&p->KhT, pk * 2);
    if (!pois) {
      if (!rc) rc = plan_alloc(p, (void**)&p->K2hi, pk * 2);
      if (!rc) rc = plan_alloc(p, (void**)&p->K2lo, pk * 2);
      if (!rc) rc = plan_alloc(p, (void**)&p->k2lo_any, (size_t)(Np / 128) * (Kp / 32));
      if (!rc) rc = plan_alloc(p, (void**)&p->glo_kb, sizeof(int) * (size_t)(Np / 128 + 1));
    }
    __half** rot_ops[6] = {&st->Gh, &st->Gl, &st->Mp, &st->MSh, &st->Hh, &st->Hl};
    for (int j = 0; j < (pois ? 2 : 6); ++j) {
      if (!rc) rc = plan_alloc(p, (void**)rot_ops[j], rk * 2);
      // rows R..Rp stay zero: the expand writes the operands of rows < R
      if (!rc) EMC_CUDA(ctx, cudaMemsetAsync(*rot_ops[j], 0, rk * 2, ctx->stream));
    }
    if (!rc) rc = plan_alloc(p, (void**)&p->Qh, (size_t)Rp * Np * 2);
    if (!rc) rc = plan_alloc(p, (void**)&p->qscale, (size_t)Rp * 4);
    if (!rc) rc = plan_alloc(p, (void**)&st->status, 64);
    if (rc) return rc;
    EMC_CUDA(ctx, cudaMemsetAsync(st->status, 0, 64, ctx->stream));
    EMC_CUDA(ctx, cudaMemsetAsync(p->Qh, 0, (size_t)Rp * Np * 2, ctx->stream));
    // tensor maps (fixed addresses for the plan's lifetime)
    if (!rc) rc = make_map(ctx, &st->mK, p->Kh, Np, Kp, 128, 32);
    if (pois) {
      if (!rc) rc = make_map(ctx, &st->mLh, st->Gh, Rp, Kp, 256, 32);
      if (!rc) rc = make_map(ctx, &st->mLl, st->Gl, Rp, Kp, 256, 32);
    } else {
      if (!rc) rc = make_map(ctx, &st->mK2h, p->K2hi, Np, Kp, 128, 32);
      if (!rc) rc = make_map(ctx, &st->mK2l, p->K2lo, Np, Kp, 128, 32);
      const __half* ro[6] = {st->Mp, st->MSh, st->Gh, st->Gl, st->Hh, st->Hl};
      for (int j = 0; j < 6 && !rc; ++j) rc = make_map(ctx, &st->rot[j], ro[j], Rp, Kp, 128, 32);
      if (!rc) rc = make_map(ctx, &st->gl64, st->Gl, Rp, Kp, 64, 32);
    }
    if (!rc) rc = make_map(ctx, &st->mQh, p->Qh, Rp, Np, 128, 64);
    if (!rc) rc = make_map(ctx, &st->mKt, p->KhT, Kp, Np, 256, 64);
    if (!rc) rc = make_map(ctx, &st->mKt128, p->KhT, Kp, Np, 128, 64);
    if (rc) return rc;
    EMC_CUDA(ctx, cudaFuncSetAttribute(tc_estep_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       es::SMEM_BYTES));
    EMC_CUDA(ctx, cudaFuncSetAttribute(tc_estep_pair_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       es2::SMEM_BYTES));
    EMC_CUDA(ctx, cudaFuncSetAttribute(tc_estep_pois_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, ep::SMEM_BYTES));
    EMC_CUDA(ctx, cudaFuncSetAttribute(tc_mstep_kernel<0>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       MsRing<0>::kSmem));
    EMC_CUDA(ctx, cudaFuncSetAttribute(tc_mstep_kernel<1>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       MsRing<1>::kSmem));
    EMC_CUDA(ctx, cudaFuncSetAttribute(tc_mstep_pair_kernel<0>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       ms2::Ring<0>::kSmem));
    EMC_CUDA(ctx, cudaFuncSetAttribute(tc_mstep_pair_kernel<1>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       ms2::Ring<1>::kSmem));
  }
  if (p->mstep_q_lo && (rc = tc_ensure_qlo(p))) return rc;
  // counts already in FP16 from the bind's pattern pass when its scale holds
  return tc_pattern_side(p, nullptr, p->fused_k2_scale == p->k2_scale);
}

// FP16 pattern operands for the pattern order perm (position -> input
// pattern; nullptr: input order).
// counts_done: pattern_ops_kernel already wrote Kh / K2h / K2l at the
// current scale (rows < N; the padding rows stay zero from the first bind).
int tc_pattern_side(emc_plan* p, const int* d_perm, bool counts_done) {
  emc_ctx* ctx = p->ctx;
  const int N = p->d.n_images, Np = p->Np, Kp = p->Kp;
  const bool pois = p->d.diff == EMC_DIFF_TRUE_POISSON;
  int rc;
  if (!counts_done) {
    tc_pattern_ops_kernel<<<(unsigned)Np * (unsigned)ceil_div(Kp, 256), 256, 0, ctx->stream>>>(
        p->images, p->pix, p->n2, N, Kp, p->Kh, pois ? nullptr : p->K2hi, p->K2lo, d_perm,
        p->k2_scale);
    if ((rc = after_launch(ctx, "tc_pattern_ops_kernel"))) return rc;
  }
  if (!pois) tc_k2lo_flags_kernel<<<dim3(Kp / 32, Np / 128), 256, 0, ctx->stream>>>(p->K2lo, Kp, p->k2lo_any,
                                                                         Kp / 32);
  if ((rc = after_launch(ctx, "tc_k2lo_flags_kernel"))) return rc;
  if (!pois && (rc = tc_glo_extent(p))) return rc;
  transpose_h_kernel<<<dim3(ceil_div(Kp, 64), ceil_div(Np, 64)), dim3(32, 8), 0, ctx->stream>>>(
      p->Kh, Np, Kp, p->KhT);
  return after_launch(ctx, "transpose_h_kernel");
}

int* tc_status(emc_plan* p) { return p->tc ? state(p)->status : nullptr; }

int tc_glo_extent(emc_plan* p) {
  if (!p->glo_kb) return EMC_OK;  // true Poisson: no G operand
  emc_ctx* ctx = p->ctx;
  const int nkb = p->Kp / es::BK, n_pt = p->Np / es::BM;
  EMC_CUDA(ctx, cudaMemsetAsync(p->glo_kb, 0, sizeof(int) * (size_t)(n_pt + 1), ctx->stream));
  tc_glo_extent_kernel<<<ceil_div(p->d.n_images, 8), 256, 0, ctx->stream>>>(
      p->Kh, p->Kp, nkb, p->d.n_images, (float)p->glo_tail_ppm * 1e-6f, p->glo_kb);
  return after_launch(ctx, "tc_glo_extent_kernel");
}

// The FP16 lo half of the M-step operand and its tensor map, allocated the
// first time an M-step that uses it is requested (it is never read otherwise).
int tc_ensure_qlo(emc_plan* p) {
  if (!p->tc || p->Ql) return EMC_OK;
  emc_ctx* ctx = p->ctx;
  const size_t bytes = (size_t)p->Rp * p->Np * 2;
  int rc = plan_alloc(p, (void**)&p->Ql, bytes);
  if (rc) return rc;
  EMC_CUDA(ctx, cudaMemsetAsync(p->Ql, 0, bytes, ctx->stream));
  return make_map(ctx, &state(p)->mQl, p->Ql, p->Rp, p->Np, 128, 64);
}

// The likelihood kernels over tiles [first, first + count) of the full
// (pattern tile, rotation tile) grid in the order `raster`, or over the plan's
// pruned tile list (full == false and a list exists; first/count ignored).
static int estep_pois_launch(emc_plan* p, int raster, int first, int count, bool full) {
  emc_ctx* ctx = p->ctx;
  TcState* st = state(p);
  TcEstepPoisArgs a;
  a.N = p->d.n_images;
  a.R = p->d.n_rot;
  a.n_pt = p->Np / ep::BM;
  a.n_rt = ceil_div(p->Rp, ep::BN);
  a.nkb = p->Kp / ep::BK;
  a.raster = raster;
  a.tiles = full ? nullptr : p->prune_tiles;
  a.n_part = p->n_rt;
  a.rot_ssum = p->rot_ssum;
  a.rotw = p->rotw;
  a.Ksum = p->Ksum;
  a.cnorm = p->cnorm;
  a.known_intensity = p->d.known_intensity;
  a.L = p->L;
  a.PHI = p->PHI;
  a.part = p->part;
  a.status = st->status;
  a.spin = p->debug_spin ? p->debug_spin : ptx::kSpinLimit;
  const int total = a.n_pt * a.n_rt;
  first = a.tiles ? 0 : std::max(0, std::min(first, total));
  const int grid = a.tiles ? p->prune_n_tiles : std::min(total - first, count);
  a.tile0 = first;
  if (grid == 0) return EMC_OK;
  tc_estep_pois_kernel<<<grid, ep::THREADS, ep::SMEM_BYTES, ctx->stream>>>(st->mK, st->mLh,
                                                                           st->mLl, a);
  return after_launch(ctx, "tc_estep_pois_kernel");
}

static int estep_launch(emc_plan* p, int raster, int first, int count, bool full) {
  if (p->d.diff == EMC_DIFF_TRUE_POISSON) return estep_pois_launch(p, raster, first, count, full);
  emc_ctx* ctx = p->ctx;
  TcState* st = state(p);
  TcEstepArgs a;
  a.N = p->d.n_images;
  a.R = p->d.n_rot;
  a.Kp = p->Kp;
  a.n_pt = p->Np / es::BM;
  a.n_rt = p->Rp / es::BN;
  a.nkb = p->Kp / es::BK;
  a.raster = raster;
  // auto: G lo always; H lo too when the intensity is known (phi = 1 leaves
  // the C = K^2 . H term unbalanced, and its rounding shows in the likelihood)
  a.gh_lo = p->estep_gh_lo >= 0 ? p->estep_gh_lo : (p->d.known_intensity ? 3 : 1);
  a.tiles = full ? nullptr : p->prune_tiles;
  a.k2lo_any = p->k2lo_any;
  a.glo_kb = p->glo_kb;
  a.k2_inv = 1.0f / p->k2_scale;
  a.rot_cnt = p->rot_cnt;
  a.rot_A = p->rot_A;
  a.rotw = p->rotw;
  a.cnorm = p->cnorm;
  a.sigma = p->sigma_dev;
  a.known_intensity = p->d.known_intensity;
  a.L = p->L;
  a.PHI = p->PHI;
  a.part = p->part;
  a.bad = p->flags + 4;
  a.status = st->status;
  a.spin = p->debug_spin ? p->debug_spin : ptx::kSpinLimit;
  const CUtensorMap* rm = st->rot;
  if (p->estep_pair && !a.tiles && !(a.gh_lo & 2)) {
    // CTA pairs: tiles are (pattern-tile pair, rotation tile)
    const int total = ((a.n_pt + 1) / 2) * a.n_rt;
    first = std::max(0, std::min(first, total));
    const int pairs = std::min(total - first, count);
    a.tile0 = first;
    if (pairs == 0) return EMC_OK;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(2 * pairs);
    cfg.blockDim = dim3(es::THREADS);
    cfg.dynamicSmemBytes = es2::SMEM_BYTES;
    cfg.stream = ctx->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, tc_estep_pair_kernel, st->mK, st->mK2h, st->mK2l,
                                             rm[0], rm[1], rm[2], st->gl64, rm[4], a);
    if (e == cudaSuccess) return after_launch(ctx, "tc_estep_pair_kernel");
    // a refused launch configuration (a GPU or partition that cannot
    // co-schedule the pairs) is not a sticky error: single CTAs from now on
    (void)cudaGetLastError();
    p->estep_pair = 0;
    first *= 2;  // about the same part of the grid, in single-CTA tiles
    count = count > INT_MAX / 2 ? INT_MAX : 2 * count;
  }
  const int total = a.n_pt * a.n_rt;
  first = a.tiles ? 0 : std::max(0, std::min(first, total));
  const int grid = a.tiles ? p->prune_n_tiles : std::min(total - first, count);
  a.tile0 = first;
  if (grid == 0) return EMC_OK;
  tc_estep_kernel<<<grid, es::THREADS, es::SMEM_BYTES, ctx->stream>>>(
      st->mK, st->mK2h, st->mK2l, rm[0], rm[1], rm[2], rm[3], rm[4], rm[5], a);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(ctx, e, "tc_estep_kernel launch");
  return after_launch(ctx, "tc_estep_kernel");
}

// The rotation operands are written by the expand (rot_ops_store4).
int tc_estep(emc_plan* p) { return estep_launch(p, p->estep_raster, 0, INT_MAX, false); }

RotOps tc_rot_ops(emc_plan* p) {
  RotOps o;
  if (!p->tc) return o;
  TcState* st = state(p);
  o.flags = p->flags;
  o.Gh = st->Gh;
  o.Gl = st->Gl;
  if (p->d.diff == EMC_DIFF_TRUE_POISSON) {
    o.logs = 1;
  } else {
    // the lo planes only where the likelihood reads them (EMC_OPT_ESTEP_GHLO;
    // auto: G lo, and H lo when the intensity is known)
    const int gh = p->estep_gh_lo >= 0 ? p->estep_gh_lo : (p->d.known_intensity ? 3 : 1);
    o.Mp = st->Mp;
    o.MSh = st->MSh;
    o.Hh = st->Hh;
    o.Gl = (gh & 1) ? st->Gl : nullptr;
    o.Hl = (gh & 2) ? st->Hl : nullptr;
    if (o.Gl && p->glo_kb) o.gl_end = p->glo_kb + p->Np / es::BM;
  }
  return o;
}

// The likelihood lo terms in force: bit 0 G lo, bit 1 H lo (auto: H lo when
// the intensity is known).
static int estep_gh_lo(const emc_plan* p) {
  return p->estep_gh_lo >= 0 ? p->estep_gh_lo : (p->d.known_intensity ? 3 : 1);
}

// Full scans of the reference likelihood run on CTA pairs unless switched
// off or H lo is needed (the pair kernel has no H lo slot).
static bool estep_uses_pair(const emc_plan* p) {
  return p->estep_pair && p->d.diff != EMC_DIFF_TRUE_POISSON && !(estep_gh_lo(p) & 2);
}

// One timed launch of the likelihood kernel over tiles [first, first + count)
// of the order `raster` (CUDA events on the plan's stream; synchronises).  The
// rotation operands are those of the last expansion.
int tc_time_estep(emc_plan* p, int raster, int first, int count, float* ms) {
  emc_ctx* ctx = p->ctx;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  EMC_CUDA(ctx, cudaEventCreate(&e0));
  cudaError_t ce = cudaEventCreate(&e1);
  int rc = EMC_OK;
  if (ce == cudaSuccess) ce = cudaEventRecord(e0, ctx->stream);
  if (ce == cudaSuccess && !(rc = estep_launch(p, raster, first, count, true)))
    ce = cudaEventRecord(e1, ctx->stream);
  if (ce == cudaSuccess && !rc) ce = cudaEventSynchronize(e1);
  if (ce == cudaSuccess && !rc) ce = cudaEventElapsedTime(ms, e0, e1);
  if (ce != cudaSuccess && !rc) rc = cuda_fail(ctx, ce, "likelihood timing");
  cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  return rc;
}

// Units of the full likelihood grid as estep_launch counts them: tiles, or
// CTA-pair tiles for the pair kernel.
int tc_estep_tiles(emc_plan* p) {
  const int n_pt = p->Np / 128;
  if (p->d.diff == EMC_DIFF_TRUE_POISSON) return n_pt * ceil_div(p->Rp, ep::BN);
  return (estep_uses_pair(p) ? (n_pt + 1) / 2 : n_pt) * (p->Rp / es::BN);
}

// Raster autotuner.  The likelihood kernel streams two operand panels per
// CTA (the pattern tile's and the rotation tile's, 128 rows x the compacted
// pixel count each); which CTAs run side by side decides how often a panel
// is served from L2 rather than HBM, and the best order depends on the panel
// length and the tile counts: on 256^3 workloads (51,020 pixels) groups of 4
// rotation tiles run at 5.7 ms per 1,000 tiles while groups of 8 swing
// between 5.5 and 10.3 ms depending on where in the grid they are timed; at
// 128^3 all orders are within 5 %.  Candidates: groups of 2..16 rotation
// tiles, or of 8..76 pattern tiles.  Each is timed on two windows of `waves`
// x SM-count tiles inside the grid (at 30 % and 65 % of its order; the whole
// grid when it is smaller) and scored by the slower window, so an order that
// is fast only at times loses to a steady one.  The rotation operands are
// those of the last expansion; the timed launches overwrite
// responsibilities and scaling of the tiles they cover.
int tc_autotune(emc_plan* p, int waves, int* best, float* best_ms) {
  emc_ctx* ctx = p->ctx;
  int rc = EMC_OK;
  const bool pois = p->d.diff == EMC_DIFF_TRUE_POISSON;
  const bool pair = !pois && estep_uses_pair(p);
  const int n_pt = pair ? (p->Np / 128 + 1) / 2 : p->Np / 128;
  const int n_rt = pois ? ceil_div(p->Rp, ep::BN) : p->Rp / es::BN;
  const int total = n_pt * n_rt;
  const int count = std::min(total, std::max(1, waves) * (pair ? ctx->sm_count / 2 : ctx->sm_count));
  std::vector<int> firsts;
  if (count >= total) {
    firsts.push_back(0);
  } else {
    for (double f : {0.30, 0.65})
      firsts.push_back(std::min(total - count, (int)(f * total)));
  }
  std::vector<int> cand;
  for (int g : {8, 2, 4, 16, -8, -19, -38, -76}) {
    const int c = g > 0 ? std::min(g, n_rt) : -std::min(-g, n_pt);
    if (std::find(cand.begin(), cand.end(), c) == cand.end()) cand.push_back(c);
  }
  std::vector<float> t(cand.size(), 0.0f);
  for (size_t j = 0; j < cand.size() && !rc; ++j) {
    for (int first : firsts) {
      float ms = 0.0f;
      if ((rc = tc_time_estep(p, cand[j], first, count, &ms))) break;
      t[j] = std::max(t[j], ms);
    }
  }
  if (rc) return rc;
  // the default order (first candidate) unless another is 2 % faster: orders
  // that tie in time differ in HBM traffic (at 128^3 from 63 to 217 GB per
  // launch), and the default one reads the least there
  size_t b = 0;
  for (size_t j = 1; j < cand.size(); ++j)
    if (t[j] < t[b]) b = j;
  if (t[0] <= 1.02f * t[b]) b = 0;
  int raster = cand[b];
  float raster_ms = t[b];
  // tile shape: CTA pairs (256 patterns x 128 rotations, 256-row MMAs) or
  // single CTAs (128 x 128).  The single-CTA kernel, in its default order,
  // is timed on the same windows in its own tile units (twice the tiles,
  // the same (pattern, rotation) work); it replaces the pairs when 2 %
  // faster.  The shapes' results differ only by the FP32 rounding of the
  // accumulation (1e-6 relative).
  if (pair) {
    p->estep_pair = 0;
    const int s_total = (p->Np / 128) * n_rt;
    const int s_count = std::min(s_total, 2 * count);
    float ts = 0.0f;
    for (int first : firsts) {
      float ms = 0.0f;
      if ((rc = tc_time_estep(p, 8, std::min(2 * first, s_total - s_count), s_count, &ms))) break;
      ts = std::max(ts, ms);
    }
    if (!rc && ts < 0.98f * raster_ms) {
      raster = 8;
      raster_ms = ts;
    } else {
      p->estep_pair = 1;
    }
    if (rc) return rc;
  }
  p->estep_raster = raster;
  if (best) *best = raster;
  if (best_ms) *best_ms = raster_ms;
  return EMC_OK;
}


int tc_mstep(emc_plan* p, float* model, float* weight) {
  emc_ctx* ctx = p->ctx;
  TcState* st = state(p);
  TcMstepArgs a;
  a.R = p->d.n_rot;
  a.Kp = p->Kp;
  a.Np = p->Np;
  a.P_eff = p->P_eff;
  a.n_qt = p->Kp / ms::BN + (p->Kp % ms::BN ? 1 : 0);
  a.n_rt = p->Rp / ms::BM;
  a.nkb = p->Np / ms::BK;
  a.raster = p->mstep_raster;
  a.T = p->T;
  a.qscale = p->qscale;
  a.rot = p->rot;
  a.cx = p->cx;
  a.cy = p->cy;
  a.cz = p->cz;
  a.side = p->d.side;
  a.interp = p->d.interp;
  a.deterministic = p->d.insert_mode == EMC_INSERT_DETERMINISTIC;
  a.model = model;
  a.weight = weight;
  a.fix_m = p->fix_m;
  a.fix_w = p->fix_w;
  a.acc2 = p->acc2;
  a.q_lo = p->mstep_q_lo;
  a.aggregate = p->mstep_aggregate;
  a.kb_off = p->prune_kb_off;
  a.kb_list = p->prune_kb_list;
  a.fix_scale = reinterpret_cast<const float2*>(p->red + kRedFixScale);
  a.u = p->d.insert_mode == EMC_INSERT_SORTED ? p->ins_u : nullptr;
  a.ldu = p->ins_ldu;
  a.status = st->status;
  a.spin = p->debug_spin ? p->debug_spin : ptx::kSpinLimit;
  a.n_tiles = a.n_qt * a.n_rt;
  if (p->mstep_pair && !a.kb_off && a.n_rt > 1 && ctx->sm_count >= 2) {
    // CTA pairs, persistent: one cluster per two SMs
    const int tiles = ((a.n_rt + 1) / 2) * a.n_qt;
    const int clusters = std::min(tiles, ctx->sm_count / 2);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(2 * clusters);
    cfg.blockDim = dim3(ms::THREADS);
    cfg.dynamicSmemBytes = a.q_lo ? ms2::Ring<1>::kSmem : ms2::Ring<0>::kSmem;
    cfg.stream = ctx->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e =
        a.q_lo ? cudaLaunchKernelEx(&cfg, tc_mstep_pair_kernel<1>, st->mQh, st->mQl, st->mKt128, a)
               : cudaLaunchKernelEx(&cfg, tc_mstep_pair_kernel<0>, st->mQh, st->mQl, st->mKt128, a);
    if (e == cudaSuccess) return after_launch(ctx, "tc_mstep_pair_kernel");
    // a refused launch configuration is not a sticky error: single CTAs from now on
    (void)cudaGetLastError();
    p->mstep_pair = 0;
  }
  const int grid = std::min(a.n_tiles, ctx->sm_count);
  if (a.q_lo)
    tc_mstep_kernel<1><<<grid, ms::THREADS, MsRing<1>::kSmem, ctx->stream>>>(st->mQh, st->mQl,
                                                                              st->mKt, a);
  else
    tc_mstep_kernel<0><<<grid, ms::THREADS, MsRing<0>::kSmem, ctx->stream>>>(st->mQh, st->mQl,
                                                                              st->mKt, a);
  return after_launch(ctx, "tc_mstep_kernel");
}

void tc_free(emc_plan* p) {
  delete state(p);
  p->tc = nullptr;
}

// ------------------------------------------------------- self-test -------
// One CTA computes D[128 x BN] = A[128 x K] B[BN x K]^T with the same TMA,
// shared-memory descriptor, MMA and TMEM-load code as the iteration kernels,
// for the tile shapes they use: (BN = 128, 64B swizzle, 32-wide k-blocks)
// and (BN = 256, 128B swizzle, 64-wide k-blocks).  Single-stage pipeline.
template <int BN, int BK>
__global__ void __launch_bounds__(128, 1)
    tc_gemm_selftest_kernel(const __grid_constant__ CUtensorMap mA,
                            const __grid_constant__ CUtensorMap mB, int K, float* D, int* status) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  constexpr int A_BYTES = 128 * BK * 2, B_BYTES = BN * BK * 2;
  constexpr uint32_t SW = BK == 64 ? 2 : 4;
  constexpr uint32_t SBO = BK * 2 * 8;
  uint64_t* full = (uint64_t*)(smem + A_BYTES + B_BYTES);
  uint64_t* done = full + 1;
  uint32_t* tslot = (uint32_t*)(done + 1);
  const int warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    ptx::mbar_init(full, 1);
    ptx::mbar_init(done, 1);
    ptx::fence_mbar_init();
  }
  if (warp == 0) {
    ptx::tmem_alloc(tslot, BN);
    ptx::tmem_relinquish();
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem = *tslot;
  bool ok = true;
  for (int kb = 0; kb < K / BK && ok; ++kb) {
    if (threadIdx.x == 0) {
      ptx::mbar_arrive_expect_tx(full, A_BYTES + B_BYTES);
      ptx::tma_load_2d(smem, &mA, kb * BK, 0, full);
      ptx::tma_load_2d(smem + A_BYTES, &mB, kb * BK, 0, full);
    }
    ok = ptx::mbar_wait(full, kb & 1, status, 0);
    ptx::tc_fence_after();
    if (threadIdx.x == 0 && ok) {
      const uint32_t base = ptx::smem_u32(smem);
      for (int ks = 0; ks < BK / 16; ++ks)
        ptx::mma_f16(tmem, ptx::smem_desc(base + ks * 32, SBO, SW),
                     ptx::smem_desc(base + A_BYTES + ks * 32, SBO, SW), ptx::idesc_f16(128, BN),
                     (kb | ks) ? 1u : 0u);
      ptx::mma_commit(done);
    }
    if (ok) ok = ptx::mbar_wait(done, kb & 1, status, 1);
    ptx::tc_fence_after();
    __syncthreads();
  }
  if (ok) {
    const int q = warp & 3;
    const uint32_t la = tmem + ((uint32_t)(q * 32) << 16);
    const int row = q * 32 + (threadIdx.x & 31);
    for (int c0 = 0; c0 < BN; c0 += 16) {
      float v[16];
      ptx::tmem_ld16(la + c0, v);
      ptx::tmem_wait_ld();
      for (int j = 0; j < 16; ++j) D[(size_t)row * BN + c0 + j] = v[j];
    }
  }
  ptx::tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc(tmem, BN);
  }
}

}  // namespace emc

// Diagnostic: D[128 x n] = A[128 x k] B[n x k]^T (FP16 in, FP32 out, device
// pointers) through the tcgen05 building blocks; n = 128 uses the E-step's
// 64B-swizzled 32-wide k-blocks, n = 256 the M-step's 128B-swizzled 64-wide
// k-blocks.  k must be a multiple of the k-block.
extern "C" int emc_tc_gemm_selftest(emc_ctx* ctx, const void* d_a, const void* d_b, float* d_d,
                                    int n, int k) {
  using namespace emc;
  EMC_CHECK_CTX(ctx);
  EMC_REQUIRE(ctx, d_a && d_b && d_d, "tc_gemm_selftest: null pointer");
  EMC_REQUIRE(ctx, n == 128 || n == 256, "tc_gemm_selftest: n must be 128 or 256");
  const int bk = n == 128 ? 32 : 64;
  EMC_REQUIRE(ctx, k > 0 && k % bk == 0, "tc_gemm_selftest: k %% %d != 0", bk);
  CUtensorMap mA, mB;
  int rc = make_map(ctx, &mA, d_a, 128, k, 128, bk);
  if (!rc) rc = make_map(ctx, &mB, d_b, n, k, n, bk);
  if (rc) return rc;
  int* status = nullptr;
  EMC_CUDA(ctx, cudaMallocAsync((void**)&status, sizeof(int), ctx->stream));
  EMC_CUDA(ctx, cudaMemsetAsync(status, 0, sizeof(int), ctx->stream));
  const int smem = 128 * bk * 2 + n * bk * 2 + 1024 + 1024;
  if (n == 128) {
    EMC_CUDA(ctx, cudaFuncSetAttribute(tc_gemm_selftest_kernel<128, 32>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    tc_gemm_selftest_kernel<128, 32><<<1, 128, smem, ctx->stream>>>(mA, mB, k, d_d, status);
  } else {
    EMC_CUDA(ctx, cudaFuncSetAttribute(tc_gemm_selftest_kernel<256, 64>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    tc_gemm_selftest_kernel<256, 64><<<1, 128, smem, ctx->stream>>>(mA, mB, k, d_d, status);
  }
  if ((rc = after_launch(ctx, "tc_gemm_selftest_kernel"))) return rc;
  int h = 0;
  EMC_CUDA(ctx, cudaMemcpyAsync(&h, status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  EMC_CUDA(ctx, cudaFreeAsync(status, ctx->stream));
  EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (h) return fail(ctx, EMC_ERR_TIMEOUT, "tc_gemm_selftest: wait timed out (0x%x)", h);
  return EMC_OK;
}
