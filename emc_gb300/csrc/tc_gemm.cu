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
constexpr float kK2Scale = 1.0f / 128.0f;  // K^2 * 2^-7 <= 2^15 for counts <= 2048
constexpr float kMSScale = 1.0f / 256.0f;  // (M' S) * 2^-8 keeps slices below 2^24 in range

// Counts -> FP16 operands, rows of Kp (patterns padded to Np with zeros):
// Kh = k, K2h + K2l = k^2 * 2^-7 exactly.
__global__ void tc_pattern_ops_kernel(const float* __restrict__ images, const int* __restrict__ pix,
                                      int n2, int N, int Kp, __half* __restrict__ Kh,
                                      __half* __restrict__ K2h, __half* __restrict__ K2l) {
  const int i = blockIdx.y;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= Kp) return;
  float k = 0.0f;
  if (i < N) {
    const int p = pix[q];
    if (p >= 0) k = __ldg(images + (size_t)i * n2 + p);
  }
  const float k2 = k * k * kK2Scale;  // exact: k^2 < 2^22
  const __half hi = __float2half_rn(k2);
  const __half lo = __float2half_rn(k2 - __half2float(hi));
  const size_t o = (size_t)i * Kp + q;
  Kh[o] = __float2half_rn(k);
  K2h[o] = hi;
  K2l[o] = lo;
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

// [rows][cols] -> [cols][rows], FP16, 32x32 tiles.
__global__ void transpose_h_kernel(const __half* __restrict__ in, int rows, int cols,
                                   __half* __restrict__ out) {
  __shared__ __half t[32][33];
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int r = r0 + y, c = c0 + threadIdx.x;
    t[y][threadIdx.x] = (r < rows && c < cols) ? in[(size_t)r * cols + c] : __float2half_rn(0.f);
  }
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int c = c0 + y, r = r0 + threadIdx.x;
    if (c < cols && r < rows) out[(size_t)c * rows + r] = t[threadIdx.x][y];
  }
}

// ---------------------------------------------------- rotation operands --
constexpr float kPoisCf = 0.02f;

// From the compacted slices S [Rp][Kp] (FP32): the six FP16 rotation-side
// operands, each [Rp][Kp]: M' = [s > 1e-10], (M' s) 2^-8 hi, G = [s > 0]
// s/(s+c) hi/lo, H = [s > 0] /(s+c) hi/lo.  flags[0] |= 4 when a slice value
// does not fit the scaled FP16 range.
__global__ void tc_rot_ops_kernel(const float* __restrict__ S, size_t n, __half* __restrict__ Mp,
                                  __half* __restrict__ MSh, __half* __restrict__ Gh,
                                  __half* __restrict__ Gl, __half* __restrict__ Hh,
                                  __half* __restrict__ Hl, int* __restrict__ flags) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride) {
    const float s = S[e];
    // (double)s > 1e-10 of the reference, as a float test: 1e-10f is the
    // first float above 1e-10, so both agree for every float s
    const bool mp = s >= 1e-10f;
    const bool m = s > 0.0f;
    const float ms = mp ? s * kMSScale : 0.0f;
    if (ms > 60000.0f) atomicOr(flags, 4);
    const float h = m ? 1.0f / (s + kPoisCf) : 0.0f;
    const float g = m ? s * h : 0.0f;
    const __half gh = __float2half_rn(g), hh = __float2half_rn(h);
    Mp[e] = __float2half_rn(mp ? 1.0f : 0.0f);
    MSh[e] = __float2half_rn(ms);
    Gh[e] = gh;
    Gl[e] = __float2half_rn(g - __half2float(gh));
    Hh[e] = hh;
    Hl[e] = __float2half_rn(h - __half2float(hh));
  }
}

// ------------------------------------------------------------ E-step -----
namespace es {
constexpr int BM = 128;        // patterns per tile (TMEM lanes)
constexpr int BN = 128;        // rotations per tile
constexpr int BK = 32;         // pixels per stage (64 B rows, 64B swizzle)
constexpr int STAGES = 3;
constexpr int TILE_BYTES = 128 * BK * 2;  // 8 KB, both operand sides
constexpr int NA = 3;          // K, K2h, K2l
constexpr int NB = 6;          // M', MS, Gh, Gl, Hh, Hl
constexpr int STAGE_BYTES = (NA + NB) * TILE_BYTES;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 2048 + 1024;
constexpr int THREADS = 192;
constexpr int GROUP = 8;       // rotation tiles per raster group
}  // namespace es

struct TcEstepArgs {
  int N, R, Kp, n_pt, n_rt, nkb;
  const unsigned char* k2lo_any;  // [n_pt][nkb]
  const float* rot_cnt;
  const float* rot_A;
  const float* rotw;
  const float* cnorm;   // c_i (phi is stored as c_i num/den)
  float inv2s2;         // 1 / (2 sigma^2)
  int known_intensity;
  float* L;
  float* PHI;
  float2* part;
  int* bad;
  int* status;
};

// CL > 1: launched in clusters of CL CTAs that share one rotation tile and
// hold CL consecutive pattern tiles.  Each CTA loads 128/CL rows of every
// rotation-side tile and multicasts them to the whole cluster, so L2 serves
// each rotation-side byte once per cluster instead of once per CTA; every
// CTA's MMA completion is multicast to all empty barriers (arrival count
// CL), so no stage is overwritten before the whole cluster has consumed it.
template <int CL>
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
  uint32_t* tmem_slot = (uint32_t*)(accum + 1);
  float* s_A = (float*)(smem + STAGES * STAGE_BYTES + 256);
  float* s_scale = s_A + BN;
  float* s_lw = s_scale + BN;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // grouped raster over clusters: GROUP rotation tiles share each cluster of
  // CL pattern tiles in turn
  const int member = CL > 1 ? (int)ptx::cluster_ctarank() : 0;
  const int cid = blockIdx.x / CL;
  const int n_ptc = a.n_pt / CL;
  const int per_group = GROUP * n_ptc;
  const int g = cid / per_group, within = cid % per_group;
  const int rt0 = g * GROUP;
  const int gsz = min(GROUP, a.n_rt - rt0);
  const int rt = rt0 + within % gsz;
  const int pt = (within / gsz) * CL + member;
  const int n0 = pt * BM, r0 = rt * BN;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      ptx::mbar_init(&full[s], 1);
      ptx::mbar_init(&empty[s], CL);
    }
    ptx::mbar_init(accum, 1);
    ptx::fence_mbar_init();
  }
  if (threadIdx.x < BN) {
    const int r = r0 + threadIdx.x;
    const float cnt = r < a.R ? a.rot_cnt[r] : 0.0f;
    s_A[threadIdx.x] = r < a.R ? a.rot_A[r] : 0.0f;
    s_scale[threadIdx.x] = cnt > 0.0f ? a.inv2s2 / cnt : -1.0f;  // < 0: invalid rotation
    s_lw[threadIdx.x] = r < a.R ? logf(a.rotw[r]) : 0.0f;
  }
  if (warp == 1) {
    ptx::tmem_alloc(tmem_slot, 512);
    ptx::tmem_relinquish();
  }
  ptx::tc_fence_before();
  __syncthreads();
  if (CL > 1) ptx::cluster_sync();  // peers' barriers exist before any multicast
  ptx::tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const unsigned char* flags = a.k2lo_any + (size_t)pt * a.nkb;
  constexpr uint16_t kAll = (uint16_t)((1u << CL) - 1);
  constexpr int kRows = BN / CL;  // rotation rows each cluster member fetches

  if (warp == 0) {
    // ------------------------------------------------ TMA producer
    if (lane == 0) {
      const CUtensorMap* amap[NA] = {&mK, &mK2h, &mK2l};
      const CUtensorMap* bmap[NB] = {&mMp, &mMS, &mGh, &mGl, &mHh, &mHl};
      for (int kb = 0; kb < a.nkb; ++kb) {
        const int s = kb % STAGES;
        const uint32_t ph = (kb / STAGES) & 1;
        if (!ptx::mbar_wait(&empty[s], ph ^ 1, a.status, 0)) break;
        const bool lo = flags[kb] != 0;
        ptx::mbar_arrive_expect_tx(&full[s], (NA + NB - (lo ? 0 : 1)) * TILE_BYTES);
        unsigned char* st = smem + s * STAGE_BYTES;
        for (int j = 0; j < NA; ++j) {
          if (j == 2 && !lo) continue;
          ptx::tma_load_2d(st + j * TILE_BYTES, amap[j], kb * BK, n0, &full[s]);
        }
        for (int j = 0; j < NB; ++j) {
          if (CL == 1) {
            ptx::tma_load_2d(st + (NA + j) * TILE_BYTES, bmap[j], kb * BK, r0, &full[s]);
          } else {
            // rows member*kRows..+kRows-1 of the tile, to the same offset in every CTA
            ptx::tma_load_2d_multicast(st + (NA + j) * TILE_BYTES + member * kRows * BK * 2,
                                       bmap[j], kb * BK, r0 + member * kRows, &full[s], kAll);
          }
        }
      }
    }
  } else if (warp == 1) {
    // ------------------------------------------------ MMA issuer
    if (lane == 0) {
      constexpr uint32_t idesc = ptx::idesc_f16(BM, BN);
      bool ok = true;
      for (int kb = 0; kb < a.nkb && ok; ++kb) {
        const int s = kb % STAGES;
        const uint32_t ph = (kb / STAGES) & 1;
        if (!ptx::mbar_wait(&full[s], ph, a.status, 1)) {
          ok = false;
          break;
        }
        ptx::tc_fence_after();
        const bool lo = flags[kb] != 0;
        const uint32_t base = ptx::smem_u32(smem + s * STAGE_BYTES);
#pragma unroll
        for (int ks = 0; ks < BK / 16; ++ks) {
          auto d = [&](int j) { return ptx::smem_desc(base + j * TILE_BYTES + ks * 32, 512, 4); };
          const uint64_t aK = d(0), aK2h = d(1), aK2l = d(2);
          const uint64_t bM = d(3), bMS = d(4), bGh = d(5), bGl = d(6), bHh = d(7), bHl = d(8);
          const uint32_t acc = (kb | ks) ? 1u : 0u;
          ptx::mma_f16(tmem + 0, aK2h, bM, idesc, acc);  // num
          if (lo) ptx::mma_f16(tmem + 0, aK2l, bM, idesc, 1);
          ptx::mma_f16(tmem + 128, aK, bMS, idesc, acc);  // den
          ptx::mma_f16(tmem + 256, aK, bGh, idesc, acc);  // B
          ptx::mma_f16(tmem + 256, aK, bGl, idesc, 1);
          ptx::mma_f16(tmem + 384, aK2h, bHh, idesc, acc);  // C
          ptx::mma_f16(tmem + 384, aK2h, bHl, idesc, 1);
          if (lo) ptx::mma_f16(tmem + 384, aK2l, bHh, idesc, 1);
        }
        if (CL == 1)
          ptx::mma_commit(&empty[s]);
        else
          ptx::mma_commit_multicast(&empty[s], kAll);  // frees the stage in every CTA
      }
      ptx::mma_commit(accum);  // fires when every MMA above has completed
    }
  } else {
    // ------------------------------------------------ epilogue (warps 2-5)
    const int quarter = warp & 3;  // TMEM lanes this warp may access
    const int row = quarter * 32 + lane;
    const int n = n0 + row;
    const bool nok = n < a.N;
    const float ci = nok ? a.cnorm[n] : 1.0f;
    float m = -INFINITY, ssum = 0.0f;
    int nbad = 0;
    if (ptx::mbar_wait(accum, 0, a.status, 2)) {
      ptx::tc_fence_after();
      const uint32_t lane_addr = tmem + ((uint32_t)(quarter * 32) << 16);
      for (int c0 = 0; c0 < BN; c0 += 16) {
        float vn[16], vd[16], vb[16], vc[16];
        ptx::tmem_ld16(lane_addr + 0 + c0, vn);
        ptx::tmem_ld16(lane_addr + 128 + c0, vd);
        ptx::tmem_ld16(lane_addr + 256 + c0, vb);
        ptx::tmem_ld16(lane_addr + 384 + c0, vc);
        ptx::tmem_wait_ld();
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int cl = c0 + j;
          const int r = r0 + cl;
          const float num = vn[j] * 128.0f, den = vd[j] * 256.0f;
          const float B = vb[j], Cc = vc[j] * 128.0f;
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
    if (nok) a.part[(size_t)rt * a.N + n] = make_float2(m, ssum);
    if (nbad) atomicAdd(a.bad, nbad);
  }
  ptx::tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc(tmem, 512);
  }
  // peers may still multicast MMA completions to this CTA's empty barriers
  // until their last MMA retires: leave only together
  if (CL > 1) ptx::cluster_sync();
}

// ------------------------------------------------------------ M-step -----
namespace ms {
constexpr int BM = 128;   // rotations per tile (TMEM lanes)
constexpr int BN = 256;   // pixels per tile
constexpr int BK = 64;    // patterns per stage (128 B rows, 128B swizzle)
constexpr int STAGES = 3;
constexpr int A_BYTES = BM * BK * 2;  // 16 KB
constexpr int B_BYTES = BN * BK * 2;  // 32 KB
constexpr int STAGE_BYTES = 2 * A_BYTES + B_BYTES;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 1024 + BM * (int)sizeof(RotMat);
constexpr int THREADS = 192;
constexpr int GROUP = 8;
}  // namespace ms

struct TcMstepArgs {
  int R, Kp, Np, P_eff, n_qt, n_rt, nkb;
  const float* T;
  const float* qscale;  // [R] 2^-e_r
  const float* rot;
  const float *cx, *cy, *cz;
  int side, interp, deterministic;
  float* model;
  float* weight;
  unsigned long long* fix_m;
  unsigned long long* fix_w;
  float2* acc2;
  const double* bounds;
  int q_lo;  // 1: Q hi + lo, 0: Q hi only
  int* status;
};

__device__ __forceinline__ double tc_fixed_scale(double b) {
  return b > 0.0 ? 2305843009213693952.0 / b : 1.0;
}

__device__ __forceinline__ void tc_add(const TcMstepArgs& a, size_t v, float val, float w) {
  if (a.deterministic) {
    atomicAdd(a.fix_m + v, (unsigned long long)__double2ll_rn((double)val * tc_fixed_scale(a.bounds[0])));
    atomicAdd(a.fix_w + v, (unsigned long long)__double2ll_rn((double)w * tc_fixed_scale(a.bounds[1])));
  } else {
    atomicAdd(a.acc2 + v, make_float2(val, w));  // model and weight in one 8-byte atomic
  }
}

__device__ __forceinline__ void tc_insert(const TcMstepArgs& a, const RotMat& R, float x, float y,
                                          float z, float val, float w) {
  const int side = a.side;
  if (a.interp == EMC_INTERP_NEAREST) {
    const long ix = lroundf(voxel_coord(side, rotate_row(R, 0, x, y, z)));
    const long iy = lroundf(voxel_coord(side, rotate_row(R, 1, x, y, z)));
    const long iz = lroundf(voxel_coord(side, rotate_row(R, 2, x, y, z)));
    if (ix < 0 || ix >= side || iy < 0 || iy >= side || iz < 0 || iz >= side) return;
    tc_add(a, ((size_t)iz * side + iy) * side + ix, val, w);
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
      tc_add(a, ((size_t)zi * side + yi) * side + xi, val * f, w * f);
    }
  }
}

__global__ void __launch_bounds__(ms::THREADS, 1)
    tc_mstep_kernel(const __grid_constant__ CUtensorMap mQh, const __grid_constant__ CUtensorMap mQl,
                    const __grid_constant__ CUtensorMap mKt, TcMstepArgs a) {
  using namespace ms;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + STAGES * STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* accum = empty + STAGES;
  uint32_t* tmem_slot = (uint32_t*)(accum + 1);
  RotMat* sR = (RotMat*)(smem + STAGES * STAGE_BYTES + 1024);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int t = blockIdx.x;
  const int per_group = GROUP * a.n_qt;
  const int g = t / per_group, within = t % per_group;
  const int rt0 = g * GROUP;
  const int gsz = min(GROUP, a.n_rt - rt0);
  const int rt = rt0 + within % gsz;
  const int qt = within / gsz;
  const int r0 = rt * BM, q0 = qt * BN;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      ptx::mbar_init(&full[s], 1);
      ptx::mbar_init(&empty[s], 1);
    }
    ptx::mbar_init(accum, 1);
    ptx::fence_mbar_init();
  }
  if (threadIdx.x < BM) {
    const int r = r0 + threadIdx.x;
    if (r < a.R) sR[threadIdx.x] = quat_to_matrix(a.rot + 4 * (size_t)r);
  }
  if (warp == 1) {
    ptx::tmem_alloc(tmem_slot, 256);
    ptx::tmem_relinquish();
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      for (int kb = 0; kb < a.nkb; ++kb) {
        const int s = kb % STAGES;
        const uint32_t ph = (kb / STAGES) & 1;
        if (!ptx::mbar_wait(&empty[s], ph ^ 1, a.status, 4)) break;
        ptx::mbar_arrive_expect_tx(&full[s], STAGE_BYTES - (a.q_lo ? 0 : A_BYTES));
        unsigned char* st = smem + s * STAGE_BYTES;
        ptx::tma_load_2d(st, &mQh, kb * BK, r0, &full[s]);
        if (a.q_lo) ptx::tma_load_2d(st + A_BYTES, &mQl, kb * BK, r0, &full[s]);
        ptx::tma_load_2d(st + 2 * A_BYTES, &mKt, kb * BK, q0, &full[s]);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = ptx::idesc_f16(BM, BN);
      for (int kb = 0; kb < a.nkb; ++kb) {
        const int s = kb % STAGES;
        const uint32_t ph = (kb / STAGES) & 1;
        if (!ptx::mbar_wait(&full[s], ph, a.status, 5)) break;
        ptx::tc_fence_after();
        const uint32_t base = ptx::smem_u32(smem + s * STAGE_BYTES);
#pragma unroll
        for (int ks = 0; ks < BK / 16; ++ks) {
          const uint64_t dQh = ptx::smem_desc(base + ks * 32, 1024, 2);
          const uint64_t dQl = ptx::smem_desc(base + A_BYTES + ks * 32, 1024, 2);
          const uint64_t dK = ptx::smem_desc(base + 2 * A_BYTES + ks * 32, 1024, 2);
          ptx::mma_f16(tmem, dQh, dK, idesc, (kb | ks) ? 1u : 0u);
          if (a.q_lo) ptx::mma_f16(tmem, dQl, dK, idesc, 1u);
        }
        ptx::mma_commit(&empty[s]);
      }
      ptx::mma_commit(accum);
    }
  } else {
    const int quarter = warp & 3;
    const int rl = quarter * 32 + lane;
    const int r = r0 + rl;
    const bool rok = r < a.R;
    const float Tr = rok ? a.T[r] : 0.0f;
    const float qs = rok ? a.qscale[r] : 0.0f;
    const bool live = rok && Tr > 1e-10f;
    if (ptx::mbar_wait(accum, 0, a.status, 6)) {
      ptx::tc_fence_after();
      const RotMat Rm = sR[rl];
      const uint32_t lane_addr = tmem + ((uint32_t)(quarter * 32) << 16);
      for (int c0 = 0; c0 < BN; c0 += 16) {
        float u[16];
        ptx::tmem_ld16(lane_addr + c0, u);
        ptx::tmem_wait_ld();
        if (!live) continue;
#pragma unroll 4
        for (int j = 0; j < 16; ++j) {
          const int q = q0 + c0 + j;
          if (q >= a.P_eff) break;
          const float U = u[j] * qs;
          const float slice = U / Tr;
          tc_insert(a, Rm, __ldg(a.cx + q), __ldg(a.cy + q), __ldg(a.cz + q), Tr * slice, Tr);
        }
      }
    }
  }
  ptx::tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc(tmem, 256);
  }
}

// ------------------------------------------------------------ host -------
struct TcState {
  CUtensorMap mK, mK2h, mK2l, mQh, mQl, mKt;
  CUtensorMap rot[3][6];  // rotation-side maps, box rows 128 / {1, 2, 4}
  __half *Mp, *MSh, *Gh, *Gl, *Hh, *Hl;
  int* status;
};

static TcState* state(emc_plan* p) { return (TcState*)p->tc; }

int tc_bind(emc_plan* p) {
  emc_ctx* ctx = p->ctx;
  if (!p->counts_fp16_exact)
    return fail(ctx, EMC_ERR_UNSUPPORTED,
                "mixed precision needs integer counts in [0, 2048] (exact in FP16)");
  if (p->d.diff != EMC_DIFF_POISSON)
    return fail(ctx, EMC_ERR_UNSUPPORTED, "mixed precision implements the reference poisson diff");
  const int N = p->d.n_images, Np = p->Np, Kp = p->Kp, Rp = p->Rp;
  int rc = EMC_OK;
  if (!p->tc) {
    TcState* st = new TcState();
    std::memset(st, 0, sizeof(*st));
    p->tc = st;
    const size_t pk = (size_t)Np * Kp, rk = (size_t)Rp * Kp;
    if (!rc) rc = plan_alloc(p, (void**)&p->Kh, pk * 2);
    if (!rc) rc = plan_alloc(p, (void**)&p->K2hi, pk * 2);
    if (!rc) rc = plan_alloc(p, (void**)&p->K2lo, pk * 2);
    if (!rc) rc = plan_alloc(p, (void**)&p->KhT, pk * 2);
    if (!rc) rc = plan_alloc(p, (void**)&p->k2lo_any, (size_t)(Np / 128) * (Kp / 32));
    __half** rot_ops[6] = {&st->Mp, &st->MSh, &st->Gh, &st->Gl, &st->Hh, &st->Hl};
    for (auto pp : rot_ops)
      if (!rc) rc = plan_alloc(p, (void**)pp, rk * 2);
    if (!rc) rc = plan_alloc(p, (void**)&p->Qh, (size_t)Rp * Np * 2);
    if (!rc) rc = plan_alloc(p, (void**)&p->Ql, (size_t)Rp * Np * 2);
    if (!rc) rc = plan_alloc(p, (void**)&p->qscale, (size_t)Rp * 4);
    if (!rc) rc = plan_alloc(p, (void**)&st->status, 64);
    if (rc) return rc;
    EMC_CUDA(ctx, cudaMemsetAsync(p->Qh, 0, (size_t)Rp * Np * 2, ctx->stream));
    EMC_CUDA(ctx, cudaMemsetAsync(p->Ql, 0, (size_t)Rp * Np * 2, ctx->stream));
    // tensor maps (fixed addresses for the plan's lifetime)
    if (!rc) rc = make_map(ctx, &st->mK, p->Kh, Np, Kp, 128, 32);
    if (!rc) rc = make_map(ctx, &st->mK2h, p->K2hi, Np, Kp, 128, 32);
    if (!rc) rc = make_map(ctx, &st->mK2l, p->K2lo, Np, Kp, 128, 32);
    const __half* ro[6] = {st->Mp, st->MSh, st->Gh, st->Gl, st->Hh, st->Hl};
    for (int c = 0; c < 3; ++c)
      for (int j = 0; j < 6 && !rc; ++j) rc = make_map(ctx, &st->rot[c][j], ro[j], Rp, Kp, 128 >> c, 32);
    if (!rc) rc = make_map(ctx, &st->mQh, p->Qh, Rp, Np, 128, 64);
    if (!rc) rc = make_map(ctx, &st->mQl, p->Ql, Rp, Np, 128, 64);
    if (!rc) rc = make_map(ctx, &st->mKt, p->KhT, Kp, Np, 256, 64);
    if (rc) return rc;
    EMC_CUDA(ctx, cudaFuncSetAttribute(tc_estep_kernel<1>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, es::SMEM_BYTES));
    EMC_CUDA(ctx, cudaFuncSetAttribute(tc_estep_kernel<2>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, es::SMEM_BYTES));
    EMC_CUDA(ctx, cudaFuncSetAttribute(tc_estep_kernel<4>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, es::SMEM_BYTES));
    EMC_CUDA(ctx, cudaFuncSetAttribute(tc_mstep_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       ms::SMEM_BYTES));
  }
  tc_pattern_ops_kernel<<<dim3(ceil_div(Kp, 256), Np), 256, 0, ctx->stream>>>(
      p->images, p->pix, p->n2, N, Kp, p->Kh, p->K2hi, p->K2lo);
  if ((rc = after_launch(ctx, "tc_pattern_ops_kernel"))) return rc;
  tc_k2lo_flags_kernel<<<dim3(Kp / 32, Np / 128), 256, 0, ctx->stream>>>(p->K2lo, Kp, p->k2lo_any,
                                                                         Kp / 32);
  if ((rc = after_launch(ctx, "tc_k2lo_flags_kernel"))) return rc;
  transpose_h_kernel<<<dim3(ceil_div(Kp, 32), ceil_div(Np, 32)), dim3(32, 8), 0, ctx->stream>>>(
      p->Kh, Np, Kp, p->KhT);
  return after_launch(ctx, "transpose_h_kernel");
}

static int check_status(emc_plan* p, const char* what) {
  emc_ctx* ctx = p->ctx;
  int h = 0, f = 0;
  EMC_CUDA(ctx, cudaMemcpyAsync(&h, state(p)->status, sizeof(int), cudaMemcpyDeviceToHost,
                                ctx->stream));
  EMC_CUDA(ctx, cudaMemcpyAsync(&f, p->flags, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (h) return fail(ctx, EMC_ERR_TIMEOUT, "%s: pipeline wait timed out (status 0x%x)", what, h);
  if (f & 4)
    return fail(ctx, EMC_ERR_UNSUPPORTED, "%s: slice values exceed the FP16 operand range", what);
  return EMC_OK;
}

int tc_estep(emc_plan* p, float sigma) {
  emc_ctx* ctx = p->ctx;
  TcState* st = state(p);
  const size_t rk = (size_t)p->Rp * p->Kp;
  int rc;
  tc_rot_ops_kernel<<<ctx->sm_count * 8, 256, 0, ctx->stream>>>(p->S, rk, st->Mp, st->MSh, st->Gh,
                                                                st->Gl, st->Hh, st->Hl, p->flags);
  if ((rc = after_launch(ctx, "tc_rot_ops_kernel"))) return rc;
  EMC_CUDA(ctx, cudaMemsetAsync(st->status, 0, sizeof(int), ctx->stream));
  TcEstepArgs a;
  a.N = p->d.n_images;
  a.R = p->d.n_rot;
  a.Kp = p->Kp;
  a.n_pt = p->Np / es::BM;
  a.n_rt = p->Rp / es::BN;
  a.nkb = p->Kp / es::BK;
  a.k2lo_any = p->k2lo_any;
  a.rot_cnt = p->rot_cnt;
  a.rot_A = p->rot_A;
  a.rotw = p->rotw;
  a.cnorm = p->cnorm;
  a.inv2s2 = 1.0f / (2.0f * sigma * sigma);
  a.known_intensity = p->d.known_intensity;
  a.L = p->L;
  a.PHI = p->PHI;
  a.part = p->part;
  a.bad = p->flags + 4;
  a.status = st->status;
  const int cl = p->estep_cluster;
  const int c = cl == 4 ? 2 : cl == 2 ? 1 : 0;
  const CUtensorMap* rm = st->rot[c];
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(a.n_pt * a.n_rt);
  cfg.blockDim = dim3(es::THREADS);
  cfg.dynamicSmemBytes = es::SMEM_BYTES;
  cfg.stream = ctx->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cl;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaError_t e;
  if (cl == 4)
    e = cudaLaunchKernelEx(&cfg, tc_estep_kernel<4>, st->mK, st->mK2h, st->mK2l, rm[0], rm[1],
                           rm[2], rm[3], rm[4], rm[5], a);
  else if (cl == 2)
    e = cudaLaunchKernelEx(&cfg, tc_estep_kernel<2>, st->mK, st->mK2h, st->mK2l, rm[0], rm[1],
                           rm[2], rm[3], rm[4], rm[5], a);
  else
    e = cudaLaunchKernelEx(&cfg, tc_estep_kernel<1>, st->mK, st->mK2h, st->mK2l, rm[0], rm[1],
                           rm[2], rm[3], rm[4], rm[5], a);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "tc_estep_kernel launch");
  return after_launch(ctx, "tc_estep_kernel");
}

int tc_mstep(emc_plan* p, float* model, float* weight) {
  emc_ctx* ctx = p->ctx;
  TcState* st = state(p);
  int rc;
  TcMstepArgs a;
  a.R = p->d.n_rot;
  a.Kp = p->Kp;
  a.Np = p->Np;
  a.P_eff = p->P_eff;
  a.n_qt = p->Kp / ms::BN + (p->Kp % ms::BN ? 1 : 0);
  a.n_rt = p->Rp / ms::BM;
  a.nkb = p->Np / ms::BK;
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
  a.bounds = p->red + kRedBoundM;
  a.status = st->status;
  const int tiles = a.n_qt * a.n_rt;
  tc_mstep_kernel<<<tiles, ms::THREADS, ms::SMEM_BYTES, ctx->stream>>>(st->mQh, st->mQl, st->mKt, a);
  if ((rc = after_launch(ctx, "tc_mstep_kernel"))) return rc;
  return check_status(p, "tensor-core iteration");
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
