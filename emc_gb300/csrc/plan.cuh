// The fused-iteration plan: workspace layout and kernels shared by the FP32
// and tensor-core paths.
#pragma once
#include <cuda_fp16.h>

#include <vector>

#include "common.cuh"
#include "kernels.cuh"

// Rotations per E-step tile; LSE partials are kept per tile of this many rows.
#define EMC_RT 128

struct emc_plan {
  emc_ctx* ctx = nullptr;
  emc_plan_desc d{};
  int n2 = 0;      // side*side
  int P_eff = 0;   // pixels with mask != 0
  int Kp = 0;      // P_eff padded (128)
  int Np = 0;      // patterns padded (128)
  int Rp = 0;      // rotations padded (128)
  int n_rt = 0;    // rotation tiles of EMC_RT
  bool bound = false;
  bool counts_fp16_exact = false;  // every count is an integer in [0, 2048]
  bool counts_integer = false;     // every count is an integer in [0, 65504]
  int count_max = 0;               // the largest count
  int counts_round = 0;            // tensor path: counts above 2048 rounded to FP16
  float k2_scale = 1.0f / 128.0f;  // K^2 operand = k^2 k2_scale (hi + lo), set at bind

  // bound inputs (caller owned)
  const float* images = nullptr;
  const int* mask = nullptr;
  const float *x = nullptr, *y = nullptr, *z = nullptr;
  const float* rot = nullptr;
  const float* rotw = nullptr;

  // compacted geometry
  int* pix = nullptr;                          // [Kp], -1 padding
  float *cx = nullptr, *cy = nullptr, *cz = nullptr;  // [Kp]

  // pattern operands, rows of Kp (FP32 path)
  float* Kraw = nullptr;  // k (x c_i when normalising); FP32 plans only
  double* ksum_part = nullptr;  // [N][Kp / 256] block sums of k
  std::vector<int> h_mask, h_pix;  // the bound mask and its compacted pixels (re-binds)
  float fused_k2_scale = 0.0f;  // K^2 scale of FP16 operands written by pattern_ops (0: none)
  float* Kt = nullptr;    // k if k > 1e-10 else 0
  float* K2 = nullptr;    // Kt^2
  float* Ksum = nullptr;  // [N] sum_p k
  float* cnorm = nullptr; // [N] c_i (1 when not normalising)

  // pattern operands (tensor-core path): counts as FP16, rows of Kp
  __half* Kh = nullptr;      // k
  __half* K2hi = nullptr;    // fp16(k^2 * 2^-e)
  __half* K2lo = nullptr;    // k^2 * 2^-e - K2hi
  unsigned char* k2lo_any = nullptr;  // [Np/128][Kp/32] block has a nonzero K2lo
  // [Np/128 + 1] the likelihood's G lo term runs on the k-blocks below glo_kb[pt]
  // of pattern tile pt: the blocks after it hold at most glo_tail_ppm / 1e6 of
  // every pattern's counts (EMC_OPT_GLO_TAIL; 0: G lo on every block);
  // glo_kb[Np/128] is the largest of them
  int* glo_kb = nullptr;
  int glo_tail_ppm = 1000;
  __half* KhT = nullptr;     // [Kp][Np] transposed counts for the M-step

  // rotation side, per iteration
  float* S = nullptr;       // [Rp][Kp] slice at the compacted pixels (FP32 path)
  float* rot_cnt = nullptr; // [Rp] count_r (pixels with s > 0)
  float* rot_A = nullptr;   // [Rp] sum s^2/(s+c) over s > 0
  float* rot_ssum = nullptr;// [Rp] sum max(s, floor) (true Poisson)

  // responsibilities
  float* L = nullptr;      // [R][N] log-likelihood, then normalised responsibility
  float* PHI = nullptr;    // [R][N] scaling
  float* Q = nullptr;      // [R][N] responsibility / scaling (FP32 M-step)
  __half* Qh = nullptr;    // [Rp][Np] hi (tensor-core M-step)
  __half* Ql = nullptr;    // [Rp][Np] lo
  float* qscale = nullptr; // [Rp] 2^-e_r of the Q rows
  float2* part = nullptr;  // [n_rt][N] (max, sumexp) per rotation tile
  double* lse = nullptr;   // [N]
  float2* lse2 = nullptr;  // [N] lse as float hi + lo
  float* T = nullptr;      // [Rp] rotation totals
  double* red = nullptr;   // reduction scratch (small)
  unsigned long long* fix_m = nullptr;  // [s^3] fixed-point model (deterministic insert)
  unsigned long long* fix_w = nullptr;
  float2* acc2 = nullptr;  // [s^3] interleaved (model, weight) sums (float atomics)
  int* flags = nullptr;    // device status words
  float* sigma_dev = nullptr;  // [1] annealing width read by the E-step kernels
  emc::BlurWork blur{};        // plan-owned blur buffers and taps (blur_sigma > 0)

  // pruned iteration (prune.cu): set for the iteration being enqueued
  int2* prune_tiles = nullptr;          // (pattern tile, rotation tile) list, device
  int prune_n_tiles = 0;
  unsigned char* prune_state = nullptr; // [n_pt][n_rt] 0 skipped, 1 evaluated, 2 margin
  double* prune_margin = nullptr;       // [R] responsibility mass in margin tiles
  int* prune_kb_off = nullptr;          // [n_rt + 1] M-step k-blocks per rotation tile
  int* prune_kb_list = nullptr;         // the 64-pattern k-blocks themselves
  void* prune = nullptr;                // PruneState
  // L holds the normalised responsibilities P of the last iteration (true),
  // or still its log-likelihoods (false: mprep left P unwritten; it is formed
  // on request by plan_respons_ready)
  bool p_written = true;

  // one captured iteration (emc_plan_capture / emc_plan_replay)
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;

  // per-phase CUDA events on the context stream (emc_plan_set_profiling)
  static constexpr int kPhases = 6;  // expand, estep, lse, mprep, mstep, finish
  bool profiling = false;
  cudaEvent_t ev[kPhases + 1] = {};

  void* tc = nullptr;  // tensor-core state (tensor maps, rotation operands)
  int estep_gh_lo = -1;   // tensor E-step lo terms: bit 0 G, bit 1 H; -1 auto
  int mstep_q_lo = 0;     // tensor M-step: Q as FP16 hi + lo (1) or hi only (0)
  int estep_raster = 8;     // tensor E-step tile order (EMC_OPT_ESTEP_RASTER)
  int estep_pair = 1;       // full scans on CTA pairs (EMC_OPT_ESTEP_PAIR)
  int mstep_raster = -16;   // tensor M-step tile order (EMC_OPT_MSTEP_RASTER)
  int mstep_aggregate = 0;  // tensor M-step: warp-aggregated float atomics (nearest)
  unsigned debug_spin = 0;  // > 0: polls per tensor-pipeline wait (EMC_OPT_DEBUG_SPIN)
  int mstep_pair = 1;       // tensor M-step full scans on CTA pairs (EMC_OPT_MSTEP_PAIR)

  // sorted-voxel insertion (EMC_INSERT_SORTED, sorted_insert.cu): the M-step
  // stores each pair's value T_r x slice in ins_u [P_eff][ins_ldu] (rotation
  // fastest) and a segmented reduction in voxel order adds them
  float* ins_u = nullptr;
  int ins_ldu = 0;
  void* sorted = nullptr;

  std::vector<void*> allocs;
  size_t bytes = 0;
};

namespace emc {

// Voxel-sum upper bound and fixed-point scale slots in plan->red.
enum RedSlot {
  kRedLL = 0,        // total log-likelihood
  kRedMass = 1,      // captured responsibility mass
  kRedBad = 2,       // invalid pairs
  kRedBoundM = 3,    // upper bound of inserted model mass
  kRedBoundW = 4,    // upper bound of inserted weight
  kRedMean = 5,      // {sum, count} of positive voxels (2 slots) + partials
  kRedFixScale = 7,  // float2 {model, weight} fixed-point scales (deterministic mode)
  kRedSlots = 8,
};

// Deterministic insertion adds round(value * scale) into 64-bit integers.
// The scale is the power of two 2^(61 - k) with bound <= 2^k (the bound is an
// upper bound of the total inserted mass), so no partial sum leaves the signed
// 64-bit range, value * scale is exact in FP32, and 1 / scale is exact too.
__host__ __device__ inline float fix_scale_pow2(double bound) {
  if (!(bound > 0.0)) return 1.0f;
  int k;
  frexp(bound, &k);  // bound = f 2^k, f in [0.5, 1)
  const int e = 61 - k;
  return ldexpf(1.0f, e < -126 ? -126 : (e > 126 ? 126 : e));
}

#ifdef __CUDACC__
// x rounded to the nearest integer (ties to even) as a signed 64-bit value,
// with FP32 and integer instructions only: below 2^23 the addition of 2^23
// rounds the fraction away; from 2^23 on x is an integer, its mantissa shifted
// by the exponent.  |x| >= 2^62 (never reached under fix_scale_pow2) saturates.
__device__ __forceinline__ long long fixed_from_float(float x) {
  const float a = fabsf(x);
  long long m;
  if (a < 8388608.0f) {
    m = (long long)(__float_as_uint(__fadd_rn(a, 8388608.0f)) - 0x4B000000u);
  } else if (a < 4611686018427387904.0f) {
    const unsigned b = __float_as_uint(a);
    m = (long long)((b & 0x7FFFFFu) | 0x800000u) << ((int)(b >> 23) - 150);
  } else {
    m = 0x4000000000000000LL;
  }
  return x < 0.0f ? -m : m;
}
#endif

int plan_alloc(emc_plan* p, void** ptr, size_t bytes);

// Sorted-voxel insertion (sorted_insert.cu).  sorted_ensure (re)builds the
// voxel map when the plan's rotations or pixel coordinates differ from those
// it was built from (a bind, a change of the rotation order); sorted_reduce
// enqueues the per-iteration reduction of ins_u into acc2.
int sorted_ensure(emc_plan* p);
int sorted_reduce(emc_plan* p);
void sorted_free(emc_plan* p);

// Tensor-core path (tc_gemm.cu).
int tc_bind(emc_plan* p);
int prune_iterate(emc_plan* p, float* model, float* weight, float sigma, emc_iter_stats* stats,
                  bool* handled);
void prune_free(emc_plan* p);
int prune_reset(emc_plan* p);
int tc_pattern_side(emc_plan* p, const int* d_perm, bool counts_done = false);
int tc_ensure_qlo(emc_plan* p);
int tc_glo_extent(emc_plan* p);  // glo_kb from the bound counts and glo_tail_ppm
int pattern_side(emc_plan* p, const int* d_perm, bool with_tc);
// Rotation-side FP16 operands of the tensor-core likelihood, written by the
// expand kernel straight from each slice value s (no FP32 slice buffer):
// reference likelihood: M' = [s >= 1e-10], M'S * 2^-8, G = s / (s + c) and
// H = 1 / (s + c) (c = 0.02; zero where s <= 0) as FP16 hi + lo; true Poisson:
// log max(s, 1e-6) as FP16 hi + lo in Gh / Gl.  flags[0] |= 4 when M'S * 2^-8
// leaves the FP16 range.
struct RotOps {
  __half *Mp = nullptr, *MSh = nullptr, *Gh = nullptr, *Gl = nullptr, *Hh = nullptr, *Hl = nullptr;
  int* flags = nullptr;
  int logs = 0;
  // device int: G lo is read (and written) only in the 32-pixel blocks below
  // it, the largest count-tail bound of the pattern tiles (null: every block)
  const int* gl_end = nullptr;
};

// The operands of four neighbouring pixels e .. e + 3 (e a multiple of 4) as
// 8-byte stores; hv = 1 / (s + 0.02) where s > 0 (0 elsewhere), computed by
// the caller.  The same values as rot_ops_store2, pixel by pixel.
__device__ __forceinline__ void rot_ops_store4(const RotOps& o, size_t e, const float (&sv)[4],
                                               const float (&hv)[4], bool g_lo) {
  union H4 {
    __half h[4];
    uint2 u;
  };
  if (o.logs) {
    H4 hi, lo;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const float l = logf(fmaxf(sv[u], 1e-6f));
      hi.h[u] = __float2half_rn(l);
      lo.h[u] = __float2half_rn(l - __half2float(hi.h[u]));
    }
    *reinterpret_cast<uint2*>(o.Gh + e) = hi.u;
    *reinterpret_cast<uint2*>(o.Gl + e) = lo.u;
    return;
  }
  H4 mp4, ms4, gh4, gl4, hh4, hl4;
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const float s = sv[u];
    const bool mp = s >= 1e-10f;
    const bool m = s > 0.0f;
    const float ms = mp ? s * (1.0f / 256.0f) : 0.0f;
    if (ms > 60000.0f) atomicOr(o.flags, 4);
    const float h = hv[u];
    const float g = m ? s * h : 0.0f;
    mp4.h[u] = __float2half_rn(mp ? 1.0f : 0.0f);
    ms4.h[u] = __float2half_rn(ms);
    gh4.h[u] = __float2half_rn(g);
    gl4.h[u] = __float2half_rn(g - __half2float(gh4.h[u]));
    hh4.h[u] = __float2half_rn(h);
    hl4.h[u] = __float2half_rn(h - __half2float(hh4.h[u]));
  }
  *reinterpret_cast<uint2*>(o.Mp + e) = mp4.u;
  *reinterpret_cast<uint2*>(o.MSh + e) = ms4.u;
  *reinterpret_cast<uint2*>(o.Gh + e) = gh4.u;
  if (o.Gl && g_lo) *reinterpret_cast<uint2*>(o.Gl + e) = gl4.u;
  *reinterpret_cast<uint2*>(o.Hh + e) = hh4.u;
  if (o.Hl) *reinterpret_cast<uint2*>(o.Hl + e) = hl4.u;
}

RotOps tc_rot_ops(emc_plan* p);  // the plan's operand buffers (all null for FP32 plans)
int tc_estep(emc_plan* p);
int tc_autotune(emc_plan* p, int waves, int* best, float* best_ms);
int tc_estep_tiles(emc_plan* p);    // tiles of the full likelihood grid
int tc_time_estep(emc_plan* p, int raster, int first, int count, float* ms);
int tc_mstep(emc_plan* p, float* model, float* weight);
int* tc_status(emc_plan* p);  // device status word of the tensor-core pipelines
void tc_free(emc_plan* p);
// Forms P = exp(L - lse) over L on the plan's stream when the last iteration
// left it unwritten (p_written false); no-op otherwise.
int plan_respons_ready(emc_plan* p);

}  // namespace emc
