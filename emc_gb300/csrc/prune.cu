// Pruned iterations: the E-step evaluates only the (pattern tile, rotation
// tile) blocks that carry the responsibility mass, with a full-scan fallback.
//
// After an iteration the plan sorts the patterns by their most probable
// rotation (so a 128-pattern tile holds patterns of similar orientation and
// needs few rotation tiles), marks as "core" every tile in which a pattern's
// responsibility mass exceeds tau = (1 - min_mass) / (10 n_rt) (the mass left
// out that way is at most a tenth of 1 - min_mass per pattern), and adds as
// "margin" every rotation tile within `dilate` nearest-neighbour angles of a
// core tile.  The next iteration evaluates core and margin tiles only.  If
// the responsibility mass that lands in margin tiles exceeds 1 - min_mass per
// pattern, the distribution has moved or spread beyond what the margin can
// vouch for: the iteration is repeated from its input model as a full scan.
// Responsibilities outside the evaluated tiles are exactly 0.
//
// While pruning is on, the plan also keeps its rotations in a spatially
// coherent order (recursive median bisection of the quaternions' vector
// parts into blocks of exactly 128), so that a 128-rotation tile is a
// compact region of rotation space and a pattern's neighbourhood touches few
// tiles.
#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "emc_gb300.h"
#include "plan.cuh"

namespace emc {

struct PruneState {
  float min_mass = 0.999f;
  float dilate = 1.0f;   // margin radius in nearest-neighbour angles
  int full_every = 0;    // a full scan every this many iterations (0: only on fallback)
  int since_full = 0;    // iterations since the last full scan
  float tau = 0.0f;      // core threshold of a tile's mass for one pattern
  bool ready = false;    // the next iteration may be pruned
  double nn_angle = 0.0; // median nearest-neighbour angle of the rotation list (rad)
  std::vector<int> h_perm;          // position -> input pattern, of the operands
  std::vector<int> h_perm_results;  // the same, of the last iteration's results
  int *d_perm = nullptr, *d_newpos = nullptr, *d_best = nullptr;
  int* d_perm_res = nullptr;  // h_perm_results on the device (emc_plan_best_quaternions)
  unsigned char *d_core = nullptr, *d_state = nullptr, *d_adj = nullptr;
  int2* d_tiles = nullptr;
  int n_tiles = 0;
  int *d_kb_off = nullptr, *d_kb_list = nullptr;  // M-step k-blocks per rotation tile
  float* d_model_in = nullptr;
  float* d_nn = nullptr;
  // rotation order: internal row -> input rotation, and the input buffers
  std::vector<int> h_rorder;
  float *d_rot = nullptr, *d_rotw = nullptr;
  const float *rot_in = nullptr, *rotw_in = nullptr;
  double* d_margin = nullptr;
  emc_prune_info info{};
};

static PruneState* pstate(emc_plan* p) { return (PruneState*)p->prune; }

__device__ __forceinline__ float qdot(float4 a, float4 b) {
  return fabsf(a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w);
}

__device__ __forceinline__ float4 load_q(const float* rot, int r) {
  return make_float4(rot[4 * r], rot[4 * r + 1], rot[4 * r + 2], rot[4 * r + 3]);
}

// nn[r] = max over r' != r of |q_r . q_r'| (cosine of half the angle to the
// nearest other rotation).
__global__ void rot_nn_kernel(const float* __restrict__ rot, int R, float* __restrict__ nn) {
  __shared__ float4 sq[256];
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const float4 q = r < R ? load_q(rot, r) : make_float4(0.f, 0.f, 0.f, 0.f);
  float best = 0.0f;
  for (int t0 = 0; t0 < R; t0 += 256) {
    const int t = t0 + threadIdx.x;
    sq[threadIdx.x] = t < R ? load_q(rot, t) : make_float4(0.f, 0.f, 0.f, 0.f);
    __syncthreads();
    const int n = min(256, R - t0);
    for (int j = 0; j < n; ++j)
      if (t0 + j != r) best = fmaxf(best, qdot(q, sq[j]));
    __syncthreads();
  }
  if (r < R) nn[r] = best;
}

// adj[a][b] = 1 when some rotation of tile a is within the angle whose
// half-angle cosine is cos_half of some rotation of tile b.
__global__ void rot_tile_adj_kernel(const float* __restrict__ rot, int R, int n_rt, float cos_half,
                                    unsigned char* __restrict__ adj) {
  const int a = blockIdx.y, b = blockIdx.x, t = threadIdx.x;  // 128 threads
  __shared__ float4 qb[128];
  const int rb = b * 128 + t, ra = a * 128 + t;
  qb[t] = rb < R ? load_q(rot, rb) : make_float4(0.f, 0.f, 0.f, 0.f);
  __syncthreads();
  int hit = 0;
  if (ra < R) {
    const float4 q = load_q(rot, ra);
    const int n = min(128, R - b * 128);
    for (int j = 0; j < n && !hit; ++j) hit = qdot(q, qb[j]) >= cos_half;
  }
  hit = __syncthreads_or(hit);
  if (t == 0) adj[(size_t)a * n_rt + b] = (unsigned char)hit;
}

// best[i] = the rotation with the largest responsibility of pattern i.
__global__ void best_rotation_kernel(const float* __restrict__ P, int R, int N,
                                     int* __restrict__ best) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  float bv = -1.0f;
  int br = 0;
  for (int r = 0; r < R; ++r) {
    const float v = P[(size_t)r * N + i];
    if (v > bv) {
      bv = v;
      br = r;
    }
  }
  best[i] = br;
}

// core[newpos[i] / 128][rt] = 1 when pattern i's mass in rotation tile rt > tau.
__global__ void tile_mass_kernel(const float* __restrict__ P, int R, int N, int n_rt,
                                 const int* __restrict__ newpos, float tau,
                                 unsigned char* __restrict__ core) {
  const int rt = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int r1 = min(R, (rt + 1) * 128);
  float m = 0.0f;
  for (int r = rt * 128; r < r1; ++r) m += P[(size_t)r * N + i];
  if (m > tau) core[(size_t)(newpos[i] >> 7) * n_rt + rt] = 1;
}

// state = 1 for core tiles, 2 for tiles adjacent to a core tile of the same
// pattern tile, 0 otherwise.
__global__ void dilate_kernel(const unsigned char* __restrict__ core,
                              const unsigned char* __restrict__ adj, int n_pt, int n_rt,
                              unsigned char* __restrict__ state) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_pt * n_rt) return;
  const int pt = e / n_rt, rt = e % n_rt;
  unsigned char s = core[e] ? 1 : 0;
  if (!s)
    for (int r2 = 0; r2 < n_rt; ++r2)
      if (core[(size_t)pt * n_rt + r2] && adj[(size_t)r2 * n_rt + rt]) {
        s = 2;
        break;
      }
  state[e] = s;
}

// The most probable rotation's quaternion of each pattern (responsibilities
// P [R][N] over the plan's rotation rows), written at the pattern's input
// index perm[i] (perm: column -> input pattern; nullptr: identity).
__global__ void best_quat_kernel(const float* __restrict__ P, int R, int N,
                                 const float* __restrict__ rot, const int* __restrict__ perm,
                                 float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  float bv = -1.0f;
  int br = 0;
  for (int r = 0; r < R; ++r) {
    const float v = P[(size_t)r * N + i];
    if (v > bv) {
      bv = v;
      br = r;
    }
  }
  const int d = perm ? perm[i] : i;
  for (int c = 0; c < 4; ++c) out[4 * (size_t)d + c] = rot[4 * (size_t)br + c];
}

// nearest[i] = the rotation row closest to pattern i's first proposal
// (props [N][n_modes][4]).  Rotations staged through shared memory.
__global__ void nearest_row_kernel(const float* __restrict__ props, int n_modes,
                                   const float* __restrict__ rot, int R, int N,
                                   int* __restrict__ nearest) {
  __shared__ float4 sq[512];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float4 q = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  if (i < N) q = load_q(props, i * n_modes);
  float bv = -1.0f;
  int br = 0;
  for (int r0 = 0; r0 < R; r0 += 512) {
    __syncthreads();
    for (int r = threadIdx.x; r < 512 && r0 + r < R; r += blockDim.x) sq[r] = load_q(rot, r0 + r);
    __syncthreads();
    const int r1 = min(512, R - r0);
    for (int r = 0; r < r1; ++r) {
      const float v = qdot(q, sq[r]);
      if (v > bv) {
        bv = v;
        br = r0 + r;
      }
    }
  }
  if (i < N) nearest[i] = br;
}

// core[newpos[i] / 128][rt] = 1 when some rotation of tile rt lies within the
// ball (half-angle cosine cos_half) around one of pattern i's proposals.
__global__ void proposal_core_kernel(const float* __restrict__ props, int n_modes,
                                     const float* __restrict__ rot, int R, int N,
                                     const int* __restrict__ newpos, float cos_half, int n_rt,
                                     unsigned char* __restrict__ core) {
  __shared__ float4 sq[128];
  const int rt = blockIdx.y;
  const int r0 = rt * 128, cnt = min(128, R - r0);
  for (int r = threadIdx.x; r < cnt; r += blockDim.x) sq[r] = load_q(rot, r0 + r);
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  bool hit = false;
  for (int m = 0; m < n_modes && !hit; ++m) {
    const float4 q = load_q(props, i * n_modes + m);
    for (int r = 0; r < cnt; ++r)
      if (qdot(q, sq[r]) >= cos_half) {
        hit = true;
        break;
      }
  }
  if (hit) core[(size_t)(newpos[i] >> 7) * n_rt + rt] = 1;
}

static int prune_alloc(emc_plan* p, PruneState* ps) {
  const int N = p->d.n_images, R = p->d.n_rot, n_rt = p->n_rt, n_pt = p->Np / 128;
  const size_t n3 = (size_t)p->d.side * p->d.side * p->d.side;
  int rc = EMC_OK;
  if (!rc) rc = plan_alloc(p, (void**)&ps->d_perm, sizeof(int) * N);
  if (!rc) rc = plan_alloc(p, (void**)&ps->d_newpos, sizeof(int) * N);
  if (!rc) rc = plan_alloc(p, (void**)&ps->d_best, sizeof(int) * N);
  if (!rc) rc = plan_alloc(p, (void**)&ps->d_perm_res, sizeof(int) * N);
  if (!rc) rc = plan_alloc(p, (void**)&ps->d_core, (size_t)n_pt * n_rt);
  if (!rc) rc = plan_alloc(p, (void**)&ps->d_state, (size_t)n_pt * n_rt);
  if (!rc) rc = plan_alloc(p, (void**)&ps->d_adj, (size_t)n_rt * n_rt);
  if (!rc) rc = plan_alloc(p, (void**)&ps->d_tiles, sizeof(int2) * n_pt * n_rt);
  if (!rc) rc = plan_alloc(p, (void**)&ps->d_model_in, sizeof(float) * n3);
  if (!rc) rc = plan_alloc(p, (void**)&ps->d_margin, sizeof(double) * (size_t)R);
  if (!rc) rc = plan_alloc(p, (void**)&ps->d_nn, sizeof(float) * (size_t)R);
  if (!rc) rc = plan_alloc(p, (void**)&ps->d_kb_off, sizeof(int) * ((size_t)n_rt + 1));
  if (!rc) rc = plan_alloc(p, (void**)&ps->d_kb_list, sizeof(int) * 2 * (size_t)n_pt * n_rt);
  if (!rc) rc = plan_alloc(p, (void**)&ps->d_rot, sizeof(float) * 4 * (size_t)R);
  if (!rc) rc = plan_alloc(p, (void**)&ps->d_rotw, sizeof(float) * (size_t)R);
  return rc;
}

// Orders idx[lo, hi) into compact blocks of 128: split at a multiple of 128
// near the middle, along the axis (q1, q2 or q3) of widest spread, recursively.
static void bisect_order(std::vector<int>& idx, int lo, int hi, const std::vector<float>& q) {
  if (hi - lo <= 128) return;
  int axis = 1;
  float best = -1.0f;
  for (int c = 1; c < 4; ++c) {
    float mn = 2.0f, mx = -2.0f;
    for (int k = lo; k < hi; ++k) {
      mn = std::min(mn, q[4 * (size_t)idx[k] + c]);
      mx = std::max(mx, q[4 * (size_t)idx[k] + c]);
    }
    if (mx - mn > best) {
      best = mx - mn;
      axis = c;
    }
  }
  const int blocks = (hi - lo + 127) / 128;
  const int mid = lo + ((blocks + 1) / 2) * 128;
  std::nth_element(idx.begin() + lo, idx.begin() + mid, idx.begin() + hi, [&](int a, int b) {
    const float va = q[4 * (size_t)a + axis], vb = q[4 * (size_t)b + axis];
    return va < vb || (va == vb && a < b);
  });
  bisect_order(idx, lo, mid, q);
  bisect_order(idx, mid, hi, q);
}

// The plan's rotations in compact 128-blocks of (q1, q2, q3) space (the
// input buffers stay untouched): p->rot / p->rotw point at the plan's
// reordered copies.
static int prune_rotation_order(emc_plan* p, PruneState* ps) {
  emc_ctx* ctx = p->ctx;
  const int R = p->d.n_rot;
  ps->rot_in = p->rot;
  ps->rotw_in = p->rotw;
  std::vector<float> q(4 * (size_t)R), w(R);
  EMC_CUDA(ctx, cudaMemcpyAsync(q.data(), ps->rot_in, sizeof(float) * 4 * R,
                                cudaMemcpyDeviceToHost, ctx->stream));
  EMC_CUDA(ctx, cudaMemcpyAsync(w.data(), ps->rotw_in, sizeof(float) * R, cudaMemcpyDeviceToHost,
                                ctx->stream));
  EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  ps->h_rorder.resize(R);
  std::iota(ps->h_rorder.begin(), ps->h_rorder.end(), 0);
  bisect_order(ps->h_rorder, 0, R, q);
  std::vector<float> q2(4 * (size_t)R), w2(R);
  for (int j = 0; j < R; ++j) {
    const int r = ps->h_rorder[j];
    for (int c = 0; c < 4; ++c) q2[4 * (size_t)j + c] = q[4 * (size_t)r + c];
    w2[j] = w[r];
  }
  EMC_CUDA(ctx, cudaMemcpyAsync(ps->d_rot, q2.data(), sizeof(float) * 4 * R,
                                cudaMemcpyHostToDevice, ctx->stream));
  EMC_CUDA(ctx, cudaMemcpyAsync(ps->d_rotw, w2.data(), sizeof(float) * R, cudaMemcpyHostToDevice,
                                ctx->stream));
  EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));  // host vectors are staged
  p->rot = ps->d_rot;
  p->rotw = ps->d_rotw;
  return EMC_OK;
}

// Rotation-tile adjacency from the bound rotation list.
static int prune_geometry(emc_plan* p, PruneState* ps) {
  emc_ctx* ctx = p->ctx;
  const int R = p->d.n_rot, n_rt = p->n_rt;
  int rc;
  float* d_nn = ps->d_nn;
  rot_nn_kernel<<<ceil_div(R, 256), 256, 0, ctx->stream>>>(p->rot, R, d_nn);
  if ((rc = after_launch(ctx, "rot_nn_kernel"))) return rc;
  std::vector<float> nn(R);
  EMC_CUDA(ctx, cudaMemcpyAsync(nn.data(), d_nn, sizeof(float) * R, cudaMemcpyDeviceToHost,
                                ctx->stream));
  EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  std::vector<double> ang(R);
  for (int r = 0; r < R; ++r) ang[r] = 2.0 * std::acos(std::min(1.0, (double)nn[r]));
  std::nth_element(ang.begin(), ang.begin() + R / 2, ang.end());
  ps->nn_angle = ang[R / 2];
  const double delta = std::min(3.14159265358979, ps->dilate * ps->nn_angle);
  rot_tile_adj_kernel<<<dim3(n_rt, n_rt), 128, 0, ctx->stream>>>(p->rot, R, n_rt,
                                                                 (float)std::cos(delta / 2.0),
                                                                 ps->d_adj);
  return after_launch(ctx, "rot_tile_adj_kernel");
}

// Masks and tile list for the next iteration from the responsibilities of
// the last one (p->L, operands in ps->h_perm order); with reorder, the
// patterns are first re-sorted by their most probable rotation.
static int prune_finish(emc_plan* p, PruneState* ps, const std::vector<int>& new_perm,
                        int probe_stride = 0, bool arm = false);

static int prune_prepare(emc_plan* p, PruneState* ps, bool reorder) {
  emc_ctx* ctx = p->ctx;
  const int N = p->d.n_images, R = p->d.n_rot, n_rt = p->n_rt, n_pt = p->Np / 128;
  int rc;
  std::vector<int> newpos(N), new_perm = ps->h_perm;
  std::iota(newpos.begin(), newpos.end(), 0);
  if ((rc = plan_respons_ready(p))) return rc;
  if (reorder) {
    best_rotation_kernel<<<ceil_div(N, 256), 256, 0, ctx->stream>>>(p->L, R, N, ps->d_best);
    if ((rc = after_launch(ctx, "best_rotation_kernel"))) return rc;
    std::vector<int> best(N), order(N);
    EMC_CUDA(ctx, cudaMemcpyAsync(best.data(), ps->d_best, sizeof(int) * N,
                                  cudaMemcpyDeviceToHost, ctx->stream));
    EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return best[a] < best[b]; });
    for (int j = 0; j < N; ++j) {
      new_perm[j] = ps->h_perm[order[j]];
      newpos[order[j]] = j;
    }
  }
  EMC_CUDA(ctx, cudaMemcpyAsync(ps->d_newpos, newpos.data(), sizeof(int) * N,
                                cudaMemcpyHostToDevice, ctx->stream));
  EMC_CUDA(ctx, cudaMemsetAsync(ps->d_core, 0, (size_t)n_pt * n_rt, ctx->stream));
  tile_mass_kernel<<<dim3(ceil_div(N, 256), n_rt), 256, 0, ctx->stream>>>(
      p->L, R, N, n_rt, ps->d_newpos, ps->tau, ps->d_core);
  if ((rc = after_launch(ctx, "tile_mass_kernel"))) return rc;
  return prune_finish(p, ps, new_perm);
}

// From the core tiles in ps->d_core (rows: pattern tiles of the order
// new_perm): margin dilation, tile lists of both kernels, the pattern-side
// operands in the new order, and whether the next iteration is pruned.
// probe_stride > 0 adds, as margin, every probe_stride-th rotation tile of
// each pattern tile (staggered by pattern tile): mass found there also
// repeats the iteration as a full scan.  arm: the next iteration is pruned
// however dense the tile set (else only below 75 % of the tiles).
static int prune_finish(emc_plan* p, PruneState* ps, const std::vector<int>& new_perm,
                        int probe_stride, bool arm) {
  emc_ctx* ctx = p->ctx;
  const int N = p->d.n_images, n_rt = p->n_rt, n_pt = p->Np / 128;
  int rc;
  dilate_kernel<<<ceil_div(n_pt * n_rt, 256), 256, 0, ctx->stream>>>(ps->d_core, ps->d_adj, n_pt,
                                                                     n_rt, ps->d_state);
  if ((rc = after_launch(ctx, "dilate_kernel"))) return rc;
  std::vector<unsigned char> state((size_t)n_pt * n_rt);
  EMC_CUDA(ctx, cudaMemcpyAsync(state.data(), ps->d_state, state.size(), cudaMemcpyDeviceToHost,
                                ctx->stream));
  EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (probe_stride > 0) {
    for (int pt = 0; pt < n_pt; ++pt)
      for (int rt = pt % probe_stride; rt < n_rt; rt += probe_stride) {
        unsigned char& st = state[(size_t)pt * n_rt + rt];
        if (!st) st = 2;
      }
    EMC_CUDA(ctx, cudaMemcpyAsync(ps->d_state, state.data(), state.size(), cudaMemcpyHostToDevice,
                                  ctx->stream));
  }
  // The true-Poisson E-step evaluates 256 rotations per CTA: both 128-row
  // halves of a pair take the stronger state, so that every evaluated row is
  // also counted by the normalisation.
  const int span = p->d.diff == EMC_DIFF_TRUE_POISSON ? 2 : 1;
  if (span == 2) {
    for (int pt = 0; pt < n_pt; ++pt)
      for (int rt = 0; rt < n_rt; rt += 2) {
        unsigned char* a = &state[(size_t)pt * n_rt + rt];
        unsigned char s = a[0];
        if (rt + 1 < n_rt) {
          const unsigned char b = a[1];
          s = (s == 1 || b == 1) ? 1 : std::max(s, b);
          a[1] = s;
        }
        a[0] = s;
      }
    EMC_CUDA(ctx, cudaMemcpyAsync(ps->d_state, state.data(), state.size(), cudaMemcpyHostToDevice,
                                  ctx->stream));
  }
  // tile list in the E-step's grouped raster: 8 rotation tiles share a pattern tile
  std::vector<int2> tiles;
  long long rows = 0;  // evaluated 128-rotation row tiles
  for (int g0 = 0; g0 < n_rt; g0 += 8 * span)
    for (int pt = 0; pt < n_pt; ++pt)
      for (int rt = g0; rt < std::min(n_rt, g0 + 8 * span); rt += span)
        if (state[(size_t)pt * n_rt + rt]) {
          tiles.push_back(make_int2(pt, rt / span));
          rows += std::min(span, n_rt - rt);
        }
  ps->n_tiles = (int)tiles.size();
  ps->info.active_fraction = (double)rows / ((double)n_pt * n_rt);
  // M-step: per rotation tile, the 64-pattern k-blocks of its evaluated pattern tiles
  std::vector<int> kb_off(n_rt + 1), kb_list;
  for (int rt = 0; rt < n_rt; ++rt) {
    kb_off[rt] = (int)kb_list.size();
    for (int pt = 0; pt < n_pt; ++pt)
      if (state[(size_t)pt * n_rt + rt]) {
        kb_list.push_back(2 * pt);
        kb_list.push_back(2 * pt + 1);
      }
  }
  kb_off[n_rt] = (int)kb_list.size();
  EMC_CUDA(ctx, cudaMemcpyAsync(ps->d_kb_off, kb_off.data(), sizeof(int) * (n_rt + 1),
                                cudaMemcpyHostToDevice, ctx->stream));
  if (!kb_list.empty())
    EMC_CUDA(ctx, cudaMemcpyAsync(ps->d_kb_list, kb_list.data(), sizeof(int) * kb_list.size(),
                                  cudaMemcpyHostToDevice, ctx->stream));
  ps->info.core_fraction =
      (double)std::count(state.begin(), state.end(), (unsigned char)1) / ((double)n_pt * n_rt);
  if (!tiles.empty())
    EMC_CUDA(ctx, cudaMemcpyAsync(ps->d_tiles, tiles.data(), sizeof(int2) * tiles.size(),
                                  cudaMemcpyHostToDevice, ctx->stream));
  if (new_perm != ps->h_perm) {
    EMC_CUDA(ctx, cudaMemcpyAsync(ps->d_perm, new_perm.data(), sizeof(int) * N,
                                  cudaMemcpyHostToDevice, ctx->stream));
    if ((rc = pattern_side(p, ps->d_perm, true))) return rc;
    ps->h_perm = new_perm;
  }
  EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));  // host vectors above are staged
  // a dense mask is cheaper as a full scan
  ps->ready = arm || (ps->info.active_fraction < 0.75 &&
                      !(ps->full_every > 0 && ps->since_full + 1 >= ps->full_every));
  return EMC_OK;
}

int prune_reset(emc_plan* p) {
  PruneState* ps = pstate(p);
  if (!ps) return EMC_OK;
  ps->ready = false;
  std::iota(ps->h_perm.begin(), ps->h_perm.end(), 0);
  ps->h_perm_results = ps->h_perm;
  // p->rot / p->rotw are the new binding's buffers: reorder them again
  int rc = prune_rotation_order(p, ps);
  if (!rc) rc = prune_geometry(p, ps);
  return rc;
}

void prune_free(emc_plan* p) {
  delete pstate(p);
  p->prune = nullptr;
}

int prune_iterate(emc_plan* p, float* model, float* weight, float sigma, emc_iter_stats* stats,
                  bool* handled) {
  PruneState* ps = pstate(p);
  emc_ctx* ctx = p->ctx;
  *handled = false;
  if (!ps || !p->bound || !model || !weight) return EMC_OK;
  *handled = true;
  const int N = p->d.n_images, R = p->d.n_rot;
  const size_t n3 = (size_t)p->d.side * p->d.side * p->d.side;
  int rc;
  ps->h_perm_results = ps->h_perm;
  ps->info.pruned = 0;
  ps->info.fallback = 0;
  if (!ps->ready) {
    if ((rc = emc_iterate_async(p, model, weight, sigma))) return rc;
    if ((rc = emc_plan_wait(p, stats))) return rc;
    ps->info.full_iterations++;
    ps->since_full = 0;
    return prune_prepare(p, ps, true);
  }
  EMC_CUDA(ctx, cudaMemcpyAsync(ps->d_model_in, model, sizeof(float) * n3,
                                cudaMemcpyDeviceToDevice, ctx->stream));
  p->prune_tiles = ps->d_tiles;
  p->prune_n_tiles = ps->n_tiles;
  p->prune_state = ps->d_state;
  p->prune_margin = ps->d_margin;
  p->prune_kb_off = ps->d_kb_off;
  p->prune_kb_list = ps->d_kb_list;
  rc = emc_iterate_async(p, model, weight, sigma);
  p->prune_tiles = nullptr;
  p->prune_n_tiles = 0;
  p->prune_state = nullptr;
  p->prune_margin = nullptr;
  p->prune_kb_off = nullptr;
  p->prune_kb_list = nullptr;
  if (rc) return rc;
  if ((rc = emc_plan_wait(p, stats))) return rc;
  std::vector<double> margin(R);
  EMC_CUDA(ctx, cudaMemcpyAsync(margin.data(), ps->d_margin, sizeof(double) * R,
                                cudaMemcpyDeviceToHost, ctx->stream));
  EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  double mg = 0.0;
  for (double v : margin) mg += v;
  ps->info.margin_mass = mg / (double)N;
  ps->info.pruned = 1;
  if (ps->info.margin_mass > 1.0 - (double)ps->min_mass) {
    // the mass reached the margin: repeat the iteration as a full scan
    EMC_CUDA(ctx, cudaMemcpyAsync(model, ps->d_model_in, sizeof(float) * n3,
                                  cudaMemcpyDeviceToDevice, ctx->stream));
    if ((rc = emc_iterate_async(p, model, weight, sigma))) return rc;
    if ((rc = emc_plan_wait(p, stats))) return rc;
    ps->info.fallback = 1;
    ps->info.fallback_iterations++;
    ps->since_full = 0;
    return prune_prepare(p, ps, true);
  }
  ps->info.pruned_iterations++;
  ps->since_full++;
  return prune_prepare(p, ps, false);
}

}  // namespace emc

using namespace emc;

static int set_pruning(emc_plan* p, int on, float min_mass, float dilate, int full_every) {
  emc_ctx* ctx = p->ctx;
  if (!on) {
    if (p->prune) {
      // back to the input pattern and rotation order
      PruneState* ps = pstate(p);
      const bool permuted = !std::is_sorted(ps->h_perm.begin(), ps->h_perm.end());
      p->rot = ps->rot_in;
      p->rotw = ps->rotw_in;
      prune_free(p);
      if (permuted && p->bound) return pattern_side(p, nullptr, true);
    }
    return EMC_OK;
  }
  EMC_REQUIRE(ctx, p->bound, "plan_set_pruning: bind the plan first");
  EMC_REQUIRE(ctx, p->d.precision == EMC_PREC_MIXED,
              "plan_set_pruning: implemented for the tensor-core path");
  EMC_REQUIRE(ctx, min_mass > 0.0f && min_mass < 1.0f, "plan_set_pruning: min_mass %g", min_mass);
  EMC_REQUIRE(ctx, dilate >= 0.0f && std::isfinite(dilate), "plan_set_pruning: dilate %g", dilate);
  EMC_REQUIRE(ctx, full_every >= 0, "plan_set_pruning: full_every %d", full_every);
  PruneState* ps = pstate(p);
  const bool fresh = ps == nullptr;
  if (fresh) {
    ps = new PruneState();
    p->prune = ps;
    ps->h_perm.resize(p->d.n_images);
    std::iota(ps->h_perm.begin(), ps->h_perm.end(), 0);
    ps->h_perm_results = ps->h_perm;
    int rc = prune_alloc(p, ps);
    if (rc) {
      prune_free(p);
      return rc;
    }
  }
  ps->min_mass = min_mass;
  ps->dilate = dilate;
  ps->full_every = full_every;
  ps->since_full = 0;
  ps->tau = (1.0f - min_mass) / (10.0f * (float)p->n_rt);
  ps->ready = false;  // the next iteration is a full scan that builds the first mask
  int rc = fresh ? prune_rotation_order(p, ps) : EMC_OK;
  if (!rc) rc = prune_geometry(p, ps);
  if (rc && fresh) {
    if (ps->rot_in) {
      p->rot = ps->rot_in;
      p->rotw = ps->rotw_in;
    }
    prune_free(p);
  }
  return rc;
}

extern "C" int emc_plan_prune_info(emc_plan* p, emc_prune_info* out) {
  if (!p || !out) return EMC_ERR_INVALID;
  PruneState* ps = pstate(p);
  if (!ps) {
    *out = emc_prune_info{};
    out->active_fraction = 1.0;
    return EMC_OK;
  }
  *out = ps->info;
  out->nn_angle = ps->nn_angle;
  return EMC_OK;
}

extern "C" int emc_plan_pattern_order(emc_plan* p, int* order) {
  if (!p || !order) return EMC_ERR_INVALID;
  PruneState* ps = pstate(p);
  for (int i = 0; i < p->d.n_images; ++i) order[i] = ps ? ps->h_perm_results[i] : i;
  return EMC_OK;
}

extern "C" int emc_plan_rotation_order(emc_plan* p, int* order) {
  if (!p || !order) return EMC_ERR_INVALID;
  PruneState* ps = pstate(p);
  for (int r = 0; r < p->d.n_rot; ++r) order[r] = ps ? ps->h_rorder[r] : r;
  return EMC_OK;
}

extern "C" int emc_plan_best_quaternions(emc_plan* p, float* d_quats) {
  if (!p) return EMC_ERR_INVALID;
  emc_ctx* ctx = p->ctx;
  EMC_REQUIRE(ctx, p->bound && d_quats, "best_quaternions: plan not bound or null output");
  const int N = p->d.n_images, R = p->d.n_rot;
  PruneState* ps = pstate(p);
  const int* perm = nullptr;
  if (ps) {
    EMC_CUDA(ctx, cudaMemcpyAsync(ps->d_perm_res, ps->h_perm_results.data(), sizeof(int) * N,
                                  cudaMemcpyHostToDevice, ctx->stream));
    perm = ps->d_perm_res;
  }
  int rr = plan_respons_ready(p);
  if (rr) return rr;
  best_quat_kernel<<<ceil_div(N, 256), 256, 0, ctx->stream>>>(p->L, R, N, p->rot, perm, d_quats);
  int rc = after_launch(ctx, "best_quat_kernel");
  if (!rc) EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));  // the host perm is staged
  return rc;
}

// Fraction of the rotation group SO(3) (uniform measure) within angle theta
// of a rotation: (theta - sin theta) / pi.
static double ball_angle(double fraction) {
  double lo = 0.0, hi = M_PI;
  for (int it = 0; it < 100; ++it) {
    const double mid = 0.5 * (lo + hi);
    if ((mid - std::sin(mid)) / M_PI < fraction)
      lo = mid;
    else
      hi = mid;
  }
  return 0.5 * (lo + hi);
}

extern "C" int emc_plan_set_proposals(emc_plan* p, const float* d_quats, int n_modes,
                                      float fraction, int probe_stride) {
  if (!p) return EMC_ERR_INVALID;
  emc_ctx* ctx = p->ctx;
  PruneState* ps = pstate(p);
  EMC_REQUIRE(ctx, ps && p->bound, "set_proposals: pruning is off or the plan is not bound");
  EMC_REQUIRE(ctx, d_quats && n_modes >= 1 && n_modes <= 8 && fraction > 0.0f &&
                       fraction < 1.0f && probe_stride >= 0,
              "set_proposals: bad arguments");
  const int N = p->d.n_images, R = p->d.n_rot, n_rt = p->n_rt, n_pt = p->Np / 128;
  const float cos_half = (float)std::cos(0.5 * ball_angle((double)fraction));
  int rc;
  // patterns sorted by the rotation row nearest to their first proposal
  nearest_row_kernel<<<ceil_div(N, 256), 256, 0, ctx->stream>>>(d_quats, n_modes, p->rot, R, N,
                                                                ps->d_best);
  if ((rc = after_launch(ctx, "nearest_row_kernel"))) return rc;
  std::vector<int> best(N), order(N), newpos(N);
  EMC_CUDA(ctx, cudaMemcpyAsync(best.data(), ps->d_best, sizeof(int) * N, cudaMemcpyDeviceToHost,
                                ctx->stream));
  EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return best[a] < best[b]; });
  for (int j = 0; j < N; ++j) newpos[order[j]] = j;
  EMC_CUDA(ctx, cudaMemcpyAsync(ps->d_newpos, newpos.data(), sizeof(int) * N,
                                cudaMemcpyHostToDevice, ctx->stream));
  EMC_CUDA(ctx, cudaMemsetAsync(ps->d_core, 0, (size_t)n_pt * n_rt, ctx->stream));
  proposal_core_kernel<<<dim3(ceil_div(N, 128), n_rt), 128, 0, ctx->stream>>>(
      d_quats, n_modes, p->rot, R, N, ps->d_newpos, cos_half, n_rt, ps->d_core);
  if ((rc = after_launch(ctx, "proposal_core_kernel"))) return rc;
  return prune_finish(p, ps, order, probe_stride, true);  // order: position -> input pattern
}

extern "C" int emc_plan_set_pruning(emc_plan* p, int on, float min_mass, float dilate,
                                    int full_every) {
  if (!p) return EMC_ERR_INVALID;
  int rc = set_pruning(p, on, min_mass, dilate, full_every);
  // the rotation order may have changed: the sorted insertion's voxel map follows it
  const int rc2 = sorted_ensure(p);
  return rc ? rc : rc2;
}
