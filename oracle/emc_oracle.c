/*
 * emc_oracle.c -- CPU restatement of the reference EMC kernels.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA path: it
 * is built into oracle/_build/liboracle.so and loaded only by tests/,
 * __graft_entry__.smoke() and the CPU-baseline leg of bench.py.  The product
 * library never links or calls it.
 *
 * Every function restates one reference kernel and follows the reference's
 * order of float operations: the 512 "threads" of a reference block become a
 * loop over t = 0..511 that accumulates pixels t, t+512, ..., and the block's
 * shared-memory tree becomes data[t] += data[t+s] for s = 256..1.  Multiply-add
 * contractions that nvcc applies to the reference source are written as
 * explicit fmaf(); the file is compiled with -ffp-contract=off so the C
 * compiler adds none of its own.  OpenMP parallelises over independent
 * (rotation, pattern) pairs only, never inside a sum, so results do not
 * depend on the thread count.
 *
 * Sources restated (file:line in the reference):
 *   slice           emc_cuda.cu:102-157
 *   scaling         emc_cuda.cu:438-454, 516-532
 *   likelihood      emc_cuda.cu:159-216, 242-276
 *   max / sumexp    emc_cuda.cu:1041-1056, 1175-1202
 *   normalise resp  emc_cuda.cu:1253-1260, main.cpp:384-391
 *   update slices   emc_atomic.cu:88-132
 *   insert          emc_atomic.cu:33-85, 183-200
 *   divide          emc_cuda.cu:758-786
 *   model average   emc_cuda.cu:639-671, 788-798
 *   preprocessing   emc_helper.cpp:226-243 (binning), 389-438 (normalise),
 *                   567-575 (per-pattern masks), 458-518 (model init 3 and 1),
 *                   81-135 (host insert_slice)
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define VT 512 /* threads of a reference block (TNUM, emc_cuda_help.h:8) */

/* ---- geometry ------------------------------------------------------------ */
static void quat_to_matrix(const float* q, float m[9]) {
  const float a = q[0], b = q[1], c = q[2], d = q[3];
  const float a2 = 2.0f * a, b2 = 2.0f * b, c2 = 2.0f * c;
  m[0] = fmaf(-d, d, fmaf(-c, c, fmaf(b, b, a * a)));
  m[1] = fmaf(-a2, d, b2 * c);
  m[2] = fmaf(a2, c, b2 * d);
  m[3] = fmaf(a2, d, b2 * c);
  m[4] = fmaf(-d, d, fmaf(c, c, fmaf(-b, b, a * a)));
  m[5] = fmaf(-a2, b, c2 * d);
  m[6] = fmaf(-a2, c, b2 * d);
  m[7] = fmaf(a2, b, c2 * d);
  m[8] = fmaf(d, d, fmaf(-c, c, fmaf(-b, b, a * a)));
}

static inline float rot_row(const float m[9], int row, float x, float y, float z) {
  return fmaf(m[3 * row + 2], z, fmaf(m[3 * row + 1], y, m[3 * row] * x));
}

static inline float vcoord(int side, float c) {
  const float off = (float)side / 2.0f - 0.5f;
  return off + c;
}

void oracle_rot_matrix(const float* q, float* m) { quat_to_matrix(q, m); }

/* Nearest voxel index of pixel p under rotation q; -1 when outside.  lo is
 * the lowest valid index (1 for slicing, 0 for insertion). */
static long nearest_voxel(const float m[9], int side, float x, float y, float z, int lo) {
  const long ix = lroundf(vcoord(side, rot_row(m, 0, x, y, z)));
  const long iy = lroundf(vcoord(side, rot_row(m, 1, x, y, z)));
  const long iz = lroundf(vcoord(side, rot_row(m, 2, x, y, z)));
  if (ix < lo || ix >= side || iy < lo || iy >= side || iz < lo || iz >= side) return -1;
  return (iz * side + iy) * side + ix;
}

/* emc_cuda.cu:102-157 (nearest) and the trilinear gather of the new path. */
void oracle_get_slices(const float* model, int side, float* slices, const float* rot,
                       const float* xc, const float* yc, const float* zc, int n_rot,
                       int interp) {
  const int n2 = side * side;
#pragma omp parallel for schedule(static)
  for (int r = 0; r < n_rot; ++r) {
    float m[9];
    quat_to_matrix(rot + 4 * (size_t)r, m);
    for (int p = 0; p < n2; ++p) {
      const float x = xc[p], y = yc[p], z = zc[p];
      float v;
      if (interp == 0) {
        const long vi = nearest_voxel(m, side, x, y, z, 1);
        v = vi >= 0 ? model[vi] : -1.0f;
      } else {
        const float cx = vcoord(side, rot_row(m, 0, x, y, z));
        const float cy = vcoord(side, rot_row(m, 1, x, y, z));
        const float cz = vcoord(side, rot_row(m, 2, x, y, z));
        const float fx0 = floorf(cx), fy0 = floorf(cy), fz0 = floorf(cz);
        const int x0 = (int)fx0, y0 = (int)fy0, z0 = (int)fz0;
        const float tx = cx - fx0, ty = cy - fy0, tz = cz - fz0;
        float acc = 0.0f, wsum = 0.0f;
        for (int c = 0; c < 8; ++c) {
          const int xi = x0 + (c & 1), yi = y0 + ((c >> 1) & 1), zi = z0 + (c >> 2);
          if (xi < 0 || xi >= side || yi < 0 || yi >= side || zi < 0 || zi >= side) continue;
          const float w = ((c & 1) ? tx : 1.0f - tx) * (((c >> 1) & 1) ? ty : 1.0f - ty) *
                          ((c >> 2) ? tz : 1.0f - tz);
          const float val = model[((size_t)zi * side + yi) * side + xi];
          if (val < 0.0f || w <= 0.0f) continue;
          acc = fmaf(w, val, acc);
          wsum += w;
        }
        v = wsum > 1e-6f ? acc / wsum : -1.0f;
      }
      slices[(size_t)r * n2 + p] = v;
    }
  }
}

/* The reference's shared-memory tree (inblock_reduce, emc_cuda.cu:49-58). */
static float tree_f(float* d) {
  for (int s = VT / 2; s > 0; s >>= 1)
    for (int t = 0; t < s; ++t) d[t] = d[t] + d[t + s];
  return d[0];
}
static int tree_i(int* d) {
  for (int s = VT / 2; s > 0; s >>= 1)
    for (int t = 0; t < s; ++t) d[t] = d[t] + d[t + s];
  return d[0];
}

/* emc_cuda.cu:438-454 + 516-532: scaling[(start+r)*N + i]. */
void oracle_update_scaling_full(const float* images, const float* slices, const int* mask,
                                float* scaling, int n2, int n_images, int start, int chunk) {
#pragma omp parallel for collapse(2) schedule(static)
  for (int r = 0; r < chunk; ++r) {
    for (int i = 0; i < n_images; ++i) {
      float num[VT];
      int den[VT];
      const float* img = images + (size_t)i * n2;
      const float* sl = slices + (size_t)r * n2;
      for (int t = 0; t < VT; ++t) {
        float a = 0.0f;
        int b = 0;
        for (int p = t; p < n2; p += VT) {
          if (mask[p] > 0 && (double)sl[p] > 1e-10 && (double)img[p] > 1e-10) {
            a = fmaf(img[p], img[p], a);
            b = (int)fmaf(img[p], sl[p], (float)b); /* int += float: truncation */
          }
        }
        num[t] = a;
        den[t] = b;
      }
      const float fn = tree_f(num);
      const int id = tree_i(den);
      scaling[(size_t)(start + r) * n_images + i] = fn / (float)id;
    }
  }
}

/* emc_cuda.cu:159-216, 242-276: respons[(start+r)*N + i] (log scale). */
void oracle_calculate_responsabilities(const float* slices, const float* images, const int* mask,
                                       float sigma, const float* scaling, float* respons,
                                       const float* weights, int n2, int n_images, int start,
                                       int chunk, int diff) {
#pragma omp parallel for collapse(2) schedule(static)
  for (int r = 0; r < chunk; ++r) {
    for (int i = 0; i < n_images; ++i) {
      float sum[VT];
      int cnt[VT];
      const float* img = images + (size_t)i * n2;
      const float* sl = slices + (size_t)r * n2;
      const float phi = scaling[(size_t)(start + r) * n_images + i];
      for (int t = 0; t < VT; ++t) {
        float a = 0.0f;
        int c = 0;
        for (int p = t; p < n2; p += VT) {
          if (mask[p] != 0 && sl[p] > 0.0f) {
            const float d = sl[p] - img[p] / phi;
            if (diff == 1) { /* poisson: FP64 per pixel */
              const double q = (double)d / sqrt((double)sl[p] + 0.02);
              a = (float)((double)a + q * q);
            } else if (diff == 0) {
              a = fmaf(d, d, a);
            } else {
              const float q = d / sl[p];
              a = fmaf(q, q, a);
            }
            c++;
          }
        }
        sum[t] = a;
        cnt[t] = c;
      }
      const float s = tree_f(sum);
      const int c = tree_i(cnt);
      const double lw = (double)logf(weights[start + r]);
      const double v = (double)s / 2.0 / (double)(float)c / (double)(sigma * sigma);
      respons[(size_t)(start + r) * n_images + i] = (float)(lw - v);
    }
  }
}

/* emc_cuda.cu:1041-1056 */
void oracle_max_vector(const float* respons, int n_images, int n_slices, float* maxr) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n_images; ++i) {
    float cache[VT];
    for (int t = 0; t < VT; ++t) {
      float m = -1.0e10f;
      for (int r = t; r < n_slices; r += VT) {
        const float v = respons[(size_t)r * n_images + i];
        if (m < v) m = v;
      }
      cache[t] = m;
    }
    for (int s = VT / 2; s > 0; s >>= 1)
      for (int t = 0; t < s; ++t)
        if (cache[t] < cache[t + s]) cache[t] = cache[t + s];
    maxr[i] = cache[0];
  }
}

/* emc_cuda.cu:1175-1202 (the temporary is not kept). */
void oracle_respons_max_expf(const float* respons, const float* maxv, int n_images, int n_slices,
                             float* out_sum) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n_images; ++i) {
    float cache[VT];
    for (int t = 0; t < VT; ++t) {
      float s = 0.0f;
      for (int r = t; r < n_slices; r += VT) {
        const float d = respons[(size_t)r * n_images + i] - maxv[i];
        if (d > -1.0e10f) s = s + expf(d);
      }
      cache[t] = s;
    }
    out_sum[i] = tree_f(cache);
  }
}

/* main.cpp:384-392: lse = logf(sum) + max on the host, then respons =
 * expf(respons - lse) (emc_cuda.cu:1253-1260). */
void oracle_normalize_respons(float* respons, const float* sum, const float* maxv, int n_images,
                              int n_slices, float* lse_out) {
  for (int i = 0; i < n_images; ++i) lse_out[i] = logf(sum[i]) + maxv[i];
#pragma omp parallel for schedule(static)
  for (int r = 0; r < n_slices; ++r)
    for (int i = 0; i < n_images; ++i) {
      float* e = respons + (size_t)r * n_images + i;
      *e = expf(*e - lse_out[i]);
    }
}

/* emc_atomic.cu:88-132: slices of the chunk and their totals. */
void oracle_update_slices(const float* images, float* slices, const int* mask,
                          const float* respons, const float* scaling, const int* active,
                          int n_images, int start, int chunk, int n2, float* totals) {
#pragma omp parallel for schedule(static)
  for (int r = 0; r < chunk; ++r) {
    const float* resp = respons + (size_t)(start + r) * n_images;
    const float* scal = scaling + (size_t)(start + r) * n_images;
    float total = 0.0f;
    for (int i = 0; i < n_images; ++i)
      if (active[i] > 0) total = total + resp[i];
    totals[r] = total;
    for (int p = 0; p < n2; ++p) {
      float v = -1.0f;
      if (mask[p] != 0) {
        float s = 0.0f;
        for (int i = 0; i < n_images; ++i)
          if (active[i] > 0) s = s + (images[(size_t)i * n2 + p] * resp[i]) / scal[i];
        v = s;
        if (total > 1e-10f) v = v / total;
      }
      slices[(size_t)r * n2 + p] = v;
    }
  }
}

/* emc_atomic.cu:33-85, 183-200: sequential insertion (rotation order, then
 * pixel order).  rot points at the chunk's first quaternion. */
void oracle_insert_slices(const float* slices, const int* mask, const float* totals,
                          const float* rot, const float* xc, const float* yc, const float* zc,
                          int side, int chunk, float* model, float* weight) {
  const int n2 = side * side;
  for (int r = 0; r < chunk; ++r) {
    const float w = totals[r];
    if (!(w > 1e-10f)) continue;
    float m[9];
    quat_to_matrix(rot + 4 * (size_t)r, m);
    for (int p = 0; p < n2; ++p) {
      const float s = slices[(size_t)r * n2 + p];
      if (mask[p] != 1 || !(s >= 0.0f)) continue;
      const long v = nearest_voxel(m, side, xc[p], yc[p], zc[p], 0);
      if (v < 0) continue;
      model[v] += w * s;
      weight[v] += w;
    }
  }
}

/* emc_cuda.cu:758-786 */
void oracle_divide_model(float* model, const float* weight, long n) {
  for (long i = 0; i < n; ++i) model[i] = weight[i] > 0.0f ? model[i] / weight[i] : -1.0f;
}

/* emc_cuda.cu:639-661: float mean of the positive voxels (512-way order). */
float oracle_model_average(const float* model, long n) {
  float s[VT];
  int c[VT];
  for (int t = 0; t < VT; ++t) {
    float a = 0.0f;
    int k = 0;
    for (long i = t; i < n; i += VT)
      if (model[i] > 0.0f) {
        a = a + model[i];
        k++;
      }
    s[t] = a;
    c[t] = k;
  }
  const float fs = tree_f(s);
  const int ic = tree_i(c);
  return ic > 0 ? fs / (float)ic : 0.0f;
}

/* emc_cuda.cu:788-798 */
float oracle_normalize_model(float* model, long n) {
  const float avg = oracle_model_average(model, n);
  const float inv = 1.0f / avg;
  for (long i = 0; i < n; ++i) model[i] = model[i] * inv;
  return avg;
}

/* Voxel index of every (rotation, pixel) pair with the kernels' arithmetic:
 * nearest (lroundf, bounds [lo, side)), -1 outside. */
void oracle_nearest_voxels(const float* rot, int R, const float* xc, const float* yc,
                           const float* zc, int P, int side, int lo, long long* out) {
#pragma omp parallel for schedule(static)
  for (int r = 0; r < R; ++r) {
    float m[9];
    quat_to_matrix(rot + 4 * (size_t)r, m);
    for (int p = 0; p < P; ++p) out[(size_t)r * P + p] = nearest_voxel(m, side, xc[p], yc[p], zc[p], lo);
  }
}

/* Trilinear stencil of every (rotation, pixel): 8 voxel indices and weights
 * (weight 0 and index 0 for corners outside the volume). */
void oracle_trilinear_stencil(const float* rot, int R, const float* xc, const float* yc,
                              const float* zc, int P, int side, long long* vox, float* wts) {
#pragma omp parallel for schedule(static)
  for (int r = 0; r < R; ++r) {
    float m[9];
    quat_to_matrix(rot + 4 * (size_t)r, m);
    for (int p = 0; p < P; ++p) {
      const float cx = vcoord(side, rot_row(m, 0, xc[p], yc[p], zc[p]));
      const float cy = vcoord(side, rot_row(m, 1, xc[p], yc[p], zc[p]));
      const float cz = vcoord(side, rot_row(m, 2, xc[p], yc[p], zc[p]));
      const float fx0 = floorf(cx), fy0 = floorf(cy), fz0 = floorf(cz);
      const int x0 = (int)fx0, y0 = (int)fy0, z0 = (int)fz0;
      const float tx = cx - fx0, ty = cy - fy0, tz = cz - fz0;
      for (int c = 0; c < 8; ++c) {
        const int xi = x0 + (c & 1), yi = y0 + ((c >> 1) & 1), zi = z0 + (c >> 2);
        const size_t o = ((size_t)r * P + p) * 8 + c;
        const float w = ((c & 1) ? tx : 1.0f - tx) * (((c >> 1) & 1) ? ty : 1.0f - ty) *
                        ((c >> 2) ? tz : 1.0f - tz);
        if (xi < 0 || xi >= side || yi < 0 || yi >= side || zi < 0 || zi >= side) {
          vox[o] = 0;
          wts[o] = 0.0f;
        } else {
          vox[o] = ((long long)zi * side + yi) * side + xi;
          wts[o] = w;
        }
      }
    }
  }
}

/* ---- preprocessing and model initialisation (host code of the reference) -- */

/* read_images binning, emc_helper.cpp:226-243: output (x, y) sums |raw| and
 * the raw mask over a stride x stride block starting at
 * (int)(stride * ((real)(o - side/2) + 0.5) + raw/2 - 0.5) per axis (double
 * arithmetic, xb outer, yb inner); value = float sum / (real)mask sum, mask =
 * mask sum > 1.  Raw pixels outside the frame count as 0 (the reference
 * reads them unchecked).  Layouts: raw [n][raw_h][raw_w], out [n][side][side],
 * x fastest. */
void oracle_bin_images(const float* raw, const int* raw_mask, int raw_w, int raw_h, int n,
                       int side, int stride, float* images, int* masks) {
  for (int i = 0; i < n; ++i)
    for (int y = 0; y < side; ++y)
      for (int x = 0; x < side; ++x) {
        const int sx0 = (int)(stride * ((double)(float)(x - side / 2) + 0.5) + raw_w / 2 - 0.5);
        const int sy0 = (int)(stride * ((double)(float)(y - side / 2) + 0.5) + raw_h / 2 - 0.5);
        float psum = 0.0f;
        int msum = 0;
        for (int xb = 0; xb < stride; ++xb)
          for (int yb = 0; yb < stride; ++yb) {
            const int sx = sx0 + xb, sy = sy0 + yb;
            if (sx < 0 || sx >= raw_w || sy < 0 || sy >= raw_h) continue;
            const size_t e = ((size_t)i * raw_h + sy) * raw_w + sx;
            psum += fabsf(raw[e]);
            msum += raw_mask[e];
          }
        const size_t o = ((size_t)i * side + y) * side + x;
        images[o] = psum / (float)msum;
        masks[o] = msum > 1 ? 1 : 0;
      }
}

/* normalize_images_central_part (emc_helper.cpp:389-418, whose central mask
 * is 1 everywhere) and normalize_images_individual_mask (:421-438, masks !=
 * NULL): factor (real)N_2d / (sequential float sum where mask == 1), images
 * *= factor.  Returns the factors in factor[n]. */
void oracle_normalize_images(float* images, const int* mask, const int* masks, int n2, int n,
                             float* factor) {
  for (int i = 0; i < n; ++i) {
    const int* m = masks ? masks + (size_t)i * n2 : mask;
    float sum = 0.0f;
    for (int p = 0; p < n2; ++p)
      if (m[p] == 1) sum += images[(size_t)i * n2 + p];
    sum = (float)n2 / sum;
    factor[i] = sum;
    for (int p = 0; p < n2; ++p) images[(size_t)i * n2 + p] *= sum;
  }
}

/* mask_model, emc_helper.cpp:567-575. */
void oracle_mask_images(float* images, const int* masks, long n) {
  for (long e = 0; e < n; ++e)
    if (masks[e] == 0) images[e] = -1.0f;
}

/* model_init, model_input 3, emc_helper.cpp:458-502.  radavg[r] accumulates
 * pattern values in float over i, x, y (sequential, as the reference) when
 * float_sums, else in double; then radavg /= (real)count.  radavg has side/2
 * + 1 entries, the last 0 (the reference reads one past its array).  The
 * model value is computed in double and stored as float; -1 outside. */
void oracle_model_init_radial(const float* images, int n, int side, int float_sums,
                              float* radavg_out, float* model) {
  const int nr = side / 2;
  float* radavg = (float*)calloc((size_t)nr + 1, sizeof(float));
  double* dsum = (double*)calloc((size_t)nr + 1, sizeof(double));
  int* cnt = (int*)calloc((size_t)nr + 1, sizeof(int));
  const double h = (double)side / 2.0;
  for (int i = 0; i < n; ++i)
    for (int x = 0; x < side; ++x)
      for (int y = 0; y < side; ++y) {
        const double dx = (double)(float)x - h + 0.5, dy = (double)(float)y - h + 0.5;
        const int r = (int)sqrt(dx * dx + dy * dy);
        if (r < h) {
          const float v = images[((size_t)i * side + y) * side + x];
          if (float_sums)
            radavg[r] += v;
          else
            dsum[r] += (double)v;
          cnt[r] += 1;
        }
      }
  for (int r = 0; r < nr; ++r) {
    if (!float_sums) radavg[r] = (float)dsum[r];
    radavg[r] = cnt[r] > 0 ? radavg[r] / (float)cnt[r] : 0.0f;
  }
  radavg[nr] = 0.0f;
  for (int x = 0; x < side; ++x)
    for (int y = 0; y < side; ++y)
      for (int z = 0; z < side; ++z) {
        const double dx = (double)(float)x - h + 0.5, dy = (double)(float)y - h + 0.5,
                     dz = (double)(float)z - h + 0.5;
        /* `real rad` in the reference (emc_helper.cpp:487): the double root
           rounded to float; rad - r is a float difference, the first product
           double (1.0 is a double literal), the second a float product */
        const float rad = (float)sqrt(dx * dx + dy * dy + dz * dz);
        const int r = (int)rad;
        const size_t v = ((size_t)z * side + y) * side + x;
        if (r < h) {
          const float f = rad - (float)r;
          const float hi = radavg[r + 1] * f;
          model[v] = (float)((double)radavg[r] * (1.0 - (double)f) + (double)hi);
        } else
          model[v] = -1.0f;
      }
  if (radavg_out) memcpy(radavg_out, radavg, sizeof(float) * ((size_t)nr + 1));
  free(radavg);
  free(dsum);
  free(cnt);
}

/* Voxel of pixel p of the common mask for quaternion q under the host
 * insert_slice (emc_helper.cpp:81-135): float diagonal terms, double
 * off-diagonal terms (2.0 * ...), coordinate sums in double stored to float,
 * round(side/2.0 + 0.5 + c), bounds [0, side).  Returns -1 outside. */
static long host_insert_voxel(const float* q, int side, float x, float y, float z) {
  const float q0 = q[0], q1 = q[1], q2 = q[2], q3 = q[3];
  const float nx = (q0 * q0 + q1 * q1 - q2 * q2 - q3 * q3) * x +
                   (2.0 * q1 * q2 - 2.0 * q0 * q3) * y + (2.0 * q1 * q3 + 2.0 * q0 * q2) * z;
  const float ny = (2.0 * q1 * q2 + 2.0 * q0 * q3) * x +
                   (q0 * q0 - q1 * q1 + q2 * q2 - q3 * q3) * y +
                   (2.0 * q2 * q3 - 2.0 * q0 * q1) * z;
  const float nz = (2.0 * q1 * q3 - 2.0 * q0 * q2) * x + (2.0 * q2 * q3 + 2.0 * q0 * q1) * y +
                   (q0 * q0 - q1 * q1 - q2 * q2 + q3 * q3) * z;
  const int rx = (int)round((float)side / 2.0 + 0.5 + nx);
  const int ry = (int)round((float)side / 2.0 + 0.5 + ny);
  const int rz = (int)round((float)side / 2.0 + 0.5 + nz);
  if (rx < 0 || rx >= side || ry < 0 || ry >= side || rz < 0 || rz >= side) return -1;
  return ((long)rz * side + ry) * side + rx;
}

/* model_init, model_input 1, emc_helper.cpp:503-518: every pattern inserted
 * once, weight 1, at quats[i] (in pattern order, pixels x outer, y inner as
 * insert_slice), then model /= weight where weight > 0, else 0. */
void oracle_model_init_orientations(const float* images, const int* mask, int n, int side,
                                    const float* quats, const float* xc, const float* yc,
                                    const float* zc, float* model, float* weight) {
  const long n3 = (long)side * side * side;
  memset(model, 0, sizeof(float) * n3);
  memset(weight, 0, sizeof(float) * n3);
  for (int i = 0; i < n; ++i)
    for (int x = 0; x < side; ++x)
      for (int y = 0; y < side; ++y) {
        const int p = y * side + x;
        if (mask[p] != 1) continue;
        const long v = host_insert_voxel(quats + 4 * (size_t)i, side, xc[p], yc[p], zc[p]);
        if (v < 0) continue;
        model[v] = model[v] + 1.0f * images[(size_t)i * side * side + p];
        weight[v] = weight[v] + 1.0f;
      }
  for (long v = 0; v < n3; ++v) model[v] = weight[v] > 0.0f ? model[v] / weight[v] : 0.0f;
}
