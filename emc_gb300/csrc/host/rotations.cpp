// 600-cell rotation sampling (host input of the EMC iteration).
//
// Restates the sampling scheme of rotations.c:43-458 (generate_rotation_list,
// n_to_samples, scalar_product_with_best_center): the 120 vertices of the
// 600-cell are joined into 720 edges, 1200 faces and 600 cells by distance
// cut-offs; every edge, face and cell is subdivided at level n; every sample is
// weighted by  f * <q, nearest cell centre> / |q|^3 / samples ; the q0 > 0
// hemisphere is kept (lexicographic tie-break), the kept weights are divided
// by their float sum, and the kept quaternions are normalised.
//
// The output must be bit-identical to the reference build, because the vertex,
// edge and face tests compare rounded sums against 3.0 / 7.5 / 13.5 and the
// 60-degree vertex pairs sit exactly on the 3.0 cut-off.  Every expression
// therefore keeps the reference's mix of float storage and double
// intermediates; the translation unit is built with -ffp-contract=off so that
// no multiply-add is fused on either x86-64 or aarch64.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../../include/emc_gb300.h"

namespace {

struct Quat {
  float q[4];
};

// Vertex ordering of the 96 "golden" vertices: the 12 even permutations of
// the four quaternion slots (rotations.c:130-141), 0-based.  The table fixes
// the vertex order and hence every later index, so it is data, not derived.
const int kEvenPerm[12][4] = {{0, 1, 2, 3}, {0, 3, 1, 2}, {0, 2, 3, 1}, {1, 2, 0, 3},
                              {1, 3, 2, 0}, {1, 0, 3, 2}, {2, 0, 1, 3}, {2, 3, 0, 1},
                              {2, 1, 3, 0}, {3, 1, 0, 2}, {3, 2, 1, 0}, {3, 0, 2, 1}};

// Squared norm of a sum of float quaternion components, accumulated the way
// the reference does it: each component sum in float, squared and summed in
// double, the result rounded to float.
inline float sum_sq_to_float(const double c[4]) {
  return (float)(c[0] * c[0] + c[1] * c[1] + c[2] * c[2] + c[3] * c[3]);
}

inline double norm_d(const Quat& a) {
  return std::sqrt((double)a.q[0] * a.q[0] + (double)a.q[1] * a.q[1] +
                   (double)a.q[2] * a.q[2] + (double)a.q[3] * a.q[3]);
}

// <q, c> / |q| for the cell centre c with the largest such value (strictly
// greater wins, first index on ties), rotations.c:60-76.
float best_center_dot(const Quat& a, const float* centers) {
  const double nrm = norm_d(a);
  float best = 0.0f;
  int best_i = 0;
  for (int i = 0; i < 600; ++i) {
    const float* c = centers + 4 * i;
    float num = a.q[0] * c[0];
    num = num + a.q[1] * c[1];
    num = num + a.q[2] * c[2];
    num = num + a.q[3] * c[3];
    const float d = (float)((double)num / nrm);
    if (d > best) {
      best = d;
      best_i = i;
    }
  }
  const float* c = centers + 4 * best_i;
  float num = a.q[0] * c[0];
  num = num + a.q[1] * c[1];
  num = num + a.q[2] * c[2];
  num = num + a.q[3] * c[3];
  return (float)((double)num / nrm);
}

inline float inv_norm_cubed_weight(const Quat& a) {
  const double s = (double)a.q[0] * a.q[0] + (double)a.q[1] * a.q[1] +
                   (double)a.q[2] * a.q[2] + (double)a.q[3] * a.q[3];
  return (float)std::pow(s, 1.5);
}

}  // namespace

extern "C" int emc_rotation_count(int n) {
  if (n < 1 || n > 64) return -1;
  // rotations.c:43 gives 20*(n+5n^3) samples over the full sphere; half are kept.
  const long full = 20L * ((long)n + 5L * (long)n * n * n);
  return (int)(full / 2);
}

extern "C" int emc_generate_rotations(int n, float* quats, float* weights, int capacity) {
  const int n_keep = emc_rotation_count(n);
  if (n_keep < 0 || quats == nullptr || weights == nullptr) return EMC_ERR_INVALID;
  if (capacity < n_keep) return EMC_ERR_INVALID;

  const float tau = (float)((1.0 + std::sqrt(5.0)) / 2.0);

  // --- 120 vertices -------------------------------------------------------
  Quat v[120];
  std::memset(v, 0, sizeof(v));
  for (int idx = 0; idx < 16; ++idx) {  // (+-1/2, +-1/2, +-1/2, +-1/2)
    for (int k = 0; k < 4; ++k) v[idx].q[k] = -0.5f + (float)((idx >> (3 - k)) & 1);
  }
  for (int i = 0; i < 8; ++i) v[16 + i].q[i / 2] = -1.0f + 2.0f * (float)(i % 2);  // (+-1,0,0,0)
  for (int p = 0; p < 12; ++p) {  // even permutations of (+-1/2, +-tau/2, +-1/(2tau), 0)
    for (int j = 0; j < 8; ++j) {
      const int j1 = (j >> 2) & 1, j2 = (j >> 1) & 1, j3 = j & 1;
      Quat& o = v[24 + 8 * p + j];
      o.q[kEvenPerm[p][0]] = (float)(-0.5 + 1.0 * (float)j1);
      o.q[kEvenPerm[p][1]] = (float)((double)tau * (-0.5 + 1.0 * (float)j2));
      o.q[kEvenPerm[p][2]] = (float)(1.0 / (double)tau * (-0.5 + 1.0 * (float)j3));
      o.q[kEvenPerm[p][3]] = 0.0f;
    }
  }

  // --- edges: vertex pairs with |a+b|^2 > 3 --------------------------------
  int edges[720][2];
  int n_edges = 0;
  for (int i = 0; i < 120; ++i) {
    for (int j = 0; j < i; ++j) {
      double c[4];
      for (int k = 0; k < 4; ++k) c[k] = (double)(v[i].q[k] + v[j].q[k]);
      if (sum_sq_to_float(c) > 3.0f) {
        if (n_edges >= 720) return EMC_ERR_INTERNAL;
        edges[n_edges][0] = i;
        edges[n_edges][1] = j;
        ++n_edges;
      }
    }
  }
  if (n_edges != 720) return EMC_ERR_INTERNAL;

  // --- faces: edge + vertex with |a+b+c|^2 > 7.5; a vertex that has appeared
  // in any edge processed so far is not used as the third corner ------------
  int faces[1200][3];
  int n_faces = 0;
  bool vert_used[120] = {false};
  for (int e = 0; e < 720; ++e) {
    vert_used[edges[e][0]] = true;
    vert_used[edges[e][1]] = true;
    for (int j = 0; j < 120; ++j) {
      if (vert_used[j]) continue;
      double c[4];
      for (int k = 0; k < 4; ++k) {
        float s = v[j].q[k] + v[edges[e][0]].q[k];
        s = s + v[edges[e][1]].q[k];
        c[k] = (double)s;
      }
      if (sum_sq_to_float(c) > 7.5f) {
        if (n_faces >= 1200) return EMC_ERR_INTERNAL;
        faces[n_faces][0] = edges[e][0];
        faces[n_faces][1] = edges[e][1];
        faces[n_faces][2] = j;
        ++n_faces;
      }
    }
  }
  if (n_faces != 1200) return EMC_ERR_INTERNAL;

  // --- cells: face + vertex with |a+b+c+d|^2 > 13.5; vertex j is retired
  // before its faces are scanned, so each cell is found once ---------------
  int cells[600][4];
  std::vector<float> centers(4 * 600);
  int n_cells = 0;
  bool vert_done[120] = {false};
  for (int j = 0; j < 120; ++j) {
    vert_done[j] = true;
    for (int f = 0; f < 1200; ++f) {
      if (vert_done[faces[f][0]] || vert_done[faces[f][1]] || vert_done[faces[f][2]]) continue;
      double c[4];
      for (int k = 0; k < 4; ++k) {
        float s = v[faces[f][0]].q[k] + v[faces[f][1]].q[k];
        s = s + v[faces[f][2]].q[k];
        s = s + v[j].q[k];
        c[k] = (double)s;
      }
      if (sum_sq_to_float(c) > 13.5f) {
        if (n_cells >= 600) return EMC_ERR_INTERNAL;
        int* cl = cells[n_cells];
        cl[0] = faces[f][0];
        cl[1] = faces[f][1];
        cl[2] = faces[f][2];
        cl[3] = j;
        float* ctr = &centers[4 * n_cells];
        for (int k = 0; k < 4; ++k) {
          float s = v[cl[0]].q[k] + v[cl[1]].q[k];
          s = s + v[cl[2]].q[k];
          s = s + v[cl[3]].q[k];
          ctr[k] = s;
        }
        const float nrm = (float)std::sqrt((double)ctr[0] * ctr[0] + (double)ctr[1] * ctr[1] +
                                           (double)ctr[2] * ctr[2] + (double)ctr[3] * ctr[3]);
        for (int k = 0; k < 4; ++k) ctr[k] = ctr[k] / nrm;
        ++n_cells;
      }
    }
  }
  if (n_cells != 600) return EMC_ERR_INTERNAL;

  // --- weight factors per sample class (rotations.c:257-262) ---------------
  const float alpha = (float)std::acos(1.0 / 3.0);
  const float f1 = (float)(5.0 * (double)alpha / 2.0 / M_PI);
  const float f0 = (float)(20.0 * (3.0 * (double)alpha - M_PI) / 4.0 / M_PI);
  const float f2 = 1.0f, f3 = 1.0f;

  const int n_samples = 2 * n_keep;
  const float ns = (float)n_samples;
  std::vector<Quat> all(n_samples);
  std::vector<float> w(n_samples);
  auto weigh = [&](int idx, float f) {
    const float dist3 = inv_norm_cubed_weight(all[idx]);
    const float sp = best_center_dot(all[idx], centers.data());
    float t = f * sp;
    t = t / ns;
    w[idx] = t / dist3;
  };

  for (int i = 0; i < 120; ++i) {
    all[i] = v[i];
    weigh(i, f0);
  }
  const int ev = n - 1;  // new vertices per edge
  const int edge_base = 120;
  for (int e = 0; e < 720; ++e) {
    for (int j = 0; j < ev; ++j) {
      const int idx = edge_base + ev * e + j;
      const float a = (float)(j + 1) / (float)(ev + 1);
      const float b = (float)(ev - j) / (float)(ev + 1);
      for (int k = 0; k < 4; ++k) {
        const float t0 = a * v[edges[e][0]].q[k];
        const float t1 = b * v[edges[e][1]].q[k];
        all[idx].q[k] = t0 + t1;
      }
      weigh(idx, f1);
    }
  }
  const int fv = ((n - 1) * (n - 2)) / 2;  // new vertices per face
  const int face_base = 120 + 720 * ev;
  if (fv > 0) {
    for (int f = 0; f < 1200; ++f) {
      int cnt = 0;
      for (int ka = 2; ka < ev + 1; ++ka) {
        for (int kb = 2; kb < ev + 1; ++kb) {
          if (ka + kb <= ev + 1) continue;
          const int kc = 2 * (ev + 1) - ka - kb;
          const float den = (float)(3 * (ev + 1) - ka - kb - kc);
          const float a = (float)(ev + 1 - ka) / den;
          const float b = (float)(ev + 1 - kb) / den;
          const float c = (float)(ev + 1 - kc) / den;
          const int idx = face_base + fv * f + cnt;
          for (int k = 0; k < 4; ++k) {
            const float t0 = a * v[faces[f][0]].q[k];
            const float t1 = b * v[faces[f][1]].q[k];
            const float t2 = c * v[faces[f][2]].q[k];
            float s = t0 + t1;
            all[idx].q[k] = s + t2;
          }
          weigh(idx, f2);
          ++cnt;
        }
      }
    }
  }
  const int cv = ((n - 1) * (n - 2) * (n - 3)) / 6;  // new vertices per cell
  const int cell_base = 120 + 720 * ev + 1200 * fv;
  if (cv > 0) {
    for (int ci = 0; ci < 600; ++ci) {
      int cnt = 0;
      for (int ka = 3; ka < ev + 1; ++ka) {
        for (int kb = 3; kb < ev + 1; ++kb) {
          for (int kc = 3; kc < ev + 1; ++kc) {
            const int kd = 3 * (ev + 1) - ka - kb - kc;
            if (kd < 3 || kd >= ev + 1) continue;
            const float den = (float)(4 * (ev + 1) - ka - kb - kc - kd);
            const float a = (float)(ev + 1 - ka) / den;
            const float b = (float)(ev + 1 - kb) / den;
            const float c = (float)(ev + 1 - kc) / den;
            const float d = (float)(ev + 1 - kd) / den;
            const int idx = cell_base + cv * ci + cnt;
            for (int k = 0; k < 4; ++k) {
              const float t0 = a * v[cells[ci][0]].q[k];
              const float t1 = b * v[cells[ci][1]].q[k];
              const float t2 = c * v[cells[ci][2]].q[k];
              const float t3 = d * v[cells[ci][3]].q[k];
              float s = t0 + t1;
              s = s + t2;
              all[idx].q[k] = s + t3;
            }
            weigh(idx, f3);
            ++cnt;
          }
        }
      }
    }
  }

  // --- keep the q0 > 0 hemisphere (ties broken on q1, q2, q3) --------------
  int kept = 0;
  for (int i = 0; i < n_samples; ++i) {
    const float* q = all[i].q;
    bool keep = false;
    for (int k = 0; k < 4; ++k) {
      if (q[k] > 0.0f) { keep = true; break; }
      if (q[k] != 0.0f) break;
    }
    if (!keep) continue;
    if (kept >= n_keep) return EMC_ERR_INTERNAL;
    std::memcpy(quats + 4 * kept, q, 4 * sizeof(float));
    weights[kept] = w[i];
    ++kept;
  }
  if (kept != n_keep) return EMC_ERR_INTERNAL;

  // --- normalise weights by their float sum, then the quaternions ----------
  float wsum = 0.0f;
  for (int i = 0; i < n_keep; ++i) wsum = wsum + weights[i];
  for (int i = 0; i < n_keep; ++i) weights[i] = weights[i] / wsum;
  for (int i = 0; i < n_keep; ++i) {
    float* q = quats + 4 * i;
    const float nrm = (float)std::sqrt((double)q[0] * q[0] + (double)q[1] * q[1] +
                                       (double)q[2] * q[2] + (double)q[3] * q[3]);
    for (int k = 0; k < 4; ++k) q[k] = q[k] / nrm;
  }
  return n_keep;
}

// quaternion_random (rotations.c:30-41) with this library's own generator in
// place of GSL's: u = top 53 bits of splitmix64(seed, k) / 2^53, stored as
// `real` (float) like gsl_rng_uniform's result, then
// q = (sqrt(1-u1) sin(2 pi u2), sqrt(1-u1) cos(2 pi u2), sqrt(u1) sin(2 pi u3),
// sqrt(u1) cos(2 pi u3)) in double, stored as float.
static uint64_t splitmix64(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

extern "C" int emc_random_rotations(unsigned long long seed, int n, float* quats) {
  if (n < 0 || (n > 0 && !quats)) return -1;
  uint64_t s = seed;
  const double two_pi = 2.0 * 3.14159265358979323846;
  for (int i = 0; i < n; ++i) {
    float u[3];
    for (float& v : u) v = (float)((double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0));
    const double a = std::sqrt((double)(1.0f - u[0])), b = std::sqrt((double)u[0]);
    quats[4 * i + 0] = (float)(a * std::sin(two_pi * u[1]));
    quats[4 * i + 1] = (float)(a * std::cos(two_pi * u[1]));
    quats[4 * i + 2] = (float)(b * std::sin(two_pi * u[2]));
    quats[4 * i + 3] = (float)(b * std::cos(two_pi * u[2]));
  }
  return 0;
}
