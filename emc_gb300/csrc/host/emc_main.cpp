// emc -- host driver of the GB300 EMC iteration, the counterpart of the
// reference's main.cpp:34-521 for one process on one GPU.  It uses only the
// C ABI of libemc_gb300.so.
//
//   emc [config] [--dropin] [--precision fp32|mixed] [--deterministic | --sorted-insert]
//       [--interp nearest|trilinear] [--out DIR] [--iterations N] [--graph]
//       [--prune] [--no-autotune]
//
// --graph records the fused iteration once as a CUDA graph and replays it
// (emc_plan_capture / emc_plan_replay); --prune turns on pruned iterations
// (emc_plan_set_pruning, mixed precision), whose debug responsibilities are
// written back in the input pattern and rotation order.  Mixed-precision
// plans pick the likelihood kernel's tile order with emc_plan_autotune on the
// start model unless --no-autotune is given (the results do not depend on it).
//
// config defaults to ../emc.conf as in main.cpp:66-70.  Inputs replace the
// reference's HDF5 reads (emc_helper.cpp:198-368, absent libraries) by raw
// little-endian files:
//   <image_prefix>raw.bin      float32 [N_images][detector_size^2] detector frames and
//   <image_prefix>raw_mask.bin int32   [N_images][detector_size^2] their masks, binned on
//                              the GPU by read_stride (emc_bin_images, emc_helper.cpp:226-243)
//                              into patterns and per-pattern masks; or, when raw.bin is
//                              absent, already-binned patterns:
//   <image_prefix>images.bin   float32 [N_images][model_side^2]  (y*side + x)
//   <mask_file>                int32   [model_side^2]
//   <model_file>               float32 [model_side^3]            (model_input 2)
// Preprocessing follows main.cpp:92-108 on the GPU: binning, normalisation
// (normalize_images), model_init, then mask_model (-1 at per-pattern masked
// pixels).  model_input 0 starts from a seeded uniform [0,1) model
// (emc_helper.cpp:449-456), 1 inserts every pattern at a seeded random
// orientation (:503-518), 3 is the radial average of the patterns (:458-502).
// Outputs follow file_helper.cpp:30-127 with raw files instead of HDF5:
//   output/model_%04d.bin (+ .mask.bin, .json)   value where weight > 0 and
//                                                model > 0, else 0 with mask 0
//   output/weight_%04d.bin (+ .json)
//   debug/respons_%04d.data                      float32 [R][N] when isDebug
//   ExeTime.data                                 "%d %d   %e" per iteration
//   debug_samples.data                           the rotation list (rotations.c:446-453)
// The default path is the fused iteration (emc_plan_*); --dropin drives the
// per-function entry points in main.cpp's order with slice_chunk chunks.
#include <sys/stat.h>

#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../../include/emc_gb300.h"

namespace {

struct Opts {
  std::string conf = "../emc.conf";
  std::string out = ".";
  bool dropin = false;
  int precision = EMC_PREC_FP32;
  int insert = EMC_INSERT_ATOMIC;
  int interp = EMC_INTERP_NEAREST;
  int iterations = -1;
  bool graph = false;
  bool prune = false;
  bool autotune = true;
};

[[noreturn]] void die(const char* what, const char* detail = "") {
  std::fprintf(stderr, "emc: %s %s\n", what, detail);
  std::exit(1);
}

void check(int rc, emc_ctx* ctx, const char* what) {
  if (rc != EMC_OK) die(what, ctx ? emc_last_error(ctx) : "");
}

template <typename T>
std::vector<T> read_raw(const std::string& path, size_t n) {
  std::vector<T> v(n);
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) die("cannot open", path.c_str());
  const size_t got = std::fread(v.data(), sizeof(T), n, f);
  std::fclose(f);
  if (got != n) die("short file", path.c_str());
  return v;
}

bool file_exists(const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (f) std::fclose(f);
  return f != nullptr;
}

template <typename T>
void write_raw(const std::string& path, const T* data, size_t n) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) die("cannot write", path.c_str());
  std::fwrite(data, sizeof(T), n, f);
  std::fclose(f);
}

void write_json(const std::string& path, int side, const char* dtype, const char* what) {
  FILE* f = std::fopen(path.c_str(), "w");
  if (!f) die("cannot write", path.c_str());
  std::fprintf(f, "{\"shape\": [%d, %d, %d], \"order\": \"z,y,x\", \"dtype\": \"%s\", "
                  "\"content\": \"%s\"}\n", side, side, side, dtype, what);
  std::fclose(f);
}

// PCG32 (O'Neill 2014), the seeded stream of the uniform initial model.
struct Pcg32 {
  uint64_t state = 0x853c49e6748fea9bULL, inc = 0xda3e39cb94b95bdbULL;
  uint32_t next() {
    const uint64_t old = state;
    state = old * 6364136223846793005ULL + inc;
    const uint32_t x = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    const uint32_t r = (uint32_t)(old >> 59u);
    return (x >> r) | (x << ((-r) & 31));
  }
  float uniform() { return (float)(next() >> 8) * (1.0f / 16777216.0f); }
};

Opts parse_args(int argc, char** argv) {
  Opts o;
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    auto next = [&]() -> std::string {
      if (i + 1 >= argc) die("missing value after", a.c_str());
      return argv[++i];
    };
    if (a == "--dropin") o.dropin = true;
    else if (a == "--deterministic") o.insert = EMC_INSERT_DETERMINISTIC;
    else if (a == "--sorted-insert") o.insert = EMC_INSERT_SORTED;
    else if (a == "--precision") o.precision = next() == "mixed" ? EMC_PREC_MIXED : EMC_PREC_FP32;
    else if (a == "--interp") o.interp = next() == "trilinear" ? EMC_INTERP_TRILINEAR : EMC_INTERP_NEAREST;
    else if (a == "--out") o.out = next();
    else if (a == "--iterations") o.iterations = std::atoi(next().c_str());
    else if (a == "--graph") o.graph = true;
    else if (a == "--prune") o.prune = true;
    else if (a == "--no-autotune") o.autotune = false;
    else if (!a.empty() && a[0] != '-') o.conf = a;
    else die("unknown option", a.c_str());
  }
  return o;
}

}  // namespace

int main(int argc, char** argv) {
  const Opts o = parse_args(argc, argv);
  emc_config cfg;
  char err[512] = {0};
  if (emc_config_read(o.conf.c_str(), &cfg, err, sizeof err) != EMC_OK) die("config:", err);
  const int side = cfg.model_side, N = cfg.N_images;
  const int n2 = side * side;
  const size_t n3 = (size_t)side * side * side;
  const int iterations = o.iterations >= 0 ? o.iterations : cfg.max_iterations;
  ::mkdir((o.out + "/output").c_str(), 0755);
  ::mkdir((o.out + "/debug").c_str(), 0755);
  FILE* timef = std::fopen((o.out + "/ExeTime.data").c_str(), "wb");
  auto t_prev = std::chrono::steady_clock::now();
  auto lap = [&]() {
    auto t = std::chrono::steady_clock::now();
    const double s = std::chrono::duration<double>(t - t_prev).count();
    t_prev = t;
    return s;
  };

  // ---- host inputs
  const int R = emc_rotation_count(cfg.rotations_n);
  if (R <= 0) die("bad rotations_n");
  std::vector<float> quats(4 * (size_t)R), rotw(R);
  if (emc_generate_rotations(cfg.rotations_n, quats.data(), rotw.data(), R) != R)
    die("rotation sampling failed");
  if (FILE* f = std::fopen((o.out + "/debug_samples.data").c_str(), "w")) {
    for (int r = 0; r < R; ++r)
      std::fprintf(f, "%g %g %g %g\n", quats[4 * r], quats[4 * r + 1], quats[4 * r + 2],
                   quats[4 * r + 3]);
    std::fclose(f);
  }
  std::vector<float> x(n2), y(n2), z(n2);
  emc_calculate_coordinates(side, (float)cfg.pixel_size, (float)cfg.detector_distance,
                            (float)cfg.wavelength, x.data(), y.data(), z.data());
  const std::string raw_path = std::string(cfg.image_prefix) + "raw.bin";
  const bool have_raw = file_exists(raw_path);
  std::vector<float> images;
  if (!have_raw) images = read_raw<float>(std::string(cfg.image_prefix) + "images.bin", (size_t)N * n2);
  std::vector<int> mask = read_raw<int>(cfg.mask_file, n2);
  std::vector<float> model(n3);
  if (cfg.model_input == 2) {
    model = read_raw<float>(cfg.model_file, n3);
  } else if (cfg.model_input == 0) {
    Pcg32 rng;
    for (auto& v : model) v = rng.uniform();
  } else if (cfg.model_input != 1 && cfg.model_input != 3) {
    die("model_input must be 0, 1, 2 or 3");
  }

  // ---- device
  emc_ctx* ctx = nullptr;
  if (emc_ctx_create(&ctx, 0) != EMC_OK) die("no CUDA device");
  float *d_images, *d_model, *d_weight, *d_x, *d_y, *d_z, *d_rot, *d_w;
  int* d_mask;
  int* d_masks = nullptr;  // per-pattern masks of the binned frames
  check(emc_allocate_real(ctx, &d_images, (size_t)N * n2), ctx, "alloc");
  check(emc_allocate_real(ctx, &d_model, n3), ctx, "alloc");
  check(emc_allocate_real(ctx, &d_weight, n3), ctx, "alloc");
  check(emc_allocate_real(ctx, &d_x, n2), ctx, "alloc");
  check(emc_allocate_real(ctx, &d_y, n2), ctx, "alloc");
  check(emc_allocate_real(ctx, &d_z, n2), ctx, "alloc");
  check(emc_allocate_real(ctx, &d_rot, 4 * (size_t)R), ctx, "alloc");
  check(emc_allocate_real(ctx, &d_w, R), ctx, "alloc");
  check(emc_allocate_int(ctx, &d_mask, n2), ctx, "alloc");
  if (have_raw) {  // read_images (emc_helper.cpp:198-245): bin the frames on the GPU
    const int D = cfg.detector_size;
    if (D <= 0 || cfg.read_stride <= 0) die("raw frames need detector_size and read_stride > 0");
    std::vector<float> raw = read_raw<float>(raw_path, (size_t)N * D * D);
    std::vector<int> raw_mask =
        read_raw<int>(std::string(cfg.image_prefix) + "raw_mask.bin", (size_t)N * D * D);
    float* d_raw = nullptr;
    int* d_raw_mask = nullptr;
    check(emc_allocate_real(ctx, &d_raw, (size_t)N * D * D), ctx, "alloc");
    check(emc_allocate_int(ctx, &d_raw_mask, (size_t)N * D * D), ctx, "alloc");
    check(emc_allocate_int(ctx, &d_masks, (size_t)N * n2), ctx, "alloc");
    check(emc_copy_real_to_device(ctx, raw.data(), d_raw, N * D * D), ctx, "copy");
    check(emc_copy_int_to_device(ctx, raw_mask.data(), d_raw_mask, N * D * D), ctx, "copy");
    for (int i0 = 0; i0 < N; i0 += 65535) {
      const int c = std::min(65535, N - i0);
      check(emc_bin_images(ctx, d_raw + (size_t)i0 * D * D, d_raw_mask + (size_t)i0 * D * D, D, D,
                           c, side, cfg.read_stride, d_images + (size_t)i0 * n2,
                           d_masks + (size_t)i0 * n2), ctx, "bin_images");
    }
    check(emc_mem_free(ctx, d_raw), ctx, "free");
    check(emc_mem_free(ctx, d_raw_mask), ctx, "free");
  } else {
    check(emc_copy_real_to_device(ctx, images.data(), d_images, N * n2), ctx, "copy");
  }
  if (cfg.model_input == 0 || cfg.model_input == 2)
    check(emc_copy_real_to_device(ctx, model.data(), d_model, (int)n3), ctx, "copy");
  check(emc_copy_real_to_device(ctx, x.data(), d_x, n2), ctx, "copy");
  check(emc_copy_real_to_device(ctx, y.data(), d_y, n2), ctx, "copy");
  check(emc_copy_real_to_device(ctx, z.data(), d_z, n2), ctx, "copy");
  check(emc_copy_real_to_device(ctx, quats.data(), d_rot, 4 * R), ctx, "copy");
  check(emc_copy_real_to_device(ctx, rotw.data(), d_w, R), ctx, "copy");
  check(emc_copy_int_to_device(ctx, mask.data(), d_mask, n2), ctx, "copy");
  // normalize_images (main.cpp:96-98).  The fused plan folds the per-pattern
  // factor into the scaling itself (so the tensor cores keep integer counts);
  // the drop-in path and the model initialisation take normalised patterns.
  float* d_norm = d_images;
  if (cfg.normalize_images) {
    if (o.dropin) {
      check(emc_normalize_images(ctx, d_images, d_mask, nullptr, n2, N), ctx, "normalize_images");
    } else if (cfg.model_input == 1 || cfg.model_input == 3) {
      check(emc_allocate_real(ctx, &d_norm, (size_t)N * n2), ctx, "alloc");
      check(emc_copy_real_d2d(ctx, d_norm, d_images, 0, N * n2), ctx, "copy");
      check(emc_normalize_images(ctx, d_norm, d_mask, nullptr, n2, N), ctx, "normalize_images");
    }
  }
  if (cfg.model_input == 3) {  // radial average (emc_helper.cpp:458-502)
    check(emc_model_init_radial(ctx, d_norm, N, side, d_model), ctx, "model_init_radial");
  } else if (cfg.model_input == 1) {  // random orientations (emc_helper.cpp:503-518)
    std::vector<float> q(4 * (size_t)N);
    if (emc_random_rotations(0, N, q.data()) != 0) die("random rotations failed");
    float* d_q = nullptr;
    check(emc_allocate_real(ctx, &d_q, 4 * (size_t)N), ctx, "alloc");
    check(emc_copy_real_to_device(ctx, q.data(), d_q, 4 * N), ctx, "copy");
    check(emc_model_init_orientations(ctx, d_norm, d_mask, N, side, d_q, d_x, d_y, d_z, d_model,
                                      d_weight), ctx, "model_init_orientations");
    check(emc_mem_free(ctx, d_q), ctx, "free");
  }
  if (d_norm != d_images) check(emc_mem_free(ctx, d_norm), ctx, "free");
  if (d_masks) check(emc_mask_images(ctx, d_images, d_masks, n2, N), ctx, "mask_images");
  check(emc_normalize_model(ctx, side, d_model, nullptr), ctx, "normalize");  // main.cpp:180

  emc_plan* plan = nullptr;
  float *d_resp = nullptr, *d_scal = nullptr, *d_slices = nullptr, *d_max = nullptr,
        *d_sum = nullptr, *d_lse = nullptr;
  int* d_active = nullptr;
  const int chunk = std::min(cfg.slice_chunk, std::min(R, 65535));
  if (!o.dropin) {
    emc_plan_desc d{};
    d.side = side;
    d.n_images = N;
    d.n_rot = R;
    d.diff = cfg.diff == EMC_DIFF_TRUE_POISSON ? EMC_DIFF_TRUE_POISSON : EMC_DIFF_POISSON;
    d.interp = o.interp;
    d.precision = o.precision;
    d.insert_mode = o.insert;
    d.known_intensity = cfg.known_intensity;
    d.normalize_images = cfg.normalize_images;
    d.blur_sigma = (float)cfg.model_blur;
    check(emc_plan_create(ctx, &d, &plan), ctx, "plan_create");
    int rc = emc_plan_bind(plan, d_images, d_mask, d_x, d_y, d_z, d_rot, d_w);
    if (rc == EMC_ERR_UNSUPPORTED && d.precision == EMC_PREC_MIXED) {
      // e.g. -1 at per-pattern masked pixels: not an FP16 count
      std::fprintf(stderr, "emc: %s; using the FP32 path\n", emc_last_error(ctx));
      emc_plan_destroy(plan);
      d.precision = EMC_PREC_FP32;
      check(emc_plan_create(ctx, &d, &plan), ctx, "plan_create");
      rc = emc_plan_bind(plan, d_images, d_mask, d_x, d_y, d_z, d_rot, d_w);
    }
    check(rc, ctx, "plan_bind");
    if (o.autotune && d.precision == EMC_PREC_MIXED) {
      int raster = 0;
      float ms = 0.0f;
      check(emc_plan_autotune(plan, d_model, emc_sigma_schedule(0, cfg.sigma_start, cfg.sigma_final,
                                                                 cfg.sigma_half_life),
                              &raster, &ms), ctx, "plan_autotune");
      std::fprintf(stderr, "emc: likelihood tile order %d (%.3f ms on the timed prefix)\n", raster,
                   ms);
    }
    if (o.prune) check(emc_plan_set_pruning(plan, 1, 0.999f, 1.0f, 0), ctx, "plan_set_pruning");
    if (o.graph) check(emc_plan_capture(plan, d_model, d_weight), ctx, "plan_capture");
  } else {
    check(emc_allocate_real(ctx, &d_resp, (size_t)R * N), ctx, "alloc");
    check(emc_allocate_real(ctx, &d_scal, (size_t)R * N), ctx, "alloc");
    check(emc_allocate_real(ctx, &d_slices, (size_t)chunk * n2), ctx, "alloc");
    check(emc_allocate_real(ctx, &d_max, N), ctx, "alloc");
    check(emc_allocate_real(ctx, &d_sum, N), ctx, "alloc");
    check(emc_allocate_real(ctx, &d_lse, N), ctx, "alloc");
    check(emc_allocate_int(ctx, &d_active, N), ctx, "alloc");
    std::vector<int> active(N, 1);
    check(emc_copy_int_to_device(ctx, active.data(), d_active, N), ctx, "copy");
    std::vector<float> ones((size_t)R * N, 1.0f);  // known_intensity: scaling stays 1
    check(emc_copy_real_to_device(ctx, ones.data(), d_scal, R * N), ctx, "copy");
  }
  if (timef) std::fprintf(timef, "%d %d   %e \n", -1, 0, lap());

  std::vector<float> h_model(n3), h_weight(n3), h_resp;
  for (int it = 0; it < iterations; ++it) {
    const float sigma = emc_sigma_schedule(it, cfg.sigma_start, cfg.sigma_final, cfg.sigma_half_life);
    double ll = 0.0, mean_before = 0.0;
    if (!o.dropin) {
      emc_iter_stats st;
      if (o.graph) {
        check(emc_plan_replay(plan, sigma), ctx, "plan_replay");
        check(emc_plan_wait(plan, &st), ctx, "plan_wait");
      } else {
        check(emc_iterate(plan, d_model, d_weight, sigma, &st), ctx, "iterate");
      }
      ll = st.total_loglik;
      mean_before = st.model_mean_before;
    } else {
      // main.cpp:242-480, one rank
      const int diff = cfg.diff == EMC_DIFF_TRUE_POISSON ? EMC_DIFF_POISSON : cfg.diff;
      if (!cfg.known_intensity)
        for (int s0 = 0; s0 < R; s0 += chunk) {
          const int c = std::min(chunk, R - s0);
          check(emc_get_slices(ctx, d_model, side, d_slices, d_rot, d_x, d_y, d_z, s0, c,
                               EMC_INTERP_NEAREST), ctx, "get_slices");
          check(emc_update_scaling_full(ctx, d_images, d_slices, d_mask, d_scal, n2, N, s0, c,
                                        diff), ctx, "update_scaling_full");
        }
      for (int s0 = 0; s0 < R; s0 += chunk) {
        const int c = std::min(chunk, R - s0);
        check(emc_get_slices(ctx, d_model, side, d_slices, d_rot, d_x, d_y, d_z, s0, c,
                             EMC_INTERP_NEAREST), ctx, "get_slices");
        check(emc_calculate_responsabilities(ctx, d_slices, d_images, d_mask, sigma, d_scal, d_resp,
                                             d_w, n2, N, s0, c, diff), ctx, "responsabilities");
      }
      check(emc_max_vector(ctx, d_resp, N, R, d_max), ctx, "max_vector");
      check(emc_respons_max_expf(ctx, d_resp, d_max, N, R, d_sum), ctx, "respons_max_expf");
      check(emc_log_sum_max(ctx, d_sum, d_max, d_lse, N), ctx, "log_sum_max");
      std::vector<float> lse(N);
      check(emc_copy_real_to_host(ctx, lse.data(), d_lse, N), ctx, "copy");
      for (float v : lse)
        if (std::isfinite(v)) ll += v;
      check(emc_norm_respons_sumexpf(ctx, d_resp, d_lse, d_max, N, R), ctx, "norm_respons");
      check(emc_reset_real(ctx, d_weight, (int)n3), ctx, "reset");
      // the updated model goes to a zeroed grid; the current one is still
      // read by the slices of the M-step loop (main.cpp:443-465)
      float* d_new = nullptr;
      check(emc_allocate_real(ctx, &d_new, n3), ctx, "alloc");
      check(emc_reset_real(ctx, d_new, (int)n3), ctx, "reset");
      for (int s0 = 0; s0 < R; s0 += chunk) {
        const int c = std::min(chunk, R - s0);
        check(emc_update_slices(ctx, d_images, d_slices, d_mask, d_resp, d_scal, d_active, N, s0,
                                c, n2, side, d_new, d_x, d_y, d_z, d_rot + 4 * (size_t)s0,
                                d_weight), ctx, "update_slices");
      }
      check(emc_mem_free(ctx, d_model), ctx, "free");
      d_model = d_new;
      check(emc_divide_model_by_weight(ctx, side, d_model, d_weight), ctx, "divide");
      float mb = 0.0f;
      check(emc_normalize_model(ctx, side, d_model, &mb), ctx, "normalize");
      mean_before = mb;
    }
    check(emc_copy_real_to_host(ctx, h_model.data(), d_model, (int)n3), ctx, "copy");
    check(emc_copy_real_to_host(ctx, h_weight.data(), d_weight, (int)n3), ctx, "copy");
    const double secs = lap();
    if (timef) {
      std::fprintf(timef, "%d %d   %e \n", it, 0, secs);
      std::fflush(timef);
    }
    std::printf("{\"iteration\": %d, \"sigma\": %.6g, \"total_loglik\": %.17g, "
                "\"model_mean_before\": %.9g, \"seconds\": %.6f}\n",
                it, sigma, ll, mean_before, secs);
    std::fflush(stdout);
    const bool write = cfg.isOutput && (!cfg.output_loop || it % std::max(1, cfg.output_period) == 0);
    if (write) {
      char name[64];
      std::vector<float> val(n3);
      std::vector<uint8_t> msk(n3);
      for (size_t v = 0; v < n3; ++v) {  // file_helper.cpp:50-65
        const bool ok = h_weight[v] > 0.0f && h_model[v] > 0.0f;
        val[v] = ok ? h_model[v] : 0.0f;
        msk[v] = ok ? 1 : 0;
      }
      std::snprintf(name, sizeof name, "/output/model_%04d", it);
      write_raw(o.out + name + ".bin", val.data(), n3);
      write_raw(o.out + name + ".mask.bin", msk.data(), n3);
      write_json(o.out + name + ".json", side, "float32", "model where weight > 0 and model > 0");
      std::snprintf(name, sizeof name, "/output/weight_%04d", it);
      write_raw(o.out + name + ".bin", h_weight.data(), n3);
      write_json(o.out + name + ".json", side, "float32", "insertion weight");
    }
    if (cfg.isDebug) {  // file_helper.cpp:30-47: raw float32 [R][N]
      h_resp.resize((size_t)R * N);
      const float* src = d_resp;
      if (!o.dropin) emc_plan_results(plan, &src, nullptr, nullptr);
      check(emc_copy_real_to_host(ctx, h_resp.data(), src, R * N), ctx, "copy");
      if (o.prune) {  // back to the input order of patterns and rotations
        std::vector<int> po(N), ro(R);
        emc_plan_pattern_order(plan, po.data());
        emc_plan_rotation_order(plan, ro.data());
        std::vector<float> t(h_resp.size());
        for (int r = 0; r < R; ++r)
          for (int i = 0; i < N; ++i) t[(size_t)ro[r] * N + po[i]] = h_resp[(size_t)r * N + i];
        h_resp.swap(t);
      }
      char name[64];
      std::snprintf(name, sizeof name, "/debug/respons_%04d.data", it);
      write_raw(o.out + name, h_resp.data(), h_resp.size());
    }
  }
  if (timef) std::fclose(timef);
  if (plan) emc_plan_destroy(plan);
  for (void* p : {(void*)d_images, (void*)d_model, (void*)d_weight, (void*)d_x, (void*)d_y,
                  (void*)d_z, (void*)d_rot, (void*)d_w, (void*)d_mask, (void*)d_resp,
                  (void*)d_scal, (void*)d_slices, (void*)d_max, (void*)d_sum, (void*)d_lse,
                  (void*)d_active})
    emc_mem_free(ctx, p);
  emc_ctx_destroy(ctx);
  return 0;
}
