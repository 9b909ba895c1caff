// The reference's cuda_* interface (emc_cuda_help.h:9-117) implemented on
// libemc_gb300's C ABI -- the file a maintainer adds to the reference's build
// in place of emc_cuda.cu and emc_atomic.cu.
//
// It is compiled here against the reference's own header (emc_cuda_help.h,
// with the spimage/GSL stand-ins of oracle/shim) so that every signature is
// checked by the compiler, and linked into tests/refshim/_build/ by
// tests/refshim/build.py for the GPU test that drives one rotation chunk
// through these functions in main.cpp's order.
//
// One context per process (= per MPI rank): cuda_set_device (main.cpp:127
// calls it with taskid % nGPUs before any other cuda_* call) creates it on
// the device it is given, replacing any earlier one, and every other function
// uses that same context.  Only a caller that never calls cuda_set_device
// gets a context on the current device, made on first use.
#include <cstdio>
#include <cstdlib>

#include "emc_cuda_help.h"  // the reference's declarations (spimage structs, diff_type)
#include "emc_gb300.h"

static emc_ctx* g_ctx = nullptr;

static emc_ctx* ctx() {
  if (!g_ctx) {
    int dev = 0;
    if (emc_ctx_create(&g_ctx, dev) != EMC_OK) {
      std::fprintf(stderr, "libemc_gb300: no usable GPU\n");
      std::exit(1);
    }
  }
  return g_ctx;
}

// The reference printed CUDA errors and went on; here an error stops the run.
static void ok(int rc, const char* what) {
  if (rc != EMC_OK) {
    std::fprintf(stderr, "%s: %s\n", what, emc_last_error(g_ctx));
    std::exit(1);
  }
}

void cuda_set_device(int i_device, int taskid) {  // emc_cuda.cu:867-870
  if (g_ctx) {
    emc_ctx_destroy(g_ctx);
    g_ctx = nullptr;
  }
  if (emc_ctx_create(&g_ctx, i_device) != EMC_OK) {
    std::fprintf(stderr, "cuda_set_device(%d) failed at task id %d\n", i_device, taskid);
    std::exit(1);
  }
}

int cuda_get_device() {  // emc_cuda.cu:861-865: the device of this rank's context
  return g_ctx ? emc_ctx_device(g_ctx) : 0;
}

void cuda_get_slices(sp_3matrix* model, real* d_model, real* d_slices, real* d_rot, real* dx,
                     real* dy, real* dz, int start, int chunk) {  // emc_cuda.cu:542
  ok(emc_get_slices(ctx(), d_model, sp_3matrix_x(model), d_slices, d_rot, dx, dy, dz, start,
                    chunk, EMC_INTERP_NEAREST),
     "get_slices");
}

void cuda_update_scaling_full(real* d_images, real* d_slices, int* d_mask, real* d_scaling,
                              int N_2d, int N_images, int start, int chunk,
                              enum diff_type diff) {  // emc_cuda.cu:516
  ok(emc_update_scaling_full(ctx(), d_images, d_slices, d_mask, d_scaling, N_2d, N_images, start,
                             chunk, (int)diff),
     "update_scaling_full");
}

void cuda_calculate_responsabilities(real* d_slices, real* d_images, int* d_mask, real sigma,
                                     real* d_scaling, real* d_respons, real* d_weights, int N_2d,
                                     int N_images, int start, int chunk,
                                     enum diff_type diff) {  // emc_cuda.cu:280
  ok(emc_calculate_responsabilities(ctx(), d_slices, d_images, d_mask, sigma, d_scaling,
                                    d_respons, d_weights, N_2d, N_images, start, chunk, (int)diff),
     "calculate_responsabilities");
}

void cuda_max_vector(real* d_respons, int N_images, int n_slices, real* d_maxr) {  // :1041
  ok(emc_max_vector(ctx(), d_respons, N_images, n_slices, d_maxr), "max_vector");
}

void cuda_respons_max_expf(real* d_respons, real* d_max, int N_images, int n_slices,
                           real* d_sum) {  // emc_cuda.cu:1205
  ok(emc_respons_max_expf(ctx(), d_respons, d_max, N_images, n_slices, d_sum),
     "respons_max_expf");
}

void cuda_norm_respons_sumexpf(real* d_respons, real* d_sum, real* d_max, int N_images,
                               int n_slices) {  // emc_cuda.cu:1263
  ok(emc_norm_respons_sumexpf(ctx(), d_respons, d_sum, d_max, N_images, n_slices),
     "norm_respons_sumexpf");
}

void cuda_update_slices(real* d_images, real* d_slices, int* d_mask, real* d_respons,
                        real* d_scaling, int* d_active, int N_images, int start, int chunk,
                        int N_2d, sp_3matrix* model, real* d_model, real* dx, real* dy, real* dz,
                        real* d_rot, real* d_weight, sp_matrix** images) {  // emc_cuda.cu:562
  (void)images;
  ok(emc_update_slices(ctx(), d_images, d_slices, d_mask, d_respons, d_scaling, d_active,
                       N_images, start, chunk, N_2d, sp_3matrix_x(model), d_model, dx, dy, dz,
                       d_rot, d_weight),
     "update_slices");
}

void cuda_divide_model_by_weight(sp_3matrix* model, real* d_model, real* d_weight) {  // :779
  ok(emc_divide_model_by_weight(ctx(), sp_3matrix_x(model), d_model, d_weight),
     "divide_model_by_weight");
}

void cuda_normalize_model(sp_3matrix* model, real* d_model) {  // emc_cuda.cu:788
  float mean = 0.0f;
  ok(emc_normalize_model(ctx(), sp_3matrix_x(model), d_model, &mean), "normalize_model");
  std::printf("model average before normalization = %g\n", mean);
}

real cuda_model_max(real* d_model, int n) {  // emc_cuda.cu:629
  float m = 0.0f;
  ok(emc_model_max(ctx(), d_model, n, &m), "model_max");
  return m;
}

real cuda_model_average(real* d_model, int n) {  // emc_cuda.cu:663
  float m = 0.0f;
  ok(emc_model_average(ctx(), d_model, n, &m), "model_average");
  return m;
}

void cuda_blur_model(real* d_model, const int side, const real sigma) {  // emc_cuda.cu:1472
  ok(emc_blur_model(ctx(), d_model, side, sigma), "blur_model");
}

void cuda_reset_real(real* d, int len) { ok(emc_reset_real(ctx(), d, len), "reset_real"); }

void cuda_set_to_zero(real* x, int n) { ok(emc_reset_real(ctx(), x, n), "set_to_zero"); }

// ---- memory (emc_cuda.cu:872-926): the reference's copies are synchronous
void cuda_allocate_real(real** x, int n) { ok(emc_allocate_real(ctx(), x, (size_t)n), "allocate_real"); }

void cuda_allocate_int(int** x, int n) { ok(emc_allocate_int(ctx(), x, (size_t)n), "allocate_int"); }

void cuda_mem_free(real* d) { ok(emc_mem_free(ctx(), d), "mem_free"); }

void cuda_copy_real_to_device(real* x, real* d_x, int n) {
  ok(emc_copy_real_to_device(ctx(), x, d_x, n), "copy_real_to_device");
  ok(emc_sync(ctx()), "copy_real_to_device");
}

void cuda_copy_real_to_device(real* x, real* d_x, int start, int n) {
  ok(emc_copy_real_to_device(ctx(), x, d_x + start, n), "copy_real_to_device");
  ok(emc_sync(ctx()), "copy_real_to_device");
}

void cuda_copy_real_d2d(real* dst, real* ori, int start, int n) {
  ok(emc_copy_real_d2d(ctx(), dst, ori, start, n), "copy_real_d2d");
  ok(emc_sync(ctx()), "copy_real_d2d");
}

void cuda_copy_weight_to_device(real* x, real* d_x, int n, int taskid) {  // rank's slice of x
  ok(emc_copy_real_to_device(ctx(), x + (size_t)taskid * n, d_x, n), "copy_weight_to_device");
  ok(emc_sync(ctx()), "copy_weight_to_device");
}

void cuda_copy_real_to_host(real* x, real* d_x, int n) {
  ok(emc_copy_real_to_host(ctx(), x, d_x, n), "copy_real_to_host");
}

void cuda_copy_int_to_device(int* x, int* d_x, int n) {
  ok(emc_copy_int_to_device(ctx(), x, d_x, n), "copy_int_to_device");
  ok(emc_sync(ctx()), "copy_int_to_device");
}
