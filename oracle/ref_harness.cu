// C wrappers around the reference's own host functions (emc_cuda.cu,
// emc_atomic.cu compiled unchanged from the reference tree for sm_103a by
// oracle/build_ref.sh --kernels).  TEST INFRASTRUCTURE ONLY: used once, on a
// machine with a GB300, by tests/golden/make_ref_kernel_golden.py to record the reference
// kernels' outputs as golden fixtures that pin the oracle.  Each wrapper
// fills the spimage structs the reference reads sizes from, calls the
// reference function and synchronises.
#include <cuda_runtime.h>

#include "emc_cuda_help.h"

static sp_3matrix cube(int side) {
  sp_3matrix m;
  m.x = m.y = m.z = (unsigned)side;
  m.data = nullptr;
  return m;
}

static int done() {
  cudaError_t e = cudaDeviceSynchronize();
  return e == cudaSuccess ? 0 : (int)e;
}

extern "C" {

int ref_get_slices(float* model, int side, float* slices, float* rot, float* x, float* y, float* z,
                   int start, int chunk) {
  sp_3matrix m = cube(side);
  cuda_get_slices(&m, model, slices, rot, x, y, z, start, chunk);
  return done();
}

int ref_update_scaling_full(float* images, float* slices, int* mask, float* scaling, int n2,
                            int n_images, int start, int chunk, int diff) {
  cuda_update_scaling_full(images, slices, mask, scaling, n2, n_images, start, chunk,
                           (enum diff_type)diff);
  return done();
}

int ref_calculate_responsabilities(float* slices, float* images, int* mask, float sigma,
                                   float* scaling, float* respons, float* weights, int n2,
                                   int n_images, int start, int chunk, int diff) {
  cuda_calculate_responsabilities(slices, images, mask, sigma, scaling, respons, weights, n2,
                                  n_images, start, chunk, (enum diff_type)diff);
  return done();
}

int ref_max_vector(float* respons, int n_images, int n_slices, float* maxr) {
  cuda_max_vector(respons, n_images, n_slices, maxr);
  return done();
}

int ref_respons_max_expf(float* respons, float* maxv, int n_images, int n_slices, float* sum) {
  cuda_respons_max_expf(respons, maxv, n_images, n_slices, sum);
  return done();
}

int ref_norm_respons_sumexpf(float* respons, float* lse, float* maxv, int n_images, int n_slices) {
  cuda_norm_respons_sumexpf(respons, lse, maxv, n_images, n_slices);
  return done();
}

int ref_update_slices(float* images, float* slices, int* mask, float* respons, float* scaling,
                      int* active, int n_images, int start, int chunk, int n2, int side,
                      float* model, float* x, float* y, float* z, float* rot, float* weight) {
  sp_3matrix m = cube(side);
  sp_matrix img;
  img.rows = img.cols = (unsigned)side;
  img.data = nullptr;
  sp_matrix* imgs[1] = {&img};
  cuda_update_slices(images, slices, mask, respons, scaling, active, n_images, start, chunk, n2,
                     &m, model, x, y, z, rot, weight, imgs);
  return done();
}

int ref_divide_model_by_weight(int side, float* model, float* weight) {
  sp_3matrix m = cube(side);
  cuda_divide_model_by_weight(&m, model, weight);
  return done();
}

int ref_normalize_model(int side, float* model) {
  sp_3matrix m = cube(side);
  cuda_normalize_model(&m, model);
  return done();
}

float ref_model_average(float* model, int n) { return cuda_model_average(model, n); }

}  // extern "C"
