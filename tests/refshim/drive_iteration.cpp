// One EMC iteration driven through the reference's own cuda_* signatures
// (emc_cuda_help.h) -- i.e. through tests/refshim/emc_cuda_gb300.cpp on
// libemc_gb300 -- in main.cpp's order for one rank: rank set-up
// (main.cpp:127-160), the scaling pass over rotation chunks (:284-295), the
// likelihood pass (:351-365), max / sum-exp / normalise (:367-392), the
// M-step with insertion over chunks (:437-462), divide and normalise
// (:463-476).  Exported with C linkage for the GPU test (ctypes); host arrays
// in, host arrays out.  Test code, not part of the library.
#include <cmath>
#include <cstring>
#include <vector>

#include "emc_cuda_help.h"

extern "C" int shim_device_after_set(int i_device, int taskid) {
  cuda_set_device(i_device, taskid);
  return cuda_get_device();
}

extern "C" int shim_run_iteration(int device, int taskid, int side, int N_images, int N_slices,
                                  int slice_chunk, float sigma, const float* h_images,
                                  const int* h_mask, const float* h_x, const float* h_y,
                                  const float* h_z, const float* h_rot, const float* h_rot_w,
                                  float* h_model /* in: start model; out: new model */,
                                  float* h_weight, float* h_respons, float* h_scaling) {
  cuda_set_device(device, taskid);
  const int N_2d = side * side, N_3d = side * side * side;
  sp_3matrix model_shape = {(unsigned)side, (unsigned)side, (unsigned)side, h_model};
  real *d_images, *d_x, *d_y, *d_z, *d_rot, *d_w, *d_model, *d_new, *d_weight, *d_slices;
  real *d_respons, *d_scaling, *d_max, *d_sum;
  int *d_mask, *d_active;
  cuda_allocate_real(&d_images, N_images * N_2d);
  cuda_allocate_int(&d_mask, N_2d);
  cuda_allocate_real(&d_x, N_2d);
  cuda_allocate_real(&d_y, N_2d);
  cuda_allocate_real(&d_z, N_2d);
  cuda_allocate_real(&d_rot, 4 * N_slices);
  cuda_allocate_real(&d_w, N_slices);
  cuda_allocate_real(&d_model, N_3d);
  cuda_allocate_real(&d_new, N_3d);
  cuda_allocate_real(&d_weight, N_3d);
  cuda_allocate_real(&d_slices, slice_chunk * N_2d);
  cuda_allocate_real(&d_respons, N_slices * N_images);
  cuda_allocate_real(&d_scaling, N_slices * N_images);
  cuda_allocate_real(&d_max, N_images);
  cuda_allocate_real(&d_sum, N_images);
  cuda_allocate_int(&d_active, N_images);
  cuda_copy_real_to_device(const_cast<float*>(h_images), d_images, N_images * N_2d);
  cuda_copy_int_to_device(const_cast<int*>(h_mask), d_mask, N_2d);
  cuda_copy_real_to_device(const_cast<float*>(h_x), d_x, N_2d);
  cuda_copy_real_to_device(const_cast<float*>(h_y), d_y, N_2d);
  cuda_copy_real_to_device(const_cast<float*>(h_z), d_z, N_2d);
  cuda_copy_real_to_device(const_cast<float*>(h_rot), d_rot, 4 * N_slices);
  cuda_copy_weight_to_device(const_cast<float*>(h_rot_w), d_w, N_slices, 0);
  cuda_copy_real_to_device(h_model, d_model, N_3d);
  std::vector<float> ones((size_t)N_slices * N_images, 1.0f);
  cuda_copy_real_to_device(ones.data(), d_scaling, N_slices * N_images);
  std::vector<int> active(N_images, 1);
  cuda_copy_int_to_device(active.data(), d_active, N_images);

  for (int s0 = 0; s0 < N_slices; s0 += slice_chunk) {  // scaling (main.cpp:284-295)
    const int c = N_slices - s0 < slice_chunk ? N_slices - s0 : slice_chunk;
    cuda_get_slices(&model_shape, d_model, d_slices, d_rot, d_x, d_y, d_z, s0, c);
    cuda_update_scaling_full(d_images, d_slices, d_mask, d_scaling, N_2d, N_images, s0, c,
                             poisson);
  }
  for (int s0 = 0; s0 < N_slices; s0 += slice_chunk) {  // likelihood (main.cpp:351-365)
    const int c = N_slices - s0 < slice_chunk ? N_slices - s0 : slice_chunk;
    cuda_get_slices(&model_shape, d_model, d_slices, d_rot, d_x, d_y, d_z, s0, c);
    cuda_calculate_responsabilities(d_slices, d_images, d_mask, sigma, d_scaling, d_respons, d_w,
                                    N_2d, N_images, s0, c, poisson);
  }
  // one rank: the exchange of main.cpp:367-392 is the identity
  cuda_max_vector(d_respons, N_images, N_slices, d_max);
  cuda_respons_max_expf(d_respons, d_max, N_images, N_slices, d_sum);
  std::vector<float> mx(N_images), sm(N_images);
  cuda_copy_real_to_host(mx.data(), d_max, N_images);
  cuda_copy_real_to_host(sm.data(), d_sum, N_images);
  for (int i = 0; i < N_images; ++i) sm[i] = std::log(sm[i]) + mx[i];  // main.cpp:384-391
  cuda_copy_real_to_device(sm.data(), d_sum, N_images);
  cuda_norm_respons_sumexpf(d_respons, d_sum, d_max, N_images, N_slices);
  cuda_reset_real(d_new, N_3d);
  cuda_reset_real(d_weight, N_3d);
  for (int s0 = 0; s0 < N_slices; s0 += slice_chunk) {  // M-step (main.cpp:437-462)
    const int c = N_slices - s0 < slice_chunk ? N_slices - s0 : slice_chunk;
    cuda_update_slices(d_images, d_slices, d_mask, d_respons, d_scaling, d_active, N_images, s0,
                       c, N_2d, &model_shape, d_new, d_x, d_y, d_z, &d_rot[s0 * 4], d_weight,
                       nullptr);
  }
  cuda_divide_model_by_weight(&model_shape, d_new, d_weight);
  cuda_normalize_model(&model_shape, d_new);
  cuda_copy_real_to_host(h_model, d_new, N_3d);
  cuda_copy_real_to_host(h_weight, d_weight, N_3d);
  cuda_copy_real_to_host(h_respons, d_respons, N_slices * N_images);
  cuda_copy_real_to_host(h_scaling, d_scaling, N_slices * N_images);
  real* bufs[] = {d_images, d_x, d_y, d_z, d_rot, d_w, d_model, d_new, d_weight, d_slices,
                  d_respons, d_scaling, d_max, d_sum};
  for (real* b : bufs) cuda_mem_free(b);
  cuda_mem_free((real*)d_mask);
  cuda_mem_free((real*)d_active);
  return cuda_get_device();
}
