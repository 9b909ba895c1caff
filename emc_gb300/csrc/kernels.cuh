// Internal launchers shared between translation units.
#pragma once
#include "common.cuh"

namespace emc {

int launch_slices(emc_ctx* ctx, const float* model, int side, float* slices, const float* rot,
                  const float* x, const float* y, const float* z, int n_rot, int interp);

// Device-wide FP64 sum and count of the positive entries of x[0..n).
// Writes {sum, count} to out[0..1] (device memory).
int launch_positive_mean(emc_ctx* ctx, const float* x, long long n, double* out);

// x *= 1 / mean, where mean = out[0]/out[1] from launch_positive_mean.
int launch_scale_by_inverse_mean(emc_ctx* ctx, float* x, long long n, const double* stats);

int launch_divide_by_weight(emc_ctx* ctx, float* model, const float* weight, long long n);

int launch_blur(emc_ctx* ctx, float* model, int side, float sigma);

// Blur in two halves: blur_prepare uploads the taps into caller-owned device
// buffers (a, b: side^3 floats, g: side floats, keep: side^3 bytes) once;
// blur_run enqueues the passes without allocating or copying from the host,
// so it can be captured in a CUDA graph.
struct BlurWork {
  float *a, *b, *g;
  unsigned char* keep;
  int side, h_lo, h_hi;
};
size_t blur_work_bytes(int side);
int blur_prepare(emc_ctx* ctx, int side, float sigma, float* a, float* b, float* g,
                 unsigned char* keep, BlurWork* w);
int blur_run(emc_ctx* ctx, float* model, const BlurWork& w);

// Nearest-voxel insertion with the reference's bounds (emc_atomic.cu:33-85).
int launch_insert_nearest(emc_ctx* ctx, const float* slices, const int* mask, const float* totals,
                          const float* rot, const float* x, const float* y, const float* z,
                          int side, int n_rot, float* model, float* weight);

}  // namespace emc
