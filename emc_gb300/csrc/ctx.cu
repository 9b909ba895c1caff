// Context, stream and small host helpers of the C ABI.
#include <cmath>
#include <cstring>

#include "common.cuh"

namespace emc {

int ensure_scratch(emc_ctx* ctx, size_t bytes) {
  if (ctx->scratch_bytes >= bytes) return EMC_OK;
  if (ctx->scratch) {
    EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    EMC_CUDA(ctx, cudaFree(ctx->scratch));
    ctx->scratch = nullptr;
    ctx->scratch_bytes = 0;
  }
  size_t want = bytes < (1u << 20) ? (1u << 20) : bytes;
  cudaError_t e = cudaMalloc(&ctx->scratch, want);
  if (e != cudaSuccess) return fail(ctx, EMC_ERR_NOMEM, "scratch alloc %zu B: %s", want, cudaGetErrorString(e));
  ctx->scratch_bytes = want;
  return EMC_OK;
}

}  // namespace emc

extern "C" int emc_ctx_create(emc_ctx** out, int device) {
  if (!out) return EMC_ERR_INVALID;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) return EMC_ERR_CUDA;
  if (device < 0 || device >= n) return EMC_ERR_INVALID;
  if (cudaSetDevice(device) != cudaSuccess) return EMC_ERR_CUDA;
  emc_ctx* ctx = new emc_ctx();
  ctx->device = device;
  cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
  if (cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete ctx;
    return EMC_ERR_CUDA;
  }
  ctx->stream = ctx->own_stream;
  if (cudaMallocHost(&ctx->host_pinned, 4096) != cudaSuccess) {
    cudaStreamDestroy(ctx->own_stream);
    delete ctx;
    return EMC_ERR_CUDA;
  }
  *out = ctx;
  return EMC_OK;
}

extern "C" int emc_ctx_destroy(emc_ctx* ctx) {
  if (!ctx) return EMC_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  if (ctx->scratch) cudaFree(ctx->scratch);
  if (ctx->host_pinned) cudaFreeHost(ctx->host_pinned);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  delete ctx;
  return EMC_OK;
}

extern "C" int emc_ctx_device(const emc_ctx* ctx) { return ctx ? ctx->device : -1; }

extern "C" const char* emc_last_error(const emc_ctx* ctx) {
  if (!ctx) return "null context";
  return ctx->last_error.c_str();
}

extern "C" int emc_set_stream(emc_ctx* ctx, void* cuda_stream) {
  EMC_CHECK_CTX(ctx);
  ctx->stream = cuda_stream ? (cudaStream_t)cuda_stream : ctx->own_stream;
  return EMC_OK;
}

extern "C" void* emc_get_stream(const emc_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

extern "C" int emc_sync(emc_ctx* ctx) {
  EMC_CHECK_CTX(ctx);
  EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return EMC_OK;
}

extern "C" long long emc_kernel_launches(const emc_ctx* ctx) { return ctx ? ctx->launches : -1; }

extern "C" int emc_reset_real(emc_ctx* ctx, float* d_real, int len) {
  EMC_CHECK_CTX(ctx);
  EMC_REQUIRE(ctx, len >= 0 && (len == 0 || d_real), "reset_real: bad buffer");
  if (len == 0) return EMC_OK;
  EMC_CUDA(ctx, cudaMemsetAsync(d_real, 0, sizeof(float) * (size_t)len, ctx->stream));
  return EMC_OK;
}

extern "C" int emc_copy_real_to_device(emc_ctx* ctx, const float* h_src, float* d_dst, int n) {
  EMC_CHECK_CTX(ctx);
  EMC_REQUIRE(ctx, n >= 0 && (n == 0 || (h_src && d_dst)), "copy_real_to_device: bad buffer");
  if (n == 0) return EMC_OK;
  EMC_CUDA(ctx, cudaMemcpyAsync(d_dst, h_src, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice,
                                ctx->stream));
  return EMC_OK;
}

extern "C" int emc_copy_real_to_host(emc_ctx* ctx, float* h_dst, const float* d_src, int n) {
  EMC_CHECK_CTX(ctx);
  EMC_REQUIRE(ctx, n >= 0 && (n == 0 || (h_dst && d_src)), "copy_real_to_host: bad buffer");
  if (n == 0) return EMC_OK;
  EMC_CUDA(ctx, cudaMemcpyAsync(h_dst, d_src, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost,
                                ctx->stream));
  EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return EMC_OK;
}

extern "C" int emc_copy_real_d2d(emc_ctx* ctx, float* d_dst, const float* d_src, int start, int n) {
  EMC_CHECK_CTX(ctx);
  EMC_REQUIRE(ctx, n >= 0 && start >= 0 && (n == 0 || (d_dst && d_src)), "copy_real_d2d: bad buffer");
  if (n == 0) return EMC_OK;
  EMC_CUDA(ctx, cudaMemcpyAsync(d_dst + start, d_src, sizeof(float) * (size_t)n,
                                cudaMemcpyDeviceToDevice, ctx->stream));
  return EMC_OK;
}

extern "C" int emc_copy_int_to_device(emc_ctx* ctx, const int* h_src, int* d_dst, int n) {
  EMC_CHECK_CTX(ctx);
  EMC_REQUIRE(ctx, n >= 0 && (n == 0 || (h_src && d_dst)), "copy_int_to_device: bad buffer");
  if (n == 0) return EMC_OK;
  EMC_CUDA(ctx, cudaMemcpyAsync(d_dst, h_src, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice,
                                ctx->stream));
  return EMC_OK;
}

extern "C" int emc_allocate_real(emc_ctx* ctx, float** d_out, size_t n) {
  EMC_CHECK_CTX(ctx);
  EMC_REQUIRE(ctx, d_out, "allocate_real: null output");
  *d_out = nullptr;
  cudaError_t e = cudaMalloc((void**)d_out, sizeof(float) * (n ? n : 1));
  if (e != cudaSuccess) return emc::fail(ctx, EMC_ERR_NOMEM, "allocate_real(%zu): %s", n, cudaGetErrorString(e));
  return EMC_OK;
}

extern "C" int emc_allocate_int(emc_ctx* ctx, int** d_out, size_t n) {
  EMC_CHECK_CTX(ctx);
  EMC_REQUIRE(ctx, d_out, "allocate_int: null output");
  *d_out = nullptr;
  cudaError_t e = cudaMalloc((void**)d_out, sizeof(int) * (n ? n : 1));
  if (e != cudaSuccess) return emc::fail(ctx, EMC_ERR_NOMEM, "allocate_int(%zu): %s", n, cudaGetErrorString(e));
  return EMC_OK;
}

extern "C" int emc_mem_free(emc_ctx* ctx, void* d_ptr) {
  EMC_CHECK_CTX(ctx);
  if (!d_ptr) return EMC_OK;
  EMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  EMC_CUDA(ctx, cudaFree(d_ptr));
  return EMC_OK;
}

// main.cpp:251 -- the annealing width of iteration t.
extern "C" float emc_sigma_schedule(int iteration, double sigma_start, double sigma_final,
                                    int half_life) {
  const double t = (double)(-iteration / (float)half_life) * std::log(2.0);
  return (float)(sigma_final + (sigma_start - sigma_final) * std::exp(t));
}

// emc_helper.cpp:55-79 calculate_coordinates.  Pixel (x, y) of a side x side
// detector sits at (x - side/2 + 0.5, y - side/2 + 0.5) pixels from the beam;
// its reciprocal-space z follows from the scattering angle
// theta = atan2(r * pixel_size, distance):  z = (1 - cos)/sin * r.
// Values are written as [y*side + x], the order the kernels read.
extern "C" int emc_calculate_coordinates(int side, float pixel_size, float detector_distance,
                                         float wavelength, float* x, float* y, float* z) {
  if (side <= 0 || !x || !y || !z) return EMC_ERR_INVALID;
  for (int ix = 0; ix < side; ++ix) {
    for (int iy = 0; iy < side; ++iy) {
      const double px = (double)(float)(ix - side / 2) + 0.5;
      const double py = (double)(float)(iy - side / 2) + 0.5;
      const float pixel_r = (float)std::sqrt(px * px + py * py);
      const float real_r = pixel_r * pixel_size;
      const float angle = std::atan2(real_r, detector_distance);
      const float fourier_r = std::sin(angle) / wavelength;
      const float fourier_z = (float)((1.0 - (double)std::cos(angle)) / (double)wavelength);
      const float pz = fourier_z / fourier_r * pixel_r;
      const int p = iy * side + ix;
      x[p] = (float)px;
      y[p] = (float)py;
      z[p] = pz;
    }
  }
  return EMC_OK;
}
