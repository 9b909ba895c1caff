/*
 * emc_gb300.h -- C ABI of the GB300 (sm_103a) EMC iteration.
 *
 * The per-function entry points below replace the C++-linkage `cuda_*`
 * functions of the reference (emc_cuda_help.h:9-117) one for one.  The
 * reference passes spimage structs only to carry sizes; here the sizes are
 * plain ints.  Every buffer argument is a raw device pointer owned by the
 * caller, laid out exactly as in the reference:
 *
 *   model, weight    float[side*side*side]     index z*side*side + y*side + x
 *   slices           float[chunk*N_2d]         index r*N_2d + p,  p = y*side + x
 *   images           float[N_images*N_2d]      index i*N_2d + p
 *   mask             int[N_2d]                 common detector mask
 *   respons, scaling float[n_slices*N_images]  rotation-major: r*N_images + i
 *   rotations        float[4*R]                unit quaternions (w, x, y, z)
 *   x/y/z coords     float[N_2d]               detector pixel -> reciprocal space
 *
 * Conventions that differ from the reference (boundary rows B2-B4 of the
 * design): every function returns an int status (EMC_OK == 0, negative on
 * error) and never prints; the text of the last error is kept per context
 * (emc_last_error).  Work is queued on the context's stream and is
 * asynchronous unless a function returns a host value; emc_sync() waits.
 * A context is not re-entrant: one host thread drives it at a time.
 */
#ifndef EMC_GB300_H
#define EMC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define EMC_OK 0
#define EMC_ERR_INVALID (-1)     /* bad argument (null pointer, size, enum)      */
#define EMC_ERR_CUDA (-2)        /* a CUDA runtime call failed                   */
#define EMC_ERR_TIMEOUT (-3)     /* a bounded device-side wait gave up           */
#define EMC_ERR_NONFINITE (-4)   /* NaN/Inf detected where the contract forbids  */
#define EMC_ERR_INTERNAL (-5)    /* invariant violated (a bug)                   */
#define EMC_ERR_NOMEM (-6)       /* device allocation failed                     */
#define EMC_ERR_UNSUPPORTED (-7) /* input outside what the chosen path handles   */

/* ---- enums ------------------------------------------------------------- */
/* diff_type of the reference (configs.h:11). */
#define EMC_DIFF_ABSOLUTE 0
#define EMC_DIFF_POISSON 1  /* the reference's "poisson": weighted least squares */
#define EMC_DIFF_RELATIVE 2
#define EMC_DIFF_TRUE_POISSON 3 /* new: counts x log(slice) Poisson likelihood  */

/* slice interpolation */
#define EMC_INTERP_NEAREST 0   /* reference: lroundf to the nearest voxel */
#define EMC_INTERP_TRILINEAR 1 /* new: trilinear gather / splat           */

/* arithmetic of the fused iteration (emc_plan_*) */
#define EMC_PREC_FP32 0  /* plain FP32 SIMT kernels                         */
#define EMC_PREC_MIXED 1 /* FP16 tensor-core GEMMs, hi+lo split, FP32 accum */

/* model insertion of the fused iteration */
#define EMC_INSERT_ATOMIC 0        /* float atomics (order-dependent rounding) */
#define EMC_INSERT_DETERMINISTIC 1 /* order-independent: bit-identical reruns  */
#define EMC_INSERT_SORTED 2        /* segmented reduction over voxel-sorted     \
                                      pairs, fixed FP32 order: bit-identical    \
                                      reruns (the pair map is built at bind)    */

typedef struct emc_ctx emc_ctx;
typedef struct emc_plan emc_plan;

/* ---- context ----------------------------------------------------------- */
/* Replaces cuda_set_device (emc_cuda.cu:867-870; main.cpp:127): binds the
 * context to `device` and creates its stream. */
int emc_ctx_create(emc_ctx** out, int device);
/* Destroy every plan and batch of a context before the context. */
int emc_ctx_destroy(emc_ctx* ctx);
/* The device the context was created on (cuda_get_device, emc_cuda.cu:861-865,
 * for a caller whose current device may have changed since); -1 for NULL. */
int emc_ctx_device(const emc_ctx* ctx);
/* Text of the last error on this context (never NULL). */
const char* emc_last_error(const emc_ctx* ctx);
/* Use an external cudaStream_t (NULL: the context's own stream). */
int emc_set_stream(emc_ctx* ctx, void* cuda_stream);
void* emc_get_stream(const emc_ctx* ctx);
int emc_sync(emc_ctx* ctx);
/* Number of kernels this context launched since creation (instrumentation). */
long long emc_kernel_launches(const emc_ctx* ctx);

/* ---- host inputs ------------------------------------------------------- */
/* rotations.c:43 n_to_samples(n)/2: rotations kept for sampling level n. */
int emc_rotation_count(int n);
/* rotations.c:77-458 generate_rotation_list: 600-cell sampling at level n,
 * q0>0 hemisphere, weights normalised by their float sum.  Writes 4*R floats
 * to quats and R floats to weights (host memory).  Returns R or < 0. */
int emc_generate_rotations(int n, float* quats, float* weights, int capacity);
/* emc_helper.cpp:55-79 calculate_coordinates: Ewald-sphere coordinates of the
 * side x side detector, written as [y*side + x] (host memory). */
int emc_calculate_coordinates(int side, float pixel_size, float detector_distance,
                              float wavelength, float* x, float* y, float* z);
/* main.cpp:251: sigma_t = sf + (ss - sf) * exp(-t / half_life * ln 2). */
float emc_sigma_schedule(int iteration, double sigma_start, double sigma_final, int half_life);

/* rotations.c:30-41 quaternion_random, n times, with this library's seeded
 * generator (splitmix64) in place of GSL's gsl_rng_taus: 4*n floats (host). */
int emc_random_rotations(unsigned long long seed, int n, float* quats);

/* ---- configuration (emc.conf) ------------------------------------------ */
/* The keys of Configuration (configs.h:11-89) read by configs.cpp:40-90. */
#define EMC_CONFIG_PATH_MAX 512
typedef struct {
  int model_side, read_stride, slice_chunk, N_images, max_iterations, rotations_n;
  double wavelength, pixel_size;
  int detector_size;
  double detector_distance, sigma_start, sigma_final;
  int sigma_half_life;
  int diff; /* EMC_DIFF_* from diff_type */
  int blur_image;
  double blur_sigma;
  char mask_file[EMC_CONFIG_PATH_MAX];
  char image_prefix[EMC_CONFIG_PATH_MAX];
  int normalize_images, known_intensity, model_input;
  char model_file[EMC_CONFIG_PATH_MAX];
  int exclude_images;
  double exclude_ratio, model_blur;
  int isDebug, isOutput, output_loop, output_period, nGPUs;
} emc_config;
/* emc.conf's own values (emc.conf:1-26), nGPU 1, and 0 for the keys emc.conf
 * leaves out (the reference leaves those uninitialised). */
int emc_config_defaults(emc_config* c);
/* Config::read_configuration_file (configs.cpp:40-90) without libconfig:
 * parses libconfig-syntax text over *c (call emc_config_defaults first);
 * EMC_ERR_INVALID with a message in err on a syntax or type error. */
int emc_config_parse(const char* text, emc_config* c, char* err, int errlen);
int emc_config_read(const char* path, emc_config* c, char* err, int errlen);

/* ---- per-function drop-ins (reference semantics) ----------------------- */
/* cuda_get_slices (emc_cuda_help.h:47-49; emc_cuda.cu:102-157, 542-560):
 * slices[r] for rotations start_slice .. start_slice+slice_chunk-1 of d_rot.
 * EMC_INTERP_NEAREST reproduces the reference bit for bit (out-of-volume
 * pixels get -1); EMC_INTERP_TRILINEAR is the new gather. */
int emc_get_slices(emc_ctx* ctx, const float* d_model, int side, float* d_slices,
                   const float* d_rot, const float* d_x, const float* d_y, const float* d_z,
                   int start_slice, int slice_chunk, int interp);

/* cuda_update_scaling_full (emc_cuda_help.h:36-37; emc_cuda.cu:438-454,
 * 516-539): scaling[(start+r)*N_images + i] = sum k^2 / sum k*s over mask>0,
 * s>1e-10, k>1e-10, with the reference's int-truncated denominator. */
int emc_update_scaling_full(emc_ctx* ctx, const float* d_images, const float* d_slices,
                            const int* d_mask, float* d_scaling, int N_2d, int N_images,
                            int slice_start, int slice_chunk, int diff);

/* cuda_calculate_responsabilities (emc_cuda_help.h:40-43; emc_cuda.cu:159-295):
 * respons[(start+r)*N_images + i] = log(w[start+r]) - S / (2 count sigma^2),
 * S the per-pixel difference sum of `diff` (FP64 per pixel for POISSON, as
 * in the reference). */
int emc_calculate_responsabilities(emc_ctx* ctx, const float* d_slices, const float* d_images,
                                   const int* d_mask, float sigma, const float* d_scaling,
                                   float* d_respons, const float* d_weights, int N_2d,
                                   int N_images, int slice_start, int slice_chunk, int diff);

/* cuda_max_vector (emc_cuda_help.h:117; emc_cuda.cu:1041-1056, 1136-1145):
 * maxr[i] = max(-1e10, max_r respons[r*N_images + i]). */
int emc_max_vector(emc_ctx* ctx, const float* d_respons, int N_images, int n_slices,
                   float* d_maxr);

/* cuda_respons_max_expf (emc_cuda_help.h:85-86; emc_cuda.cu:1175-1217):
 * sum[i] = sum_r expf(respons - max[i]) over terms with respons-max > -1e10.
 * Unlike the reference, respons is not modified and nothing is allocated. */
int emc_respons_max_expf(emc_ctx* ctx, const float* d_respons, const float* d_max,
                         int N_images, int n_slices, float* d_sum);

/* cuda_norm_respons_sumexpf (emc_cuda_help.h:89; emc_cuda.cu:1253-1272):
 * respons = expf(respons - lse[i]) in place; lse = log(sum) + max is formed
 * by the caller (main.cpp:384-391) and passed as d_sum. */
int emc_norm_respons_sumexpf(emc_ctx* ctx, float* d_respons, const float* d_sum,
                             const float* d_max, int N_images, int n_slices);

/* Allocation-free form of emc_respons_max_expf, for callers that cannot call
 * cudaMalloc when they run it (inside stream capture, in callbacks, under a
 * fixed device-memory budget).  No counterpart in the reference: its
 * cuda_respons_max_expf allocates an R x N temporary on every call.
 * Needs no context: work is queued on `cuda_stream` (NULL = legacy default
 * stream).  Scratch is a file-scope device array of EMC_NOALLOC_PARTIALS
 * floats (4 MiB per GPU that loads the library, held until exit), so
 * N_images may not exceed EMC_NOALLOC_PARTIALS (EMC_ERR_INVALID otherwise).
 * The first call on each device looks up the array's device address
 * (cudaGetSymbolAddress, no allocation) and should come before any stream
 * capture.  That address is cached per device for the life of the process:
 * after cudaDeviceReset on a device it is stale, so a process that resets a
 * device must not call this entry point on it again.  Calls that overlap on
 * the GPU share the array and race.  Returns EMC_ERR_CUDA only for this
 * call's own launches; an earlier error pending on the thread is left as is. */
#define EMC_NOALLOC_PARTIALS (1 << 20)
int emc_respons_max_expf_noalloc(const float* d_respons, const float* d_max, int N_images,
                                 int n_slices, float* d_sum, void* cuda_stream);

/* Convenience for the host step between the two calls above
 * (emc_helper.cpp:579-587 log_vector + sum_vectors, float):
 * lse[i] = logf(sum[i]) + max[i], on the device. */
int emc_log_sum_max(emc_ctx* ctx, const float* d_sum, const float* d_max, float* d_lse,
                    int N_images);

/* cuda_update_slices (emc_cuda_help.h:10-16; emc_cuda.cu:562-594;
 * emc_atomic.cu:33-132, 183-200): M-step slice average over active images
 * for rotations start..start+chunk-1 written to d_slices[0..chunk), then
 * nearest-voxel insertion of the chunk into d_model / d_weight with
 * weight T_r = sum_i respons.  d_rot points at the chunk's first quaternion
 * (the reference passes &d_rotations[start*4], main.cpp:458). */
int emc_update_slices(emc_ctx* ctx, const float* d_images, float* d_slices, const int* d_mask,
                      const float* d_respons, const float* d_scaling, const int* d_active_images,
                      int N_images, int slice_start, int slice_chunk, int N_2d, int side,
                      float* d_model, const float* d_x, const float* d_y, const float* d_z,
                      const float* d_rot, float* d_weight);

/* cuda_divide_model_by_weight (emc_cuda_help.h:60; emc_cuda.cu:758-786):
 * model /= weight where weight > 0, else -1. */
int emc_divide_model_by_weight(emc_ctx* ctx, int side, float* d_model, const float* d_weight);

/* cuda_normalize_model (emc_cuda_help.h:61; emc_cuda.cu:639-671, 788-798):
 * model *= 1/mean(model > 0).  Writes the mean before scaling to *h_mean
 * when h_mean is not NULL (synchronises). */
int emc_normalize_model(emc_ctx* ctx, int side, float* d_model, float* h_mean);

/* cuda_model_max / cuda_model_average (emc_cuda.cu:629-671): diagnostics,
 * synchronous, result in host memory. */
int emc_model_max(emc_ctx* ctx, const float* d_model, int n, float* h_out);
int emc_model_average(emc_ctx* ctx, const float* d_model, int n, float* h_out);

/* cuda_blur_model (emc_cuda_help.h:116; emc_cuda.cu:1404-1492): the
 * reference's intent (its FFT calls are commented out) -- negative voxels are
 * masked, the rest convolved with a periodic Gaussian of std `sigma` voxels,
 * masked voxels restored to -1.  Separable shared-memory stencil. */
int emc_blur_model(emc_ctx* ctx, float* d_model, int side, float sigma);

/* cuda_reset_real / cuda_reset_model (emc_cuda_help.h:9, 56). */
int emc_reset_real(emc_ctx* ctx, float* d_real, int len);

/* cuda_copy_real_to_device / cuda_copy_real_to_host / cuda_copy_real_d2d
 * (emc_cuda_help.h:92-97; emc_cuda.cu:885-911): n floats, synchronous with
 * respect to the host for the *_to_host form; d2d copies into dst[start..). */
int emc_copy_real_to_device(emc_ctx* ctx, const float* h_src, float* d_dst, int n);
int emc_copy_real_to_host(emc_ctx* ctx, float* h_dst, const float* d_src, int n);
int emc_copy_real_d2d(emc_ctx* ctx, float* d_dst, const float* d_src, int start, int n);
/* cuda_copy_int_to_device (emc_cuda_help.h:99; emc_cuda.cu:913-915). */
int emc_copy_int_to_device(emc_ctx* ctx, const int* h_src, int* d_dst, int n);

/* cuda_allocate_real / cuda_allocate_int / cuda_mem_free (emc_cuda_help.h:73-74,
 * 93; emc_cuda.cu:872-878, 1274-1279): device buffers for a host that drives
 * the drop-in entry points through this ABI only (e.g. the `emc` driver). */
int emc_allocate_real(emc_ctx* ctx, float** d_out, size_t n);
int emc_allocate_int(emc_ctx* ctx, int** d_out, size_t n);
int emc_mem_free(emc_ctx* ctx, void* d_ptr);

/* ---- preprocessing and model initialisation (main.cpp:92-108) ---------- */
/* read_images binning (emc_helper.cpp:226-243): raw patterns
 * [n_images][raw_h][raw_w] and their masks (int, x fastest) -> images
 * [n_images][side*side] = (sum of |raw|) / (sum of the raw mask) over the
 * stride x stride block of each output pixel, and per-pattern masks
 * [n_images][side*side] = 1 where that mask sum is > 1.  The block of output
 * pixel o starts at (int)(stride ((o - side/2) + 0.5) + raw/2 - 0.5) per axis;
 * raw pixels outside the frame count as 0. */
int emc_bin_images(emc_ctx* ctx, const float* d_raw, const int* d_raw_mask, int raw_w, int raw_h,
                   int n_images, int side, int stride, float* d_images, int* d_masks);
/* normalize_images_central_part (emc_helper.cpp:389-418; its central mask is
 * all ones, so the factor is N_2d / sum over d_mask == 1) or, with d_masks,
 * normalize_images_individual_mask (:421-438): images *= N_2d / (float sum of
 * the pattern's pixels whose mask is 1), summed in pixel order. */
int emc_normalize_images(emc_ctx* ctx, float* d_images, const int* d_mask, const int* d_masks,
                         int N_2d, int n_images);
/* mask_model (emc_helper.cpp:567-575): images = -1 where d_masks == 0. */
int emc_mask_images(emc_ctx* ctx, float* d_images, const int* d_masks, int N_2d, int n_images);
/* model_init with model_input 3 (emc_helper.cpp:458-502): the radial average
 * of all patterns, interpolated linearly in radius; -1 outside radius side/2.
 * Ring sums are FP64 (the reference sums in float). */
int emc_model_init_radial(emc_ctx* ctx, const float* d_images, int n_images, int side,
                          float* d_model);
/* model_init with model_input 1 (emc_helper.cpp:503-518): pattern i inserted
 * once with weight 1 at quaternion d_rot[i] (e.g. emc_random_rotations) by
 * the reference's host insert_slice arithmetic (emc_helper.cpp:81-135:
 * round(side/2 + 0.5 + c)); then model = model / weight where weight > 0,
 * else 0. */
int emc_model_init_orientations(emc_ctx* ctx, const float* d_images, const int* d_mask,
                                int n_images, int side, const float* d_rot, const float* d_x,
                                const float* d_y, const float* d_z, float* d_model,
                                float* d_weight);

/* ---- fused iteration (the fast path) ----------------------------------- */
typedef struct {
  int side;            /* model side s; detector is s x s                      */
  int n_images;        /* N                                                    */
  int n_rot;           /* R                                                    */
  int diff;            /* EMC_DIFF_POISSON (reference) or EMC_DIFF_TRUE_POISSON */
  int interp;          /* EMC_INTERP_*                                          */
  int precision;       /* EMC_PREC_*                                            */
  int insert_mode;     /* EMC_INSERT_*                                          */
  int known_intensity; /* 1: skip scaling (phi = 1), as known_intensity=1       */
  int normalize_images;/* 1: fold the reference's per-pattern normalisation     */
  float blur_sigma;    /* > 0: blur the model after normalisation               */
} emc_plan_desc;

typedef struct {
  double total_loglik;       /* sum_i lse_i (FP64)                              */
  double model_mean_before;  /* mean(model > 0) before normalisation            */
  double captured_mass;      /* sum of responsibilities / N (== 1 when full)    */
  int bad_pairs;             /* pairs with undefined scaling or empty overlap   */
  int reserved;
} emc_iter_stats;

/* Creates a plan: validates the description and allocates the workspace
 * (slice operands, responsibilities, scaling, LSE partials) once. */
int emc_plan_create(emc_ctx* ctx, const emc_plan_desc* desc, emc_plan** out);
int emc_plan_destroy(emc_plan* plan);
/* Bytes of device workspace the plan holds. */
size_t emc_plan_workspace_bytes(const emc_plan* plan);
/* Binds the problem's device inputs (caller-owned, must outlive the plan's
 * use) and pre-processes the patterns (FP16 count operands, compaction to
 * the masked pixels).  images [N*s*s], mask [s*s], coords [s*s] x3,
 * rotations [4R], rotation weights [R].  May be called again (new pattern
 * data, same mask pixel count) without reallocating.  With EMC_INSERT_SORTED
 * it also builds the voxel-sorted pair map (synchronously; kept by a re-bind
 * whose rotations and pixel coordinates are unchanged); EMC_ERR_UNSUPPORTED
 * when a pair code (pixel, rotation[, corner]) does not fit 32 bits. */
int emc_plan_bind(emc_plan* plan, const float* d_images, const int* d_mask, const float* d_x,
                  const float* d_y, const float* d_z, const float* d_rot,
                  const float* d_rot_weights);
/* One EMC iteration: expand, scaling, likelihood, log-sum-exp, M-step,
 * insertion, divide, normalise (+ blur).  d_model is read and overwritten
 * with the new normalised model; d_weight receives the insertion weights.
 * stats (host, may be NULL) is filled after a synchronise. */
int emc_iterate(emc_plan* plan, float* d_model, float* d_weight, float sigma,
                emc_iter_stats* stats);
/* emc_iterate in two halves (replaces the per-iteration body of main.cpp:
 * 239-480 without its host round trips).  emc_iterate_async only enqueues
 * the iteration on the context stream and returns; emc_plan_wait
 * synchronises, reports any device-side failure recorded since the previous
 * wait (EMC_ERR_TIMEOUT: a bounded pipeline wait gave up; EMC_ERR_UNSUPPORTED:
 * slice values outside the FP16 operand range) and fills stats (may be NULL)
 * for the last iteration. */
int emc_iterate_async(emc_plan* plan, float* d_model, float* d_weight, float sigma);
int emc_plan_wait(emc_plan* plan, emc_iter_stats* stats);
/* CUDA-graph form of the iteration.  emc_plan_capture records one iteration
 * on d_model/d_weight into a graph (the context stream must not be the legacy
 * default stream); emc_plan_replay(plan, sigma) launches it with a new sigma.
 * Each replay is one iteration in place on the captured buffers; call
 * emc_plan_wait for errors and stats.  Re-capture after emc_plan_bind. */
int emc_plan_capture(emc_plan* plan, float* d_model, float* d_weight);
int emc_plan_replay(emc_plan* plan, float sigma);
/* Pruned iterations (no counterpart in the reference; tensor-core path).  With pruning on, every emc_iterate after the first evaluates only
 * the (128-pattern, 128-rotation) tiles that held more than
 * (1 - min_mass) / (10 n_rotation_tiles) of some pattern's responsibility in
 * the previous iteration (patterns re-sorted by their most probable
 * rotation), plus a margin of the rotation tiles within `dilate`
 * nearest-neighbour angles of those.  When more than 1 - min_mass of the
 * mass per pattern falls in the margin, the iteration is repeated from its
 * input model as a full scan.  Responsibilities outside the evaluated tiles
 * are 0.  full_every > 0 also makes every full_every-th iteration a full scan
 * (a check of the pruning against distributions that move beyond the margin
 * between iterations).  While pruning is on, emc_plan_results is in the plan's pattern
 * order (emc_plan_pattern_order: position -> input pattern); emc_iterate_async
 * and the graph forms always run full scans. */
typedef struct {
  int pruned;                 /* the last emc_iterate evaluated a tile subset  */
  int fallback;               /* ... and was then repeated as a full scan      */
  double active_fraction;     /* evaluated share of the tiles, next iteration   */
  double core_fraction;       /* ... of which core tiles (before the margin)    */
  double margin_mass;         /* mass per pattern in margin tiles, last pruned  */
  double nn_angle;            /* median nearest-neighbour rotation angle (rad)  */
  long long pruned_iterations, fallback_iterations, full_iterations;
} emc_prune_info;
int emc_plan_set_pruning(emc_plan* plan, int on, float min_mass, float dilate, int full_every);
int emc_plan_prune_info(emc_plan* plan, emc_prune_info* info);
int emc_plan_pattern_order(emc_plan* plan, int* h_order);
/* Rotation order of the results while pruning is on (the plan keeps its
 * rotations in a spatially coherent order): row -> input rotation. */
int emc_plan_rotation_order(emc_plan* plan, int* h_order);
/* Learned rotation proposal (no counterpart in the reference).
 * emc_plan_best_quaternions: the most probable rotation of every pattern in
 * the last iteration's responsibilities, as quaternions d_quats[N][4] in the
 * input pattern order (the network's training labels).
 * emc_plan_set_proposals: seeds the next pruned iteration (pruning on) from
 * per-pattern rotation proposals d_quats[N][n_modes][4] (input pattern
 * order) instead of a previous iteration's responsibilities: the patterns
 * are sorted by their first proposal, a rotation tile is evaluated when one
 * of its rotations lies within the ball holding `fraction` of the rotation
 * group around one of the pattern tile's proposals, plus the usual margin
 * and, with probe_stride > 0, every probe_stride-th rotation tile as a probe
 * of the rest; mass in margin and probes above 1 - min_mass repeats the
 * iteration as a full scan.  The next iteration is pruned however dense the
 * seeded tiles are: emc_plan_prune_info's active_fraction tells the caller,
 * and emc_plan_set_pruning disarms it. */
int emc_plan_best_quaternions(emc_plan* plan, float* d_quats);
int emc_plan_set_proposals(emc_plan* plan, const float* d_quats, int n_modes, float fraction,
                           int probe_stride);
/* The proposal network: patterns binned to 64 x 64 (log1p of counts scaled
 * to a mean of 1), four 3x3 stride-2 convolutions of 64 channels with ReLU,
 * one linear layer to a 6D rotation (two matrix columns, Gram-Schmidt).
 * Loss per pattern min(|o - t|^2, |o + t|^2), t the label's 6D form: -t is
 * the 6D form of the Friedel mate M diag(-1, -1, 1).  Trained with Adam.
 * emc_proposal_set_data bins the patterns (side a multiple of 64) into the
 * network's input rows and standardises every input pixel by a mean and
 * spread, fitted on these patterns when fit_stats = 1 (training data), else
 * the stored ones (emc_proposal_stats gets/sets them: [2][4096], mean and
 * 1 / spread); train/loss_grad take labels d_quats[n][4] per row; predict
 * writes d_quats_out[n][2][4]: the prediction and its mate. */
typedef struct emc_proposal emc_proposal;
int emc_proposal_create(emc_ctx* ctx, unsigned long long seed, emc_proposal** out);
int emc_proposal_destroy(emc_proposal* net);
int emc_proposal_param_count(const emc_proposal* net);
/* get = 1 copies the parameters to h_params, 0 sets them (and resets Adam). */
int emc_proposal_params(emc_proposal* net, float* h_params, int get);
int emc_proposal_set_data(emc_proposal* net, const float* d_images, const int* d_mask, int side,
                          int n_images, int fit_stats);
int emc_proposal_stats(emc_proposal* net, float* h_stats, int get);
int emc_proposal_inputs(emc_proposal* net, int first, int count, float* h_out);
/* One batch (rows h_rows[B]): mean loss and the gradient of every parameter. */
int emc_proposal_loss_grad(emc_proposal* net, const int* h_rows, int B, const float* d_quats,
                           float* h_loss, float* h_grads);
/* Epochs of shuffled minibatches over h_rows[n_rows] (NULL: every row);
 * augment = 1 turns each sample in-plane by a random multiple of 90 degrees
 * (label composed with the matching turn about the beam axis); the Adam step
 * size decays from lr along a cosine to 5 % of it over the call;
 * h_epoch_loss[epochs] (may be NULL) receives each epoch's mean loss. */
int emc_proposal_train(emc_proposal* net, const float* d_quats, const int* h_rows, int n_rows,
                       int epochs, int batch, float lr, unsigned long long seed, int augment,
                       float* h_epoch_loss);
int emc_proposal_predict(emc_proposal* net, float* d_quats_out);
/* Batched reconstructions (no counterpart in the reference): n bound plans,
 * each with its own model/weight, captured (emc_plan_capture) and nested as
 * independent child graphs of one graph; emc_batch_run launches one
 * iteration of every plan (sigma per plan) in a single graph launch on the
 * first plan's context stream, so the problems run concurrently;
 * emc_batch_wait synchronises and fills stats[n] (may be NULL). */
typedef struct emc_batch emc_batch;
int emc_batch_create(emc_plan** plans, float** d_models, float** d_weights, int n,
                     emc_batch** out);
int emc_batch_run(emc_batch* batch, const float* sigmas);
int emc_batch_wait(emc_batch* batch, emc_iter_stats* stats);
int emc_batch_destroy(emc_batch* batch);
/* Precision knobs of the tensor-core kernels.
 * EMC_OPT_ESTEP_GHLO: which of the likelihood's rotation-side factors
 * G = s/(s+c) (bit 0) and H = 1/(s+c) (bit 1) carry an FP16 lo term besides
 * their FP16 hi term (one 128-column MMA per 16-pixel step each, ~2^-12
 * relative rounding of a factor without it).  -1 (default): G always, H too
 * when known_intensity fixes the scaling at 1; 0..3 set the bits. */
#define EMC_OPT_ESTEP_GHLO 3
/* EMC_OPT_MSTEP_QLO: 0 (default) multiplies responsibility/scaling as FP16
 * hi only (~2^-12 relative rounding per term), 1 as FP16 hi + lo (twice the
 * M-step MMAs). */
#define EMC_OPT_MSTEP_QLO 2
/* EMC_OPT_MSTEP_AGGREGATE: 1 combines, inside each warp, the nearest-voxel
 * insertions that land on the same voxel before one atomic (float atomics
 * only); 0 (default) issues one atomic per rotation-pixel pair. */
#define EMC_OPT_MSTEP_AGGREGATE 4
/* EMC_OPT_COUNTS_ROUND: the tensor-core path takes counts as FP16, exact for
 * integers up to 2048.  0 (default): bind rejects larger counts
 * (EMC_ERR_UNSUPPORTED); 1: integer counts up to 65504 are accepted and those
 * above 2048 are rounded to the nearest FP16 value (relative error <= 2^-12,
 * only at those pixels).  Set before emc_plan_bind. */
#define EMC_OPT_COUNTS_ROUND 5
/* EMC_OPT_ESTEP_RASTER: order of the likelihood kernel's (pattern tile,
 * rotation tile) CTAs.  g > 0 (default 8): groups of g rotation tiles, each
 * group running through all pattern tiles; g < 0: groups of -g pattern tiles
 * running through all rotation tiles.  |g| <= 4096.  Results do not depend on
 * it; L2 reuse of the operand panels does. */
#define EMC_OPT_ESTEP_RASTER 6
/* EMC_OPT_ESTEP_PAIR: 1 (default) runs full scans of the reference
 * likelihood on clusters of two CTAs with 256-row MMAs (each CTA stores half
 * of the rotation-side operands); 0 runs every scan on single CTAs.
 * emc_plan_autotune may switch it off where single CTAs are faster.  Pruned
 * iterations always use single CTAs.  The log-likelihoods agree to FP32
 * accumulation rounding (1e-6 relative). */
#define EMC_OPT_ESTEP_PAIR 7
/* EMC_OPT_MSTEP_RASTER: order of the persistent tensor-core M-step's
 * (rotation tile, pixel tile) work: g > 0 groups of g rotation tiles running
 * through all pixel tiles, g < 0 (default -16) groups of -g pixel tiles
 * running through all rotation tiles; |g| <= 4096.  Results do not depend
 * on it (with deterministic insertion, bit for bit).  At 128^3 and 256^3 the
 * default is 5-6 % faster than groups of 8 rotation tiles. */
#define EMC_OPT_MSTEP_RASTER 8
/* EMC_OPT_DEBUG_SPIN: test aid, no counterpart in the reference.  value > 0
 * caps every wait of the tensor-core pipelines (TMA ring, MMA completion,
 * accumulator hand-over) at `value` polls instead of the default 2^24, so
 * that a test can make them run out; 0 restores the default.  A wait that
 * runs out sets the plan's status and emc_plan_wait / emc_iterate return
 * EMC_ERR_TIMEOUT.  The waits on the way out are not capped: a CTA whose
 * pipeline gave up first waits until every TMA load it armed has landed and
 * every MMA it issued has completed, and a CTA pair pauses 200 us before it
 * frees its TMEM and exits, so no copy or MMA is in flight when a CTA leaves.
 * The next iteration with the default is unaffected. */
#define EMC_OPT_DEBUG_SPIN 9
/* EMC_OPT_MSTEP_PAIR: 1 (default) runs the full-scan tensor-core M-step on
 * clusters of two CTAs (256 rotations x 256 pixels per pair, 256-row MMAs,
 * half of the pixel-side operand per CTA), 0 on single CTAs (128 x 256); at
 * 128^3 the pairs measured 6.7 ms against 8.4 ms.  Pruned iterations always
 * use single CTAs;
 * where a cluster launch is refused the plan falls back to single CTAs.
 * The two shapes' models agree to FP32 accumulation rounding (1e-5
 * relative). */
#define EMC_OPT_MSTEP_PAIR 10
/* EMC_OPT_GLO_TAIL: the likelihood's G lo term (the FP16 lo half of
 * G = s/(s+c) in B = K.G^T) is applied per 128-pattern tile up to the last
 * 32-pixel block after which at most value / 1e6 of each pattern's counts
 * remain (pixels are ordered by detector radius, so the dropped blocks are
 * the dim outer ones): the term dropped there is below 2^-12 x value / 1e6
 * of B.  Default 1000 (0.1 %); 0 applies it on every block.  Recomputed at
 * once when the plan is bound. */
#define EMC_OPT_GLO_TAIL 11
int emc_plan_set_option(emc_plan* plan, int option, int value);
/* The option's current value (after emc_plan_autotune: the tile order and
 * shape it chose). */
int emc_plan_get_option(const emc_plan* plan, int option, int* value);
/* Tile-order and tile-shape autotuner of the tensor-core likelihood kernel:
 * expands d_model (sigma as in emc_iterate), times the kernel for each
 * candidate EMC_OPT_ESTEP_RASTER order on two windows of 256 waves of the SMs
 * inside its tile grid (the whole grid when smaller), scores each order by
 * its slower window and sets the fastest; with CTA pairs in use it then times
 * single-CTA tiles (128 x 128 instead of 256 x 128 patterns x rotations) on
 * the same windows and switches EMC_OPT_ESTEP_PAIR off when they are 2 %
 * faster (the two shapes' results differ by FP32 accumulation rounding,
 * 1e-6 relative).  *h_raster / *h_ms (may be NULL) receive the order and its time.  Synchronous.  Overwrites the plan's responsibilities and scaling
 * (the next emc_iterate rewrites them); d_model is not changed.  FP32 plans
 * have no tile order: *h_raster = 0.  Results of later iterations do not
 * depend on the order. */
int emc_plan_autotune(emc_plan* plan, const float* d_model, float sigma, int* h_raster,
                      float* h_ms);
/* Times one launch of the tensor-core likelihood kernel over tiles
 * [first_tile, first_tile + n_tiles) of the order `raster` (clipped to the
 * grid; CUDA events, synchronous) into *h_ms, and the grid's tile count into
 * *h_total_tiles (may be NULL).  d_model != NULL expands it first (sigma as
 * in emc_iterate); NULL reuses the operands of the last expansion.
 * Overwrites responsibilities and scaling of the covered tiles. */
int emc_plan_time_likelihood(emc_plan* plan, const float* d_model, float sigma, int raster,
                             int first_tile, int n_tiles, float* h_ms, int* h_total_tiles);
/* Instrumentation: with profiling on, emc_iterate records CUDA events on the
 * context stream between its phases; emc_plan_phase_ms (after the iteration
 * completes) returns the durations of expand, E-step (scaling + likelihood),
 * log-sum-exp, responsibility normalisation, M-step (+ insertion) and the
 * finishing model operations, in that order (n <= 6 values). */
int emc_plan_set_profiling(emc_plan* plan, int on);
int emc_plan_phase_ms(emc_plan* plan, float* ms, int n);
/* Diagnostic of the tensor-core building blocks (TMA, shared-memory
 * descriptors, tcgen05.mma, TMEM loads): D[128 x n] = A[128 x k] B[n x k]^T,
 * FP16 A and B (row-major, device), FP32 D.  n = 128 exercises the E-step
 * tile shape, n = 256 the M-step's.  No counterpart in the reference. */
int emc_tc_gemm_selftest(emc_ctx* ctx, const void* d_a, const void* d_b, float* d_d, int n, int k);
/* Device pointers into the plan's workspace (valid until the next call):
 * the normalised responsibilities [R*N] (rotation-major) and scaling [R*N]
 * of the last iteration, and the per-pattern lse [N] (double).  An iteration
 * writes the responsibilities only where the plan itself reads them back
 * (pruning); otherwise the first request for them (d_respons non-NULL) forms
 * them from the log-likelihoods with a kernel queued on the plan's stream,
 * so read them after that stream (emc_sync). */
int emc_plan_results(emc_plan* plan, const float** d_respons, const float** d_scaling,
                     const double** d_lse);

/* ---- one rank of a rotation split ---------------------------------------
 * The reference divides the rotations among MPI ranks (main.cpp:141-154):
 * each rank evaluates its range, the per-pattern maximum and sum of exp are
 * exchanged (main.cpp:367-392: MPI_MAX, then MPI_SUM of the rescaled sums),
 * each rank runs the M-step of its range with the global normaliser, and the
 * model and weight sums are all-reduced and divided by the number of ranks
 * before model / weight and normalisation (main.cpp:463-476).  A rank's plan
 * is an ordinary plan over its own rotations (rot / rot_weights at the start
 * of its range, n_rot = its count).  The three calls are asynchronous on the
 * plan's stream (emc_plan_wait reports pipeline timeouts); pruning is not
 * supported here.
 *
 * emc_rank_estep: expand, scaling and likelihood over the plan's rotations;
 *   d_max[N] = max_r L_ri (float) and d_sumexp[N] = sum_r exp(L_ri - max)
 *   (FP64) over them.  The caller forms lse_i = M + log sum_k s_k exp(m_k - M)
 *   over the ranks k, M = max_k m_k (FP64).  Replaces the rank's
 *   cuda_get_slices / cuda_update_scaling_full / cuda_calculate_responsabilities
 *   / cuda_max_vector / cuda_respons_max_expf sequence (main.cpp:284-380). */
int emc_rank_estep(emc_plan* plan, float* d_model, float sigma, float* d_max,
                   double* d_sumexp);
/* emc_rank_mstep: with the global lse[N] (FP64), the rank's responsibilities
 * and its M-step + insertion; writes the rank's un-normalised sums
 * d_model_sum[s^3] (sum of T_r x slice) and d_weight_sum[s^3] (sum of T_r)
 * for the all-reduce.  Replaces cuda_norm_respons_sumexpf and the
 * cuda_update_slices loop (main.cpp:384-462). */
int emc_rank_mstep(emc_plan* plan, const double* d_lse, float* d_model_sum,
                   float* d_weight_sum);
/* emc_model_from_sums: from the sums all-reduced over n_ranks ranks: weight =
 * weight_sum / n_ranks, model = (model_sum / n_ranks) / weight (-1 where the
 * weight is 0), then the model normalised to a positive mean of 1 and
 * blurred as the plan's desc asks (main.cpp:467-476).  With n_ranks = 1 and
 * one rank holding all rotations the three calls give emc_iterate's model. */
int emc_model_from_sums(emc_plan* plan, const float* d_model_sum, const float* d_weight_sum,
                        int n_ranks, float* d_model, float* d_weight);

#ifdef __cplusplus
}
#endif

#endif /* EMC_GB300_H */
