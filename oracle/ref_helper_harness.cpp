// Test infrastructure (the oracle's checker; nothing in the product links it):
// plain-array C wrappers around the reference's own host helper
// (emc_helper.cpp, compiled unchanged from the reference tree by
// build_ref.sh --helper) so that the tests can run its detector geometry,
// binning, normalisation, masking and model initialisation on given inputs:
//
//   refh_calculate_coordinates     emc_helper.cpp:55-79
//   refh_read_images               emc_helper.cpp:198-248 (sp_image_read served
//                                  from caller-registered frames)
//   refh_normalize_images          emc_helper.cpp:369-387 / 389-418 / 421-438
//   refh_mask_model                emc_helper.cpp:567-575
//   refh_model_init                emc_helper.cpp:445-518 (model_input 0, 1, 3)
//   refh_quaternion_random         rotations.c:30-41 on the stand-in generator
//
// Layouts are libspimage's (see oracle/shim/spimage.h): a side x side matrix
// element (x, y) lives at [y * side + x]; a model voxel (x, y, z) at
// [(z * side + y) * side + x]; raw frame pixel (x, y) at [y * raw_w + x].
//
// What the reference takes from libraries that are absent here is stood in
// for by the definitions below: sp_image_read hands out the registered frames
// (file name "<index>.h5"), pixels outside a frame read as 0 (the reference
// would read out of bounds), and GSL's taus generator is replaced by a seeded
// splitmix64 stream, so the uniform start model and the random orientations
// are those of that stream, not of GSL.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "emc_helper.h"
#include "hdf5.h"

// ---- libspimage stand-ins ------------------------------------------------
extern "C" {

sp_matrix* sp_matrix_alloc(unsigned rows, unsigned cols) {
  sp_matrix* m = (sp_matrix*)std::malloc(sizeof(sp_matrix));
  m->rows = rows;
  m->cols = cols;
  m->data = (real*)std::calloc((size_t)rows * cols, sizeof(real));
  return m;
}

sp_imatrix* sp_imatrix_alloc(unsigned rows, unsigned cols) {
  sp_imatrix* m = (sp_imatrix*)std::malloc(sizeof(sp_imatrix));
  m->rows = rows;
  m->cols = cols;
  m->data = (int*)std::calloc((size_t)rows * cols, sizeof(int));
  return m;
}

static const float* g_frames = nullptr;
static const int* g_frame_masks = nullptr;
static int g_raw_w = 0, g_raw_h = 0, g_n_frames = 0;

Image* sp_image_read(const char* filename, int flags) {
  (void)flags;
  const char* base = std::strrchr(filename, '/');
  const int i = std::atoi(base ? base + 1 : filename);
  if (!g_frames || i < 0 || i >= g_n_frames) return nullptr;
  const size_t n = (size_t)g_raw_w * g_raw_h;
  Image* img = (Image*)std::malloc(sizeof(Image));
  img->image = (sp_c3matrix*)std::malloc(sizeof(sp_c3matrix));
  img->mask = (sp_i3matrix*)std::malloc(sizeof(sp_i3matrix));
  img->image->x = img->mask->x = (unsigned)g_raw_w;
  img->image->y = img->mask->y = (unsigned)g_raw_h;
  img->image->z = img->mask->z = 1;
  img->image->data = (Complex*)std::malloc(n * sizeof(Complex));
  img->mask->data = (int*)std::malloc(n * sizeof(int));
  for (size_t p = 0; p < n; ++p) {
    img->image->data[p] = sp_cinit(g_frames[(size_t)i * n + p], 0.0f);
    img->mask->data[p] = g_frame_masks[(size_t)i * n + p];
  }
  return img;
}

void sp_image_free(Image* img) {
  if (!img) return;
  std::free(img->image->data);
  std::free(img->mask->data);
  std::free(img->image);
  std::free(img->mask);
  std::free(img);
}

Image* sp_image_alloc(int, int, int) { return nullptr; }
int sp_image_write(const Image*, const char*, long long) { return -1; }
Image* sp_gaussian_blur(Image*, real) { return nullptr; }  // blur_image is never set here

static bool inside(const Image* img, int x, int y, int z) {
  return x >= 0 && y >= 0 && z >= 0 && x < (int)img->image->x && y < (int)img->image->y &&
         z < (int)img->image->z;
}

Complex sp_image_get(const Image* img, int x, int y, int z) {
  if (!inside(img, x, y, z)) return sp_cinit(0.0f, 0.0f);
  return img->image->data[((size_t)z * img->image->y + y) * img->image->x + x];
}

int sp_image_mask_get(const Image* img, int x, int y, int z) {
  if (!inside(img, x, y, z)) return 0;
  return img->mask->data[((size_t)z * img->mask->y + y) * img->mask->x + x];
}

int sp_image_x(const Image* img) { return (int)img->image->x; }
int sp_image_y(const Image* img) { return (int)img->image->y; }
int sp_image_z(const Image* img) { return (int)img->image->z; }

// ---- GSL stand-in: a seeded splitmix64 stream ---------------------------
struct gsl_rng_type { int unused; };
static const gsl_rng_type g_taus = {0};
const gsl_rng_type* gsl_rng_taus = &g_taus;
struct gsl_rng { uint64_t state; };
static gsl_rng g_rng = {0};
static uint64_t g_rng_base = 0;

gsl_rng* gsl_rng_alloc(const gsl_rng_type*) { return &g_rng; }
void gsl_rng_set(const gsl_rng*, unsigned long seed) { g_rng.state = g_rng_base + seed; }
double gsl_rng_uniform(const gsl_rng*) {
  uint64_t z = (g_rng.state += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

// ---- HDF5 stand-ins: the HDF5 reader is not used ------------------------
hid_t H5Fopen(const char*, unsigned, hid_t) { return -1; }
hid_t H5Dopen(hid_t, const char*, hid_t) { return -1; }
herr_t H5Dread(hid_t, hid_t, hid_t, hid_t, hid_t, void*) { return -1; }
herr_t H5Dclose(hid_t) { return -1; }
herr_t H5Fclose(hid_t) { return -1; }

}  // extern "C"

// ---- wrappers -------------------------------------------------------------
namespace {

sp_matrix view(float* data, int side) { return sp_matrix{(unsigned)side, (unsigned)side, data}; }
sp_imatrix iview(int* data, int side) { return sp_imatrix{(unsigned)side, (unsigned)side, data}; }

Configuration config(int side, int n_images, int stride) {
  Configuration c;
  std::memset(&c, 0, sizeof(c));
  c.model_side = side;
  c.N_images = n_images;
  c.read_stride = stride;
  c.image_prefix = "";
  return c;
}

}  // namespace

extern "C" {

int refh_calculate_coordinates(int side, float pixel_size, float distance, float wavelength,
                               float* x, float* y, float* z) {
  emc_helper h;
  sp_matrix mx = view(x, side), my = view(y, side), mz = view(z, side);
  h.calculate_coordinates(side, pixel_size, distance, wavelength, &mx, &my, &mz);
  return 0;
}

// frames [n][raw_h][raw_w] and their masks -> images [n][side*side] and
// per-pattern masks [n][side*side]
int refh_read_images(const float* frames, const int* frame_masks, int raw_w, int raw_h, int n,
                     int side, int stride, float* images, int* masks) {
  g_frames = frames;
  g_frame_masks = frame_masks;
  g_raw_w = raw_w;
  g_raw_h = raw_h;
  g_n_frames = n;
  emc_helper h;
  Configuration c = config(side, n, stride);
  sp_imatrix** m = (sp_imatrix**)std::malloc(sizeof(sp_imatrix*) * (size_t)n);
  sp_matrix** im = h.read_images(c, m);
  const size_t n2 = (size_t)side * side;
  for (int i = 0; i < n; ++i) {
    std::memcpy(images + i * n2, im[i]->data, n2 * sizeof(float));
    std::memcpy(masks + i * n2, m[i]->data, n2 * sizeof(int));
    std::free(im[i]->data);
    std::free(im[i]);
    std::free(m[i]->data);
    std::free(m[i]);
  }
  std::free(im);
  std::free(m);
  g_frames = nullptr;
  g_frame_masks = nullptr;
  return 0;
}

// mode 0: normalize_images (common mask), 1: normalize_images_central_part
// (radius), 2: normalize_images_individual_mask (masks [n][side*side])
int refh_normalize_images(float* images, const int* mask, const int* masks, int n, int side,
                          int mode, float radius) {
  emc_helper h;
  Configuration c = config(side, n, 1);
  const size_t n2 = (size_t)side * side;
  sp_matrix* v = (sp_matrix*)std::malloc(sizeof(sp_matrix) * (size_t)n);
  sp_matrix** pv = (sp_matrix**)std::malloc(sizeof(sp_matrix*) * (size_t)n);
  sp_imatrix* mv = (sp_imatrix*)std::malloc(sizeof(sp_imatrix) * (size_t)n);
  sp_imatrix** pm = (sp_imatrix**)std::malloc(sizeof(sp_imatrix*) * (size_t)n);
  for (int i = 0; i < n; ++i) {
    v[i] = view(images + i * n2, side);
    pv[i] = &v[i];
    if (masks) {
      mv[i] = iview(const_cast<int*>(masks) + i * n2, side);
      pm[i] = &mv[i];
    }
  }
  sp_imatrix common = iview(const_cast<int*>(mask), side);
  int rc = 0;
  if (mode == 0) h.normalize_images(pv, &common, c);
  else if (mode == 1) h.normalize_images_central_part(pv, &common, radius, c);
  else if (mode == 2 && masks) h.normalize_images_individual_mask(pv, pm, c);
  else rc = -1;
  std::free(v);
  std::free(pv);
  std::free(mv);
  std::free(pm);
  return rc;
}

int refh_mask_model(float* images, const int* masks, int n, int side) {
  emc_helper h;
  const size_t n2 = (size_t)side * side;
  sp_matrix* v = (sp_matrix*)std::malloc(sizeof(sp_matrix) * (size_t)n);
  sp_matrix** pv = (sp_matrix**)std::malloc(sizeof(sp_matrix*) * (size_t)n);
  sp_imatrix* mv = (sp_imatrix*)std::malloc(sizeof(sp_imatrix) * (size_t)n);
  sp_imatrix** pm = (sp_imatrix**)std::malloc(sizeof(sp_imatrix*) * (size_t)n);
  for (int i = 0; i < n; ++i) {
    v[i] = view(images + i * n2, side);
    pv[i] = &v[i];
    mv[i] = iview(const_cast<int*>(masks) + i * n2, side);
    pm[i] = &mv[i];
  }
  h.mask_model(n, pv, pm, (int)n2);
  std::free(v);
  std::free(pv);
  std::free(mv);
  std::free(pm);
  return 0;
}

// model_init for model_input 0, 1 or 3; the stand-in generator starts from
// `seed` (gsl_rng_set(rng, 0) inside model_init adds 0)
int refh_model_init(int model_input, const float* images, const int* mask, int n, int side,
                    const float* x, const float* y, const float* z, unsigned long long seed,
                    float* model, float* weight) {
  if (model_input != 0 && model_input != 1 && model_input != 3) return -1;
  emc_helper h;
  Configuration c = config(side, n, 1);
  c.model_input = model_input;
  const size_t n2 = (size_t)side * side;
  sp_matrix* v = (sp_matrix*)std::malloc(sizeof(sp_matrix) * (size_t)(n > 0 ? n : 1));
  sp_matrix** pv = (sp_matrix**)std::malloc(sizeof(sp_matrix*) * (size_t)(n > 0 ? n : 1));
  for (int i = 0; i < n; ++i) {
    v[i] = view(const_cast<float*>(images) + i * n2, side);
    pv[i] = &v[i];
  }
  sp_imatrix mk = iview(const_cast<int*>(mask), side);
  sp_matrix mx = view(const_cast<float*>(x), side), my = view(const_cast<float*>(y), side),
            mz = view(const_cast<float*>(z), side);
  sp_3matrix m{(unsigned)side, (unsigned)side, (unsigned)side, model};
  sp_3matrix w{(unsigned)side, (unsigned)side, (unsigned)side, weight};
  g_rng_base = seed;
  h.model_init(c, &m, &w, pv, &mk, &mx, &my, &mz);
  std::free(v);
  std::free(pv);
  return 0;
}

// the n quaternions model_init(model_input 1) draws from the stand-in
// generator started at `seed`: [n][4]
int refh_quaternion_random(unsigned long long seed, int n, float* quats) {
  g_rng_base = seed;
  gsl_rng* r = gsl_rng_alloc(gsl_rng_taus);
  gsl_rng_set(r, 0);
  for (int i = 0; i < n; ++i) {
    Quaternion* q = quaternion_random(r);
    for (int k = 0; k < 4; ++k) quats[4 * i + k] = q->q[k];
    std::free(q);
  }
  return 0;
}

}  // extern "C"
