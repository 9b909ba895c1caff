/* Minimal stand-in for libspimage's header, written for this project so that
 * the reference's rotations.c, host helper (emc_helper.cpp) and CUDA kernels compile
 * for the oracle build.  It declares only what those files name: the `real` type (float, as the
 * reference is built), the matrix structs with the fields they read, the size
 * macros and element accessors, and the image I/O prototypes (stubbed in
 * spimage_stubs.c and ref_helper_harness.cpp).  Test infrastructure; not part
 * of the product. */
#ifndef EMC_SHIM_SPIMAGE_H
#define EMC_SHIM_SPIMAGE_H
#include <math.h>
#include <stdlib.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef float real;
typedef struct { real re, im; } Complex;
typedef struct { unsigned int rows, cols; real* data; } sp_matrix;
typedef struct { unsigned int rows, cols; int* data; } sp_imatrix;
typedef struct { unsigned int x, y, z; real* data; } sp_3matrix;
typedef struct { unsigned int x, y, z; Complex* data; } sp_c3matrix;
typedef struct { unsigned int x, y, z; int* data; } sp_i3matrix;
typedef struct { sp_c3matrix* image; sp_i3matrix* mask; } Image;
#define sp_matrix_rows(m) ((m)->rows)
#define sp_matrix_cols(m) ((m)->cols)
#define sp_matrix_size(m) ((m)->rows * (m)->cols)
#define sp_imatrix_size(m) ((m)->rows * (m)->cols)
#define sp_3matrix_x(m) ((m)->x)
#define sp_3matrix_y(m) ((m)->y)
#define sp_3matrix_z(m) ((m)->z)
#define sp_3matrix_size(m) ((m)->x * (m)->y * (m)->z)
static inline Complex sp_cinit(real re, real im) { Complex c; c.re = re; c.im = im; return c; }
/* element access as libspimage lays matrices out: a 2D matrix's element
 * (row, col) at data[col * rows + row]; a 3D matrix's (x, y, z) at
 * data[(z * y_size + y) * x_size + x] */
static inline real sp_matrix_get(const sp_matrix* m, unsigned r, unsigned c) { return m->data[c * m->rows + r]; }
static inline void sp_matrix_set(sp_matrix* m, unsigned r, unsigned c, real v) { m->data[c * m->rows + r] = v; }
static inline int sp_imatrix_get(const sp_imatrix* m, unsigned r, unsigned c) { return m->data[c * m->rows + r]; }
static inline void sp_imatrix_set(sp_imatrix* m, unsigned r, unsigned c, int v) { m->data[c * m->rows + r] = v; }
static inline real sp_3matrix_get(const sp_3matrix* m, unsigned x, unsigned y, unsigned z) {
  return m->data[(z * m->y + y) * m->x + x];
}
static inline void sp_3matrix_set(sp_3matrix* m, unsigned x, unsigned y, unsigned z, real v) {
  m->data[(z * m->y + y) * m->x + x] = v;
}
static inline real sp_real(Complex c) { return c.re; }
static inline real sp_cabs(Complex c) { return (real)sqrt((double)c.re * c.re + (double)c.im * c.im); }
Image* sp_image_alloc(int x, int y, int z);
int sp_image_write(const Image* img, const char* filename, long long flags);
void sp_image_free(Image* img);
/* defined only by the host-helper harness (ref_helper_harness.cpp) */
sp_matrix* sp_matrix_alloc(unsigned rows, unsigned cols);
sp_imatrix* sp_imatrix_alloc(unsigned rows, unsigned cols);
Image* sp_image_read(const char* filename, int flags);
Image* sp_gaussian_blur(Image* in, real radius);
Complex sp_image_get(const Image* img, int x, int y, int z);
int sp_image_mask_get(const Image* img, int x, int y, int z);
int sp_image_x(const Image* img);
int sp_image_y(const Image* img);
int sp_image_z(const Image* img);
#ifdef __cplusplus
}
#endif
#endif
