/* Minimal stand-in for libspimage's header, written for this project so that
 * the reference's rotations.c and CUDA kernels compile for the oracle build.
 * It declares only what those files name: the `real` type (float, as the
 * reference is built), the matrix structs with the fields they read, the size
 * macros and the image I/O prototypes (stubbed in spimage_stubs.c, never
 * called by the oracle).  Test infrastructure; not part of the product. */
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
Image* sp_image_alloc(int x, int y, int z);
int sp_image_write(const Image* img, const char* filename, long long flags);
void sp_image_free(Image* img);
#ifdef __cplusplus
}
#endif
#endif
