/* Link stubs for the shim headers.  None is reached by the oracle: the
 * reference functions that would call them (model file output, random
 * quaternions) are not used. */
#include <stddef.h>
#include "spimage.h"
#include "gsl/gsl_rng.h"
Image* sp_image_alloc(int x, int y, int z) { (void)x; (void)y; (void)z; return NULL; }
int sp_image_write(const Image* img, const char* filename, long long flags) {
  (void)img; (void)filename; (void)flags; return -1;
}
void sp_image_free(Image* img) { (void)img; }
double gsl_rng_uniform(const gsl_rng* r) { (void)r; return 0.5; }
