/* Stand-in for GSL's RNG header (declarations only): rotations.c names
 * gsl_rng in quaternion_random, which the oracle never calls. */
#ifndef EMC_SHIM_GSL_RNG_H
#define EMC_SHIM_GSL_RNG_H
#ifdef __cplusplus
extern "C" {
#endif
typedef struct gsl_rng gsl_rng;
double gsl_rng_uniform(const gsl_rng* r);
#ifdef __cplusplus
}
#endif
#endif
