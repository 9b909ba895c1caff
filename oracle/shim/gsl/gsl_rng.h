/* Stand-in for GSL's RNG header (declarations only): rotations.c names
 * gsl_rng in quaternion_random and emc_helper.cpp allocates a taus generator
 * in model_init.  The oracle's definitions (spimage_stubs.c,
 * ref_helper_harness.cpp) replace GSL's generator by a seeded stand-in; GSL's
 * own sequence is not reproduced. */
#ifndef EMC_SHIM_GSL_RNG_H
#define EMC_SHIM_GSL_RNG_H
#ifdef __cplusplus
extern "C" {
#endif
typedef struct gsl_rng gsl_rng;
typedef struct gsl_rng_type gsl_rng_type;
extern const gsl_rng_type* gsl_rng_taus;
gsl_rng* gsl_rng_alloc(const gsl_rng_type* T);
void gsl_rng_set(const gsl_rng* r, unsigned long seed);
double gsl_rng_uniform(const gsl_rng* r);
#ifdef __cplusplus
}
#endif
#endif
