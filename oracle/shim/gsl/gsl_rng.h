/* GSL RNG shim (oracle only): the reference draws sub-box/sub-sphere randoms
 * with gsl_rng_uniform (src/gal.c:105-113,142-152). This shim is a seeded
 * splitmix64 generator; GSL_RNG_SEED in the environment sets the seed. It does
 * not reproduce GSL's mt19937 stream (randoms are out of the hot path). */
#ifndef ORACLE_SHIM_GSL_RNG_H
#define ORACLE_SHIM_GSL_RNG_H
#include <stdlib.h>
#include <stdint.h>
typedef struct { uint64_t s; } gsl_rng;
typedef int gsl_rng_type;
static const gsl_rng_type *gsl_rng_default = 0;
static inline void gsl_rng_env_setup(void) {}
static inline gsl_rng *gsl_rng_alloc(const gsl_rng_type *t) {
    (void)t;
    gsl_rng *r = (gsl_rng *)malloc(sizeof(gsl_rng));
    const char *e = getenv("GSL_RNG_SEED");
    r->s = e ? strtoull(e, NULL, 10) : 0;
    return r;
}
static inline double gsl_rng_uniform(gsl_rng *r) {
    uint64_t z = (r->s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}
#endif
