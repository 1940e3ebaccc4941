/* Minimal <gsl/gsl_math.h> for drivers built against libfftgal_gb300: the
 * reference's drivers use gsl_pow_2/3/4 and M_SQRT3 from GSL
 * (src/app/DLsb.c:7, src/app/DLss.c:7); the library itself needs no GSL. */
#ifndef FFTGAL_GSL_MATH_H
#define FFTGAL_GSL_MATH_H
#include <math.h>
#ifndef M_PI
#define M_PI 3.14159265358979323846264338328
#endif
#ifndef M_SQRT3
#define M_SQRT3 1.73205080756887729352744634151
#endif
static inline double gsl_pow_2(const double x) { return x * x; }
static inline double gsl_pow_3(const double x) { return x * x * x; }
static inline double gsl_pow_4(const double x) { double x2 = x * x; return x2 * x2; }
#endif
