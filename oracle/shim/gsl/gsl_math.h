/* GSL math shim (oracle and reference-compatible headers): the reference uses
 * gsl_pow_2/3/4 and M_SQRT3 (src/fft.c:83-88,243; src/power.c:22,36,58). */
#ifndef ORACLE_SHIM_GSL_MATH_H
#define ORACLE_SHIM_GSL_MATH_H
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
