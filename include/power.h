/* power-spectrum estimators -- drop-in replacement for the reference's
 * src/power.h:1-13 (same prototypes, same output text format). */
#ifndef POWER_H
#define POWER_H
#include "fft.h"
#include "gal.h"

#ifdef __cplusplus
extern "C" {
#endif

/* P(k) = |delta(k)|^2 / V - Pshot, in place; call this first (src/power.c:12-27) */
void P(fft_t *grid, gal_t *part);

/* power spectrum multipoles l = 0,2,4,6 written to `file` (src/power.c:30-101);
 * Pl's all proportional to P0 when los[] = {0,0,0}; los is normalised in place */
void Pl(fft_t *grid, gal_t *part, double los[3], double dK, char *file);
/* power spectrum wedges, 3 mu bins, written to `file` (src/power.c:104-178) */
void Pmu(fft_t *grid, gal_t *part, double los[3], double dK, char *file);

#ifdef __cplusplus
}
#endif
#endif
