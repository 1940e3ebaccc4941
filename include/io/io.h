/* catalog loader -- drop-in replacement for the reference's src/io/io.h:1-6 */
#ifndef FFTGAL_IO_H
#define FFTGAL_IO_H
#include "../gal.h"

#ifdef __cplusplus
extern "C" {
#endif

/* load QPM galaxies from periodic boxes,
 * 6 columns skipping the halo mass, satellite flag, and halo id
 * (src/io/qpm.c:9-34) */
gal_t *gal_loadqpm_cubic(char *file, double L);

#ifdef __cplusplus
}
#endif
#endif
