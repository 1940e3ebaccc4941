/* External definitions of the C99 `inline` helpers declared in the reference
 * header gal.h (pdist2, hat; src/gal.h:10-26), so that any call the compiler
 * does not inline still links.  Used only when building the reference as an
 * oracle (oracle/Makefile, target `ref`). */
#include "gal.h"
extern inline double pdist2(double x1, double y1, double z1,
                            double x0, double y0, double z0, double L);
extern inline void hat(double vec[3]);
