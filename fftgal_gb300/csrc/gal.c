/* Catalog container and host-side catalog transforms of the reference's
 * src/gal.h API (src/gal.c:11-159), in plain C.  The catalog stays on the
 * host; the GPU library uploads positions when a paint needs them. */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <time.h>
#include <math.h>
#include "gal.h"

/* external definitions of the C99 inline helpers declared in gal.h */
extern inline double pdist2(double x1, double y1, double z1,
                            double x0, double y0, double z0, double L);
extern inline void hat(double vec[3]);

static void fail(const char *what) {
    fprintf(stderr, "%s: out of memory\n", what);
    abort();
}

gal_t *gal_init(long Np, double V) {
    gal_t *self = (gal_t *)malloc(sizeof(gal_t));
    if (!self) fail("gal_init()");
    self->Np = Np;
    self->V = V;
    size_t n = (size_t)(Np > 0 ? Np : 1);
    self->x = (double *)malloc(n * sizeof(double));
    self->y = (double *)malloc(n * sizeof(double));
    self->z = (double *)malloc(n * sizeof(double));
    if (!self->x || !self->y || !self->z) fail("gal_init()");
    self->vx = self->vy = self->vz = NULL;
    self->rand = NULL;
    return self;
}

static double *grow(double *p, long Np, const char *what) {
    double *q = (double *)realloc(p, (size_t)(Np > 0 ? Np : 1) * sizeof(double));
    if (!q) fail(what);
    return q;
}

void gal_resize(gal_t *self, long Np) {
    self->Np = Np;
    self->x = grow(self->x, Np, "gal_resize()");
    self->y = grow(self->y, Np, "gal_resize()");
    self->z = grow(self->z, Np, "gal_resize()");
    if (self->vx) self->vx = grow(self->vx, Np, "gal_resize()");
    if (self->vy) self->vy = grow(self->vy, Np, "gal_resize()");
    if (self->vz) self->vz = grow(self->vz, Np, "gal_resize()");
}

void gal_free(gal_t *self) {
    if (self != NULL) {
        gal_free(self->rand);
        free(self->x); free(self->y); free(self->z);
        free(self->vx); free(self->vy); free(self->vz);
    }
    free(self);
}

void gal_wrap(gal_t *self, double L) {
    clock_t t = clock();
    double Linv = 1 / L;
    for (long p = 0; p < self->Np; ++p) {
        self->x[p] -= L * floor(self->x[p] * Linv);
        self->y[p] -= L * floor(self->y[p] * Linv);
        self->z[p] -= L * floor(self->z[p] * Linv);
    }
    fprintf(stderr, "gal_wrap() %.2fs\n", (double)(clock() - t) / CLOCKS_PER_SEC);
}

gal_t *gal_rsd(gal_t *self, double los[3], double aH) {
    clock_t t = clock();
    hat(los);
    double aHinv = 1 / aH;
    gal_t *out = gal_init(self->Np, self->V);
    for (long p = 0; p < out->Np; ++p) {
        double vdl = los[0] * self->vx[p] + los[1] * self->vy[p] + los[2] * self->vz[p];
        out->x[p] = self->x[p] + aHinv * vdl * los[0];
        out->y[p] = self->y[p] + aHinv * vdl * los[1];
        out->z[p] = self->z[p] + aHinv * vdl * los[2];
    }
    fprintf(stderr, "gal_rsd() %.2fs, los[]={%.3f,%.3f,%.3f}\n",
            (double)(clock() - t) / CLOCKS_PER_SEC, los[0], los[1], los[2]);
    return out;
}

/* Seeded uniform generator for the sub-volume randoms: splitmix64, seed from
 * GSL_RNG_SEED (the reference draws them from GSL's default generator with
 * the same environment variable, src/gal.c:105-109; its stream is not
 * reproduced). */
static uint64_t rng_state;
static int rng_ready = 0;

static double uniform01(void) {
    if (!rng_ready) {
        const char *e = getenv("GSL_RNG_SEED");
        rng_state = e ? strtoull(e, NULL, 10) : 0;
        rng_ready = 1;
    }
    uint64_t z = (rng_state += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

gal_t *gal_subbox(gal_t *self, double box[7], double alpha) {
    clock_t t = clock();
    double x0 = box[0], x1 = box[1], y0 = box[2], y1 = box[3];
    double z0 = box[4], z1 = box[5], L = box[6];
    x1 = x0 + remainder(x1 - x0, L);
    y1 = y0 + remainder(y1 - y0, L);
    z1 = z0 + remainder(z1 - z0, L);
    if (!(x1 > x0 && y1 > y0 && z1 > z0)) {
        fprintf(stderr, "gal_subbox(): empty sub-box\n");
        abort();
    }
    double Vsub = (x1 - x0) * (y1 - y0) * (z1 - z0);
    gal_t *sub = gal_init(self->Np, Vsub);
    long n = 0;
    for (long p = 0; p < self->Np; ++p)
        if (remainder(self->x[p] - x0, L) >= 0 && remainder(self->x[p] - x1, L) < 0
         && remainder(self->y[p] - y0, L) >= 0 && remainder(self->y[p] - y1, L) < 0
         && remainder(self->z[p] - z0, L) >= 0 && remainder(self->z[p] - z1, L) < 0) {
            sub->x[n] = self->x[p];
            sub->y[n] = self->y[p];
            sub->z[n] = self->z[p];
            ++n;
        }
    gal_resize(sub, n);
    long Nr = lround(n / alpha);
    gal_t *rand = gal_init(Nr, Vsub);
    for (long p = 0; p < Nr; ++p) {
        rand->x[p] = x0 + (x1 - x0) * uniform01();
        rand->y[p] = y0 + (y1 - y0) * uniform01();
        rand->z[p] = z0 + (z1 - z0) * uniform01();
    }
    sub->rand = rand;
    fprintf(stderr, "gal_subbox() %.2fs, picked out %ld+%ld particles\n",
            (double)(clock() - t) / CLOCKS_PER_SEC, n, Nr);
    return sub;
}

gal_t *gal_subsphere(gal_t *self, double sphere[5], double alpha) {
    clock_t t = clock();
    double x0 = sphere[0], y0 = sphere[1], z0 = sphere[2];
    double R = sphere[3], L = sphere[4];
    if (!(2 * R <= L)) {
        fprintf(stderr, "gal_subsphere(): sphere larger than the box\n");
        abort();
    }
    double R2 = R * R, Vsub = 4 * M_PI / 3 * R2 * R;
    gal_t *sub = gal_init(self->Np, Vsub);
    long n = 0;
    for (long p = 0; p < self->Np; ++p)
        if (pdist2(self->x[p], self->y[p], self->z[p], x0, y0, z0, L) < R2) {
            sub->x[n] = self->x[p];
            sub->y[n] = self->y[p];
            sub->z[n] = self->z[p];
            ++n;
        }
    gal_resize(sub, n);
    long Nr = lround(n / alpha);
    gal_t *rand = gal_init(Nr, Vsub);
    for (long p = 0; p < Nr; ++p) {
        do {
            rand->x[p] = x0 + R * (2 * uniform01() - 1);
            rand->y[p] = y0 + R * (2 * uniform01() - 1);
            rand->z[p] = z0 + R * (2 * uniform01() - 1);
        } while (pdist2(rand->x[p], rand->y[p], rand->z[p], x0, y0, z0, L) >= R2);
    }
    sub->rand = rand;
    fprintf(stderr, "gal_subsphere() %.2fs, picked out %ld+%ld particles\n",
            (double)(clock() - t) / CLOCKS_PER_SEC, n, Nr);
    return sub;
}
