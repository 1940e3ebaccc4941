/* QPM cubic-box mock loader of the reference's io.h (src/io/qpm.c:9-34):
 * one galaxy per line, columns x y z vx vy vz mass flag id, the last three
 * skipped. */
#include <stdio.h>
#include <stdlib.h>
#include <time.h>
#include "io/io.h"

gal_t *gal_loadqpm_cubic(char *file, double L) {
    clock_t t = clock();
    FILE *fp = fopen(file, "r");
    if (!fp) {
        fprintf(stderr, "gal_loadqpm_cubic(): cannot open %s\n", file);
        abort();
    }
    long Np = 0;
    int c;
    while ((c = fgetc(fp)) != EOF)
        if (c == '\n') ++Np;
    rewind(fp);
    gal_t *part = gal_init(Np, L * L * L);
    size_t n = (size_t)(Np > 0 ? Np : 1);
    part->vx = (double *)malloc(n * sizeof(double));
    part->vy = (double *)malloc(n * sizeof(double));
    part->vz = (double *)malloc(n * sizeof(double));
    if (!part->vx || !part->vy || !part->vz) {
        fprintf(stderr, "gal_loadqpm_cubic(): out of memory\n");
        abort();
    }
    for (long i = 0; i < Np; ++i) {
        int got = fscanf(fp, "%lf %lf %lf %lf %lf %lf %*f %*d %*d\n", part->x + i, part->y + i,
                         part->z + i, part->vx + i, part->vy + i, part->vz + i);
        if (got != 6) {
            fprintf(stderr, "gal_loadqpm_cubic(): bad line %ld in %s\n", i + 1, file);
            abort();
        }
    }
    fclose(fp);
    fprintf(stderr, "gal_loadqpm_cubic() %.2fs, loaded %ld galaxies\n",
            (double)(clock() - t) / CLOCKS_PER_SEC, Np);
    return part;
}
