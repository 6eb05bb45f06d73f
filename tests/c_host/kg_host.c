/* A C host on the C ABI (include/kestrel_gpu.h), as a Fortran or C program would drive the
 * library in place of Run (src/TimeStepper.f90:73-112): it reads a kg_params struct (raw
 * bytes, the header's layout), creates a context, places the sources, integrates to t_end
 * and prints the step statistics, the four volume sums and the sum of the free surface
 * over the active tiles, read tile by tile and again in one call (kg_get_state).
 * Usage: kg_host PARAMS_FILE PRECISION */
#include <stdio.h>
#include <stdlib.h>

#include "kestrel_gpu.h"

int main(int argc, char** argv) {
    if (argc != 3) {
        fprintf(stderr, "usage: %s PARAMS_FILE PRECISION\n", argv[0]);
        return 2;
    }
    kg_params p;
    FILE* f = fopen(argv[1], "rb");
    if (!f || fread(&p, sizeof p, 1, f) != 1) {
        fprintf(stderr, "cannot read %s\n", argv[1]);
        return 2;
    }
    fclose(f);
    kg_ctx* ctx = NULL;
    int rc = kg_create(&p, atoi(argv[2]), &ctx);
    if (rc != KG_OK) {
        /* no GPU, or a struct the library refuses: the status and its reason, no host compute */
        printf("create %d\n%s\n", rc, kg_last_error(NULL));
        return 0;
    }
    rc = kg_load_sources(ctx);
    if (rc != KG_OK) {
        printf("load_sources %d %s\n", rc, kg_last_error(ctx));
        kg_destroy(ctx);
        return 1;
    }
    kg_step_stats st;
    rc = kg_integrate_to(ctx, p.tend, &st);
    if (rc != KG_OK) {
        printf("integrate_to %d %s\n", rc, kg_last_error(ctx));
        kg_destroy(ctx);
        return 1;
    }
    double vol[4];
    kg_volume(ctx, vol);
    int32_t n = 0;
    kg_get_active_tiles(ctx, NULL, &n);
    int32_t* ids = (int32_t*)malloc(sizeof(int32_t) * (n > 0 ? n : 1));
    kg_get_active_tiles(ctx, ids, &n);
    int cells = p.nXpertile * p.nYpertile;
    double* w = (double*)malloc(sizeof(double) * cells);
    double sw = 0.0;
    for (int k = 0; k < n; ++k) {
        kg_get_tile_field(ctx, ids[k], 1, w);
        for (int c = 0; c < cells; ++c) sw += w[c];
    }
    /* the same sum from the whole state in one call (kg_get_state) */
    int32_t n2 = n;
    int32_t* ids2 = (int32_t*)malloc(sizeof(int32_t) * (n > 0 ? n : 1));
    double* state = (double*)malloc(sizeof(double) * 4 * (size_t)cells * (n > 0 ? n : 1));
    double sw2 = 0.0;
    if (kg_get_state(ctx, ids2, &n2, state, NULL) == KG_OK && n2 == n)
        for (int k = 0; k < n; ++k)
            for (int c = 0; c < cells; ++c) sw2 += state[(size_t)k * 4 * cells + c];
    printf("ok %.17g %lld %lld %d %.17g %.17g %.17g %.17g %.17g %.17g\n", st.t, (long long)st.steps, (long long)st.rejected,
           n, vol[0], vol[1], vol[2], vol[3], sw, sw2);
    free(state);
    free(ids2);
    free(w);
    free(ids);
    kg_destroy(ctx);
    return 0;
}
