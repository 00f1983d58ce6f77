/* A plain-C caller of the C ABI (include/pisco_gb300.h), written as an FFI
 * binding would use it: builds the CPU-runnable workload's beam with the host
 * PolBeam steps, convolves (TUNED, scan order and sky order), maps the TOD
 * back with the map-maker and writes the results.
 *
 *   ffi_c1 <nside_sky> <n> <sky.f32: 3 x npix> <scan.f32: 3 x n (ra, dec, pa)>
 *          <tod.f32 out: 2 x n> <map.f32 out: 4 x npix (I, Q, U, hits)>
 *
 * Exit status 0 on success; the sky-order TOD must equal the scan-order TOD
 * bit for bit (exit 3 otherwise). */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "pisco_gb300.h"

#define PI 3.14159265358979323846

static int fail(const char* what, pisco_status st, const pisco_ctx* ctx)
{
    fprintf(stderr, "%s: %s (%s)\n", what, pisco_status_string(st),
            ctx ? pisco_last_error(ctx) : "");
    return 1;
}

static void* load(const char* path, size_t bytes)
{
    FILE* f = fopen(path, "rb");
    void* p = malloc(bytes);
    if (!f || !p || fread(p, 1, bytes, f) != bytes) {
        fprintf(stderr, "cannot read %s\n", path);
        exit(2);
    }
    fclose(f);
    return p;
}

static void save(const char* path, const void* p, size_t bytes)
{
    FILE* f = fopen(path, "wb");
    if (!f || fwrite(p, 1, bytes, f) != bytes) {
        fprintf(stderr, "cannot write %s\n", path);
        exit(2);
    }
    fclose(f);
}

int main(int argc, char** argv)
{
    if (argc != 7) {
        fprintf(stderr, "usage: %s nside n sky.f32 scan.f32 tod.f32 map.f32\n", argv[0]);
        return 2;
    }
    const int nside = atoi(argv[1]);
    const long n = atol(argv[2]);
    const long npix = 12L * nside * nside;
    float* sky = (float*)load(argv[3], sizeof(float) * 3 * (size_t)npix);
    float* scan = (float*)load(argv[4], sizeof(float) * 3 * (size_t)n);
    const float *ra = scan, *dec = scan + n, *pa = scan + 2 * n;

    /* beam: nside 256, 5 deg, circular FWHM 2 deg, epsilon 0.01, both detectors */
    const int nsb = 256;
    const long npb = pisco_beam_npix_for_radius(nsb, 5.0 * PI / 180.0);
    double* f[4];
    float *t[8], *o[8];
    for (int k = 0; k < 4; ++k) f[k] = (double*)malloc(sizeof(double) * (size_t)npb);
    for (int k = 0; k < 8; ++k) {
        t[k] = (float*)malloc(sizeof(float) * (size_t)npb);
        o[k] = (float*)malloc(sizeof(float) * (size_t)npb);
    }
    pisco_status st = pisco_beam_gaussian_fields(nsb, npb, 2.0, 2.0, 0.0, f[0], f[1], f[2], f[3]);
    if (st != PISCO_OK) return fail("gaussian fields", st, NULL);
    for (int d = 0; d < 2; ++d) {
        st = pisco_beam_from_fields(npb, f[0], f[1], f[2], f[3], t[4 * d], t[4 * d + 1],
                                    t[4 * d + 2], t[4 * d + 3]);
        if (st != PISCO_OK) return fail("beam from fields", st, NULL);
    }
    const float* const ta[4] = {t[0], t[1], t[2], t[3]};
    const float* const tb[4] = {t[4], t[5], t[6], t[7]};
    float* const oa[4] = {o[0], o[1], o[2], o[3]};
    float* const ob[4] = {o[4], o[5], o[6], o[7]};
    st = pisco_beam_build(nsb, npb, 0.01, 'p', nside, ta, tb, oa, ob);
    if (st != PISCO_OK) return fail("beam build", st, NULL);

    /* convolver: create, set sky / beam / scan, forward, destroy */
    pisco_run_config cfg = {1, 0, 0, 0, 0, 0, 0, 1 << 20, 0};
    pisco_ctx* ctx = NULL;
    st = pisco_create(&cfg, &ctx);
    if (st != PISCO_OK) return fail("create", st, NULL);
    const void* a[4] = {o[0], o[1], o[2], o[3]};
    const void* b[4] = {o[4], o[5], o[6], o[7]};
    if ((st = pisco_set_beam(ctx, nsb, npb, a, b, PISCO_FLOAT32)) != PISCO_OK)
        return fail("set_beam", st, ctx);
    if ((st = pisco_set_sky(ctx, nside, sky, sky + npix, sky + 2 * npix, NULL, PISCO_FLOAT32)) !=
        PISCO_OK)
        return fail("set_sky", st, ctx);
    if ((st = pisco_set_scan(ctx, n, ra, dec, pa, PISCO_FLOAT32)) != PISCO_OK)
        return fail("set_scan", st, ctx);
    float* tod = (float*)malloc(sizeof(float) * 2 * (size_t)n);
    float* tod2 = (float*)malloc(sizeof(float) * 2 * (size_t)n);
    if ((st = pisco_forward(ctx, 'p', tod, tod + n, PISCO_FLOAT32, PISCO_FORM_TUNED)) != PISCO_OK)
        return fail("forward", st, ctx);
    if ((st = pisco_set_sample_order(ctx, PISCO_ORDER_SKY)) != PISCO_OK)
        return fail("set_sample_order", st, ctx);
    if ((st = pisco_forward(ctx, 'p', tod2, tod2 + n, PISCO_FLOAT32, PISCO_FORM_TUNED)) != PISCO_OK)
        return fail("forward (sky order)", st, ctx);
    pisco_destroy(ctx);
    if (memcmp(tod, tod2, sizeof(float) * 2 * (size_t)n) != 0) {
        fprintf(stderr, "sky-order TOD differs from scan-order TOD\n");
        return 3;
    }
    save(argv[5], tod, sizeof(float) * 2 * (size_t)n);

    /* map-maker: detectors a (0 deg) and b (90 deg), data [det][s] */
    float* ra2 = (float*)malloc(sizeof(float) * 2 * (size_t)n);
    float* dec2 = (float*)malloc(sizeof(float) * 2 * (size_t)n);
    float* pa2 = (float*)malloc(sizeof(float) * 2 * (size_t)n);
    for (int d = 0; d < 2; ++d) {
        memcpy(ra2 + d * n, ra, sizeof(float) * (size_t)n);
        memcpy(dec2 + d * n, dec, sizeof(float) * (size_t)n);
        memcpy(pa2 + d * n, pa, sizeof(float) * (size_t)n);
    }
    const float pol[2] = {0.0f, (float)(PI / 2)};
    pisco_map* map = NULL;
    if ((st = pisco_map_create(nside, 0, &map)) != PISCO_OK) return fail("map_create", st, NULL);
    st = pisco_map_accumulate(map, n, ra2, dec2, pa2, 2, pol, tod, PISCO_FLOAT32);
    if (st != PISCO_OK) {
        fprintf(stderr, "map_accumulate: %s\n", pisco_map_last_error(map));
        return 1;
    }
    if ((st = pisco_map_solve(map)) != PISCO_OK) return fail("map_solve", st, NULL);
    float* m = (float*)malloc(sizeof(float) * 4 * (size_t)npix);
    int* hits = (int*)malloc(sizeof(int) * (size_t)npix);
    if ((st = pisco_map_get(map, m, m + npix, m + 2 * npix, hits)) != PISCO_OK)
        return fail("map_get", st, NULL);
    for (long p = 0; p < npix; ++p) m[3 * npix + p] = (float)hits[p];
    pisco_map_destroy(map);
    save(argv[6], m, sizeof(float) * 4 * (size_t)npix);
    printf("ok %ld samples, %ld beam pixels\n", n, npb);
    return 0;
}
