/*
 * c_abi_harness.c: the calls the sky-cuda Rust crate makes through the C ABI
 * (sky-tracer_gb300/rust/sky-cuda/src/lib.rs), made from C, so that a test
 * exercises the crate's exact call sequence where no Rust toolchain exists.
 *
 *   c_abi_harness SCENE_FILE WIDTH HEIGHT SPP SEED PROJECTION FILM_OUT
 *
 * SCENE_FILE holds the scene's tables as tests/test_c_harness.py writes them:
 * "SKYT", five uint32 counts (bands, atmosphere rows, aerosol rows, majorant
 * layers, phase bins), eleven float scalars (ground radius, atmosphere
 * radius, top altitude, sun direction x/y/z, sun angular radius, sun solid
 * angle, ground albedo, two unused), then the rows of SkyBand, SkyAtmosphere
 * Point, SkyAerosolPoint, SkyAerosolOptics, the majorants and the phase
 * values, in that order.
 *
 * It renders the film once through sky_cuda_render_desc (sky_cuda::render)
 * and once through a resident scene (sky_cuda::GpuScene), checks that both
 * films are equal, checks the error path (an invalid config returns
 * SKY_ERR_INVALID_CONFIG with the reference's message, as RenderError::
 * InvalidConfig), and writes the film as float32 to FILM_OUT.  Exit status 0
 * on success, 2 without a CUDA device (the reference's NoAdapter skip).
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "sky_cuda.h"

static void* read_rows(FILE* f, size_t count, size_t size) {
    void* p = malloc(count * size + 1);
    if (!p || fread(p, size, count, f) != count) {
        fprintf(stderr, "short scene file\n");
        exit(1);
    }
    return p;
}

int main(int argc, char** argv) {
    if (argc != 8) {
        fprintf(stderr, "usage: %s SCENE_FILE WIDTH HEIGHT SPP SEED PROJECTION FILM_OUT\n", argv[0]);
        return 1;
    }
    FILE* f = fopen(argv[1], "rb");
    if (!f) {
        perror(argv[1]);
        return 1;
    }
    char magic[4];
    uint32_t n[5];
    float sc[11];
    if (fread(magic, 1, 4, f) != 4 || memcmp(magic, "SKYT", 4) != 0 || fread(n, 4, 5, f) != 5 ||
        fread(sc, 4, 11, f) != 11) {
        fprintf(stderr, "not a scene file\n");
        return 1;
    }
    SkySceneDesc d;
    memset(&d, 0, sizeof(d));
    d.band_count = n[0];
    d.atmosphere_len = n[1];
    d.aerosol_len = n[2];
    d.majorant_layers = n[3];
    d.phase_bins = n[4];
    d.ground_radius_km = sc[0];
    d.atmosphere_radius_km = sc[1];
    d.top_altitude_km = sc[2];
    d.sun_direction[0] = sc[3];
    d.sun_direction[1] = sc[4];
    d.sun_direction[2] = sc[5];
    d.sun_angular_radius_rad = sc[6];
    d.sun_solid_angle_sr = sc[7];
    d.ground_albedo = sc[8];
    d.bands = read_rows(f, n[0], sizeof(SkyBand));
    d.atmosphere = read_rows(f, n[1], sizeof(SkyAtmospherePoint));
    d.aerosol = read_rows(f, n[2], sizeof(SkyAerosolPoint));
    d.aerosol_optics = read_rows(f, (size_t)n[0] * SKY_SPECIES_COUNT, sizeof(SkyAerosolOptics));
    d.majorants_km_inv = read_rows(f, (size_t)n[0] * n[3], sizeof(float));
    d.phase_values = read_rows(f, (size_t)SKY_SPECIES_COUNT * n[0] * n[4], sizeof(float));
    d.band_xyz_weights = NULL;
    fclose(f);

    /* render_config(): the reference's fields, extensions zero */
    SkyRenderConfig c;
    memset(&c, 0, sizeof(c));
    c.width = (uint32_t)strtoul(argv[2], NULL, 10);
    c.height = (uint32_t)strtoul(argv[3], NULL, 10);
    c.spp = (uint32_t)strtoul(argv[4], NULL, 10);
    c.direct_light_samples = 1;
    c.seed = strtoull(argv[5], NULL, 0);
    c.observer_altitude_km = 0.2f;
    c.output_projection = (uint32_t)strtoul(argv[6], NULL, 10);
    const size_t len = (size_t)c.width * c.height * d.band_count;
    float* film = malloc(len * sizeof(float));
    float* film2 = malloc(len * sizeof(float));
    char msg[1024];

    /* sky_cuda::render */
    int st = sky_cuda_render_desc(&d, &c, film, len, NULL);
    if (st == SKY_ERR_NO_DEVICE) {
        sky_cuda_last_error(msg, sizeof(msg));
        printf("no CUDA device: %s\n", msg);
        return 2;
    }
    if (st != SKY_OK) {
        sky_cuda_last_error(msg, sizeof(msg));
        fprintf(stderr, "sky_cuda_render_desc: status %d: %s\n", st, msg);
        return 1;
    }
    /* sky_cuda::GpuScene::new + render + drop */
    SkyScene* scene = NULL;
    if ((st = sky_cuda_scene_create(&d, &scene)) != SKY_OK ||
        (st = sky_cuda_render(scene, &c, film2, len, NULL)) != SKY_OK) {
        sky_cuda_last_error(msg, sizeof(msg));
        fprintf(stderr, "resident render: status %d: %s\n", st, msg);
        return 1;
    }
    size_t differ = 0;
    for (size_t i = 0; i < len; ++i) {
        const float a = film[i], b = film2[i];
        const float tol = 1e-6f * (a > b ? a : b);
        if (a - b > tol || b - a > tol) ++differ;
    }
    if (differ) {
        fprintf(stderr, "one-shot and resident films differ in %zu values\n", differ);
        return 1;
    }
    /* the error path: RenderError::InvalidConfig and its message */
    SkyRenderConfig bad = c;
    bad.width = 0;
    st = sky_cuda_render(scene, &bad, film2, len, NULL);
    const int err_status = sky_cuda_last_error(msg, sizeof(msg));
    if (st != SKY_ERR_INVALID_CONFIG || err_status != st || !strstr(msg, "greater than zero")) {
        fprintf(stderr, "invalid config: status %d (%d), message '%s'\n", st, err_status, msg);
        return 1;
    }
    st = sky_cuda_render_desc(NULL, &c, film2, len, NULL);
    if (st != SKY_ERR_INVALID_CONFIG) {
        fprintf(stderr, "a null descriptor returned %d\n", st);
        return 1;
    }
    sky_cuda_scene_destroy(scene);

    FILE* out = fopen(argv[7], "wb");
    if (!out || fwrite(film, sizeof(float), len, out) != len) {
        perror(argv[7]);
        return 1;
    }
    fclose(out);
    printf("%s: %ux%u x %u bands x %u spp, film written\n", sky_cuda_version(), c.width, c.height, d.band_count,
           c.spp);
    return 0;
}
