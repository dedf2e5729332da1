/*
 * c_adjoint_harness.c: the calls the sky-cuda Rust crate's `Adjoint` makes
 * through the C ABI (sky-tracer_gb300/rust/sky-cuda/src/lib.rs), made from
 * C with device buffers from the CUDA runtime, so that a test exercises the
 * crate's forward/backward sequence where no Rust toolchain exists.
 *
 *   c_adjoint_harness SCENE_FILE WIDTH HEIGHT SPP SEED PARAMS_FILE DLOSS_FILE OUT_PREFIX
 *
 * SCENE_FILE as for c_abi_harness.c; PARAMS_FILE holds the float32 layer
 * parameters [3 * layers + 2]; DLOSS_FILE the float32 dLoss/dfilm
 * [pixels][bands].  With all band multipliers one, merged-layer tracking and
 * tabulated phase sampling (Adjoint::new), it runs the forward with a
 * chain-radiance buffer, then the backward that reads it, and writes
 * OUT_PREFIX.film (float32), OUT_PREFIX.layer_grad and OUT_PREFIX.band_grad
 * (float64).  Then Adjoint::forward_batch / backward_batch over two renders,
 * one at the scene's sun (a zero direction) and one at the sun direction
 * (0, 0.5, 0.8660254), each with its own chain-radiance buffer and the same
 * dLoss/dfilm: OUT_PREFIX.batch_film0, .batch_film1 (float32),
 * .batch_layer_grad and .batch_band_grad (float64, the gradient of the summed
 * loss).  It also checks the refusals the crate maps to
 * RenderError::InvalidConfig (segment-restart tracking, a chain buffer shorter
 * than the render's chains, a missing status, an empty batch).
 * Exit status 0 on success, 2 without a CUDA device.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime.h>

#include "sky_cuda.h"

static void* read_rows(FILE* f, size_t count, size_t size) {
    void* p = malloc(count * size + 1);
    if (!p || fread(p, size, count, f) != count) {
        fprintf(stderr, "short input file\n");
        exit(1);
    }
    return p;
}

static void* device(size_t bytes) {
    void* p = NULL;
    if (cudaMalloc(&p, bytes) != cudaSuccess || cudaMemset(p, 0, bytes) != cudaSuccess) {
        fprintf(stderr, "cudaMalloc of %zu bytes failed\n", bytes);
        exit(1);
    }
    return p;
}

static void write_file(const char* prefix, const char* ext, const void* dev, size_t bytes) {
    char path[4096];
    snprintf(path, sizeof(path), "%s.%s", prefix, ext);
    void* host = malloc(bytes);
    FILE* f = fopen(path, "wb");
    if (!host || cudaMemcpy(host, dev, bytes, cudaMemcpyDeviceToHost) != cudaSuccess || !f ||
        fwrite(host, 1, bytes, f) != bytes) {
        fprintf(stderr, "writing %s failed\n", path);
        exit(1);
    }
    fclose(f);
    free(host);
}

static int fail(const char* what, int st) {
    char msg[1024];
    sky_cuda_last_error(msg, sizeof(msg));
    fprintf(stderr, "%s: status %d: %s\n", what, st, msg);
    return 1;
}

int main(int argc, char** argv) {
    if (argc != 9) {
        fprintf(stderr, "usage: %s SCENE_FILE WIDTH HEIGHT SPP SEED PARAMS_FILE DLOSS_FILE OUT_PREFIX\n", argv[0]);
        return 1;
    }
    int devices = 0;
    if (cudaGetDeviceCount(&devices) != cudaSuccess || devices == 0) {
        printf("no CUDA device\n");
        return 2;
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
    memcpy(d.sun_direction, sc + 3, 3 * sizeof(float));
    d.sun_angular_radius_rad = sc[6];
    d.sun_solid_angle_sr = sc[7];
    d.ground_albedo = sc[8];
    d.bands = read_rows(f, n[0], sizeof(SkyBand));
    d.atmosphere = read_rows(f, n[1], sizeof(SkyAtmospherePoint));
    d.aerosol = read_rows(f, n[2], sizeof(SkyAerosolPoint));
    d.aerosol_optics = read_rows(f, (size_t)n[0] * SKY_SPECIES_COUNT, sizeof(SkyAerosolOptics));
    d.majorants_km_inv = read_rows(f, (size_t)n[0] * n[3], sizeof(float));
    d.phase_values = read_rows(f, (size_t)SKY_SPECIES_COUNT * n[0] * n[4], sizeof(float));
    fclose(f);

    /* GpuScene::new */
    SkyScene* scene = NULL;
    int st = sky_cuda_scene_create(&d, &scene);
    if (st != SKY_OK) return fail("sky_cuda_scene_create", st);
    /* Adjoint::new: render_config() of the reference fields, then merged-layer
       tracking and tabulated phase sampling */
    SkyRenderConfig c;
    memset(&c, 0, sizeof(c));
    c.width = (uint32_t)strtoul(argv[2], NULL, 10);
    c.height = (uint32_t)strtoul(argv[3], NULL, 10);
    c.spp = (uint32_t)strtoul(argv[4], NULL, 10);
    c.direct_light_samples = 1;
    c.seed = strtoull(argv[5], NULL, 0);
    c.observer_altitude_km = 0.2f;
    c.tracking = SKY_TRACKING_MERGED_LAYERS;
    c.phase_sampling = SKY_PHASE_TABULATED;
    const uint32_t B = d.band_count;
    const size_t pixels = (size_t)c.width * c.height, cells = pixels * B;
    /* Adjoint::param_count */
    const uint32_t np = sky_cuda_adjoint_param_count(scene);
    if (np != 3u * d.majorant_layers + 2u) {
        fprintf(stderr, "param count %u\n", np);
        return 1;
    }
    FILE* pf = fopen(argv[6], "rb");
    FILE* lf = fopen(argv[7], "rb");
    if (!pf || !lf) {
        perror("inputs");
        return 1;
    }
    float* host_params = read_rows(pf, np, sizeof(float));
    float* host_dloss = read_rows(lf, cells, sizeof(float));
    fclose(pf);
    fclose(lf);

    /* the caller's device buffers */
    float* layer = device(np * sizeof(float));
    float* band = device((size_t)B * SKY_ADJOINT_BAND_PARAMS * sizeof(float));
    float* ones = malloc((size_t)B * SKY_ADJOINT_BAND_PARAMS * sizeof(float));
    for (size_t i = 0; i < (size_t)B * SKY_ADJOINT_BAND_PARAMS; ++i) ones[i] = 1.0f;
    float* dloss = device(cells * sizeof(float));
    if (cudaMemcpy(layer, host_params, np * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(band, ones, (size_t)B * SKY_ADJOINT_BAND_PARAMS * sizeof(float), cudaMemcpyHostToDevice) !=
            cudaSuccess ||
        cudaMemcpy(dloss, host_dloss, cells * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) {
        fprintf(stderr, "upload failed\n");
        return 1;
    }
    double* cell_sum = device(cells * sizeof(double));
    double* cell_sumsq = device(cells * sizeof(double));
    float* film = device(cells * sizeof(float));
    uint32_t* status = device(sizeof(uint32_t));
    float* chains = device(cells * c.spp * sizeof(float));
    double* layer_grad = device(np * sizeof(double));
    double* band_grad = device((size_t)B * SKY_ADJOINT_BAND_PARAMS * sizeof(double));

    SkyAdjointParams p;
    memset(&p, 0, sizeof(p));
    p.layer_params = layer;
    p.band_params = band;
    p.estimator = SKY_ADJOINT_SEGMENT_INTEGRALS;
    p.chain_radiance = chains;
    p.chain_radiance_len = cells * c.spp;
    SkyDeviceOutputs o;
    memset(&o, 0, sizeof(o));
    o.cell_sum = cell_sum;
    o.cell_sumsq = cell_sumsq;
    o.film = film;
    o.status = status;
    SkyAdjointGrads g;
    memset(&g, 0, sizeof(g));
    g.dloss_dfilm = dloss;
    g.layer_grad = layer_grad;
    g.band_grad = band_grad;
    g.status = status;

    /* Adjoint::forward, Adjoint::backward on the default stream */
    if ((st = sky_cuda_adjoint_forward(scene, &c, &p, &o, NULL)) != SKY_OK) return fail("adjoint forward", st);
    if ((st = sky_cuda_adjoint_backward(scene, &c, &p, &g, NULL)) != SKY_OK) return fail("adjoint backward", st);
    uint32_t watchdog = 1;
    if (cudaDeviceSynchronize() != cudaSuccess ||
        cudaMemcpy(&watchdog, status, sizeof(watchdog), cudaMemcpyDeviceToHost) != cudaSuccess || watchdog != 0) {
        fprintf(stderr, "forward/backward failed or tripped the watchdog (%u)\n", watchdog);
        return 1;
    }
    /* refusals that the crate maps to RenderError::InvalidConfig */
    SkyRenderConfig restart = c;
    restart.tracking = SKY_TRACKING_SEGMENT_RESTART;
    if ((st = sky_cuda_adjoint_forward(scene, &restart, &p, &o, NULL)) != SKY_ERR_INVALID_CONFIG) {
        fprintf(stderr, "segment-restart tracking returned %d\n", st);
        return 1;
    }
    /* a chain buffer shorter than the render's chains is refused */
    SkyAdjointParams short_buffer = p;
    short_buffer.chain_radiance_len = cells * c.spp - 1u;
    if ((st = sky_cuda_adjoint_forward(scene, &c, &short_buffer, &o, NULL)) != SKY_ERR_INVALID_CONFIG) {
        fprintf(stderr, "a short chain buffer returned %d\n", st);
        return 1;
    }
    SkyAdjointGrads no_status = g;
    no_status.status = NULL;
    if ((st = sky_cuda_adjoint_backward(scene, &c, &p, &no_status, NULL)) != SKY_ERR_INVALID_CONFIG) {
        fprintf(stderr, "a backward without status returned %d\n", st);
        return 1;
    }
    write_file(argv[8], "film", film, cells * sizeof(float));
    write_file(argv[8], "layer_grad", layer_grad, np * sizeof(double));
    write_file(argv[8], "band_grad", band_grad, (size_t)B * SKY_ADJOINT_BAND_PARAMS * sizeof(double));

    /* Adjoint::forward_batch, Adjoint::backward_batch: two renders, one launch
       per direction; the parameter set's own chain buffer is not read */
    static const float batch_sun[2][3] = {{0.0f, 0.0f, 0.0f}, {0.0f, 0.5f, 0.8660254f}};
    SkyAdjointJob jobs[2];
    memset(jobs, 0, sizeof(jobs));
    void* batch_buffers[2][4];
    for (int i = 0; i < 2; ++i) {
        SkyAdjointJob* j = &jobs[i];
        j->config = c;
        memcpy(j->sun_direction, batch_sun[i], sizeof(batch_sun[i]));
        batch_buffers[i][0] = j->outputs.cell_sum = device(cells * sizeof(double));
        batch_buffers[i][1] = j->outputs.cell_sumsq = device(cells * sizeof(double));
        batch_buffers[i][2] = j->outputs.film = device(cells * sizeof(float));
        batch_buffers[i][3] = j->chain_radiance = device(cells * c.spp * sizeof(float));
        j->outputs.status = status;
        j->chain_radiance_len = cells * c.spp;
        j->dloss_dfilm = dloss;
    }
    double* batch_layer_grad = device(np * sizeof(double));
    double* batch_band_grad = device((size_t)B * SKY_ADJOINT_BAND_PARAMS * sizeof(double));
    SkyAdjointGrads bg = g;
    bg.dloss_dfilm = NULL;
    bg.layer_grad = batch_layer_grad;
    bg.band_grad = batch_band_grad;
    if ((st = sky_cuda_adjoint_forward_batch(scene, jobs, 2, &p, NULL)) != SKY_OK)
        return fail("adjoint forward batch", st);
    if ((st = sky_cuda_adjoint_backward_batch(scene, jobs, 2, &p, &bg, NULL)) != SKY_OK)
        return fail("adjoint backward batch", st);
    if (cudaDeviceSynchronize() != cudaSuccess ||
        cudaMemcpy(&watchdog, status, sizeof(watchdog), cudaMemcpyDeviceToHost) != cudaSuccess || watchdog != 0) {
        fprintf(stderr, "the batch failed or tripped the watchdog (%u)\n", watchdog);
        return 1;
    }
    if ((st = sky_cuda_adjoint_forward_batch(scene, jobs, 0, &p, NULL)) != SKY_ERR_INVALID_CONFIG) {
        fprintf(stderr, "an empty batch returned %d\n", st);
        return 1;
    }
    write_file(argv[8], "batch_film0", jobs[0].outputs.film, cells * sizeof(float));
    write_file(argv[8], "batch_film1", jobs[1].outputs.film, cells * sizeof(float));
    write_file(argv[8], "batch_layer_grad", batch_layer_grad, np * sizeof(double));
    write_file(argv[8], "batch_band_grad", batch_band_grad, (size_t)B * SKY_ADJOINT_BAND_PARAMS * sizeof(double));
    for (int i = 0; i < 2; ++i)
        for (int k = 0; k < 4; ++k) cudaFree(batch_buffers[i][k]);
    cudaFree(batch_layer_grad);
    cudaFree(batch_band_grad);
    cudaFree(layer);
    cudaFree(band);
    cudaFree(dloss);
    cudaFree(cell_sum);
    cudaFree(cell_sumsq);
    cudaFree(film);
    cudaFree(status);
    cudaFree(chains);
    cudaFree(layer_grad);
    cudaFree(band_grad);
    sky_cuda_scene_destroy(scene);
    printf("%s: adjoint %zux%u x %u bands x %u spp, %u parameters\n", sky_cuda_version(), (size_t)c.width, c.height,
           B, c.spp, np);
    return 0;
}
