/*
 * sky_cuda.h — C ABI of the GB300 spectral sky path tracer.
 *
 * This is the drop-in boundary for the hot path of the reference's
 * `sky-spectral-path-tracer` crate: every entry point takes plain pointers and
 * sizes, and every table row below has the byte layout the reference uploads
 * to its compute shader, so a host that already packs those rows
 * (crates/sky-spectral-path-tracer/src/integrator.rs:319-418) can hand them to
 * this library unchanged.
 *
 * Conventions
 *   - Every function returns an `int` status (SkyStatus); 0 is success.  The
 *     message of the last failure on the calling thread is available through
 *     sky_cuda_last_error().
 *   - The caller owns every host buffer.  The library owns the device memory
 *     behind an opaque SkyScene and frees it in sky_cuda_scene_destroy().
 *   - Calls are thread-compatible per scene: one scene is used by one thread
 *     at a time; different scenes may be used from different threads.
 */
#ifndef SKY_CUDA_H
#define SKY_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SKY_CUDA_ABI_VERSION 1u
/* Aerosol species per band: inso, waso, soot, suso
 * (crates/sky-core/src/atmosphere.rs:6-8). */
#define SKY_SPECIES_COUNT 4u

/* Status codes.  Codes 1-6 correspond one-to-one to the reference's
 * `RenderError` variants (integrator.rs:18-26). */
typedef enum SkyStatus {
    SKY_OK = 0,
    SKY_ERR_INVALID_CONFIG = 1, /* RenderError::InvalidConfig */
    SKY_ERR_NO_DEVICE = 2,      /* RenderError::NoAdapter     */
    SKY_ERR_DEVICE_INIT = 3,    /* RenderError::RequestDevice */
    SKY_ERR_COPY = 4,           /* RenderError::BufferMap     */
    SKY_ERR_SYNC = 5,           /* RenderError::Poll          */
    SKY_ERR_WATCHDOG = 6,       /* RenderError::Watchdog      */
    SKY_ERR_OUT_OF_MEMORY = 7,
    SKY_ERR_LAUNCH = 8,
    SKY_ERR_IO = 9              /* host-side table loading      */
} SkyStatus;

/* ---- Table rows (layouts of integrator.rs:77-112) ---------------------- */

/* = GpuBand (integrator.rs:79-86), 24 bytes. */
typedef struct SkyBand {
    float center_nm;
    float lower_nm;
    float upper_nm;
    float ozone_cross_section_cm2;
    float solar_radiance_w_m2_sr;
    float rayleigh_cross_section_m2;
} SkyBand;

/* = GpuAtmospherePoint (integrator.rs:90-95), 16 bytes. */
typedef struct SkyAtmospherePoint {
    float altitude_km;
    float temperature_k;
    float air_cm3;
    float ozone_cm3;
} SkyAtmospherePoint;

/* = GpuAerosolPoint (integrator.rs:99-105), 32 bytes. */
typedef struct SkyAerosolPoint {
    float altitude_km;
    float mass_g_m3[SKY_SPECIES_COUNT];
    float _pad[3];
} SkyAerosolPoint;

/* = GpuAerosolOptics (integrator.rs:109-112), 8 bytes. */
typedef struct SkyAerosolOptics {
    float scattering_km_inv_per_g_m3;
    float absorption_km_inv_per_g_m3;
} SkyAerosolOptics;

/* ---- Scene ------------------------------------------------------------- */

/*
 * Everything the reference's `SceneData` contributes to the shader
 * (atmosphere.rs:121-133, packed at integrator.rs:321-416).  Band count and
 * phase-bin count are run-time fields here, not the reference's compile-time
 * 41 and 1024.
 */
typedef struct SkySceneDesc {
    uint32_t band_count;
    uint32_t atmosphere_len;      /* rows in `atmosphere`, ascending altitude */
    uint32_t aerosol_len;         /* rows in `aerosol`, ascending altitude    */
    uint32_t majorant_layers;     /* MajorantGrid::layer_count                */
    uint32_t phase_bins;          /* bins per (species, band) phase table     */
    uint32_t _reserved0;
    float ground_radius_km;       /* Planet (geometry.rs:12-17)               */
    float atmosphere_radius_km;
    float top_altitude_km;        /* MajorantGrid::top_altitude_km            */
    float sun_direction[3];       /* Sun (atmosphere.rs:12-37)                */
    float sun_angular_radius_rad;
    float sun_solid_angle_sr;
    float ground_albedo;          /* GROUND_ALBEDO, 0.18 in atmosphere.rs:9   */
    float _reserved1;
    const SkyBand* bands;                    /* [band_count]                   */
    const SkyAtmospherePoint* atmosphere;    /* [atmosphere_len]               */
    const SkyAerosolPoint* aerosol;          /* [aerosol_len]                  */
    const SkyAerosolOptics* aerosol_optics;  /* [band_count][SPECIES]          */
    const float* majorants_km_inv;           /* [band_count][majorant_layers]  */
    const float* phase_values;               /* [SPECIES][band_count][bins], cube-root mu grid */
    const float* band_xyz_weights;           /* [band_count][3] CIE 1931 at band centre; may be NULL */
} SkySceneDesc;

typedef struct SkyScene SkyScene;

/* ---- Render configuration ---------------------------------------------- */

typedef enum SkyProjection {
    SKY_PROJECTION_PANORAMA = 0,     /* OutputProjection::Panorama   */
    SKY_PROJECTION_SKY_VIEW_LUT = 1  /* OutputProjection::SkyViewLut */
} SkyProjection;

typedef enum SkyPhaseSampling {
    /* The reference shader: isotropic direction, weighted by the mixed phase
     * (sky_trace.wgsl:735-738). */
    SKY_PHASE_ISOTROPIC = 0,
    /* Pick a component by sigma_s,i / sigma_s and invert its tabulated CDF
     * (phase.rs:53-69, sampling.rs:182-185). */
    SKY_PHASE_TABULATED = 1
} SkyPhaseSampling;

typedef enum SkyTracking {
    /* The reference's layered delta tracking: every majorant segment starts a
     * fresh exponential flight and the draw that overshoots the segment is
     * discarded (sky_trace.wgsl:405-475).  Reproduces its random stream. */
    SKY_TRACKING_SEGMENT_RESTART = 0,
    /* Same collision distribution, one exponential draw per tentative
     * collision: the residual optical depth is carried across segment
     * boundaries instead of being re-drawn. */
    SKY_TRACKING_RESIDUAL_CARRY = 1,
    /* Residual carry over a coarser tracking grid: adjacent majorant layers
     * of each band are merged (majorant = max of the merged layers, so still
     * a bound) where the extra null collisions cost less than the saved
     * layer crossings.  Same collision distribution again. */
    SKY_TRACKING_MERGED_LAYERS = 2
} SkyTracking;

typedef enum SkyKernel {
    SKY_KERNEL_AUTO = 0,       /* the wavefront kernel                                   */
    SKY_KERNEL_PLAIN = 1,      /* one chain per lane, a warp per cell; cell sums in a
                                  fixed order                                            */
    SKY_KERNEL_WAVEFRONT = 2   /* persistent ray loop: one ray per lane per iteration,
                                  per-lane chain regeneration                            */
} SkyKernel;

/* Add into the sums already held by the outputs instead of overwriting them
 * (progressive rendering; the reference accumulates 2-spp dispatches the
 * same way, integrator.rs:252-283). */
#define SKY_FLAG_ACCUMULATE 1u
/* Fill SkyRenderStats.events in sky_cuda_render / _xyz / _rgb.  The kernels
 * that count events run ~3 % slower, so without this flag the events are
 * left zero.  (sky_cuda_render_device counts into SkyDeviceOutputs.counters
 * whenever that pointer is given.) */
#define SKY_FLAG_COUNT_EVENTS 2u

/*
 * = RenderConfig (config.rs:2-12) followed by extensions.  A config whose
 * extension fields are all zero renders exactly what the reference shader
 * renders.
 */
typedef struct SkyRenderConfig {
    uint32_t width;
    uint32_t height;
    uint32_t spp;
    uint32_t direct_light_samples;  /* 0 is treated as 1 (integrator.rs:325); at most 1024 */
    uint64_t seed;
    float sun_elevation_deg;        /* recorded only; the sun is in the scene */
    float sun_azimuth_deg;
    float observer_altitude_km;
    uint32_t output_projection;     /* SkyProjection */
    /* extensions */
    uint32_t sample_offset;         /* index of the first sample (resume)      */
    uint32_t phase_sampling;        /* SkyPhaseSampling                        */
    uint32_t rr_start_depth;        /* 0 -> 4 (sky_trace.wgsl:692)            */
    uint32_t max_orders;            /* 0 -> unbounded; else paths end after this many events */
    uint32_t watchdog_limit;        /* 0 -> 1024 (integrator.rs:14)           */
    uint32_t kernel;                /* SkyKernel                               */
    uint32_t flags;                 /* SKY_FLAG_*                              */
    uint32_t tracking;              /* SkyTracking                             */
    /* Pixel-row slab: render only rows [row_begin, row_begin + row_count) of
     * the width x height image (row_count 0 = every row; row_begin must then
     * be 0).  Every output holds the slab only (width * row_count pixels,
     * pixel-major from row row_begin).  Pixels keep their whole-image index
     * in the random-number counter and the camera, so slabs rendered
     * separately (on several GPUs) and concatenated equal the whole render.
     * The reference splits its dispatch the same way, over (x, y, band)
     * workgroups (integrator.rs:252-283). */
    uint32_t row_begin;
    uint32_t row_count;
} SkyRenderConfig;

/* Event counters, indexed by these values (the per-event work weights of
 * the roofline are defined over them). */
typedef enum SkyEvent {
    SKY_EVENT_TRACK_STEP = 0,  /* free-flight sample inside a segment + accept test */
    SKY_EVENT_SEGMENT = 1,     /* majorant-layer segment set-up                   */
    SKY_EVENT_BOUNDARY = 2,    /* ground / top-of-atmosphere intersection          */
    SKY_EVENT_SCATTER = 3,     /* real scattering event                            */
    SKY_EVENT_NEE = 4,         /* sun-cone light sample                            */
    SKY_EVENT_GROUND = 5,      /* ground hit                                       */
    SKY_EVENT_CHAIN = 6,       /* camera ray start + accumulation                  */
    SKY_EVENT_COUNT = 8
} SkyEvent;

typedef struct SkyRenderStats {
    double kernel_ms;       /* device time of the tracing kernel(s), CUDA events */
    double total_ms;        /* host wall time of the call                         */
    uint64_t chains;        /* pixel x band x sample paths traced                 */
    uint64_t events[SKY_EVENT_COUNT];  /* counted only with SKY_FLAG_COUNT_EVENTS, else 0 */
    uint32_t watchdog;      /* nonzero when a path reached the watchdog           */
    uint32_t kernel_used;   /* SkyKernel actually launched                         */
} SkyRenderStats;

/*
 * Device-resident outputs of sky_cuda_render_device().  All pointers are
 * device pointers; every one except `cell_sum` may be NULL.
 *   cell_sum   [pixels][bands]  sum of path radiance over the samples (FP64)
 *   cell_sumsq [pixels][bands]  sum of squared path radiance (FP64)
 *   film       [pixels][bands]  mean radiance, clamped >= 0 (the reference Film)
 *   xyz        [pixels][3]      CIE XYZ of the mean spectrum (FP64)
 *   xyz_var    [pixels][3]      variance of that XYZ estimate (FP64)
 *   counters   [SKY_EVENT_COUNT] event counts, added to (not overwritten)
 *   status     [1]              nonzero after a watchdog; left for the caller
 *   rgb        [pixels][3]      linear sRGB of that XYZ after the Bradford
 *                               solar-white-to-D65 white balance, non-finite
 *                               values as 0 (SpectralRgbConverter::new_solar_d65
 *                               and to_linear_srgb, spectrum.rs:132-165)
 * xyz, xyz_var and rgb need the scene's band_xyz_weights.
 */
typedef struct SkyDeviceOutputs {
    double* cell_sum;
    double* cell_sumsq;
    float* film;
    double* xyz;
    double* xyz_var;
    unsigned long long* counters;
    uint32_t* status;
    float* rgb;
} SkyDeviceOutputs;

/*
 * Launch shape of the wavefront tracer, per scene.  No counterpart in the
 * reference, whose dispatch shape is fixed (workgroup 8x8x1, one dispatch per
 * 2 samples, integrator.rs:254-283).  The Python package's autotuner times
 * candidates of these on the caller's workload and keeps the fastest.
 */
typedef struct SkyTuning {
    uint32_t variant;            /* resident blocks of 256 threads per SM the kernel is compiled
                                    for: 0 = 3 (80 registers), 1 = 2 (128), 2 = 4 (64)         */
    uint32_t max_blocks_per_sm;  /* 0 = occupancy limit                                          */
    uint32_t all_species;        /* 1 = the kernels evaluate all four aerosol species; 0 = only
                                    species 0 when species 1-3 carry no aerosol anywhere in the
                                    scene (the default: same results, fewer instructions)      */
    uint32_t _unused;            /* zero                                                         */
    float crossing_cost;         /* merged tracking grid: cost of a layer crossing relative to a
                                    null collision; <= 0 leaves the grid as it is              */
    uint32_t iteration_limit;    /* backstop of the wavefront kernel: loop iterations (one ray
                                    per lane each) a warp may run before it stops and reports
                                    SKY_ERR_WATCHDOG; 0 = 2^31.  A render needs about
                                    3 x chains / (32 x resident warps) iterations per warp.    */
    uint32_t _reserved[2];
} SkyTuning;

/* ---- Entry points ------------------------------------------------------ */

/* Library version string, e.g. "sky_cuda 0.1.0 (abi 1, sm_103a)". */
const char* sky_cuda_version(void);

/* Copy the last error message of the calling thread into `buf` (always NUL
 * terminated); returns the status that produced it. */
int sky_cuda_last_error(char* buf, size_t buf_len);

/*
 * Device allocations (cudaMalloc) the library has made in this process, on
 * every device.  Diagnostic; no counterpart in the reference.  Every device
 * allocation of the library goes through one routine, which counts it; when
 * the environment variable SKY_CUDA_FAIL_DEVICE_ALLOC is set to a nonzero
 * value that routine fails instead, as if the device were out of memory
 * (the call returns SKY_ERR_OUT_OF_MEMORY), so that a host can test its
 * handling of the reference's allocation failures without exhausting a GPU.
 */
uint64_t sky_cuda_device_allocations(void);

/*
 * Diagnostic: the tracer's own FP32 ray-shell geometry for caller rays.  The
 * reference intersects a ray with a sphere in f32 as b^2 - c with
 * c = (|o| - R)(|o| + R) (sky_trace.wgsl:211-221); the tracer evaluates the
 * same roots as t = -b -+ sqrt((R - p)(R + p)) from the impact parameter
 * p = |o x d|, and the altitude at t as sqrt(t (t + 2b) + |o|^2) - ground.
 * For ray i (origins / directions: device float [ray_count][3], unit
 * directions) and shell j (radii: device float [radius_count], km):
 *   t_out  [(i * radius_count + j) * 2 + {0, 1}]  near and far crossing
 *   alt_out[(i * radius_count + j) * 2 + {0, 1}]  altitude the tracker
 *                                                 computes at that crossing
 * NaN where the ray misses the shell.  Asynchronous on `cuda_stream`.
 */
int sky_cuda_probe_shell_geometry(const float* origins, const float* directions, uint32_t ray_count,
                                  const float* radii, uint32_t radius_count, float ground_radius_km, float* t_out,
                                  float* alt_out, void* cuda_stream);

/* Validate a scene (integrator.rs:130-163, :401-407) and upload its tables to
 * the current CUDA device.  Replaces the buffer creation of
 * integrator.rs:192-216. */
int sky_cuda_scene_create(const SkySceneDesc* desc, SkyScene** out_scene);

void sky_cuda_scene_destroy(SkyScene* scene);

/* Set / read the scene's launch shape (SkyTuning).  Setting a positive
 * crossing_cost rebuilds the merged tracking grid (SKY_TRACKING_MERGED_LAYERS)
 * from the scene's majorant grid.  No counterpart in the reference. */
int sky_cuda_scene_set_tuning(SkyScene* scene, const SkyTuning* tuning);
int sky_cuda_scene_get_tuning(const SkyScene* scene, SkyTuning* tuning);

/*
 * Render the spectral film into host memory: `film_out` receives
 * width*height*band_count floats, pixel-major and band-minor, divided by the
 * sample count and clamped at zero, exactly like the `Film` returned by
 * `render` (integrator.rs:125-128, :306-316).  Synchronous.
 */
int sky_cuda_render(const SkyScene* scene, const SkyRenderConfig* config,
                    float* film_out, size_t film_len, SkyRenderStats* stats);

/*
 * Like sky_cuda_render, and also returns per-pixel CIE XYZ (FP64, [pixels][3])
 * and its variance.  `film_out` may be NULL.  Requires band_xyz_weights in
 * the scene.
 */
int sky_cuda_render_xyz(const SkyScene* scene, const SkyRenderConfig* config,
                        float* film_out, size_t film_len,
                        double* xyz_out, double* xyz_var_out, size_t pixel_count,
                        SkyRenderStats* stats);

/*
 * One-shot form of `render(&SceneData, &RenderConfig)`: uploads the scene,
 * renders, copies the film back and frees the device tables, all inside the
 * call (integrator.rs:125-317).
 */
/*
 * Film and per-pixel linear sRGB (white-balanced as in SkyDeviceOutputs.rgb)
 * to host buffers: what sky-reference-render writes to its band EXRs and its
 * RGB EXR/PNG (film_output.rs:12-124).  film_out may be NULL.
 */
int sky_cuda_render_rgb(const SkyScene* scene, const SkyRenderConfig* config,
                        float* film_out, size_t film_len,
                        float* rgb_out, size_t pixel_count, SkyRenderStats* stats);

int sky_cuda_render_desc(const SkySceneDesc* desc, const SkyRenderConfig* config,
                         float* film_out, size_t film_len, SkyRenderStats* stats);

/*
 * Asynchronous render into device buffers on `cuda_stream` (a cudaStream_t,
 * NULL for the legacy default stream).  Returns after the launches are
 * queued; the watchdog word is left in `outputs->status`.
 */
int sky_cuda_render_device(const SkyScene* scene, const SkyRenderConfig* config,
                           const SkyDeviceOutputs* outputs, void* cuda_stream);

/* ---- Batched sweeps ------------------------------------------------------ */

/*
 * One render of a batch: a config, the sun direction for this render (the
 * scene's medium, bands and phase tables are shared by the whole batch; an
 * elevation sweep only moves the sun) and its device outputs.  No
 * counterpart in the reference, which renders one image per process
 * (scripts/bake_skyview_elevations.ps1 loops the CLI over elevations).
 */
typedef struct SkyBatchJob {
    SkyRenderConfig config;
    float sun_direction[3];     /* unit vector; all zero = the scene's sun */
    float _reserved;
    SkyDeviceOutputs outputs;   /* as for sky_cuda_render_device; outputs.status is
                                   used from the first job only */
} SkyBatchJob;

/*
 * Render every job of the batch in ONE wavefront launch on `cuda_stream`
 * (asynchronous; three kernels: prepare, trace, finalize).  All jobs must
 * share tracking and phase sampling; at most 65535 jobs.  The batch's
 * watchdog bits go to jobs[0].outputs.status, its event counts to
 * jobs[0].outputs.counters.
 */
int sky_cuda_render_batch(const SkyScene* scene, const SkyBatchJob* jobs, uint32_t job_count, void* cuda_stream);

/*
 * A batch captured once into a CUDA graph (job-table upload and the wavefront
 * launch) and replayed with one graph launch per sweep.  The outputs named in
 * `jobs` and the scene must stay valid while the graph is launched; destroy
 * the graph before the scene.
 */
typedef struct SkyBatchGraph SkyBatchGraph;
int sky_cuda_batch_graph_create(const SkyScene* scene, const SkyBatchJob* jobs, uint32_t job_count,
                                SkyBatchGraph** out_graph);
int sky_cuda_batch_graph_launch(SkyBatchGraph* graph, void* cuda_stream);
void sky_cuda_batch_graph_destroy(SkyBatchGraph* graph);

/* ---- Differentiable rendering ------------------------------------------ */

/*
 * No counterpart in the reference, which renders a fixed medium.  A
 * differentiable render evaluates the scene's medium with parameters applied
 * and returns dLoss/dparameters by path-replay backpropagation (each chain is
 * traced, then replayed from the same counter-based random numbers; no path
 * is stored).  The scene must hold one aerosol species (species 0, "Mie");
 * species 1-3 must carry no mass or no optics.
 *
 * layer_params, float [3 * majorant_layers + 2], device memory:
 *   [3 l + 0]  Rayleigh density scale of majorant layer l
 *   [3 l + 1]  Mie density scale of layer l (scales species 0's extinction)
 *   [3 l + 2]  ozone density scale of layer l
 *   [3 L]      Mie single-scattering albedo (replaces species 0's)
 *   [3 L + 1]  Mie Henyey-Greenstein asymmetry g, tabulated on the scene's
 *              phase grid (held inside [-0.99, 0.99])
 * band_params, float [band_count][4], device memory, or NULL for all ones:
 *   multipliers of the band's Rayleigh cross section, Mie extinction, ozone
 *   cross section and solar radiance (how a band-position change enters).
 * Each call bakes the majorant grid of the parameterised medium on the device
 * (medium.rs:63-102 probe rule) and, for SKY_TRACKING_MERGED_LAYERS, merges
 * its layers as the scene's tracking grid does; SKY_TRACKING_RESIDUAL_CARRY
 * tracks the uniform layers.  Segment-restart tracking is not offered.
 *
 * sample_layer_params / sample_band_params, when non-NULL, select a second
 * parameter set whose medium drives every sampling decision while
 * layer_params is evaluated (each path reweighted by the ratio of the two
 * path densities): renders at nearby parameters then share their samples,
 * which finite differences of the estimator need.  The evaluated medium's
 * extinction must stay below the sampling medium's majorants.
 */
#define SKY_ADJOINT_BAND_PARAMS 4u

/*
 * How the backward pass estimates the derivative of each traversed segment's
 * transmittance, -integral of d(sigma_t)/d(theta) along it:
 *   SEGMENT_INTEGRALS  stratified points placed along the segment in
 *                      majorant optical depth, from a random stream of their
 *                      own (the default; far lower variance);
 *   NULL_COLLISIONS    the null collisions the tracker drew: the exact
 *                      derivative of the forward estimator with its samples
 *                      held fixed, which central differences with
 *                      sample_layer_params reproduce to rounding.
 * Both are unbiased.
 */
typedef enum SkyAdjointEstimator {
    SKY_ADJOINT_SEGMENT_INTEGRALS = 0,
    SKY_ADJOINT_NULL_COLLISIONS = 1
} SkyAdjointEstimator;

/*
 * chain_radiance (optional, device float [slab pixels][band_count][spp],
 * the slab's cells in film order, each cell's samples in order;
 * chain_radiance_len its length in floats, at least that count): a forward
 * call writes every chain's radiance into it (before the band's solar
 * multiplier); a backward call at the same config, parameters and sun reads
 * it instead of tracing each chain a first time for its radiance, and skips
 * the chains whose radiance is zero (they carry no gradient).  Path replay
 * still stores no path: one float per chain.  Not with sample_* parameters;
 * a backward given a buffer that another config or parameter set wrote
 * returns a wrong gradient.
 */
typedef struct SkyAdjointParams {
    const float* layer_params;
    const float* band_params;
    const float* sample_layer_params;
    const float* sample_band_params;
    float sun_direction[3];  /* unit vector; all zero = the scene's sun */
    uint32_t estimator;      /* SkyAdjointEstimator (backward only) */
    float* chain_radiance;   /* optional: see above */
    uint64_t chain_radiance_len;
} SkyAdjointParams;

/*
 * Gradient request.  dloss_dfilm [pixels][band_count] is dLoss/d(film value)
 * of the mean film the forward call wrote; the gradients are ADDED to
 * layer_grad [3 * majorant_layers + 2] and band_grad [band_count][4] (either
 * may be NULL to skip it, not both).  status (required) and counters
 * (optional) as in SkyDeviceOutputs.
 */
typedef struct SkyAdjointGrads {
    const float* dloss_dfilm;
    double* layer_grad;
    double* band_grad;
    unsigned long long* counters;
    uint32_t* status;
} SkyAdjointGrads;

/* Number of layer parameters of the scene (3 * majorant_layers + 2). */
uint32_t sky_cuda_adjoint_param_count(const SkyScene* scene);

/*
 * Forward render over the parameterised medium into device outputs (as
 * sky_cuda_render_device: cell_sum and status required), asynchronous on
 * `cuda_stream`.  config->kernel is ignored; the whole call (table bake and
 * render) is ordered on the stream.
 */
int sky_cuda_adjoint_forward(const SkyScene* scene, const SkyRenderConfig* config, const SkyAdjointParams* params,
                             const SkyDeviceOutputs* outputs, void* cuda_stream);

/*
 * Backward: the gradient at `params` (sample_* must be NULL) of a loss whose
 * derivative with respect to the film of the forward render with the same
 * config is grads->dloss_dfilm.  Asynchronous on `cuda_stream`.
 */
int sky_cuda_adjoint_backward(const SkyScene* scene, const SkyRenderConfig* config, const SkyAdjointParams* params,
                              const SkyAdjointGrads* grads, void* cuda_stream);

/*
 * One render of a differentiable batch: its config and sun (all zero = the
 * params' sun, else the scene's), its outputs (forward: cell_sum required;
 * outputs.status and outputs.counters of job 0 serve the whole batch), its
 * dLoss/dfilm (backward) and its optional chain-radiance buffer (as
 * SkyAdjointParams.chain_radiance, per render).
 */
typedef struct SkyAdjointJob {
    SkyRenderConfig config;
    float sun_direction[3];
    float _reserved;
    SkyDeviceOutputs outputs;
    const float* dloss_dfilm;
    float* chain_radiance;
    uint64_t chain_radiance_len;
} SkyAdjointJob;

/*
 * Batched forward / backward: `job_count` renders over one parameter set
 * (params.layer_params / band_params / estimator; sample_* must be NULL and
 * params.chain_radiance is not read) in one launch of the differentiable
 * renderer per 32 renders, instead of one launch each: an elevation sweep of
 * a fit renders all its suns in one launch per direction.  Every render needs
 * the same tracking mode, phase sampling and accumulate flag.  Every render
 * is checked before the first launch: a refused batch launches nothing.  The
 * backward ADDS the gradient of sum_i Loss_i to grads->layer_grad / band_grad
 * (grads->dloss_dfilm is not read: each job carries its own).  Asynchronous on
 * `cuda_stream`.  No counterpart in the reference.
 */
int sky_cuda_adjoint_forward_batch(const SkyScene* scene, const SkyAdjointJob* jobs, uint32_t job_count,
                                   const SkyAdjointParams* params, void* cuda_stream);
int sky_cuda_adjoint_backward_batch(const SkyScene* scene, const SkyAdjointJob* jobs, uint32_t job_count,
                                    const SkyAdjointParams* params, const SkyAdjointGrads* grads, void* cuda_stream);

/*
 * Device majorant bake (compute_majorant_grid, medium.rs:63-102) of the
 * parameterised medium: writes majorants [band_count][majorant_layers] to
 * device memory.  With all scales 1 it reproduces the scene's own grid.
 */
int sky_cuda_bake_majorants(const SkyScene* scene, const SkyAdjointParams* params, float* majorants_out,
                            void* cuda_stream);

/* ---- Optimizer scoring --------------------------------------------------- */

/*
 * The wavelength optimizer's score of primary-band combinations
 * (sky-wavelength-optimizer/src/main.rs:414-488, 1121-1156), on the GPU.
 * Combination c rebuilds each sample's XYZ as
 *     xyz[s] = sum_ch bands[combo_bands[c][ch]][s] * combo_xyz[c][ch]
 * (combo_xyz = the channel's quadrature weight / band width * CIE at its
 * centre), maps it and the reference to Oklab after dividing by
 * reference_scale, and summarises the per-sample distances: mean, rmse, the
 * order statistics p50/p90/p95/p99 (element round((n - 1) q) of the sorted
 * finite distances, exact) and the maximum; score = rmse + 0.25 p95.
 *   bands      device, float [band_count][samples]
 *   ref_oklab  device, float [samples][3]: Oklab of reference XYZ / scale
 *   combo_bands, combo_xyz   host, [combo_count][channels] and [..][3]
 *   results    host, [combo_count]
 * Synchronous on `cuda_stream`; device scratch is allocated per call.
 */
typedef struct SkyComboScore {
    double mean, rmse, p50, p90, p95, p99, max, score;
    uint64_t finite;  /* samples with a finite distance */
} SkyComboScore;
int sky_cuda_score_combos(const float* bands, uint32_t band_count, uint64_t samples, const float* ref_oklab,
                          float reference_scale, const uint32_t* combo_bands, const float* combo_xyz,
                          uint32_t combo_count, uint32_t channels, SkyComboScore* results, void* cuda_stream);

/* ---- Mie phase-table bake ---------------------------------------------- */

/* Lognormal size distribution of one aerosol species: r_count radii spaced
 * geometrically on [r_min_um, r_max_um], weights exp(-ln^2(r/r_mode) /
 * (2 ln^2 sigma_g)) normalised to 1 (scripts/bake_opac_data.py:20-53, :103-109). */
typedef struct SkyMieDistribution {
    double r_mode_um;
    double sigma_g;      /* geometric standard deviation, > 1 */
    double r_min_um;
    double r_max_um;
    uint32_t r_count;
    uint32_t _reserved;
} SkyMieDistribution;

/* Size-averaged optics of one band (weights summing to 1; um^2). */
typedef struct SkyMieBand {
    double sigma_sca_um2;  /* sum_r w_r pi r^2 Q_sca(r)                         */
    double sigma_ext_um2;  /* sum_r w_r pi r^2 Q_ext(r)                         */
    double g;              /* asymmetry parameter of the averaged phase function */
} SkyMieBand;

/*
 * Bake the size-averaged Mie phase function of one species, per band, on the
 * cube-root mu grid mu_j = 1 - 2 ((j + 0.5) / phase_bins)^3:
 * phase_out[band * phase_bins + j], normalised to 1 over the sphere, i.e.
 * size_dist_phase of scripts/bake_opac_data.py:112-121 (its miepython sphere
 * restated from the published Mie series).  The particle's refractive index
 * per band is refr_re + i refr_im (refr_im >= 0 absorbs); wavelengths in um.
 * band_out (may be null) receives the averaged cross sections and g.
 * Synchronous, on the current device; no scene needed.
 */
int sky_cuda_bake_mie_phase(const SkyMieDistribution* dist, const double* wavelength_um, const double* refr_re,
                            const double* refr_im, uint32_t band_count, uint32_t phase_bins, double* phase_out,
                            SkyMieBand* band_out);

/*
 * Allocation-free render of up to SKY_NOALLOC_MAX_JOBS jobs of one scene in a
 * single launch of the wavefront tracer.  No counterpart in the reference.
 *
 * For callers that must not allocate device memory while rendering: engines
 * that reserve all device memory up front through their own allocator, or
 * that forbid allocations on their render path.  Such a caller creates the
 * scene once at start-up, owns every output buffer, and renders through this
 * call, which calls no cudaMalloc, cudaFree or allocating library routine.
 *
 * job_configs[i] / outputs[i] describe job i as in sky_cuda_render_device(),
 * except that this call always runs the wavefront kernel: a job whose
 * `kernel` is SKY_KERNEL_PLAIN is rejected with SKY_ERR_INVALID_CONFIG.
 * Every job must use the same tracking mode and phase sampling.
 * outputs[0].status is required and receives the watchdog bits of the whole
 * batch (OR-ed in; the caller clears it); outputs[0].counters receives the
 * batch's event counts.  More than SKY_NOALLOC_MAX_JOBS jobs are rejected
 * with SKY_ERR_INVALID_CONFIG.
 *
 * The kernel's job table and work counter live in one fixed scratch area of
 * the library (SKY_NOALLOC_SCRATCH_BYTES of device memory on every GPU that
 * loads it, held until the process exits).  The job table reaches that area
 * through the argument of a small kernel launched on `cuda_stream`, not
 * through a host-to-device copy, so the call neither waits for earlier work
 * on the stream nor reads host memory once it has returned.  Each call looks
 * up the area's address in the current CUDA context; the first call in a
 * process may make the CUDA runtime load the library's device code (lazy
 * module loading), so make it before any stream capture.  All calls share
 * the area and it keeps the last call's contents: calls that overlap on the
 * GPU (different streams without ordering, or different host threads) race
 * on it, so order them.
 */
#define SKY_NOALLOC_MAX_JOBS 16u
#define SKY_NOALLOC_SCRATCH_BYTES 16384u
int sky_cuda_render_batch_noalloc(const SkyScene* scene, const SkyRenderConfig* job_configs,
                                  const SkyDeviceOutputs* outputs, uint32_t job_count, void* cuda_stream);

#ifdef __cplusplus
}
#endif

#endif /* SKY_CUDA_H */
