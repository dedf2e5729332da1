// sky_cuda_api.cu — the C ABI declared in include/sky_cuda.h.
//
// Mirrors the reference integrator's host flow (integrator.rs:125-317):
// validate, pack tables into device memory, dispatch the tracer, read back,
// divide by the sample count and clamp at zero, and map failures to the
// RenderError kinds.  Device tables live in one allocation per scene; the
// per-render workspace is kept on the scene and grown on demand.

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstddef>
#include <atomic>
#include <cstdlib>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/sky_cuda.h"
#include "adjoint_kernels.h"
#include "mie_kernels.h"
#include "scene_build.h"
#include "score_kernels.h"
#include "trace_kernels.h"

using namespace sky;

struct SkyScene {
    int device = 0;
    DevScene dev{};
    void* blob = nullptr;
    bool has_xyz = false;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_start = nullptr, ev_stop = nullptr;
    // workspace
    double* ws_sum = nullptr;
    double* ws_sumsq = nullptr;
    float* ws_film = nullptr;
    double* ws_xyz = nullptr;
    double* ws_xyz_var = nullptr;
    float* ws_rgb = nullptr;
    unsigned long long* ws_counters = nullptr;
    uint32_t* ws_status = nullptr;
    uint64_t ws_cells = 0, ws_pixels = 0;
    // wavefront-kernel job table and work counter (one job per render call)
    DevJob* jobs = nullptr;
    uint32_t* work_counter = nullptr;
    // batch job tables: device table + pinned host staging, grown on demand
    DevJob* batch_jobs = nullptr;
    DevJob* batch_host = nullptr;
    uint32_t* batch_counter = nullptr;
    uint32_t batch_capacity = 0;
    SkyTuning tuning{};
    // merged tracking grid in its own allocation (rebuilt by set_tuning)
    void* trk_blob = nullptr;
    std::vector<float> host_majorants;
    float host_ground_radius = 0.0f, host_top = 0.0f;
    uint32_t host_layers = 0;
    // differentiable rendering: tables rebuilt per call, allocated on first use
    void* adj_ws = nullptr;
    std::string adjoint_unsupported;  // empty when the scene's medium can be parameterised
};

namespace {

thread_local std::string g_error;
thread_local int g_error_status = SKY_OK;

int set_error(int status, const std::string& msg) {
    g_error = msg;
    g_error_status = status;
    return status;
}

int cuda_fail(int status, const char* what, cudaError_t e) {
    std::string msg = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) status = SKY_ERR_OUT_OF_MEMORY;
    return set_error(status, msg);
}

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Every device allocation of the library: counted (sky_cuda_device_allocations)
// and, while SKY_CUDA_FAIL_DEVICE_ALLOC is set to a nonzero value, failed as
// out of memory without touching the device.
std::atomic<uint64_t> g_device_allocations{0};

bool allocation_failure_injected() {
    const char* v = std::getenv("SKY_CUDA_FAIL_DEVICE_ALLOC");
    return v && *v && std::strcmp(v, "0") != 0;
}

template <class T>
cudaError_t dev_malloc(T** ptr, size_t bytes) {
    if (allocation_failure_injected()) {
        *ptr = nullptr;
        return cudaErrorMemoryAllocation;
    }
    void* p = nullptr;
    const cudaError_t e = cudaMalloc(&p, bytes);
    if (e == cudaSuccess) g_device_allocations.fetch_add(1, std::memory_order_relaxed);
    *ptr = static_cast<T*>(p);
    return e;
}

// Pixels of the rows a config renders (its slab, or the whole image).
uint32_t slab_rows(const SkyRenderConfig* c) { return c->row_count ? c->row_count : c->height; }
uint64_t slab_pixels(const SkyRenderConfig* c) { return uint64_t(c->width) * slab_rows(c); }

void free_workspace(SkyScene* s) {
    cudaFree(s->ws_sum);
    cudaFree(s->ws_sumsq);
    cudaFree(s->ws_film);
    cudaFree(s->ws_xyz);
    cudaFree(s->ws_xyz_var);
    cudaFree(s->ws_rgb);
    s->ws_rgb = nullptr;
    cudaFree(s->ws_counters);
    cudaFree(s->ws_status);
    s->ws_sum = s->ws_sumsq = nullptr;
    s->ws_film = nullptr;
    s->ws_xyz = s->ws_xyz_var = nullptr;
    s->ws_counters = nullptr;
    s->ws_status = nullptr;
    s->ws_cells = s->ws_pixels = 0;
}

// Grow the render workspace to `pixels`.  The new buffers are allocated
// before the old ones are freed, so a failed allocation leaves the scene with
// its old workspace: renders that fit it still run without allocating.
int ensure_workspace(SkyScene* s, uint64_t pixels) {
    uint64_t cells = pixels * s->dev.band_count;
    if (cells <= s->ws_cells && pixels <= s->ws_pixels && s->ws_sum) return SKY_OK;
    SkyScene grown;
    grown.dev = s->dev;
    cudaError_t e = cudaSuccess;
    if ((e = dev_malloc(&grown.ws_sum, cells * sizeof(double))) != cudaSuccess ||
        (e = dev_malloc(&grown.ws_sumsq, cells * sizeof(double))) != cudaSuccess ||
        (e = dev_malloc(&grown.ws_film, cells * sizeof(float))) != cudaSuccess ||
        (e = dev_malloc(&grown.ws_xyz, pixels * 3 * sizeof(double))) != cudaSuccess ||
        (e = dev_malloc(&grown.ws_xyz_var, pixels * 3 * sizeof(double))) != cudaSuccess ||
        (e = dev_malloc(&grown.ws_rgb, pixels * 3 * sizeof(float))) != cudaSuccess ||
        (e = dev_malloc(&grown.ws_counters, SKY_EVENT_COUNT * sizeof(unsigned long long))) != cudaSuccess ||
        (e = dev_malloc(&grown.ws_status, sizeof(uint32_t))) != cudaSuccess) {
        free_workspace(&grown);
        return cuda_fail(SKY_ERR_OUT_OF_MEMORY, "workspace allocation", e);
    }
    // the old buffers may still be read by work queued on the scene's stream
    if (s->stream) cudaStreamSynchronize(s->stream);
    free_workspace(s);
    s->ws_sum = grown.ws_sum;
    s->ws_sumsq = grown.ws_sumsq;
    s->ws_film = grown.ws_film;
    s->ws_xyz = grown.ws_xyz;
    s->ws_xyz_var = grown.ws_xyz_var;
    s->ws_rgb = grown.ws_rgb;
    s->ws_counters = grown.ws_counters;
    s->ws_status = grown.ws_status;
    s->ws_cells = cells;
    s->ws_pixels = pixels;
    return SKY_OK;
}

// validate_config (integrator.rs:130-163) with run-time band count.
int validate_config(const SkyScene* scene, const SkyRenderConfig* c) {
    if (!scene) return set_error(SKY_ERR_INVALID_CONFIG, "scene is null");
    if (!c) return set_error(SKY_ERR_INVALID_CONFIG, "render config is null");
    if (c->width == 0 || c->height == 0 || c->spp == 0)
        return set_error(SKY_ERR_INVALID_CONFIG, "width, height, and spp must be greater than zero");
    if (c->row_count == 0 && c->row_begin != 0)
        return set_error(SKY_ERR_INVALID_CONFIG, "row_begin needs a nonzero row_count");
    if (uint64_t(c->row_begin) + c->row_count > c->height)
        return set_error(SKY_ERR_INVALID_CONFIG, "rows [row_begin, row_begin + row_count) exceed the image height");
    // the reference's own limit is on the whole image (integrator.rs:143-147)
    uint64_t cells = uint64_t(c->width) * c->height * scene->dev.band_count;
    if (cells > 0xffffffffull)
        return set_error(SKY_ERR_INVALID_CONFIG, "film is too large for the GPU shader index type");
    if (uint64_t(c->sample_offset) + c->spp > 0xffffffffull)
        return set_error(SKY_ERR_INVALID_CONFIG, "sample indices overflow 32 bits");
    // the kernels hand out samples in steps of up to 32 with 32-bit counters
    if (c->spp > 0x7fffffffu) return set_error(SKY_ERR_INVALID_CONFIG, "spp must be below 2^31");
    // each NEE sample is a shadow ray per vertex: an unbounded count would keep a launch running for hours
    if (c->direct_light_samples > kMaxLightSamples)
        return set_error(SKY_ERR_INVALID_CONFIG, "direct_light_samples must be at most 1024");
    if (c->output_projection > SKY_PROJECTION_SKY_VIEW_LUT)
        return set_error(SKY_ERR_INVALID_CONFIG, "unknown output projection");
    if (c->phase_sampling > SKY_PHASE_TABULATED)
        return set_error(SKY_ERR_INVALID_CONFIG, "unknown phase sampling mode");
    if (c->tracking > SKY_TRACKING_MERGED_LAYERS)
        return set_error(SKY_ERR_INVALID_CONFIG, "unknown tracking mode");
    if (c->kernel > SKY_KERNEL_WAVEFRONT) return set_error(SKY_ERR_INVALID_CONFIG, "unknown kernel");
    if (!std::isfinite(c->observer_altitude_km))
        return set_error(SKY_ERR_INVALID_CONFIG, "observer altitude must be finite");
    if (c->observer_altitude_km >= scene->dev.atmosphere_radius - scene->dev.ground_radius)
        return set_error(SKY_ERR_INVALID_CONFIG, "observer must be inside the atmosphere");
    return SKY_OK;
}

// Per-launch constants, including the sky-view LUT frame of
// sky_trace.wgsl:632-681 evaluated once on the host.
DevLaunch make_launch(const SkyScene* s, const SkyRenderConfig* c) {
    DevLaunch L{};
    L.width = c->width;
    L.height = c->height;
    L.row_begin = c->row_begin;
    L.rows = slab_rows(c);
    L.spp = c->spp;
    L.sample_offset = c->sample_offset;
    L.band_count = s->dev.band_count;
    L.direct_light_samples = c->direct_light_samples ? c->direct_light_samples : 1u;
    L.projection = c->output_projection;
    L.phase_sampling = c->phase_sampling;
    L.rr_start_depth = c->rr_start_depth ? c->rr_start_depth : kDefaultRrDepth;
    L.max_orders = c->max_orders;
    L.watchdog_limit = c->watchdog_limit ? c->watchdog_limit : kDefaultWatchdog;
    L.tracking = c->tracking;
    L.seed_lo = uint32_t(c->seed);
    L.seed_hi = uint32_t(c->seed >> 32);
    L.observer_altitude = c->observer_altitude_km;
    L.inv_width = 1.0f / float(c->width);
    L.inv_height = 1.0f / float(c->height);
    const float rg = s->dev.ground_radius;
    const float oy = rg + std::max(c->observer_altitude_km, 0.0f);
    const float view_height = std::sqrt(0.0f * 0.0f + oy * oy + 0.0f * 0.0f);
    const float v_horizon = std::sqrt(std::max(view_height * view_height - rg * rg, 0.0f));
    const float cos_beta = std::min(std::max(v_horizon / std::max(view_height, 0.000001f), 0.0f), 1.0f);
    const float beta = std::acos(cos_beta);
    L.lut_beta = beta;
    L.lut_zenith_horizon_angle = 3.14159265358979323846f - beta;
    const float* sun = s->dev.sun;
    float sh[3] = {sun[0], sun[1] - sun[1], sun[2]};
    float sh_len = std::sqrt(sh[0] * sh[0] + sh[1] * sh[1] + sh[2] * sh[2]);
    float f[3] = {1.0f, 0.0f, 0.0f};
    if (sh_len > 0.00001f)
        for (int i = 0; i < 3; ++i) f[i] = sh[i] / std::max(sh_len, 0.00001f);
    // side = normalize(cross(up, forward))
    float side[3] = {f[2], 0.0f, -f[0]};
    float sl = std::sqrt(side[0] * side[0] + side[1] * side[1] + side[2] * side[2]);
    for (int i = 0; i < 3; ++i) {
        L.lut_forward[i] = f[i];
        L.lut_side[i] = side[i] / sl;
    }
    return L;
}

// Cells a wavefront launch may hold: the 32-bit work counter also counts the
// claims that find no cell left (one per warp), so stay well below 2^32.
constexpr uint64_t kMaxLaunchCells = 0xF0000000ull;

// Place a job in the launch's cell space after the cells already placed.
int place_job(DevJob& job, uint64_t pixels, uint32_t bands, uint64_t& cells_so_far, uint32_t& max_cells) {
    const uint64_t cells = pixels * bands;
    if (cells_so_far + cells > kMaxLaunchCells)
        return set_error(SKY_ERR_INVALID_CONFIG, "a launch holds at most 4026531840 (pixel, band) cells");
    job.cell_begin = uint32_t(cells_so_far);
    job.cell_count = uint32_t(cells);
    cells_so_far += cells;
    max_cells = std::max(max_cells, uint32_t(cells));
    return SKY_OK;
}

WaveLaunch wave_launch(const SkyScene* s, const DevJob& first, const DevJob* dev_jobs, uint32_t n, uint64_t cells,
                       uint32_t max_cells, uint32_t tracking, uint32_t phase_sampling, uint32_t* counter,
                       unsigned long long* counters, uint32_t* status) {
    WaveLaunch w{};
    w.scene = first.S;
    w.launch0 = first.L;
    w.jobs = dev_jobs;
    w.num_jobs = n;
    w.total_cells = uint32_t(cells);
    w.max_job_cells = max_cells;
    w.variant = s->tuning.variant;
    w.max_blocks_per_sm = s->tuning.max_blocks_per_sm;
    w.tracking = tracking;
    w.phase_sampling = phase_sampling;
    w.work_counter = counter;
    w.counters = counters;
    w.status = status;
    w.iteration_limit = s->tuning.iteration_limit;
    w.aerosol_species = aerosol_species(first.S, s->tuning.all_species != 0u);
    return w;
}

// The launch checks read cudaGetLastError(), which also returns an error that
// an unrelated runtime call of the calling thread left behind; clear it
// before launching so that only this call's own errors are reported.
void clear_stale_error() { (void)cudaGetLastError(); }

int launch_render(SkyScene* s, const SkyRenderConfig* c, const SkyDeviceOutputs* o, cudaStream_t stream,
                  bool timed) {
    clear_stale_error();
    DevLaunch L = make_launch(s, c);
    const uint64_t pixels = slab_pixels(c);
    cudaError_t e;
    const bool accumulate = (c->flags & SKY_FLAG_ACCUMULATE) != 0;
    const uint32_t total_spp = accumulate ? c->sample_offset + c->spp : c->spp;
    double* xyz = s->has_xyz ? o->xyz : nullptr;
    double* xyz_var = s->has_xyz ? o->xyz_var : nullptr;
    float* rgb = s->has_xyz ? o->rgb : nullptr;
    if (c->kernel == SKY_KERNEL_PLAIN) {
        if (timed) cudaEventRecord(s->ev_start, stream);
        e = launch_trace_plain(s->dev, L, o->cell_sum, o->cell_sumsq, o->counters, o->status, accumulate,
                               aerosol_species(s->dev, s->tuning.all_species != 0u), stream);
        if (e != cudaSuccess) return cuda_fail(SKY_ERR_LAUNCH, "tracing kernel launch", e);
        if (timed) cudaEventRecord(s->ev_stop, stream);
        e = launch_finalize(s->dev, pixels, total_spp, o->cell_sum, o->cell_sumsq, o->film, xyz, xyz_var, rgb,
                            stream);
        if (e != cudaSuccess) return cuda_fail(SKY_ERR_LAUNCH, "finalize kernel launch", e);
        return SKY_OK;
    }
    DevJob job{};
    job.S = s->dev;
    job.L = L;
    job.cell_sum = o->cell_sum;
    job.cell_sumsq = o->cell_sumsq;
    job.film = o->film;
    job.xyz = xyz;
    job.xyz_var = xyz_var;
    job.rgb = rgb;
    job.accumulate = accumulate ? 1u : 0u;
    job.total_spp = total_spp;
    uint64_t cells = 0;
    uint32_t max_cells = 0;
    int st = place_job(job, pixels, s->dev.band_count, cells, max_cells);
    if (st) return st;
    const WaveLaunch w = wave_launch(s, job, s->jobs, 1, cells, max_cells, c->tracking, c->phase_sampling,
                                     s->work_counter, o->counters, o->status);
    if ((e = cudaMemcpyAsync(s->jobs, &job, sizeof(job), cudaMemcpyHostToDevice, stream)) != cudaSuccess)
        return cuda_fail(SKY_ERR_COPY, "job upload", e);
    if (timed) cudaEventRecord(s->ev_start, stream);
    e = launch_trace_wave(w, stream);
    if (e != cudaSuccess) return cuda_fail(SKY_ERR_LAUNCH, "wavefront tracing launch", e);
    if (timed) cudaEventRecord(s->ev_stop, stream);
    return SKY_OK;
}

// Synchronous render into the scene workspace, with host copies.
int render_host(SkyScene* s, const SkyRenderConfig* c, float* film_out, size_t film_len, double* xyz_out,
                double* xyz_var_out, size_t pixel_count, SkyRenderStats* stats, float* rgb_out = nullptr) {
    auto t0 = std::chrono::steady_clock::now();
    int st = validate_config(s, c);
    if (st) return st;
    const uint64_t pixels = slab_pixels(c);
    const uint64_t cells = pixels * s->dev.band_count;
    if (film_out && film_len < cells)
        return set_error(SKY_ERR_INVALID_CONFIG, "film buffer is smaller than width*rows*bands");
    if ((xyz_out || xyz_var_out || rgb_out) && pixel_count < pixels)
        return set_error(SKY_ERR_INVALID_CONFIG, "xyz / rgb buffer is smaller than width*rows");
    if ((xyz_out || xyz_var_out || rgb_out) && !s->has_xyz)
        return set_error(SKY_ERR_INVALID_CONFIG, "scene has no band_xyz_weights");
    if (cudaSetDevice(s->device) != cudaSuccess) return set_error(SKY_ERR_NO_DEVICE, "cannot select the device");
    if ((st = ensure_workspace(s, pixels))) return st;
    cudaError_t e;
    e = cudaMemsetAsync(s->ws_counters, 0, SKY_EVENT_COUNT * sizeof(unsigned long long), s->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->ws_status, 0, sizeof(uint32_t), s->stream);
    if (e != cudaSuccess) return cuda_fail(SKY_ERR_LAUNCH, "clearing counters", e);
    // events are counted only when the caller asks for them (counting costs the wavefront kernel ~3 %)
    const bool count = stats && (c->flags & SKY_FLAG_COUNT_EVENTS) != 0;
    SkyDeviceOutputs o{s->ws_sum, s->ws_sumsq, film_out ? s->ws_film : nullptr, xyz_out ? s->ws_xyz : nullptr,
                       xyz_var_out ? s->ws_xyz_var : nullptr, count ? s->ws_counters : nullptr, s->ws_status,
                       rgb_out ? s->ws_rgb : nullptr};
    if ((st = launch_render(s, c, &o, s->stream, true))) return st;
    uint32_t status = 0;
    unsigned long long counters[SKY_EVENT_COUNT] = {};
    if (film_out &&
        (e = cudaMemcpyAsync(film_out, s->ws_film, cells * sizeof(float), cudaMemcpyDeviceToHost, s->stream)))
        return cuda_fail(SKY_ERR_COPY, "film readback", e);
    if (xyz_out &&
        (e = cudaMemcpyAsync(xyz_out, s->ws_xyz, pixels * 3 * sizeof(double), cudaMemcpyDeviceToHost, s->stream)))
        return cuda_fail(SKY_ERR_COPY, "xyz readback", e);
    if (xyz_var_out && (e = cudaMemcpyAsync(xyz_var_out, s->ws_xyz_var, pixels * 3 * sizeof(double),
                                            cudaMemcpyDeviceToHost, s->stream)))
        return cuda_fail(SKY_ERR_COPY, "xyz variance readback", e);
    if (rgb_out &&
        (e = cudaMemcpyAsync(rgb_out, s->ws_rgb, pixels * 3 * sizeof(float), cudaMemcpyDeviceToHost, s->stream)))
        return cuda_fail(SKY_ERR_COPY, "rgb readback", e);
    if ((e = cudaMemcpyAsync(counters, s->ws_counters, sizeof(counters), cudaMemcpyDeviceToHost, s->stream)) ||
        (e = cudaMemcpyAsync(&status, s->ws_status, sizeof(status), cudaMemcpyDeviceToHost, s->stream)))
        return cuda_fail(SKY_ERR_COPY, "diagnostics readback", e);
    if ((e = cudaStreamSynchronize(s->stream)) != cudaSuccess) return cuda_fail(SKY_ERR_SYNC, "waiting for the GPU", e);
    if (stats) {
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, s->ev_start, s->ev_stop);
        stats->kernel_ms = ms;
        stats->chains = uint64_t(cells) * c->spp;
        for (int i = 0; i < SKY_EVENT_COUNT; ++i) stats->events[i] = counters[i];
        stats->watchdog = status;
        stats->kernel_used = c->kernel == SKY_KERNEL_PLAIN ? SKY_KERNEL_PLAIN : SKY_KERNEL_WAVEFRONT;
        stats->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    if (status & 2u) return set_error(SKY_ERR_WATCHDOG, "the tracing kernel reached its iteration limit");
    if (status) return set_error(SKY_ERR_WATCHDOG, "GPU path watchdog was reached");
    return SKY_OK;
}

// Upload the merged tracking grid of `h` into its own device allocation.
int upload_tracking_grid(SkyScene* s, const HostTables& h) {
    size_t off = 0;
    auto reserve = [&off](size_t bytes) {
        size_t at = off;
        off = align_up(off + bytes, 256);
        return at;
    };
    const size_t o_tr = reserve(h.trk_radius.size() * sizeof(float));
    const size_t o_tm = reserve(h.trk_maj.size() * sizeof(float));
    const size_t o_tp = reserve(h.trk_map.size() * sizeof(uint16_t));
    const size_t o_tc = reserve(h.trk_count.size() * sizeof(uint32_t));
    const size_t o_to = reserve(h.trk_off.size() * sizeof(uint32_t));
    std::vector<unsigned char> host(off, 0);
    std::memcpy(host.data() + o_tr, h.trk_radius.data(), h.trk_radius.size() * sizeof(float));
    std::memcpy(host.data() + o_tm, h.trk_maj.data(), h.trk_maj.size() * sizeof(float));
    std::memcpy(host.data() + o_tp, h.trk_map.data(), h.trk_map.size() * sizeof(uint16_t));
    std::memcpy(host.data() + o_tc, h.trk_count.data(), h.trk_count.size() * sizeof(uint32_t));
    std::memcpy(host.data() + o_to, h.trk_off.data(), h.trk_off.size() * sizeof(uint32_t));
    void* blob = nullptr;
    cudaError_t e = dev_malloc(&blob, off);
    if (e != cudaSuccess) return cuda_fail(SKY_ERR_OUT_OF_MEMORY, "tracking grid allocation", e);
    if ((e = cudaMemcpy(blob, host.data(), off, cudaMemcpyHostToDevice)) != cudaSuccess) {
        cudaFree(blob);
        return cuda_fail(SKY_ERR_COPY, "tracking grid upload", e);
    }
    if (s->trk_blob) {
        if (s->stream) cudaStreamSynchronize(s->stream);
        cudaFree(s->trk_blob);
    }
    s->trk_blob = blob;
    unsigned char* base = static_cast<unsigned char*>(blob);
    s->dev.trk_radius = reinterpret_cast<const float*>(base + o_tr);
    s->dev.trk_maj = reinterpret_cast<const float*>(base + o_tm);
    s->dev.trk_map = reinterpret_cast<const uint16_t*>(base + o_tp);
    s->dev.trk_count = reinterpret_cast<const uint32_t*>(base + o_tc);
    s->dev.trk_off = reinterpret_cast<const uint32_t*>(base + o_to);
    s->dev.trk_total = uint32_t(h.trk_radius.size());
    return SKY_OK;
}

// Rebuild the merged grid for a new crossing cost from the stored majorants.
int rebuild_tracking_grid(SkyScene* s, double crossing_cost) {
    HostTables h;
    const uint32_t B = s->dev.band_count, L = s->host_layers;
    const float dzl = s->host_top / float(L);
    h.trk_map.assign(size_t(B) * L, 0);
    h.trk_count.assign(B, 0);
    h.trk_off.assign(B, 0);
    for (uint32_t b = 0; b < B; ++b) {
        const float* maj = s->host_majorants.data() + size_t(b) * L;
        std::vector<uint32_t> starts = merge_majorant_layers(maj, L, dzl, crossing_cost);
        const uint32_t M = uint32_t(starts.size());
        h.trk_count[b] = M;
        h.trk_off[b] = uint32_t(h.trk_radius.size());
        for (uint32_t m = 0; m < M; ++m) {
            const uint32_t k0 = starts[m], k1 = m + 1 < M ? starts[m + 1] : L;
            float mx = 0.0f;
            for (uint32_t k = k0; k < k1; ++k) {
                mx = std::max(mx, std::max(maj[k], 0.00000001f));
                h.trk_map[size_t(b) * L + k] = uint16_t(m);
            }
            h.trk_maj.push_back(mx);
            h.trk_radius.push_back(s->host_ground_radius + float(k0) * dzl);
        }
        h.trk_maj.push_back(0.0f);
        h.trk_radius.push_back(s->host_ground_radius + s->host_top);
    }
    return upload_tracking_grid(s, h);
}

}  // namespace

extern "C" {

int sky_cuda_scene_set_tuning(SkyScene* s, const SkyTuning* t) {
    if (!s || !t) return set_error(SKY_ERR_INVALID_CONFIG, "scene and tuning must not be null");
    if (t->variant >= kWaveVariants) return set_error(SKY_ERR_INVALID_CONFIG, "unknown wavefront kernel variant");
    if (t->max_blocks_per_sm > 64) return set_error(SKY_ERR_INVALID_CONFIG, "max_blocks_per_sm out of range");
    if (t->all_species > 1u) return set_error(SKY_ERR_INVALID_CONFIG, "all_species must be 0 or 1");
    if (!(t->crossing_cost <= 0.0f) && !(t->crossing_cost < 1e6f))
        return set_error(SKY_ERR_INVALID_CONFIG, "crossing_cost out of range");
    if (cudaSetDevice(s->device) != cudaSuccess) return set_error(SKY_ERR_NO_DEVICE, "cannot select the device");
    if (t->crossing_cost > 0.0f && t->crossing_cost != s->tuning.crossing_cost) {
        int st = rebuild_tracking_grid(s, double(t->crossing_cost));
        if (st) return st;
    }
    const float keep = s->tuning.crossing_cost;
    s->tuning = *t;
    if (!(t->crossing_cost > 0.0f)) s->tuning.crossing_cost = keep;
    return SKY_OK;
}

int sky_cuda_scene_get_tuning(const SkyScene* s, SkyTuning* t) {
    if (!s || !t) return set_error(SKY_ERR_INVALID_CONFIG, "scene and tuning must not be null");
    *t = s->tuning;
    return SKY_OK;
}


const char* sky_cuda_version(void) { return "sky_cuda 0.1.0 (abi 1, sm_103a)"; }

uint64_t sky_cuda_device_allocations(void) { return g_device_allocations.load(std::memory_order_relaxed); }

int sky_cuda_probe_shell_geometry(const float* origins, const float* directions, uint32_t ray_count,
                                  const float* radii, uint32_t radius_count, float ground_radius_km, float* t_out,
                                  float* alt_out, void* cuda_stream) {
    if (!origins || !directions || !radii || !t_out || !alt_out)
        return set_error(SKY_ERR_INVALID_CONFIG, "every buffer of the shell probe is required");
    if (ray_count == 0 || radius_count == 0 || uint64_t(ray_count) * radius_count > (uint64_t(1) << 36))
        return set_error(SKY_ERR_INVALID_CONFIG, "ray_count * radius_count must be in [1, 2^36]");
    if (!std::isfinite(ground_radius_km)) return set_error(SKY_ERR_INVALID_CONFIG, "ground radius must be finite");
    clear_stale_error();
    const cudaError_t e = launch_shell_probe(origins, directions, ray_count, radii, radius_count, ground_radius_km,
                                             t_out, alt_out, static_cast<cudaStream_t>(cuda_stream));
    if (e != cudaSuccess) return cuda_fail(SKY_ERR_LAUNCH, "shell probe launch", e);
    return SKY_OK;
}

int sky_cuda_last_error(char* buf, size_t buf_len) {
    if (buf && buf_len) {
        std::snprintf(buf, buf_len, "%s", g_error.c_str());
    }
    return g_error_status;
}

int sky_cuda_scene_create(const SkySceneDesc* desc, SkyScene** out_scene) {
    if (!out_scene) return set_error(SKY_ERR_INVALID_CONFIG, "out_scene is null");
    *out_scene = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0)
        return set_error(SKY_ERR_NO_DEVICE, std::string("no usable CUDA device: ") + cudaGetErrorString(e));
    HostTables h;
    std::string err;
    int st = build_host_tables(desc, h, err);
    if (st) return set_error(st, err);

    SkyScene* s = new SkyScene();
    cudaGetDevice(&s->device);
    const size_t A = 256;
    size_t off = 0;
    auto reserve = [&](size_t bytes) {
        size_t at = off;
        off = align_up(off + bytes, A);
        return at;
    };
    size_t o_knot = reserve(h.knot_z.size() * sizeof(float));
    size_t o_finder = reserve(h.finder.size() * sizeof(uint16_t));
    size_t o_sig = reserve(h.sigma_t.size() * sizeof(float2));
    size_t o_cell = reserve(h.sig_cell.size() * sizeof(float4));
    size_t o_maj = reserve(h.majorants.size() * sizeof(float));
    size_t o_band = reserve(h.bands.size() * sizeof(DevBand));
    size_t o_prof = reserve(h.profile.size() * sizeof(DevProfileKnot));
    size_t o_opt = reserve(h.optics.size() * sizeof(SkyAerosolOptics));
    size_t o_pv = reserve(h.phase_values.size() * sizeof(float));
    size_t o_pc = reserve(h.phase_cdf.size() * sizeof(float));
    size_t o_pp = reserve(h.phase_bin_pdf.size() * sizeof(float));
    size_t o_pg = reserve(h.phase_guide.size() * sizeof(uint16_t));

    std::vector<unsigned char> host(off, 0);
    auto put = [&](size_t at, const void* src, size_t bytes) { std::memcpy(host.data() + at, src, bytes); };
    put(o_knot, h.knot_z.data(), h.knot_z.size() * sizeof(float));
    put(o_finder, h.finder.data(), h.finder.size() * sizeof(uint16_t));
    put(o_sig, h.sigma_t.data(), h.sigma_t.size() * sizeof(float2));
    put(o_cell, h.sig_cell.data(), h.sig_cell.size() * sizeof(float4));
    put(o_maj, h.majorants.data(), h.majorants.size() * sizeof(float));
    put(o_band, h.bands.data(), h.bands.size() * sizeof(DevBand));
    put(o_prof, h.profile.data(), h.profile.size() * sizeof(DevProfileKnot));
    put(o_opt, h.optics.data(), h.optics.size() * sizeof(SkyAerosolOptics));
    put(o_pv, h.phase_values.data(), h.phase_values.size() * sizeof(float));
    put(o_pc, h.phase_cdf.data(), h.phase_cdf.size() * sizeof(float));
    put(o_pp, h.phase_bin_pdf.data(), h.phase_bin_pdf.size() * sizeof(float));
    put(o_pg, h.phase_guide.data(), h.phase_guide.size() * sizeof(uint16_t));

    if ((e = dev_malloc(&s->blob, off)) != cudaSuccess) {
        delete s;
        return cuda_fail(SKY_ERR_OUT_OF_MEMORY, "scene table allocation", e);
    }
    if ((e = cudaMemcpy(s->blob, host.data(), off, cudaMemcpyHostToDevice)) != cudaSuccess) {
        cudaFree(s->blob);
        delete s;
        return cuda_fail(SKY_ERR_COPY, "scene table upload", e);
    }
    unsigned char* base = static_cast<unsigned char*>(s->blob);
    s->dev = h.scene;
    s->dev.knot_z = reinterpret_cast<const float*>(base + o_knot);
    s->dev.finder = reinterpret_cast<const uint16_t*>(base + o_finder);
    s->dev.sigma_t = reinterpret_cast<const float2*>(base + o_sig);
    s->dev.sig_cell = reinterpret_cast<const float4*>(base + o_cell);
    s->dev.majorants = reinterpret_cast<const float*>(base + o_maj);
    s->dev.bands = reinterpret_cast<const DevBand*>(base + o_band);
    s->dev.profile = reinterpret_cast<const DevProfileKnot*>(base + o_prof);
    s->dev.optics = reinterpret_cast<const SkyAerosolOptics*>(base + o_opt);
    s->dev.phase_values = reinterpret_cast<const float*>(base + o_pv);
    s->dev.phase_cdf = reinterpret_cast<const float*>(base + o_pc);
    s->dev.phase_bin_pdf = reinterpret_cast<const float*>(base + o_pp);
    s->dev.phase_guide = reinterpret_cast<const uint16_t*>(base + o_pg);
    s->host_majorants = h.majorants;
    s->host_layers = desc->majorant_layers;
    s->host_ground_radius = desc->ground_radius_km;
    s->host_top = desc->top_altitude_km;
    s->tuning.crossing_cost = float(kDefaultCrossingCost);
    s->tuning.variant = 2;  // 4 blocks per SM: the fastest shape on the production render
    if ((st = upload_tracking_grid(s, h))) {
        sky_cuda_scene_destroy(s);
        return st;
    }
    s->has_xyz = h.has_xyz;
    // Differentiable renders parameterise aerosol species 0 only.
    for (uint32_t sp = 1; sp < kSpecies && s->adjoint_unsupported.empty(); ++sp) {
        bool mass = false, optics = false;
        for (uint32_t i = 0; i < desc->aerosol_len; ++i) mass = mass || desc->aerosol[i].mass_g_m3[sp] != 0.0f;
        for (uint32_t b = 0; b < desc->band_count; ++b) {
            const SkyAerosolOptics& o = desc->aerosol_optics[size_t(b) * kSpecies + sp];
            optics = optics || o.scattering_km_inv_per_g_m3 != 0.0f || o.absorption_km_inv_per_g_m3 != 0.0f;
        }
        if (mass && optics)
            s->adjoint_unsupported = "differentiable renders need a scene whose only aerosol is species 0; species " +
                                     std::to_string(sp) + " has mass and optics";
    }
    if ((e = dev_malloc(&s->jobs, sizeof(DevJob))) != cudaSuccess ||
        (e = dev_malloc(&s->work_counter, sizeof(uint32_t))) != cudaSuccess) {
        sky_cuda_scene_destroy(s);
        return cuda_fail(SKY_ERR_OUT_OF_MEMORY, "job table allocation", e);
    }
    if ((e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreate(&s->ev_start)) != cudaSuccess || (e = cudaEventCreate(&s->ev_stop)) != cudaSuccess) {
        sky_cuda_scene_destroy(s);
        return cuda_fail(SKY_ERR_DEVICE_INIT, "stream creation", e);
    }
    *out_scene = s;
    return SKY_OK;
}

void sky_cuda_scene_destroy(SkyScene* s) {
    if (!s) return;
    cudaSetDevice(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    free_workspace(s);
    cudaFree(s->batch_jobs);
    cudaFreeHost(s->batch_host);
    cudaFree(s->batch_counter);
    cudaFree(s->trk_blob);
    cudaFree(s->adj_ws);
    cudaFree(s->jobs);
    cudaFree(s->work_counter);
    cudaFree(s->blob);
    if (s->ev_start) cudaEventDestroy(s->ev_start);
    if (s->ev_stop) cudaEventDestroy(s->ev_stop);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

int sky_cuda_render(const SkyScene* scene, const SkyRenderConfig* config, float* film_out, size_t film_len,
                    SkyRenderStats* stats) {
    if (!film_out) return set_error(SKY_ERR_INVALID_CONFIG, "film_out is null");
    return render_host(const_cast<SkyScene*>(scene), config, film_out, film_len, nullptr, nullptr, 0, stats);
}

int sky_cuda_render_xyz(const SkyScene* scene, const SkyRenderConfig* config, float* film_out, size_t film_len,
                        double* xyz_out, double* xyz_var_out, size_t pixel_count, SkyRenderStats* stats) {
    if (!xyz_out) return set_error(SKY_ERR_INVALID_CONFIG, "xyz_out is null");
    return render_host(const_cast<SkyScene*>(scene), config, film_out, film_len, xyz_out, xyz_var_out, pixel_count,
                       stats);
}

int sky_cuda_render_rgb(const SkyScene* scene, const SkyRenderConfig* config, float* film_out, size_t film_len,
                        float* rgb_out, size_t pixel_count, SkyRenderStats* stats) {
    if (!rgb_out) return set_error(SKY_ERR_INVALID_CONFIG, "rgb_out is null");
    return render_host(const_cast<SkyScene*>(scene), config, film_out, film_len, nullptr, nullptr, pixel_count, stats,
                       rgb_out);
}

int sky_cuda_render_desc(const SkySceneDesc* desc, const SkyRenderConfig* config, float* film_out, size_t film_len,
                         SkyRenderStats* stats) {
    SkyScene* s = nullptr;
    int st = sky_cuda_scene_create(desc, &s);
    if (st) return st;
    st = sky_cuda_render(s, config, film_out, film_len, stats);
    std::string keep = g_error;
    int keep_status = g_error_status;
    sky_cuda_scene_destroy(s);
    g_error = keep;
    g_error_status = keep_status;
    return st;
}

int sky_cuda_render_device(const SkyScene* scene, const SkyRenderConfig* config, const SkyDeviceOutputs* outputs,
                           void* cuda_stream) {
    int st = validate_config(scene, config);
    if (st) return st;
    if (!outputs || !outputs->cell_sum) return set_error(SKY_ERR_INVALID_CONFIG, "outputs.cell_sum is required");
    if (!outputs->status) return set_error(SKY_ERR_INVALID_CONFIG, "outputs.status is required");
    SkyScene* s = const_cast<SkyScene*>(scene);
    return launch_render(s, config, outputs, static_cast<cudaStream_t>(cuda_stream), false);
}

}  // extern "C"

// ---- batched sweeps ----------------------------------------------------------------

struct SkyBatchGraph {
    int device = 0;                // the scene's device, kept: the graph may outlive its scene handle
    DevJob* jobs = nullptr;        // device job table owned by the graph
    DevJob* host = nullptr;        // pinned copy the graph's memcpy node reads
    uint32_t* counter = nullptr;
    uint32_t job_count = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace {

// Fill DevJob rows for a batch; returns the batch's cells and its largest job.
int build_batch_jobs(SkyScene* s, const SkyBatchJob* jobs, uint32_t n, DevJob* out, uint64_t& cells,
                     uint32_t& max_cells) {
    if (!s || !jobs || n == 0) return set_error(SKY_ERR_INVALID_CONFIG, "scene and at least one job are required");
    if (!jobs[0].outputs.status) return set_error(SKY_ERR_INVALID_CONFIG, "jobs[0].outputs.status is required");
    if (n > 65535u) return set_error(SKY_ERR_INVALID_CONFIG, "a batch holds at most 65535 jobs");
    cells = 0;
    max_cells = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const SkyRenderConfig* c = &jobs[i].config;
        int st = validate_config(s, c);
        if (st) return st;
        if (c->tracking != jobs[0].config.tracking || c->phase_sampling != jobs[0].config.phase_sampling)
            return set_error(SKY_ERR_INVALID_CONFIG, "all jobs of a batch need the same tracking and phase sampling");
        if (!jobs[i].outputs.cell_sum) return set_error(SKY_ERR_INVALID_CONFIG, "every job needs outputs.cell_sum");
        DevJob& job = out[i];
        job = DevJob{};
        job.S = s->dev;
        const float* d = jobs[i].sun_direction;
        const float len = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        if (len > 0.0f) {
            if (!std::isfinite(len)) return set_error(SKY_ERR_INVALID_CONFIG, "sun direction must be finite");
            for (int k = 0; k < 3; ++k) job.S.sun[k] = d[k] / len;
            host_orthonormal_basis(job.S.sun, job.S.sun_t, job.S.sun_b);
        }
        job.L = make_launch(s, c);
        if (len > 0.0f) {  // the sky-view LUT frame follows the job's sun
            SkyScene tmp_view;
            tmp_view.dev = job.S;
            job.L = make_launch(&tmp_view, c);
            tmp_view.dev = DevScene{};
        }
        const bool accumulate = (c->flags & SKY_FLAG_ACCUMULATE) != 0;
        job.cell_sum = jobs[i].outputs.cell_sum;
        job.cell_sumsq = jobs[i].outputs.cell_sumsq;
        job.film = jobs[i].outputs.film;
        job.xyz = s->has_xyz ? jobs[i].outputs.xyz : nullptr;
        job.xyz_var = s->has_xyz ? jobs[i].outputs.xyz_var : nullptr;
        job.rgb = s->has_xyz ? jobs[i].outputs.rgb : nullptr;
        job.accumulate = accumulate ? 1u : 0u;
        job.total_spp = accumulate ? c->sample_offset + c->spp : c->spp;
        if ((st = place_job(job, slab_pixels(c), s->dev.band_count, cells, max_cells))) return st;
    }
    return SKY_OK;
}

int ensure_batch_capacity(SkyScene* s, uint32_t n) {
    if (n <= s->batch_capacity) return SKY_OK;
    if (s->stream) cudaStreamSynchronize(s->stream);
    cudaFree(s->batch_jobs);
    cudaFreeHost(s->batch_host);
    cudaFree(s->batch_counter);
    s->batch_jobs = nullptr;
    s->batch_host = nullptr;
    s->batch_counter = nullptr;
    s->batch_capacity = 0;
    cudaError_t e;
    if ((e = dev_malloc(&s->batch_jobs, size_t(n) * sizeof(DevJob))) != cudaSuccess ||
        (e = cudaMallocHost(&s->batch_host, size_t(n) * sizeof(DevJob))) != cudaSuccess ||
        (e = dev_malloc(&s->batch_counter, sizeof(uint32_t))) != cudaSuccess)
        return cuda_fail(SKY_ERR_OUT_OF_MEMORY, "batch job table allocation", e);
    s->batch_capacity = n;
    return SKY_OK;
}

}  // namespace

extern "C" int sky_cuda_render_batch(const SkyScene* scene, const SkyBatchJob* jobs, uint32_t job_count,
                                     void* cuda_stream) {
    SkyScene* s = const_cast<SkyScene*>(scene);
    if (!s) return set_error(SKY_ERR_INVALID_CONFIG, "scene is null");
    if (cudaSetDevice(s->device) != cudaSuccess) return set_error(SKY_ERR_NO_DEVICE, "cannot select the device");
    int st = ensure_batch_capacity(s, job_count);
    if (st) return st;
    cudaStream_t stream = static_cast<cudaStream_t>(cuda_stream);
    // the previous batch may still read the pinned staging table
    cudaStreamSynchronize(stream);
    uint64_t cells = 0;
    uint32_t max_cells = 0;
    if ((st = build_batch_jobs(s, jobs, job_count, s->batch_host, cells, max_cells))) return st;
    clear_stale_error();
    cudaError_t e = cudaMemcpyAsync(s->batch_jobs, s->batch_host, size_t(job_count) * sizeof(DevJob),
                                    cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) return cuda_fail(SKY_ERR_COPY, "batch job table upload", e);
    const WaveLaunch w = wave_launch(s, s->batch_host[0], s->batch_jobs, job_count, cells, max_cells,
                                     jobs[0].config.tracking, jobs[0].config.phase_sampling, s->batch_counter,
                                     jobs[0].outputs.counters, jobs[0].outputs.status);
    e = launch_trace_wave(w, stream);
    if (e != cudaSuccess) return cuda_fail(SKY_ERR_LAUNCH, "batched wavefront launch", e);
    return SKY_OK;
}

extern "C" int sky_cuda_batch_graph_create(const SkyScene* scene, const SkyBatchJob* jobs, uint32_t job_count,
                                           SkyBatchGraph** out_graph) {
    if (!out_graph) return set_error(SKY_ERR_INVALID_CONFIG, "out_graph is null");
    *out_graph = nullptr;
    SkyScene* s = const_cast<SkyScene*>(scene);
    if (!s) return set_error(SKY_ERR_INVALID_CONFIG, "scene is null");
    if (cudaSetDevice(s->device) != cudaSuccess) return set_error(SKY_ERR_NO_DEVICE, "cannot select the device");
    SkyBatchGraph* g = new SkyBatchGraph();
    g->device = s->device;
    g->job_count = job_count;
    uint64_t cells = 0;
    uint32_t max_cells = 0;
    cudaError_t e;
    int st = SKY_OK;
    cudaStream_t cap = nullptr;
    if ((e = cudaMallocHost(&g->host, size_t(std::max(job_count, 1u)) * sizeof(DevJob))) != cudaSuccess ||
        (e = dev_malloc(&g->jobs, size_t(std::max(job_count, 1u)) * sizeof(DevJob))) != cudaSuccess ||
        (e = dev_malloc(&g->counter, sizeof(uint32_t))) != cudaSuccess) {
        st = cuda_fail(SKY_ERR_OUT_OF_MEMORY, "batch graph allocation", e);
    } else if ((st = build_batch_jobs(s, jobs, job_count, g->host, cells, max_cells)) == SKY_OK) {
        const WaveLaunch w = wave_launch(s, g->host[0], g->jobs, job_count, cells, max_cells,
                                         jobs[0].config.tracking, jobs[0].config.phase_sampling, g->counter,
                                         jobs[0].outputs.counters, jobs[0].outputs.status);
        clear_stale_error();
        if ((e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking)) != cudaSuccess ||
            (e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) {
            st = cuda_fail(SKY_ERR_DEVICE_INIT, "graph capture", e);
        } else {
            cudaError_t e1 = cudaMemcpyAsync(g->jobs, g->host, size_t(job_count) * sizeof(DevJob),
                                             cudaMemcpyHostToDevice, cap);
            cudaError_t e2 = cudaSuccess;
            cudaError_t e3 = launch_trace_wave(w, cap);
            e = cudaStreamEndCapture(cap, &g->graph);
            if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess || e != cudaSuccess)
                st = cuda_fail(SKY_ERR_LAUNCH, "graph capture of the batch",
                               e3 != cudaSuccess ? e3 : (e1 != cudaSuccess ? e1 : (e2 != cudaSuccess ? e2 : e)));
            else if ((e = cudaGraphInstantiate(&g->exec, g->graph, 0)) != cudaSuccess)
                st = cuda_fail(SKY_ERR_LAUNCH, "graph instantiation", e);
        }
    }
    if (cap) cudaStreamDestroy(cap);
    if (st) {
        sky_cuda_batch_graph_destroy(g);
        return st;
    }
    *out_graph = g;
    return SKY_OK;
}

extern "C" int sky_cuda_batch_graph_launch(SkyBatchGraph* g, void* cuda_stream) {
    if (!g || !g->exec) return set_error(SKY_ERR_INVALID_CONFIG, "graph is null");
    if (cudaSetDevice(g->device) != cudaSuccess) return set_error(SKY_ERR_NO_DEVICE, "cannot select the device");
    clear_stale_error();
    cudaError_t e = cudaGraphLaunch(g->exec, static_cast<cudaStream_t>(cuda_stream));
    if (e != cudaSuccess) return cuda_fail(SKY_ERR_LAUNCH, "graph launch", e);
    return SKY_OK;
}

extern "C" void sky_cuda_batch_graph_destroy(SkyBatchGraph* g) {
    if (!g) return;
    cudaSetDevice(g->device);
    cudaDeviceSynchronize();
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    cudaFree(g->jobs);
    cudaFree(g->counter);
    cudaFreeHost(g->host);
    delete g;
}

// ---- differentiable rendering -----------------------------------------------------

namespace {

// Kernel context of a differentiable render: the scene (with the caller's
// sun), both parameter sets and the device workspace their tables go to.
int adjoint_setup(SkyScene* s, const SkyAdjointParams* p, AdjCtx& A, AdjWorkspace& W) {
    if (!s) return set_error(SKY_ERR_INVALID_CONFIG, "scene is null");
    if (!p || !p->layer_params) return set_error(SKY_ERR_INVALID_CONFIG, "params.layer_params is required");
    if (!s->adjoint_unsupported.empty()) return set_error(SKY_ERR_INVALID_CONFIG, s->adjoint_unsupported);
    if (cudaSetDevice(s->device) != cudaSuccess) return set_error(SKY_ERR_NO_DEVICE, "cannot select the device");
    const uint32_t B = s->dev.band_count, L = s->dev.layer_count, bins = s->dev.phase_bins;
    if (!s->adj_ws) {
        cudaError_t e = dev_malloc(&s->adj_ws, adjoint_workspace_bytes(B, L, bins));
        if (e != cudaSuccess) {
            s->adj_ws = nullptr;
            return cuda_fail(SKY_ERR_OUT_OF_MEMORY, "differentiable-render workspace allocation", e);
        }
    }
    W = adjoint_workspace(s->adj_ws, B, L, bins);
    A = AdjCtx{};
    A.S = s->dev;
    const float* d = p->sun_direction;
    const float len = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    if (len > 0.0f) {
        if (!std::isfinite(len)) return set_error(SKY_ERR_INVALID_CONFIG, "sun direction must be finite");
        for (int k = 0; k < 3; ++k) A.S.sun[k] = d[k] / len;
        host_orthonormal_basis(A.S.sun, A.S.sun_t, A.S.sun_b);
    }
    auto tables = [bins](AdjParamSet& X, const float* t) {
        X.phase = t;
        X.dphase = t + bins;
        X.cdf = t + 2 * bins;
        X.bin_pdf = t + 3 * bins;
    };
    A.P.layer = p->layer_params;
    A.P.band = p->band_params;
    tables(A.P, W.p_tables);
    A.distinct = (p->sample_layer_params && p->sample_layer_params != p->layer_params) ||
                 (p->sample_band_params && p->sample_band_params != p->band_params);
    if (A.distinct) {
        A.Q.layer = p->sample_layer_params ? p->sample_layer_params : p->layer_params;
        A.Q.band = p->sample_band_params ? p->sample_band_params : p->band_params;
        tables(A.Q, W.q_tables);
    } else {
        A.Q = A.P;
    }
    if (p->chain_radiance && A.distinct)
        return set_error(SKY_ERR_INVALID_CONFIG, "chain_radiance cannot be used with sample_* parameters");
    A.G.layer_maj = W.layer_maj;
    A.G.radius = W.radius;
    A.G.maj = W.maj;
    A.G.map = W.map;
    A.G.count = W.count;
    A.crossing_cost = s->tuning.crossing_cost;
    if (p->estimator > SKY_ADJOINT_NULL_COLLISIONS)
        return set_error(SKY_ERR_INVALID_CONFIG, "unknown adjoint estimator");
    A.estimator = p->estimator;
    return SKY_OK;
}

// One render of a differentiable launch: its launch constants for its sun (a
// non-zero sun_direction, else the context's sun), its sun frame and its
// chain-radiance buffer.  The first render of a launch sets the tracking mode
// (A.merge) the others must share.
int adjoint_job(SkyScene* s, const SkyRenderConfig* c, const float* sun_direction, float* chain_rad,
                uint64_t chain_len, bool first, AdjCtx& A, AdjJob& job) {
    int st = validate_config(s, c);
    if (st) return st;
    // the ray loop's 32-bit cell counter also counts one failed claim per warp
    if (slab_pixels(c) * s->dev.band_count > kMaxLaunchCells)
        return set_error(SKY_ERR_INVALID_CONFIG, "a launch holds at most 4026531840 (pixel, band) cells");
    if (c->tracking != SKY_TRACKING_RESIDUAL_CARRY && c->tracking != SKY_TRACKING_MERGED_LAYERS)
        return set_error(SKY_ERR_INVALID_CONFIG,
                         "differentiable renders track with SKY_TRACKING_RESIDUAL_CARRY or SKY_TRACKING_MERGED_LAYERS");
    const uint32_t merge = c->tracking == SKY_TRACKING_MERGED_LAYERS ? 1u : 0u;
    if (first) A.merge = merge;
    else if (merge != A.merge) return set_error(SKY_ERR_INVALID_CONFIG, "all renders of a batch need the same tracking");
    job = AdjJob{};
    SkyScene view;  // launch constants (sky-view LUT frame) for the render's sun
    view.dev = A.S;
    const float len = sun_direction ? std::sqrt(sun_direction[0] * sun_direction[0] +
                                                sun_direction[1] * sun_direction[1] +
                                                sun_direction[2] * sun_direction[2])
                                    : 0.0f;
    if (len > 0.0f) {
        if (!std::isfinite(len)) return set_error(SKY_ERR_INVALID_CONFIG, "sun direction must be finite");
        for (int k = 0; k < 3; ++k) view.dev.sun[k] = sun_direction[k] / len;
        host_orthonormal_basis(view.dev.sun, view.dev.sun_t, view.dev.sun_b);
    }
    job.L = make_launch(&view, c);
    for (int k = 0; k < 3; ++k) {
        job.sun[k] = view.dev.sun[k];
        job.sun_t[k] = view.dev.sun_t[k];
        job.sun_b[k] = view.dev.sun_b[k];
    }
    view.dev = DevScene{};
    const uint64_t cells = slab_pixels(c) * uint64_t(s->dev.band_count);
    job.cell_count = uint32_t(cells);
    if (chain_rad) {
        if (A.distinct)
            return set_error(SKY_ERR_INVALID_CONFIG, "chain_radiance cannot be used with sample_* parameters");
        const uint64_t chains = cells * c->spp;
        if (chain_len < chains)
            return set_error(SKY_ERR_INVALID_CONFIG, "chain_radiance holds " + std::to_string(chain_len) +
                                                         " floats; the render has " + std::to_string(chains) +
                                                         " chains");
    }
    job.chain_rad = chain_rad;
    return SKY_OK;
}

// Append `job` to the launch J (cells numbered in a row).
int adjoint_place(AdjJobs& J, AdjJob& job) {
    if (uint64_t(J.cells) + job.cell_count > kMaxLaunchCells)
        return set_error(SKY_ERR_INVALID_CONFIG, "a launch holds at most 4026531840 (pixel, band) cells");
    job.cell_begin = J.cells;
    J.j[J.count++] = job;
    J.cells += job.cell_count;
    return SKY_OK;
}

}  // namespace

extern "C" uint32_t sky_cuda_adjoint_param_count(const SkyScene* scene) {
    return scene ? 3u * scene->dev.layer_count + 2u : 0u;
}

namespace {

// The primal launches of renders `jobs` (n of them, outputs[i] each) over one
// parameter set, in launches of at most kAdjMaxJobs renders, then each
// render's finalize.  Every render is checked before the first launch (a
// refused batch writes nothing); the context's tables are baked first, once.
int adjoint_forward_jobs(SkyScene* s, AdjCtx& A, const AdjWorkspace& W, const SkyRenderConfig* const* configs,
                         const float* const* suns, float* const* chains, const uint64_t* chain_lens,
                         const SkyDeviceOutputs* const* outputs, uint32_t n, cudaStream_t stream) {
    if (n == 0) return set_error(SKY_ERR_INVALID_CONFIG, "at least one render is required");
    if (!outputs[0]->status) return set_error(SKY_ERR_INVALID_CONFIG, "outputs.status is required");
    if (A.distinct && n > 1)
        return set_error(SKY_ERR_INVALID_CONFIG, "a batch is rendered at its sampling parameters: no sample_*");
    const bool accumulate = (configs[0]->flags & SKY_FLAG_ACCUMULATE) != 0;
    std::vector<AdjJobs> launches((n + kAdjMaxJobs - 1u) / kAdjMaxJobs);
    std::memset(launches.data(), 0, launches.size() * sizeof(AdjJobs));
    int st;
    for (uint32_t i = 0; i < n; ++i) {
        AdjJob job;
        if ((st = adjoint_job(s, configs[i], suns[i], chains[i], chain_lens[i], i == 0, A, job))) return st;
        if (!outputs[i] || !outputs[i]->cell_sum)
            return set_error(SKY_ERR_INVALID_CONFIG, "outputs.cell_sum is required");
        if (configs[i]->phase_sampling != configs[0]->phase_sampling)
            return set_error(SKY_ERR_INVALID_CONFIG, "all renders of a batch need the same phase sampling");
        if (((configs[i]->flags & SKY_FLAG_ACCUMULATE) != 0) != accumulate)
            return set_error(SKY_ERR_INVALID_CONFIG, "all renders of a batch accumulate, or none");
        job.cell_sum = outputs[i]->cell_sum;
        job.cell_sumsq = outputs[i]->cell_sumsq;
        if ((st = adjoint_place(launches[i / kAdjMaxJobs], job))) return st;
    }
    clear_stale_error();
    cudaError_t e;
    if ((e = launch_adjoint_prepare(A, W, stream)) != cudaSuccess)
        return cuda_fail(SKY_ERR_LAUNCH, "majorant bake launch", e);
    for (const AdjJobs& J : launches) {
        e = launch_adjoint_primal(A, J, accumulate, outputs[0]->counters, outputs[0]->status, W.next_cell, stream);
        if (e != cudaSuccess) return cuda_fail(SKY_ERR_LAUNCH, "differentiable render launch", e);
    }
    for (uint32_t i = 0; i < n; ++i) {
        const SkyRenderConfig* c = configs[i];
        const uint32_t total_spp = accumulate ? c->sample_offset + c->spp : c->spp;
        const SkyDeviceOutputs* o = outputs[i];
        e = launch_finalize(A.S, slab_pixels(c), total_spp, o->cell_sum, o->cell_sumsq, o->film,
                            s->has_xyz ? o->xyz : nullptr, s->has_xyz ? o->xyz_var : nullptr,
                            s->has_xyz ? o->rgb : nullptr, stream);
        if (e != cudaSuccess) return cuda_fail(SKY_ERR_LAUNCH, "finalize kernel launch", e);
    }
    return SKY_OK;
}

// The gradient launches of renders over one parameter set (dloss[i] each),
// every render checked before the first launch.
int adjoint_backward_jobs(SkyScene* s, AdjCtx& A, const AdjWorkspace& W, const SkyRenderConfig* const* configs,
                          const float* const* suns, float* const* chains, const uint64_t* chain_lens,
                          const float* const* dloss, uint32_t n, const SkyAdjointGrads* grads,
                          cudaStream_t stream) {
    if (n == 0) return set_error(SKY_ERR_INVALID_CONFIG, "at least one render is required");
    if (!grads || (!grads->layer_grad && !grads->band_grad))
        return set_error(SKY_ERR_INVALID_CONFIG, "at least one of grads.layer_grad, grads.band_grad is required");
    if (!grads->status) return set_error(SKY_ERR_INVALID_CONFIG, "grads.status is required");
    std::vector<AdjJobs> launches((n + kAdjMaxJobs - 1u) / kAdjMaxJobs);
    std::memset(launches.data(), 0, launches.size() * sizeof(AdjJobs));
    int st;
    for (uint32_t i = 0; i < n; ++i) {
        AdjJob job;
        if ((st = adjoint_job(s, configs[i], suns[i], chains[i], chain_lens[i], i == 0, A, job))) return st;
        if (!dloss[i]) return set_error(SKY_ERR_INVALID_CONFIG, "dloss_dfilm is required for every render");
        if (configs[i]->phase_sampling != configs[0]->phase_sampling)
            return set_error(SKY_ERR_INVALID_CONFIG, "all renders of a batch need the same phase sampling");
        job.dloss = dloss[i];
        if ((st = adjoint_place(launches[i / kAdjMaxJobs], job))) return st;
    }
    clear_stale_error();
    cudaError_t e;
    if ((e = launch_adjoint_prepare(A, W, stream)) != cudaSuccess)
        return cuda_fail(SKY_ERR_LAUNCH, "majorant bake launch", e);
    for (const AdjJobs& J : launches) {
        e = launch_adjoint_grad(A, J, grads->layer_grad, grads->band_grad, grads->counters, grads->status, W.next_cell,
                                stream);
        if (e != cudaSuccess) return cuda_fail(SKY_ERR_LAUNCH, "adjoint launch", e);
    }
    return SKY_OK;
}

int require_sampling_at_evaluation(const SkyAdjointParams* params) {
    if (params && (params->sample_layer_params || params->sample_band_params))
        return set_error(SKY_ERR_INVALID_CONFIG,
                         "the gradient is taken at the sampling parameters: sample_layer_params and "
                         "sample_band_params must be NULL");
    return SKY_OK;
}

}  // namespace

extern "C" int sky_cuda_adjoint_forward(const SkyScene* scene, const SkyRenderConfig* config,
                                        const SkyAdjointParams* params, const SkyDeviceOutputs* outputs,
                                        void* cuda_stream) {
    SkyScene* s = const_cast<SkyScene*>(scene);
    AdjCtx A;
    AdjWorkspace W;
    int st = adjoint_setup(s, params, A, W);
    if (st) return st;
    if (!outputs) return set_error(SKY_ERR_INVALID_CONFIG, "outputs.cell_sum is required");
    const float* sun = nullptr;  // the context's sun: the params' or the scene's
    float* chain = params->chain_radiance;
    const uint64_t chain_len = params->chain_radiance_len;
    return adjoint_forward_jobs(s, A, W, &config, &sun, &chain, &chain_len, &outputs, 1,
                                static_cast<cudaStream_t>(cuda_stream));
}

extern "C" int sky_cuda_adjoint_backward(const SkyScene* scene, const SkyRenderConfig* config,
                                         const SkyAdjointParams* params, const SkyAdjointGrads* grads,
                                         void* cuda_stream) {
    SkyScene* s = const_cast<SkyScene*>(scene);
    int st = require_sampling_at_evaluation(params);
    if (st) return st;
    AdjCtx A;
    AdjWorkspace W;
    if ((st = adjoint_setup(s, params, A, W))) return st;
    if (!grads || !grads->dloss_dfilm || (!grads->layer_grad && !grads->band_grad))
        return set_error(SKY_ERR_INVALID_CONFIG,
                         "grads.dloss_dfilm and at least one of grads.layer_grad, grads.band_grad are required");
    const float* sun = nullptr;
    float* chain = params->chain_radiance;
    const uint64_t chain_len = params->chain_radiance_len;
    const float* dloss = grads->dloss_dfilm;
    return adjoint_backward_jobs(s, A, W, &config, &sun, &chain, &chain_len, &dloss, 1, grads,
                                 static_cast<cudaStream_t>(cuda_stream));
}

extern "C" int sky_cuda_adjoint_forward_batch(const SkyScene* scene, const SkyAdjointJob* jobs, uint32_t job_count,
                                              const SkyAdjointParams* params, void* cuda_stream) {
    SkyScene* s = const_cast<SkyScene*>(scene);
    int st = require_sampling_at_evaluation(params);
    if (st) return st;
    if (!jobs || job_count == 0) return set_error(SKY_ERR_INVALID_CONFIG, "jobs and job_count >= 1 are required");
    AdjCtx A;
    AdjWorkspace W;
    if ((st = adjoint_setup(s, params, A, W))) return st;
    std::vector<const SkyRenderConfig*> configs(job_count);
    std::vector<const float*> suns(job_count);
    std::vector<float*> chains(job_count);
    std::vector<uint64_t> lens(job_count);
    std::vector<const SkyDeviceOutputs*> outs(job_count);
    for (uint32_t i = 0; i < job_count; ++i) {
        configs[i] = &jobs[i].config;
        suns[i] = jobs[i].sun_direction;
        chains[i] = jobs[i].chain_radiance;
        lens[i] = jobs[i].chain_radiance_len;
        outs[i] = &jobs[i].outputs;
    }
    return adjoint_forward_jobs(s, A, W, configs.data(), suns.data(), chains.data(), lens.data(), outs.data(),
                                job_count, static_cast<cudaStream_t>(cuda_stream));
}

extern "C" int sky_cuda_adjoint_backward_batch(const SkyScene* scene, const SkyAdjointJob* jobs, uint32_t job_count,
                                               const SkyAdjointParams* params, const SkyAdjointGrads* grads,
                                               void* cuda_stream) {
    SkyScene* s = const_cast<SkyScene*>(scene);
    int st = require_sampling_at_evaluation(params);
    if (st) return st;
    if (!jobs || job_count == 0) return set_error(SKY_ERR_INVALID_CONFIG, "jobs and job_count >= 1 are required");
    AdjCtx A;
    AdjWorkspace W;
    if ((st = adjoint_setup(s, params, A, W))) return st;
    std::vector<const SkyRenderConfig*> configs(job_count);
    std::vector<const float*> suns(job_count);
    std::vector<float*> chains(job_count);
    std::vector<uint64_t> lens(job_count);
    std::vector<const float*> dloss(job_count);
    for (uint32_t i = 0; i < job_count; ++i) {
        configs[i] = &jobs[i].config;
        suns[i] = jobs[i].sun_direction;
        chains[i] = jobs[i].chain_radiance;
        lens[i] = jobs[i].chain_radiance_len;
        dloss[i] = jobs[i].dloss_dfilm;
    }
    return adjoint_backward_jobs(s, A, W, configs.data(), suns.data(), chains.data(), lens.data(), dloss.data(),
                                 job_count, grads, static_cast<cudaStream_t>(cuda_stream));
}

extern "C" int sky_cuda_bake_majorants(const SkyScene* scene, const SkyAdjointParams* params, float* majorants_out,
                                       void* cuda_stream) {
    SkyScene* s = const_cast<SkyScene*>(scene);
    if (!majorants_out) return set_error(SKY_ERR_INVALID_CONFIG, "majorants_out is null");
    SkyAdjointParams p{};
    if (params) {
        p = *params;
        if (p.sample_layer_params) p.layer_params = p.sample_layer_params;
        if (p.sample_band_params) p.band_params = p.sample_band_params;
        p.sample_layer_params = nullptr;
        p.sample_band_params = nullptr;
        p.chain_radiance = nullptr;
        p.chain_radiance_len = 0;
    }
    AdjCtx A;
    AdjWorkspace W;
    int st = adjoint_setup(s, params ? &p : nullptr, A, W);
    if (st) return st;
    cudaStream_t stream = static_cast<cudaStream_t>(cuda_stream);
    clear_stale_error();
    cudaError_t e = launch_adjoint_prepare(A, W, stream);
    if (e != cudaSuccess) return cuda_fail(SKY_ERR_LAUNCH, "majorant bake launch", e);
    e = cudaMemcpyAsync(majorants_out, W.layer_maj, size_t(s->dev.band_count) * s->dev.layer_count * sizeof(float),
                        cudaMemcpyDeviceToDevice, stream);
    if (e != cudaSuccess) return cuda_fail(SKY_ERR_COPY, "majorant copy", e);
    return SKY_OK;
}

// ---- optimizer scoring ---------------------------------------------------------------

namespace {

struct DeviceScratch {  // frees what it allocated when the call returns
    std::vector<void*> ptrs;
    ~DeviceScratch() {
        for (void* p : ptrs) cudaFree(p);
    }
    template <class T>
    cudaError_t alloc(T** out, size_t count) {
        void* p = nullptr;
        cudaError_t e = dev_malloc(&p, std::max<size_t>(count, 1) * sizeof(T));
        if (e == cudaSuccess) ptrs.push_back(p);
        *out = static_cast<T*>(p);
        return e;
    }
};

}  // namespace

extern "C" int sky_cuda_score_combos(const float* bands, uint32_t band_count, uint64_t samples,
                                     const float* ref_oklab, float reference_scale, const uint32_t* combo_bands,
                                     const float* combo_xyz, uint32_t combo_count, uint32_t channels,
                                     SkyComboScore* results, void* cuda_stream) {
    if (!bands || !ref_oklab || !combo_bands || !combo_xyz || !results)
        return set_error(SKY_ERR_INVALID_CONFIG, "bands, ref_oklab, combos and results are required");
    if (samples == 0 || band_count == 0 || channels == 0 || combo_count == 0)
        return set_error(SKY_ERR_INVALID_CONFIG, "samples, band_count, channels and combo_count must be positive");
    if (!(reference_scale > 0.0f) || !std::isfinite(reference_scale))
        return set_error(SKY_ERR_INVALID_CONFIG, "reference_scale must be positive and finite");
    for (size_t i = 0; i < size_t(combo_count) * channels; ++i)
        if (combo_bands[i] >= band_count) return set_error(SKY_ERR_INVALID_CONFIG, "combo band index out of range");
    int device = 0, sms = 1;
    if (cudaGetDevice(&device) != cudaSuccess) return set_error(SKY_ERR_NO_DEVICE, "no usable CUDA device");
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    cudaStream_t stream = static_cast<cudaStream_t>(cuda_stream);
    // combinations per pass: distances of at most 2^28 (1 GB) and 8192 combinations
    const uint32_t chunk =
        uint32_t(std::max<uint64_t>(1, std::min<uint64_t>({combo_count, 8192u, (1ull << 28) / samples})));
    constexpr uint32_t kTargets = 5;  // p50, p90, p95, p99, max
    const double quantiles[kTargets] = {0.50, 0.90, 0.95, 0.99, 1.0};
    DeviceScratch mem;
    float* dist;
    double* sums;
    uint32_t *d_bands, *d_tcombo, *d_tprefix, *d_hist;
    float* d_xyz;
    cudaError_t e;
    if ((e = mem.alloc(&dist, size_t(chunk) * samples)) || (e = mem.alloc(&sums, size_t(chunk) * 3)) ||
        (e = mem.alloc(&d_bands, size_t(chunk) * channels)) || (e = mem.alloc(&d_xyz, size_t(chunk) * channels * 3)) ||
        (e = mem.alloc(&d_tcombo, size_t(chunk) * kTargets)) || (e = mem.alloc(&d_tprefix, size_t(chunk) * kTargets)) ||
        (e = mem.alloc(&d_hist, size_t(chunk) * kTargets * kScoreHistBins)))
        return cuda_fail(SKY_ERR_OUT_OF_MEMORY, "scoring scratch allocation", e);
    std::vector<double> h_sums(size_t(chunk) * 3);
    std::vector<uint32_t> h_hist(size_t(chunk) * kTargets * kScoreHistBins), tcombo(size_t(chunk) * kTargets),
        tprefix(size_t(chunk) * kTargets);
    std::vector<uint64_t> rank(size_t(chunk) * kTargets);
    clear_stale_error();
    for (uint32_t c0 = 0; c0 < combo_count; c0 += chunk) {
        const uint32_t nc = std::min(chunk, combo_count - c0);
        if ((e = cudaMemcpyAsync(d_bands, combo_bands + size_t(c0) * channels, size_t(nc) * channels * 4,
                                 cudaMemcpyHostToDevice, stream)) ||
            (e = cudaMemcpyAsync(d_xyz, combo_xyz + size_t(c0) * channels * 3, size_t(nc) * channels * 12,
                                 cudaMemcpyHostToDevice, stream)) ||
            (e = cudaMemsetAsync(sums, 0, size_t(nc) * 3 * sizeof(double), stream)))
            return cuda_fail(SKY_ERR_COPY, "scoring upload", e);
        if ((e = launch_score_distances(bands, samples, ref_oklab, 1.0f / reference_scale, d_bands, d_xyz, nc,
                                        channels, dist, sums, stream)))
            return cuda_fail(SKY_ERR_LAUNCH, "distance kernel launch", e);
        if ((e = cudaMemcpyAsync(h_sums.data(), sums, size_t(nc) * 3 * sizeof(double), cudaMemcpyDeviceToHost,
                                 stream)) ||
            (e = cudaStreamSynchronize(stream)))
            return cuda_fail(SKY_ERR_SYNC, "distance sums", e);
        uint32_t targets = 0;
        for (uint32_t c = 0; c < nc; ++c) {
            const uint64_t n = uint64_t(h_sums[c * 3 + 2] + 0.5);
            SkyComboScore& r = results[c0 + c];
            r = SkyComboScore{};
            r.finite = n;
            if (n == 0) {
                r.mean = r.rmse = r.p50 = r.p90 = r.p95 = r.p99 = r.max = r.score = std::nan("");
                continue;
            }
            r.mean = h_sums[c * 3] / double(n);
            r.rmse = std::sqrt(h_sums[c * 3 + 1] / double(n));
            for (uint32_t q = 0; q < kTargets; ++q) {  // percentile_sorted: round((n - 1) q), half away from 0
                tcombo[targets] = c;
                tprefix[targets] = 0;
                rank[targets] = uint64_t(std::floor(double(n - 1) * quantiles[q] + 0.5));
                ++targets;
            }
        }
        // three radix-selection passes over the bits of the non-negative distances
        const uint32_t shifts[3] = {21u, 10u, 0u}, widths[3] = {11u, 11u, 10u};
        for (int pass = 0; pass < 3 && targets > 0; ++pass) {
            if ((e = cudaMemcpyAsync(d_tcombo, tcombo.data(), targets * 4, cudaMemcpyHostToDevice, stream)) ||
                (e = cudaMemcpyAsync(d_tprefix, tprefix.data(), targets * 4, cudaMemcpyHostToDevice, stream)) ||
                (e = cudaMemsetAsync(d_hist, 0, size_t(targets) * kScoreHistBins * 4, stream)))
                return cuda_fail(SKY_ERR_COPY, "selection upload", e);
            if ((e = launch_select_hist(dist, samples, d_tcombo, d_tprefix, targets, shifts[pass], widths[pass], d_hist,
                                        uint32_t(sms), stream)))
                return cuda_fail(SKY_ERR_LAUNCH, "selection kernel launch", e);
            if ((e = cudaMemcpyAsync(h_hist.data(), d_hist, size_t(targets) * kScoreHistBins * 4,
                                     cudaMemcpyDeviceToHost, stream)) ||
                (e = cudaStreamSynchronize(stream)))
                return cuda_fail(SKY_ERR_SYNC, "selection histogram", e);
            const uint32_t bins = 1u << widths[pass];
            for (uint32_t t = 0; t < targets; ++t) {
                const uint32_t* h = h_hist.data() + size_t(t) * kScoreHistBins;
                uint64_t below = 0;
                uint32_t b = 0;
                for (; b + 1 < bins && below + h[b] <= rank[t]; ++b) below += h[b];
                rank[t] -= below;
                tprefix[t] = (tprefix[t] << widths[pass]) | b;
            }
        }
        for (uint32_t t = 0; t < targets; ++t) {
            float v;
            std::memcpy(&v, &tprefix[t], 4);
            SkyComboScore& r = results[c0 + tcombo[t]];
            double* slot[kTargets] = {&r.p50, &r.p90, &r.p95, &r.p99, &r.max};
            *slot[t % kTargets] = double(v);
        }
        for (uint32_t c = 0; c < nc; ++c) {
            SkyComboScore& r = results[c0 + c];
            if (r.finite) r.score = r.rmse + 0.25 * r.p95;
        }
    }
    return SKY_OK;
}

// ---- Mie phase-table bake -----------------------------------------------------------

extern "C" int sky_cuda_bake_mie_phase(const SkyMieDistribution* dist, const double* wavelength_um,
                                       const double* refr_re, const double* refr_im, uint32_t band_count,
                                       uint32_t phase_bins, double* phase_out, SkyMieBand* band_out) {
    if (!dist || !wavelength_um || !refr_re || !refr_im || !phase_out)
        return set_error(SKY_ERR_INVALID_CONFIG, "dist, wavelengths, refractive indices and phase_out are required");
    if (band_count == 0 || phase_bins == 0) return set_error(SKY_ERR_INVALID_CONFIG, "band_count and phase_bins must be positive");
    const SkyMieDistribution& D = *dist;
    if (!(D.r_min_um > 0.0) || !(D.r_max_um >= D.r_min_um) || !(D.r_mode_um > 0.0) || !(D.sigma_g > 1.0) ||
        D.r_count == 0 || !std::isfinite(D.r_max_um) || !std::isfinite(D.sigma_g))
        return set_error(SKY_ERR_INVALID_CONFIG, "size distribution needs 0 < r_min <= r_max, r_mode > 0, "
                                                 "sigma_g > 1 and r_count >= 1");
    // radii (numpy.geomspace) and lognormal weights (bake_opac_data.py:103-109)
    std::vector<double> r(D.r_count), w(D.r_count);
    const double l0 = std::log(D.r_min_um), l1 = std::log(D.r_max_um), ls = std::log(D.sigma_g);
    double wsum = 0.0;
    for (uint32_t i = 0; i < D.r_count; ++i) {
        r[i] = D.r_count == 1 ? D.r_min_um
               : i == 0       ? D.r_min_um
               : i + 1 == D.r_count ? D.r_max_um
                                    : std::exp(l0 + (l1 - l0) * double(i) / double(D.r_count - 1));
        const double z = std::log(r[i] / D.r_mode_um);
        w[i] = std::exp(-z * z / (2.0 * ls * ls));
        wsum += w[i];
    }
    if (!(wsum > 0.0)) return set_error(SKY_ERR_INVALID_CONFIG, "the size distribution has no weight on its radii");
    const double two_pi = 2.0 * 3.14159265358979323846;
    std::vector<MieItem> items(size_t(band_count) * D.r_count);
    uint64_t aoff = 0, doff = 0;
    uint32_t max_terms = 0;
    for (uint32_t b = 0; b < band_count; ++b) {
        const double lam = wavelength_um[b], mre = refr_re[b], mim = refr_im[b];
        if (!(lam > 0.0) || !std::isfinite(lam) || !(mre > 0.0) || !std::isfinite(mre) || !(mim >= 0.0) ||
            !std::isfinite(mim))
            return set_error(SKY_ERR_INVALID_CONFIG, "band " + std::to_string(b) +
                                                         ": wavelength and refractive index must be finite, "
                                                         "wavelength > 0, n > 0, k >= 0");
        for (uint32_t i = 0; i < D.r_count; ++i) {
            MieItem& it = items[size_t(b) * D.r_count + i];
            it.k = two_pi / lam;
            it.x = it.k * r[i];
            it.m_re = mre;
            it.m_im = mim;
            it.weight = w[i] / wsum;
            it.band = b;
            if (!(it.x <= 12000.0))
                return set_error(SKY_ERR_INVALID_CONFIG, "size parameter 2 pi r / lambda above 12000");
            it.terms = mie_terms(it.x);
            const double mx = it.x * std::sqrt(mre * mre + mim * mim);
            it.dterms = uint32_t(std::max(double(it.terms), mx)) + 16u;
            it.aoff = aoff;
            it.doff = doff;
            it._pad = 0;
            aoff += it.terms;
            doff += uint64_t(it.dterms) + 1u;
            max_terms = std::max(max_terms, it.terms);
        }
    }
    if (doff * sizeof(double2) + aoff * sizeof(float4) > (uint64_t(16) << 30))
        return set_error(SKY_ERR_INVALID_CONFIG, "bake too large: more than 16 GB of series scratch");
    DeviceScratch mem;
    MieItem* d_items = nullptr;
    double2* d_scr = nullptr;
    float4* d_ab = nullptr;
    double *d_q = nullptr, *d_acc = nullptr;
    cudaError_t e;
    if ((e = mem.alloc(&d_items, items.size())) || (e = mem.alloc(&d_scr, doff)) || (e = mem.alloc(&d_ab, aoff)) ||
        (e = mem.alloc(&d_q, items.size() * 3)) || (e = mem.alloc(&d_acc, size_t(band_count) * phase_bins)))
        return cuda_fail(SKY_ERR_OUT_OF_MEMORY, "Mie bake scratch allocation", e);
    clear_stale_error();
    if ((e = cudaMemcpy(d_items, items.data(), items.size() * sizeof(MieItem), cudaMemcpyHostToDevice)) ||
        (e = cudaMemset(d_acc, 0, size_t(band_count) * phase_bins * sizeof(double))))
        return cuda_fail(SKY_ERR_COPY, "Mie bake upload", e);
    if ((e = launch_mie_bake(d_items, uint32_t(items.size()), max_terms, d_scr, d_ab, d_q, phase_bins, d_acc,
                             nullptr)))
        return cuda_fail(SKY_ERR_LAUNCH, "Mie bake kernels", e);
    std::vector<double> q(items.size() * 3);
    if ((e = cudaMemcpy(q.data(), d_q, q.size() * sizeof(double), cudaMemcpyDeviceToHost)) ||
        (e = cudaMemcpy(phase_out, d_acc, size_t(band_count) * phase_bins * sizeof(double), cudaMemcpyDeviceToHost)))
        return cuda_fail(SKY_ERR_COPY, "Mie bake readback", e);
    const double pi = 0.5 * two_pi;
    for (uint32_t b = 0; b < band_count; ++b) {
        double sca = 0.0, ext = 0.0, g = 0.0;
        for (uint32_t i = 0; i < D.r_count; ++i) {
            const MieItem& it = items[size_t(b) * D.r_count + i];
            const double area = pi * r[i] * r[i] * it.weight;
            sca += area * q[3 * (size_t(b) * D.r_count + i)];
            ext += area * q[3 * (size_t(b) * D.r_count + i) + 1];
            g += area * q[3 * (size_t(b) * D.r_count + i)] * q[3 * (size_t(b) * D.r_count + i) + 2];
        }
        double* row = phase_out + size_t(b) * phase_bins;
        for (uint32_t j = 0; j < phase_bins; ++j) row[j] = sca > 0.0 ? row[j] / sca : 0.0;
        if (band_out) band_out[b] = SkyMieBand{sca, ext, sca > 0.0 ? g / sca : 0.0};
    }
    return SKY_OK;
}

// ---- allocation-free batch render -------------------------------------------------

namespace {

struct NoAllocScratch {
    DevJob jobs[SKY_NOALLOC_MAX_JOBS];
    uint32_t work_counter;
};
static_assert(sizeof(NoAllocScratch) <= SKY_NOALLOC_SCRATCH_BYTES, "scratch area too small");

// The job rows of one call, handed to the install kernel by value: kernel
// arguments may hold up to 32764 bytes on this architecture, so the rows
// travel with the launch itself and no host buffer is read after the call.
struct NoAllocTable {
    DevJob jobs[SKY_NOALLOC_MAX_JOBS];
    uint32_t words;  // 32-bit words of the rows in use
};
static_assert(sizeof(NoAllocTable) <= 32000, "job table exceeds the kernel-argument limit");
static_assert(sizeof(DevJob) % 4 == 0, "job rows are copied as 32-bit words");

// The job table and work counter of sky_cuda_render_batch_noalloc().  Host
// code may not use this name as a device address: it is resolved with
// cudaGetSymbolAddress() below.  Device code names it directly.
static __device__ __align__(256) unsigned char g_noalloc_scratch[SKY_NOALLOC_SCRATCH_BYTES];

// Copy the call's job rows from the kernel argument into the scratch area,
// ordered on the caller's stream before the tracing kernels that read them.
__global__ void __launch_bounds__(256) noalloc_install_kernel(const __grid_constant__ NoAllocTable table) {
    const uint32_t* src = reinterpret_cast<const uint32_t*>(table.jobs);
    uint32_t* dst = reinterpret_cast<uint32_t*>(reinterpret_cast<NoAllocScratch*>(g_noalloc_scratch)->jobs);
    for (uint32_t i = threadIdx.x; i < table.words; i += blockDim.x) dst[i] = src[i];
}

}  // namespace

extern "C" int sky_cuda_render_batch_noalloc(const SkyScene* scene, const SkyRenderConfig* job_configs,
                                             const SkyDeviceOutputs* outputs, uint32_t job_count,
                                             void* cuda_stream) {
    if (!scene || !job_configs || !outputs) return set_error(SKY_ERR_INVALID_CONFIG, "scene, job_configs and outputs are required");
    if (job_count == 0) return set_error(SKY_ERR_INVALID_CONFIG, "job_count must be at least 1");
    if (job_count > SKY_NOALLOC_MAX_JOBS)
        return set_error(SKY_ERR_INVALID_CONFIG, "job_count " + std::to_string(job_count) +
                                                     " exceeds SKY_NOALLOC_MAX_JOBS (" +
                                                     std::to_string(SKY_NOALLOC_MAX_JOBS) + ")");
    if (!outputs[0].status) return set_error(SKY_ERR_INVALID_CONFIG, "outputs[0].status is required");
    SkyScene* s = const_cast<SkyScene*>(scene);
    NoAllocTable table;
    std::memset(&table, 0, sizeof(table));
    uint64_t cells = 0;
    uint32_t max_cells = 0;
    for (uint32_t i = 0; i < job_count; ++i) {
        const SkyRenderConfig* c = &job_configs[i];
        int st = validate_config(s, c);
        if (st) return st;
        if (c->kernel == SKY_KERNEL_PLAIN)
            return set_error(SKY_ERR_INVALID_CONFIG,
                             "the allocation-free render runs the wavefront kernel only; SKY_KERNEL_PLAIN was asked for");
        if (c->tracking != job_configs[0].tracking || c->phase_sampling != job_configs[0].phase_sampling)
            return set_error(SKY_ERR_INVALID_CONFIG, "all jobs of a batch need the same tracking and phase sampling");
        if (!outputs[i].cell_sum) return set_error(SKY_ERR_INVALID_CONFIG, "outputs[i].cell_sum is required");
        const bool accumulate = (c->flags & SKY_FLAG_ACCUMULATE) != 0;
        DevJob& job = table.jobs[i];
        job.S = s->dev;
        job.L = make_launch(s, c);
        job.cell_sum = outputs[i].cell_sum;
        job.cell_sumsq = outputs[i].cell_sumsq;
        job.film = outputs[i].film;
        job.xyz = s->has_xyz ? outputs[i].xyz : nullptr;
        job.xyz_var = s->has_xyz ? outputs[i].xyz_var : nullptr;
        job.rgb = s->has_xyz ? outputs[i].rgb : nullptr;
        job.accumulate = accumulate ? 1u : 0u;
        job.total_spp = accumulate ? c->sample_offset + c->spp : c->spp;
        if ((st = place_job(job, slab_pixels(c), s->dev.band_count, cells, max_cells))) return st;
    }
    table.words = uint32_t(job_count * sizeof(DevJob) / 4u);
    if (cudaSetDevice(s->device) != cudaSuccess) return set_error(SKY_ERR_NO_DEVICE, "cannot select the device");
    // The area's address in the current context, looked up on every call (a
    // cached address would outlive a context reset).
    void* scratch = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&scratch, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(SKY_ERR_DEVICE_INIT, "locating the allocation-free scratch area", e);
    cudaStream_t stream = static_cast<cudaStream_t>(cuda_stream);
    clear_stale_error();
    noalloc_install_kernel<<<1, 256, 0, stream>>>(table);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(SKY_ERR_LAUNCH, "job table install launch", e);
    uint32_t* counter = reinterpret_cast<uint32_t*>(static_cast<unsigned char*>(scratch) +
                                                    offsetof(NoAllocScratch, work_counter));
    // the launch resets the work counter itself
    const WaveLaunch w = wave_launch(s, table.jobs[0], static_cast<const DevJob*>(scratch), job_count, cells,
                                     max_cells, job_configs[0].tracking, job_configs[0].phase_sampling, counter,
                                     outputs[0].counters, outputs[0].status);
    e = launch_trace_wave(w, stream);
    if (e != cudaSuccess) return cuda_fail(SKY_ERR_LAUNCH, "wavefront tracing launch", e);
    return SKY_OK;
}
