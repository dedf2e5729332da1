// trace_plain.cu — the plain tracer: one thread per (pixel, band, sample)
// chain, one launch per render.
//
// A warp owns one (pixel, band) cell and traces its samples 32 at a time,
// one chain per lane (sky_trace.wgsl:703-776); after each round the warp
// reduces the 32 radiances in FP64 with shuffles, and one lane stores the
// cell's sum and sum of squares.  The reference instead loops over a
// 2-sample chunk inside one invocation per (pixel, band) and re-dispatches
// per chunk (sky_trace.wgsl:778-816, integrator.rs:252-283).

#include "trace_kernels.h"

#include "sky_device.cuh"

namespace sky {
namespace {

// Binary transmittance of a shadow ray from `pos` towards `ldir` (sky_trace.wgsl:574-577):
// 0 when the ray hits the ground or collides, 1 otherwise.
template <int kTracking>
__device__ __forceinline__ float shadow_transmittance(const DevScene& S, V3 pos, V3 ldir, uint32_t band, Rng& rng,
                                                      Counters& n, bool& watchdog) {
    V3 so = madd(pos, ldir, kRayEpsilonKm);
    RayGeo sg = ray_geo(so, ldir);
    float t_b;
    uint32_t kind;
    ++n.e[SKY_EVENT_BOUNDARY];
    if (!next_boundary(S, sg, t_b, kind) || kind != 1u) return -1.0f;  // no sun visible: no contribution
    float t_hit;
    return track_ray<kTracking>(S, global_medium(S), sg, t_b, band, rng, t_hit, n, watchdog, true) ? 0.0f : 1.0f;
}

// trace_path (sky_trace.wgsl:703-776) for one chain.
template <int kTracking, int kPhase, int kAer>
__device__ float trace_chain(const DevScene& S, const DevLaunch& L, uint32_t x, uint32_t y, uint32_t band,
                             uint32_t sample, Counters& n, bool& watchdog) {
    const uint32_t pixel = y * L.width + x;
    Rng rng;
    rng.init(pixel, sample, band, L.seed_lo, L.seed_hi);
    V3 dir = camera_dir(L, x, y, rng);
    V3 org = mk(0.0f, S.ground_radius + fmaxf(L.observer_altitude, 0.0f), 0.0f);
    ++n.e[SKY_EVENT_CHAIN];
    const float l_sun = __ldg(&S.bands[band].solar_radiance);
    const float inv_lights = 1.0f / float(L.direct_light_samples);
    float throughput = 1.0f, radiance = 0.0f;
    for (uint32_t depth = 0;; ++depth) {
        if (depth >= L.watchdog_limit) {
            watchdog = true;
            return radiance;
        }
        if (L.max_orders != 0u && depth >= L.max_orders) break;
        RayGeo g = ray_geo(org, dir);
        float t_b;
        uint32_t kind;
        ++n.e[SKY_EVENT_BOUNDARY];
        if (!next_boundary(S, g, t_b, kind)) break;
        float t_hit;
        if (track_ray<kTracking>(S, global_medium(S), g, t_b, band, rng, t_hit, n, watchdog, false)) {
            ++n.e[SKY_EVENT_SCATTER];
            V3 pos = madd(org, dir, t_hit);
            Coeffs c = coefficients_at<kAer>(S, S.knot_z, S.finder, band, altitude_at(g, t_hit, S.ground_radius));
            if (c.extinction <= 0.0f || c.scattering <= 0.0f) break;
            throughput *= fminf(fmaxf(c.scattering / c.extinction, 0.0f), 1.0f);
            if (throughput <= 0.0f) break;
            // direct_sun_at_scatter (sky_trace.wgsl:566-585)
            float nee = 0.0f;
            for (uint32_t ls = 0; ls < L.direct_light_samples; ++ls) {
                V3 ldir = sample_sun_cone(S, rng);
                ++n.e[SKY_EVENT_NEE];
                float trans = shadow_transmittance<kTracking>(S, pos, ldir, band, rng, n, watchdog);
                if (trans > 0.0f) nee += l_sun * trans * mixed_phase<kAer>(S, c, band, dot3(dir, ldir)) / S.light_pdf;
            }
            radiance += throughput * (nee * inv_lights);
            V3 new_dir;
            if (kPhase == SKY_PHASE_TABULATED) {
                throughput *= sample_tabulated<kAer>(S, c, band, dir, rng, new_dir);
            } else {
                new_dir = sample_isotropic(rng);
                throughput *= mixed_phase<kAer>(S, c, band, dot3(dir, new_dir)) / kIsotropicPdf;
            }
            if (depth >= L.rr_start_depth) {  // russian_roulette (sky_trace.wgsl:691-701)
                float q = fminf(fmaxf(throughput, 0.05f), 0.95f);
                if (rng.next() > q) break;
                throughput = throughput / q;
            }
            org = madd(pos, new_dir, kRayEpsilonKm);
            dir = new_dir;
        } else if (kind == 1u) {
            if (depth == 0u && dot3(dir, load3(S.sun)) >= S.cos_max) radiance += throughput * l_sun;
            break;
        } else {
            // ground_radiance (sky_trace.wgsl:587-608) and the Lambert bounce (:750-766)
            ++n.e[SKY_EVENT_GROUND];
            V3 pos = madd(org, dir, t_b);
            V3 normal = normalize_or_y(pos);
            float ground = 0.0f;
            for (uint32_t ls = 0; ls < L.direct_light_samples; ++ls) {
                V3 ldir = sample_sun_cone(S, rng);
                ++n.e[SKY_EVENT_NEE];
                float cos_sun = fmaxf(dot3(normal, ldir), 0.0f);
                if (cos_sun > 0.0f) {
                    float trans = shadow_transmittance<kTracking>(S, pos, ldir, band, rng, n, watchdog);
                    if (trans > 0.0f) ground += S.ground_albedo * kInvPi * l_sun * trans * cos_sun / S.light_pdf;
                }
            }
            radiance += throughput * (ground * inv_lights);
            float pdf;
            V3 bounce = sample_cosine_hemisphere(normal, rng, pdf);
            float cos_out = fmaxf(dot3(normal, bounce), 0.0f);
            if (pdf <= 0.0f || cos_out <= 0.0f) break;
            throughput *= S.ground_albedo * kInvPi * cos_out / pdf;
            if (depth >= L.rr_start_depth) {
                float q = fminf(fmaxf(throughput, 0.05f), 0.95f);
                if (rng.next() > q) break;
                throughput = throughput / q;
            }
            org = madd(pos, bounce, kRayEpsilonKm);
            dir = bounce;
        }
        if (radiance < 0.0f || radiance != radiance || throughput < 0.0f || throughput != throughput) return 0.0f;
    }
    return fmaxf(radiance, 0.0f);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ uint32_t warp_sum_u32(uint32_t v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// kAer: aerosol species the medium functions evaluate (coefficients_at()).
template <int kTracking, int kPhase, int kAer>
__global__ void __launch_bounds__(256) trace_plain_kernel(DevScene S, DevLaunch L, double* __restrict__ cell_sum,
                                                          double* __restrict__ cell_sumsq,
                                                          unsigned long long* __restrict__ counters,
                                                          uint32_t* __restrict__ status, uint64_t cells,
                                                          uint32_t accumulate) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t q = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    if (q >= cells) return;  // whole warps only: blockDim is a multiple of 32
    // warps run band-major (consecutive warps: consecutive pixels of one band), so the
    // resident warps share one band's tables in L1; the cells keep the pixel-major layout
    const uint64_t npix = cells / L.band_count;
    const uint32_t band = uint32_t(q / npix);
    const uint64_t pixel = q - uint64_t(band) * npix;  // pixel of the slab; y is the image row
    const uint64_t cell = pixel * L.band_count + band;
    const uint32_t x = uint32_t(pixel % L.width), y = uint32_t(pixel / L.width) + L.row_begin;
    Counters n;
    n.clear();
    bool watchdog = false;
    // The warp owns the cell: rounds of 32 samples are reduced in a fixed
    // order, so sums are reproducible and progressive renders whose sample
    // offsets are multiples of 32 add up bit-exactly to a single render.
    double sum = 0.0, sumsq = 0.0;
    if (accumulate) {
        sum = cell_sum[cell];
        if (cell_sumsq) sumsq = cell_sumsq[cell];
    }
    for (uint32_t base = 0; base < L.spp; base += 32u) {
        const uint32_t s_local = base + lane;
        float r = 0.0f;
        if (s_local < L.spp)
            r = trace_chain<kTracking, kPhase, kAer>(S, L, x, y, band, L.sample_offset + s_local, n, watchdog);
        const double rd = double(r);
        sum += warp_sum(rd);
        sumsq += warp_sum(rd * rd);
    }
    if (lane == 0) {
        cell_sum[cell] = sum;
        if (cell_sumsq) cell_sumsq[cell] = sumsq;
    }
    if (counters) {
#pragma unroll
        for (int e = 0; e < SKY_EVENT_COUNT; ++e) {
            uint32_t v = warp_sum_u32(n.e[e]);
            if (lane == 0 && v) atomicAdd(counters + e, (unsigned long long)v);
        }
    }
    if (__any_sync(0xffffffffu, watchdog) && lane == 0) atomicOr(status, 1u);
}

}  // namespace

cudaError_t launch_trace_plain(const DevScene& S, const DevLaunch& L, double* cell_sum, double* cell_sumsq,
                               unsigned long long* counters, uint32_t* status, bool accumulate,
                               uint32_t aerosol_species, cudaStream_t stream) {
    const uint64_t cells = uint64_t(L.width) * L.rows * L.band_count;
    const uint32_t block = 256;
    const uint64_t blocks = (cells * 32u + block - 1) / block;
    if (blocks > 0x7fffffffull) return cudaErrorInvalidConfiguration;
    const dim3 grid(static_cast<uint32_t>(blocks));
    const uint32_t acc = accumulate ? 1u : 0u;
#define SKY_PLAIN_CASE(TR, PH)                                                                                   \
    if (L.tracking == TR && L.phase_sampling == PH) {                                                            \
        if (aerosol_species == 1u)                                                                               \
            trace_plain_kernel<TR, PH, 1><<<grid, block, 0, stream>>>(S, L, cell_sum, cell_sumsq, counters,      \
                                                                      status, cells, acc);                       \
        else                                                                                                     \
            trace_plain_kernel<TR, PH, int(kSpecies)><<<grid, block, 0, stream>>>(S, L, cell_sum, cell_sumsq,    \
                                                                                  counters, status, cells, acc); \
        return cudaGetLastError();                                                                               \
    }
    SKY_PLAIN_CASE(SKY_TRACKING_SEGMENT_RESTART, SKY_PHASE_ISOTROPIC)
    SKY_PLAIN_CASE(SKY_TRACKING_SEGMENT_RESTART, SKY_PHASE_TABULATED)
    SKY_PLAIN_CASE(SKY_TRACKING_RESIDUAL_CARRY, SKY_PHASE_ISOTROPIC)
    SKY_PLAIN_CASE(SKY_TRACKING_RESIDUAL_CARRY, SKY_PHASE_TABULATED)
    SKY_PLAIN_CASE(SKY_TRACKING_MERGED_LAYERS, SKY_PHASE_ISOTROPIC)
    SKY_PLAIN_CASE(SKY_TRACKING_MERGED_LAYERS, SKY_PHASE_TABULATED)
#undef SKY_PLAIN_CASE
    return cudaErrorInvalidValue;
}

}  // namespace sky
