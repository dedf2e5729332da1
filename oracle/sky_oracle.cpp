// sky_oracle.cpp — CPU ORACLE for the spectral sky path tracer.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle the tests compare with and
// the timed CPU baseline; the product (libsky_cuda.so) never links, loads or
// calls it.  Only tests/, __graft_entry__.smoke() and bench.py's CPU legs may
// use it.
//
// What it is: a scalar single-precision restatement of the reference's WGSL
// path tracer (crates/sky-spectral-path-tracer/src/sky_trace.wgsl:156-816),
// function by function, in the shader's own evaluation order, plus the
// sky-core pieces that prepare its inputs: the majorant-grid bake
// (crates/sky-core/src/medium.rs:28-159) and the phase-table CDF
// (crates/sky-core/src/phase.rs:37-146).  Each function cites the lines it
// follows.  Compiled with -ffp-contract=off so that no FMA contraction
// changes the shader's rounding.
//
// Extensions beyond the shader (run-time band count, bin count, ground
// albedo, Russian-roulette start depth, order truncation and tabulated
// phase sampling) are off when the matching SkyRenderConfig fields are zero,
// and then the oracle executes exactly the shader's algorithm.
//
// Parity status: the reference's tracer runs only through wgpu and no
// graphics API exists on these machines, so no reference image exists to pin
// the oracle's radiance ("image-level parity unpinned by the reference").
// The oracle is pinned instead by the reference's own known-answer tests for
// the pieces it restates (geometry.rs:101-117, phase.rs:155-169,
// sampling.rs:269-274, data.rs:253-276, spectrum.rs:375-382) and by analytic
// known answers (vacuum, ground-only and single-scattering integrals) in
// tests/.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "../include/sky_cuda.h"

namespace {

constexpr uint32_t kSpecies = SKY_SPECIES_COUNT;
constexpr float PI = 3.14159265358979323846f;
constexpr float INV_PI = 0.31830988618379067154f;
constexpr float TAU = 6.28318530717958647692f;
constexpr float RAY_EPSILON_KM = 0.005f;           // sky_trace.wgsl:8
constexpr float ISOTROPIC_PDF = 0.07957747154594766788f;
constexpr float SKY_VIEW_SKY_FRACTION = 0.75f;     // sky_trace.wgsl:13-14
constexpr float SKY_VIEW_GROUND_FRACTION = 0.25f;
constexpr float F32_EPSILON = 1.1920929e-7f;

struct V3 {
    float x, y, z;
};
inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
inline V3 operator*(float s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
inline V3 operator/(V3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float length(V3 a) { return std::sqrt(dot(a, a)); }
inline V3 cross(V3 a, V3 b) {
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline V3 normalize(V3 a) { return a / length(a); }
inline float clampf(float x, float lo, float hi) { return std::min(std::max(x, lo), hi); }

// ---- RNG: sky_trace.wgsl:156-189 -----------------------------------------

struct U4 {
    uint32_t x, y, z, w;
};

inline U4 pcg4d(U4 v) {  // sky_trace.wgsl:156-168
    v.x = v.x * 1664525u + 1013904223u;
    v.y = v.y * 1664525u + 1013904223u;
    v.z = v.z * 1664525u + 1013904223u;
    v.w = v.w * 1664525u + 1013904223u;
    v.x = v.x + v.y * v.w;
    v.y = v.y + v.z * v.x;
    v.z = v.z + v.x * v.y;
    v.w = v.w + v.y * v.z;
    v.x ^= v.x >> 16u;
    v.y ^= v.y >> 16u;
    v.z ^= v.z >> 16u;
    v.w ^= v.w >> 16u;
    v.x = v.x + v.y * v.w;
    v.y = v.y + v.z * v.x;
    v.z = v.z + v.x * v.y;
    v.w = v.w + v.y * v.z;
    return v;
}

struct Rng {  // sky_trace.wgsl:134-139, make_rng :170-172
    uint32_t pixel, sample, band, dimension;
    uint32_t seed_lo, seed_hi;
};

inline uint32_t rng_next_u32(Rng& r) {  // sky_trace.wgsl:174-184
    U4 c{r.pixel ^ r.seed_lo, r.sample ^ r.seed_hi, r.band, r.dimension};
    r.dimension += 1u;
    U4 v = pcg4d(c);
    return v.x ^ v.y ^ v.z ^ v.w;
}

inline float rng_f32(Rng& r) {  // sky_trace.wgsl:186-189
    uint32_t value = rng_next_u32(r) >> 8u;
    return float(value) * 0.000000059604644775390625f;
}

// ---- Scene / constants ----------------------------------------------------

struct Coeffs {  // MediumCoefficients, sky_trace.wgsl:101-106
    float rayleigh;
    float sca[kSpecies];
    float abs[kSpecies];
    float ozone;
};

struct Ray {
    V3 origin, dir;
};

struct Ctx {
    const SkySceneDesc* s;
    uint32_t width, height, spp, direct_light_samples, sample_offset;
    uint32_t atmosphere_len, aerosol_len, majorant_layers, phase_bins, band_count;
    uint32_t seed_lo, seed_hi, watchdog_limit, output_projection;
    uint32_t phase_sampling, rr_start_depth, max_orders, tracking;
    float observer_altitude_km, ground_radius_km, atmosphere_radius_km, top_altitude_km;
    V3 sun;
    float sun_angular_radius_rad, ground_albedo;
    std::vector<float> cdf, bin_pdf;  // phase.rs:105-126 layout [species][band][bin]
    // merged tracking grid (tracking mode 2): per band, merged-layer bounds
    // (altitudes of the first uniform layer of each group, then top), majorant
    // of each group, and the group of every uniform layer
    std::vector<std::vector<float>> merged_lo, merged_maj;
    std::vector<std::vector<uint32_t>> merged_of;
};

// Grouping of uniform majorant layers for tracking mode 2: contiguous groups
// minimising sum_groups [0.1 + dz * sum_k (max_group - maj_k)] (the cost of a
// layer crossing against the expected extra null collisions of a vertical ray;
// 0.1 is the CUDA library's default crossing cost).
std::vector<uint32_t> merge_groups(const float* maj, uint32_t L, float dz) {
    std::vector<double> best(L + 1, 0.0);
    std::vector<uint32_t> from(L + 1, 0);
    for (uint32_t j = 1; j <= L; ++j) {
        best[j] = 1e300;
        double mx = 0.0, sum = 0.0;
        for (uint32_t i = j; i-- > 0;) {
            double m = std::max(double(maj[i]), 1e-8);
            mx = std::max(mx, m);
            sum += m;
            double c = best[i] + 0.1 + (mx * double(j - i) - sum) * double(dz);
            if (c < best[j]) {
                best[j] = c;
                from[j] = i;
            }
        }
    }
    std::vector<uint32_t> starts;
    for (uint32_t j = L; j > 0; j = from[j]) starts.push_back(from[j]);
    std::reverse(starts.begin(), starts.end());
    return starts;
}

// ---- phase.rs sampling tables: phase.rs:105-146 ----------------------------

inline float mu_edge(uint32_t edge, uint32_t bins) {  // phase.rs:137-140
    float u = float(edge) / float(bins);
    return 1.0f - 2.0f * u * u * u;
}

void build_sampling_tables(const float* values, uint32_t band_count, uint32_t bins,
                           std::vector<float>& cdf, std::vector<float>& bin_pdf) {
    size_t n = size_t(kSpecies) * band_count * bins;
    cdf.assign(n, 0.0f);
    bin_pdf.assign(n, 0.0f);
    for (uint32_t species = 0; species < kSpecies; ++species) {
        for (uint32_t band = 0; band < band_count; ++band) {
            size_t base = (size_t(species) * band_count + band) * bins;
            float norm = 0.0f;  // phase_norm, phase.rs:128-135
            for (uint32_t bin = 0; bin < bins; ++bin) {
                float delta_mu = std::fabs(mu_edge(bin, bins) - mu_edge(bin + 1, bins));
                norm += 2.0f * PI * std::max(values[base + bin], 0.0f) * delta_mu;
            }
            norm = std::max(norm, 1.0e-20f);
            float cumulative = 0.0f;
            for (uint32_t bin = 0; bin < bins; ++bin) {
                float value = std::max(values[base + bin], 0.0f);
                float delta_mu = std::fabs(mu_edge(bin, bins) - mu_edge(bin + 1, bins));
                cumulative += 2.0f * PI * value * delta_mu / norm;
                cdf[base + bin] = std::min(cumulative, 1.0f);
                bin_pdf[base + bin] = value / norm;
            }
            cdf[base + bins - 1] = 1.0f;
        }
    }
}

// ---- geometry: sky_trace.wgsl:191-294 --------------------------------------

inline V3 normalize_or_y(V3 v) {  // :191-197
    float len = length(v);
    if (len > 0.0f) return v / len;
    return v3(0.0f, 1.0f, 0.0f);
}
inline V3 ray_at(const Ray& r, float t) { return r.origin + r.dir * t; }  // :199-201
inline float altitude_km(const Ctx& c, V3 p) { return length(p) - c.ground_radius_km; }

struct SphereHit {
    bool hit;
    float t0, t1;
};
inline SphereHit intersect_sphere(const Ray& ray, float radius) {  // :211-221
    float b = dot(ray.origin, ray.dir);
    float origin_radius = length(ray.origin);
    float c = (origin_radius - radius) * (origin_radius + radius);
    float discriminant = b * b - c;
    if (discriminant < 0.0f) return SphereHit{false, 0.0f, 0.0f};
    float s = std::sqrt(discriminant);
    return SphereHit{true, -b - s, -b + s};
}
inline float positive_root(float t0, float t1) {  // :223-231
    if (t0 > RAY_EPSILON_KM) return t0;
    if (t1 > RAY_EPSILON_KM) return t1;
    return -1.0f;
}
struct BoundaryHit {
    bool hit;
    float t;
    uint32_t kind;  // 0 ground, 1 atmosphere exit
};
inline BoundaryHit next_boundary(const Ctx& c, const Ray& ray) {  // :233-250
    SphereHit atmosphere_hit = intersect_sphere(ray, c.atmosphere_radius_km);
    if (!atmosphere_hit.hit) return BoundaryHit{false, 0.0f, 0u};
    SphereHit ground_hit = intersect_sphere(ray, c.ground_radius_km);
    float t_ground = -1.0f;
    if (ground_hit.hit) t_ground = positive_root(ground_hit.t0, ground_hit.t1);
    float t_exit = std::max(atmosphere_hit.t1, RAY_EPSILON_KM);
    if (t_ground > RAY_EPSILON_KM && t_ground < t_exit) return BoundaryHit{true, t_ground, 0u};
    return BoundaryHit{true, t_exit, 1u};
}
inline uint32_t layer_for_altitude(const Ctx& c, float altitude) {  // :252-257
    float top = std::max(c.top_altitude_km, 0.000001f);
    float clamped = clampf(altitude, 0.0f, top - 0.000001f);
    uint32_t layer = uint32_t(std::floor(clamped / top * float(c.majorant_layers)));
    return std::min(layer, c.majorant_layers - 1u);
}
inline float majorant_for_layer(const Ctx& c, uint32_t band, uint32_t layer) {  // :259-261
    return std::max(c.s->majorants_km_inv[band * c.majorant_layers + layer], 0.00000001f);
}
inline float boundary_candidate(const Ctx& c, const Ray& ray, float t, float current_next,
                                float altitude_boundary) {  // :263-282
    if (altitude_boundary <= 0.0f || altitude_boundary >= c.top_altitude_km) return current_next;
    float radius = c.ground_radius_km + altitude_boundary;
    SphereHit hit = intersect_sphere(ray, radius);
    if (!hit.hit) return current_next;
    float next_t = current_next;
    if (hit.t0 > t + RAY_EPSILON_KM && hit.t0 < next_t) next_t = hit.t0;
    if (hit.t1 > t + RAY_EPSILON_KM && hit.t1 < next_t) next_t = hit.t1;
    return next_t;
}
inline float next_majorant_segment_end(const Ctx& c, const Ray& ray, float t,
                                       float t_max) {  // :284-294
    float probe_t = std::min(t + RAY_EPSILON_KM, t_max);
    uint32_t layer = layer_for_altitude(c, altitude_km(c, ray_at(ray, probe_t)));
    float dz = c.top_altitude_km / float(c.majorant_layers);
    float lo = float(layer) * dz;
    float hi = float(layer + 1u) * dz;
    float next_t = t_max;
    next_t = boundary_candidate(c, ray, t, next_t, lo);
    next_t = boundary_candidate(c, ray, t, next_t, hi);
    return next_t;
}

// Altitude of ray_at(ray, t) evaluated in double precision.  The reference's
// f32 probe (next_majorant_segment_end, sky_trace.wgsl:284-294) resolves
// altitude to ~0.5 m at Earth radius, while a ray descending at less than
// ~6 degrees drops less than that in RAY_EPSILON_KM: at a downward shell
// crossing the f32 probe still reads the upper layer, and the segment then
// runs past the tangent point under the upper layer's majorant (optical depth
// skipped; see tests/test_oracle.py::test_transmittance_on_descending_rays).
// Tracking modes 0 and 1 keep the reference's probe, defect included, since
// they restate the reference; mode 2, an extension, probes exactly.
inline double altitude_exact(const Ctx& c, const Ray& ray, float t) {
    const double x = double(ray.origin.x) + double(ray.dir.x) * double(t);
    const double y = double(ray.origin.y) + double(ray.dir.y) * double(t);
    const double z = double(ray.origin.z) + double(ray.dir.z) * double(t);
    return std::sqrt(x * x + y * y + z * z) - double(c.ground_radius_km);
}
inline uint32_t layer_for_altitude_exact(const Ctx& c, double altitude) {
    const double top = std::max(double(c.top_altitude_km), 0.000001);
    const double clamped = std::min(std::max(altitude, 0.0), top - 0.000001);
    return std::min(uint32_t(std::floor(clamped / top * double(c.majorant_layers))), c.majorant_layers - 1u);
}

// Tracking mode 2: the next segment end over the merged grid with the
// reference's candidate rule (both roots of both shells of the current merged
// layer beyond t + epsilon), the layer taken from an exact probe at t + epsilon.
inline float merged_segment_end(const Ctx& c, const Ray& ray, uint32_t band, float t, float t_max, float& majorant) {
    float probe_t = std::min(t + RAY_EPSILON_KM, t_max);
    uint32_t k = layer_for_altitude_exact(c, altitude_exact(c, ray, probe_t));
    uint32_t g = c.merged_of[band][k];
    float next_t = t_max;
    next_t = boundary_candidate(c, ray, t, next_t, c.merged_lo[band][g]);
    next_t = boundary_candidate(c, ray, t, next_t, c.merged_lo[band][g + 1]);
    float probe2 = std::min(t + RAY_EPSILON_KM, next_t);
    uint32_t k2 = layer_for_altitude_exact(c, altitude_exact(c, ray, probe2));
    majorant = c.merged_maj[band][c.merged_of[band][k2]];
    return next_t;
}

// ---- medium: sky_trace.wgsl:296-403 ----------------------------------------

inline float lerp(float a, float b, float t) { return a * (1.0f - t) + b * t; }  // :296-298

struct AtmSample {
    float temperature_k, air_cm3, ozone_cm3;
};
inline AtmSample interpolate_atmosphere(const Ctx& c, float altitude) {  // :300-327
    const SkyAtmospherePoint* p = c.s->atmosphere;
    uint32_t hi = 0;
    while (!(hi >= c.atmosphere_len || p[hi].altitude_km >= altitude)) hi++;
    if (hi == 0u) return AtmSample{p[0].temperature_k, p[0].air_cm3, p[0].ozone_cm3};
    if (hi >= c.atmosphere_len) {
        const SkyAtmospherePoint& q = p[c.atmosphere_len - 1];
        return AtmSample{q.temperature_k, q.air_cm3, q.ozone_cm3};
    }
    const SkyAtmospherePoint& lo = p[hi - 1];
    const SkyAtmospherePoint& high = p[hi];
    float denom = std::max(high.altitude_km - lo.altitude_km, 0.000001f);
    float t = clampf((altitude - lo.altitude_km) / denom, 0.0f, 1.0f);
    return AtmSample{lerp(lo.temperature_k, high.temperature_k, t), lerp(lo.air_cm3, high.air_cm3, t),
                     lerp(lo.ozone_cm3, high.ozone_cm3, t)};
}
inline void interpolate_aerosol(const Ctx& c, float altitude, float mass[kSpecies]) {  // :333-354
    const SkyAerosolPoint* p = c.s->aerosol;
    uint32_t hi = 0;
    while (!(hi >= c.aerosol_len || p[hi].altitude_km >= altitude)) hi++;
    if (hi == 0u) {
        for (uint32_t i = 0; i < kSpecies; ++i) mass[i] = p[0].mass_g_m3[i];
        return;
    }
    if (hi >= c.aerosol_len) {
        for (uint32_t i = 0; i < kSpecies; ++i) mass[i] = p[c.aerosol_len - 1].mass_g_m3[i];
        return;
    }
    const SkyAerosolPoint& lo = p[hi - 1];
    const SkyAerosolPoint& high = p[hi];
    float denom = std::max(high.altitude_km - lo.altitude_km, 0.000001f);
    float t = clampf((altitude - lo.altitude_km) / denom, 0.0f, 1.0f);
    for (uint32_t i = 0; i < kSpecies; ++i)
        mass[i] = std::max(lo.mass_g_m3[i] * (1.0f - t) + high.mass_g_m3[i] * t, 0.0f);
}
inline Coeffs coefficients_at(const Ctx& c, V3 position, uint32_t band) {  // :356-386
    Coeffs k{};
    float altitude = altitude_km(c, position);
    if (altitude < 0.0f || altitude > c.top_altitude_km) return k;
    AtmSample atm = interpolate_atmosphere(c, altitude);
    float mass[kSpecies];
    interpolate_aerosol(c, altitude, mass);
    const SkyBand& b = c.s->bands[band];
    for (uint32_t i = 0; i < kSpecies; ++i) {
        const SkyAerosolOptics& o = c.s->aerosol_optics[band * kSpecies + i];
        k.sca[i] = std::max(mass[i] * o.scattering_km_inv_per_g_m3, 0.0f);
        k.abs[i] = std::max(mass[i] * o.absorption_km_inv_per_g_m3, 0.0f);
    }
    k.rayleigh = std::max(atm.air_cm3 * b.rayleigh_cross_section_m2 * 1000000000.0f, 0.0f);
    k.ozone = std::max(atm.ozone_cm3 * b.ozone_cross_section_cm2 * 100000.0f, 0.0f);
    return k;
}
inline float scattering_total(const Coeffs& k) {  // :388-394
    return k.rayleigh + k.sca[0] + k.sca[1] + k.sca[2] + k.sca[3];
}
inline float extinction_total(const Coeffs& k) {  // :396-403
    return scattering_total(k) + k.ozone + k.abs[0] + k.abs[1] + k.abs[2] + k.abs[3];
}

struct Counters {
    uint64_t e[SKY_EVENT_COUNT] = {};
};

struct CollisionSample {
    bool hit;
    float t;
    Coeffs coeffs;
};

// sky_trace.wgsl:405-439.  With SKY_TRACKING_RESIDUAL_CARRY the exponential
// optical depth left over at a segment end is carried into the next segment
// (same collision distribution by memorylessness, fewer draws).
CollisionSample sample_real_collision(const Ctx& c, const Ray& ray, float t_max, uint32_t band,
                                      Rng& rng, bool& watchdog, Counters& n) {
    float t = 0.0f;
    uint32_t guard = 0;
    float tau = 0.0f;        // residual optical depth (SKY_TRACKING_RESIDUAL_CARRY)
    bool need_draw = true;
    for (;;) {
        if (t >= t_max) return CollisionSample{false, 0.0f, Coeffs{}};
        if (guard > 100000u) {
            watchdog = true;
            return CollisionSample{false, 0.0f, Coeffs{}};
        }
        guard++;
        float segment_end, majorant;
        if (c.tracking == SKY_TRACKING_MERGED_LAYERS) {
            segment_end = merged_segment_end(c, ray, band, t, t_max, majorant);
        } else {
            segment_end = next_majorant_segment_end(c, ray, t, t_max);
            uint32_t layer = layer_for_altitude(
                c, altitude_km(c, ray_at(ray, std::min(t + RAY_EPSILON_KM, segment_end))));
            majorant = majorant_for_layer(c, band, layer);
        }
        n.e[SKY_EVENT_SEGMENT]++;
        if (c.tracking != SKY_TRACKING_SEGMENT_RESTART) {
            for (;;) {
                if (need_draw) {
                    tau = -std::log(std::max(1.0f - rng_f32(rng), 0.0000001f));
                    need_draw = false;
                }
                float dt = tau / majorant;
                if (t + dt >= segment_end) {
                    tau = std::max(tau - (segment_end - t) * majorant, 0.0f);
                    break;
                }
                t = t + dt;
                need_draw = true;
                n.e[SKY_EVENT_TRACK_STEP]++;
                Coeffs coeffs = coefficients_at(c, ray_at(ray, t), band);
                float accept = clampf(extinction_total(coeffs) / majorant, 0.0f, 1.0f);
                if (rng_f32(rng) < accept) return CollisionSample{true, t, coeffs};
            }
            t = segment_end;
            continue;
        }
        for (;;) {
            if (t >= segment_end) break;
            float u = std::max(1.0f - rng_f32(rng), 0.0000001f);
            t = t - std::log(u) / majorant;
            if (t >= segment_end) break;
            n.e[SKY_EVENT_TRACK_STEP]++;
            Coeffs coeffs = coefficients_at(c, ray_at(ray, t), band);
            float accept = clampf(extinction_total(coeffs) / majorant, 0.0f, 1.0f);
            if (rng_f32(rng) < accept) return CollisionSample{true, t, coeffs};
        }
        t = segment_end;
    }
}

// sky_trace.wgsl:441-475
float delta_transmittance(const Ctx& c, const Ray& ray, float t_max, uint32_t band, Rng& rng,
                          bool& watchdog, Counters& n) {
    float t = 0.0f;
    uint32_t guard = 0;
    float tau = 0.0f;
    bool need_draw = true;
    for (;;) {
        if (t >= t_max) return 1.0f;
        if (guard > 100000u) {
            watchdog = true;
            return 0.0f;
        }
        guard++;
        float segment_end, majorant;
        if (c.tracking == SKY_TRACKING_MERGED_LAYERS) {
            segment_end = merged_segment_end(c, ray, band, t, t_max, majorant);
        } else {
            segment_end = next_majorant_segment_end(c, ray, t, t_max);
            uint32_t layer = layer_for_altitude(
                c, altitude_km(c, ray_at(ray, std::min(t + RAY_EPSILON_KM, segment_end))));
            majorant = majorant_for_layer(c, band, layer);
        }
        n.e[SKY_EVENT_SEGMENT]++;
        if (c.tracking != SKY_TRACKING_SEGMENT_RESTART) {
            for (;;) {
                if (need_draw) {
                    tau = -std::log(std::max(1.0f - rng_f32(rng), 0.0000001f));
                    need_draw = false;
                }
                float dt = tau / majorant;
                if (t + dt >= segment_end) {
                    tau = std::max(tau - (segment_end - t) * majorant, 0.0f);
                    break;
                }
                t = t + dt;
                need_draw = true;
                n.e[SKY_EVENT_TRACK_STEP]++;
                Coeffs coeffs = coefficients_at(c, ray_at(ray, t), band);
                float accept = clampf(extinction_total(coeffs) / majorant, 0.0f, 1.0f);
                if (rng_f32(rng) < accept) return 0.0f;
            }
            t = segment_end;
            continue;
        }
        for (;;) {
            if (t >= segment_end) break;
            float u = std::max(1.0f - rng_f32(rng), 0.0000001f);
            t = t - std::log(u) / majorant;
            if (t >= segment_end) break;
            n.e[SKY_EVENT_TRACK_STEP]++;
            Coeffs coeffs = coefficients_at(c, ray_at(ray, t), band);
            float accept = clampf(extinction_total(coeffs) / majorant, 0.0f, 1.0f);
            if (rng_f32(rng) < accept) return 0.0f;
        }
        t = segment_end;
    }
}

// ---- phase: sky_trace.wgsl:477-510, phase.rs:37-75 --------------------------

inline float rayleigh_phase(float mu) { return 3.0f / (16.0f * PI) * (1.0f + mu * mu); }  // :477-479

inline float mie_phase(const Ctx& c, uint32_t species, uint32_t band, float mu) {  // :485-494
    uint32_t bins = c.phase_bins;
    float u = std::pow((1.0f - clampf(mu, -1.0f, 1.0f)) * 0.5f, 0.3333333333333333f);
    float f = u * float(bins) - 0.5f;
    uint32_t i0 = std::min(uint32_t(clampf(std::floor(f), 0.0f, float(bins - 1u))), bins - 1u);
    uint32_t i1 = std::min(i0 + 1u, bins - 1u);
    float t = clampf(f - float(i0), 0.0f, 1.0f);
    size_t base = (size_t(species) * c.band_count + band) * bins;  // phase_index :481-483
    float p0 = c.s->phase_values[base + i0];
    float p1 = c.s->phase_values[base + i1];
    return std::max(lerp(p0, p1, t), 0.0f);
}

inline float mixed_phase_value(const Ctx& c, const Coeffs& k, uint32_t band, float mu) {  // :496-510
    float scattering = scattering_total(k);
    if (scattering <= 0.0f) return 0.0f;
    float phase = 0.0f;
    float rayleigh_weight = k.rayleigh / scattering;
    phase = phase + rayleigh_weight * rayleigh_phase(mu);
    for (uint32_t i = 0; i < kSpecies; ++i)
        phase = phase + k.sca[i] / scattering * mie_phase(c, i, band, mu);
    return phase;
}

// phase.rs:53-69 (MiePhaseTable::sample_mu_pdf)
inline float sample_mu(const Ctx& c, uint32_t species, uint32_t band, float xi) {
    uint32_t bins = c.phase_bins;
    size_t base = (size_t(species) * c.band_count + band) * bins;
    const float* cdf = c.cdf.data() + base;
    xi = clampf(xi, 0.0f, 1.0f - F32_EPSILON);
    uint32_t bin = uint32_t(std::upper_bound(cdf, cdf + bins, xi) - cdf);  // partition_point(<= xi)
    bin = std::min(bin, bins - 1u);
    float prev = bin == 0 ? 0.0f : cdf[bin - 1];
    float next = cdf[bin];
    float t = next > prev ? (xi - prev) / (next - prev) : 0.5f;
    return lerp(mu_edge(bin, bins), mu_edge(bin + 1, bins), t);
}

// phase.rs:71-75 (sampling_pdf) with mu_to_bin phase.rs:142-146
inline float sampling_pdf(const Ctx& c, uint32_t species, uint32_t band, float mu) {
    uint32_t bins = c.phase_bins;
    float u = std::cbrt((1.0f - clampf(mu, -1.0f, 1.0f)) * 0.5f);
    uint32_t bin = std::min(uint32_t(std::floor(u * float(bins))), bins - 1u);
    size_t base = (size_t(species) * c.band_count + band) * bins;
    return std::max(c.bin_pdf[base + bin], 1.0e-12f);
}

// sampling.rs:182-185
inline float invert_rayleigh_cdf(float xi) {
    float y = 4.0f * clampf(xi, 0.0f, 1.0f) - 2.0f;
    return clampf(2.0f * std::sinh(std::asinh(y) / 3.0f), -1.0f, 1.0f);
}

// ---- directions: sky_trace.wgsl:512-564 -------------------------------------

struct Basis {
    V3 tangent, bitangent;
};
inline Basis orthonormal_basis(V3 n_in) {  // :512-520
    V3 n = normalize_or_y(n_in);
    float sign = n.z >= 0.0f ? 1.0f : -1.0f;
    float a = -1.0f / (sign + n.z);
    float b = n.x * n.y * a;
    V3 tangent = normalize_or_y(v3(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x));
    V3 bitangent = normalize_or_y(v3(b, sign + n.y * n.y * a, -n.y));
    return Basis{tangent, bitangent};
}
inline V3 direction_from_axis_mu(V3 axis, float mu_in, float xi_phi) {  // :522-532
    float mu = clampf(mu_in, -1.0f, 1.0f);
    float sin_theta = std::sqrt(std::max(1.0f - mu * mu, 0.0f));
    float phi = TAU * xi_phi;
    Basis basis = orthonormal_basis(axis);
    return normalize_or_y(basis.tangent * (sin_theta * std::cos(phi)) +
                          basis.bitangent * (sin_theta * std::sin(phi)) + normalize_or_y(axis) * mu);
}
struct DirPdf {
    V3 dir;
    float pdf;
};
inline DirPdf sample_isotropic(Rng& rng) {  // :534-539
    float z = 1.0f - 2.0f * rng_f32(rng);
    float r = std::sqrt(std::max(1.0f - z * z, 0.0f));
    float phi = TAU * rng_f32(rng);
    return DirPdf{v3(r * std::cos(phi), z, r * std::sin(phi)), ISOTROPIC_PDF};
}
inline DirPdf sample_uniform_cone(V3 axis, float angular_radius, Rng& rng) {  // :541-546
    float cos_max = std::cos(angular_radius);
    float cos_theta = 1.0f - clampf(rng_f32(rng), 0.0f, 0.99999994f) * (1.0f - cos_max);
    float pdf = 1.0f / (TAU * (1.0f - cos_max));
    float xi_phi = rng_f32(rng);
    return DirPdf{direction_from_axis_mu(axis, cos_theta, xi_phi), pdf};
}
inline DirPdf sample_cosine_hemisphere(V3 axis, Rng& rng) {  // :548-560
    float u = rng_f32(rng);
    float r = std::sqrt(u);
    float phi = TAU * rng_f32(rng);
    float cos_theta = std::sqrt(std::max(1.0f - u, 0.0f));
    Basis basis = orthonormal_basis(axis);
    V3 dir = normalize_or_y(basis.tangent * (r * std::cos(phi)) + basis.bitangent * (r * std::sin(phi)) +
                            normalize_or_y(axis) * cos_theta);
    return DirPdf{dir, std::max(dot(normalize_or_y(axis), dir), 0.0f) * INV_PI};
}
inline bool direction_in_cone(V3 dir, V3 axis, float angular_radius) {  // :562-564
    return dot(normalize_or_y(dir), normalize_or_y(axis)) >= std::cos(angular_radius);
}
inline V3 sun_dir(const Ctx& c) { return normalize_or_y(c.sun); }  // :207-209

// ---- light transport: sky_trace.wgsl:566-608 --------------------------------

float direct_sun_at_scatter(const Ctx& c, V3 pos, V3 view_dir, uint32_t band, const Coeffs& k,
                            Rng& rng, bool& watchdog, Counters& n) {  // :566-585
    float sum = 0.0f;
    for (uint32_t sample = 0; sample < c.direct_light_samples; ++sample) {
        DirPdf light = sample_uniform_cone(sun_dir(c), c.sun_angular_radius_rad, rng);
        n.e[SKY_EVENT_NEE]++;
        Ray shadow{pos + light.dir * RAY_EPSILON_KM, light.dir};
        BoundaryHit boundary = next_boundary(c, shadow);
        n.e[SKY_EVENT_BOUNDARY]++;
        if (boundary.hit && boundary.kind == 1u) {
            float trans = delta_transmittance(c, shadow, boundary.t, band, rng, watchdog, n);
            float mu = dot(view_dir, light.dir);
            float phase = mixed_phase_value(c, k, band, mu);
            sum = sum + c.s->bands[band].solar_radiance_w_m2_sr * trans * phase / light.pdf;
        }
    }
    return sum / float(c.direct_light_samples);
}

float ground_radiance(const Ctx& c, V3 pos, uint32_t band, Rng& rng, bool& watchdog,
                      Counters& n) {  // :587-608
    V3 normal = normalize_or_y(pos);
    float sum = 0.0f;
    for (uint32_t sample = 0; sample < c.direct_light_samples; ++sample) {
        DirPdf light = sample_uniform_cone(sun_dir(c), c.sun_angular_radius_rad, rng);
        n.e[SKY_EVENT_NEE]++;
        float cos_sun = std::max(dot(normal, light.dir), 0.0f);
        if (cos_sun > 0.0f) {
            Ray shadow{pos + light.dir * RAY_EPSILON_KM, light.dir};
            BoundaryHit boundary = next_boundary(c, shadow);
            n.e[SKY_EVENT_BOUNDARY]++;
            if (boundary.hit && boundary.kind == 1u) {
                float trans = delta_transmittance(c, shadow, boundary.t, band, rng, watchdog, n);
                sum = sum + c.ground_albedo * INV_PI * c.s->bands[band].solar_radiance_w_m2_sr * trans *
                                cos_sun / light.pdf;
            }
        }
    }
    return sum / float(c.direct_light_samples);
}

// ---- cameras: sky_trace.wgsl:610-689 ----------------------------------------

inline V3 observer_origin(const Ctx& c) {  // :610-612
    return v3(0.0f, c.ground_radius_km + std::max(c.observer_altitude_km, 0.0f), 0.0f);
}
inline V3 panorama_dir(float u, float v) {  // :614-623
    float azimuth = (u - 0.5f) * TAU;
    float elevation = (0.5f - v) * PI;
    float cos_e = std::cos(elevation);
    return normalize_or_y(v3(cos_e * std::sin(azimuth), std::sin(elevation), cos_e * std::cos(azimuth)));
}
inline float from_sub_uvs_to_unit(float u, float resolution) {  // :625-630
    if (resolution <= 1.0f) return 0.5f;
    return (u - 0.5f / resolution) * (resolution / (resolution - 1.0f));
}
inline V3 sky_view_lut_dir(const Ctx& c, float u_in, float v_in) {  // :632-681
    float ux = clampf(from_sub_uvs_to_unit(u_in, float(c.width)), 0.0f, 1.0f);
    float uy = clampf(from_sub_uvs_to_unit(v_in, float(c.height)), 0.0f, 1.0f);
    float view_height = length(observer_origin(c));
    float bottom = c.ground_radius_km;
    float v_horizon = std::sqrt(std::max(view_height * view_height - bottom * bottom, 0.0f));
    float cos_beta = clampf(v_horizon / std::max(view_height, 0.000001f), 0.0f, 1.0f);
    float beta = std::acos(cos_beta);
    float zenith_horizon_angle = PI - beta;
    float view_zenith_cos_angle;
    if (uy < SKY_VIEW_SKY_FRACTION) {
        float coord = uy / SKY_VIEW_SKY_FRACTION;
        coord = 1.0f - coord;
        coord = coord * coord;
        coord = 1.0f - coord;
        view_zenith_cos_angle = std::cos(zenith_horizon_angle * coord);
    } else {
        float coord = (uy - SKY_VIEW_SKY_FRACTION) / SKY_VIEW_GROUND_FRACTION;
        coord = coord * coord;
        view_zenith_cos_angle = std::cos(zenith_horizon_angle + beta * coord);
    }
    float coord = ux;
    coord = coord * coord;
    float light_view_cos_angle = -(coord * 2.0f - 1.0f);
    V3 up = v3(0.0f, 1.0f, 0.0f);
    V3 sun_h = sun_dir(c) - up * dot(sun_dir(c), up);
    float sun_h_len = length(sun_h);
    V3 forward = sun_h / std::max(sun_h_len, 0.00001f);
    V3 forward_safe = sun_h_len > 0.00001f ? forward : v3(1.0f, 0.0f, 0.0f);
    V3 side = normalize(cross(up, forward_safe));
    float sin_view = std::sqrt(std::max(1.0f - view_zenith_cos_angle * view_zenith_cos_angle, 0.0f));
    float side_scale = std::sqrt(std::max(1.0f - light_view_cos_angle * light_view_cos_angle, 0.0f));
    return normalize_or_y(up * view_zenith_cos_angle +
                          sin_view * (forward_safe * light_view_cos_angle + side * side_scale));
}
inline Ray camera_ray(const Ctx& c, float u, float v) {  // :683-689
    V3 origin = observer_origin(c);
    if (c.output_projection == SKY_PROJECTION_SKY_VIEW_LUT) return Ray{origin, sky_view_lut_dir(c, u, v)};
    return Ray{origin, panorama_dir(u, v)};
}

// ---- path: sky_trace.wgsl:691-776 -------------------------------------------

inline bool russian_roulette(const Ctx& c, float& throughput, uint32_t depth, Rng& rng) {  // :691-701
    if (depth < c.rr_start_depth) return true;
    float q = clampf(throughput, 0.05f, 0.95f);
    if (rng_f32(rng) > q) return false;
    throughput = throughput / q;
    return true;
}

// Tabulated continuation direction (extension; semantics of phase.rs:53-75
// and sampling.rs:182-185): component chosen by sigma_s,i / sigma_s, then
// mu from that component's inverse CDF, then phi.  Returns the weight
// mixed_phase(mu) / mixture_pdf(mu).
inline float sample_tabulated_direction(const Ctx& c, const Coeffs& k, uint32_t band, V3 axis, Rng& rng,
                                        V3& out_dir) {
    float scattering = scattering_total(k);
    float comp[1 + kSpecies] = {k.rayleigh, k.sca[0], k.sca[1], k.sca[2], k.sca[3]};
    float target = rng_f32(rng) * scattering;
    int chosen = -1;
    float acc = 0.0f;
    for (int i = 0; i < int(1 + kSpecies); ++i) {
        acc = acc + comp[i];
        if (target < acc) {
            chosen = i;
            break;
        }
    }
    if (chosen < 0) {
        for (int i = int(kSpecies); i >= 0; --i)
            if (comp[i] > 0.0f) {
                chosen = i;
                break;
            }
    }
    float xi_mu = rng_f32(rng);
    float mu = chosen == 0 ? invert_rayleigh_cdf(xi_mu) : sample_mu(c, uint32_t(chosen - 1), band, xi_mu);
    float xi_phi = rng_f32(rng);
    out_dir = direction_from_axis_mu(axis, mu, xi_phi);
    float pdf = k.rayleigh / scattering * rayleigh_phase(mu);
    for (uint32_t i = 0; i < kSpecies; ++i)
        if (k.sca[i] > 0.0f) pdf = pdf + k.sca[i] / scattering * sampling_pdf(c, i, band, mu);
    float phase = mixed_phase_value(c, k, band, mu);
    return phase / pdf;
}

struct TraceResult {
    float radiance;
    bool watchdog;
};

TraceResult trace_path(const Ctx& c, Ray ray, uint32_t band, Rng& rng, Counters& n) {  // :703-776
    float throughput = 1.0f;
    float radiance = 0.0f;
    uint32_t depth = 0;
    bool wd = false;
    for (;;) {
        if (depth >= c.watchdog_limit) return TraceResult{radiance, true};
        if (c.max_orders != 0u && depth >= c.max_orders) break;  // extension: order truncation
        BoundaryHit boundary = next_boundary(c, ray);
        n.e[SKY_EVENT_BOUNDARY]++;
        if (!boundary.hit) break;
        CollisionSample collision = sample_real_collision(c, ray, boundary.t, band, rng, wd, n);
        if (collision.hit) {
            n.e[SKY_EVENT_SCATTER]++;
            V3 pos = ray_at(ray, collision.t);
            float scattering = scattering_total(collision.coeffs);
            float extinction = extinction_total(collision.coeffs);
            if (extinction <= 0.0f || scattering <= 0.0f) break;
            throughput = throughput * clampf(scattering / extinction, 0.0f, 1.0f);
            if (throughput <= 0.0f) break;
            radiance = radiance +
                       throughput * direct_sun_at_scatter(c, pos, ray.dir, band, collision.coeffs, rng, wd, n);
            V3 new_dir;
            if (c.phase_sampling == SKY_PHASE_TABULATED) {
                float weight = sample_tabulated_direction(c, collision.coeffs, band, ray.dir, rng, new_dir);
                throughput = throughput * weight;
            } else {
                DirPdf phase_sample = sample_isotropic(rng);
                float mu = dot(ray.dir, phase_sample.dir);
                float phase = mixed_phase_value(c, collision.coeffs, band, mu);
                throughput = throughput * phase / phase_sample.pdf;
                new_dir = phase_sample.dir;
            }
            if (!russian_roulette(c, throughput, depth, rng)) break;
            ray = Ray{pos + new_dir * RAY_EPSILON_KM, new_dir};
        } else if (boundary.kind == 1u) {
            if (depth == 0u && direction_in_cone(ray.dir, sun_dir(c), c.sun_angular_radius_rad))
                radiance = radiance + throughput * c.s->bands[band].solar_radiance_w_m2_sr;
            break;
        } else {
            n.e[SKY_EVENT_GROUND]++;
            V3 pos = ray_at(ray, boundary.t);
            radiance = radiance + throughput * ground_radiance(c, pos, band, rng, wd, n);
            V3 normal = normalize_or_y(pos);
            DirPdf bounce = sample_cosine_hemisphere(normal, rng);
            float cos_out = std::max(dot(normal, bounce.dir), 0.0f);
            if (bounce.pdf <= 0.0f || cos_out <= 0.0f) break;
            throughput = throughput * c.ground_albedo * INV_PI * cos_out / bounce.pdf;
            if (!russian_roulette(c, throughput, depth, rng)) break;
            ray = Ray{pos + bounce.dir * RAY_EPSILON_KM, bounce.dir};
        }
        if (radiance < 0.0f || radiance != radiance || throughput < 0.0f || throughput != throughput)
            return TraceResult{0.0f, wd};
        depth = depth + 1u;
    }
    return TraceResult{std::max(radiance, 0.0f), wd};
}

// One (pixel, band) cell: sky_trace.wgsl:778-816, with the film's per-sample
// sum kept in FP64 together with the sum of squares.
void trace_cell(const Ctx& c, uint32_t x, uint32_t y, uint32_t band, double& sum, double& sumsq,
                bool& watchdog, Counters& n) {
    uint32_t pixel = y * c.width + x;
    sum = 0.0;
    sumsq = 0.0;
    for (uint32_t sample = 0; sample < c.spp; ++sample) {
        uint32_t sample_index = c.sample_offset + sample;
        Rng rng{pixel, sample_index, band, 0u, c.seed_lo, c.seed_hi};
        float u = (float(x) + rng_f32(rng)) / float(c.width);
        float v = (float(y) + rng_f32(rng)) / float(c.height);
        if (c.output_projection == SKY_PROJECTION_SKY_VIEW_LUT) {
            u = (float(x) + 0.5f) / float(c.width);
            v = (float(y) + 0.5f) / float(c.height);
        }
        n.e[SKY_EVENT_CHAIN]++;
        TraceResult traced = trace_path(c, camera_ray(c, u, v), band, rng, n);
        if (traced.watchdog) watchdog = true;
        double r = double(traced.radiance);
        sum += r;
        sumsq += r * r;
    }
}

bool make_ctx(const SkySceneDesc* s, const SkyRenderConfig* cfg, Ctx& c) {
    if (!s || !cfg || s->band_count == 0 || s->atmosphere_len == 0 || s->aerosol_len == 0 ||
        s->majorant_layers == 0 || s->phase_bins == 0 || cfg->width == 0 || cfg->height == 0 ||
        cfg->spp == 0)
        return false;
    c.s = s;
    c.width = cfg->width;
    c.height = cfg->height;
    c.spp = cfg->spp;
    c.direct_light_samples = std::max(cfg->direct_light_samples, 1u);
    c.sample_offset = cfg->sample_offset;
    c.atmosphere_len = s->atmosphere_len;
    c.aerosol_len = s->aerosol_len;
    c.majorant_layers = s->majorant_layers;
    c.phase_bins = s->phase_bins;
    c.band_count = s->band_count;
    c.seed_lo = uint32_t(cfg->seed);
    c.seed_hi = uint32_t(cfg->seed >> 32);
    c.watchdog_limit = cfg->watchdog_limit ? cfg->watchdog_limit : 1024u;
    c.output_projection = cfg->output_projection;
    c.phase_sampling = cfg->phase_sampling;
    c.rr_start_depth = cfg->rr_start_depth ? cfg->rr_start_depth : 4u;
    c.max_orders = cfg->max_orders;
    c.tracking = cfg->tracking;
    c.observer_altitude_km = cfg->observer_altitude_km;
    c.ground_radius_km = s->ground_radius_km;
    c.atmosphere_radius_km = s->atmosphere_radius_km;
    c.top_altitude_km = s->top_altitude_km;
    c.sun = v3(s->sun_direction[0], s->sun_direction[1], s->sun_direction[2]);
    c.sun_angular_radius_rad = s->sun_angular_radius_rad;
    c.ground_albedo = s->ground_albedo;
    if (c.phase_sampling == SKY_PHASE_TABULATED)
        build_sampling_tables(s->phase_values, s->band_count, s->phase_bins, c.cdf, c.bin_pdf);
    if (c.tracking == SKY_TRACKING_MERGED_LAYERS) {
        const uint32_t L = s->majorant_layers;
        const float dz = c.top_altitude_km / float(L);
        c.merged_lo.resize(s->band_count);
        c.merged_maj.resize(s->band_count);
        c.merged_of.resize(s->band_count);
        for (uint32_t b = 0; b < s->band_count; ++b) {
            const float* maj = s->majorants_km_inv + size_t(b) * L;
            std::vector<uint32_t> starts = merge_groups(maj, L, dz);
            c.merged_of[b].assign(L, 0);
            for (uint32_t g = 0; g < starts.size(); ++g) {
                uint32_t k1 = g + 1 < starts.size() ? starts[g + 1] : L;
                float mx = 0.0f;
                for (uint32_t k = starts[g]; k < k1; ++k) {
                    mx = std::max(mx, std::max(maj[k], 0.00000001f));
                    c.merged_of[b][k] = g;
                }
                c.merged_lo[b].push_back(float(starts[g]) * dz);
                c.merged_maj[b].push_back(mx);
            }
            c.merged_lo[b].push_back(c.top_altitude_km);
        }
    }
    return true;
}

// ---- sky-core bake restated: medium.rs:28-159 ------------------------------

struct CpuCoeffs {
    float rayleigh, sca[kSpecies], abs[kSpecies], ozone;
};

// medium.rs:130-155 `bracket` (partition_point of key < x, then lerp weight)
template <class Row>
void bracket(const Row* items, uint32_t len, float x, uint32_t& lo, uint32_t& hi, float& t) {
    uint32_t hi_idx = 0;
    while (hi_idx < len && items[hi_idx].altitude_km < x) hi_idx++;
    if (hi_idx == 0) {
        lo = hi = 0;
        t = 0.0f;
        return;
    }
    if (hi_idx >= len) {
        lo = hi = len - 1;
        t = 0.0f;
        return;
    }
    lo = hi_idx - 1;
    hi = hi_idx;
    float klo = items[lo].altitude_km, khi = items[hi].altitude_km;
    t = khi > klo ? (x - klo) / (khi - klo) : 0.0f;
    t = clampf(t, 0.0f, 1.0f);
}

// medium.rs:28-55 (CPU coefficients_at; altitude from |(0, Rg + alt, 0)| - Rg)
CpuCoeffs cpu_coefficients_at(const SkySceneDesc* s, float probe_altitude, uint32_t band) {
    CpuCoeffs k{};
    float y = s->ground_radius_km + probe_altitude;
    float len = std::sqrt(0.0f * 0.0f + y * y + 0.0f * 0.0f);
    float altitude = len - s->ground_radius_km;
    float top = s->atmosphere_radius_km - s->ground_radius_km;
    if (!(altitude >= 0.0f && altitude <= top)) return k;
    uint32_t lo, hi;
    float t;
    bracket(s->atmosphere, s->atmosphere_len, altitude, lo, hi, t);
    float air = lerp(s->atmosphere[lo].air_cm3, s->atmosphere[hi].air_cm3, t);
    float ozone = lerp(s->atmosphere[lo].ozone_cm3, s->atmosphere[hi].ozone_cm3, t);
    bracket(s->aerosol, s->aerosol_len, altitude, lo, hi, t);
    float mass[kSpecies];
    for (uint32_t i = 0; i < kSpecies; ++i)
        mass[i] = std::max(lerp(s->aerosol[lo].mass_g_m3[i], s->aerosol[hi].mass_g_m3[i], t), 0.0f);
    float rayleigh = air * s->bands[band].rayleigh_cross_section_m2 * 1.0e9f;
    float oz = ozone * s->bands[band].ozone_cross_section_cm2 * 1.0e5f;
    for (uint32_t i = 0; i < kSpecies; ++i) {
        const SkyAerosolOptics& o = s->aerosol_optics[band * kSpecies + i];
        k.sca[i] = mass[i] * o.scattering_km_inv_per_g_m3;
        k.abs[i] = mass[i] * o.absorption_km_inv_per_g_m3;
    }
    k.rayleigh = std::max(rayleigh, 0.0f);
    k.ozone = std::max(oz, 0.0f);
    return k;
}

// medium.rs:17-25 summation order (iterator sums start at zero)
float cpu_extinction_total(const CpuCoeffs& k) {
    float sca_sum = 0.0f, abs_sum = 0.0f;
    for (uint32_t i = 0; i < kSpecies; ++i) sca_sum += k.sca[i];
    for (uint32_t i = 0; i < kSpecies; ++i) abs_sum += k.abs[i];
    float scattering = k.rayleigh + sca_sum;
    float absorption = k.ozone + abs_sum;
    return scattering + absorption;
}

}  // namespace

// ============================ exported oracle API ===========================

extern "C" {

// Trace every (pixel, band) cell of rows row_begin, row_begin+row_step, ...
// and write per-cell FP64 sums and sums of squares over the config's samples
// ([pixel][band], other rows left untouched).  `counters` (SKY_EVENT_COUNT
// entries) and `watchdog` may be NULL.  Returns 0 on success.
int oracle_render(const SkySceneDesc* scene, const SkyRenderConfig* config, uint32_t row_begin,
                  uint32_t row_step, double* cell_sum, double* cell_sumsq, uint64_t* counters,
                  uint32_t* watchdog, int threads) {
    Ctx c;
    if (!make_ctx(scene, config, c)) return SKY_ERR_INVALID_CONFIG;
    if (row_step == 0) row_step = 1;
    std::vector<uint32_t> rows;
    for (uint32_t y = row_begin; y < c.height; y += row_step) rows.push_back(y);
    const uint64_t cells_per_row = uint64_t(c.width) * c.band_count;
    const uint64_t total = cells_per_row * rows.size();
    if (threads <= 0) threads = int(std::max(1u, std::thread::hardware_concurrency()));
    std::atomic<uint64_t> next{0};
    std::atomic<bool> wd_any{false};
    std::vector<Counters> per_thread(static_cast<size_t>(threads));
    auto worker = [&](int tid) {
        Counters& n = per_thread[size_t(tid)];
        const uint64_t chunk = 16;
        for (;;) {
            uint64_t begin = next.fetch_add(chunk);
            if (begin >= total) break;
            uint64_t end = std::min(total, begin + chunk);
            for (uint64_t i = begin; i < end; ++i) {
                uint32_t y = rows[size_t(i / cells_per_row)];
                uint64_t rem = i % cells_per_row;
                uint32_t x = uint32_t(rem / c.band_count);
                uint32_t band = uint32_t(rem % c.band_count);
                double sum, sumsq;
                bool wd = false;
                trace_cell(c, x, y, band, sum, sumsq, wd, n);
                if (wd) wd_any.store(true);
                size_t cell = (size_t(y) * c.width + x) * c.band_count + band;
                cell_sum[cell] = sum;
                if (cell_sumsq) cell_sumsq[cell] = sumsq;
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; ++t) pool.emplace_back(worker, t);
    worker(0);
    for (auto& th : pool) th.join();
    if (counters) {
        for (uint32_t e = 0; e < SKY_EVENT_COUNT; ++e) {
            uint64_t s = 0;
            for (auto& n : per_thread) s += n.e[e];
            counters[e] = s;
        }
    }
    if (watchdog) *watchdog = wd_any.load() ? 1u : 0u;
    return 0;
}

// pcg4d of one counter (sky_trace.wgsl:156-168).
void oracle_pcg4d(const uint32_t in[4], uint32_t out[4]) {
    U4 v = pcg4d(U4{in[0], in[1], in[2], in[3]});
    out[0] = v.x;
    out[1] = v.y;
    out[2] = v.z;
    out[3] = v.w;
}

// The first `n` rng_f32 draws of the chain (pixel, sample, band) under `seed`.
void oracle_rng_stream(uint32_t pixel, uint32_t sample, uint32_t band, uint64_t seed, uint32_t n,
                       uint32_t* out_u32, float* out_f32) {
    Rng r{pixel, sample, band, 0u, uint32_t(seed), uint32_t(seed >> 32)};
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t u = rng_next_u32(r);
        if (out_u32) out_u32[i] = u;
        if (out_f32) out_f32[i] = float(u >> 8u) * 0.000000059604644775390625f;
    }
}

// next_boundary for a ray (sky_trace.wgsl:233-250); returns hit, writes t, kind.
int oracle_next_boundary(float ground_radius_km, float atmosphere_radius_km, const float origin[3],
                         const float dir[3], float* t_out, uint32_t* kind_out) {
    Ctx c;
    c.ground_radius_km = ground_radius_km;
    c.atmosphere_radius_km = atmosphere_radius_km;
    BoundaryHit h = next_boundary(c, Ray{v3(origin[0], origin[1], origin[2]), v3(dir[0], dir[1], dir[2])});
    *t_out = h.t;
    *kind_out = h.kind;
    return h.hit ? 1 : 0;
}

// Shader coefficients_at at an altitude straight above the origin
// (sky_trace.wgsl:356-386).  out: rayleigh, sca[4], abs[4], ozone,
// scattering_total, extinction_total (12 floats).
void oracle_coefficients(const SkySceneDesc* scene, float altitude_km_in, uint32_t band, float out[12]) {
    SkyRenderConfig cfg{};
    cfg.width = cfg.height = cfg.spp = 1;
    Ctx c;
    make_ctx(scene, &cfg, c);
    Coeffs k = coefficients_at(c, v3(0.0f, scene->ground_radius_km + altitude_km_in, 0.0f), band);
    out[0] = k.rayleigh;
    for (int i = 0; i < 4; ++i) out[1 + i] = k.sca[i];
    for (int i = 0; i < 4; ++i) out[5 + i] = k.abs[i];
    out[9] = k.ozone;
    out[10] = scattering_total(k);
    out[11] = extinction_total(k);
}

// mie_phase (sky_trace.wgsl:485-494) for each mu.
void oracle_mie_phase(const SkySceneDesc* scene, uint32_t species, uint32_t band, const float* mu,
                      uint32_t n, float* out) {
    SkyRenderConfig cfg{};
    cfg.width = cfg.height = cfg.spp = 1;
    Ctx c;
    make_ctx(scene, &cfg, c);
    for (uint32_t i = 0; i < n; ++i) out[i] = mie_phase(c, species, band, mu[i]);
}

// MiePhaseTable::sample_mu_pdf / sampling_pdf (phase.rs:53-75) for each xi.
void oracle_sample_mu_pdf(const SkySceneDesc* scene, uint32_t species, uint32_t band, const float* xi,
                          uint32_t n, float* mu_out, float* pdf_out) {
    SkyRenderConfig cfg{};
    cfg.width = cfg.height = cfg.spp = 1;
    cfg.phase_sampling = SKY_PHASE_TABULATED;
    Ctx c;
    make_ctx(scene, &cfg, c);
    for (uint32_t i = 0; i < n; ++i) {
        float mu = sample_mu(c, species, band, xi[i]);
        mu_out[i] = mu;
        // pdf of the bin the search selected (phase.rs:68)
        uint32_t bins = c.phase_bins;
        size_t base = (size_t(species) * c.band_count + band) * bins;
        const float* cdf = c.cdf.data() + base;
        float x = clampf(xi[i], 0.0f, 1.0f - F32_EPSILON);
        uint32_t bin = std::min(uint32_t(std::upper_bound(cdf, cdf + bins, x) - cdf), bins - 1u);
        pdf_out[i] = std::max(c.bin_pdf[base + bin], 1.0e-12f);
    }
}

// sampling_pdf(mu) (phase.rs:71-75).
void oracle_sampling_pdf(const SkySceneDesc* scene, uint32_t species, uint32_t band, const float* mu,
                         uint32_t n, float* out) {
    SkyRenderConfig cfg{};
    cfg.width = cfg.height = cfg.spp = 1;
    cfg.phase_sampling = SKY_PHASE_TABULATED;
    Ctx c;
    make_ctx(scene, &cfg, c);
    for (uint32_t i = 0; i < n; ++i) out[i] = sampling_pdf(c, species, band, mu[i]);
}

float oracle_invert_rayleigh_cdf(float xi) { return invert_rayleigh_cdf(xi); }

// compute_majorant_grid (medium.rs:63-102): majorants and minorants
// [band][layer] over [0, atmosphere - ground].
void oracle_bake_majorant_grid(const SkySceneDesc* s, uint32_t layer_count, float* majorants,
                               float* minorants) {
    float top = s->atmosphere_radius_km - s->ground_radius_km;
    float dz = top / float(layer_count);
    for (uint32_t band = 0; band < s->band_count; ++band) {
        for (uint32_t layer = 0; layer < layer_count; ++layer) {
            float lo = float(layer) * dz, hi = float(layer + 1) * dz;
            std::vector<float> probes{lo, hi, 0.5f * (lo + hi)};  // medium.rs:85-102
            for (uint32_t i = 0; i < s->atmosphere_len; ++i) {
                float z = s->atmosphere[i].altitude_km;
                if (z > lo && z < hi) probes.push_back(z);
            }
            for (uint32_t i = 0; i < s->aerosol_len; ++i) {
                float z = s->aerosol[i].altitude_km;
                if (z > lo && z < hi) probes.push_back(z);
            }
            float min_ext = INFINITY, max_ext = 0.0f;
            for (float z : probes) {
                float e = cpu_extinction_total(cpu_coefficients_at(s, z, band));
                min_ext = std::min(min_ext, e);
                max_ext = std::max(max_ext, e);
            }
            float majorant = std::max(max_ext * 1.05f, 1.0e-8f);
            float minorant = std::min(std::max(min_ext, 0.0f) * 0.99f, majorant);
            // MajorantGrid::set_bounds (atmosphere.rs:102-106)
            float mn = clampf(minorant, 0.0f, std::max(majorant, 0.0f));
            majorants[band * layer_count + layer] = std::max(majorant, mn);
            if (minorants) minorants[band * layer_count + layer] = mn;
        }
    }
}

// CPU coefficients_at extinction (medium.rs:28-55, :23-25) at an altitude.
float oracle_cpu_extinction(const SkySceneDesc* s, float altitude, uint32_t band) {
    return cpu_extinction_total(cpu_coefficients_at(s, altitude, band));
}

// Mean of the binary transmittance estimator (delta_transmittance,
// sky_trace.wgsl:441-475) along one ray to its boundary (next_boundary; 0 when
// the ray misses the top shell), over `n` independent random streams, in the
// given tracking mode.  Returns -1 for an invalid scene.
double oracle_transmittance(const SkySceneDesc* scene, uint32_t tracking, const float origin[3], const float dir[3],
                            uint32_t band, uint32_t n) {
    SkyRenderConfig cfg{};
    cfg.width = cfg.height = cfg.spp = 1;
    cfg.tracking = tracking;
    Ctx c;
    if (!make_ctx(scene, &cfg, c)) return -1.0;
    const Ray ray{v3(origin[0], origin[1], origin[2]), normalize_or_y(v3(dir[0], dir[1], dir[2]))};
    const BoundaryHit h = next_boundary(c, ray);
    if (!h.hit) return 0.0;
    Counters cnt;
    double sum = 0.0;
    for (uint32_t i = 0; i < n; ++i) {
        Rng rng{i, 0x9E37u, band, 0u, 0x5EC7u, 0x2026u};
        bool wd = false;
        sum += double(delta_transmittance(c, ray, h.t, band, rng, wd, cnt));
    }
    return sum / double(n);
}

// The merged-layer grouping of tracking mode 2 for one band's majorants: writes
// the first uniform layer of each group to starts_out[0..L) and returns the
// number of groups.
uint32_t oracle_merge_groups(const float* majorants, uint32_t layer_count, float layer_dz, uint32_t* starts_out) {
    const std::vector<uint32_t> starts = merge_groups(majorants, layer_count, layer_dz);
    for (size_t i = 0; i < starts.size(); ++i) starts_out[i] = starts[i];
    return uint32_t(starts.size());
}

}  // extern "C"
