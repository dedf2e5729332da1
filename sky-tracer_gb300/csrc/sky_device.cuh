// sky_device.cuh — device building blocks shared by the tracing kernels.
//
// Each function follows the reference shader's semantics (the WGSL line
// ranges are cited) but is laid out for the GPU:
//   * the pcg4d counter RNG is bit-exact with sky_trace.wgsl:156-189; the
//     three chain-constant lanes of the counter are hashed once per chain;
//   * a ray is described by its impact parameter p = |o x d| and b = o.d, so
//     the majorant-layer crossings of the tracker, t = -b +- sqrt(R^2 - p^2),
//     are evaluated as sqrt((R - p)(R + p)), one square root per shell
//     instead of the two full sphere intersections of sky_trace.wgsl:211-221
//     (an error there only moves where a majorant changes); the ground and
//     top-of-atmosphere boundary keeps the reference's b^2 - c form, whose
//     roots stay consistent with the origin's altitude;
//   * the medium is read from the union-knot tables of sky_scene.h (one
//     lookup + one FMA instead of two linear profile scans).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "sky_scene.h"

namespace sky {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvPi = 0.31830988618379067154f;
constexpr float kTau = 6.28318530717958647692f;
constexpr float kIsotropicPdf = 0.07957747154594766788f;
constexpr float kRayleighNorm = 3.0f / (16.0f * kPi);
constexpr float kF32Epsilon = 1.1920929e-7f;

// ---- counters ---------------------------------------------------------------

struct Counters {
    uint32_t e[SKY_EVENT_COUNT];
    __device__ __forceinline__ void clear() {
#pragma unroll
        for (int i = 0; i < SKY_EVENT_COUNT; ++i) e[i] = 0;
    }
};

// ---- RNG: pcg4d counter hash (sky_trace.wgsl:156-189) -----------------------

struct Rng {
    uint32_t k0, k1, k2;  // first LCG step of (pixel^seed_lo, sample^seed_hi, band)
    uint32_t dim;

    __device__ __forceinline__ void init(uint32_t pixel, uint32_t sample, uint32_t band, uint32_t seed_lo,
                                         uint32_t seed_hi) {
        k0 = (pixel ^ seed_lo) * 1664525u + 1013904223u;
        k1 = (sample ^ seed_hi) * 1664525u + 1013904223u;
        k2 = band * 1664525u + 1013904223u;
        dim = 0u;
    }
    __device__ __forceinline__ uint32_t next_u32() {
        uint32_t x = k0, y = k1, z = k2, w = dim * 1664525u + 1013904223u;
        dim += 1u;
        x += y * w;
        y += z * x;
        z += x * y;
        w += y * z;
        x ^= x >> 16;
        y ^= y >> 16;
        z ^= z >> 16;
        w ^= w >> 16;
        x += y * w;
        y += z * x;
        z += x * y;
        w += y * z;
        return x ^ y ^ z ^ w;
    }
    // rng_f32: 24 high bits scaled by 2^-24 (exact conversion).
    __device__ __forceinline__ float next() {
        return __uint2float_rz(next_u32() >> 8) * 0.000000059604644775390625f;
    }
};

// ---- small vector helpers -----------------------------------------------------

struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 mk(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 add(V3 a, V3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 scale(V3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ V3 madd(V3 a, V3 b, float s) {  // a + b*s
    return mk(fmaf(b.x, s, a.x), fmaf(b.y, s, a.y), fmaf(b.z, s, a.z));
}
__device__ __forceinline__ float dot3(V3 a, V3 b) { return fmaf(a.x, b.x, fmaf(a.y, b.y, a.z * b.z)); }
__device__ __forceinline__ V3 cross3(V3 a, V3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
// normalize_or_y (sky_trace.wgsl:191-197)
__device__ __forceinline__ V3 normalize_or_y(V3 v) {
    float l2 = dot3(v, v);
    if (l2 > 0.0f) return scale(v, rsqrtf(l2));
    return mk(0.0f, 1.0f, 0.0f);
}
__device__ __forceinline__ V3 load3(const float* p) { return mk(p[0], p[1], p[2]); }

// ---- ray geometry -----------------------------------------------------------------

// Invariants of a ray o + t d (|d| = 1) with respect to the planet centre.
struct RayGeo {
    float b;     // o . d      (t = s - b, s measured from the closest approach)
    float p;     // impact parameter |o x d|
    float r0sq;  // |o|^2
};

__device__ __forceinline__ RayGeo ray_geo(V3 o, V3 d) {
    RayGeo g;
    g.b = dot3(o, d);
    V3 c = cross3(o, d);
    g.p = sqrtf(dot3(c, c));
    g.r0sq = dot3(o, o);
    return g;
}

// Altitude at distance t along the ray.
__device__ __forceinline__ float altitude_at(const RayGeo& g, float t, float ground_radius) {
    return sqrtf(fmaxf(fmaf(t, t + 2.0f * g.b, g.r0sq), 0.0f)) - ground_radius;
}

// Half chord sqrt(R^2 - p^2) (negative when the ray misses the shell).
__device__ __forceinline__ float half_chord(float radius, float p) {
    float disc = (radius - p) * (radius + p);
    return disc >= 0.0f ? sqrtf(disc) : -1.0f;
}

// Both roots -b -+ sqrt(b^2 - c) of the sphere of `radius` with
// c = (|o| - R)(|o| + R), the form of intersect_sphere (sky_trace.wgsl:211-221).
// Here the sign of c is the sign of the origin's computed altitude above the
// sphere, so a ray that leaves the ground upwards (b > 0, c > 0) has two
// negative roots and cannot re-enter it.  The impact-parameter form's far root
// sqrt((R - p)(R + p)) - b carries the FP32 rounding of p amplified by
// cot(elevation) (6 m at 5 degrees, more than the 5 m ray epsilon), which made
// some shadow rays leaving the ground towards a low sun hit it again.
// The rounding is fixed by intrinsics (no contraction left to the compiler),
// so that every kernel that inlines it takes the same decisions on grazing rays.
__device__ __forceinline__ bool sphere_roots(const RayGeo& g, float r0, float radius, float& t0, float& t1) {
    const float c = __fmul_rn(__fsub_rn(r0, radius), __fadd_rn(r0, radius));
    const float disc = __fmaf_rn(g.b, g.b, -c);
    if (disc < 0.0f) return false;
    const float s = sqrtf(disc);
    t0 = -g.b - s;
    t1 = -g.b + s;
    return true;
}

// next_boundary (sky_trace.wgsl:233-250): ground (kind 0) or top exit (kind 1).
__device__ __forceinline__ bool next_boundary(const DevScene& S, const RayGeo& g, float& t_out, uint32_t& kind) {
    const float r0 = sqrtf(g.r0sq);
    float a0, a1;
    if (!sphere_roots(g, r0, S.atmosphere_radius, a0, a1)) return false;
    float t_exit = fmaxf(a1, kRayEpsilonKm);
    float t_ground = -1.0f, t0, t1;
    if (sphere_roots(g, r0, S.ground_radius, t0, t1))
        t_ground = t0 > kRayEpsilonKm ? t0 : (t1 > kRayEpsilonKm ? t1 : -1.0f);
    if (t_ground > kRayEpsilonKm && t_ground < t_exit) {
        t_out = t_ground;
        kind = 0u;
    } else {
        t_out = t_exit;
        kind = 1u;
    }
    return true;
}

// layer_for_altitude (sky_trace.wgsl:252-257)
__device__ __forceinline__ uint32_t layer_for_altitude(const DevScene& S, float altitude) {
    float top = fmaxf(S.top_altitude, 0.000001f);
    float clamped = fminf(fmaxf(altitude, 0.0f), top - 0.000001f);
    uint32_t layer = uint32_t(floorf(clamped / top * float(S.layer_count)));
    return min(layer, S.layer_count - 1u);
}

// boundary_candidate for one layer shell (sky_trace.wgsl:263-282), both roots.
__device__ __forceinline__ void shell_candidate(const DevScene& S, const RayGeo& g, float t, float alt_boundary,
                                                float& next_t) {
    if (alt_boundary <= 0.0f || alt_boundary >= S.top_altitude) return;
    float q = half_chord(S.ground_radius + alt_boundary, g.p);
    if (q < 0.0f) return;
    float t0 = -q - g.b, t1 = q - g.b;
    if (t0 > t + kRayEpsilonKm && t0 < next_t) next_t = t0;
    if (t1 > t + kRayEpsilonKm && t1 < next_t) next_t = t1;
}

// next_majorant_segment_end (sky_trace.wgsl:284-294): the nearest crossing of
// the current layer's lower or upper shell beyond t + epsilon; also returns
// the layer whose majorant covers the segment (:419).
__device__ __forceinline__ float next_segment_end(const DevScene& S, const RayGeo& g, float t, float t_max,
                                                  uint32_t& layer) {
    float probe = fminf(t + kRayEpsilonKm, t_max);
    uint32_t k = layer_for_altitude(S, altitude_at(g, probe, S.ground_radius));
    float next_t = t_max;
    shell_candidate(S, g, t, float(k) * S.layer_dz, next_t);
    shell_candidate(S, g, t, float(k + 1u) * S.layer_dz, next_t);
    float probe2 = fminf(t + kRayEpsilonKm, next_t);
    layer = probe2 == probe ? k : layer_for_altitude(S, altitude_at(g, probe2, S.ground_radius));
    return next_t;
}

// ---- merged tracking grid (SKY_TRACKING_MERGED_LAYERS) -------------------------------

struct MergedGrid {
    const float* radius;    // [count + 1] shell radii
    const float* maj;       // [count]
    const uint16_t* map;    // [layers] uniform layer -> merged layer
    int count;
};

__device__ __forceinline__ MergedGrid merged_grid(const DevScene& S, uint32_t band) {
    MergedGrid G;
    const uint32_t off = S.trk_off[band];
    G.radius = S.trk_radius + off;
    G.maj = S.trk_maj + off;
    G.map = S.trk_map + band * S.layer_count;
    G.count = int(S.trk_count[band]);
    return G;
}

__device__ __forceinline__ int merged_layer_at(const DevScene& S, const MergedGrid& G, float alt) {
    int k = min(max(int(alt * S.inv_layer_dz), 0), int(S.layer_count) - 1);
    return int(G.map[k]);
}

// The next shell crossing of merged layer m after t: inbound rays (s = t + b
// < 0) that reach the lower shell leave through it (dir -1); otherwise the
// ray leaves through the upper shell (dir +1); dir 0 when the boundary
// (ground / top, t_max) comes first.  One square root per crossing.
__device__ __forceinline__ float merged_crossing(const MergedGrid& G, const RayGeo& g, int m, float t, float t_max,
                                                 int& dir) {
    dir = 0;
    float tn = t_max;
    if (t + g.b < 0.0f && m > 0) {
        float r = G.radius[m];
        if (g.p < r) {
            tn = -sqrtf((r - g.p) * (r + g.p)) - g.b;
            dir = -1;
        }
    }
    if (dir == 0 && m + 1 < G.count) {
        float r = G.radius[m + 1];
        tn = sqrtf(fmaxf((r - g.p) * (r + g.p), 0.0f)) - g.b;
        dir = 1;
    }
    if (tn >= t_max) {
        tn = t_max;
        dir = 0;
    }
    return fmaxf(tn, t);
}

// ---- medium ---------------------------------------------------------------------------

// The band-independent knot tables and the per-band constants that the
// medium functions read, wherever they are held: the scene's global copies,
// or the copies a kernel staged in its block's shared memory.
struct Medium {
    const float* knot_z;            // [K]
    const uint16_t* finder;         // [kFinderCells]
    const DevProfileKnot* profile;  // [K]
    const DevBand* bands;           // [B]
    const SkyAerosolOptics* optics; // [B][species]
};

__device__ __forceinline__ Medium global_medium(const DevScene& S) {
    return Medium{S.knot_z, S.finder, S.profile, S.bands, S.optics};
}

// Knot interval containing `alt` (alt in [0, top]).
__device__ __forceinline__ uint32_t knot_interval(const DevScene& S, const float* knot_z, const uint16_t* finder,
                                                  float alt) {
    int cell = min(int(alt * S.finder_scale), int(kFinderCells) - 1);
    uint32_t k = finder[cell];
    while (k + 2u < S.knot_count && alt >= knot_z[k + 1u]) ++k;
    return k;
}

// Total extinction of a band at `alt` (extinction_total(coefficients_at()),
// sky_trace.wgsl:356-403), from the band's (value, slope) knot table
// `sig_row` and its finder-cell table `cell_row` (DevScene::sig_cell).  A
// tentative collision reads one 16-byte cell entry: the knot interval that
// holds the cell's lower edge, with its value, slope, knot and the next knot.
// Below the next knot the interval is the one knot_interval() finds, so the
// result is the same FMA on the same operands; above it (the cell holds a
// knot) the knot search runs.
__device__ __forceinline__ float sigma_t_at(const DevScene& S, const float* knot_z, const uint16_t* finder,
                                            const float2* sig_row, const float4* cell_row, float alt) {
    if (!(alt >= 0.0f && alt <= S.top_altitude)) return 0.0f;
    const int cell = min(int(alt * S.finder_scale), int(kFinderCells) - 1);
    const float4 c = __ldg(cell_row + cell);
    if (alt < c.w) return fmaf(alt - c.z, c.y, c.x);
    const uint32_t k = knot_interval(S, knot_z, finder, alt);
    const float2 e = sig_row[k];
    return fmaf(alt - knot_z[k], e.y, e.x);
}

struct Coeffs {  // MediumCoefficients (sky_trace.wgsl:101-106)
    float rayleigh;
    float sca[kSpecies];
    float abs_total;  // ozone + aerosol absorption
    float scattering;
    float extinction;
};

// coefficients_at (sky_trace.wgsl:356-386) from the band-independent knot
// profile and the per-band cross sections.
//
// kAer: the aerosol species evaluated, the first kAer of the four.  A kernel
// instantiated with kAer = 1 serves scenes whose species 1-3 carry no
// aerosol (DevScene::aerosol_mask): their terms are exactly +0 in the
// four-species evaluation (the clamped masses are 0, or their optics are),
// so both forms return the same bits, and the single-species one skips
// three species' loads and arithmetic in every medium evaluation (-7.5 % on
// a 512x256, 81-band, 256-spp render).  The phase functions below take the
// same parameter; the species beyond kAer have sca[i] = 0.
template <int kAer = int(kSpecies)>
__device__ __forceinline__ Coeffs coefficients_at(const DevScene& S, const Medium& M, uint32_t band, float alt) {
    Coeffs c;
    c.rayleigh = 0.0f;
#pragma unroll
    for (int i = 0; i < int(kSpecies); ++i) c.sca[i] = 0.0f;
    c.abs_total = 0.0f;
    c.scattering = 0.0f;
    c.extinction = 0.0f;
    if (!(alt >= 0.0f && alt <= S.top_altitude)) return c;
    uint32_t k = knot_interval(S, M.knot_z, M.finder, alt);
    float dz = alt - M.knot_z[k];
    const DevProfileKnot& P = M.profile[k];
    const DevBand& B = M.bands[band];
    float air = fmaf(dz, P.air_slope, P.air);
    float ozone = fmaf(dz, P.ozone_slope, P.ozone);
    c.rayleigh = fmaxf(air * B.rayleigh_xs, 0.0f);
    float absorption = fmaxf(ozone * B.ozone_xs, 0.0f);
    float scattering = c.rayleigh;
#pragma unroll
    for (int i = 0; i < kAer; ++i) {
        float mass = fmaxf(fmaf(dz, P.mass_slope[i], P.mass[i]), 0.0f);
        SkyAerosolOptics o = M.optics[band * kSpecies + i];
        c.sca[i] = fmaxf(mass * o.scattering_km_inv_per_g_m3, 0.0f);
        absorption += fmaxf(mass * o.absorption_km_inv_per_g_m3, 0.0f);
        scattering += c.sca[i];
    }
    c.abs_total = absorption;
    c.scattering = scattering;
    c.extinction = scattering + absorption;
    return c;
}

// The same from the scene's global tables.
template <int kAer = int(kSpecies)>
__device__ __forceinline__ Coeffs coefficients_at(const DevScene& S, const float* knot_z, const uint16_t* finder,
                                                  uint32_t band, float alt) {
    return coefficients_at<kAer>(S, Medium{knot_z, finder, S.profile, S.bands, S.optics}, band, alt);
}

// ---- phase functions ----------------------------------------------------------------

// Cube root of x >= 0 as 2^(log2(x)/3) on the special-function unit (relative
// error ~1e-6; only used to place mu on the cube-root phase grid and in the
// Rayleigh inverse CDF).
__device__ __forceinline__ float cbrt_pos(float x) { return x > 0.0f ? exp2f(__log2f(x) * (1.0f / 3.0f)) : 0.0f; }

__device__ __forceinline__ float rayleigh_phase(float mu) { return kRayleighNorm * (1.0f + mu * mu); }

// Position of mu on the cube-root phase grid: u = ((1 - mu) / 2)^(1/3).
__device__ __forceinline__ float phase_grid_u(float mu) {
    return cbrt_pos((1.0f - fminf(fmaxf(mu, -1.0f), 1.0f)) * 0.5f);
}

// mie_phase (sky_trace.wgsl:485-494): lerp between bin centres on the
// cube-root mu grid, at grid position u.
__device__ __forceinline__ float mie_phase_u(const DevScene& S, uint32_t species, uint32_t band, float u) {
    uint32_t bins = S.phase_bins;
    float f = u * float(bins) - 0.5f;
    uint32_t i0 = min(uint32_t(fminf(fmaxf(floorf(f), 0.0f), float(bins - 1u))), bins - 1u);
    uint32_t i1 = min(i0 + 1u, bins - 1u);
    float t = fminf(fmaxf(f - float(i0), 0.0f), 1.0f);
    const float* row = S.phase_values + (size_t(species) * S.band_count + band) * bins;
    float p0 = __ldg(row + i0), p1 = __ldg(row + i1);
    return fmaxf(fmaf(t, p1 - p0, p0), 0.0f);
}

// mixed_phase_value (sky_trace.wgsl:496-510), at grid position u of mu.
template <int kAer = int(kSpecies)>
__device__ __forceinline__ float mixed_phase_u(const DevScene& S, const Coeffs& c, uint32_t band, float mu, float u) {
    if (c.scattering <= 0.0f) return 0.0f;
    float acc = c.rayleigh * rayleigh_phase(mu);
#pragma unroll
    for (int i = 0; i < kAer; ++i)
        if (c.sca[i] > 0.0f) acc = fmaf(c.sca[i], mie_phase_u(S, uint32_t(i), band, u), acc);
    return acc / c.scattering;
}

template <int kAer = int(kSpecies)>
__device__ __forceinline__ float mixed_phase(const DevScene& S, const Coeffs& c, uint32_t band, float mu) {
    if (c.scattering <= 0.0f) return 0.0f;
    return mixed_phase_u<kAer>(S, c, band, mu, phase_grid_u(mu));
}

// phase.rs:137-140
__device__ __forceinline__ float mu_edge(uint32_t edge, uint32_t bins) {
    float u = float(edge) / float(bins);
    return 1.0f - 2.0f * u * u * u;
}

// MiePhaseTable::sample_mu_pdf (phase.rs:53-69): the first CDF entry above
// xi (a binary search of the row in the reference), found by a forward scan
// from the guide table's lower bound for xi's 1/bins cell.
__device__ __forceinline__ float sample_mie_mu(const DevScene& S, uint32_t species, uint32_t band, float xi) {
    uint32_t bins = S.phase_bins;
    const size_t row = (size_t(species) * S.band_count + band) * bins;
    const float* cdf = S.phase_cdf + row;
    xi = fminf(fmaxf(xi, 0.0f), 1.0f - kF32Epsilon);
    uint32_t lo = __ldg(S.phase_guide + row + min(uint32_t(xi * float(bins)), bins - 1u));
    while (lo < bins && __ldg(cdf + lo) <= xi) ++lo;
    uint32_t bin = min(lo, bins - 1u);
    float prev = bin == 0u ? 0.0f : __ldg(cdf + bin - 1u);
    float next = __ldg(cdf + bin);
    float t = next > prev ? (xi - prev) / (next - prev) : 0.5f;
    float e0 = mu_edge(bin, bins), e1 = mu_edge(bin + 1u, bins);
    return e0 * (1.0f - t) + e1 * t;
}

// MiePhaseTable::sampling_pdf (phase.rs:71-75, mu_to_bin :142-146), at grid position u.
__device__ __forceinline__ float mie_sampling_pdf_u(const DevScene& S, uint32_t species, uint32_t band, float u) {
    uint32_t bins = S.phase_bins;
    uint32_t bin = min(uint32_t(floorf(u * float(bins))), bins - 1u);
    return fmaxf(__ldg(S.phase_bin_pdf + (size_t(species) * S.band_count + band) * bins + bin), 1.0e-12f);
}

// Inverse Rayleigh CDF (sampling.rs:182-185): 2 sinh(asinh(y)/3) = u - 1/u
// with u = cbrt(y + sqrt(y^2 + 1)), y = 4 xi - 2.
__device__ __forceinline__ float invert_rayleigh_cdf(float xi) {
    float y = 4.0f * fminf(fmaxf(xi, 0.0f), 1.0f) - 2.0f;
    float u = cbrt_pos(y + sqrtf(fmaf(y, y, 1.0f)));
    return fminf(fmaxf(u - 1.0f / u, -1.0f), 1.0f);
}

// ---- directions (sky_trace.wgsl:512-564) ----------------------------------------------

__device__ __forceinline__ void orthonormal_basis(V3 n_in, V3& t, V3& bt) {  // :512-520
    V3 n = normalize_or_y(n_in);
    float sign = n.z >= 0.0f ? 1.0f : -1.0f;
    float a = -1.0f / (sign + n.z);
    float b = n.x * n.y * a;
    t = normalize_or_y(mk(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x));
    bt = normalize_or_y(mk(b, sign + n.y * n.y * a, -n.y));
}

// direction_from_axis_mu with sin(theta) given by the caller (:522-532).
__device__ __forceinline__ V3 direction_from_frame(V3 axis, V3 t, V3 bt, float mu, float sin_theta, float xi_phi) {
    float s, c;
    __sincosf(kTau * xi_phi, &s, &c);
    V3 d = scale(axis, mu);
    d = madd(d, t, sin_theta * c);
    d = madd(d, bt, sin_theta * s);
    return normalize_or_y(d);
}

__device__ __forceinline__ V3 direction_from_axis_mu(V3 axis_in, float mu_in, float xi_phi) {
    float mu = fminf(fmaxf(mu_in, -1.0f), 1.0f);
    float sin_theta = sqrtf(fmaxf(1.0f - mu * mu, 0.0f));
    V3 t, bt;
    orthonormal_basis(axis_in, t, bt);
    return direction_from_frame(normalize_or_y(axis_in), t, bt, mu, sin_theta, xi_phi);
}

// sample_uniform_cone around the sun (:541-546); the sun's frame is
// precomputed per scene, and sin(theta) uses (1-c)(1+c) to stay accurate for
// the 0.27-degree cone.
// The cone around a sun frame given apart from its scene (a batch's render).
__device__ __forceinline__ V3 sample_sun_cone(const float* sun, const float* sun_t, const float* sun_b,
                                              float one_minus_cos_max, Rng& rng) {
    float xi = fminf(fmaxf(rng.next(), 0.0f), 0.99999994f);
    float one_minus_cos = xi * one_minus_cos_max;
    float cos_theta = 1.0f - one_minus_cos;
    float sin_theta = sqrtf(fmaxf(one_minus_cos * (2.0f - one_minus_cos), 0.0f));
    float xi_phi = rng.next();
    return direction_from_frame(load3(sun), load3(sun_t), load3(sun_b), cos_theta, sin_theta, xi_phi);
}
__device__ __forceinline__ V3 sample_sun_cone(const DevScene& S, Rng& rng) {
    return sample_sun_cone(S.sun, S.sun_t, S.sun_b, S.one_minus_cos_max, rng);
}

// sample_isotropic (:534-539)
__device__ __forceinline__ V3 sample_isotropic(Rng& rng) {
    float z = 1.0f - 2.0f * rng.next();
    float r = sqrtf(fmaxf(1.0f - z * z, 0.0f));
    float s, c;
    __sincosf(kTau * rng.next(), &s, &c);
    return mk(r * c, z, r * s);
}

// sample_cosine_hemisphere (:548-560); returns the direction and its pdf.
__device__ __forceinline__ V3 sample_cosine_hemisphere(V3 axis, Rng& rng, float& pdf) {
    float u = rng.next();
    float r = sqrtf(u);
    float xi_phi = rng.next();
    float cos_theta = sqrtf(fmaxf(1.0f - u, 0.0f));
    V3 t, bt;
    orthonormal_basis(axis, t, bt);
    V3 n = normalize_or_y(axis);
    V3 dir = direction_from_frame(n, t, bt, cos_theta, r, xi_phi);
    pdf = fmaxf(dot3(n, dir), 0.0f) * kInvPi;
    return dir;
}

// Tabulated continuation (phase.rs:53-75, sampling.rs:182-185): component by
// sigma_s,i / sigma_s, mu from its inverse CDF, and the draw for phi; returns
// mixed_phase(mu) / mixture_pdf(mu), which does not depend on phi.
template <int kAer = int(kSpecies)>
__device__ __forceinline__ float tabulated_mu(const DevScene& S, const Coeffs& c, uint32_t band, Rng& rng, float& mu,
                                             float& xi_phi) {
    float target = rng.next() * c.scattering;
    int chosen = -1;
    float acc = c.rayleigh;
    if (target < acc) chosen = 0;
#pragma unroll
    for (int i = 0; i < kAer; ++i) {
        acc = acc + c.sca[i];
        if (chosen < 0 && target < acc) chosen = i + 1;
    }
    if (chosen < 0) {
        chosen = 0;
#pragma unroll
        for (int i = 0; i < kAer; ++i)
            if (c.sca[i] > 0.0f) chosen = i + 1;
    }
    float xi_mu = rng.next();
    mu = chosen == 0 ? invert_rayleigh_cdf(xi_mu) : sample_mie_mu(S, uint32_t(chosen - 1), band, xi_mu);
    xi_phi = rng.next();
    float inv_s = 1.0f / c.scattering;
    const float u = phase_grid_u(mu);  // shared by the pdf and the phase lookups
    float pdf = c.rayleigh * inv_s * rayleigh_phase(mu);
#pragma unroll
    for (int i = 0; i < kAer; ++i)
        if (c.sca[i] > 0.0f) pdf = fmaf(c.sca[i] * inv_s, mie_sampling_pdf_u(S, uint32_t(i), band, u), pdf);
    return mixed_phase_u<kAer>(S, c, band, mu, u) / pdf;
}

// The tabulated continuation direction around `axis`; returns the weight.
template <int kAer = int(kSpecies)>
__device__ __forceinline__ float sample_tabulated(const DevScene& S, const Coeffs& c, uint32_t band, V3 axis,
                                                  Rng& rng, V3& out_dir) {
    float mu, xi_phi;
    const float w = tabulated_mu<kAer>(S, c, band, rng, mu, xi_phi);
    out_dir = direction_from_axis_mu(axis, mu, xi_phi);
    return w;
}

// ---- cameras (sky_trace.wgsl:610-689) --------------------------------------------------

__device__ __forceinline__ V3 panorama_dir(float u, float v) {  // :614-623
    float azimuth = (u - 0.5f) * kTau;
    float elevation = (0.5f - v) * kPi;
    float sa, ca, se, ce;
    sincosf(azimuth, &sa, &ca);
    sincosf(elevation, &se, &ce);
    return normalize_or_y(mk(ce * sa, se, ce * ca));
}

__device__ __forceinline__ float from_sub_uvs_to_unit(float u, float resolution) {  // :625-630
    if (resolution <= 1.0f) return 0.5f;
    return (u - 0.5f / resolution) * (resolution / (resolution - 1.0f));
}

__device__ __forceinline__ V3 sky_view_lut_dir(const DevLaunch& L, float u_in, float v_in) {  // :641-681
    float ux = fminf(fmaxf(from_sub_uvs_to_unit(u_in, float(L.width)), 0.0f), 1.0f);
    float uy = fminf(fmaxf(from_sub_uvs_to_unit(v_in, float(L.height)), 0.0f), 1.0f);
    float view_zenith_cos;
    if (uy < 0.75f) {
        float coord = uy / 0.75f;
        coord = 1.0f - coord;
        coord = coord * coord;
        coord = 1.0f - coord;
        view_zenith_cos = cosf(L.lut_zenith_horizon_angle * coord);
    } else {
        float coord = (uy - 0.75f) / 0.25f;
        coord = coord * coord;
        view_zenith_cos = cosf(L.lut_zenith_horizon_angle + L.lut_beta * coord);
    }
    float coord = ux * ux;
    float light_view_cos = -(coord * 2.0f - 1.0f);
    float sin_view = sqrtf(fmaxf(1.0f - view_zenith_cos * view_zenith_cos, 0.0f));
    float side_scale = sqrtf(fmaxf(1.0f - light_view_cos * light_view_cos, 0.0f));
    V3 f = load3(L.lut_forward), s = load3(L.lut_side);
    V3 h = madd(scale(f, light_view_cos), s, side_scale);
    return normalize_or_y(mk(sin_view * h.x, view_zenith_cos + sin_view * h.y, sin_view * h.z));
}

// (i + offset) / n correctly rounded, as the shader divides: a product with the
// exact reciprocal 1/n when n is a power of two (the same bits, without the
// division's instruction sequence), else the division.
__device__ __forceinline__ float pixel_coord(uint32_t i, float offset, uint32_t n, float inv_n) {
    const float a = __fadd_rn(float(i), offset);
    return (n & (n - 1u)) == 0u ? __fmul_rn(a, inv_n) : __fdiv_rn(a, float(n));
}

// Camera ray of sample `rng` for pixel (x, y) (sky_trace.wgsl:800-807): two
// jitter draws are always consumed, also for the sky-view LUT.
__device__ __forceinline__ V3 camera_dir(const DevLaunch& L, uint32_t x, uint32_t y, Rng& rng) {
    float u = pixel_coord(x, rng.next(), L.width, L.inv_width);
    float v = pixel_coord(y, rng.next(), L.height, L.inv_height);
    if (L.projection == SKY_PROJECTION_SKY_VIEW_LUT) {
        u = pixel_coord(x, 0.5f, L.width, L.inv_width);
        v = pixel_coord(y, 0.5f, L.height, L.inv_height);
        return sky_view_lut_dir(L, u, v);
    }
    return panorama_dir(u, v);
}

// ---- delta tracking (shared by the plain and wavefront kernels) ----------

// Layered delta tracking along one ray (sample_real_collision and
// delta_transmittance, sky_trace.wgsl:405-475).  Returns true at a real
// collision (t_hit set).  kTracking selects the reference's per-segment
// restart or the residual carry (same distribution, fewer draws).
// A ray that crosses more than 100000 segments sets the watchdog and ends as
// the reference ends it: a camera or continuation ray (shadow = false)
// without a collision (sky_trace.wgsl:412-415), a shadow ray (shadow = true)
// as blocked, transmittance 0 (:448-451).
// Residual-carry delta tracking over the band's merged tracking grid.
__device__ __forceinline__ bool track_ray_merged(const DevScene& S, const Medium& M, const RayGeo& g, float t_max,
                                                 uint32_t band, Rng& rng, float& t_hit, Counters& n, bool& watchdog,
                                                 bool shadow) {
    const MergedGrid G = merged_grid(S, band);
    const float2* sig_row = S.sigma_t + band * S.knot_count;
    const float4* cell_row = S.sig_cell + band * kFinderCells;
    float t = 0.0f;
    int m = merged_layer_at(S, G, altitude_at(g, fminf(kRayEpsilonKm, t_max), S.ground_radius));
    int dir;
    float t_seg = merged_crossing(G, g, m, t, t_max, dir);
    float maj = __ldg(G.maj + m);
    ++n.e[SKY_EVENT_SEGMENT];
    float tau = -__logf(fmaxf(1.0f - rng.next(), 0.0000001f));
    uint32_t guard = 0;
    for (;;) {
        // the crossings up to the segment that holds the next tentative collision
        float dt = tau / maj;
        while (!(t + dt < t_seg)) {
            if (dir == 0) return false;
            if (++guard > 100000u) {
                watchdog = true;
                return shadow;
            }
            tau = fmaxf(tau - (t_seg - t) * maj, 0.0f);
            t = t_seg;
            m += dir;
            t_seg = merged_crossing(G, g, m, t, t_max, dir);
            maj = __ldg(G.maj + m);
            ++n.e[SKY_EVENT_SEGMENT];
            dt = tau / maj;
        }
        t = t + dt;
        ++n.e[SKY_EVENT_TRACK_STEP];
        float sig = sigma_t_at(S, M.knot_z, M.finder, sig_row, cell_row, altitude_at(g, t, S.ground_radius));
        if (rng.next() * maj < sig) {
            t_hit = t;
            return true;
        }
        tau = -__logf(fmaxf(1.0f - rng.next(), 0.0000001f));
    }
}

template <int kTracking>
__device__ __forceinline__ bool track_ray(const DevScene& S, const Medium& M, const RayGeo& g, float t_max,
                                          uint32_t band, Rng& rng, float& t_hit, Counters& n, bool& watchdog,
                                          bool shadow) {
    if (kTracking == SKY_TRACKING_MERGED_LAYERS)
        return track_ray_merged(S, M, g, t_max, band, rng, t_hit, n, watchdog, shadow);
    const float* maj_row = S.majorants + band * S.layer_count;
    const float2* sig_row = S.sigma_t + band * S.knot_count;
    const float4* cell_row = S.sig_cell + band * kFinderCells;
    float t = 0.0f;
    uint32_t guard = 0;
    float tau = 0.0f;
    bool need_draw = true;
    for (;;) {
        if (t >= t_max) return false;
        if (guard > 100000u) {
            watchdog = true;
            return shadow;
        }
        ++guard;
        uint32_t layer;
        float seg_end = next_segment_end(S, g, t, t_max, layer);
        ++n.e[SKY_EVENT_SEGMENT];
        float maj = fmaxf(__ldg(maj_row + layer), 0.00000001f);
        if (kTracking == SKY_TRACKING_RESIDUAL_CARRY) {
            for (;;) {
                if (need_draw) {
                    tau = -__logf(fmaxf(1.0f - rng.next(), 0.0000001f));
                    need_draw = false;
                }
                float dt = tau / maj;
                if (t + dt >= seg_end) {
                    tau = fmaxf(tau - (seg_end - t) * maj, 0.0f);
                    break;
                }
                t = t + dt;
                need_draw = true;
                ++n.e[SKY_EVENT_TRACK_STEP];
                float alt = altitude_at(g, t, S.ground_radius);
                float sig = sigma_t_at(S, M.knot_z, M.finder, sig_row, cell_row, alt);
                if (rng.next() * maj < sig) {
                    t_hit = t;
                    return true;
                }
            }
        } else {
            for (;;) {
                if (t >= seg_end) break;
                float u = fmaxf(1.0f - rng.next(), 0.0000001f);
                t = t - __logf(u) / maj;
                if (t >= seg_end) break;
                ++n.e[SKY_EVENT_TRACK_STEP];
                float alt = altitude_at(g, t, S.ground_radius);
                float sig = sigma_t_at(S, M.knot_z, M.finder, sig_row, cell_row, alt);
                if (rng.next() * maj < sig) {
                    t_hit = t;
                    return true;
                }
            }
        }
        t = seg_end;
    }
}

}  // namespace sky
