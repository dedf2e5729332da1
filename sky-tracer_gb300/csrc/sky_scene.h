// sky_scene.h — device-resident scene layout shared by the host set-up code
// and the kernels.
//
// The reference shader reads its medium through linear scans of the raw
// atmosphere and aerosol profiles on every null-collision candidate
// (sky_trace.wgsl:300-354).  Here the scene is re-tabulated once, at scene
// creation, onto the union of both profiles' altitude knots: every
// coefficient is linear in altitude between consecutive union knots, so the
// extinction of a band is stored as (value, slope) per knot interval and a
// lookup is one table read plus one FMA.  A uniform "finder" grid maps an
// altitude to its knot interval in O(1).  Nothing about the medium changes:
// between knots the reference's lerp of each profile is exactly linear, and
// the tables are evaluated with the reference's own formulas at the knots
// (sky_trace.wgsl:356-386).
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

#include "../../include/sky_cuda.h"

namespace sky {

constexpr uint32_t kSpecies = SKY_SPECIES_COUNT;
constexpr uint32_t kMaxBands = 256;
constexpr uint32_t kMaxKnots = 1024;
constexpr uint32_t kFinderCells = 512;
constexpr uint32_t kMaxLayers = 1024;
constexpr uint32_t kDefaultWatchdog = 1024;  // integrator.rs:14
constexpr uint32_t kDefaultRrDepth = 4;      // sky_trace.wgsl:692
constexpr uint32_t kMaxLightSamples = 1024;  // NEE samples per vertex accepted by a render config
constexpr float kRayEpsilonKm = 0.005f;      // sky_trace.wgsl:8

// Per-band constants.
struct DevBand {
    float solar_radiance;  // SkyBand::solar_radiance_w_m2_sr
    float rayleigh_xs;     // rayleigh_cross_section_m2 * 1e9 (sky_trace.wgsl:383)
    float ozone_xs;        // ozone_cross_section_cm2 * 1e5  (sky_trace.wgsl:384)
    float xyz[3];          // CIE 1931 weights at the band centre
    float _pad[2];
};
static_assert(sizeof(DevBand) == 32, "DevBand layout");

// Band-independent profile on the union knots: value at the knot and slope
// per km up to the next knot, for air, ozone and the four aerosol masses.
struct DevProfileKnot {
    float air, air_slope;
    float ozone, ozone_slope;
    float mass[kSpecies];
    float mass_slope[kSpecies];
};
static_assert(sizeof(DevProfileKnot) == 48, "DevProfileKnot layout");

// Everything a kernel needs, passed by value as a kernel parameter.
struct DevScene {
    uint32_t band_count;
    uint32_t knot_count;
    uint32_t layer_count;
    uint32_t phase_bins;
    float ground_radius;
    float atmosphere_radius;
    float top_altitude;
    float layer_dz;          // top / layers
    float finder_scale;      // kFinderCells / top
    float ground_albedo;
    float sun[3];            // normalised sun direction
    float sun_t[3];          // orthonormal basis of the sun axis
    float sun_b[3];
    float cos_max;           // cos(sun angular radius)
    float one_minus_cos_max;
    float light_pdf;         // 1 / (2 pi (1 - cos_max))
    uint32_t aerosol_mask;   // bit i set when species i has mass and optics somewhere: the others add
                             // exactly 0 to every coefficient, and the kernels skip them
    // device tables
    const float* knot_z;               // [K]
    const uint16_t* finder;            // [kFinderCells] knot interval of each cell's lower edge
    const float2* sigma_t;             // [B][K] extinction (value, slope) per knot interval
    const float4* sig_cell;            // [B][kFinderCells] per finder cell: the knot interval k that holds
                                       // its lower edge as (value, slope, knot_z[k], knot_z[k + 1]; +inf for
                                       // the last interval)
    const float* majorants;            // [B][L]
    const DevBand* bands;              // [B]
    const DevProfileKnot* profile;     // [K]
    const SkyAerosolOptics* optics;    // [B][species]
    const float* phase_values;         // [species][B][bins]
    const float* phase_cdf;            // [species][B][bins]
    const float* phase_bin_pdf;        // [species][B][bins]
    const uint16_t* phase_guide;       // [species][B][bins]: search start of the CDF inversion
    // Merged tracking grid (SKY_TRACKING_MERGED_LAYERS): per band, the
    // merged layers' shell radii, majorants, and the map from a uniform
    // majorant layer to the merged layer that contains it.
    const float* trk_radius;           // [trk_off[b] + m], m <= count: lower shell radius of merged layer m
    const float* trk_maj;              // [trk_off[b] + m], m < count: majorant of merged layer m
    const uint16_t* trk_map;           // [B][L]: uniform layer -> merged layer
    const uint32_t* trk_count;         // [B]: merged layers of the band
    const uint32_t* trk_off;           // [B]: row offset of the band in trk_radius / trk_maj
    uint32_t trk_total;                // entries in trk_radius / trk_maj
    float inv_layer_dz;                // layers / top
    // linear sRGB from XYZ: the sRGB matrix times the Bradford solar-white-to-
    // D65 white balance (row-major; zero when the scene has no XYZ weights)
    float rgb_from_xyz[9];
};

// Per-launch constants.
struct DevLaunch {
    uint32_t width, height, spp, sample_offset;
    uint32_t row_begin;       // first image row of the rendered slab
    uint32_t rows;            // rows of the slab (height when the whole image is rendered)
    uint32_t band_count;
    uint32_t direct_light_samples;
    uint32_t projection;
    uint32_t phase_sampling;
    uint32_t rr_start_depth;
    uint32_t max_orders;      // 0 = unbounded
    uint32_t watchdog_limit;
    uint32_t tracking;        // SkyTracking
    uint32_t seed_lo, seed_hi;
    float observer_altitude;
    // sky-view LUT frame (sky_trace.wgsl:641-681), computed once per launch
    float lut_zenith_horizon_angle;
    float lut_beta;
    float lut_forward[3];
    float lut_side[3];
    float inv_width, inv_height;
};

// One render inside a persistent launch: its scene (tables may be shared
// with other jobs; only the sun differs across an elevation sweep), its
// launch constants, its outputs and its range of the launch's cells.  Cells
// are (pixel, band) pairs, pixel-major; job j owns the global cells
// [cell_begin, cell_begin + cell_count).
struct DevJob {
    DevScene S;
    DevLaunch L;
    double* cell_sum;
    double* cell_sumsq;
    float* film;
    double* xyz;
    double* xyz_var;
    float* rgb;
    uint32_t accumulate;
    uint32_t total_spp;   // samples behind the sums after this launch
    uint32_t cell_begin;  // first global cell of the job
    uint32_t cell_count;  // width * height * bands
};

}  // namespace sky
