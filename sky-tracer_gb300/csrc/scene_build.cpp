// scene_build.cpp — validation and re-tabulation of a SkySceneDesc.
//
// Follows the reference's scene packing (integrator.rs:319-418) and
// validation (integrator.rs:130-163, :401-407); the medium re-tabulation onto
// union knots is described in sky_scene.h.

#include "scene_build.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>

namespace sky {
namespace {

constexpr float kTauF = 6.28318530717958647692f;
constexpr float kPiF = 3.14159265358979323846f;

// Shader interpolation of the atmosphere profile (sky_trace.wgsl:300-327).
void atmosphere_at(const SkySceneDesc* d, float altitude, float& air, float& ozone) {
    const SkyAtmospherePoint* p = d->atmosphere;
    uint32_t n = d->atmosphere_len, hi = 0;
    while (hi < n && p[hi].altitude_km < altitude) hi++;
    if (hi == 0) {
        air = p[0].air_cm3;
        ozone = p[0].ozone_cm3;
        return;
    }
    if (hi >= n) {
        air = p[n - 1].air_cm3;
        ozone = p[n - 1].ozone_cm3;
        return;
    }
    const SkyAtmospherePoint& lo = p[hi - 1];
    const SkyAtmospherePoint& up = p[hi];
    float denom = std::max(up.altitude_km - lo.altitude_km, 0.000001f);
    float t = std::min(std::max((altitude - lo.altitude_km) / denom, 0.0f), 1.0f);
    air = lo.air_cm3 * (1.0f - t) + up.air_cm3 * t;
    ozone = lo.ozone_cm3 * (1.0f - t) + up.ozone_cm3 * t;
}

// Shader interpolation of the aerosol profile (sky_trace.wgsl:333-354).
void aerosol_at(const SkySceneDesc* d, float altitude, float mass[kSpecies]) {
    const SkyAerosolPoint* p = d->aerosol;
    uint32_t n = d->aerosol_len, hi = 0;
    while (hi < n && p[hi].altitude_km < altitude) hi++;
    if (hi == 0 || hi >= n) {
        const SkyAerosolPoint& q = p[hi == 0 ? 0 : n - 1];
        for (uint32_t i = 0; i < kSpecies; ++i) mass[i] = q.mass_g_m3[i];
        return;
    }
    const SkyAerosolPoint& lo = p[hi - 1];
    const SkyAerosolPoint& up = p[hi];
    float denom = std::max(up.altitude_km - lo.altitude_km, 0.000001f);
    float t = std::min(std::max((altitude - lo.altitude_km) / denom, 0.0f), 1.0f);
    for (uint32_t i = 0; i < kSpecies; ++i)
        mass[i] = std::max(lo.mass_g_m3[i] * (1.0f - t) + up.mass_g_m3[i] * t, 0.0f);
}

bool finite_all(const float* v, size_t n) {
    for (size_t i = 0; i < n; ++i)
        if (!std::isfinite(v[i])) return false;
    return true;
}

}  // namespace

// ---- colorimetry: spectrum.rs:13-19, :84-109, :132-165, :297-351 ----------------------
//
// Standard published matrices: linear sRGB from XYZ (D65), the Bradford cone
// response and its inverse, the D65 white at Y = 1.
namespace {
using Mat3f = float[3][3];
constexpr float kSrgbFromXyz[3][3] = {{3.2404542f, -1.5371385f, -0.4985314f},
                                      {-0.969266f, 1.8760108f, 0.041556f},
                                      {0.0556434f, -0.2040259f, 1.0572252f}};
constexpr float kBradfordLmsFromXyz[3][3] = {{0.8951f, 0.2664f, -0.1614f},
                                             {-0.7502f, 1.7135f, 0.0367f},
                                             {0.0389f, -0.0685f, 1.0296f}};
constexpr float kXyzFromBradfordLms[3][3] = {{0.9869929f, -0.1470543f, 0.1599627f},
                                             {0.4323053f, 0.5183603f, 0.0492912f},
                                             {-0.0085287f, 0.0400428f, 0.9684867f}};
constexpr float kD65WhiteY1[3] = {0.9504559f, 1.0f, 1.0890578f};

void mat3_vec(const float m[3][3], const float v[3], float out[3]) {
    for (int r = 0; r < 3; ++r) out[r] = m[r][0] * v[0] + m[r][1] * v[1] + m[r][2] * v[2];
}
void mat3_mul(const float a[3][3], const float b[3][3], float out[3][3]) {
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) out[r][c] = a[r][0] * b[0][c] + a[r][1] * b[1][c] + a[r][2] * b[2][c];
}
void normalized_to_y1(const float v[3], float out[3]) {
    if (std::fabs(v[1]) <= 1.1920929e-7f) {
        for (int i = 0; i < 3; ++i) out[i] = kD65WhiteY1[i];
        return;
    }
    const float inv = 1.0f / v[1];
    out[0] = v[0] * inv;
    out[1] = 1.0f;
    out[2] = v[2] * inv;
}
}  // namespace

void solar_d65_white_balance(const float* solar, const float* band_xyz, uint32_t bands, float wb[3][3]) {
    float white[3] = {0.0f, 0.0f, 0.0f};  // spectrum_to_xyz_with_weights of the solar spectrum
    for (uint32_t b = 0; b < bands; ++b)
        for (int c = 0; c < 3; ++c) white[c] += solar[b] * band_xyz[b * 3 + c];
    float src[3], s_lms[3], t_lms[3], scale[3][3] = {}, tmp[3][3];
    normalized_to_y1(white, src);
    mat3_vec(kBradfordLmsFromXyz, src, s_lms);
    mat3_vec(kBradfordLmsFromXyz, kD65WhiteY1, t_lms);
    for (int i = 0; i < 3; ++i) scale[i][i] = std::fabs(s_lms[i]) > 1.0e-12f ? t_lms[i] / s_lms[i] : 1.0f;
    mat3_mul(scale, kBradfordLmsFromXyz, tmp);
    mat3_mul(kXyzFromBradfordLms, tmp, wb);
}

void host_orthonormal_basis(const float n_in[3], float t[3], float b[3]) {
    float len = std::sqrt(n_in[0] * n_in[0] + n_in[1] * n_in[1] + n_in[2] * n_in[2]);
    float n[3] = {0.0f, 1.0f, 0.0f};
    if (len > 0.0f)
        for (int i = 0; i < 3; ++i) n[i] = n_in[i] / len;
    float sign = n[2] >= 0.0f ? 1.0f : -1.0f;
    float a = -1.0f / (sign + n[2]);
    float bb = n[0] * n[1] * a;
    float tv[3] = {1.0f + sign * n[0] * n[0] * a, sign * bb, -sign * n[0]};
    float bv[3] = {bb, sign + n[1] * n[1] * a, -n[1]};
    float lt = std::sqrt(tv[0] * tv[0] + tv[1] * tv[1] + tv[2] * tv[2]);
    float lb = std::sqrt(bv[0] * bv[0] + bv[1] * bv[1] + bv[2] * bv[2]);
    for (int i = 0; i < 3; ++i) {
        t[i] = lt > 0.0f ? tv[i] / lt : (i == 1 ? 1.0f : 0.0f);
        b[i] = lb > 0.0f ? bv[i] / lb : (i == 1 ? 1.0f : 0.0f);
    }
}

void build_phase_sampling_tables(const float* values, uint32_t band_count, uint32_t bins, std::vector<float>& cdf,
                                 std::vector<float>& bin_pdf, std::vector<uint16_t>* guide) {
    size_t n = size_t(kSpecies) * band_count * bins;
    cdf.assign(n, 0.0f);
    bin_pdf.assign(n, 0.0f);
    if (guide) guide->assign(n, 0);
    auto edge = [bins](uint32_t e) {
        float u = float(e) / float(bins);
        return 1.0f - 2.0f * u * u * u;
    };
    for (uint32_t species = 0; species < kSpecies; ++species) {
        for (uint32_t band = 0; band < band_count; ++band) {
            size_t base = (size_t(species) * band_count + band) * bins;
            float norm = 0.0f;
            for (uint32_t bin = 0; bin < bins; ++bin)
                norm += 2.0f * kPiF * std::max(values[base + bin], 0.0f) * std::fabs(edge(bin) - edge(bin + 1));
            norm = std::max(norm, 1.0e-20f);
            float cumulative = 0.0f;
            for (uint32_t bin = 0; bin < bins; ++bin) {
                float value = std::max(values[base + bin], 0.0f);
                cumulative += 2.0f * kPiF * value * std::fabs(edge(bin) - edge(bin + 1)) / norm;
                cdf[base + bin] = std::min(cumulative, 1.0f);
                bin_pdf[base + bin] = value / norm;
            }
            cdf[base + bins - 1] = 1.0f;
            if (!guide) continue;
            // guide[j]: the first bin whose CDF exceeds (j - 1) / bins, a lower
            // bound of the bin of every xi with floor(xi * bins) = j even when
            // that product rounds up; a forward scan from it finds the same bin
            // as a binary search of the whole row
            uint32_t first = 0;
            for (uint32_t j = 0; j < bins; ++j) {
                const double threshold = (double(j) - 1.0) / double(bins);
                while (first + 1 < bins && double(cdf[base + first]) <= threshold) ++first;
                (*guide)[base + j] = uint16_t(first);
            }
        }
    }
}

std::vector<uint32_t> merge_majorant_layers(const float* maj, uint32_t L, float dz, double crossing_cost) {
    std::vector<double> best(L + 1, 0.0);
    std::vector<uint32_t> from(L + 1, 0);
    for (uint32_t j = 1; j <= L; ++j) {
        best[j] = 1e300;
        double mx = 0.0, sum = 0.0;
        for (uint32_t i = j; i-- > 0;) {  // group [i, j)
            double m = std::max(double(maj[i]), 1e-8);
            mx = std::max(mx, m);
            sum += m;
            double excess = (mx * double(j - i) - sum) * double(dz);
            double c = best[i] + crossing_cost + excess;
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

int build_host_tables(const SkySceneDesc* d, HostTables& out, std::string& err, double crossing_cost) {
    auto fail = [&err](const std::string& msg) {
        err = msg;
        return int(SKY_ERR_INVALID_CONFIG);
    };
    if (!d) return fail("scene descriptor is null");
    if (d->band_count == 0 || d->band_count > kMaxBands)
        return fail("expected between 1 and " + std::to_string(kMaxBands) + " spectral bands, found " +
                    std::to_string(d->band_count));
    if (d->atmosphere_len == 0 || d->aerosol_len == 0)
        return fail("atmosphere and aerosol profiles must not be empty");
    if (d->majorant_layers == 0) return fail("majorant grid must contain at least one layer");
    if (d->majorant_layers > kMaxLayers) return fail("majorant grid has too many layers");
    if (d->phase_bins < 2) return fail("phase tables need at least two bins");
    if (!d->bands || !d->atmosphere || !d->aerosol || !d->aerosol_optics || !d->majorants_km_inv ||
        !d->phase_values)
        return fail("scene descriptor has a null table pointer");
    if (!(d->ground_radius_km > 0.0f) || !(d->atmosphere_radius_km > d->ground_radius_km))
        return fail("atmosphere radius must exceed a positive ground radius");
    if (!(d->top_altitude_km > 0.0f) || !std::isfinite(d->top_altitude_km))
        return fail("majorant grid top altitude must be positive");
    if (!(d->sun_angular_radius_rad > 0.0f) || !(d->sun_angular_radius_rad < 0.5f))
        return fail("sun angular radius must be in (0, 0.5) rad");
    for (uint32_t i = 1; i < d->atmosphere_len; ++i)
        if (d->atmosphere[i].altitude_km < d->atmosphere[i - 1].altitude_km)
            return fail("atmosphere profile must be sorted by altitude");
    for (uint32_t i = 1; i < d->aerosol_len; ++i)
        if (d->aerosol[i].altitude_km < d->aerosol[i - 1].altitude_km)
            return fail("aerosol profile must be sorted by altitude");
    const size_t nmaj = size_t(d->band_count) * d->majorant_layers;
    if (!finite_all(d->majorants_km_inv, nmaj)) return fail("majorant grid contains non-finite values");
    const size_t nphase = size_t(kSpecies) * d->band_count * d->phase_bins;
    if (!finite_all(d->phase_values, nphase)) return fail("phase table contains non-finite values");

    const uint32_t B = d->band_count;
    const float top = d->top_altitude_km;

    // Union knots in [0, top].
    std::vector<float> z{0.0f, top};
    for (uint32_t i = 0; i < d->atmosphere_len; ++i) {
        float a = d->atmosphere[i].altitude_km;
        if (a > 0.0f && a < top) z.push_back(a);
    }
    for (uint32_t i = 0; i < d->aerosol_len; ++i) {
        float a = d->aerosol[i].altitude_km;
        if (a > 0.0f && a < top) z.push_back(a);
    }
    std::sort(z.begin(), z.end());
    z.erase(std::unique(z.begin(), z.end()), z.end());
    if (z.size() > kMaxKnots) return fail("profiles have too many distinct altitudes");
    const uint32_t K = uint32_t(z.size());

    // Band-independent profile values at the knots, then slopes.
    std::vector<float> air(K), oz(K), mass(size_t(K) * kSpecies);
    for (uint32_t k = 0; k < K; ++k) {
        atmosphere_at(d, z[k], air[k], oz[k]);
        aerosol_at(d, z[k], &mass[size_t(k) * kSpecies]);
    }
    out.profile.assign(K, DevProfileKnot{});
    for (uint32_t k = 0; k < K; ++k) {
        DevProfileKnot& P = out.profile[k];
        double dz = k + 1 < K ? double(z[k + 1]) - double(z[k]) : 0.0;
        auto slope = [&](float a, float b) { return dz > 0.0 ? float((double(b) - double(a)) / dz) : 0.0f; };
        uint32_t k1 = std::min(k + 1, K - 1);
        P.air = air[k];
        P.air_slope = slope(air[k], air[k1]);
        P.ozone = oz[k];
        P.ozone_slope = slope(oz[k], oz[k1]);
        for (uint32_t i = 0; i < kSpecies; ++i) {
            P.mass[i] = mass[size_t(k) * kSpecies + i];
            P.mass_slope[i] = slope(mass[size_t(k) * kSpecies + i], mass[size_t(k1) * kSpecies + i]);
        }
    }

    // Per-band constants and extinction tables.
    out.bands.assign(B, DevBand{});
    out.has_xyz = d->band_xyz_weights != nullptr;
    for (uint32_t b = 0; b < B; ++b) {
        DevBand& db = out.bands[b];
        db.solar_radiance = d->bands[b].solar_radiance_w_m2_sr;
        db.rayleigh_xs = d->bands[b].rayleigh_cross_section_m2 * 1000000000.0f;
        db.ozone_xs = d->bands[b].ozone_cross_section_cm2 * 100000.0f;
        for (int c = 0; c < 3; ++c) db.xyz[c] = out.has_xyz ? d->band_xyz_weights[b * 3 + c] : 0.0f;
    }
    out.optics.assign(d->aerosol_optics, d->aerosol_optics + size_t(B) * kSpecies);
    out.sigma_t.assign(size_t(B) * K, float2{0.0f, 0.0f});
    uint32_t aerosol_mask = 0;
    for (uint32_t b = 0; b < B; ++b) {
        std::vector<double> ext(K);
        for (uint32_t k = 0; k < K; ++k) {
            double e = std::max(double(air[k]) * out.bands[b].rayleigh_xs, 0.0) +
                       std::max(double(oz[k]) * out.bands[b].ozone_xs, 0.0);
            for (uint32_t i = 0; i < kSpecies; ++i) {
                const SkyAerosolOptics& o = d->aerosol_optics[b * kSpecies + i];
                double m = mass[size_t(k) * kSpecies + i];
                e += std::max(m * o.scattering_km_inv_per_g_m3, 0.0) + std::max(m * o.absorption_km_inv_per_g_m3, 0.0);
                if (m > 0.0 && (o.scattering_km_inv_per_g_m3 != 0.0f || o.absorption_km_inv_per_g_m3 != 0.0f))
                    aerosol_mask |= 1u << i;
            }
            ext[k] = e;
        }
        for (uint32_t k = 0; k < K; ++k) {
            double dz = k + 1 < K ? double(z[k + 1]) - double(z[k]) : 0.0;
            float slope = dz > 0.0 ? float((ext[k + 1] - ext[k]) / dz) : 0.0f;
            out.sigma_t[size_t(b) * K + k] = float2{float(ext[k]), slope};
        }
    }

    // Finder: interval index at (slightly below) each cell's lower edge.
    out.finder.assign(kFinderCells, 0);
    for (uint32_t c = 0; c < kFinderCells; ++c) {
        double edge = double(c) * double(top) / kFinderCells;
        edge = edge * (1.0 - 1.0e-6) - 1.0e-6;
        uint32_t k = 0;
        while (k + 2 < K && double(z[k + 1]) <= edge) ++k;
        out.finder[c] = uint16_t(k);
    }
    // Per band and finder cell, the knot interval at the cell's lower edge with its next
    // knot: below that knot a lookup needs no search (sigma_t_at).
    out.sig_cell.assign(size_t(B) * kFinderCells, float4{0.0f, 0.0f, 0.0f, 0.0f});
    for (uint32_t b = 0; b < B; ++b)
        for (uint32_t c = 0; c < kFinderCells; ++c) {
            const uint32_t k = out.finder[c];
            const float2 e = out.sigma_t[size_t(b) * K + k];
            const float next = k + 2 < K ? z[k + 1] : std::numeric_limits<float>::infinity();
            out.sig_cell[size_t(b) * kFinderCells + c] = float4{e.x, e.y, z[k], next};
        }
    out.knot_z = z;
    out.majorants.assign(d->majorants_km_inv, d->majorants_km_inv + nmaj);

    // Merged tracking grid per band (compact rows: count + 1 radii, count majorants).
    {
        const uint32_t L = d->majorant_layers;
        const float dzl = top / float(L);
        out.trk_radius.clear();
        out.trk_maj.clear();
        out.trk_map.assign(size_t(B) * L, 0);
        out.trk_count.assign(B, 0);
        out.trk_off.assign(B, 0);
        for (uint32_t b = 0; b < B; ++b) {
            const float* maj = d->majorants_km_inv + size_t(b) * L;
            std::vector<uint32_t> starts = merge_majorant_layers(maj, L, dzl, crossing_cost);
            const uint32_t M = uint32_t(starts.size());
            out.trk_count[b] = M;
            out.trk_off[b] = uint32_t(out.trk_radius.size());
            for (uint32_t m = 0; m < M; ++m) {
                uint32_t k0 = starts[m], k1 = m + 1 < M ? starts[m + 1] : L;
                float mx = 0.0f;
                for (uint32_t k = k0; k < k1; ++k) {
                    mx = std::max(mx, std::max(maj[k], 0.00000001f));
                    out.trk_map[size_t(b) * L + k] = uint16_t(m);
                }
                out.trk_maj.push_back(mx);
                out.trk_radius.push_back(d->ground_radius_km + float(k0) * dzl);
            }
            out.trk_maj.push_back(0.0f);  // keeps both arrays the same length
            out.trk_radius.push_back(d->ground_radius_km + top);
        }
    }

    // Phase tables and their sampling CDFs.
    out.phase_values.assign(d->phase_values, d->phase_values + nphase);
    if (d->phase_bins > 65535u) return fail("phase tables have more than 65535 bins");
    build_phase_sampling_tables(d->phase_values, B, d->phase_bins, out.phase_cdf, out.phase_bin_pdf, &out.phase_guide);

    // Constants.
    DevScene& S = out.scene;
    S.band_count = B;
    S.knot_count = K;
    S.layer_count = d->majorant_layers;
    S.phase_bins = d->phase_bins;
    S.ground_radius = d->ground_radius_km;
    S.atmosphere_radius = d->atmosphere_radius_km;
    S.top_altitude = top;
    S.layer_dz = top / float(d->majorant_layers);
    S.inv_layer_dz = float(d->majorant_layers) / top;
    S.trk_total = uint32_t(out.trk_radius.size());
    S.finder_scale = float(kFinderCells) / top;
    S.ground_albedo = d->ground_albedo;
    float sl = std::sqrt(d->sun_direction[0] * d->sun_direction[0] + d->sun_direction[1] * d->sun_direction[1] +
                         d->sun_direction[2] * d->sun_direction[2]);
    for (int i = 0; i < 3; ++i) S.sun[i] = sl > 0.0f ? d->sun_direction[i] / sl : (i == 1 ? 1.0f : 0.0f);
    host_orthonormal_basis(S.sun, S.sun_t, S.sun_b);
    if (out.has_xyz) {  // rgb = sRGB * (white balance * xyz), folded into one matrix
        std::vector<float> solar(B);
        for (uint32_t b = 0; b < B; ++b) solar[b] = d->bands[b].solar_radiance_w_m2_sr;
        float wb[3][3], m[3][3];
        solar_d65_white_balance(solar.data(), d->band_xyz_weights, B, wb);
        mat3_mul(kSrgbFromXyz, wb, m);
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) S.rgb_from_xyz[r * 3 + c] = m[r][c];
    }
    S.cos_max = std::cos(d->sun_angular_radius_rad);
    S.one_minus_cos_max = 1.0f - S.cos_max;
    S.light_pdf = 1.0f / (kTauF * (1.0f - S.cos_max));
    S.aerosol_mask = aerosol_mask;
    return SKY_OK;
}

}  // namespace sky
