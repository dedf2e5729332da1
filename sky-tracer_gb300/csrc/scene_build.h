// scene_build.h — host-side preparation of a SkySceneDesc into the device
// table layout of sky_scene.h.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "sky_scene.h"

namespace sky {

struct HostTables {
    DevScene scene{};  // sizes and constants; table pointers filled at upload
    std::vector<float> knot_z;
    std::vector<uint16_t> finder;
    std::vector<float2> sigma_t;
    std::vector<float4> sig_cell;
    std::vector<float> majorants;
    std::vector<DevBand> bands;
    std::vector<DevProfileKnot> profile;
    std::vector<SkyAerosolOptics> optics;
    std::vector<float> phase_values, phase_cdf, phase_bin_pdf;
    std::vector<uint16_t> phase_guide;
    std::vector<float> trk_radius, trk_maj;
    std::vector<uint16_t> trk_map;
    std::vector<uint32_t> trk_count, trk_off;
    bool has_xyz = false;
};

// Relative cost of one layer crossing against one null collision, used to
// merge majorant layers for SKY_TRACKING_MERGED_LAYERS (0.1: the fastest
// setting of the wavefront kernel on a 512x256, 81-band, 256-spp render).
constexpr double kDefaultCrossingCost = 0.1;

// Partition the `layers` uniform majorant layers of one band into contiguous
// groups minimising  sum_groups [crossing_cost + dz * sum_k (max_group - maj_k)],
// i.e. crossings plus the extra null collisions of a vertical ray.  Returns
// the first uniform layer of each group (ascending, starting at 0).
std::vector<uint32_t> merge_majorant_layers(const float* maj, uint32_t layers, float dz, double crossing_cost);

// Validates `desc` (the checks of integrator.rs:130-163 and :401-407, with
// the band and bin counts as run-time values) and fills `out`.  Returns
// SKY_OK or SKY_ERR_INVALID_CONFIG with a message in `err`.
int build_host_tables(const SkySceneDesc* desc, HostTables& out, std::string& err,
                      double crossing_cost = kDefaultCrossingCost);

// MiePhaseTable sampling tables (phase.rs:105-135): per (species, band) the
// CDF over the cube-root mu bins and the per-bin pdf.
void build_phase_sampling_tables(const float* values, uint32_t band_count, uint32_t bins, std::vector<float>& cdf,
                                 std::vector<float>& bin_pdf, std::vector<uint16_t>* guide = nullptr);

// orthonormal_basis (sky_trace.wgsl:512-520) evaluated on the host.
void host_orthonormal_basis(const float n_in[3], float t[3], float b[3]);

// Bradford white balance from the solar spectrum's white to D65
// (SpectralRgbConverter::new_solar_d65, spectrum.rs:132-147): a 3x3 XYZ->XYZ
// matrix from per-band solar values and CIE weights [bands][3].
void solar_d65_white_balance(const float* solar, const float* band_xyz, uint32_t bands, float wb[3][3]);

}  // namespace sky
