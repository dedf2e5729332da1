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
    std::vector<float> majorants;
    std::vector<DevBand> bands;
    std::vector<DevProfileKnot> profile;
    std::vector<SkyAerosolOptics> optics;
    std::vector<float> phase_values, phase_cdf, phase_bin_pdf;
    bool has_xyz = false;
};

// Validates `desc` (the checks of integrator.rs:130-163 and :401-407, with
// the band and bin counts as run-time values) and fills `out`.  Returns
// SKY_OK or SKY_ERR_INVALID_CONFIG with a message in `err`.
int build_host_tables(const SkySceneDesc* desc, HostTables& out, std::string& err);

// MiePhaseTable sampling tables (phase.rs:105-135): per (species, band) the
// CDF over the cube-root mu bins and the per-bin pdf.
void build_phase_sampling_tables(const float* values, uint32_t band_count, uint32_t bins, std::vector<float>& cdf,
                                 std::vector<float>& bin_pdf);

// orthonormal_basis (sky_trace.wgsl:512-520) evaluated on the host.
void host_orthonormal_basis(const float n_in[3], float t[3], float b[3]);

}  // namespace sky
