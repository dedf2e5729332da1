// trace_kernels.h — host-callable launchers of the tracing kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "sky_scene.h"

namespace sky {

// Plain tracer: writes per-cell sums / sums of squares of this launch's
// samples into cell_sum / cell_sumsq, or adds to them when `accumulate`.
cudaError_t launch_trace_plain(const DevScene& S, const DevLaunch& L, double* cell_sum, double* cell_sumsq,
                               unsigned long long* counters, uint32_t* status, bool accumulate,
                               cudaStream_t stream);

// Shared-memory plan of the persistent kernel (byte offsets and sizes).
struct StageLayout {
    uint32_t jobs, acc, max_cells;
    uint32_t knot_z, finder, sigma_t, bands, trk_radius, trk_maj, trk_map, trk_count, trk_off, majorants;
    uint32_t knot_z_bytes, finder_bytes, sigma_t_bytes, bands_bytes, trk_bytes, trk_map_bytes, trk_count_bytes,
        majorants_bytes;
    uint32_t total;
};

// Everything one persistent launch needs.
struct WaveLaunch {
    const DevJob* jobs;           // device array of num_jobs jobs, ascending group_begin
    uint32_t num_jobs;
    uint32_t total_groups;
    StageLayout layout;
    bool staged;                  // tables staged in shared memory (all jobs share them)
    uint32_t smem_bytes;
    uint32_t block_threads;       // 256
    uint32_t max_blocks_per_sm;   // 0 = as many as fit
    uint32_t tracking, phase_sampling;
    uint32_t* work_counter;       // zeroed before the launch
    unsigned long long* counters; // may be null
    uint32_t* status;
};

constexpr uint32_t kWaveBlockThreads = 256;

// Persistent regenerating tracer over a job table.  Writes cell sums, film
// and XYZ of every job directly (no finalize launch needed).
cudaError_t launch_trace_wavefront(const WaveLaunch& w, cudaStream_t stream);

StageLayout plan_stage_layout(const DevScene& S, uint32_t warps, uint32_t max_cells, bool with_majorants,
                              bool stage_tables);

// Mean film, XYZ and XYZ variance from the per-cell sums (any output may be
// null; xyz_var needs cell_sumsq).
cudaError_t launch_finalize(const DevScene& S, uint64_t pixels, uint32_t total_spp, const double* cell_sum,
                            const double* cell_sumsq, float* film, double* xyz, double* xyz_var,
                            cudaStream_t stream);

}  // namespace sky
