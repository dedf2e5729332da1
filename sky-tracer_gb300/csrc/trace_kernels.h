// trace_kernels.h — host-callable launchers of the tracing kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "sky_scene.h"

namespace sky {

// Aerosol species the tracing kernels evaluate for a scene: 1 when species
// 1-3 carry no aerosol (DevScene::aerosol_mask), else all four; `all_species`
// (SkyTuning) asks for all four always.  Either count gives the same results.
inline uint32_t aerosol_species(const DevScene& S, bool all_species) {
    return (all_species || (S.aerosol_mask & ~1u) != 0u) ? kSpecies : 1u;
}

// Plain tracer: writes per-cell sums / sums of squares of this launch's
// samples into cell_sum / cell_sumsq, or adds to them when `accumulate`.
cudaError_t launch_trace_plain(const DevScene& S, const DevLaunch& L, double* cell_sum, double* cell_sumsq,
                               unsigned long long* counters, uint32_t* status, bool accumulate,
                               uint32_t aerosol_species, cudaStream_t stream);

// Persistent wavefront tracer (trace_wave.cu): a ray loop with per-lane chain
// regeneration over a job table.
constexpr uint32_t kWaveThreads = 256;
constexpr uint32_t kWaveVariants = 3;  // resident blocks per SM: variant 0 -> 3, 1 -> 2, 2 -> 4

struct WaveLaunch {
    DevScene scene;                // the first job's scene: its tables and constants are every job's
                                   // (jobs differ in their sun frame only)
    DevLaunch launch0;             // the first job's launch constants
    const DevJob* jobs;            // device array, ascending cell_begin
    uint32_t num_jobs;             // at most 65535
    uint32_t total_cells;          // sum of the jobs' cell counts
    uint32_t max_job_cells;        // cells of the largest job
    uint32_t variant;              // kernel shape, < kWaveVariants
    uint32_t max_blocks_per_sm;    // 0 = as many as fit
    uint32_t tracking, phase_sampling;
    uint32_t aerosol_species;      // 1 or kSpecies (aerosol_species())
    uint32_t* work_counter;        // reset by the launch itself
    unsigned long long* counters;  // may be null
    uint32_t* status;
    uint32_t iteration_limit;      // loop iterations per warp before status bit 2 (SkyTuning.iteration_limit)
};

// Prepare, trace and finalize every job of `w` (three kernels on `stream`):
// the jobs' cell sums (zeroed first unless a job accumulates), film, XYZ,
// XYZ variance and linear sRGB.
cudaError_t launch_trace_wave(const WaveLaunch& w, cudaStream_t stream);
// The tracing kernel alone, per tracking mode (trace_wave_*.cu).
cudaError_t launch_wave_segment_restart(const WaveLaunch& w, cudaStream_t stream);
cudaError_t launch_wave_residual_carry(const WaveLaunch& w, cudaStream_t stream);
cudaError_t launch_wave_merged_layers(const WaveLaunch& w, cudaStream_t stream);

// Mean film, XYZ, XYZ variance and linear sRGB from the per-cell sums (any
// output may be null; xyz_var needs cell_sumsq).
cudaError_t launch_finalize(const DevScene& S, uint64_t pixels, uint32_t total_spp, const double* cell_sum,
                            const double* cell_sumsq, float* film, double* xyz, double* xyz_var, float* rgb,
                            cudaStream_t stream);

// The same for every job of a job table (four lanes per pixel of the jobs'
// concatenated pixels; jobs without film / XYZ / RGB outputs are skipped).
cudaError_t launch_finalize_jobs(const DevScene& S, const DevJob* jobs, uint32_t num_jobs, uint32_t total_cells,
                                 cudaStream_t stream);

// The tracer's FP32 shell crossings and altitudes for caller rays (probe.cu):
// t_out / alt_out [ray][shell][near, far], NaN where a ray misses a shell.
cudaError_t launch_shell_probe(const float* origins, const float* directions, uint32_t rays, const float* radii,
                               uint32_t shells, float ground_radius, float* t_out, float* alt_out,
                               cudaStream_t stream);

// XYZ -> white-balanced linear sRGB of a scene (kernel argument copy).
struct RgbMatrix {
    float m[9];
};
__host__ __device__ inline RgbMatrix rgb_matrix(const DevScene& S) {
    RgbMatrix r;
    for (int i = 0; i < 9; ++i) r.m[i] = S.rgb_from_xyz[i];
    return r;
}

}  // namespace sky
