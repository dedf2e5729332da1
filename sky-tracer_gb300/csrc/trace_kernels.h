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

// Block path pool of the persistent wavefront kernel (trace_pool.cu).
constexpr uint32_t kPoolThreads = 256;
constexpr uint32_t kPoolMaxSlotsPerThread = 4;  // variant 0: 4 slots/thread, 2 blocks/SM; 1: 2 and 3
constexpr uint32_t kPoolRing = 4;         // work groups in flight per block
constexpr uint32_t kPoolMaxCells = 256;   // (pixel, band) cells per work group

struct PoolLayout {
    uint32_t header, jobs, acc, slots, lists, staged;
    uint32_t knot_z, finder, sigma_t, bands, trk_radius, trk_maj, trk_map, trk_count, trk_off, majorants;
    uint32_t knot_z_bytes, finder_bytes, sigma_t_bytes, bands_bytes, trk_bytes, trk_map_bytes, trk_count_bytes,
        majorants_bytes;
    uint32_t total;
};

struct PoolLaunch {
    const DevJob* jobs;            // device array, ascending group_begin
    uint32_t num_jobs;
    uint32_t total_groups;
    PoolLayout layout;
    uint32_t max_blocks_per_sm;    // 0 = as many as fit
    uint32_t variant;              // pool shape (slots per thread, blocks per SM)
    uint32_t tracking, phase_sampling;
    uint32_t* work_counter;        // zeroed before the launch
    unsigned long long* counters;  // may be null
    uint32_t* status;
};

// Persistent wavefront tracer over a job table.  Writes the cell sums, film
// and XYZ of every job directly (no finalize launch needed).
cudaError_t launch_trace_pool(const PoolLaunch& w, cudaStream_t stream);
PoolLayout plan_pool_layout(const DevScene& S, bool with_majorants, bool stage_tables, uint32_t variant);
uint32_t pool_slots_per_thread(uint32_t variant);

// Mean film, XYZ, XYZ variance and linear sRGB from the per-cell sums (any
// output may be null; xyz_var needs cell_sumsq).
cudaError_t launch_finalize(const DevScene& S, uint64_t pixels, uint32_t total_spp, const double* cell_sum,
                            const double* cell_sumsq, float* film, double* xyz, double* xyz_var, float* rgb,
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

// rgb = M xyz in FP64, stored as float; black when any component is not
// finite (Rgb::finite_or_black, math.rs:137-143).
__device__ __forceinline__ void store_rgb(const RgbMatrix& M, const double xyz[3], float* out) {
    float f[3];
    bool finite = true;
    for (int r = 0; r < 3; ++r) {
        f[r] = float(double(M.m[r * 3]) * xyz[0] + double(M.m[r * 3 + 1]) * xyz[1] + double(M.m[r * 3 + 2]) * xyz[2]);
        finite = finite && isfinite(f[r]);
    }
    for (int r = 0; r < 3; ++r) out[r] = finite ? f[r] : 0.0f;
}

}  // namespace sky
