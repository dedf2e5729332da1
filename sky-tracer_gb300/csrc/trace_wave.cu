// trace_wave.cu — the launch sequence of the wavefront tracer: prepare (zero
// the sums of jobs that do not accumulate, reset the work counter), trace
// (trace_wave.cuh, instantiated per tracking mode in trace_wave_*.cu) and
// finalize (film, XYZ, variance, linear sRGB of every job).

#include <algorithm>

#include "trace_kernels.h"

namespace sky {
namespace {

// Zero the sums of every job that does not accumulate (blockIdx.y = job) and
// reset the work counter.
__global__ void __launch_bounds__(256) wave_prepare_kernel(const DevJob* __restrict__ jobs,
                                                           uint32_t* __restrict__ work_counter) {
    const DevJob& J = jobs[blockIdx.y];
    if (blockIdx.x == 0u && blockIdx.y == 0u && threadIdx.x == 0u) *work_counter = 0u;
    if (J.accumulate) return;
    double* sum = J.cell_sum;
    double* sq = J.cell_sumsq;
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < J.cell_count;
         i += uint64_t(gridDim.x) * blockDim.x) {
        sum[i] = 0.0;
        if (sq) sq[i] = 0.0;
    }
}

}  // namespace

cudaError_t launch_trace_wave(const WaveLaunch& w, cudaStream_t stream) {
    if (w.num_jobs == 0u || w.num_jobs > 65535u || w.total_cells == 0u) return cudaErrorInvalidValue;
    const uint32_t xblocks =
        uint32_t(std::min<uint64_t>((uint64_t(w.max_job_cells) + 255u) / 256u, 1024u));
    wave_prepare_kernel<<<dim3(std::max(xblocks, 1u), w.num_jobs), 256, 0, stream>>>(w.jobs, w.work_counter);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    switch (w.tracking) {
        case SKY_TRACKING_SEGMENT_RESTART: e = launch_wave_segment_restart(w, stream); break;
        case SKY_TRACKING_RESIDUAL_CARRY: e = launch_wave_residual_carry(w, stream); break;
        case SKY_TRACKING_MERGED_LAYERS: e = launch_wave_merged_layers(w, stream); break;
        default: return cudaErrorInvalidValue;
    }
    if (e != cudaSuccess) return e;
    return launch_finalize_jobs(w.scene, w.jobs, w.num_jobs, w.total_cells, stream);
}

}  // namespace sky
