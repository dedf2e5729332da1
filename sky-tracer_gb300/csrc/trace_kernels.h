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

// Mean film, XYZ and XYZ variance from the per-cell sums (any output may be
// null; xyz_var needs cell_sumsq).
cudaError_t launch_finalize(const DevScene& S, uint64_t pixels, uint32_t total_spp, const double* cell_sum,
                            const double* cell_sumsq, float* film, double* xyz, double* xyz_var,
                            cudaStream_t stream);

}  // namespace sky
