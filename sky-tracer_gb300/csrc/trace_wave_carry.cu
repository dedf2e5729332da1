// trace_wave_carry.cu — the wavefront kernels of residual-carry tracking.

#include "trace_wave.cuh"

namespace sky {

cudaError_t launch_wave_residual_carry(const WaveLaunch& w, cudaStream_t stream) {
    return wave::launch_wave_tracking<SKY_TRACKING_RESIDUAL_CARRY>(w, stream);
}

}  // namespace sky
