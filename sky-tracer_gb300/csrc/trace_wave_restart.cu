// trace_wave_restart.cu — the wavefront kernels of segment-restart tracking (the reference's).

#include "trace_wave.cuh"

namespace sky {

cudaError_t launch_wave_segment_restart(const WaveLaunch& w, cudaStream_t stream) {
    return wave::launch_wave_tracking<SKY_TRACKING_SEGMENT_RESTART>(w, stream);
}

}  // namespace sky
