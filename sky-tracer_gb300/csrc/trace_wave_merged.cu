// trace_wave_merged.cu — the wavefront kernels of merged-layer tracking (the default).

#include "trace_wave.cuh"

namespace sky {

cudaError_t launch_wave_merged_layers(const WaveLaunch& w, cudaStream_t stream) {
    return wave::launch_wave_tracking<SKY_TRACKING_MERGED_LAYERS>(w, stream);
}

}  // namespace sky
