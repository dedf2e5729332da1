// probe.cu — the tracer's FP32 ray-shell geometry evaluated for caller rays
// (sky_cuda_probe_shell_geometry).  A diagnostic: it runs the same inlined
// device functions the tracking kernels run (ray_geo, half_chord,
// altitude_at from sky_device.cuh), so that the error of the FP32
// impact-parameter form against an FP64 evaluation of the reference's
// quadratic (sky_trace.wgsl:211-221) can be measured on grazing rays.

#include "sky_device.cuh"
#include "trace_kernels.h"

namespace sky {
namespace {

__global__ void __launch_bounds__(256) shell_probe_kernel(const float* __restrict__ origins,
                                                          const float* __restrict__ directions, uint32_t rays,
                                                          const float* __restrict__ radii, uint32_t shells,
                                                          float ground_radius, float* __restrict__ t_out,
                                                          float* __restrict__ alt_out) {
    const uint64_t k = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= uint64_t(rays) * shells) return;
    const uint32_t i = uint32_t(k / shells), j = uint32_t(k - uint64_t(i) * shells);
    const V3 o = load3(origins + 3u * i), d = load3(directions + 3u * i);
    const RayGeo g = ray_geo(o, d);
    const float q = half_chord(__ldg(radii + j), g.p);
    float t[2] = {nanf(""), nanf("")}, a[2] = {nanf(""), nanf("")};
    if (q >= 0.0f) {
        t[0] = -q - g.b;  // the crossings as merged_crossing and next_boundary form them
        t[1] = q - g.b;
        a[0] = altitude_at(g, t[0], ground_radius);
        a[1] = altitude_at(g, t[1], ground_radius);
    }
    t_out[2 * k] = t[0];
    t_out[2 * k + 1] = t[1];
    alt_out[2 * k] = a[0];
    alt_out[2 * k + 1] = a[1];
}

}  // namespace

cudaError_t launch_shell_probe(const float* origins, const float* directions, uint32_t rays, const float* radii,
                               uint32_t shells, float ground_radius, float* t_out, float* alt_out,
                               cudaStream_t stream) {
    const uint64_t blocks = (uint64_t(rays) * shells + 255u) / 256u;
    if (blocks == 0 || blocks > 0x7fffffffull) return cudaErrorInvalidValue;
    shell_probe_kernel<<<dim3(uint32_t(blocks)), 256, 0, stream>>>(origins, directions, rays, radii, shells,
                                                                   ground_radius, t_out, alt_out);
    return cudaGetLastError();
}

}  // namespace sky
