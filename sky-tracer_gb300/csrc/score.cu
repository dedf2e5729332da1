// score.cu — the wavelength optimizer's combination score on the GPU.
//
// sky-wavelength-optimizer scores a combination of primary bands by
// rebuilding every sample's XYZ from the selected bands
// (xyz = sum_ch band[idx_ch][s] * c_ch, c_ch = weight_nm / band_width * CIE),
// mapping it and the full-spectrum reference to Oklab at a common scale, and
// summarising the per-sample distances: mean, RMS, the p50/p90/p95/p99
// percentiles of the sorted finite distances (element round((n-1) q)) and
// the maximum; score = rmse + 0.25 p95 (main.rs:414-488, 1121-1156).
//
// Here one launch computes every sample's distance for a batch of
// combinations (one thread per (sample, combination)) with block-level FP64
// sums, and the percentiles are exact order statistics found by radix
// selection over the distances' IEEE bits (non-negative floats order like
// their bit patterns): an 11-bit, an 11-bit and a 10-bit histogram pass.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "score_kernels.h"

namespace sky {
namespace {

__device__ __forceinline__ float signed_cbrt(float x) {
    const float a = fabsf(x);
    const float r = a > 0.0f ? exp2f(__log2f(a) * (1.0f / 3.0f)) : a;  // keeps 0 and NaN
    return copysignf(r, x);
}

// Oklab of XYZ (Ottosson's published matrices), main.rs:1121-1130.
__device__ __forceinline__ void xyz_to_oklab(float x, float y, float z, float lab[3]) {
    const float l = signed_cbrt(0.8189330101f * x + 0.3618667424f * y - 0.1288597137f * z);
    const float m = signed_cbrt(0.0329845436f * x + 0.9293118715f * y + 0.0361456387f * z);
    const float s = signed_cbrt(0.0482003018f * x + 0.2643662691f * y + 0.6338517070f * z);
    lab[0] = 0.2104542553f * l + 0.7936177850f * m - 0.0040720468f * s;
    lab[1] = 1.9779984951f * l - 2.4285922050f * m + 0.4505937099f * s;
    lab[2] = 0.0259040371f * l + 0.7827717662f * m - 0.8086757660f * s;
}

__device__ __forceinline__ double block_sum(double v, double* scratch) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) scratch[warp] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (uint32_t w = 0; w < blockDim.x / 32u; ++w) t += scratch[w];
    return t;
}

// Distances of combination blockIdx.y for 256 samples; FP64 sum, sum of
// squares and count of the finite ones.
__global__ void __launch_bounds__(256) distance_kernel(const float* __restrict__ bands, uint64_t samples,
                                                       const float* __restrict__ ref_lab, float inv_scale,
                                                       const uint32_t* __restrict__ combo_bands,
                                                       const float* __restrict__ combo_xyz, uint32_t channels,
                                                       float* __restrict__ dist, double* __restrict__ sums) {
    __shared__ double scratch[8];
    const uint32_t c = blockIdx.y;
    const uint64_t s = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    double d = 0.0, d2 = 0.0, ok = 0.0;
    if (s < samples) {
        float x = 0.0f, y = 0.0f, z = 0.0f;
        for (uint32_t ch = 0; ch < channels; ++ch) {
            const float v = __ldg(bands + uint64_t(__ldg(combo_bands + c * channels + ch)) * samples + s);
            const float* w = combo_xyz + (size_t(c) * channels + ch) * 3u;
            x = fmaf(v, __ldg(w), x);
            y = fmaf(v, __ldg(w + 1), y);
            z = fmaf(v, __ldg(w + 2), z);
        }
        float lab[3];
        xyz_to_oklab(x * inv_scale, y * inv_scale, z * inv_scale, lab);
        const float dl = lab[0] - __ldg(ref_lab + s * 3), da = lab[1] - __ldg(ref_lab + s * 3 + 1),
                    db = lab[2] - __ldg(ref_lab + s * 3 + 2);
        float e = sqrtf(dl * dl + da * da + db * db);
        if (!isfinite(e)) {
            e = __int_as_float(0x7fffffff);  // NaN: not counted, not selected
        } else {
            d = e;
            d2 = double(e) * double(e);
            ok = 1.0;
        }
        dist[size_t(c) * samples + s] = e;
    }
    d = block_sum(d, scratch);
    d2 = block_sum(d2, scratch);
    ok = block_sum(ok, scratch);
    if (threadIdx.x == 0) {
        atomicAdd(sums + c * 3, d);
        atomicAdd(sums + c * 3 + 1, d2);
        atomicAdd(sums + c * 3 + 2, ok);
    }
}

// One radix-selection pass: for target blockIdx.y (its combination, the bits
// already fixed above `shift + width`), the histogram of the next `width` bits
// of the distances that share that prefix.
__global__ void __launch_bounds__(256) select_hist_kernel(const float* __restrict__ dist, uint64_t samples,
                                                          const uint32_t* __restrict__ target_combo,
                                                          const uint32_t* __restrict__ target_prefix,
                                                          uint32_t shift, uint32_t width,
                                                          uint32_t* __restrict__ hist) {
    __shared__ uint32_t h[kScoreHistBins];
    const uint32_t t = blockIdx.y;
    const uint32_t bins = 1u << width;
    for (uint32_t i = threadIdx.x; i < bins; i += blockDim.x) h[i] = 0u;
    __syncthreads();
    const uint32_t c = target_combo[t];
    const uint32_t top = shift + width;  // bits at and above `top` must equal the prefix
    const uint32_t prefix = target_prefix[t];
    const float* row = dist + size_t(c) * samples;
    for (uint64_t s = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; s < samples;
         s += uint64_t(gridDim.x) * blockDim.x) {
        const float e = __ldg(row + s);
        if (!(e == e)) continue;  // NaN
        const uint32_t bits = __float_as_uint(e);
        if (top < 32u && (bits >> top) != prefix) continue;
        atomicAdd(&h[(bits >> shift) & (bins - 1u)], 1u);
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < bins; i += blockDim.x)
        if (h[i]) atomicAdd(hist + size_t(t) * kScoreHistBins + i, h[i]);
}

}  // namespace

cudaError_t launch_score_distances(const float* bands, uint64_t samples, const float* ref_lab, float inv_scale,
                                   const uint32_t* combo_bands, const float* combo_xyz, uint32_t combos,
                                   uint32_t channels, float* dist, double* sums, cudaStream_t stream) {
    const dim3 grid(uint32_t((samples + 255) / 256), combos);
    distance_kernel<<<grid, 256, 0, stream>>>(bands, samples, ref_lab, inv_scale, combo_bands, combo_xyz, channels,
                                              dist, sums);
    return cudaGetLastError();
}

cudaError_t launch_select_hist(const float* dist, uint64_t samples, const uint32_t* target_combo,
                               const uint32_t* target_prefix, uint32_t targets, uint32_t shift, uint32_t width,
                               uint32_t* hist, uint32_t sms, cudaStream_t stream) {
    const uint32_t per_target = uint32_t(std::min<uint64_t>((samples + 255) / 256, std::max(1u, 4u * sms)));
    const dim3 grid(per_target, targets);
    select_hist_kernel<<<grid, 256, 0, stream>>>(dist, samples, target_combo, target_prefix, shift, width, hist);
    return cudaGetLastError();
}

}  // namespace sky
