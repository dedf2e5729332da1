// score_kernels.h — launchers of the combination-score kernels (score.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace sky {

constexpr uint32_t kScoreHistBins = 2048;  // widest radix-selection pass: 11 bits

// dist[c][s] = Oklab distance of combination c at sample s (NaN when not
// finite); sums[c] += (sum, sum of squares, count) of the finite distances.
cudaError_t launch_score_distances(const float* bands, uint64_t samples, const float* ref_lab, float inv_scale,
                                   const uint32_t* combo_bands, const float* combo_xyz, uint32_t combos,
                                   uint32_t channels, float* dist, double* sums, cudaStream_t stream);

// hist[t][bin] += count of finite distances of combination target_combo[t]
// whose bits above shift + width equal target_prefix[t], binned by
// bits [shift, shift + width).
cudaError_t launch_select_hist(const float* dist, uint64_t samples, const uint32_t* target_combo,
                               const uint32_t* target_prefix, uint32_t targets, uint32_t shift, uint32_t width,
                               uint32_t* hist, uint32_t sms, cudaStream_t stream);

}  // namespace sky
