// finalize.cu — per-pixel epilogue: mean film (the reference's
// `values *= 1/spp; max(0)`, integrator.rs:306-310), CIE XYZ of the mean
// spectrum (spectrum_to_xyz_with_weights, spectrum.rs:232-241, FP64) and the
// variance of that XYZ estimate from the per-band sums of squares, and the
// white-balanced linear sRGB of that XYZ (film_output.rs:96-124 on the host
// in the reference).
//
// The epilogue reads 16 B and writes 4 B per (pixel, band), but its FP64
// arithmetic, not HBM, bounds it on this part (FP64 runs at ~2 FMA per clock
// per SM).  So a group of kGroup = 4 lanes shares a pixel: the group's lanes
// stride over the bands (each group load is one 32-byte sector, the film
// stores of a warp's eight groups fill whole sectors), the band weights sit
// in shared memory already in FP64 (no conversion per cell), the divisions by
// the sample count are reciprocals taken once, and the cross-lane sum is two
// shuffle steps instead of five.  The group's lanes 0-2 then store X, Y, Z
// (and the variance and sRGB components) of their pixel: a warp's XYZ store
// is one coalesced 192-byte write.

#include "trace_kernels.h"

namespace sky {
namespace {

constexpr uint32_t kGroup = 4;                       // lanes per pixel
constexpr uint32_t kFinalizeThreads = 256;
constexpr uint32_t kPixelsPerBlock = kFinalizeThreads / kGroup;

struct BandWeights {
    double w[3];   // CIE x, y, z weight of the band
    double w2[3];  // their squares (the variance of a weighted sum)
};

// The band weights of the scene, widened to FP64 once per block.
__device__ __forceinline__ void stage_weights(const DevBand* __restrict__ bands, uint32_t band_count,
                                              BandWeights* W) {
    for (uint32_t b = threadIdx.x; b < band_count; b += blockDim.x) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double w = double(bands[b].xyz[c]);
            W[b].w[c] = w;
            W[b].w2[c] = w * w;
        }
    }
    __syncthreads();
}

__device__ __forceinline__ double group_sum(double v) {
    v += __shfl_xor_sync(0xffffffffu, v, 2);
    v += __shfl_xor_sync(0xffffffffu, v, 1);
    return v;
}

__device__ __forceinline__ double pick3(const double v[3], uint32_t c) { return c == 0 ? v[0] : c == 1 ? v[1] : v[2]; }

// One pixel by the kGroup lanes of a group (every lane of the warp takes part
// in the shuffles; `active` is false for the lanes past the last pixel).
// inv_n = 1 / n and inv_var = 1 / (n (n - 1)) for n samples per cell.
__device__ __forceinline__ void finalize_pixel(const BandWeights* W, uint32_t band_count, bool active, uint64_t pixel,
                                               double inv_n, double inv_var, const double* __restrict__ cell_sum,
                                               const double* __restrict__ cell_sumsq, float* __restrict__ film,
                                               double* __restrict__ xyz, double* __restrict__ xyz_var,
                                               float* __restrict__ rgb, const RgbMatrix& m) {
    const uint32_t lane = threadIdx.x & 31u, g = lane & (kGroup - 1u);
    double acc[3] = {0.0, 0.0, 0.0}, var[3] = {0.0, 0.0, 0.0};
    // the variance is zero without sums of squares or with one sample per cell
    const bool want_var = xyz_var && cell_sumsq && inv_var > 0.0;
    if (active) {
        const uint64_t base = pixel * band_count;
#pragma unroll 4
        for (uint32_t b = g; b < band_count; b += kGroup) {
            const double s = cell_sum[base + b];
            const double mean = s * inv_n;
            if (film) film[base + b] = fmaxf(float(mean), 0.0f);
            const BandWeights& bw = W[b];
#pragma unroll
            for (int c = 0; c < 3; ++c) acc[c] = fma(mean, bw.w[c], acc[c]);
            if (want_var) {
                // (sumsq - sum * mean) / (n - 1) / n, clamped at zero
                const double v = fmax(fma(-s, mean, cell_sumsq[base + b]), 0.0) * inv_var;
#pragma unroll
                for (int c = 0; c < 3; ++c) var[c] = fma(v, bw.w2[c], var[c]);
            }
        }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        acc[c] = group_sum(acc[c]);
        if (want_var) var[c] = group_sum(var[c]);
    }
    // lane c < 3 of the group stores component c
    const uint32_t c = g;
    float f = 0.0f;
    bool finite = true;
    if (rgb && c < 3u) {
        // rgb = M xyz in FP64, stored as float; black when any component is not
        // finite (Rgb::finite_or_black, math.rs:137-143)
        const float r0 = c == 0u ? m.m[0] : c == 1u ? m.m[3] : m.m[6];  // row c of M, by selects
        const float r1 = c == 0u ? m.m[1] : c == 1u ? m.m[4] : m.m[7];
        const float r2 = c == 0u ? m.m[2] : c == 1u ? m.m[5] : m.m[8];
        f = float(double(r0) * acc[0] + double(r1) * acc[1] + double(r2) * acc[2]);
        finite = isfinite(f);
    }
    const uint32_t ok = __ballot_sync(0xffffffffu, finite);
    if (!active || c >= 3u) return;
    if (xyz) xyz[pixel * 3 + c] = pick3(acc, c);
    if (xyz_var) xyz_var[pixel * 3 + c] = pick3(var, c);
    if (rgb) {
        const uint32_t group_bits = (ok >> (lane & ~(kGroup - 1u))) & 0x7u;
        rgb[pixel * 3 + c] = group_bits == 0x7u ? f : 0.0f;
    }
}

__global__ void __launch_bounds__(kFinalizeThreads) finalize_kernel(
    const DevBand* __restrict__ bands, uint32_t band_count, uint64_t pixels, double inv_n, double inv_var,
    const double* __restrict__ cell_sum, const double* __restrict__ cell_sumsq, float* __restrict__ film,
    double* __restrict__ xyz, double* __restrict__ xyz_var, float* __restrict__ rgb, RgbMatrix m) {
    __shared__ BandWeights W[kMaxBands];
    stage_weights(bands, band_count, W);
    const uint64_t pixel = uint64_t(blockIdx.x) * kPixelsPerBlock + threadIdx.x / kGroup;
    finalize_pixel(W, band_count, pixel < pixels, pixel, inv_n, inv_var, cell_sum, cell_sumsq, film, xyz, xyz_var,
                   rgb, m);
}

// Pixels of all jobs in a row; the job of a pixel by binary search over the
// jobs' first cells (every job's cell range is a whole number of pixels).
__global__ void __launch_bounds__(kFinalizeThreads) finalize_jobs_kernel(
    const DevBand* __restrict__ bands, uint32_t band_count, const DevJob* __restrict__ jobs, uint32_t num_jobs,
    uint64_t total_pixels, RgbMatrix m) {
    __shared__ BandWeights W[kMaxBands];
    stage_weights(bands, band_count, W);
    const uint64_t gp = uint64_t(blockIdx.x) * kPixelsPerBlock + threadIdx.x / kGroup;
    const bool in_range = gp < total_pixels;
    const uint64_t gc = (in_range ? gp : 0u) * band_count;
    uint32_t lo = 0u, hi = num_jobs;
    while (hi - lo > 1u) {
        const uint32_t mid = (lo + hi) >> 1;
        if (jobs[mid].cell_begin <= gc) lo = mid;
        else hi = mid;
    }
    const DevJob& J = jobs[lo];
    const bool active = in_range && (J.film || J.xyz || J.xyz_var || J.rgb);
    const double n = double(J.total_spp);
    const double inv_n = 1.0 / n, inv_var = J.total_spp > 1u ? inv_n / (n - 1.0) : 0.0;
    finalize_pixel(W, band_count, active, (gc - J.cell_begin) / band_count, inv_n, inv_var, J.cell_sum, J.cell_sumsq,
                   J.film, J.xyz, J.xyz_var, J.rgb, m);
}

uint32_t finalize_blocks(uint64_t pixels) { return uint32_t((pixels + kPixelsPerBlock - 1) / kPixelsPerBlock); }

}  // namespace

cudaError_t launch_finalize(const DevScene& S, uint64_t pixels, uint32_t total_spp, const double* cell_sum,
                            const double* cell_sumsq, float* film, double* xyz, double* xyz_var, float* rgb,
                            cudaStream_t stream) {
    if (!film && !xyz && !xyz_var && !rgb) return cudaSuccess;
    if (pixels == 0) return cudaSuccess;
    const double n = double(total_spp);
    const double inv_n = 1.0 / n, inv_var = total_spp > 1u ? inv_n / (n - 1.0) : 0.0;
    finalize_kernel<<<finalize_blocks(pixels), kFinalizeThreads, 0, stream>>>(
        S.bands, S.band_count, pixels, inv_n, inv_var, cell_sum, cell_sumsq, film, xyz, xyz_var, rgb,
        rgb_matrix(S));
    return cudaGetLastError();
}

cudaError_t launch_finalize_jobs(const DevScene& S, const DevJob* jobs, uint32_t num_jobs, uint32_t total_cells,
                                 cudaStream_t stream) {
    const uint64_t pixels = uint64_t(total_cells) / S.band_count;
    if (pixels == 0) return cudaSuccess;
    finalize_jobs_kernel<<<finalize_blocks(pixels), kFinalizeThreads, 0, stream>>>(S.bands, S.band_count, jobs,
                                                                                   num_jobs, pixels, rgb_matrix(S));
    return cudaGetLastError();
}

}  // namespace sky
