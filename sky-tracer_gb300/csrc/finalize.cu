// finalize.cu — per-pixel epilogue: mean film (the reference's
// `values *= 1/spp; max(0)`, integrator.rs:306-310), CIE XYZ of the mean
// spectrum (spectrum_to_xyz_with_weights, spectrum.rs:232-241, FP64) and the
// variance of that XYZ estimate from the per-band sums of squares.
//
// One warp per pixel: lanes stride over the bands (coalesced film stores),
// then a shuffle reduction forms XYZ and its variance, and the white-balanced
// linear sRGB of that XYZ (film_output.rs:96-124 on the host in the reference).

#include "trace_kernels.h"

namespace sky {
namespace {

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// One pixel by one warp: lanes stride over the bands.
__device__ __forceinline__ void finalize_pixel(const DevBand* __restrict__ bands, uint32_t band_count,
                                               uint64_t pixel, uint32_t total_spp, const double* __restrict__ cell_sum,
                                               const double* __restrict__ cell_sumsq, float* __restrict__ film,
                                               double* __restrict__ xyz, double* __restrict__ xyz_var,
                                               float* __restrict__ rgb, const RgbMatrix& m, uint32_t lane) {
    const double n = double(total_spp);
    const double inv_n = 1.0 / n;
    double acc[3] = {0.0, 0.0, 0.0}, var[3] = {0.0, 0.0, 0.0};
    for (uint32_t b = lane; b < band_count; b += 32u) {
        const uint64_t cell = pixel * band_count + b;
        const double s = cell_sum[cell];
        const double mean = s * inv_n;
        if (film) film[cell] = fmaxf(float(mean), 0.0f);
        double var_mean = 0.0;
        if (xyz_var && cell_sumsq && total_spp > 1u) {
            double sample_var = (cell_sumsq[cell] - s * mean) / (n - 1.0);
            var_mean = fmax(sample_var, 0.0) * inv_n;
        }
        const DevBand& bd = bands[b];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            double w = double(bd.xyz[c]);
            acc[c] += mean * w;
            var[c] += var_mean * w * w;
        }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        acc[c] = warp_sum_d(acc[c]);
        var[c] = warp_sum_d(var[c]);
    }
    if (lane == 0) {
        if (xyz)
            for (int c = 0; c < 3; ++c) xyz[pixel * 3 + c] = acc[c];
        if (xyz_var)
            for (int c = 0; c < 3; ++c) xyz_var[pixel * 3 + c] = var[c];
        if (rgb) store_rgb(m, acc, rgb + pixel * 3);
    }
}

__global__ void __launch_bounds__(256) finalize_kernel(const DevBand* __restrict__ bands, uint32_t band_count,
                                                       uint64_t pixels, uint32_t total_spp,
                                                       const double* __restrict__ cell_sum,
                                                       const double* __restrict__ cell_sumsq,
                                                       float* __restrict__ film, double* __restrict__ xyz,
                                                       double* __restrict__ xyz_var, float* __restrict__ rgb,
                                                       RgbMatrix m) {
    const uint64_t pixel = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    if (pixel >= pixels) return;
    finalize_pixel(bands, band_count, pixel, total_spp, cell_sum, cell_sumsq, film, xyz, xyz_var, rgb, m,
                   threadIdx.x & 31u);
}

// Pixels of all jobs in a row; the job of a pixel by binary search over the
// jobs' first cells (every job's cell range is a whole number of pixels).
__global__ void __launch_bounds__(256) finalize_jobs_kernel(const DevBand* __restrict__ bands, uint32_t band_count,
                                                            const DevJob* __restrict__ jobs, uint32_t num_jobs,
                                                            uint64_t total_pixels, RgbMatrix m) {
    const uint64_t gp = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    if (gp >= total_pixels) return;
    const uint64_t gc = gp * band_count;
    uint32_t lo = 0u, hi = num_jobs;
    while (hi - lo > 1u) {
        const uint32_t mid = (lo + hi) >> 1;
        if (jobs[mid].cell_begin <= gc) lo = mid;
        else hi = mid;
    }
    const DevJob& J = jobs[lo];
    if (!J.film && !J.xyz && !J.xyz_var && !J.rgb) return;
    const uint64_t pixel = (gc - J.cell_begin) / band_count;
    finalize_pixel(bands, band_count, pixel, J.total_spp, J.cell_sum, J.cell_sumsq, J.film, J.xyz, J.xyz_var, J.rgb,
                   m, threadIdx.x & 31u);
}

}  // namespace

cudaError_t launch_finalize(const DevScene& S, uint64_t pixels, uint32_t total_spp, const double* cell_sum,
                            const double* cell_sumsq, float* film, double* xyz, double* xyz_var, float* rgb,
                            cudaStream_t stream) {
    if (!film && !xyz && !xyz_var && !rgb) return cudaSuccess;
    const uint32_t block = 256;
    const uint64_t blocks = (pixels * 32u + block - 1) / block;
    finalize_kernel<<<dim3(uint32_t(blocks)), block, 0, stream>>>(S.bands, S.band_count, pixels, total_spp, cell_sum,
                                                                 cell_sumsq, film, xyz, xyz_var, rgb,
                                                                 rgb_matrix(S));
    return cudaGetLastError();
}

cudaError_t launch_finalize_jobs(const DevScene& S, const DevJob* jobs, uint32_t num_jobs, uint32_t total_cells,
                                 cudaStream_t stream) {
    const uint64_t pixels = uint64_t(total_cells) / S.band_count;
    if (pixels == 0) return cudaSuccess;
    const uint32_t block = 256;
    const uint64_t blocks = (pixels * 32u + block - 1) / block;
    finalize_jobs_kernel<<<dim3(uint32_t(blocks)), block, 0, stream>>>(S.bands, S.band_count, jobs, num_jobs, pixels,
                                                                       rgb_matrix(S));
    return cudaGetLastError();
}

}  // namespace sky
