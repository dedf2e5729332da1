// mie.cu — the Mie phase-table bake of scripts/bake_opac_data.py:103-121 and
// :192-204: for one aerosol species, the phase function on the cube-root mu
// grid averaged over a lognormal size distribution with scattering cross
// section weights,
//
//   p(mu) = sum_r w_r sigma_sca(r) p_r(mu) / sum_r w_r sigma_sca(r),
//
// where p_r is a sphere's unpolarised phase function normalised to 1 over the
// sphere.  The reference evaluates each sphere with miepython (efficiencies
// and i_unpolarized, norm="one"); miepython is not vendored and its version
// is not pinned, so the sphere is computed here from the published Mie series
// (Bohren & Huffman, "Absorption and Scattering of Light by Small Particles",
// 1983, appendix A, BHMIE; term count after Wiscombe, Appl. Opt. 19, 1505,
// 1980).  Since sigma_sca p_r = (|S1|^2 + |S2|^2) / (2 k^2), the average
// needs only the amplitude functions and Q_sca.
//
// Two kernels.  Coefficients: one thread per (band, radius) runs the series
// recurrences in FP64 (the logarithmic derivative D_n(mx) downward from
// max(N, |mx|) + 16, the Riccati-Bessel functions upward) and stores
// a_n, b_n pre-multiplied by (2n+1)/(n(n+1)) in FP32, with Q_sca, Q_ext and
// the asymmetry parameter.  Angles: one block per (band, radius) stages the
// coefficients in shared memory and each thread sums S1, S2 for its mu bins
// in FP32 (pi_n, tau_n recurrences), adding w (|S1|^2 + |S2|^2) / (2 k^2) to
// the band's FP64 accumulator.

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "mie_kernels.h"

namespace sky {
namespace {

struct Cd {
    double re, im;
};
__device__ __forceinline__ Cd cd(double re, double im) { return Cd{re, im}; }
__device__ __forceinline__ Cd operator+(Cd a, Cd b) { return cd(a.re + b.re, a.im + b.im); }
__device__ __forceinline__ Cd operator-(Cd a, Cd b) { return cd(a.re - b.re, a.im - b.im); }
__device__ __forceinline__ Cd operator*(Cd a, Cd b) { return cd(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
__device__ __forceinline__ Cd operator*(double s, Cd a) { return cd(s * a.re, s * a.im); }
// Smith's division, robust to the large magnitudes of xi_n beyond n ~ x.
__device__ __forceinline__ Cd operator/(Cd a, Cd b) {
    if (fabs(b.re) >= fabs(b.im)) {
        const double r = b.im / b.re, d = b.re + r * b.im;
        return cd((a.re + r * a.im) / d, (a.im - r * a.re) / d);
    }
    const double r = b.re / b.im, d = b.im + r * b.re;
    return cd((a.re * r + a.im) / d, (a.im * r - a.re) / d);
}
__device__ __forceinline__ double norm2(Cd a) { return a.re * a.re + a.im * a.im; }

__global__ void __launch_bounds__(64) mie_coefficients_kernel(const MieItem* __restrict__ items, uint32_t count,
                                                              double2* __restrict__ dscratch,
                                                              float4* __restrict__ ab, double* __restrict__ q) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const MieItem it = items[i];
    const double x = it.x;
    const Cd m = cd(it.m_re, it.m_im);
    const Cd mx = x * m;
    const uint32_t N = it.terms, nmx = it.dterms;
    double2* D = dscratch + it.doff;
    // D_{n-1} = n/(mx) - 1/(D_n + n/(mx)), D_nmx = 0
    const Cd inv_mx = cd(1.0, 0.0) / mx;
    Cd d = cd(0.0, 0.0);
    D[nmx] = make_double2(0.0, 0.0);
    for (uint32_t n = nmx; n >= 1u; --n) {
        const Cd t = double(n) * inv_mx;
        d = t - cd(1.0, 0.0) / (d + t);
        D[n - 1u] = make_double2(d.re, d.im);
    }
    const Cd inv_m = cd(1.0, 0.0) / m;
    double psi0 = cos(x), psi1 = sin(x), chi0 = -sin(x), chi1 = cos(x);
    Cd xi1 = cd(psi1, -chi1);
    double qsca = 0.0, qext = 0.0, gsum = 0.0;
    Cd a_prev = cd(0.0, 0.0), b_prev = cd(0.0, 0.0);
    float4* out = ab + it.aoff;
    for (uint32_t n = 1u; n <= N; ++n) {
        const double rn = double(n);
        const double psi = (2.0 * rn - 1.0) * psi1 / x - psi0;
        const double chi = (2.0 * rn - 1.0) * chi1 / x - chi0;
        const Cd xi = cd(psi, -chi);
        const double2 dn2 = D[n];
        const Cd dn = cd(dn2.x, dn2.y);
        const Cd ta = dn * inv_m + cd(rn / x, 0.0);
        const Cd tb = m * dn + cd(rn / x, 0.0);
        const Cd an = (psi * ta - cd(psi1, 0.0)) / (ta * xi - xi1);
        const Cd bn = (psi * tb - cd(psi1, 0.0)) / (tb * xi - xi1);
        qsca += (2.0 * rn + 1.0) * (norm2(an) + norm2(bn));
        qext += (2.0 * rn + 1.0) * (an.re + bn.re);
        // asymmetry: (n-1)(n+1)/n Re(a_{n-1} a_n* + b_{n-1} b_n*) + (2n+1)/(n(n+1)) Re(a_n b_n*)
        if (n > 1u) {
            const double rm = rn - 1.0;
            gsum += rm * (rm + 2.0) / (rm + 1.0) *
                    (a_prev.re * an.re + a_prev.im * an.im + b_prev.re * bn.re + b_prev.im * bn.im);
        }
        gsum += (2.0 * rn + 1.0) / (rn * (rn + 1.0)) * (an.re * bn.re + an.im * bn.im);
        const double fn = (2.0 * rn + 1.0) / (rn * (rn + 1.0));
        out[n - 1u] = make_float4(float(fn * an.re), float(fn * an.im), float(fn * bn.re), float(fn * bn.im));
        a_prev = an;
        b_prev = bn;
        psi0 = psi1;
        psi1 = psi;
        chi0 = chi1;
        chi1 = chi;
        xi1 = cd(psi1, -chi1);
    }
    const double x2 = x * x;
    qsca *= 2.0 / x2;
    q[3 * i] = qsca;
    q[3 * i + 1] = qext * 2.0 / x2;
    q[3 * i + 2] = qsca > 0.0 ? gsum * 4.0 / (x2 * qsca) : 0.0;
}

__global__ void __launch_bounds__(256) mie_angles_kernel(const MieItem* __restrict__ items,
                                                         const float4* __restrict__ ab, uint32_t bins,
                                                         double* __restrict__ phase_acc) {
    extern __shared__ float4 coef[];
    const MieItem it = items[blockIdx.x];
    const uint32_t N = it.terms;
    for (uint32_t n = threadIdx.x; n < N; n += blockDim.x) coef[n] = ab[it.aoff + n];
    __syncthreads();
    const double scale = it.weight / (2.0 * it.k * it.k);  // w / (2 k^2)
    double* acc = phase_acc + size_t(it.band) * bins;
    for (uint32_t j = threadIdx.x; j < bins; j += blockDim.x) {
        const double u = (double(j) + 0.5) / double(bins);
        const float mu = float(1.0 - 2.0 * u * u * u);  // cube-root grid (bake_opac_data.py:99-101)
        float pi0 = 0.0f, pi1 = 1.0f;
        float s1r = 0.0f, s1i = 0.0f, s2r = 0.0f, s2i = 0.0f;
        for (uint32_t n = 1u; n <= N; ++n) {
            const float rn = float(n);
            const float pi = pi1;
            const float tau = rn * mu * pi - (rn + 1.0f) * pi0;
            const float4 c = coef[n - 1u];
            s1r = fmaf(c.x, pi, fmaf(c.z, tau, s1r));
            s1i = fmaf(c.y, pi, fmaf(c.w, tau, s1i));
            s2r = fmaf(c.x, tau, fmaf(c.z, pi, s2r));
            s2i = fmaf(c.y, tau, fmaf(c.w, pi, s2i));
            pi1 = ((2.0f * rn + 1.0f) * mu * pi - (rn + 1.0f) * pi0) / rn;
            pi0 = pi;
        }
        const double i2 = double(s1r) * s1r + double(s1i) * s1i + double(s2r) * s2r + double(s2i) * s2i;
        atomicAdd(acc + j, scale * i2);
    }
}

}  // namespace

cudaError_t launch_mie_bake(const MieItem* items, uint32_t count, uint32_t max_terms, double2* dscratch, float4* ab,
                            double* q, uint32_t bins, double* phase_acc, cudaStream_t stream) {
    if (count == 0) return cudaSuccess;
    mie_coefficients_kernel<<<(count + 63u) / 64u, 64, 0, stream>>>(items, count, dscratch, ab, q);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const size_t smem = size_t(max_terms) * sizeof(float4);
    if (smem > 48u * 1024u) {
        e = cudaFuncSetAttribute(mie_angles_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if (e != cudaSuccess) return e;
    }
    mie_angles_kernel<<<count, 256, smem, stream>>>(items, ab, bins, phase_acc);
    return cudaGetLastError();
}

}  // namespace sky
