// mie_kernels.h — launcher of the Mie phase-table bake (mie.cu).
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

namespace sky {

// One sphere of a bake (one radius of one band): its size parameter,
// refractive index and weight, and its slices of the scratch arrays.
struct MieItem {
    double x;       // size parameter 2 pi r / lambda
    double m_re;    // refractive index n + i k (k >= 0 absorbs)
    double m_im;
    double k;       // wavenumber 2 pi / lambda, 1/um
    double weight;  // lognormal weight of the radius; a band's weights sum to 1
    uint64_t aoff;  // first coefficient (float4) of the item
    uint64_t doff;  // first D_n (double2) of the item
    uint32_t band;
    uint32_t terms;   // N: series terms
    uint32_t dterms;  // start index of the downward D_n recurrence
    uint32_t _pad;
};

// Series terms for size parameter x: x + 4.05 x^(1/3) + 2 (Wiscombe 1980), plus one.
inline uint32_t mie_terms(double x) { return uint32_t(x + 4.05 * std::cbrt(x) + 2.0) + 1u; }

// Coefficients (one thread per item) then angles (one block per item): adds
// w (|S1|^2 + |S2|^2) / (2 k^2) of every item to phase_acc[band][bins] (FP64,
// zeroed by the caller) and writes Q_sca, Q_ext and g per item to q[3 * item].
cudaError_t launch_mie_bake(const MieItem* items, uint32_t count, uint32_t max_terms, double2* dscratch,
                            float4* ab, double* q, uint32_t bins, double* phase_acc, cudaStream_t stream);

}  // namespace sky
