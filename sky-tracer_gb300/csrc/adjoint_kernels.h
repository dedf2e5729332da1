// adjoint_kernels.h — launchers of the differentiable renderer (adjoint.cu).
//
// The medium of a differentiable render is the scene's medium with
// parameters applied: per majorant layer l, density scales of Rayleigh,
// aerosol species 0 ("Mie") and ozone; a Mie single-scattering albedo; a Mie
// Henyey-Greenstein asymmetry g; and per band, multipliers of the Rayleigh,
// Mie and ozone cross sections and of the solar radiance.  Two parameter
// sets take part in a render: P, whose medium is evaluated, and Q, whose
// medium drives every sampling decision (tracking majorants, collision
// choices, phase sampling, Russian roulette).  With P == Q this is the
// ordinary tracer over the parameterised medium; with P != Q each path is
// reweighted by f_P / f_Q, which keeps the samples fixed while P moves (the
// common-random-numbers form that finite differences of the estimator need).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "sky_scene.h"

namespace sky {

constexpr uint32_t kAdjBandParams = 4;  // Rayleigh, Mie, ozone, solar multipliers

// One parameter set with its Henyey-Greenstein tables.
struct AdjParamSet {
    const float* layer;    // [3 L + 2]: (s_R, s_M, s_O) per layer, then omega, g
    const float* band;     // [B][4] multipliers, or null for all ones
    const float* phase;    // [bins] HG values of g at the cube-root bin centres
    const float* dphase;   // [bins] their derivative in g
    const float* cdf;      // [bins] sampling CDF of the HG table
    const float* bin_pdf;  // [bins] per-bin sampling pdf
};

// Tracking grid of the sampling medium Q, rebuilt on the device per call.
struct AdjGrid {
    const float* layer_maj;  // [B][L] majorant of each uniform layer
    const float* radius;     // [B][L + 1] lower shell radius of each tracking layer (+ top)
    const float* maj;        // [B][L + 1] majorant of each tracking layer
    const uint16_t* map;     // [B][L] uniform layer -> tracking layer
    const uint32_t* count;   // [B] tracking layers of the band
};

struct AdjCtx {
    DevScene S;
    AdjParamSet P, Q;
    AdjGrid G;
    uint32_t distinct;     // P and Q differ
    uint32_t merge;        // merge uniform layers into tracking layers (else one per layer)
    float crossing_cost;   // merge cost of a shell crossing, in optical-depth units
    uint32_t estimator;    // SkyAdjointEstimator of the backward pass
    // Optional [cells][spp] radiance of every chain (SkyAdjointParams::chain_radiance):
    // written by the primal ray loop, read by the gradient pass in place of its first
    // trace of each chain.
    float* chain_rad;
    uint64_t chain_rad_len;  // floats in chain_rad (checked against the render's chains)
};

// Writable views of the tables the prepare kernel fills.
struct AdjWorkspace {
    float* p_tables;  // [4][bins]: phase, dphase, cdf, bin_pdf of P
    float* q_tables;  // the same for Q (== p_tables when P == Q)
    float* layer_maj;
    float* radius;
    float* maj;
    uint16_t* map;
    uint32_t* count;
    uint32_t* next_cell;  // work counter of the adjoint kernel
};

// Scene workspace layout for a scene of B bands, L layers and `bins` phase bins.
size_t adjoint_workspace_bytes(uint32_t B, uint32_t L, uint32_t bins);
AdjWorkspace adjoint_workspace(void* base, uint32_t B, uint32_t L, uint32_t bins);

// Bake the majorants of Q and its tracking grid, and the HG tables of P and Q.
cudaError_t launch_adjoint_prepare(const AdjCtx& A, const AdjWorkspace& W, cudaStream_t stream);

// Primal render over the parameterised medium: per-cell sums (and squares)
// of the radiance of P, sampled with Q.  With P = Q it runs the ray loop of
// the adjoint kernel (next_cell is its work counter); otherwise a warp per
// cell.
cudaError_t launch_adjoint_primal(const AdjCtx& A, const DevLaunch& L, double* cell_sum, double* cell_sumsq,
                                  bool accumulate, unsigned long long* counters, uint32_t* status,
                                  uint32_t* next_cell, cudaStream_t stream);

// Path-replay gradient (P == Q): adds dLoss/dparams to layer_grad [3 L + 2]
// and band_grad [B][4] (may be null) given dLoss/dfilm [pixels][B].
cudaError_t launch_adjoint_grad(const AdjCtx& A, const DevLaunch& L, const float* dloss_dfilm, double* layer_grad,
                                double* band_grad, unsigned long long* counters, uint32_t* status,
                                uint32_t* next_cell, cudaStream_t stream);

}  // namespace sky
