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
};

// One render of a ray-loop launch: its launch constants and sun frame (the
// renders of a batch share the parameterised medium and differ in sun and
// view), its outputs and its range of the launch's cells.  Cells are the
// render's (pixel, band) pairs, band-major in the claim order.
struct AdjJob {
    DevLaunch L;
    float sun[3], sun_t[3], sun_b[3];
    const float* dloss;   // gradient pass: dLoss/dfilm [pixels][bands]
    double* cell_sum;     // primal: FP64 sums [pixels][bands]
    double* cell_sumsq;
    // Optional [cells][spp] radiance of every chain (SkyAdjointParams::chain_radiance):
    // written by the primal, read by the gradient pass in place of its first trace
    // of each chain.
    float* chain_rad;
    uint32_t cell_begin;  // first global cell of the render in the launch
    uint32_t cell_count;
};

// The renders of one launch, passed by value as a kernel parameter (no job
// table in device memory; a larger batch takes several launches).
constexpr uint32_t kAdjMaxJobs = 32;
struct AdjJobs {
    AdjJob j[kAdjMaxJobs];
    uint32_t count;
    uint32_t cells;  // sum of the renders' cells
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
// A batch (J) takes the ray loop and needs P = Q; the warp-per-cell form
// renders J.j[0] alone.
cudaError_t launch_adjoint_primal(const AdjCtx& A, const AdjJobs& J, bool accumulate, unsigned long long* counters,
                                  uint32_t* status, uint32_t* next_cell, cudaStream_t stream);

// Path-replay gradient (P == Q): adds dLoss/dparams to layer_grad [3 L + 2]
// and band_grad [B][4] (may be null) given each render's dLoss/dfilm
// [pixels][B] (J.j[i].dloss).
cudaError_t launch_adjoint_grad(const AdjCtx& A, const AdjJobs& J, double* layer_grad, double* band_grad,
                                unsigned long long* counters, uint32_t* status, uint32_t* next_cell,
                                cudaStream_t stream);

}  // namespace sky
