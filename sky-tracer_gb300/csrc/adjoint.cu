// adjoint.cu — differentiable rendering of the sky: the device bake of the
// majorants of a parameterised medium, its primal render, and the
// path-replay adjoint that returns dLoss/dparams.  No counterpart in the
// reference; the transport is the reference's (sky_trace.wgsl:703-776) over
// the parameterised medium described in adjoint_kernels.h.
//
// Parameters of a set X (layer l, band b, altitude h inside layer l):
//   sigma_R  = s_R[l] k_R[b] air(h) xs_R[b]            (sky_trace.wgsl:383)
//   sigma_M  = s_M[l] k_M[b] m0(h) (sca0[b] + abs0[b])  (:370-380, species 0)
//   sigma_O  = s_O[l] k_O[b] o3(h) xs_O[b]             (:384)
//   sigma_Ms = omega sigma_M, sigma_t = sigma_R + sigma_M + sigma_O,
//   sigma_s  = sigma_R + sigma_Ms, Mie phase = HG(g) tabulated on the scene's
//   cube-root mu grid (phase.rs:37-46), solar radiance x k_S[b].
//
// Gradient estimator (path replay: a chain is traced once for its radiance
// L, then replayed from the same counter-based random numbers; no path is
// stored).  Each contribution C to L (an NEE term, the sun disc) is a
// product of factors, and dC = C sum d log(factor):
//   traversed segment       transmittance exp(-integral sigma_t): its
//                           d log is -integral d(sigma_t) along the segment
//   scattering vertex       sum_i sigma_i p_i(mu) for the direction mu that
//                           the contribution uses (the sun direction of an
//                           NEE term, the continuation direction for
//                           everything after it); the albedo and the mixed
//                           phase's normalisation cancel into it
//   sun radiance            k_S (L is linear in it)
// Russian roulette, camera, light and Lambert sampling carry no parameter.
// The replay adds w * C_after * d log(factor) for each factor, where C_after
// is the radiance the factor multiplies (L minus what was collected before
// it, or the single NEE term for a shadow ray's factors) and w is dLoss/dL
// of the chain (dLoss/dfilm of its cell / spp).
// The segment integrals are estimated either by stratified points placed in
// majorant optical depth from a random stream of their own
// (SKY_ADJOINT_SEGMENT_INTEGRALS), or by the null collisions the tracker drew
// (SKY_ADJOINT_NULL_COLLISIONS: factor mu_bar - sigma_t per null collision;
// with the samples held fixed this is the exact derivative of the forward
// estimator, and the shadow ray of an NEE term is traced a second time for
// its null collisions).

#include <algorithm>
#include <cmath>

#include "adjoint_kernels.h"
#include "sky_device.cuh"

namespace sky {
namespace {

// Unscaled coefficients at a point: air xs_R, m0 ext0 and o3 xs_O of the
// band, and the uniform layer that holds the point.
struct AdjBase {
    float uR, uM, uO;
    int layer;
};

// Coefficients of one parameter set at a point.
struct AdjMed {
    float R, M, O, Ms, t, s;
};

// A parameter set resolved for one band.
struct AdjSet {
    const float* layer;
    float kR, kM, kO, kS;
    float omega;
    const float* phase;
    const float* dphase;
    const float* cdf;
    const float* bin_pdf;
};

__device__ __forceinline__ AdjSet resolve(const AdjParamSet& X, uint32_t layers, uint32_t band) {
    AdjSet r;
    r.layer = X.layer;
    if (X.band) {
        const float* k = X.band + band * kAdjBandParams;
        r.kR = __ldg(k);
        r.kM = __ldg(k + 1);
        r.kO = __ldg(k + 2);
        r.kS = __ldg(k + 3);
    } else {
        r.kR = r.kM = r.kO = r.kS = 1.0f;
    }
    r.omega = __ldg(X.layer + 3 * layers);
    r.phase = X.phase;
    r.dphase = X.dphase;
    r.cdf = X.cdf;
    r.bin_pdf = X.bin_pdf;
    return r;
}

__device__ __forceinline__ AdjBase adj_base(const DevScene& S, uint32_t band, float alt) {
    AdjBase b;
    b.uR = b.uM = b.uO = 0.0f;
    b.layer = 0;
    if (!(alt >= 0.0f && alt <= S.top_altitude)) return b;
    const uint32_t k = knot_interval(S, S.knot_z, S.finder, alt);
    const float dz = alt - S.knot_z[k];
    const DevProfileKnot& P = S.profile[k];
    const DevBand& B = S.bands[band];
    b.uR = fmaxf(fmaf(dz, P.air_slope, P.air) * B.rayleigh_xs, 0.0f);
    b.uO = fmaxf(fmaf(dz, P.ozone_slope, P.ozone) * B.ozone_xs, 0.0f);
    const float mass = fmaxf(fmaf(dz, P.mass_slope[0], P.mass[0]), 0.0f);
    const SkyAerosolOptics o = S.optics[band * kSpecies];
    b.uM = fmaxf(mass * o.scattering_km_inv_per_g_m3, 0.0f) + fmaxf(mass * o.absorption_km_inv_per_g_m3, 0.0f);
    b.layer = min(int(alt * S.inv_layer_dz), int(S.layer_count) - 1);
    return b;
}

__device__ __forceinline__ AdjMed adj_med(const AdjSet& X, const AdjBase& b) {
    const float* p = X.layer + 3 * b.layer;
    AdjMed m;
    m.R = __ldg(p) * X.kR * b.uR;
    m.M = __ldg(p + 1) * X.kM * b.uM;
    m.O = __ldg(p + 2) * X.kO * b.uO;
    m.Ms = X.omega * m.M;
    m.s = m.R + m.Ms;
    m.t = m.R + m.M + m.O;
    return m;
}

// Position of mu on the cube-root grid (mie_phase, sky_trace.wgsl:485-494).
__device__ __forceinline__ void hg_slot(uint32_t bins, float mu, uint32_t& i0, uint32_t& i1, float& t) {
    const float u = cbrt_pos((1.0f - fminf(fmaxf(mu, -1.0f), 1.0f)) * 0.5f);
    const float f = u * float(bins) - 0.5f;
    i0 = min(uint32_t(fminf(fmaxf(floorf(f), 0.0f), float(bins - 1u))), bins - 1u);
    i1 = min(i0 + 1u, bins - 1u);
    t = fminf(fmaxf(f - float(i0), 0.0f), 1.0f);
}

__device__ __forceinline__ float hg_value(const AdjSet& X, uint32_t bins, float mu) {
    uint32_t i0, i1;
    float t;
    hg_slot(bins, mu, i0, i1, t);
    const float p0 = __ldg(X.phase + i0), p1 = __ldg(X.phase + i1);
    return fmaxf(fmaf(t, p1 - p0, p0), 0.0f);
}

// sum_i sigma_i p_i(mu): the scattering-vertex factor.
__device__ __forceinline__ float vertex_phase(const AdjSet& X, uint32_t bins, const AdjMed& m, float mu) {
    return m.R * rayleigh_phase(mu) + (m.Ms > 0.0f ? m.Ms * hg_value(X, bins, mu) : 0.0f);
}

// Gradient accumulator of one lane: per-layer scales in the warp's copy of
// the layer gradient in shared memory; the Mie albedo and g, and the
// multipliers of the lane's band, in registers.
struct AdjAcc {
    float* sg;  // [3 L + 2]
    uint32_t L;
    float gR, gM, gO;  // band multipliers
    float gW, gG;      // Mie albedo, Mie g
};

// d sigma_t terms of a null collision, times c (= -weight / sigma_n).
__device__ __forceinline__ void null_terms(AdjAcc& a, const AdjSet& X, const AdjBase& b, float c) {
    const float* p = X.layer + 3 * b.layer;
    float* g = a.sg ? a.sg + 3 * b.layer : nullptr;  // null: band gradients only
    if (b.uR > 0.0f) {
        if (g) atomicAdd(g, c * X.kR * b.uR);
        a.gR = fmaf(c * __ldg(p), b.uR, a.gR);
    }
    if (b.uM > 0.0f) {
        if (g) atomicAdd(g + 1, c * X.kM * b.uM);
        a.gM = fmaf(c * __ldg(p + 1), b.uM, a.gM);
    }
    if (b.uO > 0.0f) {
        if (g) atomicAdd(g + 2, c * X.kO * b.uO);
        a.gO = fmaf(c * __ldg(p + 2), b.uO, a.gO);
    }
}

// weight * d log(sum_i sigma_i p_i(mu)) of a scattering vertex.
__device__ __forceinline__ void vertex_terms(AdjAcc& a, const AdjSet& X, uint32_t bins, const AdjBase& b,
                                             const AdjMed& m, float mu, float weight) {
    if (weight == 0.0f) return;
    uint32_t i0, i1;
    float t;
    hg_slot(bins, mu, i0, i1, t);
    const float p0 = __ldg(X.phase + i0), p1 = __ldg(X.phase + i1);
    const float pm = fmaxf(fmaf(t, p1 - p0, p0), 0.0f);
    const float d0 = __ldg(X.dphase + i0), d1 = __ldg(X.dphase + i1);
    const float dpm = fmaf(t, d1 - d0, d0);
    const float pr = rayleigh_phase(mu);
    const float sum = m.R * pr + m.Ms * pm;
    if (!(sum > 0.0f)) return;
    const float w = weight / sum;
    const float* p = X.layer + 3 * b.layer;
    float* g = a.sg ? a.sg + 3 * b.layer : nullptr;
    if (b.uR > 0.0f) {
        if (g) atomicAdd(g, w * X.kR * b.uR * pr);
        a.gR = fmaf(w * __ldg(p), b.uR * pr, a.gR);
    }
    if (b.uM > 0.0f) {
        if (g) atomicAdd(g + 1, w * X.omega * X.kM * b.uM * pm);
        a.gW = fmaf(w * m.M, pm, a.gW);
        a.gG = fmaf(w * m.Ms, dpm, a.gG);
        a.gM = fmaf(w * X.omega * __ldg(p + 1), b.uM * pm, a.gM);
    }
}

// Residual-carry delta tracking over Q's tracking grid (track_ray_merged of
// the plain tracer with the parameterised medium).  w_eval collects the
// null-collision ratios of P over Q (kMayDiffer: P and Q may be distinct
// sets; the ray loop has P = Q); with kNullTerms (the null-collision
// estimator) and gw != 0 every null collision adds gw * d log(mu_bar - sigma_t).
// At the 100000-segment guard a shadow ray (shadow = true) ends blocked and
// any other ray without a collision, as in track_ray.
template <bool kNullTerms, bool kMayDiffer = true>
__device__ __forceinline__ bool adj_track(const AdjCtx& A, const AdjSet& P, const AdjSet& Q, uint32_t band,
                                          const RayGeo& g, float t_max, Rng& rng, float& t_hit, AdjBase& hit,
                                          float& w_eval, float& tau_bar, float gw, AdjAcc& acc, Counters& n,
                                          bool& watchdog, bool shadow) {
    const DevScene& S = A.S;
    const uint32_t L = S.layer_count;
    MergedGrid G;
    G.radius = A.G.radius + band * (L + 1u);
    G.maj = A.G.maj + band * (L + 1u);
    G.map = A.G.map + band * L;
    G.count = int(__ldg(A.G.count + band));
    float t = 0.0f, t_piece = 0.0f;
    tau_bar = 0.0f;  // majorant optical depth of the traversed part
    int m = merged_layer_at(S, G, altitude_at(g, fminf(kRayEpsilonKm, t_max), S.ground_radius));
    int dir;
    float t_seg = merged_crossing(G, g, m, t, t_max, dir);
    float maj = __ldg(G.maj + m);
    ++n.e[SKY_EVENT_SEGMENT];
    float tau = -__logf(fmaxf(1.0f - rng.next(), 0.0000001f));
    uint32_t guard = 0;
    for (;;) {
        const float dt = tau / maj;
        if (t + dt < t_seg) {
            t = t + dt;
            ++n.e[SKY_EVENT_TRACK_STEP];
            const AdjBase b = adj_base(S, band, altitude_at(g, t, S.ground_radius));
            const AdjMed mq = adj_med(Q, b);
            if (rng.next() * maj < mq.t) {
                t_hit = t;
                hit = b;
                tau_bar += (t - t_piece) * maj;
                return true;
            }
            const float sn = maj - mq.t;
            if (kMayDiffer && A.distinct && sn > 0.0f) w_eval *= (maj - adj_med(P, b).t) / sn;
            if (kNullTerms && gw != 0.0f && sn > 0.0f)
                null_terms(acc, Q, b, -gw / sn);
            tau = -__logf(fmaxf(1.0f - rng.next(), 0.0000001f));
        } else {
            tau_bar += (t_seg - t_piece) * maj;
            if (dir == 0) return false;
            if (++guard > 100000u) {
                watchdog = true;
                return shadow;
            }
            tau = fmaxf(tau - (t_seg - t) * maj, 0.0f);
            t = t_seg;
            t_piece = t_seg;
            m += dir;
            t_seg = merged_crossing(G, g, m, t, t_max, dir);
            maj = __ldg(G.maj + m);
            ++n.e[SKY_EVENT_SEGMENT];
        }
    }
}

// Estimate of -integral d(sigma_t) over [0, t_end] of a ray, times weight:
// N points stratified in the majorant optical depth of Q's tracking grid
// (density mu_bar / tau_bar along the ray; tau_bar as the tracker summed
// it), each adding -weight (tau_bar / N) d(sigma_t) / mu_bar.  N grows with
// tau_bar.  The
// points' random numbers come from a stream of their own (another pcg4d
// key, 16 draws per position of the path's stream), so the path's own
// draws are untouched.
constexpr int kMaxSegmentPoints = 4;

__device__ __forceinline__ void segment_terms(const AdjCtx& A, const AdjSet& Q, uint32_t band, const RayGeo& g,
                                              float t_end, float tau, float weight, const Rng& rng, AdjAcc& acc) {
    if (weight == 0.0f || !(t_end > 0.0f) || !(tau > 0.0f)) return;
    const DevScene& S = A.S;
    const uint32_t L = S.layer_count;
    MergedGrid G;
    G.radius = A.G.radius + band * (L + 1u);
    G.maj = A.G.maj + band * (L + 1u);
    G.map = A.G.map + band * L;
    G.count = int(__ldg(A.G.count + band));
    const int m0 = merged_layer_at(S, G, altitude_at(g, fminf(kRayEpsilonKm, t_end), S.ground_radius));
    const int guard_max = 2 * G.count + 4;
    float t = 0.0f;
    int m = m0, dir = 0;
    const int n = min(kMaxSegmentPoints, 1 + int(tau));
    const float step = tau / float(n);
    Rng r2 = rng;  // 16 draws of its own per position of the path's stream
    r2.k2 ^= 0x68E31DA4u;
    r2.dim = rng.dim * 16u;
    int j = 0;
    float uj = r2.next() * step;
    float u0 = 0.0f;
    t = 0.0f;
    m = m0;
    for (int guard = 0; guard < guard_max && j < n; ++guard) {
        const float t_seg = merged_crossing(G, g, m, t, t_end, dir);
        const float maj = __ldg(G.maj + m);
        const float u1 = u0 + (t_seg - t) * maj;
        while (j < n && (uj < u1 || dir == 0)) {
            const float tj = fminf(t + (uj - u0) / maj, t_seg);
            const AdjBase b = adj_base(S, band, altitude_at(g, tj, S.ground_radius));
            null_terms(acc, Q, b, -weight * step / maj);
            ++j;
            uj = (float(j) + r2.next()) * step;
        }
        if (dir == 0) break;
        u0 = u1;
        t = t_seg;
        m += dir;
    }
}

// Inverse CDF of an HG table (MiePhaseTable::sample_mu_pdf, phase.rs:53-69).
__device__ __forceinline__ float hg_sample_mu(const AdjSet& X, uint32_t bins, float xi) {
    xi = fminf(fmaxf(xi, 0.0f), 1.0f - kF32Epsilon);
    uint32_t lo = 0, hi = bins;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(X.cdf + mid) <= xi) lo = mid + 1u;
        else hi = mid;
    }
    const uint32_t bin = min(lo, bins - 1u);
    const float prev = bin == 0u ? 0.0f : __ldg(X.cdf + bin - 1u);
    const float next = __ldg(X.cdf + bin);
    const float t = next > prev ? (xi - prev) / (next - prev) : 0.5f;
    return mu_edge(bin, bins) * (1.0f - t) + mu_edge(bin + 1u, bins) * t;
}

// MiePhaseTable::sampling_pdf (phase.rs:71-75)
__device__ __forceinline__ float hg_sampling_pdf(const AdjSet& X, uint32_t bins, float mu) {
    const float u = cbrt_pos((1.0f - fminf(fmaxf(mu, -1.0f), 1.0f)) * 0.5f);
    const uint32_t bin = min(uint32_t(floorf(u * float(bins))), bins - 1u);
    return fmaxf(__ldg(X.bin_pdf + bin), 1.0e-12f);
}

// Shadow ray of an NEE sample: the P/Q weight of a ray that reaches the sun,
// 0 when it hits the ground, leaves through no sun or collides.
__device__ __forceinline__ float adj_shadow(const AdjCtx& A, const AdjSet& P, const AdjSet& Q, uint32_t band, V3 pos,
                                            V3 ldir, Rng& rng, AdjAcc& acc, Counters& n, bool& watchdog) {
    const RayGeo sg = ray_geo(madd(pos, ldir, kRayEpsilonKm), ldir);
    float st;
    uint32_t sk;
    ++n.e[SKY_EVENT_BOUNDARY];
    if (!(next_boundary(A.S, sg, st, sk) && sk == 1u)) return 0.0f;
    float th, w = 1.0f, tau_bar;
    AdjBase bh;
    if (adj_track<false>(A, P, Q, band, sg, st, rng, th, bh, w, tau_bar, 0.0f, acc, n, watchdog, true)) return 0.0f;
    return w;
}

// One chain of the parameterised medium (trace_path, sky_trace.wgsl:703-776)
// at unit solar multiplier: sampled under Q, evaluated under P.
template <int kPhase>
__device__ __forceinline__ float adj_chain(const AdjCtx& A, const AdjSet& P, const AdjSet& Q, const DevLaunch& L,
                                           uint32_t x, uint32_t y, uint32_t band, uint32_t sample, Counters& n,
                                           bool& watchdog) {
    const DevScene& S = A.S;
    const uint32_t bins = S.phase_bins;
    AdjAcc acc{nullptr, 0u, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};  // no gradient terms in a primal render
    Rng rng;
    rng.init(y * L.width + x, sample, band, L.seed_lo, L.seed_hi);
    V3 dir = camera_dir(L, x, y, rng);
    V3 org = mk(0.0f, S.ground_radius + fmaxf(L.observer_altitude, 0.0f), 0.0f);
    ++n.e[SKY_EVENT_CHAIN];
    const float l_sun = __ldg(&S.bands[band].solar_radiance);
    const float inv_lights = 1.0f / float(L.direct_light_samples);
    // thr_q: throughput under Q (drives Russian roulette); thr: under P.
    float thr = 1.0f, thr_q = 1.0f, rad = 0.0f;
    for (uint32_t depth = 0;; ++depth) {
        if (depth >= L.watchdog_limit) {
            watchdog = true;
            return rad;
        }
        if (L.max_orders != 0u && depth >= L.max_orders) break;
        const RayGeo g = ray_geo(org, dir);
        float t_b;
        uint32_t kind;
        ++n.e[SKY_EVENT_BOUNDARY];
        if (!next_boundary(S, g, t_b, kind)) break;
        float t_hit, w_eval = 1.0f, tau_bar;
        AdjBase hb;
        const bool hit =
            adj_track<false>(A, P, Q, band, g, t_b, rng, t_hit, hb, w_eval, tau_bar, 0.0f, acc, n, watchdog, false);
        thr *= w_eval;
        if (hit) {
            ++n.e[SKY_EVENT_SCATTER];
            const V3 pos = madd(org, dir, t_hit);
            const AdjMed mq = adj_med(Q, hb);
            if (mq.t <= 0.0f || mq.s <= 0.0f) break;
            const AdjMed mp = A.distinct ? adj_med(P, hb) : mq;
            thr_q *= fminf(fmaxf(mq.s / mq.t, 0.0f), 1.0f);
            thr = A.distinct ? thr * (mp.s / mq.t) : thr_q;
            if (thr_q <= 0.0f) break;
            // direct_sun_at_scatter (sky_trace.wgsl:566-585)
            float nee = 0.0f;
            for (uint32_t ls = 0; ls < L.direct_light_samples; ++ls) {
                const V3 ldir = sample_sun_cone(S, rng);
                ++n.e[SKY_EVENT_NEE];
                const float trans = adj_shadow(A, P, Q, band, pos, ldir, rng, acc, n, watchdog);
                if (!(trans != 0.0f)) continue;
                const float mu = dot3(dir, ldir);
                const float ph = mp.s > 0.0f ? vertex_phase(P, bins, mp, mu) / mp.s : 0.0f;
                nee += l_sun * trans * ph / S.light_pdf;
            }
            rad += thr * (nee * inv_lights);
            V3 nd;
            float mu_c, fq, fp;
            if (kPhase == SKY_PHASE_TABULATED) {
                // phase.rs:53-75, sampling.rs:182-185 over Q's mixture
                const float target = rng.next() * mq.s;
                const bool rayleigh = target < mq.R || !(mq.Ms > 0.0f);
                const float xi_mu = rng.next();
                mu_c = rayleigh ? invert_rayleigh_cdf(xi_mu) : hg_sample_mu(Q, bins, xi_mu);
                const float xi_phi = rng.next();
                nd = direction_from_axis_mu(dir, mu_c, xi_phi);
                const float pdf = mq.R * rayleigh_phase(mu_c) +
                                  (mq.Ms > 0.0f ? mq.Ms * hg_sampling_pdf(Q, bins, mu_c) : 0.0f);
                fq = vertex_phase(Q, bins, mq, mu_c) / pdf;
                fp = A.distinct ? (mp.s > 0.0f ? vertex_phase(P, bins, mp, mu_c) / mp.s : 0.0f) * mq.s / pdf : fq;
            } else {
                nd = sample_isotropic(rng);
                mu_c = dot3(dir, nd);
                fq = vertex_phase(Q, bins, mq, mu_c) / mq.s / kIsotropicPdf;
                fp = A.distinct ? (mp.s > 0.0f ? vertex_phase(P, bins, mp, mu_c) / mp.s : 0.0f) / kIsotropicPdf : fq;
            }
            thr_q *= fq;
            thr = A.distinct ? thr * fp : thr_q;
            if (depth >= L.rr_start_depth) {  // russian_roulette (sky_trace.wgsl:691-701)
                const float q = fminf(fmaxf(thr_q, 0.05f), 0.95f);
                if (rng.next() > q) break;
                thr_q = thr_q / q;
                thr = A.distinct ? thr / q : thr_q;
            }
            org = madd(pos, nd, kRayEpsilonKm);
            dir = nd;
        } else if (kind == 1u) {
            if (depth == 0u && dot3(dir, load3(S.sun)) >= S.cos_max) rad += thr * l_sun;
            break;
        } else {
            // ground_radiance (sky_trace.wgsl:587-608) and the Lambert bounce (:750-766)
            ++n.e[SKY_EVENT_GROUND];
            const V3 pos = madd(org, dir, t_b);
            const V3 normal = normalize_or_y(pos);
            float ground = 0.0f;
            for (uint32_t ls = 0; ls < L.direct_light_samples; ++ls) {
                const V3 ldir = sample_sun_cone(S, rng);
                ++n.e[SKY_EVENT_NEE];
                const float cos_sun = fmaxf(dot3(normal, ldir), 0.0f);
                if (!(cos_sun > 0.0f)) continue;
                const float trans = adj_shadow(A, P, Q, band, pos, ldir, rng, acc, n, watchdog);
                if (!(trans != 0.0f)) continue;
                ground += S.ground_albedo * kInvPi * l_sun * trans * cos_sun / S.light_pdf;
            }
            rad += thr * (ground * inv_lights);
            float pdf;
            const V3 bounce = sample_cosine_hemisphere(normal, rng, pdf);
            const float cos_out = fmaxf(dot3(normal, bounce), 0.0f);
            if (pdf <= 0.0f || cos_out <= 0.0f) break;
            const float f = S.ground_albedo * kInvPi * cos_out / pdf;
            thr_q *= f;
            thr = A.distinct ? thr * f : thr_q;
            if (depth >= L.rr_start_depth) {
                const float q = fminf(fmaxf(thr_q, 0.05f), 0.95f);
                if (rng.next() > q) break;
                thr_q = thr_q / q;
                thr = A.distinct ? thr / q : thr_q;
            }
            org = madd(pos, bounce, kRayEpsilonKm);
            dir = bounce;
        }
        if (rad < 0.0f || rad != rad || thr_q < 0.0f || thr_q != thr_q || thr != thr) return 0.0f;
    }
    return fmaxf(rad, 0.0f);
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ uint32_t warp_sum_u(uint32_t v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ void flush_counters(const Counters& n, unsigned long long* counters, uint32_t lane) {
    if (!counters) return;
#pragma unroll
    for (int e = 0; e < SKY_EVENT_COUNT; ++e) {
        const uint32_t v = warp_sum_u(n.e[e]);
        if (lane == 0 && v) atomicAdd(counters + e, (unsigned long long)v);
    }
}

// Primal: one warp per (pixel, band) cell, 32 samples per round, FP64 cell
// sums in a fixed order (as the plain tracer).
template <int kPhase>
__global__ void __launch_bounds__(256) adjoint_primal_kernel(const __grid_constant__ AdjCtx A,
                                                             const __grid_constant__ DevLaunch L,
                                                             double* __restrict__ cell_sum,
                                                             double* __restrict__ cell_sumsq, uint32_t accumulate,
                                                             unsigned long long* __restrict__ counters,
                                                             uint32_t* __restrict__ status, uint64_t cells) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t q = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    if (q >= cells) return;  // whole warps only: blockDim is a multiple of 32
    // band-major warps, pixel-major cells (as the plain tracer)
    const uint64_t npix = cells / L.band_count;
    const uint32_t band = uint32_t(q / npix);
    const uint64_t pixel = q - uint64_t(band) * npix;  // pixel of the slab; y is the image row
    const uint64_t cell = pixel * L.band_count + band;
    const uint32_t x = uint32_t(pixel % L.width), y = uint32_t(pixel / L.width) + L.row_begin;
    const AdjSet P = resolve(A.P, A.S.layer_count, band);
    const AdjSet Q = A.distinct ? resolve(A.Q, A.S.layer_count, band) : P;
    Counters n;
    n.clear();
    bool watchdog = false;
    double sum = 0.0, sumsq = 0.0;
    if (accumulate) {
        sum = cell_sum[cell];
        if (cell_sumsq) sumsq = cell_sumsq[cell];
    }
    for (uint32_t base = 0; base < L.spp; base += 32u) {
        const uint32_t s = base + lane;
        float r = 0.0f;
        if (s < L.spp) r = P.kS * adj_chain<kPhase>(A, P, Q, L, x, y, band, L.sample_offset + s, n, watchdog);
        const double rd = double(r);
        sum += warp_sum_d(rd);
        sumsq += warp_sum_d(rd * rd);
    }
    if (lane == 0) {
        cell_sum[cell] = sum;
        if (cell_sumsq) cell_sumsq[cell] = sumsq;
    }
    flush_counters(n, counters, lane);
    if (__any_sync(0xffffffffu, watchdog) && lane == 0) atomicOr(status, 1u);
}

// ---------------------------------------------------------------------------
// Path replay as a ray loop.  A chain is a sequence of rays: the primary
// segment from each vertex, the shadow ray of each NEE sample and, with the
// null-collision estimator, the second trace of an unblocked shadow ray.
// Each iteration of the kernel's loop traces one ray per lane through the one
// inlined tracker and adds that ray's segment integral; the event code then
// runs up to the lane's next ray.  The lanes of a warp therefore enter the
// tracker together whatever vertex, pass or chain each is at, and a lane
// whose chain ends takes the next sample of its warp's cell (the warp takes a
// new cell from a counter when the samples run out) instead of waiting for
// the other lanes.
//
// Every chain runs twice on the same code: pass 0 for its radiance L (the
// C_after of the factors needs it), pass 1 for the gradient terms; both take
// the same path.  Random numbers are drawn in adj_chain's order, so the
// replay follows the primal render's paths.  P = Q (a gradient is taken at
// the sampling parameters).  Without kGrad the kernel is the primal render
// of P = Q: pass 0 only, each lane keeping the FP64 sums of its current cell
// and adding them to the cell when it moves on (cells add in no fixed order).
enum : uint32_t { kRayPrimary = 0u, kRayShadow = 1u, kRayRetrace = 2u };
enum : uint32_t { kNextTrace = 0u, kNextStart = 1u, kNextPrimary = 2u, kNextLights = 3u, kNextEnd = 4u,
                  kNextIdle = 5u };

// Render of global cell `g` in a launch: the last one whose first cell is <= g.
__device__ __forceinline__ uint32_t adj_job_of(const AdjJobs& J, uint32_t g) {
    uint32_t lo = 0u, hi = J.count;
    while (hi - lo > 1u) {
        const uint32_t mid = (lo + hi) >> 1;
        if (J.j[mid].cell_begin <= g) lo = mid;
        else hi = mid;
    }
    return lo;
}

// The slab cell (pixel-major, band-minor) of render-local claim index c
// (band-major), and its band and pixel.
__device__ __forceinline__ uint32_t adj_claimed_cell(const DevLaunch& L, uint32_t c, uint32_t& band, uint32_t& pixel) {
    const uint32_t npix = L.width * L.rows;
    band = c / npix;
    pixel = c - band * npix;
    return pixel * L.band_count + band;
}

// kCount: count events (counters given); without it the counters are never
// read and their increments compile away.  kSegEst: the segment-integral
// estimator (else null collisions); each instantiation holds only its own
// gradient code.  Resident blocks: 4 of 256 per SM (64 registers) for the
// primal and the gradient passes (the latter spill ~150 B but hide more latency
// than at 3 blocks and 80 registers).  J: the renders of the launch (one, or a
// batch sharing the parameterised medium); their cells are numbered in a row.
// kBatch: J holds more than one render (a single render reads J.j[0] at fixed
// offsets, with no per-lane render index: 7 % faster).
template <int kPhase, bool kGrad, bool kCount, bool kSegEst, bool kBatch>
__global__ void __launch_bounds__(256, 4) adjoint_grad_kernel(const __grid_constant__ AdjCtx A,
                                                              const __grid_constant__ AdjJobs J,
                                                              double* __restrict__ layer_grad,
                                                              double* __restrict__ band_grad,
                                                              unsigned long long* __restrict__ counters,
                                                              uint32_t* __restrict__ status,
                                                              uint32_t copies, uint32_t* __restrict__ next_cell) {
    extern __shared__ float smem[];
    const DevScene& S = A.S;
    const uint32_t Lc = S.layer_count, B = S.band_count, bins = S.phase_bins;
    const uint32_t nlayer = 3u * Lc + 2u;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    // layer gradients: one FP32 copy per warp when they fit (only a warp's own
    // lanes contend); band gradients: one copy per block
    float* sg = kGrad && layer_grad ? smem + (warp % copies) * nlayer : nullptr;
    float* sb = smem + copies * nlayer;
    if (kGrad) {
        for (uint32_t i = threadIdx.x; i < copies * nlayer + kAdjBandParams * B; i += blockDim.x) smem[i] = 0.0f;
        __syncthreads();
    }
    const uint32_t cells = J.cells;
    // primal: FP64 sums of the lane's current cell
    uint32_t acc_cell = 0xffffffffu, acc_job = 0u;
    double acc_sum = 0.0, acc_sq = 0.0;
    Counters n;
    n.clear();
    bool watchdog = false;
    AdjAcc acc{sg, Lc, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    // the warp's cell and its next unclaimed sample (warp-uniform)
    uint32_t claim_cell = 0u, claim_next = 0u, claim_spp = 0u, claim_job = 0u;
    uint32_t claim_band = 0u, claim_x = 0u, claim_y = 0u;  // divided out once per cell
    bool exhausted = false;
    // the lane's chain
    uint32_t next = kNextIdle, pass = 0u, job = 0u, cell = 0u, sample = 0u, band = 0u, px = 0u, py = 0u,
             ray = kRayPrimary,
             depth = 0u,
             ls = 0u, boundary = 0u, dim0 = 0u, dim1 = 0u;
    bool ground = false;
    Rng rng;
    rng.k0 = rng.k1 = rng.k2 = rng.dim = 0u;
    V3 org = mk(0.0f, 0.0f, 0.0f), dir = org;  // org is the vertex position between rays
    float thr = 0.0f, rad = 0.0f, nee = 0.0f, total = 0.0f, wc = 0.0f;
    float term = 0.0f, mu = 0.0f, c = 0.0f, t_max = 0.0f;  // pending shadow ray: its NEE term, cosine, weight
    AdjBase hb{0.0f, 0.0f, 0.0f, 0};
    RayGeo g{0.0f, 0.0f, 0.0f};

    for (;;) {
#pragma unroll 1
        for (int round = 0; round < 2; ++round) {
            // idle lanes take the next samples of the warp's cell
#pragma unroll 1
            for (;;) {
                const uint32_t need = __ballot_sync(0xffffffffu, next == kNextIdle);
                if (need == 0u || exhausted) break;
                if (claim_next >= claim_spp) {
                    // claims run band-major, as in the wavefront tracer (the warps of an SM
                    // share a band's tables in L1); cells keep the pixel-major layout
                    uint32_t cn = 0u;
                    if (lane == 0u) {
                        for (;;) {
                            cn = atomicAdd(next_cell, 1u);
                            if (!kGrad || cn >= cells) break;
                            const AdjJob& Jc = J.j[kBatch ? adj_job_of(J, cn) : 0u];
                            uint32_t b_, p_;
                            const uint32_t lc = adj_claimed_cell(Jc.L, cn - Jc.cell_begin, b_, p_);
                            if (__ldg(Jc.dloss + lc) != 0.0f) break;  // no loss: no gradient
                        }
                    }
                    cn = __shfl_sync(0xffffffffu, cn, 0);
                    if (cn >= cells) {
                        exhausted = true;
                        break;
                    }
                    claim_job = kBatch ? adj_job_of(J, cn) : 0u;
                    const DevLaunch& CL = J.j[claim_job].L;
                    uint32_t pixel;
                    claim_cell = adj_claimed_cell(CL, cn - J.j[claim_job].cell_begin, claim_band, pixel);
                    const uint32_t row = pixel / CL.width;  // row within the slab
                    claim_x = pixel - row * CL.width;
                    claim_y = row + CL.row_begin;
                    claim_spp = CL.spp;
                    claim_next = 0u;
                }
                const uint32_t rank = __popc(need & ((1u << lane) - 1u));
                if (next == kNextIdle && claim_next + rank < claim_spp) {
                    job = claim_job;
                    cell = claim_cell;
                    band = claim_band;
                    px = claim_x;
                    py = claim_y;
                    sample = claim_next + rank;
                    pass = 0u;
                    next = kNextStart;
                }
                claim_next = min(claim_spp, claim_next + uint32_t(__popc(need)));
            }
            // event code up to the lane's next ray
#pragma unroll 1
            while (next != kNextIdle && next != kNextTrace) {
                const AdjJob& JJ = J.j[kBatch ? job : 0u];
                const DevLaunch& L = JJ.L;
                if (next == kNextEnd) {
                    if (!kGrad) {
                        if (JJ.chain_rad) JJ.chain_rad[uint64_t(cell) * L.spp + sample] = rad;
                        const double rd = double(resolve(A.P, Lc, band).kS * rad);
                        acc_sum += rd;
                        acc_sq += rd * rd;
                        next = kNextIdle;
                    } else if (pass == 0u) {
                        total = rad;
                        if (total > 0.0f) {
                            pass = 1u;
                            next = kNextStart;
                        } else {
                            if (total != 0.0f) atomicAdd(sb + band * kAdjBandParams + 3u, wc * total);
                            next = kNextIdle;
                        }
                    } else {
                        float* bg = sb + band * kAdjBandParams;
                        atomicAdd(bg, acc.gR);
                        atomicAdd(bg + 1, acc.gM);
                        atomicAdd(bg + 2, acc.gO);
                        atomicAdd(bg + 3, wc * total);
                        if (sg) {
                            atomicAdd(sg + 3u * Lc, acc.gW);
                            atomicAdd(sg + 3u * Lc + 1u, acc.gG);
                        }
                        acc.gR = acc.gM = acc.gO = acc.gW = acc.gG = 0.0f;
                        next = kNextIdle;
                    }
                    continue;
                }
                if (next == kNextStart) {
                    if (!kGrad && (cell != acc_cell || (kBatch && job != acc_job))) {
                        if (acc_cell != 0xffffffffu) {
                            const AdjJob& JA = J.j[kBatch ? acc_job : 0u];
                            atomicAdd(JA.cell_sum + acc_cell, acc_sum);
                            if (JA.cell_sumsq) atomicAdd(JA.cell_sumsq + acc_cell, acc_sq);
                        }
                        acc_job = job;
                        acc_cell = cell;
                        acc_sum = acc_sq = 0.0;
                    }
                    const uint32_t pixel = py * L.width + px;
                    wc = kGrad ? __ldg(JJ.dloss + cell) * (1.0f / float(L.spp)) : 0.0f;
                    if (kGrad && pass == 0u && JJ.chain_rad) {
                        // the forward's radiance of this chain stands in for its first trace
                        total = __ldg(JJ.chain_rad + uint64_t(cell) * L.spp + sample);
                        if (!(total > 0.0f)) {
                            if (total != 0.0f) atomicAdd(sb + band * kAdjBandParams + 3u, wc * total);
                            next = kNextIdle;
                            continue;
                        }
                        pass = 1u;
                    }
                    rng.init(pixel, L.sample_offset + sample, band, L.seed_lo, L.seed_hi);
                    dir = camera_dir(L, px, py, rng);
                    org = mk(0.0f, S.ground_radius + fmaxf(L.observer_altitude, 0.0f), 0.0f);
                    ++n.e[SKY_EVENT_CHAIN];
                    thr = 1.0f;
                    rad = 0.0f;
                    depth = 0u;
                    next = kNextPrimary;
                }
                if (next == kNextPrimary) {
                    if (depth >= L.watchdog_limit) {
                        watchdog = true;
                        next = kNextEnd;
                        continue;
                    }
                    g = ray_geo(org, dir);
                    ++n.e[SKY_EVENT_BOUNDARY];
                    if ((L.max_orders != 0u && depth >= L.max_orders) || !next_boundary(S, g, t_max, boundary)) {
                        rad = fmaxf(rad, 0.0f);
                        next = kNextEnd;
                        continue;
                    }
                    ray = kRayPrimary;
                    next = kNextTrace;
                    continue;
                }
                // kNextLights: the vertex's next NEE sample that needs a shadow
                // ray (direct_sun_at_scatter, sky_trace.wgsl:566-585; ground
                // radiance, :587-608), else its continuation
                const AdjSet P = resolve(A.P, Lc, band);
                const float l_sun = __ldg(&S.bands[band].solar_radiance);
                const float w = wc * P.kS;
                bool shadow = false;
                while (ls < L.direct_light_samples) {
                    ++ls;
                    const V3 ldir = sample_sun_cone(JJ.sun, JJ.sun_t, JJ.sun_b, S.one_minus_cos_max, rng);
                    ++n.e[SKY_EVENT_NEE];
                    float cos_sun = 0.0f;
                    if (ground) {
                        cos_sun = fmaxf(dot3(normalize_or_y(org), ldir), 0.0f);
                        if (!(cos_sun > 0.0f)) continue;
                    }
                    g = ray_geo(madd(org, ldir, kRayEpsilonKm), ldir);
                    uint32_t sk;
                    ++n.e[SKY_EVENT_BOUNDARY];
                    if (!(next_boundary(S, g, t_max, sk) && sk == 1u)) continue;
                    dim0 = rng.dim;
                    if (ground) {
                        term = S.ground_albedo * kInvPi * l_sun * cos_sun / S.light_pdf;
                    } else {
                        mu = dot3(dir, ldir);
                        const AdjMed mp = adj_med(P, hb);
                        const float ph = mp.s > 0.0f ? vertex_phase(P, bins, mp, mu) / mp.s : 0.0f;
                        term = l_sun * ph / S.light_pdf;
                    }
                    c = w * thr * term * (1.0f / float(L.direct_light_samples));
                    shadow = true;
                    break;
                }
                if (shadow) {
                    ray = kRayShadow;
                    next = kNextTrace;
                    continue;
                }
                rad += thr * (nee * (1.0f / float(L.direct_light_samples)));
                // each branch draws its angles; one shared frame step turns them into
                // the direction (as direction_from_axis_mu / sample_cosine_hemisphere)
                V3 nd = mk(0.0f, 1.0f, 0.0f), axis = dir;
                float cos_t = 1.0f, sin_t = 0.0f, xi_phi = 0.0f;
                bool framed = true;
                if (!ground) {
                    const AdjMed mq = adj_med(P, hb);
                    float mu_c, fq;
                    if (kPhase == SKY_PHASE_TABULATED) {
                        const float target = rng.next() * mq.s;
                        const bool rayleigh = target < mq.R || !(mq.Ms > 0.0f);
                        const float xi_mu = rng.next();
                        mu_c = rayleigh ? invert_rayleigh_cdf(xi_mu) : hg_sample_mu(P, bins, xi_mu);
                        xi_phi = rng.next();
                        cos_t = fminf(fmaxf(mu_c, -1.0f), 1.0f);
                        sin_t = sqrtf(fmaxf(1.0f - cos_t * cos_t, 0.0f));
                        const float pdf = mq.R * rayleigh_phase(mu_c) +
                                          (mq.Ms > 0.0f ? mq.Ms * hg_sampling_pdf(P, bins, mu_c) : 0.0f);
                        fq = vertex_phase(P, bins, mq, mu_c) / pdf;
                    } else {
                        nd = sample_isotropic(rng);
                        framed = false;
                        mu_c = dot3(dir, nd);
                        fq = vertex_phase(P, bins, mq, mu_c) / mq.s / kIsotropicPdf;
                    }
                    thr *= fq;
                    if (kGrad && pass == 1u) vertex_terms(acc, P, bins, hb, mq, mu_c, w * (total - rad));
                } else {
                    // the Lambert bounce (sky_trace.wgsl:750-766)
                    axis = normalize_or_y(org);
                    const float u = rng.next();
                    sin_t = sqrtf(u);
                    xi_phi = rng.next();
                    cos_t = sqrtf(fmaxf(1.0f - u, 0.0f));
                }
                V3 fn = axis;
                if (framed) {
                    V3 t, bt;
                    orthonormal_basis(axis, t, bt);
                    fn = normalize_or_y(axis);
                    nd = direction_from_frame(fn, t, bt, cos_t, sin_t, xi_phi);
                }
                if (ground) {
                    const float pdf = fmaxf(dot3(fn, nd), 0.0f) * kInvPi;
                    const float cos_out = fmaxf(dot3(axis, nd), 0.0f);
                    if (pdf <= 0.0f || cos_out <= 0.0f) {
                        rad = fmaxf(rad, 0.0f);
                        next = kNextEnd;
                        continue;
                    }
                    const float f = S.ground_albedo * kInvPi * cos_out / pdf;
                    thr *= f;
                }
                if (depth >= L.rr_start_depth) {  // russian_roulette (sky_trace.wgsl:691-701)
                    const float q = fminf(fmaxf(thr, 0.05f), 0.95f);
                    if (rng.next() > q) {
                        rad = fmaxf(rad, 0.0f);
                        next = kNextEnd;
                        continue;
                    }
                    thr = thr / q;
                }
                org = madd(org, nd, kRayEpsilonKm);
                dir = nd;
                if (rad < 0.0f || rad != rad || thr < 0.0f || thr != thr) {
                    rad = 0.0f;
                    next = kNextEnd;
                    continue;
                }
                ++depth;
                next = kNextPrimary;
            }
        }
        const bool tracing = next == kNextTrace;
        if (!__any_sync(0xffffffffu, tracing)) {
            if (exhausted && __all_sync(0xffffffffu, next == kNextIdle)) break;  // no cell left, every lane idle
            continue;
        }
        if (tracing) {
            const AdjSet P = resolve(A.P, Lc, band);
            const float w = wc * P.kS;
            const bool grad = kGrad && pass == 1u;
            const float gw = ray == kRayPrimary ? (grad ? w * (total - rad) : 0.0f) : (ray == kRayRetrace ? c : 0.0f);
            const uint32_t dim_seg = rng.dim;
            float t_hit = 0.0f, w_eval = 1.0f, tau_bar = 0.0f;
            AdjBase hit_b;
            const bool hit = adj_track<!kSegEst, false>(A, P, P, band, g, t_max, rng, t_hit, hit_b, w_eval, tau_bar,
                                                        gw, acc, n, watchdog, ray != kRayPrimary);
            if (grad && kSegEst) {
                // the segment integral of the traced part: a primary segment
                // from its first random number, an unblocked shadow ray from
                // the position after its tracking
                float sw = 0.0f, t_end = t_max;
                Rng at = rng;
                if (ray == kRayPrimary) {
                    sw = gw;
                    at.dim = dim_seg;
                    if (hit) t_end = t_hit;
                } else if (ray == kRayShadow && !hit) {
                    sw = c;
                }
                segment_terms(A, P, band, g, t_end, tau_bar, sw, at, acc);
            }
            if (ray == kRayPrimary) {
                if (hit) {
                    ++n.e[SKY_EVENT_SCATTER];
                    org = madd(org, dir, t_hit);
                    hb = hit_b;
                    const AdjMed mq = adj_med(P, hb);
                    if (mq.t > 0.0f && mq.s > 0.0f) thr *= fminf(fmaxf(mq.s / mq.t, 0.0f), 1.0f);
                    if (!(mq.t > 0.0f && mq.s > 0.0f) || thr <= 0.0f) {
                        rad = fmaxf(rad, 0.0f);
                        next = kNextEnd;
                    } else {
                        ground = false;
                        ls = 0u;
                        nee = 0.0f;
                        next = kNextLights;
                    }
                } else if (boundary == 1u) {
                    if (depth == 0u && dot3(dir, load3(J.j[kBatch ? job : 0u].sun)) >= S.cos_max)
                        rad += thr * __ldg(&S.bands[band].solar_radiance);
                    rad = fmaxf(rad, 0.0f);
                    next = kNextEnd;
                } else {
                    ++n.e[SKY_EVENT_GROUND];
                    org = madd(org, dir, t_max);
                    ground = true;
                    ls = 0u;
                    nee = 0.0f;
                    next = kNextLights;
                }
            } else if (ray == kRayShadow) {
                next = kNextLights;
                if (!hit) {
                    nee += term;
                    if (grad) {
                        if (!ground) vertex_terms(acc, P, bins, hb, adj_med(P, hb), mu, c);
                        if (!kSegEst && c != 0.0f) {  // trace it again for its null collisions
                            dim1 = rng.dim;
                            rng.dim = dim0;
                            ray = kRayRetrace;
                            next = kNextTrace;
                        }
                    }
                }
            } else {
                rng.dim = dim1;
                next = kNextLights;
            }
        }
    }
    if (kCount) flush_counters(n, counters, lane);
    if (__any_sync(0xffffffffu, watchdog) && lane == 0) atomicOr(status, 1u);
    if (!kGrad) {
        if (acc_cell != 0xffffffffu) {
            const AdjJob& JA = J.j[kBatch ? acc_job : 0u];
            atomicAdd(JA.cell_sum + acc_cell, acc_sum);
            if (JA.cell_sumsq) atomicAdd(JA.cell_sumsq + acc_cell, acc_sq);
        }
        return;
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; layer_grad && i < nlayer; i += blockDim.x) {
        float v = 0.0f;
        for (uint32_t k = 0; k < copies; ++k) v += smem[k * nlayer + i];
        if (v != 0.0f) atomicAdd(layer_grad + i, double(v));
    }
    if (band_grad)
        for (uint32_t i = threadIdx.x; i < kAdjBandParams * B; i += blockDim.x)
            if (sb[i] != 0.0f) atomicAdd(band_grad + i, double(sb[i]));
}

// Majorant of Q's medium over one uniform layer: compute_majorant_grid's
// probe rule (medium.rs:63-102: layer edges, mid-point and every profile
// knot inside the layer; 1.05 x max, at least 1e-8) with the layer's own
// scales applied at its edges.
__device__ float bake_one(const AdjCtx& A, const AdjSet& Q, uint32_t band, uint32_t layer) {
    const DevScene& S = A.S;
    const float lo = float(layer) * S.layer_dz, hi = float(layer + 1u) * S.layer_dz;
    const float* p = Q.layer + 3 * layer;
    const float sR = p[0] * Q.kR, sM = p[1] * Q.kM, sO = p[2] * Q.kO;
    auto ext = [&](float h) {
        const AdjBase b = adj_base(S, band, h);
        return sR * b.uR + sM * b.uM + sO * b.uO;
    };
    float mx = fmaxf(fmaxf(ext(lo), ext(hi)), ext(0.5f * (lo + hi)));
    for (uint32_t k = 0; k < S.knot_count; ++k) {
        const float z = S.knot_z[k];
        if (z > lo && z < hi) mx = fmaxf(mx, ext(z));
    }
    return fmaxf(fmaxf(mx, 0.0f) * 1.05f, 1.0e-8f);
}

// Henyey-Greenstein table of g at the cube-root bin centres, its derivative
// in g, and the sampling CDF / per-bin pdf of one row
// (build_phase_sampling_tables, phase.rs:105-135).  |g| is held below 0.99.
__device__ void build_hg_tables(float g_in, uint32_t bins, float* values, float* dvalues, float* cdf,
                                float* bin_pdf) {
    const double g = double(fminf(fmaxf(g_in, -0.99f), 0.99f));
    const double four_pi = 4.0 * 3.14159265358979323846;
    for (uint32_t i = threadIdx.x; i < bins; i += blockDim.x) {
        const double u = (double(i) + 0.5) / double(bins);
        const double mu = 1.0 - 2.0 * u * u * u;
        const double d = 1.0 + g * g - 2.0 * g * mu;
        const double sd = sqrt(d);
        values[i] = float((1.0 - g * g) / (four_pi * d * sd));
        dvalues[i] = float((-2.0 * g * d - 3.0 * (1.0 - g * g) * (g - mu)) / (four_pi * d * d * sd));
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const float two_pi = 2.0f * kPi;
        float norm = 0.0f;
        for (uint32_t b = 0; b < bins; ++b)
            norm += two_pi * fmaxf(values[b], 0.0f) * fabsf(mu_edge(b, bins) - mu_edge(b + 1u, bins));
        norm = fmaxf(norm, 1.0e-20f);
        float cum = 0.0f;
        for (uint32_t b = 0; b < bins; ++b) {
            const float v = fmaxf(values[b], 0.0f);
            cum += two_pi * v * fabsf(mu_edge(b, bins) - mu_edge(b + 1u, bins)) / norm;
            cdf[b] = fminf(cum, 1.0f);
            bin_pdf[b] = v / norm;
        }
        cdf[bins - 1u] = 1.0f;
    }
}

// Blocks [0, B) bake one band each: majorants of every uniform layer, then
// the tracking grid (the layers merged by the dynamic programme of the
// scene's merged grid, or one tracking layer per uniform layer).  Block B
// builds P's HG tables, block B + 1 Q's.
__global__ void __launch_bounds__(128) adjoint_prepare_kernel(AdjCtx A, AdjWorkspace W) {
    extern __shared__ float smem[];
    const DevScene& S = A.S;
    const uint32_t B = S.band_count, L = S.layer_count, bins = S.phase_bins;
    if (blockIdx.x >= B) {
        const bool q = blockIdx.x > B;
        const AdjParamSet& X = q ? A.Q : A.P;
        float* base = q ? W.q_tables : W.p_tables;
        build_hg_tables(X.layer[3 * L + 1], bins, base, base + bins, base + 2 * bins, base + 3 * bins);
        return;
    }
    const uint32_t band = blockIdx.x;
    const AdjSet Q = resolve(A.Q, L, band);
    float* maj = smem;                                           // [L]
    float* best = smem + L;                                      // [L + 1]
    uint32_t* from = reinterpret_cast<uint32_t*>(best + L + 1);  // [L + 1]
    for (uint32_t l = threadIdx.x; l < L; l += blockDim.x) {
        const float v = bake_one(A, Q, band, l);
        maj[l] = v;
        W.layer_maj[band * L + l] = v;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    const float dz = S.layer_dz;
    if (A.merge) {
        best[0] = 0.0f;
        for (uint32_t j = 1; j <= L; ++j) {
            float bj = INFINITY, mx = 0.0f, sum = 0.0f;
            uint32_t fj = 0;
            for (uint32_t i = j; i-- > 0;) {  // group [i, j)
                const float m = fmaxf(maj[i], 1e-8f);
                mx = fmaxf(mx, m);
                sum += m;
                const float c = best[i] + A.crossing_cost + (mx * float(j - i) - sum) * dz;
                if (c < bj) {
                    bj = c;
                    fj = i;
                }
            }
            best[j] = bj;
            from[j] = fj;
        }
    } else {
        for (uint32_t j = 1; j <= L; ++j) from[j] = j - 1u;
    }
    uint32_t groups = 0;
    for (uint32_t j = L; j > 0; j = from[j]) ++groups;
    float* radius = W.radius + band * (L + 1u);
    float* gmaj = W.maj + band * (L + 1u);
    uint16_t* map = W.map + band * L;
    uint32_t idx = groups;
    for (uint32_t j = L; j > 0; j = from[j]) {
        --idx;
        const uint32_t k0 = from[j];
        float mx = 0.0f;
        for (uint32_t k = k0; k < j; ++k) {
            mx = fmaxf(mx, fmaxf(maj[k], 0.00000001f));
            map[k] = uint16_t(idx);
        }
        gmaj[idx] = mx;
        radius[idx] = S.ground_radius + float(k0) * dz;
    }
    gmaj[groups] = 0.0f;
    radius[groups] = S.ground_radius + S.top_altitude;
    W.count[band] = groups;
}

uint32_t grid_blocks(const void* kernel, uint32_t threads, size_t smem, uint64_t want) {
    int device = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, int(threads), smem);
    const uint64_t resident = uint64_t(std::max(sms, 1)) * uint64_t(std::max(per_sm, 1));
    return uint32_t(std::max<uint64_t>(1, std::min<uint64_t>(want, resident)));
}

size_t align256(size_t v) { return (v + 255) / 256 * 256; }

}  // namespace

size_t adjoint_workspace_bytes(uint32_t B, uint32_t L, uint32_t bins) {
    return 2 * align256(4 * size_t(bins) * sizeof(float)) + align256(size_t(B) * L * sizeof(float)) +
           2 * align256(size_t(B) * (L + 1) * sizeof(float)) + align256(size_t(B) * L * sizeof(uint16_t)) +
           align256(size_t(B) * sizeof(uint32_t)) + align256(sizeof(uint32_t));
}

AdjWorkspace adjoint_workspace(void* base, uint32_t B, uint32_t L, uint32_t bins) {
    unsigned char* p = static_cast<unsigned char*>(base);
    AdjWorkspace W;
    W.p_tables = reinterpret_cast<float*>(p);
    p += align256(4 * size_t(bins) * sizeof(float));
    W.q_tables = reinterpret_cast<float*>(p);
    p += align256(4 * size_t(bins) * sizeof(float));
    W.layer_maj = reinterpret_cast<float*>(p);
    p += align256(size_t(B) * L * sizeof(float));
    W.radius = reinterpret_cast<float*>(p);
    p += align256(size_t(B) * (L + 1) * sizeof(float));
    W.maj = reinterpret_cast<float*>(p);
    p += align256(size_t(B) * (L + 1) * sizeof(float));
    W.map = reinterpret_cast<uint16_t*>(p);
    p += align256(size_t(B) * L * sizeof(uint16_t));
    W.count = reinterpret_cast<uint32_t*>(p);
    p += align256(size_t(B) * sizeof(uint32_t));
    W.next_cell = reinterpret_cast<uint32_t*>(p);
    return W;
}

cudaError_t launch_adjoint_prepare(const AdjCtx& A, const AdjWorkspace& W, cudaStream_t stream) {
    const uint32_t L = A.S.layer_count;
    const size_t smem = (size_t(L) + 2u * (size_t(L) + 1u)) * sizeof(float);
    const uint32_t blocks = A.S.band_count + (A.distinct ? 2u : 1u);
    adjoint_prepare_kernel<<<blocks, 128, smem, stream>>>(A, W);
    return cudaGetLastError();
}

// Kernel arguments may hold up to 32764 bytes on this architecture.
static_assert(sizeof(AdjCtx) + sizeof(AdjJobs) + 64 <= 32000, "ray-loop kernel arguments exceed the limit");

// One launch of the ray-loop kernel, persistent grid.
template <int kPhase, bool kGrad, bool kCount, bool kSegEst, bool kBatch>
cudaError_t launch_ray_loop_shape(const AdjCtx& A, const AdjJobs& J, double* layer_grad, double* band_grad,
                                  unsigned long long* counters, uint32_t* status, uint32_t copies,
                                  uint32_t* next_cell, size_t smem, cudaStream_t stream) {
    const void* k = reinterpret_cast<const void*>(adjoint_grad_kernel<kPhase, kGrad, kCount, kSegEst, kBatch>);
    const uint64_t want = (uint64_t(J.cells) * 32u + 255u) / 256u;  // a warp per cell at most
    adjoint_grad_kernel<kPhase, kGrad, kCount, kSegEst, kBatch>
        <<<grid_blocks(k, 256, smem, want), 256, smem, stream>>>(A, J, layer_grad, band_grad, counters, status,
                                                                 copies, next_cell);
    return cudaGetLastError();
}

template <int kPhase, bool kGrad, bool kCount, bool kSegEst>
cudaError_t launch_ray_loop_est(const AdjCtx& A, const AdjJobs& J, double* layer_grad, double* band_grad,
                                unsigned long long* counters, uint32_t* status, uint32_t copies, uint32_t* next_cell,
                                size_t smem, cudaStream_t stream) {
    if (J.count > 1u)
        return launch_ray_loop_shape<kPhase, kGrad, kCount, kSegEst, true>(A, J, layer_grad, band_grad, counters,
                                                                           status, copies, next_cell, smem, stream);
    return launch_ray_loop_shape<kPhase, kGrad, kCount, kSegEst, false>(A, J, layer_grad, band_grad, counters, status,
                                                                        copies, next_cell, smem, stream);
}

// The estimator's instantiation (the primal needs no gradient code: segment form).
template <int kPhase, bool kGrad, bool kCount>
cudaError_t launch_ray_loop(const AdjCtx& A, const AdjJobs& J, double* layer_grad, double* band_grad,
                            unsigned long long* counters, uint32_t* status, uint32_t copies, uint32_t* next_cell,
                            size_t smem, cudaStream_t stream) {
    if (kGrad && A.estimator == SKY_ADJOINT_NULL_COLLISIONS)
        return launch_ray_loop_est<kPhase, kGrad, kCount, false>(A, J, layer_grad, band_grad, counters, status, copies,
                                                                 next_cell, smem, stream);
    return launch_ray_loop_est<kPhase, kGrad, kCount, true>(A, J, layer_grad, band_grad, counters, status, copies,
                                                            next_cell, smem, stream);
}

template <bool kGrad>
cudaError_t launch_ray_loop_phase(const AdjCtx& A, const AdjJobs& J, double* layer_grad, double* band_grad,
                                  unsigned long long* counters, uint32_t* status, uint32_t copies,
                                  uint32_t* next_cell, size_t smem, cudaStream_t stream) {
    if (J.j[0].L.phase_sampling == SKY_PHASE_TABULATED)
        return counters ? launch_ray_loop<SKY_PHASE_TABULATED, kGrad, true>(A, J, layer_grad, band_grad, counters,
                                                                             status, copies, next_cell, smem, stream)
                        : launch_ray_loop<SKY_PHASE_TABULATED, kGrad, false>(A, J, layer_grad, band_grad, counters,
                                                                              status, copies, next_cell, smem, stream);
    return counters ? launch_ray_loop<SKY_PHASE_ISOTROPIC, kGrad, true>(A, J, layer_grad, band_grad, counters, status,
                                                                         copies, next_cell, smem, stream)
                    : launch_ray_loop<SKY_PHASE_ISOTROPIC, kGrad, false>(A, J, layer_grad, band_grad, counters,
                                                                          status, copies, next_cell, smem, stream);
}

cudaError_t launch_adjoint_primal(const AdjCtx& A, const AdjJobs& J, bool accumulate, unsigned long long* counters,
                                  uint32_t* status, uint32_t* next_cell, cudaStream_t stream) {
    cudaError_t e;
    if (!A.distinct) {
        // P = Q: the ray loop, adding into the cell sums
        if (!accumulate)
            for (uint32_t i = 0; i < J.count; ++i) {
                const AdjJob& j = J.j[i];
                if ((e = cudaMemsetAsync(j.cell_sum, 0, size_t(j.cell_count) * sizeof(double), stream)) != cudaSuccess)
                    return e;
                if (j.cell_sumsq &&
                    (e = cudaMemsetAsync(j.cell_sumsq, 0, size_t(j.cell_count) * sizeof(double), stream)) != cudaSuccess)
                    return e;
            }
        if ((e = cudaMemsetAsync(next_cell, 0, sizeof(uint32_t), stream)) != cudaSuccess) return e;
        return launch_ray_loop_phase<false>(A, J, nullptr, nullptr, counters, status, 0u, next_cell, 0, stream);
    }
    // sampling under Q, evaluation under P: a warp per cell (one render)
    const AdjJob& j = J.j[0];
    const uint64_t cells = j.cell_count;
    const uint64_t blocks = (cells * 32u + 255u) / 256u;
    if (blocks > 0x7fffffffull) return cudaErrorInvalidConfiguration;
    const dim3 grid(static_cast<uint32_t>(blocks));
    const uint32_t acc = accumulate ? 1u : 0u;
    if (j.L.phase_sampling == SKY_PHASE_TABULATED)
        adjoint_primal_kernel<SKY_PHASE_TABULATED>
            <<<grid, 256, 0, stream>>>(A, j.L, j.cell_sum, j.cell_sumsq, acc, counters, status, cells);
    else
        adjoint_primal_kernel<SKY_PHASE_ISOTROPIC>
            <<<grid, 256, 0, stream>>>(A, j.L, j.cell_sum, j.cell_sumsq, acc, counters, status, cells);
    return cudaGetLastError();
}

cudaError_t launch_adjoint_grad(const AdjCtx& A, const AdjJobs& J, double* layer_grad, double* band_grad,
                                unsigned long long* counters, uint32_t* status, uint32_t* next_cell,
                                cudaStream_t stream) {
    cudaError_t e = cudaMemsetAsync(next_cell, 0, sizeof(uint32_t), stream);
    if (e != cudaSuccess) return e;
    const size_t nlayer = size_t(3u * A.S.layer_count + 2u), nband = size_t(kAdjBandParams) * A.S.band_count;
    // one layer-gradient copy per warp while it stays within the default 48 KB
    const uint32_t copies = (8 * nlayer + nband) * sizeof(float) <= 48u * 1024u ? 8u : 1u;
    const size_t smem = (copies * nlayer + nband) * sizeof(float);
    return launch_ray_loop_phase<true>(A, J, layer_grad, band_grad, counters, status, copies, next_cell, smem, stream);
}

}  // namespace sky
