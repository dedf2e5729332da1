// trace_wavefront.cu — persistent tracer with per-lane path regeneration.
//
// The plain kernel runs each chain to completion, so a warp waits for its
// longest path (escaping rays finish after a few layer crossings, rays that
// scatter near the horizon run dozens of events).  Here the whole path loop
// of sky_trace.wgsl:703-776 is turned into a small state machine: every loop
// iteration a lane performs ONE action (a delta-tracking step or layer
// crossing, a scattering / ground / light-sample event), and a lane whose
// chain ends immediately takes the next chain of its warp's work group.  The
// random stream of every chain is consumed in exactly the order the plain
// kernel (and the reference shader) consumes it, so both kernels trace the
// same paths.
//
// Work: a persistent grid (a few blocks per SM) pulls work groups from a
// global counter.  A group is `pixels_per_group` pixels x all bands x all
// samples of one job; its chains are handed to lanes in order, and finished
// chains add their radiance to the group's per-cell FP64 sums in shared
// memory.  When a group is done the warp writes the cell sums, the mean film
// and the per-pixel CIE XYZ and its variance (shuffle reductions over the
// bands) with coalesced stores.
//
// Tables: when every job of a launch shares one set of scene tables (an
// elevation sweep differs only in the sun) the extinction knots, finder,
// band constants and tracking grids are staged once per block in shared
// memory; each warp keeps a copy of its current job's constants in shared
// memory with the table pointers redirected there.

#include <algorithm>
#include <cstdio>

#include "sky_device.cuh"
#include "trace_kernels.h"

namespace sky {
namespace {

constexpr uint32_t kFull = 0xffffffffu;
// Upper bound on state-machine iterations of one warp for one work group; a
// typical group needs ~1e4-1e5.  Exceeding it abandons the group and sets
// status bit 2 (reported as a watchdog error) instead of running on.
constexpr uint32_t kMaxGroupIterations = 1u << 26;

enum : uint32_t {
    ST_IDLE = 0,
    ST_BOUNDARY,
    ST_TRACK,
    ST_SCATTER,
    ST_GROUND,
    ST_LIGHT,
    ST_SHADOW_DONE,
    ST_CONTINUE,
};

// Delta tracking state along the current ray (camera/continuation or shadow).
struct Tracker {
    RayGeo g;
    float t, t_max, t_seg, tau, maj;
    int m;       // merged layer (mode 2)
    int mdir;    // mode 2: crossing direction; modes 0/1: 1 while a segment is set up
    uint32_t guard;
    bool need_draw;
};

template <int kTracking>
__device__ __forceinline__ void track_begin(const DevScene& S, uint32_t band, Tracker& k, Rng& rng, Counters& n) {
    k.t = 0.0f;
    k.guard = 0;
    k.need_draw = true;
    k.mdir = 0;
    if (kTracking == SKY_TRACKING_MERGED_LAYERS) {
        const MergedGrid G = merged_grid(S, band);
        k.m = merged_layer_at(S, G, altitude_at(k.g, fminf(kRayEpsilonKm, k.t_max), S.ground_radius));
        k.t_seg = merged_crossing(G, k.g, k.m, 0.0f, k.t_max, k.mdir);
        k.maj = G.maj[k.m];
        ++n.e[SKY_EVENT_SEGMENT];
        k.tau = -__logf(fmaxf(1.0f - rng.next(), 0.0000001f));
        k.need_draw = false;
    }
}

// One tracking action: 0 = continue, 1 = real collision at k.t, 2 = reached
// k.t_max without a collision.  Draw order identical to track_ray() of the
// plain kernel for each mode.
template <int kTracking>
__device__ __forceinline__ int track_action(const DevScene& S, uint32_t band, Tracker& k, Rng& rng, Counters& n,
                                           bool& watchdog) {
    const float2* sig_row = S.sigma_t + band * S.knot_count;
    if (kTracking == SKY_TRACKING_MERGED_LAYERS) {
        const float dt = k.tau / k.maj;
        if (k.t + dt < k.t_seg) {
            k.t = k.t + dt;
            ++n.e[SKY_EVENT_TRACK_STEP];
            const float sig =
                sigma_t_at(S, S.knot_z, S.finder, sig_row, 0u, altitude_at(k.g, k.t, S.ground_radius));
            if (rng.next() * k.maj < sig) return 1;
            k.tau = -__logf(fmaxf(1.0f - rng.next(), 0.0000001f));
            return 0;
        }
        if (k.mdir == 0) return 2;
        if (++k.guard > 100000u) {
            watchdog = true;
            return 2;
        }
        k.tau = fmaxf(k.tau - (k.t_seg - k.t) * k.maj, 0.0f);
        k.t = k.t_seg;
        k.m += k.mdir;
        const MergedGrid G = merged_grid(S, band);
        k.t_seg = merged_crossing(G, k.g, k.m, k.t, k.t_max, k.mdir);
        k.maj = G.maj[k.m];
        ++n.e[SKY_EVENT_SEGMENT];
        return 0;
    }
    if (k.mdir == 0) {  // set up the next reference segment (sky_trace.wgsl:409-420)
        if (k.t >= k.t_max) return 2;
        if (k.guard > 100000u) {
            watchdog = true;
            return 2;
        }
        ++k.guard;
        uint32_t layer;
        k.t_seg = next_segment_end(S, k.g, k.t, k.t_max, layer);
        k.maj = fmaxf(S.majorants[band * S.layer_count + layer], 0.00000001f);
        ++n.e[SKY_EVENT_SEGMENT];
        k.mdir = 1;
        return 0;
    }
    if (kTracking == SKY_TRACKING_RESIDUAL_CARRY) {
        if (k.need_draw) {
            k.tau = -__logf(fmaxf(1.0f - rng.next(), 0.0000001f));
            k.need_draw = false;
        }
        const float dt = k.tau / k.maj;
        if (k.t + dt >= k.t_seg) {
            k.tau = fmaxf(k.tau - (k.t_seg - k.t) * k.maj, 0.0f);
            k.t = k.t_seg;
            k.mdir = 0;
            return 0;
        }
        k.t = k.t + dt;
        k.need_draw = true;
    } else {
        if (k.t >= k.t_seg) {
            k.t = k.t_seg;
            k.mdir = 0;
            return 0;
        }
        const float u = fmaxf(1.0f - rng.next(), 0.0000001f);
        const float tn = k.t - __logf(u) / k.maj;
        if (tn >= k.t_seg) {
            k.t = k.t_seg;
            k.mdir = 0;
            return 0;
        }
        k.t = tn;
    }
    ++n.e[SKY_EVENT_TRACK_STEP];
    const float sig = sigma_t_at(S, S.knot_z, S.finder, sig_row, 0u, altitude_at(k.g, k.t, S.ground_radius));
    return rng.next() * k.maj < sig ? 1 : 0;
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

__device__ __forceinline__ void copy_words(void* dst, const void* src, uint32_t bytes, uint32_t tid, uint32_t nthreads) {
    const uint32_t* s = static_cast<const uint32_t*>(src);
    uint32_t* d = static_cast<uint32_t*>(dst);
    for (uint32_t i = tid; i < bytes / 4u; i += nthreads) d[i] = s[i];
}

template <int kTracking, int kPhase, bool kStaged>
__global__ void __launch_bounds__(256) wavefront_kernel(const DevJob* __restrict__ jobs, uint32_t num_jobs,
                                                        uint32_t total_groups, StageLayout lay,
                                                        uint32_t* __restrict__ work_counter,
                                                        unsigned long long* __restrict__ counters,
                                                        uint32_t* __restrict__ status) {
    extern __shared__ __align__(16) unsigned char smem[];
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warp = threadIdx.x >> 5;
    const uint32_t nwarps = blockDim.x >> 5;

    // Stage the shared scene tables once per block.
    if (kStaged) {
        const DevScene& S0 = jobs[0].S;
        copy_words(smem + lay.knot_z, S0.knot_z, lay.knot_z_bytes, threadIdx.x, blockDim.x);
        copy_words(smem + lay.finder, S0.finder, lay.finder_bytes, threadIdx.x, blockDim.x);
        copy_words(smem + lay.sigma_t, S0.sigma_t, lay.sigma_t_bytes, threadIdx.x, blockDim.x);
        copy_words(smem + lay.bands, S0.bands, lay.bands_bytes, threadIdx.x, blockDim.x);
        copy_words(smem + lay.trk_radius, S0.trk_radius, lay.trk_bytes, threadIdx.x, blockDim.x);
        copy_words(smem + lay.trk_maj, S0.trk_maj, lay.trk_bytes, threadIdx.x, blockDim.x);
        copy_words(smem + lay.trk_map, S0.trk_map, lay.trk_map_bytes, threadIdx.x, blockDim.x);
        copy_words(smem + lay.trk_count, S0.trk_count, lay.trk_count_bytes, threadIdx.x, blockDim.x);
        copy_words(smem + lay.trk_off, S0.trk_off, lay.trk_count_bytes, threadIdx.x, blockDim.x);
        if (lay.majorants_bytes)
            copy_words(smem + lay.majorants, S0.majorants, lay.majorants_bytes, threadIdx.x, blockDim.x);
        __syncthreads();
    }
    DevJob& J = *reinterpret_cast<DevJob*>(smem + lay.jobs + warp * sizeof(DevJob));
    double* acc_sum = reinterpret_cast<double*>(smem + lay.acc) + size_t(warp) * 2u * lay.max_cells;
    double* acc_sq = acc_sum + lay.max_cells;

    Counters n;
    n.clear();
    bool watchdog = false;
    bool stalled = false;

    uint32_t group = 0;
    if (lane == 0) group = atomicAdd(work_counter, 1u);
    group = __shfl_sync(kFull, group, 0);
    uint32_t cached_job = 0xffffffffu;
    while (group < total_groups) {
        uint32_t ji = 0;
        while (ji + 1 < num_jobs && jobs[ji + 1].group_begin <= group) ++ji;
        if (ji != cached_job) {
            __syncwarp();
            copy_words(&J, &jobs[ji], sizeof(DevJob), lane, 32u);
            __syncwarp();
            if (kStaged && lane == 0) {
                J.S.knot_z = reinterpret_cast<const float*>(smem + lay.knot_z);
                J.S.finder = reinterpret_cast<const uint16_t*>(smem + lay.finder);
                J.S.sigma_t = reinterpret_cast<const float2*>(smem + lay.sigma_t);
                J.S.bands = reinterpret_cast<const DevBand*>(smem + lay.bands);
                J.S.trk_radius = reinterpret_cast<const float*>(smem + lay.trk_radius);
                J.S.trk_maj = reinterpret_cast<const float*>(smem + lay.trk_maj);
                J.S.trk_map = reinterpret_cast<const uint16_t*>(smem + lay.trk_map);
                J.S.trk_count = reinterpret_cast<const uint32_t*>(smem + lay.trk_count);
                J.S.trk_off = reinterpret_cast<const uint32_t*>(smem + lay.trk_off);
                if (lay.majorants_bytes) J.S.majorants = reinterpret_cast<const float*>(smem + lay.majorants);
            }
            __syncwarp();
            cached_job = ji;
        }
        const DevScene& S = J.S;
        const DevLaunch& L = J.L;
        const uint32_t B = L.band_count;
        const uint64_t pixels_total = uint64_t(L.width) * L.height;
        const uint64_t pixel0 = uint64_t(group - J.group_begin) * J.pixels_per_group;
        const uint32_t npix = uint32_t(min(uint64_t(J.pixels_per_group), pixels_total - pixel0));
        const uint32_t G = npix * B;
        const uint32_t total = G * L.spp;
        for (uint32_t c = lane; c < G; c += 32u) {
            acc_sum[c] = 0.0;
            acc_sq[c] = 0.0;
        }
        __syncwarp();

        // ---- lane state ----
        uint32_t state = ST_IDLE;
        uint32_t cell = 0, band = 0, x = 0, y = 0;
        Rng rng;
        rng.k0 = rng.k1 = rng.k2 = rng.dim = 0;
        V3 org = mk(0.0f, 0.0f, 0.0f), dir = mk(0.0f, 1.0f, 0.0f), pos = org, ldir = dir;
        float throughput = 0.0f, radiance = 0.0f, nee = 0.0f, alt_pos = 0.0f, trans = 0.0f, l_sun = 0.0f;
        uint32_t depth = 0, light_i = 0, kind = 0;
        bool shadow = false, ground_event = false;
        Tracker k;
        k.t = k.t_max = k.t_seg = k.tau = k.maj = 0.0f;
        k.m = k.mdir = 0;
        k.guard = 0;
        k.need_draw = true;
        k.g = RayGeo{0.0f, 0.0f, 0.0f};
        const float inv_lights = 1.0f / float(L.direct_light_samples);
        uint32_t issued = 0;
        uint32_t iterations = 0;  // warp-uniform

        for (;;) {
            const uint32_t idle = __ballot_sync(kFull, state == ST_IDLE);
            if (idle == kFull && issued >= total) break;
            if (++iterations > kMaxGroupIterations) {  // never expected: abandon the group, report it
                stalled = true;
                break;
            }
            if (idle != 0u && issued < total) {
                const uint32_t j = issued + __popc(idle & ((1u << lane) - 1u));
                issued += __popc(idle);
                if (state == ST_IDLE && j < total) {
                    // new chain: cell-major within a sample so all cells progress together
                    cell = j % G;
                    const uint32_t sample = L.sample_offset + j / G;
                    band = cell % B;
                    const uint64_t pixel = pixel0 + cell / B;
                    x = uint32_t(pixel % L.width);
                    y = uint32_t(pixel / L.width);
                    rng.init(uint32_t(pixel), sample, band, L.seed_lo, L.seed_hi);
                    dir = camera_dir(L, x, y, rng);
                    org = mk(0.0f, S.ground_radius + fmaxf(L.observer_altitude, 0.0f), 0.0f);
                    throughput = 1.0f;
                    radiance = 0.0f;
                    depth = 0;
                    l_sun = S.bands[band].solar_radiance;
                    ++n.e[SKY_EVENT_CHAIN];
                    state = ST_BOUNDARY;
                }
            }
            if (state == ST_IDLE) continue;

            bool finished = false;
            float result = 0.0f;
            if (state == ST_TRACK) {
                const int r = track_action<kTracking>(S, band, k, rng, n, watchdog);
                if (r == 1) {
                    if (shadow) {
                        trans = 0.0f;
                        state = ST_SHADOW_DONE;
                    } else {
                        state = ST_SCATTER;
                    }
                } else if (r == 2) {
                    if (shadow) {
                        trans = 1.0f;
                        state = ST_SHADOW_DONE;
                    } else if (kind == 1u) {
                        if (depth == 0u && dot3(dir, load3(S.sun)) >= S.cos_max) radiance += throughput * l_sun;
                        finished = true;
                        result = fmaxf(radiance, 0.0f);
                    } else {
                        state = ST_GROUND;
                    }
                }
            } else if (state == ST_BOUNDARY) {
                if (depth >= L.watchdog_limit) {
                    watchdog = true;
                    finished = true;
                    result = radiance;
                } else if (L.max_orders != 0u && depth >= L.max_orders) {
                    finished = true;
                    result = fmaxf(radiance, 0.0f);
                } else {
                    k.g = ray_geo(org, dir);
                    ++n.e[SKY_EVENT_BOUNDARY];
                    float tb;
                    uint32_t kd;
                    if (!next_boundary(S, k.g, tb, kd)) {
                        finished = true;
                        result = fmaxf(radiance, 0.0f);
                    } else {
                        kind = kd;
                        k.t_max = tb;
                        shadow = false;
                        track_begin<kTracking>(S, band, k, rng, n);
                        state = ST_TRACK;
                    }
                }
            } else if (state == ST_SCATTER) {
                ++n.e[SKY_EVENT_SCATTER];
                pos = madd(org, dir, k.t);
                alt_pos = altitude_at(k.g, k.t, S.ground_radius);
                const Coeffs c = coefficients_at(S, S.knot_z, S.finder, band, alt_pos);
                if (c.extinction <= 0.0f || c.scattering <= 0.0f) {
                    finished = true;
                    result = fmaxf(radiance, 0.0f);
                } else {
                    throughput *= fminf(fmaxf(c.scattering / c.extinction, 0.0f), 1.0f);
                    if (throughput <= 0.0f) {
                        finished = true;
                        result = fmaxf(radiance, 0.0f);
                    } else {
                        ground_event = false;
                        light_i = 0;
                        nee = 0.0f;
                        state = ST_LIGHT;
                    }
                }
            } else if (state == ST_GROUND) {
                ++n.e[SKY_EVENT_GROUND];
                pos = madd(org, dir, k.t_max);
                ground_event = true;
                light_i = 0;
                nee = 0.0f;
                state = ST_LIGHT;
            } else if (state == ST_LIGHT) {
                if (light_i >= L.direct_light_samples) {
                    state = ST_CONTINUE;
                } else {
                    ldir = sample_sun_cone(S, rng);
                    ++n.e[SKY_EVENT_NEE];
                    bool go = true;
                    if (ground_event) go = fmaxf(dot3(normalize_or_y(pos), ldir), 0.0f) > 0.0f;
                    if (go) {
                        k.g = ray_geo(madd(pos, ldir, kRayEpsilonKm), ldir);
                        ++n.e[SKY_EVENT_BOUNDARY];
                        float tb;
                        uint32_t kd;
                        go = next_boundary(S, k.g, tb, kd) && kd == 1u;
                        if (go) {
                            k.t_max = tb;
                            shadow = true;
                            track_begin<kTracking>(S, band, k, rng, n);
                            state = ST_TRACK;
                        }
                    }
                    if (!go) ++light_i;
                }
            } else if (state == ST_SHADOW_DONE) {
                if (trans > 0.0f) {
                    if (ground_event) {
                        const float cos_sun = fmaxf(dot3(normalize_or_y(pos), ldir), 0.0f);
                        nee += S.ground_albedo * kInvPi * l_sun * trans * cos_sun / S.light_pdf;
                    } else {
                        const Coeffs c = coefficients_at(S, S.knot_z, S.finder, band, alt_pos);
                        nee += l_sun * trans * mixed_phase(S, c, band, dot3(dir, ldir)) / S.light_pdf;
                    }
                }
                ++light_i;
                state = ST_LIGHT;
            } else {  // ST_CONTINUE
                radiance += throughput * (nee * inv_lights);
                bool alive = true;
                V3 nd;
                if (!ground_event) {
                    const Coeffs c = coefficients_at(S, S.knot_z, S.finder, band, alt_pos);
                    if (kPhase == SKY_PHASE_TABULATED) {
                        throughput *= sample_tabulated(S, c, band, dir, rng, nd);
                    } else {
                        nd = sample_isotropic(rng);
                        throughput *= mixed_phase(S, c, band, dot3(dir, nd)) / kIsotropicPdf;
                    }
                } else {
                    const V3 normal = normalize_or_y(pos);
                    float pdf;
                    nd = sample_cosine_hemisphere(normal, rng, pdf);
                    const float cos_out = fmaxf(dot3(normal, nd), 0.0f);
                    if (pdf <= 0.0f || cos_out <= 0.0f) alive = false;
                    else throughput *= S.ground_albedo * kInvPi * cos_out / pdf;
                }
                if (alive && depth >= L.rr_start_depth) {
                    const float q = fminf(fmaxf(throughput, 0.05f), 0.95f);
                    if (rng.next() > q) alive = false;
                    else throughput = throughput / q;
                }
                if (!alive) {
                    finished = true;
                    result = fmaxf(radiance, 0.0f);
                } else {
                    org = madd(pos, nd, kRayEpsilonKm);
                    dir = nd;
                    if (radiance < 0.0f || radiance != radiance || throughput < 0.0f || throughput != throughput) {
                        finished = true;
                        result = 0.0f;
                    } else {
                        ++depth;
                        state = ST_BOUNDARY;
                    }
                }
            }
            if (finished) {
                const double rd = double(result);
                atomicAdd(acc_sum + cell, rd);
                atomicAdd(acc_sq + cell, rd * rd);
                state = ST_IDLE;
            }
        }
        __syncwarp();

        // ---- group epilogue: cell sums, film, XYZ (coalesced, shuffle-reduced) ----
        const double n_total = double(J.total_spp);
        const double inv_n = 1.0 / n_total;
        const uint64_t cell0 = pixel0 * B;
        for (uint32_t p = 0; p < npix; ++p) {
            double xyz[3] = {0.0, 0.0, 0.0}, var[3] = {0.0, 0.0, 0.0};
            for (uint32_t b = lane; b < B; b += 32u) {
                const uint32_t c = p * B + b;
                double s = acc_sum[c], q = acc_sq[c];
                if (J.accumulate) {
                    s += J.cell_sum[cell0 + c];
                    if (J.cell_sumsq) q += J.cell_sumsq[cell0 + c];
                }
                J.cell_sum[cell0 + c] = s;
                if (J.cell_sumsq) J.cell_sumsq[cell0 + c] = q;
                const double mean = s * inv_n;
                if (J.film) J.film[cell0 + c] = fmaxf(float(mean), 0.0f);
                double var_mean = 0.0;
                if (J.total_spp > 1u) var_mean = fmax((q - s * mean) / (n_total - 1.0), 0.0) * inv_n;
                const DevBand& bd = S.bands[b];
#pragma unroll
                for (int ch = 0; ch < 3; ++ch) {
                    const double w = double(bd.xyz[ch]);
                    xyz[ch] += mean * w;
                    var[ch] += var_mean * w * w;
                }
            }
            if (J.xyz || J.xyz_var) {
#pragma unroll
                for (int ch = 0; ch < 3; ++ch) {
                    xyz[ch] = warp_sum_d(xyz[ch]);
                    var[ch] = warp_sum_d(var[ch]);
                }
                if (lane < 3u) {
                    const double vx = lane == 0 ? xyz[0] : (lane == 1 ? xyz[1] : xyz[2]);
                    const double vv = lane == 0 ? var[0] : (lane == 1 ? var[1] : var[2]);
                    const uint64_t px = pixel0 + p;
                    if (J.xyz) J.xyz[px * 3 + lane] = vx;
                    if (J.xyz_var) J.xyz_var[px * 3 + lane] = vv;
                }
            }
        }
        __syncwarp();
        if (lane == 0) group = atomicAdd(work_counter, 1u);
        group = __shfl_sync(kFull, group, 0);
    }

    if (counters) {
#pragma unroll
        for (int e = 0; e < SKY_EVENT_COUNT; ++e) {
            uint32_t v = n.e[e];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
            if (lane == 0 && v) atomicAdd(counters + e, (unsigned long long)v);
        }
    }
    if (__any_sync(kFull, watchdog) && lane == 0) atomicOr(status, 1u);
    if (__any_sync(kFull, stalled) && lane == 0) atomicOr(status, 2u);
    (void)nwarps;
}

template <int kTracking, int kPhase, bool kStaged>
cudaError_t launch_one(const WaveLaunch& w, cudaStream_t stream) {
    auto fn = wavefront_kernel<kTracking, kPhase, kStaged>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(w.smem_bytes));
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, int(w.block_threads), w.smem_bytes);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    if (w.max_blocks_per_sm > 0) per_sm = std::min(per_sm, int(w.max_blocks_per_sm));
    int device = 0, sms = 0;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    uint32_t blocks = uint32_t(sms) * uint32_t(per_sm);
    const uint32_t warps_needed = (w.total_groups + 0u);
    const uint32_t max_blocks = (warps_needed + w.block_threads / 32u - 1u) / (w.block_threads / 32u);
    if (blocks > max_blocks) blocks = std::max(1u, max_blocks);
    fn<<<blocks, w.block_threads, w.smem_bytes, stream>>>(w.jobs, w.num_jobs, w.total_groups, w.layout,
                                                        w.work_counter, w.counters, w.status);
    return cudaGetLastError();
}

template <int kTracking, int kPhase>
cudaError_t launch_staged(const WaveLaunch& w, cudaStream_t stream) {
    return w.staged ? launch_one<kTracking, kPhase, true>(w, stream) : launch_one<kTracking, kPhase, false>(w, stream);
}

}  // namespace

cudaError_t launch_trace_wavefront(const WaveLaunch& w, cudaStream_t stream) {
#define SKY_WAVE_CASE(TR, PH) \
    if (w.tracking == TR && w.phase_sampling == PH) return launch_staged<TR, PH>(w, stream);
    SKY_WAVE_CASE(SKY_TRACKING_SEGMENT_RESTART, SKY_PHASE_ISOTROPIC)
    SKY_WAVE_CASE(SKY_TRACKING_SEGMENT_RESTART, SKY_PHASE_TABULATED)
    SKY_WAVE_CASE(SKY_TRACKING_RESIDUAL_CARRY, SKY_PHASE_ISOTROPIC)
    SKY_WAVE_CASE(SKY_TRACKING_RESIDUAL_CARRY, SKY_PHASE_TABULATED)
    SKY_WAVE_CASE(SKY_TRACKING_MERGED_LAYERS, SKY_PHASE_ISOTROPIC)
    SKY_WAVE_CASE(SKY_TRACKING_MERGED_LAYERS, SKY_PHASE_TABULATED)
#undef SKY_WAVE_CASE
    return cudaErrorInvalidValue;
}

// Shared-memory layout for the tables of `S` (staged when they fit).
StageLayout plan_stage_layout(const DevScene& S, uint32_t warps, uint32_t max_cells, bool with_majorants,
                              bool stage_tables) {
    StageLayout l{};
    size_t off = 0;
    auto take = [&off](size_t bytes) {
        size_t at = off;
        off = (off + bytes + 15) / 16 * 16;
        return uint32_t(at);
    };
    l.jobs = take(size_t(warps) * sizeof(DevJob));
    l.max_cells = max_cells;
    l.acc = take(size_t(warps) * 2u * max_cells * sizeof(double));
    if (stage_tables) {
        l.knot_z_bytes = S.knot_count * 4u;
        l.finder_bytes = kFinderCells * 2u;
        l.sigma_t_bytes = S.band_count * S.knot_count * 8u;
        l.bands_bytes = S.band_count * uint32_t(sizeof(DevBand));
        l.trk_bytes = S.trk_total * 4u;
        l.trk_map_bytes = (S.band_count * S.layer_count * 2u + 3u) / 4u * 4u;
        l.trk_count_bytes = S.band_count * 4u;
        l.majorants_bytes = with_majorants ? S.band_count * S.layer_count * 4u : 0u;
        l.knot_z = take(l.knot_z_bytes);
        l.finder = take(l.finder_bytes);
        l.sigma_t = take(l.sigma_t_bytes);
        l.bands = take(l.bands_bytes);
        l.trk_radius = take(l.trk_bytes);
        l.trk_maj = take(l.trk_bytes);
        l.trk_map = take(l.trk_map_bytes);
        l.trk_count = take(l.trk_count_bytes);
        l.trk_off = take(l.trk_count_bytes);
        l.majorants = take(l.majorants_bytes);
    }
    l.total = uint32_t(off);
    return l;
}

}  // namespace sky
