// trace_wave.cuh — the wavefront tracing kernel (a ray loop with per-lane
// chain regeneration over a job table) and its launch shapes, included by one
// translation unit per tracking mode (trace_wave_*.cu) so that its
// instantiations compile in parallel.  trace_wave.cu holds the launch
// sequence (prepare, trace, finalize).
//
// The plain kernel runs every chain to completion inside one lane, so a warp
// executes the union of 32 different paths.  Here a chain is a sequence of
// rays: the camera / continuation ray of each vertex and the sun shadow ray
// of each NEE sample.  Every iteration of the kernel's loop traces exactly
// one ray per lane through the one inlined tracker (sample_real_collision /
// delta_transmittance, sky_trace.wgsl:405-475); the event code (scattering,
// NEE, ground, Russian roulette, sky_trace.wgsl:566-776) then runs up to the
// lane's next ray.  A lane whose chain ends takes the next sample of its
// warp's current (pixel, band) cell, and the warp takes a new cell from a
// global counter when the cell's samples run out.  So the 32 lanes enter the
// tracker together on every iteration whatever vertex or chain each is at,
// no lane waits for the slowest chain of a cell, and nothing waits at a block
// barrier.
//
// Each chain consumes its random stream in the plain kernel's order
// (trace_path, sky_trace.wgsl:703-776), so both kernels trace the same paths.
// A lane keeps the FP64 sums of its current cell in registers and adds them
// to the job's cell sums when it moves to another cell; the cells' sums
// therefore add in no fixed order (they agree with the plain kernel's to FP64
// rounding).
//
// A launch is three kernels: prepare (zero the sums of jobs that do not
// accumulate, reset the work counter), trace, and finalize (mean film, XYZ
// and its variance, linear sRGB of every pixel of every job).

#pragma once

#include <algorithm>

#include "sky_device.cuh"
#include "trace_kernels.h"

namespace sky {
namespace wave {


constexpr uint32_t kFull = 0xffffffffu;
constexpr uint32_t kNoCell = 0xffffffffu;
// Default backstop on the loop iterations of one warp (one ray per lane
// each; SkyTuning.iteration_limit overrides it); a render needs ~3 rays per
// chain / lanes in flight.  Beyond it the warp sets status bit 2 and returns.
constexpr uint32_t kMaxIterations = 1u << 31;

// What a lane does next.
enum : uint32_t {
    kTrace = 0u,    // a ray is set up: trace it in the next tracking step
    kStart = 1u,    // a new chain: camera ray
    kPrimary = 2u,  // depth checks and the boundary of the vertex's outgoing ray
    kLights = 3u,   // the vertex's next NEE sample, else its continuation
    kEnd = 4u,      // the chain's radiance is final
    kIdle = 5u      // no chain
};

// Job of global cell `g`: the last job whose first cell is <= g.
__device__ __forceinline__ uint32_t job_of(const DevJob* __restrict__ jobs, uint32_t num_jobs, uint32_t g) {
    uint32_t lo = 0u, hi = num_jobs;
    while (hi - lo > 1u) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&jobs[mid].cell_begin) <= g) lo = mid;
        else hi = mid;
    }
    return lo;
}

// The launch constants and the sun frame of a lane's job: kernel parameters
// when the launch holds one job, the job table otherwise.
template <bool kSingle>
__device__ __forceinline__ const DevLaunch& job_launch(const DevLaunch& L0, const DevJob* jobs, uint32_t job) {
    if constexpr (kSingle) return L0;
    else return jobs[job].L;
}
template <bool kSingle>
__device__ __forceinline__ const DevScene& job_scene(const DevScene& S0, const DevJob* jobs, uint32_t job) {
    if constexpr (kSingle) return S0;
    else return jobs[job].S;
}

// Bytes of shared memory that stage_medium() fills: the band-independent knot
// profile (48 B per knot), the per-band constants (32 B per band) and aerosol
// optics (32 B per band), the union knots and the knot finder.
__host__ __device__ inline size_t staged_medium_bytes(uint32_t knots, uint32_t bands) {
    return size_t(knots) * sizeof(DevProfileKnot) + size_t(bands) * sizeof(DevBand) +
           size_t(bands) * kSpecies * sizeof(SkyAerosolOptics) + size_t(knots) * sizeof(float) +
           size_t(kFinderCells) * sizeof(uint16_t);
}

// Copy the medium tables every collision and NEE evaluation reads into the
// block's shared memory (once per block, before the loop), and return the
// view of them.  The per-band extinction rows and the phase tables stay in
// global memory, read through the L1 cache.
__device__ __forceinline__ Medium stage_medium(const DevScene& S, unsigned char* smem) {
    DevProfileKnot* profile = reinterpret_cast<DevProfileKnot*>(smem);
    DevBand* bands = reinterpret_cast<DevBand*>(profile + S.knot_count);
    SkyAerosolOptics* optics = reinterpret_cast<SkyAerosolOptics*>(bands + S.band_count);
    float* knot_z = reinterpret_cast<float*>(optics + S.band_count * kSpecies);
    uint16_t* finder = reinterpret_cast<uint16_t*>(knot_z + S.knot_count);
    // 4-byte words throughout (every table is a multiple of 4 bytes; the finder's 512 halves are 256 words)
    auto copy = [](void* dst, const void* src, size_t bytes) {
        uint32_t* d = static_cast<uint32_t*>(dst);
        const uint32_t* s = static_cast<const uint32_t*>(src);
        for (size_t i = threadIdx.x; i < bytes / 4u; i += blockDim.x) d[i] = __ldg(s + i);
    };
    copy(profile, S.profile, size_t(S.knot_count) * sizeof(DevProfileKnot));
    copy(bands, S.bands, size_t(S.band_count) * sizeof(DevBand));
    copy(optics, S.optics, size_t(S.band_count) * kSpecies * sizeof(SkyAerosolOptics));
    copy(knot_z, S.knot_z, size_t(S.knot_count) * sizeof(float));
    copy(finder, S.finder, size_t(kFinderCells) * sizeof(uint16_t));
    __syncthreads();
    return Medium{knot_z, finder, profile, bands, optics};
}

// The medium coefficients at each lane's current scattering vertex, kept in
// shared memory (one word per thread per value, thread-minor) from the real
// collision that made the vertex to its NEE terms and its continuation, so
// that a vertex evaluates coefficients_at() once instead of three times
// (-1.6 % on the production render): the Rayleigh coefficient, the kAer
// species' scattering coefficients and the total scattering coefficient.
template <int kAer>
struct VertexCoeffCache {
    float* at;  // this thread's first word
    __device__ __forceinline__ void store(const Coeffs& c) const {
        at[0] = c.rayleigh;
#pragma unroll
        for (int i = 0; i < kAer; ++i) at[(1 + i) * kWaveThreads] = c.sca[i];
        at[(1 + kAer) * kWaveThreads] = c.scattering;
    }
    // What the NEE term and the continuation read: rayleigh, sca[] and
    // scattering (the species beyond kAer are 0; absorption is not kept).
    __device__ __forceinline__ Coeffs load() const {
        Coeffs c;
        c.rayleigh = at[0];
#pragma unroll
        for (int i = 0; i < int(kSpecies); ++i) c.sca[i] = i < kAer ? at[(1 + i) * kWaveThreads] : 0.0f;
        c.scattering = at[(1 + kAer) * kWaveThreads];
        c.abs_total = 0.0f;
        c.extinction = c.scattering;
        return c;
    }
};

// Byte offset of the vertex cache in the dynamic shared memory (after the
// staged medium tables) and the block's total dynamic shared memory.
__host__ __device__ inline size_t vertex_cache_offset(uint32_t knots, uint32_t bands) {
    return (staged_medium_bytes(knots, bands) + 15u) & ~size_t(15u);
}
__host__ __device__ inline size_t wave_smem_bytes(uint32_t knots, uint32_t bands, uint32_t aerosol_species) {
    return vertex_cache_offset(knots, bands) + size_t(2u + aerosol_species) * kWaveThreads * sizeof(float);
}

// kCount: count events (SkyDeviceOutputs.counters given).  Without it the
// counters are never read, so their increments compile away (the registers
// they would hold are worth ~5 % at 64 registers per lane).
// kAer: aerosol species evaluated by the medium functions (1 or kSpecies,
// coefficients_at()).
template <int kTracking, int kPhase, int kMinBlocks, bool kSingle, bool kCount, int kAer>
__global__ void __launch_bounds__(kWaveThreads, kMinBlocks)
    wave_kernel(const __grid_constant__ DevScene S, const __grid_constant__ DevLaunch L0,
                const DevJob* __restrict__ jobs, uint32_t num_jobs,
                uint32_t total_cells, uint32_t* __restrict__ work_counter, unsigned long long* __restrict__ counters,
                uint32_t* __restrict__ status, uint32_t iteration_limit) {
    extern __shared__ __align__(16) unsigned char medium_smem[];
    const Medium M = stage_medium(S, medium_smem);
    const VertexCoeffCache<kAer> vc{
        reinterpret_cast<float*>(medium_smem + vertex_cache_offset(S.knot_count, S.band_count)) + threadIdx.x};
    const uint32_t lane = threadIdx.x & 31u;
    Counters n;
    n.clear();
    bool watchdog = false;
    // the warp's current cell and its next unclaimed sample (warp-uniform)
    uint32_t claim_job = 0u, claim_spp = 0u, claim_next = 0u;
    uint32_t claim_band = 0u, claim_x = 0u, claim_y = 0u;  // the cell's band and pixel, divided out once per cell
    bool exhausted = false;
    // the lane's chain
    uint32_t next = kIdle, job = 0u, sample = 0u, band = 0u, px = 0u, py = 0u, depth = 0u, ls = 0u, boundary = 0u;
    bool shadow_ray = false, ground = false;
    Rng rng;
    rng.k0 = rng.k1 = rng.k2 = rng.dim = 0u;
    V3 org = mk(0.0f, 0.0f, 0.0f), dir = org;  // org is the vertex position between rays
    // nee_mu: the pending shadow ray's cosine (to the incoming direction at a
    // medium vertex, to the normal on the ground); its NEE term is evaluated
    // after the trace, and only when the ray reaches the sun
    float thr = 0.0f, rad = 0.0f, nee = 0.0f, alt = 0.0f, nee_mu = 0.0f, t_max = 0.0f;
    RayGeo g{0.0f, 0.0f, 0.0f};
    // FP64 sums of the lane's current cell
    uint32_t acc_job = 0u, acc_cell = kNoCell;
    double acc_sum = 0.0, acc_sq = 0.0;

    for (uint32_t iter = 0u;; ++iter) {
        if (iter >= iteration_limit) {  // warp-uniform
            if (lane == 0u) atomicOr(status, 2u);
            break;
        }
        // a chain that ended after its last ray: its radiance joins the cell's sums
        if (next == kEnd) {
            const double rd = double(rad);
            acc_sum += rd;
            acc_sq += rd * rd;
            next = kIdle;
        }
        // idle lanes take the next samples of the warp's cell
#pragma unroll 1
        for (;;) {
            const uint32_t need = __ballot_sync(kFull, next == kIdle);
            if (need == 0u || exhausted) break;
            if (claim_next >= claim_spp) {
                uint32_t gc = 0u;
                if (lane == 0u) gc = atomicAdd(work_counter, 1u);
                gc = __shfl_sync(kFull, gc, 0);
                if (gc >= total_cells) {
                    exhausted = true;
                    break;
                }
                claim_job = job_of(jobs, num_jobs, gc);
                const uint32_t c = gc - __ldg(&jobs[claim_job].cell_begin);
                // claims run band-major (all pixels of a band, then the next band), so the
                // warps of an SM work on one or two bands at a time and that band's
                // extinction row, merged grid and phase rows stay in L1 (-0.9 % on the
                // production render, -4 % on a 128x64 one); the sums keep their
                // pixel-major, band-minor layout
                const uint32_t width = __ldg(&jobs[claim_job].L.width);
                const uint32_t npix = width * __ldg(&jobs[claim_job].L.rows);
                claim_band = c / npix;
                const uint32_t pixel = c - claim_band * npix;
                const uint32_t row = pixel / width;  // row within the job's slab
                claim_x = pixel - row * width;
                claim_y = row + __ldg(&jobs[claim_job].L.row_begin);
                claim_spp = __ldg(&jobs[claim_job].L.spp);
                claim_next = 0u;
            }
            const uint32_t rank = __popc(need & ((1u << lane) - 1u));
            if (next == kIdle && claim_next + rank < claim_spp) {
                job = claim_job;
                band = claim_band;
                px = claim_x;
                py = claim_y;
                sample = claim_next + rank;
                next = kStart;
            }
            claim_next = min(claim_spp, claim_next + uint32_t(__popc(need)));
        }
        // event code up to the lane's next ray, one pass in flow order (start,
        // lights / continuation, outgoing ray), so that each block runs once
        // per iteration for every lane that needs it
        if (next != kIdle && next != kTrace) {
            const DevLaunch& JL = job_launch<kSingle>(L0, jobs, job);
            if (next == kStart) {
                // the image pixel drives the random stream, the slab pixel indexes the sums
                const uint32_t pixel = py * JL.width + px;
                const uint32_t cell = ((py - JL.row_begin) * JL.width + px) * S.band_count + band;
                if (cell != acc_cell || job != acc_job) {
                    if (acc_cell != kNoCell) {
                        const DevJob& A = jobs[acc_job];
                        atomicAdd(A.cell_sum + acc_cell, acc_sum);
                        double* sq = A.cell_sumsq;
                        if (sq) atomicAdd(sq + acc_cell, acc_sq);
                    }
                    acc_job = job;
                    acc_cell = cell;
                    acc_sum = acc_sq = 0.0;
                }
                rng.init(pixel, JL.sample_offset + sample, band, JL.seed_lo, JL.seed_hi);
                dir = camera_dir(JL, px, py, rng);
                org = mk(0.0f, S.ground_radius + fmaxf(JL.observer_altitude, 0.0f), 0.0f);
                ++n.e[SKY_EVENT_CHAIN];
                thr = 1.0f;
                rad = 0.0f;
                depth = 0u;
                next = kPrimary;
            }
            if (next == kLights) {
                // direct_sun_at_scatter (sky_trace.wgsl:566-585) and ground_radiance
                // (:587-608), one shadow ray at a time
                const uint32_t lights = JL.direct_light_samples;
                while (ls < lights) {
                    ++ls;
                    const V3 ldir = sample_sun_cone(job_scene<kSingle>(S, jobs, job), rng);
                    ++n.e[SKY_EVENT_NEE];
                    float cos_sun = 0.0f;
                    if (ground) {
                        cos_sun = fmaxf(dot3(normalize_or_y(org), ldir), 0.0f);
                        if (!(cos_sun > 0.0f)) continue;
                    }
                    g = ray_geo(madd(org, ldir, kRayEpsilonKm), ldir);
                    uint32_t kind;
                    ++n.e[SKY_EVENT_BOUNDARY];
                    if (!(next_boundary(S, g, t_max, kind) && kind == 1u)) continue;
                    nee_mu = ground ? cos_sun : dot3(dir, ldir);
                    shadow_ray = true;
                    next = kTrace;
                    break;
                }
                if (next == kLights) {
                    // the continuation (sky_trace.wgsl:728-767): each branch draws its
                    // angles, then one shared frame step turns them into the direction
                    // (orthonormal_basis + direction_from_frame, as direction_from_axis_mu
                    // and sample_cosine_hemisphere compute it), so that medium and ground
                    // lanes run that step together
                    rad += thr * (nee * (1.0f / float(lights)));
                    V3 nd = mk(0.0f, 1.0f, 0.0f), axis = dir;
                    float cos_t = 1.0f, sin_t = 0.0f, xi_phi = 0.0f, weight = 1.0f;
                    bool framed = true;
                    if (!ground) {
                        const Coeffs c = vc.load();
                        if (kPhase == SKY_PHASE_TABULATED) {
                            float mu;
                            weight = tabulated_mu<kAer>(S, c, band, rng, mu, xi_phi);
                            cos_t = fminf(fmaxf(mu, -1.0f), 1.0f);
                            sin_t = sqrtf(fmaxf(1.0f - cos_t * cos_t, 0.0f));
                        } else {
                            nd = sample_isotropic(rng);
                            weight = mixed_phase<kAer>(S, c, band, dot3(dir, nd)) / kIsotropicPdf;
                            framed = false;
                        }
                    } else {
                        axis = normalize_or_y(org);  // the ground normal
                        const float u = rng.next();
                        sin_t = sqrtf(u);
                        xi_phi = rng.next();
                        cos_t = sqrtf(fmaxf(1.0f - u, 0.0f));
                    }
                    V3 n = axis;
                    if (framed) {
                        V3 t, bt;
                        orthonormal_basis(axis, t, bt);
                        n = normalize_or_y(axis);
                        nd = direction_from_frame(n, t, bt, cos_t, sin_t, xi_phi);
                    }
                    bool alive = true;
                    if (ground) {
                        const float pdf = fmaxf(dot3(n, nd), 0.0f) * kInvPi;
                        const float cos_out = fmaxf(dot3(axis, nd), 0.0f);
                        if (pdf <= 0.0f || cos_out <= 0.0f) alive = false;
                        else thr *= S.ground_albedo * kInvPi * cos_out / pdf;
                    } else {
                        thr *= weight;
                    }
                    if (alive && depth >= JL.rr_start_depth) {  // russian_roulette (:691-701)
                        const float q = fminf(fmaxf(thr, 0.05f), 0.95f);
                        if (rng.next() > q) alive = false;
                        else thr = thr / q;
                    }
                    if (!alive) {
                        rad = fmaxf(rad, 0.0f);
                        next = kEnd;
                    } else {
                        org = madd(org, nd, kRayEpsilonKm);
                        dir = nd;
                        if (rad < 0.0f || rad != rad || thr < 0.0f || thr != thr) {
                            rad = 0.0f;
                            next = kEnd;
                        } else {
                            ++depth;
                            next = kPrimary;
                        }
                    }
                }
            }
            if (next == kPrimary) {  // the outgoing ray (sky_trace.wgsl:709-717)
                const uint32_t max_orders = JL.max_orders;
                if (depth >= JL.watchdog_limit) {
                    watchdog = true;
                    next = kEnd;
                } else {
                    g = ray_geo(org, dir);
                    ++n.e[SKY_EVENT_BOUNDARY];
                    if ((max_orders != 0u && depth >= max_orders) || !next_boundary(S, g, t_max, boundary)) {
                        rad = fmaxf(rad, 0.0f);
                        next = kEnd;
                    } else {
                        shadow_ray = false;
                        next = kTrace;
                    }
                }
            }
        }
        const bool tracing = next == kTrace;
        if (!__any_sync(kFull, tracing)) {
            // no cell left and every lane idle (a lane ending its chain is summed next
            // iteration)
            if (exhausted && __all_sync(kFull, next == kIdle)) break;
            continue;
        }
        if (tracing) {
            float t_hit = 0.0f;
            const bool hit = track_ray<kTracking>(S, M, g, t_max, band, rng, t_hit, n, watchdog, shadow_ray);
            // the medium coefficients at a real collision (albedo; kept for the new
            // vertex's NEE terms and continuation) and at the vertex of an unblocked
            // shadow ray (phase of its NEE term, from the vertex cache)
            const bool lit = shadow_ray && !hit;
            Coeffs c;
            if (!shadow_ray && hit) {
                org = madd(org, dir, t_hit);
                alt = altitude_at(g, t_hit, S.ground_radius);
                c = coefficients_at<kAer>(S, M, band, alt);
                vc.store(c);
            } else if (lit && !ground) {
                c = vc.load();
            }
            if (shadow_ray) {
                if (lit) {  // the sample's term, transmittance 1 (sky_trace.wgsl:566-608)
                    const float l_sun = M.bands[band].solar_radiance;
                    nee += ground ? S.ground_albedo * kInvPi * l_sun * 1.0f * nee_mu / S.light_pdf
                                  : l_sun * 1.0f * mixed_phase<kAer>(S, c, band, nee_mu) / S.light_pdf;
                }
                next = kLights;
            } else if (hit) {
                ++n.e[SKY_EVENT_SCATTER];
                const bool medium = c.extinction > 0.0f && c.scattering > 0.0f;
                if (medium) thr *= fminf(fmaxf(c.scattering / c.extinction, 0.0f), 1.0f);
                if (!medium || thr <= 0.0f) {
                    rad = fmaxf(rad, 0.0f);
                    next = kEnd;
                } else {
                    ground = false;
                    ls = 0u;
                    nee = 0.0f;
                    next = kLights;
                }
            } else if (boundary == 1u) {
                if (depth == 0u && dot3(dir, load3(job_scene<kSingle>(S, jobs, job).sun)) >= S.cos_max)
                    rad += thr * M.bands[band].solar_radiance;
                rad = fmaxf(rad, 0.0f);
                next = kEnd;
            } else {
                ++n.e[SKY_EVENT_GROUND];
                org = madd(org, dir, t_max);
                ground = true;
                ls = 0u;
                nee = 0.0f;
                next = kLights;
            }
        }
    }
    if (acc_cell != kNoCell) {
        const DevJob& A = jobs[acc_job];
        atomicAdd(A.cell_sum + acc_cell, acc_sum);
        double* sq = A.cell_sumsq;
        if (sq) atomicAdd(sq + acc_cell, acc_sq);
    }
    if (kCount) {
#pragma unroll
        for (int e = 0; e < SKY_EVENT_COUNT; ++e) {
            uint32_t v = n.e[e];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
            if (lane == 0u && v) atomicAdd(counters + e, (unsigned long long)v);
        }
    }
    if (__any_sync(kFull, watchdog) && lane == 0u) atomicOr(status, 1u);
}

template <int kTracking, int kPhase, int kMinBlocks, bool kSingle, bool kCount, int kAer>
cudaError_t launch_wave_shape(const WaveLaunch& w, cudaStream_t stream) {
    const void* k =
        reinterpret_cast<const void*>(wave_kernel<kTracking, kPhase, kMinBlocks, kSingle, kCount, kAer>);
    int dev = 0, sms = 0, per_sm = 0;
    cudaError_t e;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    // the staged medium tables and the vertex cache: 12.7 KB for 81 bands over 68 knots and one
    // aerosol species; the largest scenes the library accepts (1024 knots, 256 bands) need 77 KB,
    // beyond the 48 KB a launch gets without opting in
    const size_t smem = wave_smem_bytes(w.scene.knot_count, w.scene.band_count, uint32_t(kAer));
    if (smem > 48u * 1024u &&
        (e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem))) != cudaSuccess)
        return e;
    // Prefer the smallest shared-memory carveout that holds kMinBlocks blocks' tables: the
    // rest of the SM's L1/shared array caches the phase tables, extinction rows and merged
    // grid (the largest carveout costs 6 % on the production render).  A hint: if the
    // driver refuses it, the launch goes ahead with its own choice.
    int smem_sm = 0, reserved = 0;
    if (cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev) == cudaSuccess &&
        smem_sm > 0) {
        const size_t need = size_t(kMinBlocks) * (smem + size_t(reserved));
        const int pct = int(std::min<size_t>(100u, (need * 100u + size_t(smem_sm) - 1u) / size_t(smem_sm)));
        if (cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, std::max(pct, 1)) != cudaSuccess)
            (void)cudaGetLastError();  // clear the refused hint so the launch check does not see it
    } else {
        (void)cudaGetLastError();
    }
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kWaveThreads, smem)) != cudaSuccess) return e;
    per_sm = std::max(per_sm, 1);
    if (w.max_blocks_per_sm) per_sm = std::min(per_sm, int(w.max_blocks_per_sm));
    // a warp per cell at most
    const uint64_t want = (uint64_t(w.total_cells) * 32u + kWaveThreads - 1u) / kWaveThreads;
    const uint32_t blocks = uint32_t(std::max<uint64_t>(1u, std::min<uint64_t>(uint64_t(per_sm) * sms, want)));
    wave_kernel<kTracking, kPhase, kMinBlocks, kSingle, kCount, kAer><<<blocks, kWaveThreads, smem, stream>>>(
        w.scene, w.launch0, w.jobs, w.num_jobs, w.total_cells, w.work_counter, w.counters, w.status,
        w.iteration_limit ? w.iteration_limit : kMaxIterations);
    return cudaGetLastError();
}

template <int kTracking, int kPhase, bool kSingle, bool kCount, int kAer>
cudaError_t launch_wave_variant(const WaveLaunch& w, cudaStream_t stream) {
    switch (w.variant) {
        case 0: return launch_wave_shape<kTracking, kPhase, 3, kSingle, kCount, kAer>(w, stream);
        case 1: return launch_wave_shape<kTracking, kPhase, 2, kSingle, kCount, kAer>(w, stream);
        case 2: return launch_wave_shape<kTracking, kPhase, 4, kSingle, kCount, kAer>(w, stream);
        default: return cudaErrorInvalidValue;
    }
}

template <int kTracking, int kPhase, int kAer>
cudaError_t launch_wave_species(const WaveLaunch& w, cudaStream_t stream) {
    if (w.num_jobs == 1u)
        return w.counters ? launch_wave_variant<kTracking, kPhase, true, true, kAer>(w, stream)
                          : launch_wave_variant<kTracking, kPhase, true, false, kAer>(w, stream);
    return w.counters ? launch_wave_variant<kTracking, kPhase, false, true, kAer>(w, stream)
                      : launch_wave_variant<kTracking, kPhase, false, false, kAer>(w, stream);
}

template <int kTracking, int kPhase>
cudaError_t launch_wave_mode(const WaveLaunch& w, cudaStream_t stream) {
    if (w.aerosol_species == 1u) return launch_wave_species<kTracking, kPhase, 1>(w, stream);
    if (w.aerosol_species == kSpecies) return launch_wave_species<kTracking, kPhase, int(kSpecies)>(w, stream);
    return cudaErrorInvalidValue;
}

// The kernels of one tracking mode, both phase samplings.
template <int kTracking>
cudaError_t launch_wave_tracking(const WaveLaunch& w, cudaStream_t stream) {
    if (w.phase_sampling == SKY_PHASE_TABULATED) return launch_wave_mode<kTracking, SKY_PHASE_TABULATED>(w, stream);
    if (w.phase_sampling == SKY_PHASE_ISOTROPIC) return launch_wave_mode<kTracking, SKY_PHASE_ISOTROPIC>(w, stream);
    return cudaErrorInvalidValue;
}

}  // namespace wave
}  // namespace sky
