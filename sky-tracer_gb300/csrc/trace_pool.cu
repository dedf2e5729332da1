// trace_pool.cu — persistent wavefront tracer: a pool of paths per block,
// regrouped by the work they need next.
//
// The plain kernel runs every chain to completion inside one lane, so the
// warp executes the union of 32 different paths (profiled: ~5 of 32 lanes
// active per instruction).  Here each block keeps kPoolSlots paths in shared
// memory (structure of arrays) and advances all of them in lock-step phases:
//
//   generate  free slots take the next chains of the block's work groups and
//             build camera rays (sky_trace.wgsl:795-807);
//   trace     every ray that needs delta tracking (camera/continuation rays
//             and sun shadow rays alike) is put on one compacted list, and
//             lanes drain the list with per-lane refill, so the tracking loop
//             (sky_trace.wgsl:405-475) runs with nearly full warps;
//   shade     finished rays are split into three lists — shadow results,
//             real collisions, ground/escape — and each list is processed by
//             all threads: NEE accumulation, scattering, phase sampling,
//             Russian roulette and the next ray (sky_trace.wgsl:566-776).
//
// Each chain's random stream is consumed in exactly the order of the plain
// kernel (and of the reference shader), so both kernels trace the same paths.
//
// Work groups: `pixels_per_group` pixels x all bands x all samples of one
// job, taken from a global counter; up to kRing groups are in flight per
// block, each with FP64 per-cell sums in shared memory.  When a group's last
// chain finishes the block writes its cell sums, mean film and per-pixel CIE
// XYZ with its variance (warp-shuffle reductions over the bands).

#include <algorithm>

#include "sky_device.cuh"
#include "trace_kernels.h"

namespace sky {
namespace {

constexpr uint32_t kFull = 0xffffffffu;
constexpr uint32_t kThreads = kPoolThreads;
constexpr uint32_t kWarps = kThreads / 32u;
constexpr uint32_t kMaxSlots = kPoolThreads * kPoolMaxSlotsPerThread;
constexpr uint32_t kRing = kPoolRing;
constexpr uint32_t kMaxCells = kPoolMaxCells;
// Upper bound on the phase iterations of one block in one launch (a block
// needs ~3 per chain / kSlots); exceeding it sets status bit 2 and the block
// returns instead of running on.
constexpr uint32_t kMaxIterations = 1u << 24;

// slot meta word
constexpr uint32_t M_STATE = 0x3u;  // 0 free, 1 needs tracking, 2 tracked
constexpr uint32_t S_FREE = 0u, S_TRACE = 1u, S_TRACED = 2u;
constexpr uint32_t M_HIT = 1u << 2;
constexpr uint32_t M_SHADOW = 1u << 3;
constexpr uint32_t M_GROUND = 1u << 4;
constexpr uint32_t M_EXIT = 1u << 5;
constexpr uint32_t M_LIGHT_SHIFT = 8u;
constexpr uint32_t M_DEPTH_SHIFT = 16u;

// Slot fields (one u32 word each, structure of arrays).  O holds the origin
// of the camera/continuation ray or, after an event, the event position; T
// holds the distance to the boundary while a ray waits for tracking and the
// collision distance after it.
enum SlotField : uint32_t {
    F_CELL, F_K0, F_K1, F_K2, F_DIM, F_META,
    F_OX, F_OY, F_OZ, F_DX, F_DY, F_DZ, F_LX, F_LY, F_LZ,
    F_THR, F_RAD, F_NEE, F_ALT, F_T, F_COUNT
};

struct RingEntry {
    unsigned long long pixel0;
    uint32_t job, total, issued, done, cells, npix, active, _pad;
};

struct PoolHeader {
    RingEntry ring[kRing];
    uint32_t order[kRing];  // active ring entries, oldest first
    uint32_t ring_count, no_more_work, fetch, _pad;
    uint32_t list_count[5];
    uint32_t warp_totals[kWarps];
};

template <uint32_t kSlots>
struct PoolSmem {
    static constexpr uint32_t slots_n = kSlots;
    PoolHeader* hdr;
    DevJob* jobs;       // [kRing] job constants of the ring entries
    double* acc;        // [kRing][kMaxCells][2]
    uint32_t* slots;    // [F_COUNT][kSlots]
    uint16_t* lists;    // [5][kSlots]: 0 trace, 1-3 shade, 4 free
    __device__ __forceinline__ uint32_t& u(uint32_t f, uint32_t s) const { return slots[f * kSlots + s]; }
    __device__ __forceinline__ float& f(uint32_t fld, uint32_t s) const {
        return reinterpret_cast<float*>(slots)[fld * kSlots + s];
    }
};

// F_CELL packs the cell within the work group (9 bits), the band (8 bits) and
// the ring entry (3 bits), so the hot phases need no integer division.
__device__ __forceinline__ uint32_t pack_cell(uint32_t cell, uint32_t band, uint32_t ring) {
    return cell | (band << 9) | (ring << 17);
}
__device__ __forceinline__ uint32_t cell_of(uint32_t c) { return c & 0x1ffu; }
__device__ __forceinline__ uint32_t band_of(uint32_t c) { return (c >> 9) & 0xffu; }
__device__ __forceinline__ uint32_t ring_of(uint32_t c) { return c >> 17; }

// Registers of one path while a thread shades it.
struct Path {
    uint32_t slot, cell, band, ring, meta;
    Rng rng;
    V3 o, dir, ldir;
    float thr, rad, nee, alt, t;
};

template <class PS>
__device__ __forceinline__ void load_path(const PS& P, uint32_t s, Path& p) {
    p.slot = s;
    const uint32_t c = P.u(F_CELL, s);
    p.cell = cell_of(c);
    p.band = band_of(c);
    p.ring = ring_of(c);
    p.rng.k0 = P.u(F_K0, s);
    p.rng.k1 = P.u(F_K1, s);
    p.rng.k2 = P.u(F_K2, s);
    p.rng.dim = P.u(F_DIM, s);
    p.meta = P.u(F_META, s);
    p.o = mk(P.f(F_OX, s), P.f(F_OY, s), P.f(F_OZ, s));
    p.dir = mk(P.f(F_DX, s), P.f(F_DY, s), P.f(F_DZ, s));
    p.ldir = mk(P.f(F_LX, s), P.f(F_LY, s), P.f(F_LZ, s));
    p.thr = P.f(F_THR, s);
    p.rad = P.f(F_RAD, s);
    p.nee = P.f(F_NEE, s);
    p.alt = P.f(F_ALT, s);
    p.t = P.f(F_T, s);
}

template <class PS>
__device__ __forceinline__ void store_path(const PS& P, const Path& p) {
    const uint32_t s = p.slot;
    P.u(F_CELL, s) = pack_cell(p.cell, p.band, p.ring);
    P.u(F_K0, s) = p.rng.k0;
    P.u(F_K1, s) = p.rng.k1;
    P.u(F_K2, s) = p.rng.k2;
    P.u(F_DIM, s) = p.rng.dim;
    P.u(F_META, s) = p.meta;
    P.f(F_OX, s) = p.o.x;
    P.f(F_OY, s) = p.o.y;
    P.f(F_OZ, s) = p.o.z;
    P.f(F_DX, s) = p.dir.x;
    P.f(F_DY, s) = p.dir.y;
    P.f(F_DZ, s) = p.dir.z;
    P.f(F_LX, s) = p.ldir.x;
    P.f(F_LY, s) = p.ldir.y;
    P.f(F_LZ, s) = p.ldir.z;
    P.f(F_THR, s) = p.thr;
    P.f(F_RAD, s) = p.rad;
    P.f(F_NEE, s) = p.nee;
    P.f(F_ALT, s) = p.alt;
    P.f(F_T, s) = p.t;
}

__device__ __forceinline__ uint32_t depth_of(uint32_t meta) { return meta >> M_DEPTH_SHIFT; }
__device__ __forceinline__ uint32_t light_of(uint32_t meta) { return (meta >> M_LIGHT_SHIFT) & 0xffu; }
__device__ __forceinline__ uint32_t with_light(uint32_t meta, uint32_t l) {
    return (meta & ~(0xffu << M_LIGHT_SHIFT)) | (min(l, 255u) << M_LIGHT_SHIFT);
}
__device__ __forceinline__ uint32_t with_state(uint32_t meta, uint32_t st) { return (meta & ~M_STATE) | st; }

// Delta tracking state along one ray (camera/continuation or shadow).
struct Tracker {
    RayGeo g;
    float t, t_max, t_seg, tau, maj;
    int m, mdir;
    uint32_t guard;
    bool need_draw;
};

template <int kTracking>
__device__ __forceinline__ void track_begin(const DevScene& S, uint32_t band, Tracker& k, Rng& rng, Counters& n) {
    k.t = 0.0f;
    k.guard = 0;
    k.need_draw = true;
    k.mdir = 0;
    k.m = 0;
    k.t_seg = 0.0f;
    k.tau = 0.0f;
    k.maj = 1.0f;
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

// One tracking action: 0 continue, 1 real collision at k.t, 2 reached
// k.t_max.  Draw order identical to the plain kernel's track_ray().
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

__device__ __forceinline__ void copy_words(void* dst, const void* src, uint32_t bytes, uint32_t tid, uint32_t n) {
    const uint32_t* s = static_cast<const uint32_t*>(src);
    uint32_t* d = static_cast<uint32_t*>(dst);
    for (uint32_t i = tid; i < bytes / 4u; i += n) d[i] = s[i];
}

// A path ends: its radiance joins its cell's FP64 sums and the slot frees.
template <class PS>
__device__ __forceinline__ void finish(const PS& P, Path& p, float result) {
    const double rd = double(result);
    double* a = P.acc + (size_t(p.ring) * kMaxCells + p.cell) * 2u;
    atomicAdd(a, rd);
    atomicAdd(a + 1, rd * rd);
    atomicAdd(&P.hdr->ring[p.ring].done, 1u);
    p.meta = S_FREE;
}

// Depth checks and the boundary of a new camera/continuation ray
// (sky_trace.wgsl:709-717); leaves the path waiting for tracking or ends it.
template <class PS>
__device__ __forceinline__ void start_ray(const PS& P, const DevScene& S, const DevLaunch& L, Path& p,
                                          Counters& n, bool& watchdog) {
    const uint32_t depth = depth_of(p.meta);
    if (depth >= L.watchdog_limit) {
        watchdog = true;
        finish(P, p, p.rad);
        return;
    }
    if (L.max_orders != 0u && depth >= L.max_orders) {
        finish(P, p, fmaxf(p.rad, 0.0f));
        return;
    }
    const RayGeo g = ray_geo(p.o, p.dir);
    ++n.e[SKY_EVENT_BOUNDARY];
    float tb;
    uint32_t kind;
    if (!next_boundary(S, g, tb, kind)) {
        finish(P, p, fmaxf(p.rad, 0.0f));
        return;
    }
    p.t = tb;
    p.meta = (p.meta & ~(M_STATE | M_SHADOW | M_HIT | M_EXIT)) | S_TRACE | (kind == 1u ? M_EXIT : 0u);
}

// Light samples of the current event (sky_trace.wgsl:566-608) until one needs
// a shadow ray traced; then the continuation (:728-767) and the next ray.
// p.o is the event position here.
template <int kPhase, class PS>
__device__ void lights_and_continue(const PS& P, const DevScene& S, const DevLaunch& L, Path& p, Counters& n,
                                    bool& watchdog) {
    const uint32_t band = p.band;
    const bool ground = (p.meta & M_GROUND) != 0u;
    uint32_t light = light_of(p.meta);
    while (light < L.direct_light_samples) {
        p.ldir = sample_sun_cone(S, p.rng);
        ++n.e[SKY_EVENT_NEE];
        bool go = true;
        if (ground) go = fmaxf(dot3(normalize_or_y(p.o), p.ldir), 0.0f) > 0.0f;
        if (go) {
            const RayGeo g = ray_geo(madd(p.o, p.ldir, kRayEpsilonKm), p.ldir);
            ++n.e[SKY_EVENT_BOUNDARY];
            float tb;
            uint32_t kind;
            if (next_boundary(S, g, tb, kind) && kind == 1u) {
                p.t = tb;
                p.meta = (with_light(p.meta, light) & ~(M_STATE | M_HIT)) | S_TRACE | M_SHADOW;
                return;
            }
        }
        ++light;
    }
    // continuation
    p.rad += p.thr * (p.nee * (1.0f / float(L.direct_light_samples)));
    const uint32_t depth = depth_of(p.meta);
    V3 nd;
    if (!ground) {
        const Coeffs c = coefficients_at(S, S.knot_z, S.finder, band, p.alt);
        if (kPhase == SKY_PHASE_TABULATED) {
            p.thr *= sample_tabulated(S, c, band, p.dir, p.rng, nd);
        } else {
            nd = sample_isotropic(p.rng);
            p.thr *= mixed_phase(S, c, band, dot3(p.dir, nd)) / kIsotropicPdf;
        }
    } else {
        const V3 normal = normalize_or_y(p.o);
        float pdf;
        nd = sample_cosine_hemisphere(normal, p.rng, pdf);
        const float cos_out = fmaxf(dot3(normal, nd), 0.0f);
        if (pdf <= 0.0f || cos_out <= 0.0f) {
            finish(P, p, fmaxf(p.rad, 0.0f));
            return;
        }
        p.thr *= S.ground_albedo * kInvPi * cos_out / pdf;
    }
    if (depth >= L.rr_start_depth) {
        const float q = fminf(fmaxf(p.thr, 0.05f), 0.95f);
        if (p.rng.next() > q) {
            finish(P, p, fmaxf(p.rad, 0.0f));
            return;
        }
        p.thr = p.thr / q;
    }
    p.o = madd(p.o, nd, kRayEpsilonKm);
    p.dir = nd;
    if (p.rad < 0.0f || p.rad != p.rad || p.thr < 0.0f || p.thr != p.thr) {
        finish(P, p, 0.0f);
        return;
    }
    p.meta = (p.meta & 0xffffu & ~(0xffu << M_LIGHT_SHIFT) & ~M_GROUND) | ((depth + 1u) << M_DEPTH_SHIFT);
    start_ray(P, S, L, p, n, watchdog);
}

// Build a compacted list of the slots satisfying pred (any order).
template <class PS, class Pred>
__device__ __forceinline__ void build_list(const PS& P, uint32_t which, Pred pred) {
    constexpr uint32_t kSlots = PS::slots_n;
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t base = 0; base < kSlots; base += kThreads) {
        const uint32_t s = base + threadIdx.x;
        const bool take = pred(s);
        const uint32_t mask = __ballot_sync(kFull, take);
        uint32_t at = 0;
        if (lane == 0 && mask) at = atomicAdd(&P.hdr->list_count[which], __popc(mask));
        at = __shfl_sync(kFull, at, 0);
        if (take) P.lists[which * kSlots + at + __popc(mask & ((1u << lane) - 1u))] = uint16_t(s);
    }
}

// One pass over the slots: tracked rays go to list 1 (shadow results),
// 2 (real collisions) or 3 (ground / escape).
template <class PS>
__device__ __forceinline__ void build_shade_lists(const PS& P) {
    constexpr uint32_t kSlots = PS::slots_n;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lt = (1u << lane) - 1u;
    for (uint32_t base = 0; base < kSlots; base += kThreads) {
        const uint32_t s = base + threadIdx.x;
        const uint32_t m = P.u(F_META, s);
        const bool traced = (m & M_STATE) == S_TRACED;
        const uint32_t cls = !traced ? 0u : ((m & M_SHADOW) ? 1u : ((m & M_HIT) ? 2u : 3u));
#pragma unroll
        for (uint32_t w = 1; w <= 3; ++w) {
            const uint32_t mask = __ballot_sync(kFull, cls == w);
            uint32_t at = 0;
            if (lane == 0 && mask) at = atomicAdd(&P.hdr->list_count[w], __popc(mask));
            at = __shfl_sync(kFull, at, 0);
            if (cls == w) P.lists[w * kSlots + at + __popc(mask & lt)] = uint16_t(s);
        }
    }
}

template <int kTracking, int kPhase, uint32_t kPer, int kMinBlocks>
__global__ void __launch_bounds__(kThreads, kMinBlocks) pool_kernel(const DevJob* __restrict__ jobs, uint32_t num_jobs,
                                                        uint32_t total_groups, PoolLayout lay,
                                                        uint32_t* __restrict__ work_counter,
                                                        unsigned long long* __restrict__ counters,
                                                        uint32_t* __restrict__ status) {
    extern __shared__ __align__(16) unsigned char smem[];
    const uint32_t tid = threadIdx.x;
    const uint32_t lane = tid & 31u;
    const uint32_t warp = tid >> 5;
    constexpr uint32_t kSlots = kPer * kThreads;
    PoolSmem<kSlots> P;
    P.hdr = reinterpret_cast<PoolHeader*>(smem + lay.header);
    P.jobs = reinterpret_cast<DevJob*>(smem + lay.jobs);
    P.acc = reinterpret_cast<double*>(smem + lay.acc);
    P.slots = reinterpret_cast<uint32_t*>(smem + lay.slots);
    P.lists = reinterpret_cast<uint16_t*>(smem + lay.lists);

    if (lay.staged) {
        const DevScene& S0 = jobs[0].S;
        copy_words(smem + lay.knot_z, S0.knot_z, lay.knot_z_bytes, tid, kThreads);
        copy_words(smem + lay.finder, S0.finder, lay.finder_bytes, tid, kThreads);
        copy_words(smem + lay.sigma_t, S0.sigma_t, lay.sigma_t_bytes, tid, kThreads);
        copy_words(smem + lay.bands, S0.bands, lay.bands_bytes, tid, kThreads);
        copy_words(smem + lay.trk_radius, S0.trk_radius, lay.trk_bytes, tid, kThreads);
        copy_words(smem + lay.trk_maj, S0.trk_maj, lay.trk_bytes, tid, kThreads);
        copy_words(smem + lay.trk_map, S0.trk_map, lay.trk_map_bytes, tid, kThreads);
        copy_words(smem + lay.trk_count, S0.trk_count, lay.trk_count_bytes, tid, kThreads);
        copy_words(smem + lay.trk_off, S0.trk_off, lay.trk_count_bytes, tid, kThreads);
        if (lay.majorants_bytes) copy_words(smem + lay.majorants, S0.majorants, lay.majorants_bytes, tid, kThreads);
    }
    for (uint32_t s = tid; s < kSlots; s += kThreads) P.u(F_META, s) = S_FREE;
    if (tid == 0) {
        for (uint32_t r = 0; r < kRing; ++r) P.hdr->ring[r].active = 0;
        P.hdr->ring_count = 0;
        P.hdr->no_more_work = 0;
        for (uint32_t i = 0; i < 5; ++i) P.hdr->list_count[i] = 0;
        P.hdr->fetch = 0;
    }
    __syncthreads();

    Counters n;
    n.clear();
    bool watchdog = false;
    bool stalled = false;
    uint32_t iterations = 0;

    for (;;) {
        // ---- ring maintenance: epilogues of finished groups, then refill ----
        for (uint32_t q = 0; q < kRing; ++q) {
            RingEntry& R = P.hdr->ring[q];
            if (!(R.active && R.done == R.total)) continue;  // block-uniform
            const DevJob& J = P.jobs[q];
            const uint32_t B = J.L.band_count;
            const double n_total = double(J.total_spp);
            const double inv_n = 1.0 / n_total;
            for (uint32_t px = warp; px < R.npix; px += kWarps) {
                double xyz[3] = {0.0, 0.0, 0.0}, var[3] = {0.0, 0.0, 0.0};
                const unsigned long long cell0 = (R.pixel0 + px) * B;
                for (uint32_t b = lane; b < B; b += 32u) {
                    const uint32_t c = px * B + b;
                    double s = P.acc[(size_t(q) * kMaxCells + c) * 2u];
                    double sq = P.acc[(size_t(q) * kMaxCells + c) * 2u + 1u];
                    if (J.accumulate) {
                        s += J.cell_sum[cell0 + b];
                        if (J.cell_sumsq) sq += J.cell_sumsq[cell0 + b];
                    }
                    J.cell_sum[cell0 + b] = s;
                    if (J.cell_sumsq) J.cell_sumsq[cell0 + b] = sq;
                    const double mean = s * inv_n;
                    if (J.film) J.film[cell0 + b] = fmaxf(float(mean), 0.0f);
                    double var_mean = 0.0;
                    if (J.total_spp > 1u) var_mean = fmax((sq - s * mean) / (n_total - 1.0), 0.0) * inv_n;
                    const DevBand& bd = J.S.bands[b];
#pragma unroll
                    for (int ch = 0; ch < 3; ++ch) {
                        const double w = double(bd.xyz[ch]);
                        xyz[ch] += mean * w;
                        var[ch] += var_mean * w * w;
                    }
                }
                if (J.xyz || J.xyz_var || J.rgb) {
#pragma unroll
                    for (int ch = 0; ch < 3; ++ch) {
                        xyz[ch] = warp_sum_d(xyz[ch]);
                        var[ch] = warp_sum_d(var[ch]);
                    }
                    const unsigned long long pix = R.pixel0 + px;
                    if (lane < 3u) {
                        const double vx = lane == 0 ? xyz[0] : (lane == 1 ? xyz[1] : xyz[2]);
                        const double vv = lane == 0 ? var[0] : (lane == 1 ? var[1] : var[2]);
                        if (J.xyz) J.xyz[pix * 3 + lane] = vx;
                        if (J.xyz_var) J.xyz_var[pix * 3 + lane] = vv;
                    }
                    if (J.rgb && lane == 0) store_rgb(rgb_matrix(J.S), xyz, J.rgb + pix * 3);
                }
            }
            __syncthreads();
            if (tid == 0) {
                R.active = 0;
                uint32_t w = 0;
                for (uint32_t i = 0; i < P.hdr->ring_count; ++i)
                    if (P.hdr->order[i] != q) P.hdr->order[w++] = P.hdr->order[i];
                P.hdr->ring_count = w;
            }
            __syncthreads();
        }
        if (warp == 0) {
            // fetch groups until the unissued chains cover the pool or the ring is full
            for (;;) {
                uint32_t pending = 0, count = P.hdr->ring_count;
                for (uint32_t q = 0; q < kRing; ++q) {
                    const RingEntry& R = P.hdr->ring[q];
                    if (R.active) pending += R.total - R.issued;
                }
                if (pending >= kSlots || count >= kRing || P.hdr->no_more_work) break;
                uint32_t group = 0;
                if (lane == 0) group = atomicAdd(work_counter, 1u);
                group = __shfl_sync(kFull, group, 0);
                if (group >= total_groups) {
                    if (lane == 0) P.hdr->no_more_work = 1;
                    __syncwarp();
                    break;
                }
                uint32_t ji = 0;
                while (ji + 1 < num_jobs && jobs[ji + 1].group_begin <= group) ++ji;
                uint32_t q = 0;
                while (P.hdr->ring[q].active) ++q;  // count < kRing: a free entry exists
                copy_words(&P.jobs[q], &jobs[ji], sizeof(DevJob), lane, 32u);
                __syncwarp();
                if (lane == 0) {
                    DevJob& J = P.jobs[q];
                    if (lay.staged) {
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
                    const unsigned long long pixels = (unsigned long long)J.L.width * J.L.height;
                    const unsigned long long pixel0 =
                        (unsigned long long)(group - J.group_begin) * J.pixels_per_group;
                    const uint32_t npix = uint32_t(min((unsigned long long)J.pixels_per_group, pixels - pixel0));
                    RingEntry& R = P.hdr->ring[q];
                    R.pixel0 = pixel0;
                    R.job = ji;
                    R.npix = npix;
                    R.cells = npix * J.L.band_count;
                    R.total = R.cells * J.L.spp;
                    R.issued = 0;
                    R.done = 0;
                    R.active = 1;
                    P.hdr->order[count] = q;
                    P.hdr->ring_count = count + 1u;
                }
                __syncwarp();
                const uint32_t cells = P.hdr->ring[q].cells;
                for (uint32_t c = lane; c < cells * 2u; c += 32u) P.acc[size_t(q) * kMaxCells * 2u + c] = 0.0;
                __syncwarp();
            }
        }
        __syncthreads();
        if (P.hdr->no_more_work && P.hdr->ring_count == 0) break;  // every slot is free here

        // ---- generate: free slots take the next chains, in ring order ----
        build_list(P, 4, [&](uint32_t s) { return (P.u(F_META, s) & M_STATE) == S_FREE; });
        __syncthreads();
        {
            const uint32_t nfree = P.hdr->list_count[4];
            uint32_t e = 0, cum = 0;  // ring cursor, advanced monotonically over the ranks
            for (uint32_t rank = tid; rank < nfree; rank += kThreads) {
                uint32_t q = 0xffffffffu, j = 0;
                while (e < P.hdr->ring_count) {
                    const RingEntry& R = P.hdr->ring[P.hdr->order[e]];
                    const uint32_t rem = R.total - R.issued;
                    if (rank < cum + rem) {
                        q = P.hdr->order[e];
                        j = R.issued + (rank - cum);
                        break;
                    }
                    cum += rem;
                    ++e;
                }
                if (q == 0xffffffffu) break;  // later ranks find no chain either
                const DevJob& J = P.jobs[q];
                const DevScene& S = J.S;
                const DevLaunch& L = J.L;
                const RingEntry& R = P.hdr->ring[q];
                Path p;
                p.slot = P.lists[4 * kSlots + rank];
                p.ring = q;
                const uint32_t sample_local = j / R.cells;
                p.cell = j - sample_local * R.cells;
                const uint32_t pix_local = p.cell / L.band_count;
                p.band = p.cell - pix_local * L.band_count;
                const uint32_t pixel = uint32_t(R.pixel0) + pix_local;
                const uint32_t y = pixel / L.width, x = pixel - y * L.width;
                p.rng.init(pixel, L.sample_offset + sample_local, p.band, L.seed_lo, L.seed_hi);
                p.dir = camera_dir(L, x, y, p.rng);
                p.o = mk(0.0f, S.ground_radius + fmaxf(L.observer_altitude, 0.0f), 0.0f);
                p.thr = 1.0f;
                p.rad = 0.0f;
                p.meta = 0u;
                p.ldir = mk(0.0f, 0.0f, 0.0f);
                p.alt = p.nee = p.t = 0.0f;
                ++n.e[SKY_EVENT_CHAIN];
                start_ray(P, S, L, p, n, watchdog);
                store_path(P, p);
            }
            __syncthreads();
            if (tid == 0) {
                uint32_t left = nfree;
                for (uint32_t i = 0; i < P.hdr->ring_count && left; ++i) {
                    RingEntry& R = P.hdr->ring[P.hdr->order[i]];
                    const uint32_t take = min(left, R.total - R.issued);
                    R.issued += take;
                    left -= take;
                }
                for (uint32_t i = 0; i < 5; ++i) P.hdr->list_count[i] = 0;
                P.hdr->fetch = 0;
            }
            __syncthreads();
        }

        // ---- trace: every ray that needs tracking, lanes refilled from one list ----
        build_list(P, 0, [&](uint32_t s) { return (P.u(F_META, s) & M_STATE) == S_TRACE; });
        __syncthreads();
        {
            const uint32_t total = P.hdr->list_count[0];
            uint32_t slot = 0, band = 0;
            const DevScene* S = nullptr;
            Tracker k;
            Rng rng;
            bool have = false, exhausted = false, shadow = false;
            for (;;) {
                const uint32_t need = __ballot_sync(kFull, !have && !exhausted);
                if (need) {
                    const uint32_t leader = __ffs(need) - 1u;
                    uint32_t base = 0;
                    if (lane == leader) base = atomicAdd(&P.hdr->fetch, __popc(need));
                    base = __shfl_sync(kFull, base, leader);
                    if (!have && !exhausted) {
                        const uint32_t idx = base + __popc(need & ((1u << lane) - 1u));
                        if (idx < total) {
                            slot = P.lists[idx];
                            const uint32_t c = P.u(F_CELL, slot);
                            S = &P.jobs[ring_of(c)].S;
                            band = band_of(c);
                            rng.k0 = P.u(F_K0, slot);
                            rng.k1 = P.u(F_K1, slot);
                            rng.k2 = P.u(F_K2, slot);
                            rng.dim = P.u(F_DIM, slot);
                            shadow = (P.u(F_META, slot) & M_SHADOW) != 0u;
                            const V3 o = mk(P.f(F_OX, slot), P.f(F_OY, slot), P.f(F_OZ, slot));
                            if (shadow) {
                                const V3 l = mk(P.f(F_LX, slot), P.f(F_LY, slot), P.f(F_LZ, slot));
                                k.g = ray_geo(madd(o, l, kRayEpsilonKm), l);
                            } else {
                                k.g = ray_geo(o, mk(P.f(F_DX, slot), P.f(F_DY, slot), P.f(F_DZ, slot)));
                            }
                            k.t_max = P.f(F_T, slot);
                            track_begin<kTracking>(*S, band, k, rng, n);
                            have = true;
                        } else {
                            exhausted = true;
                        }
                    }
                }
                if (__ballot_sync(kFull, have) == 0u) break;
                if (have) {
                    const int r = track_action<kTracking>(*S, band, k, rng, n, watchdog);
                    if (r != 0) {
                        if (r == 1 && !shadow) {
                            P.f(F_T, slot) = k.t;
                            P.f(F_ALT, slot) = altitude_at(k.g, k.t, S->ground_radius);
                        }
                        P.u(F_DIM, slot) = rng.dim;
                        const uint32_t meta = P.u(F_META, slot);
                        P.u(F_META, slot) = (meta & ~(M_STATE | M_HIT)) | S_TRACED | (r == 1 ? M_HIT : 0u);
                        have = false;
                    }
                }
            }
        }
        __syncthreads();

        // ---- shade: shadow results, real collisions, ground / escape ----
        build_shade_lists(P);
        __syncthreads();
        for (uint32_t which = 1; which <= 3; ++which) {
            const uint32_t cnt = P.hdr->list_count[which];
            for (uint32_t i = tid; i < cnt; i += kThreads) {
                Path p;
                load_path(P, P.lists[which * kSlots + i], p);
                const DevJob& J = P.jobs[p.ring];
                const DevScene& S = J.S;
                const DevLaunch& L = J.L;
                const uint32_t band = p.band;
                const float l_sun = S.bands[band].solar_radiance;
                if (which == 1) {
                    // shadow result (sky_trace.wgsl:576-581, :600-603); p.o is the event position
                    if (!(p.meta & M_HIT)) {
                        if (p.meta & M_GROUND) {
                            const float cos_sun = fmaxf(dot3(normalize_or_y(p.o), p.ldir), 0.0f);
                            p.nee += S.ground_albedo * kInvPi * l_sun * 1.0f * cos_sun / S.light_pdf;
                        } else {
                            const Coeffs c = coefficients_at(S, S.knot_z, S.finder, band, p.alt);
                            p.nee += l_sun * 1.0f * mixed_phase(S, c, band, dot3(p.dir, p.ldir)) / S.light_pdf;
                        }
                    }
                    p.meta = with_light(p.meta & ~M_SHADOW, light_of(p.meta) + 1u);
                    lights_and_continue<kPhase>(P, S, L, p, n, watchdog);
                } else if (which == 2) {
                    // real collision (sky_trace.wgsl:720-733); p.alt was set by the tracker
                    ++n.e[SKY_EVENT_SCATTER];
                    p.o = madd(p.o, p.dir, p.t);
                    const Coeffs c = coefficients_at(S, S.knot_z, S.finder, band, p.alt);
                    if (c.extinction <= 0.0f || c.scattering <= 0.0f) {
                        finish(P, p, fmaxf(p.rad, 0.0f));
                    } else {
                        p.thr *= fminf(fmaxf(c.scattering / c.extinction, 0.0f), 1.0f);
                        if (p.thr <= 0.0f) {
                            finish(P, p, fmaxf(p.rad, 0.0f));
                        } else {
                            p.nee = 0.0f;
                            p.meta = with_light(p.meta & ~M_GROUND, 0u);
                            lights_and_continue<kPhase>(P, S, L, p, n, watchdog);
                        }
                    }
                } else {
                    if (p.meta & M_EXIT) {  // escape (sky_trace.wgsl:745-749)
                        if (depth_of(p.meta) == 0u && dot3(p.dir, load3(S.sun)) >= S.cos_max) p.rad += p.thr * l_sun;
                        finish(P, p, fmaxf(p.rad, 0.0f));
                    } else {  // ground (sky_trace.wgsl:750-752): T still holds the ground distance
                        ++n.e[SKY_EVENT_GROUND];
                        p.o = madd(p.o, p.dir, p.t);
                        p.nee = 0.0f;
                        p.meta = with_light(p.meta | M_GROUND, 0u);
                        lights_and_continue<kPhase>(P, S, L, p, n, watchdog);
                    }
                }
                store_path(P, p);
            }
        }
        __syncthreads();
        if (++iterations > kMaxIterations) {  // never expected: give up, report it
            stalled = true;
            break;
        }
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
}

template <int kTracking, int kPhase, uint32_t kPer, int kMinBlocks>
cudaError_t launch_one(const PoolLaunch& w, cudaStream_t stream) {
    auto fn = pool_kernel<kTracking, kPhase, kPer, kMinBlocks>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(w.layout.total));
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, int(kThreads), w.layout.total);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    if (w.max_blocks_per_sm > 0) per_sm = std::min(per_sm, int(w.max_blocks_per_sm));
    int device = 0, sms = 0;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    uint32_t blocks = std::max(1u, std::min(uint32_t(sms) * uint32_t(per_sm), w.total_groups));
    fn<<<blocks, kThreads, w.layout.total, stream>>>(w.jobs, w.num_jobs, w.total_groups, w.layout, w.work_counter,
                                                     w.counters, w.status);
    return cudaGetLastError();
}

template <int kTracking, int kPhase>
cudaError_t launch_variant(const PoolLaunch& w, cudaStream_t stream) {
    if (w.variant == 1) return launch_one<kTracking, kPhase, 2u, 3>(w, stream);
    return launch_one<kTracking, kPhase, 4u, 2>(w, stream);
}

}  // namespace

uint32_t pool_slots_per_thread(uint32_t variant) { return variant == 1 ? 2u : 4u; }

cudaError_t launch_trace_pool(const PoolLaunch& w, cudaStream_t stream) {
#define SKY_POOL_CASE(TR, PH) \
    if (w.tracking == TR && w.phase_sampling == PH) return launch_variant<TR, PH>(w, stream);
    SKY_POOL_CASE(SKY_TRACKING_SEGMENT_RESTART, SKY_PHASE_ISOTROPIC)
    SKY_POOL_CASE(SKY_TRACKING_SEGMENT_RESTART, SKY_PHASE_TABULATED)
    SKY_POOL_CASE(SKY_TRACKING_RESIDUAL_CARRY, SKY_PHASE_ISOTROPIC)
    SKY_POOL_CASE(SKY_TRACKING_RESIDUAL_CARRY, SKY_PHASE_TABULATED)
    SKY_POOL_CASE(SKY_TRACKING_MERGED_LAYERS, SKY_PHASE_ISOTROPIC)
    SKY_POOL_CASE(SKY_TRACKING_MERGED_LAYERS, SKY_PHASE_TABULATED)
#undef SKY_POOL_CASE
    return cudaErrorInvalidValue;
}

PoolLayout plan_pool_layout(const DevScene& S, bool with_majorants, bool stage_tables, uint32_t variant) {
    const uint32_t kSlots = kThreads * pool_slots_per_thread(variant);
    PoolLayout l{};
    size_t off = 0;
    auto take = [&off](size_t bytes) {
        const size_t at = off;
        off = (off + bytes + 15) / 16 * 16;
        return uint32_t(at);
    };
    l.header = take(sizeof(PoolHeader));
    l.jobs = take(kRing * sizeof(DevJob));
    l.acc = take(size_t(kRing) * kMaxCells * 2u * sizeof(double));
    l.slots = take(size_t(F_COUNT) * kSlots * 4u);
    l.lists = take(5u * kSlots * 2u);
    l.staged = stage_tables ? 1u : 0u;
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
