// March kernels for sm_103a.
//
// k_march_one / k_march_multi: persistent FP32 march, one ray per lane, 32 rays in flight per
//   warp. Retired lanes are refilled from a per-warp ring of rays that were set up 32 at a time
//   (convergent) into shared memory, so ray setup never runs one lane at a time and the step
//   loop stays full. Work comes from a global chunk counter (context scratch), `chunk`
//   consecutive work items at a time: pixels in row-major order, or (tile_shift < 5) 32-pixel
//   tiles of 16x2 or 8x4 pixels, so that a setup batch covers a compact patch of the image. A record is 64 B: a lane writes its two start words when the
//   ray starts and its two end words when it retires, each a whole 32 B sector, so lane-
//   scattered stores move no extra DRAM bytes.
//     k_march_one:   one view; view and rule are __grid_constant__ parameters (constant bank).
//     k_march_multi: up to kMaxViews views sharing one rule; views are copied to shared memory;
//                    work chunks never straddle views; per-view completion times are recorded.
//   With kMixed, rays with |b - sqrt(27)| < promote_band are queued for FP64 from the start,
//   and rays that reach r < promote_r hand their state to the FP64 queue.
// k_march_fp64_*: drains the FP64 queue in double precision.
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <set>
#include <utility>

#include "kernels.cuh"
#include "march.cuh"

namespace bhr {

namespace {

constexpr int kPool = 64;  // ring entries per warp (two setup batches)
constexpr int kStepsPerCheck = 3;  // steps between a warp's retire checks (2: +4%, 4: +1.4% time on the 16 poses)
constexpr float kSqrt27f = 5.19615242270663f;

__device__ __forceinline__ unsigned long long globaltimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// End words of a finished record (words 0-7).
__device__ __forceinline__ void write_end(bhr_hit* rec, uint32_t info, uint32_t steps, float min_r, float3 d,
                                          uint32_t flags) {
    const uint32_t status = (info >> kStatusShift) & 0xfu;
    const uint32_t w0 = status | (((info >> kNcrossShift) & 3u) << 8) | (flags << 16) | ((info & 0xffu) << 24);
    float4* p = reinterpret_cast<float4*>(rec);
    p[0] = make_float4(__uint_as_float(w0), __uint_as_float(steps), d.x, d.y);
    p[1] = make_float4(d.z, min_r, 0.f, 0.f);
}

// Start words of a record (words 8-15): b_axis, b, crossing slots cleared.
__device__ __forceinline__ void write_start(bhr_hit* rec, float b_axis, float b) {
    float4* p = reinterpret_cast<float4*>(rec);
    p[2] = make_float4(b_axis, b, 0.f, 0.f);
    p[3] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// A state that went non-finite marches on (comparisons with NaN fail) until the budget; it is
// flagged when the ray retires.
template <class T>
__device__ __forceinline__ bool nonfinite_state(const RayState<T>& s) {
    return !isfinite(dot3(s.x, s.x) + dot3(s.v, s.v));
}

template <class T>
__device__ __forceinline__ float3 exit_dir(const RayState<T>& s, bool lensing) {
    const uint32_t status = (s.info >> kStatusShift) & 0xfu;
    if (status != BHR_STATUS_ESCAPED) return make_float3(0.f, 0.f, 0.f);
    if (lensing) {
        const V3<T> o = far_field_dir(s.x, s.v, s.h2);
        return make_float3(float(o.x), float(o.y), float(o.z));
    }
    const T vi = M<T>::rsqrt(dot3(s.v, s.v));
    return make_float3(float(s.v.x * vi), float(s.v.y * vi), float(s.v.z * vi));
}

// Per-warp ring of set-up rays in shared memory, structure of arrays.
struct Pool {
    float* f;       // [6][kPool]: v.x v.y v.z h2 ssf ray
    uint8_t* view;  // [kPool] view slot (multi-view launches)
    __device__ __forceinline__ float& at(int k, int slot) const { return f[k * kPool + slot]; }
};
constexpr int kPoolFields = 6;

// Warp-aggregated append of one entry per calling lane; returns this lane's slot.
__device__ __forceinline__ unsigned long long warp_append(unsigned long long* ctr) {
    const unsigned m = __activemask();
    const int leader = __ffs(m) - 1;
    const int lane = threadIdx.x & 31;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(ctr, (unsigned long long)__popc(m));
    base = __shfl_sync(m, base, leader);
    return base + __popc(m & ((1u << lane) - 1u));
}

// kList: the rays of view 0 are the `list_len` pixel indices in `list` (the surrogate's
// fallback rays), written with BHR_FLAG_FALLBACK.
template <bool kMulti, int kTerm, int kDisk, bool kMixed, bool kList = false>
__device__ __forceinline__ void march_warp(const DevView* views, int nviews, int64_t total_chunks, const Rule& R,
                                           const Scratch sc, int chunk, int refill_min, Pool pool,
                                           const int* list = nullptr, int64_t list_len = 0) {
    WorkQueue* q = sc.q;
    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    int64_t cbeg = 0, cend = 0;  // warp's current chunk [cbeg, cend), ray indices of view cview
    int cview = 0;
    int phead = 0, pcount = 0;   // pool ring
    bool dry = false;
    bool active = false, pending = false, stamp = false;
    RayState<float> s;
    s.x = {0.f, 0.f, 0.f};
    s.v = {0.f, 0.f, 0.f};
    s.h2 = 0.f;
    s.ssf = 0.f;
    s.min_r = 0.f;
    s.steps = 0;
    s.info = 0;
    bhr_hit* rec = nullptr;
    int ridx = 0;      // ray index within its view
    int vslot = 0;     // view slot of the lane's ray
    int lane_budget = kMulti ? 0 : views[0].max_steps;
    float lane_dstep = kMulti ? 0.f : views[0].disk_step;
    unsigned long long steps_sum = 0, promoted = 0, nonfinite = 0;

    for (;;) {
        const unsigned idle = __ballot_sync(0xffffffffu, !active);
        const int nidle = __popc(idle);
        if (nidle != 0 && (nidle >= refill_min || dry)) {
            // ---- retire the finished rays of this warp
            if (pending) {
                const uint32_t st = (s.info >> kStatusShift) & 0xfu;
                bool counted = true;
                if (kMixed && st == kPromote) {
                    PromoEntry& e = sc.promo[warp_append(&q->promo_count)];
                    e.ray = ridx;
                    e.view = vslot;
                    e.steps = s.steps;
                    e.info = s.info & ~(0xfu << kStatusShift);
                    e.x[0] = s.x.x; e.x[1] = s.x.y; e.x[2] = s.x.z;
                    e.v[0] = s.v.x; e.v[1] = s.v.y; e.v[2] = s.v.z;
                    e.min_r = s.min_r;
                    ++promoted;
                    counted = false;  // the FP64 pass finishes it
                } else {
                    const bool bad = nonfinite_state(s);
                    write_end(rec, s.info, s.steps, s.min_r, exit_dir(s, R.lensing != 0),
                              (bad ? BHR_FLAG_NONFINITE : 0u) | (kList ? BHR_FLAG_FALLBACK : 0u));
                    nonfinite += bad ? 1 : 0;
                }
                steps_sum += s.steps;
                stamp = counted;
                pending = false;
            }
            if constexpr (kMulti) {
                // a view's completion time = the latest retire time of its rays: one atomicMax
                // per distinct view among the rays retired now (usually one)
                unsigned sm = __ballot_sync(0xffffffffu, stamp);
                while (sm) {
                    const int leader = __ffs(sm) - 1;
                    const int v0 = __shfl_sync(0xffffffffu, vslot, leader);
                    sm &= ~__ballot_sync(0xffffffffu, stamp && vslot == v0);
                    if (lane == leader) atomicMax(&q->view_t_end[v0], globaltimer());
                }
                stamp = false;
            }
            // ---- top up the pool with convergent setup batches of up to 32 rays
            while (pcount < nidle && !dry) {
                if (cbeg >= cend) {
                    unsigned long long base = 0;
                    if (lane == 0) base = atomicAdd(&q->next_chunk, 1ull);
                    base = __shfl_sync(0xffffffffu, base, 0);
                    if ((int64_t)base >= total_chunks) {
                        dry = true;
                        break;
                    }
                    int v = 0;
                    if constexpr (kMulti) {
                        // chunks never straddle views: the last v with chunk_start[v] <= base
                        for (int g = 0; g < nviews; g += 32) {
                            const int k = g + lane;
                            const bool ge = k < nviews && (int64_t)base >= views[k].chunk_start;
                            const unsigned bm = __ballot_sync(0xffffffffu, ge);
                            if (bm) v = g + 31 - __clz(bm);
                        }
                    }
                    cview = v;
                    cbeg = ((int64_t)base - views[v].chunk_start) * chunk;
                    cend = min(cbeg + (int64_t)chunk,
                               kList ? (kMulti ? views[v].nrays : list_len) : views[v].work);
                }
                const int n = (int)min((int64_t)32, cend - cbeg);
                const DevView& w = views[cview];
                bool keep = false;
                RayInit<float> ri;
                bool inside = lane < n;
                int my;
                if constexpr (kList) {
                    my = inside ? list[(kMulti ? w.list_off : 0) + cbeg + lane] : 0;
                } else if (w.tile_shift == 5) {
                    my = (int)(cbeg + lane);
                } else {  // work item -> pixel of a (1 << tile_shift) x (32 >> tile_shift) tile
                    const int64_t m = cbeg + lane;
                    const int t = (int)(m >> 5), l = (int)(m & 31);
                    const int ty = t / w.tiles_x, tx = t - ty * w.tiles_x;
                    const int pi = (tx << w.tile_shift) + (l & ((1 << w.tile_shift) - 1));
                    const int pj = ty * (32 >> w.tile_shift) + (l >> w.tile_shift);
                    inside = inside && pi < w.width && pj < w.height;
                    my = pj * w.width + pi;
                }
                if (inside) {
                    const int j = my / w.width;
                    const int i = my - j * w.width;
                    ri = setup_ray<float>(w, R, i, j);
                    write_start(w.out + my, ri.b_axis, ri.b);
                    keep = true;
                    if constexpr (kMixed) {
                        if (R.lensing && fabsf(ri.b - kSqrt27f) < R.promote_band) {
                            keep = false;  // the whole ray runs in FP64
                            sc.band[warp_append(&q->band_count)] = make_int2(my, cview);
                        }
                    }
                }
                const unsigned km = __ballot_sync(0xffffffffu, keep);
                if (keep) {
                    const int slot = (phead + pcount + __popc(km & lt_mask)) & (kPool - 1);
                    pool.at(0, slot) = ri.v.x;
                    pool.at(1, slot) = ri.v.y;
                    pool.at(2, slot) = ri.v.z;
                    pool.at(3, slot) = ri.h2;
                    pool.at(4, slot) = ri.ssf;
                    pool.at(5, slot) = __int_as_float(my);
                    if constexpr (kMulti) pool.view[slot] = (uint8_t)cview;
                }
                pcount += __popc(km);
                cbeg += n;
            }
            __syncwarp();
            // ---- refill idle lanes from the pool
            const int rank = __popc(idle & lt_mask);
            if (!active && rank < pcount) {
                const int slot = (phead + rank) & (kPool - 1);
                vslot = kMulti ? (int)pool.view[slot] : 0;
                const DevView& w = views[vslot];
                s.v = {pool.at(0, slot), pool.at(1, slot), pool.at(2, slot)};
                s.h2 = pool.at(3, slot);
                s.ssf = pool.at(4, slot);
                ridx = __float_as_int(pool.at(5, slot));
                rec = w.out + ridx;
                s.x = {w.cam[0], w.cam[1], w.cam[2]};
                s.min_r = __int_as_float(0x7f800000);  // +inf
                s.steps = 0;
                s.info = 0;
                if constexpr (kMulti) {
                    lane_budget = w.max_steps;
                    lane_dstep = w.disk_step;
                }
                active = true;
            }
            const int taken = min(nidle, pcount);
            phead = (phead + taken) & (kPool - 1);
            pcount -= taken;
            __syncwarp();
            if (dry && pcount == 0 && !__any_sync(0xffffffffu, active)) break;
        }
        // ---- march
#pragma unroll
        for (int u = 0; u < kStepsPerCheck; ++u) {
            if (active) {
                if (march_step<float, kTerm, kDisk, kMixed>(R, lane_budget, lane_dstep, s, rec)) {
                    active = false;
                    pending = true;
                }
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        steps_sum += __shfl_xor_sync(0xffffffffu, steps_sum, o);
        promoted += __shfl_xor_sync(0xffffffffu, promoted, o);
        nonfinite += __shfl_xor_sync(0xffffffffu, nonfinite, o);
    }
    if (lane == 0) {
        atomicAdd(&q->steps, steps_sum);
        if (promoted) atomicAdd(&q->fp64_rays, promoted);
        if (nonfinite) atomicAdd(&q->nonfinite, nonfinite);
    }
}

__device__ __forceinline__ void note_start(WorkQueue* q) {
    if (threadIdx.x == 0) atomicCAS(&q->t_start, 0ull, globaltimer());
}

// FP64 continuation: band rays from scratch, then promoted FP32 states. One ray per thread
// with dynamic fetch; FP64 runs at a small fraction of the FP32 rate, so the queues are short.
template <bool kMulti, int kTerm, int kDisk>
__device__ __forceinline__ void march_fp64(const DevView* views, const Rule& R, const Scratch sc) {
    WorkQueue* q = sc.q;
    const unsigned long long nband = q->band_count;
    const unsigned long long nprom = q->promo_count;
    unsigned long long steps_sum = 0, nrays = 0, nonfinite = 0;
    for (;;) {
        const unsigned long long k = atomicAdd(&q->fp64_next, 1ull);
        if (k >= nband + nprom) break;
        RayState<double> s;
        int ray, vs;
        uint32_t base_steps = 0;
        if (k < nband) {
            const int2 e = sc.band[k];
            ray = e.x;
            vs = kMulti ? e.y : 0;
            const DevView& w = views[vs];
            const int j = ray / w.width;
            const int i = ray - j * w.width;
            const RayInit<double> ri = setup_ray<double>(w, R, i, j);
            s.x = {w.cam_d[0], w.cam_d[1], w.cam_d[2]};
            s.v = ri.v;
            s.h2 = ri.h2;
            s.ssf = ri.ssf;
            s.min_r = __longlong_as_double(0x7ff0000000000000ll);
            s.steps = 0;
            s.info = 0;
            write_start(w.out + ray, (float)ri.b_axis, (float)ri.b);
            ++nrays;
        } else {
            const PromoEntry& e = sc.promo[k - nband];
            ray = (int)e.ray;
            vs = kMulti ? e.view : 0;
            const DevView& w = views[vs];
            // continue from the FP32 state; h2 and the step factor are recomputed in FP64
            const int j = ray / w.width;
            const int i = ray - j * w.width;
            const RayInit<double> ri = setup_ray<double>(w, R, i, j);
            s.x = {e.x[0], e.x[1], e.x[2]};
            s.v = {e.v[0], e.v[1], e.v[2]};
            s.h2 = ri.h2;
            s.ssf = ri.ssf;
            s.min_r = e.min_r;
            s.steps = e.steps;
            s.info = e.info;
            base_steps = e.steps;
        }
        const DevView& w = views[vs];
        bhr_hit* rec = w.out + ray;
        while (!march_step<double, kTerm, kDisk, false>(R, w.max_steps, (double)w.disk_step, s, rec)) {
        }
        steps_sum += s.steps - base_steps;
        const bool bad = nonfinite_state(s);
        nonfinite += bad ? 1 : 0;
        write_end(rec, s.info, s.steps, (float)s.min_r, exit_dir(s, R.lensing != 0),
                  BHR_FLAG_FP64 | (bad ? BHR_FLAG_NONFINITE : 0u));
        if constexpr (kMulti) atomicMax(&q->view_t_end[vs], globaltimer());
    }
    if (steps_sum | nrays | nonfinite) {
        atomicAdd(&q->fp64_steps, steps_sum);
        atomicAdd(&q->steps, steps_sum);
        if (nrays) atomicAdd(&q->fp64_rays, nrays);
        if (nonfinite) atomicAdd(&q->nonfinite, nonfinite);
    }
}

}  // namespace

template <int BS, int kTerm, int kDisk, bool kMixed>
__global__ void __launch_bounds__(BS) k_march_one(const __grid_constant__ DevView view, const __grid_constant__ Rule rule,
                                                  const Scratch sc, int chunk, int refill_min) {
    __shared__ float s_pool[BS / 32][kPoolFields * kPool];
    note_start(sc.q);
    const int wid = threadIdx.x >> 5;
    const int64_t total_chunks = (view.work + chunk - 1) / chunk;
    march_warp<false, kTerm, kDisk, kMixed>(&view, 1, total_chunks, rule, sc, chunk, refill_min,
                                            Pool{s_pool[wid], nullptr});
}

template <int BS, int kTerm, int kDisk, bool kMixed>
__global__ void __launch_bounds__(BS) k_march_multi(const __grid_constant__ ViewBatch batch, const Scratch sc,
                                                    int chunk, int refill_min) {
    __shared__ float s_pool[BS / 32][kPoolFields * kPool];
    __shared__ uint8_t s_pool_view[BS / 32][kPool];
    __shared__ DevView s_views[kMaxViews];
    note_start(sc.q);
    const int nwords = batch.nviews * (int)(sizeof(DevView) / 4);
    for (int k = threadIdx.x; k < nwords; k += BS)
        reinterpret_cast<uint32_t*>(s_views)[k] = reinterpret_cast<const uint32_t*>(batch.views)[k];
    __syncthreads();
    const int wid = threadIdx.x >> 5;
    march_warp<true, kTerm, kDisk, kMixed>(s_views, batch.nviews, batch.total_chunks, batch.rule, sc, chunk,
                                           refill_min, Pool{s_pool[wid], s_pool_view[wid]});
}

template <int kTerm, int kDisk>
__global__ void __launch_bounds__(512) k_march_list(const __grid_constant__ DevView view,
                                                    const __grid_constant__ Rule rule, const Scratch sc,
                                                    const int* list, const unsigned long long* list_len, int chunk,
                                                    int refill_min) {
    __shared__ float s_pool[512 / 32][kPoolFields * kPool];
    const int wid = threadIdx.x >> 5;
    const int64_t n = (int64_t)*list_len;
    if (n == 0) return;
    const int64_t total_chunks = (n + chunk - 1) / chunk;
    march_warp<false, kTerm, kDisk, false, true>(&view, 1, total_chunks, rule, sc, chunk, refill_min,
                                                 Pool{s_pool[wid], nullptr}, list, n);
}

// The surrogate's fallback rays of several views in one launch: view v's list is
// list[list_off_v .. list_off_v + qv[2v].fb_count) (counts written on the device). 512-thread
// blocks after the surrogate pass; 64-thread blocks for the band march beside it, which holds
// few warps and must leave the SMs' registers to the pass.
template <int BS, int kTerm, int kDisk>
__global__ void __launch_bounds__(BS) k_march_multi_list(const __grid_constant__ ViewBatch batch, const Scratch sc,
                                                         const int* list, const WorkQueue* qv, int chunk,
                                                         int refill_min) {
    __shared__ float s_pool[BS / 32][kPoolFields * kPool];
    __shared__ uint8_t s_pool_view[BS / 32][kPool];
    __shared__ DevView s_views[kMaxViews];
    __shared__ int64_t s_total;
    // the lists' lengths first: an empty set of lists (the usual case after the band march) ends
    // the block before it copies the views or claims work
    if (threadIdx.x == 0) {
        int64_t n = 0;
        for (int v = 0; v < batch.nviews; ++v) n += (int64_t)qv[2 * v].fb_count;
        s_total = n;
    }
    __syncthreads();
    if (s_total == 0) return;
    const int nwords = batch.nviews * (int)(sizeof(DevView) / 4);
    for (int k = threadIdx.x; k < nwords; k += BS)
        reinterpret_cast<uint32_t*>(s_views)[k] = reinterpret_cast<const uint32_t*>(batch.views)[k];
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t acc = 0;
        for (int v = 0; v < batch.nviews; ++v) {
            const int64_t n = (int64_t)qv[2 * v].fb_count;
            s_views[v].nrays = n;
            s_views[v].chunk_start = acc;
            acc += (n + chunk - 1) / chunk;
        }
        s_total = acc;
    }
    __syncthreads();
    const int wid = threadIdx.x >> 5;
    march_warp<true, kTerm, kDisk, false, true>(s_views, batch.nviews, s_total, batch.rule, sc, chunk, refill_min,
                                                Pool{s_pool[wid], s_pool_view[wid]}, list, 0);
}

template <int kTerm, int kDisk>
__global__ void __launch_bounds__(128) k_march_fp64_one(const __grid_constant__ DevView view,
                                                        const __grid_constant__ Rule rule, const Scratch sc) {
    march_fp64<false, kTerm, kDisk>(&view, rule, sc);
}

template <int kTerm, int kDisk>
__global__ void __launch_bounds__(128) k_march_fp64_multi(const __grid_constant__ ViewBatch batch,
                                                          const Scratch sc) {
    march_fp64<true, kTerm, kDisk>(batch.views, batch.rule, sc);
}

// ---------------------------------------------------------------------------------------
// dispatch: (term, disk) -> compiled variant; anything else runs the generic variant
namespace {

template <int BS, int kTerm, int kDisk, bool kMixed>
struct Kern {
    static const void* one() { return (const void*)k_march_one<BS, kTerm, kDisk, kMixed>; }
    static const void* multi() { return (const void*)k_march_multi<BS, kTerm, kDisk, kMixed>; }
};

template <int BS, bool kMixed>
const void* pick(int variant, bool multi) {
    switch (variant) {
        case kVariantConfigThin:
            return multi ? Kern<BS, BHR_TERM_CONFIG, BHR_DISK_THIN, kMixed>::multi()
                         : Kern<BS, BHR_TERM_CONFIG, BHR_DISK_THIN, kMixed>::one();
        case kVariantShaderThin:
            return multi ? Kern<BS, BHR_TERM_SHADER, BHR_DISK_THIN, kMixed>::multi()
                         : Kern<BS, BHR_TERM_SHADER, BHR_DISK_THIN, kMixed>::one();
        case kVariantCpuNone:
            return multi ? Kern<BS, BHR_TERM_CPU, BHR_DISK_NONE, kMixed>::multi()
                         : Kern<BS, BHR_TERM_CPU, BHR_DISK_NONE, kMixed>::one();
        default:
            return multi ? Kern<BS, -1, -1, kMixed>::multi() : Kern<BS, -1, -1, kMixed>::one();
    }
}

const void* pick_kernel(int block, int variant, bool multi, bool mixed) {
    switch (block) {
        case 256: return mixed ? pick<256, true>(variant, multi) : pick<256, false>(variant, multi);
        case 512: return mixed ? pick<512, true>(variant, multi) : pick<512, false>(variant, multi);
        default: return nullptr;
    }
}

}  // namespace

int rule_variant(const Rule& r) {
    if (!r.lensing || r.far_mode) return kVariantGeneric;
    if (r.term_mode == BHR_TERM_CONFIG && r.disk_mode == BHR_DISK_THIN) return kVariantConfigThin;
    if (r.term_mode == BHR_TERM_SHADER && r.disk_mode == BHR_DISK_THIN) return kVariantShaderThin;
    if (r.term_mode == BHR_TERM_CPU && r.disk_mode == BHR_DISK_NONE) return kVariantCpuNone;
    return kVariantGeneric;
}

cudaError_t launch_march_one(const DevView& v, const Rule& r, const Scratch& s, bool mixed, const LaunchCfg& c,
                             cudaStream_t st) {
    const void* fn = pick_kernel(c.block, c.variant, false, mixed);
    if (!fn) return cudaErrorInvalidValue;
    int chunk = c.chunk, refill = c.refill;
    void* args[] = {(void*)&v, (void*)&r, (void*)&s, &chunk, &refill};
    return cudaLaunchKernel(fn, dim3(c.grid), dim3(c.block), args, 0, st);
}

cudaError_t launch_march_multi(const ViewBatch& b, const Scratch& s, bool mixed, const LaunchCfg& c,
                               cudaStream_t st) {
    const void* fn = pick_kernel(c.block, c.variant, true, mixed);
    if (!fn) return cudaErrorInvalidValue;
    int chunk = c.chunk, refill = c.refill;
    void* args[] = {(void*)&b, (void*)&s, &chunk, &refill};
    return cudaLaunchKernel(fn, dim3(c.grid), dim3(c.block), args, 0, st);
}

cudaError_t launch_march_fp64_one(const DevView& v, const Rule& r, const Scratch& s, int grid, cudaStream_t st) {
    switch (rule_variant(r)) {
        case kVariantConfigThin: k_march_fp64_one<BHR_TERM_CONFIG, BHR_DISK_THIN><<<grid, 128, 0, st>>>(v, r, s); break;
        case kVariantShaderThin: k_march_fp64_one<BHR_TERM_SHADER, BHR_DISK_THIN><<<grid, 128, 0, st>>>(v, r, s); break;
        case kVariantCpuNone: k_march_fp64_one<BHR_TERM_CPU, BHR_DISK_NONE><<<grid, 128, 0, st>>>(v, r, s); break;
        default: k_march_fp64_one<-1, -1><<<grid, 128, 0, st>>>(v, r, s); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_march_fp64_multi(const ViewBatch& b, const Scratch& s, int grid, cudaStream_t st) {
    switch (rule_variant(b.rule)) {
        case kVariantConfigThin: k_march_fp64_multi<BHR_TERM_CONFIG, BHR_DISK_THIN><<<grid, 128, 0, st>>>(b, s); break;
        case kVariantShaderThin: k_march_fp64_multi<BHR_TERM_SHADER, BHR_DISK_THIN><<<grid, 128, 0, st>>>(b, s); break;
        case kVariantCpuNone: k_march_fp64_multi<BHR_TERM_CPU, BHR_DISK_NONE><<<grid, 128, 0, st>>>(b, s); break;
        default: k_march_fp64_multi<-1, -1><<<grid, 128, 0, st>>>(b, s); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_march_list(const DevView& v, const Rule& r, const Scratch& s, const int* list,
                              const unsigned long long* list_len, const LaunchCfg& c, cudaStream_t st) {
    int chunk = c.chunk, refill = c.refill;
    const void* fn;
    switch (c.variant) {
        case kVariantConfigThin: fn = (const void*)k_march_list<BHR_TERM_CONFIG, BHR_DISK_THIN>; break;
        case kVariantShaderThin: fn = (const void*)k_march_list<BHR_TERM_SHADER, BHR_DISK_THIN>; break;
        case kVariantCpuNone: fn = (const void*)k_march_list<BHR_TERM_CPU, BHR_DISK_NONE>; break;
        default: fn = (const void*)k_march_list<-1, -1>; break;
    }
    const int grid = c.grid > 0 ? c.grid : 1;
    void* args[] = {(void*)&v, (void*)&r, (void*)&s, (void*)&list, (void*)&list_len, &chunk, &refill};
    return cudaLaunchKernel(fn, dim3(grid), dim3(512), args, 0, st);
}

namespace {
template <int BS>
const void* multi_list_kernel(int variant) {
    switch (variant) {
        case kVariantConfigThin: return (const void*)k_march_multi_list<BS, BHR_TERM_CONFIG, BHR_DISK_THIN>;
        case kVariantShaderThin: return (const void*)k_march_multi_list<BS, BHR_TERM_SHADER, BHR_DISK_THIN>;
        case kVariantCpuNone: return (const void*)k_march_multi_list<BS, BHR_TERM_CPU, BHR_DISK_NONE>;
        default: return (const void*)k_march_multi_list<BS, -1, -1>;
    }
}
}  // namespace

cudaError_t launch_march_multi_list(const ViewBatch& b, const Scratch& s, const int* list, const WorkQueue* qv,
                                    const LaunchCfg& c, cudaStream_t st) {
    int chunk = c.chunk, refill = c.refill;
    if (c.block != 64 && c.block != 512) return cudaErrorInvalidValue;
    const void* fn = c.block == 64 ? multi_list_kernel<64>(c.variant) : multi_list_kernel<512>(c.variant);
    if (c.block == 64) {  // the band march, beside the surrogate pass (the driver's carveout, as the pass's)
        const cudaError_t e = prefer_max_smem(fn, 0, false);
        if (e != cudaSuccess) return e;
    }
    void* args[] = {(void*)&b, (void*)&s, (void*)&list, (void*)&qv, &chunk, &refill};
    return cudaLaunchKernel(fn, dim3(c.grid > 0 ? c.grid : 1), dim3(c.block), args, 0, st);
}

cudaError_t prefer_max_smem(const void* fn, int dyn_smem, bool max_carveout) {
    static std::mutex mu;
    static std::set<std::pair<int, const void*>> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu);
    if (done.count({dev, fn})) return cudaSuccess;
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn_smem);
    if (e == cudaSuccess && max_carveout)
        e = cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (e == cudaSuccess) done.insert({dev, fn});
    return e;
}

int march_blocks_per_sm(int block, int variant, bool multi, bool mixed) {
    // cached per kernel, so that traces captured into a graph make no occupancy queries
    static std::mutex mu;
    static std::map<const void*, int> cache;
    const void* fn = pick_kernel(block, variant, multi, mixed);
    if (!fn) return 0;
    std::lock_guard<std::mutex> lk(mu);
    const auto it = cache.find(fn);
    if (it != cache.end()) return it->second;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, block, 0) != cudaSuccess) return 0;
    cache[fn] = n;
    return n;
}

}  // namespace bhr
