// March kernels for sm_103a.
//
// k_march_one / k_march_multi: persistent FP32 march, one ray per lane, 32 rays in flight
//   per warp. Retired lanes are refilled from a per-warp ring of rays that were set up 32
//   at a time (convergent) into shared memory, so ray setup never runs one lane at a time
//   and the step loop stays full. Work comes from a global chunk counter (scratch), `chunk`
//   consecutive pixels at a time. Finished rays are written as 16-byte stores into the
//   caller's hit buffer; a record is 64 B, two whole 32 B sectors, so lane-scattered stores
//   move no extra DRAM bytes.
//     k_march_one:   one view, passed as a __grid_constant__ parameter (constant bank).
//     k_march_multi: up to kMaxViews views in one launch, copied to shared memory; work
//                    chunks never straddle views; per-view completion times are recorded.
//   With kMixed, rays with |b - sqrt(27)| < promote_band are queued for FP64 from the start,
//   and rays that reach r < promote_r hand their state to the FP64 queue.
// k_march_fp64_*: drains the FP64 queue in double precision.
#include <cuda_runtime.h>

#include "kernels.cuh"
#include "march.cuh"

namespace bhr {

namespace {

constexpr int kPool = 64;  // ring entries per warp (two setup batches)
constexpr int kStepsPerCheck = 2;
constexpr float kSqrt27f = 5.19615242270663f;

__device__ __forceinline__ unsigned long long globaltimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// First two 16-byte words of a finished record (the crossing words are written during the march).
__device__ __forceinline__ void write_hit(bhr_hit* rec, uint32_t info, uint32_t steps, float min_r, float3 d,
                                          float b_axis, float b, uint32_t flags) {
    const uint32_t status = (info >> kStatusShift) & 0xfu;
    if ((info >> 16) & 1u) flags |= BHR_FLAG_NONFINITE;
    const uint32_t w0 = status | (((info >> kNcrossShift) & 3u) << 8) | (flags << 16) | ((info & 0xffu) << 24);
    float4* p = reinterpret_cast<float4*>(rec);
    p[0] = make_float4(__uint_as_float(w0), __uint_as_float(steps), d.x, d.y);
    p[1] = make_float4(d.z, b_axis, b, min_r);
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
    float* f;         // [8][kPool]: v.x v.y v.z h2 ssf b_axis b ray
    uint8_t* view;    // [kPool] view slot (multi-view launches)
    __device__ __forceinline__ float& at(int k, int slot) const { return f[k * kPool + slot]; }
};

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

template <bool kMulti, bool kMixed>
__device__ __forceinline__ void march_warp(const DevView* views, int nviews, int64_t total_chunks,
                                           const Scratch sc, int chunk, int refill_min, Pool pool) {
    WorkQueue* q = sc.q;
    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    int64_t cbeg = 0, cend = 0;  // warp's current chunk [cbeg, cend), ray indices of view cview
    int cview = 0;
    int phead = 0, pcount = 0;   // pool ring
    bool dry = false;
    bool active = false, pending = false;
    RayState<float> s;
    s.x = {0.f, 0.f, 0.f};
    s.v = {0.f, 0.f, 0.f};
    s.h2 = 0.f;
    s.ssf = 0.f;
    s.min_r = 0.f;
    s.steps = 0;
    s.info = 0;
    float b_axis = 0.f, b = 0.f;
    int ridx = 0;   // ray index within its view
    int vslot = 0;  // view slot of the lane's ray
    unsigned long long steps_sum = 0, promoted = 0, nonfinite = 0;

    for (;;) {
        const unsigned idle = __ballot_sync(0xffffffffu, !active);
        const int nidle = __popc(idle);
        if (nidle != 0 && (nidle >= refill_min || dry)) {
            // ---- retire the finished rays of this warp
            if (pending) {
                const DevView& w = views[vslot];
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
                    e.b_axis = b_axis;
                    e.b = b;
                    ++promoted;
                    counted = false;  // the FP64 pass finishes it
                    steps_sum += s.steps;
                } else {
                    write_hit(w.out + ridx, s.info, s.steps, s.min_r, exit_dir(s, w.lensing != 0), b_axis, b, 0u);
                    steps_sum += s.steps;
                    nonfinite += (s.info >> 16) & 1u;
                }
                if constexpr (kMulti) {
                    if (counted) {
                        const unsigned m = __match_any_sync(__activemask(), vslot);
                        if (lane == __ffs(m) - 1) {
                            const unsigned long long c = __popc(m);
                            const unsigned long long old = atomicAdd(&q->view_done[vslot], c);
                            if (old + c == (unsigned long long)w.nrays) q->view_t_end[vslot] = globaltimer();
                        }
                    }
                }
                pending = false;
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
                        // chunks never straddle views: find v with chunk_start[v] <= base
                        for (int g = 0; g < nviews; g += 32) {
                            const int k = g + lane;
                            const bool ge = k < nviews && (int64_t)base >= views[k].chunk_start;
                            const unsigned bm = __ballot_sync(0xffffffffu, ge);
                            if (bm) v = g + 31 - __clz(bm);
                        }
                    }
                    cview = v;
                    cbeg = ((int64_t)base - views[v].chunk_start) * chunk;
                    cend = min(cbeg + (int64_t)chunk, views[v].nrays);
                }
                const int n = (int)min((int64_t)32, cend - cbeg);
                const DevView& w = views[cview];
                bool keep = false;
                RayInit<float> ri;
                const int my = (int)(cbeg + lane);
                if (lane < n) {
                    const int j = my / w.width;
                    const int i = my - j * w.width;
                    V3<float> dir;
                    ri = setup_ray<float>(w, i, j, &dir);
                    keep = true;
                    if constexpr (kMixed) {
                        if (w.lensing && fabsf(ri.b - kSqrt27f) < w.promote_band) {
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
                    pool.at(5, slot) = ri.b_axis;
                    pool.at(6, slot) = ri.b;
                    pool.at(7, slot) = __int_as_float(my);
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
                b_axis = pool.at(5, slot);
                b = pool.at(6, slot);
                ridx = __float_as_int(pool.at(7, slot));
                s.x = {w.cam[0], w.cam[1], w.cam[2]};
                s.min_r = __int_as_float(0x7f800000);  // +inf
                s.steps = 0;
                s.info = 0;
                // crossing words start at zero; march_step fills them as crossings happen
                float4* p = reinterpret_cast<float4*>(w.out + ridx);
                p[2] = make_float4(0.f, 0.f, 0.f, 0.f);
                p[3] = make_float4(0.f, 0.f, 0.f, 0.f);
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
                const DevView& w = views[vslot];
                if (march_step<float, kMixed>(w, s, w.out + ridx)) {
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
template <bool kMulti>
__device__ __forceinline__ void march_fp64(const DevView* views, const Scratch sc) {
    WorkQueue* q = sc.q;
    const unsigned long long nband = q->band_count;
    const unsigned long long nprom = q->promo_count;
    unsigned long long steps_sum = 0, nrays = 0, nonfinite = 0;
    for (;;) {
        const unsigned long long k = atomicAdd(&q->fp64_next, 1ull);
        if (k >= nband + nprom) break;
        RayState<double> s;
        float b_axis, b;
        int ray, vs;
        uint32_t base_steps = 0;
        if (k < nband) {
            const int2 e = sc.band[k];
            ray = e.x;
            vs = kMulti ? e.y : 0;
            const DevView& w = views[vs];
            const int j = ray / w.width;
            const int i = ray - j * w.width;
            V3<double> dir;
            const RayInit<double> ri = setup_ray<double>(w, i, j, &dir);
            s.x = {w.cam_d[0], w.cam_d[1], w.cam_d[2]};
            s.v = ri.v;
            s.h2 = ri.h2;
            s.ssf = ri.ssf;
            s.min_r = __longlong_as_double(0x7ff0000000000000ll);
            s.steps = 0;
            s.info = 0;
            b_axis = (float)ri.b_axis;
            b = (float)ri.b;
            float4* p = reinterpret_cast<float4*>(w.out + ray);
            p[2] = make_float4(0.f, 0.f, 0.f, 0.f);
            p[3] = make_float4(0.f, 0.f, 0.f, 0.f);
            ++nrays;
        } else {
            const PromoEntry& e = sc.promo[k - nband];
            ray = (int)e.ray;
            vs = kMulti ? e.view : 0;
            const DevView& w = views[vs];
            // continue from the FP32 state; h2 and the step factor are recomputed in FP64
            const int j = ray / w.width;
            const int i = ray - j * w.width;
            V3<double> dir;
            const RayInit<double> ri = setup_ray<double>(w, i, j, &dir);
            s.x = {e.x[0], e.x[1], e.x[2]};
            s.v = {e.v[0], e.v[1], e.v[2]};
            s.h2 = ri.h2;
            s.ssf = ri.ssf;
            s.min_r = e.min_r;
            s.steps = e.steps;
            s.info = e.info;
            base_steps = e.steps;
            b_axis = e.b_axis;
            b = e.b;
        }
        const DevView& w = views[vs];
        bhr_hit* rec = w.out + ray;
        while (!march_step<double, false>(w, s, rec)) {
        }
        steps_sum += s.steps - base_steps;
        nonfinite += (s.info >> 16) & 1u;
        write_hit(rec, s.info, s.steps, (float)s.min_r, exit_dir(s, w.lensing != 0), b_axis, b, BHR_FLAG_FP64);
        if constexpr (kMulti) {
            const unsigned long long old = atomicAdd(&q->view_done[vs], 1ull);
            if (old + 1 == (unsigned long long)w.nrays) q->view_t_end[vs] = globaltimer();
        }
    }
    if (steps_sum | nrays | nonfinite) {
        atomicAdd(&q->fp64_steps, steps_sum);
        atomicAdd(&q->steps, steps_sum);
        if (nrays) atomicAdd(&q->fp64_rays, nrays);
        if (nonfinite) atomicAdd(&q->nonfinite, nonfinite);
    }
}

}  // namespace

template <int BS, bool kMixed>
__global__ void __launch_bounds__(BS) k_march_one(const __grid_constant__ DevView view, const Scratch sc,
                                                  int chunk, int refill_min) {
    __shared__ float s_pool[BS / 32][8 * kPool];
    note_start(sc.q);
    const int wid = threadIdx.x >> 5;
    const int64_t total_chunks = (view.nrays + chunk - 1) / chunk;
    march_warp<false, kMixed>(&view, 1, total_chunks, sc, chunk, refill_min, Pool{s_pool[wid], nullptr});
}

template <int BS, bool kMixed>
__global__ void __launch_bounds__(BS) k_march_multi(const __grid_constant__ ViewBatch batch, const Scratch sc,
                                                    int chunk, int refill_min) {
    __shared__ float s_pool[BS / 32][8 * kPool];
    __shared__ uint8_t s_pool_view[BS / 32][kPool];
    __shared__ DevView s_views[kMaxViews];
    note_start(sc.q);
    const int nwords = batch.nviews * (int)(sizeof(DevView) / 4);
    for (int k = threadIdx.x; k < nwords; k += BS)
        reinterpret_cast<uint32_t*>(s_views)[k] = reinterpret_cast<const uint32_t*>(batch.views)[k];
    __syncthreads();
    const int wid = threadIdx.x >> 5;
    march_warp<true, kMixed>(s_views, batch.nviews, batch.total_chunks, sc, chunk, refill_min,
                             Pool{s_pool[wid], s_pool_view[wid]});
}

__global__ void __launch_bounds__(128) k_march_fp64_one(const __grid_constant__ DevView view, const Scratch sc) {
    march_fp64<false>(&view, sc);
}

__global__ void __launch_bounds__(128) k_march_fp64_multi(const __grid_constant__ ViewBatch batch,
                                                          const Scratch sc) {
    march_fp64<true>(batch.views, sc);
}

// ---------------------------------------------------------------------------------------
// launchers
template <int BS>
static cudaError_t launch_one_bs(const DevView& v, const Scratch& s, bool mixed, const LaunchCfg& c,
                                 cudaStream_t st) {
    if (mixed)
        k_march_one<BS, true><<<c.grid, BS, 0, st>>>(v, s, c.chunk, c.refill);
    else
        k_march_one<BS, false><<<c.grid, BS, 0, st>>>(v, s, c.chunk, c.refill);
    return cudaGetLastError();
}

template <int BS>
static cudaError_t launch_multi_bs(const ViewBatch& b, const Scratch& s, bool mixed, const LaunchCfg& c,
                                   cudaStream_t st) {
    if (mixed)
        k_march_multi<BS, true><<<c.grid, BS, 0, st>>>(b, s, c.chunk, c.refill);
    else
        k_march_multi<BS, false><<<c.grid, BS, 0, st>>>(b, s, c.chunk, c.refill);
    return cudaGetLastError();
}

cudaError_t launch_march_one(const DevView& v, const Scratch& s, bool mixed, const LaunchCfg& c, cudaStream_t st) {
    switch (c.block) {
        case 128: return launch_one_bs<128>(v, s, mixed, c, st);
        case 256: return launch_one_bs<256>(v, s, mixed, c, st);
        case 512: return launch_one_bs<512>(v, s, mixed, c, st);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_march_multi(const ViewBatch& b, const Scratch& s, bool mixed, const LaunchCfg& c,
                               cudaStream_t st) {
    switch (c.block) {
        case 128: return launch_multi_bs<128>(b, s, mixed, c, st);
        case 256: return launch_multi_bs<256>(b, s, mixed, c, st);
        case 512: return launch_multi_bs<512>(b, s, mixed, c, st);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_march_fp64_one(const DevView& v, const Scratch& s, int grid, cudaStream_t st) {
    k_march_fp64_one<<<grid, 128, 0, st>>>(v, s);
    return cudaGetLastError();
}

cudaError_t launch_march_fp64_multi(const ViewBatch& b, const Scratch& s, int grid, cudaStream_t st) {
    k_march_fp64_multi<<<grid, 128, 0, st>>>(b, s);
    return cudaGetLastError();
}

template <int BS>
static int bps(bool multi, bool mixed) {
    int n = 0;
    if (multi)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &n, mixed ? (const void*)k_march_multi<BS, true> : (const void*)k_march_multi<BS, false>, BS, 0);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &n, mixed ? (const void*)k_march_one<BS, true> : (const void*)k_march_one<BS, false>, BS, 0);
    return n;
}

int march_blocks_per_sm(int block, bool multi, bool mixed) {
    switch (block) {
        case 128: return bps<128>(multi, mixed);
        case 256: return bps<256>(multi, mixed);
        case 512: return bps<512>(multi, mixed);
        default: return 0;
    }
}

}  // namespace bhr
