// Structures shared by the march kernels and the host side of the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "march.cuh"

namespace bhr {

constexpr int kMaxViews = 64;  // views per persistent launch (larger batches run as several)

// Work counters in device memory, owned by the context and zeroed before every trace.
struct WorkQueue {
    unsigned long long next_chunk;   // next work chunk handed to a warp
    unsigned long long band_count;   // FP64 band rays queued (mixed)
    unsigned long long promo_count;  // FP32 states handed to FP64 (mixed)
    unsigned long long fp64_next;    // FP64 work handed out
    unsigned long long steps;        // executed march steps (all precisions)
    unsigned long long fp64_rays;    // rays that ran partly or wholly in FP64
    unsigned long long fp64_steps;   // steps taken in FP64
    unsigned long long nonfinite;    // rays that met a non-finite state
    unsigned long long t_start;      // globaltimer when the first block started
    unsigned long long view_done[kMaxViews];   // finished rays per view
    unsigned long long view_t_end[kMaxViews];  // globaltimer when a view's last ray finished
};

// An FP32 ray state handed to the FP64 pass (mixed precision). 64 bytes.
struct PromoEntry {
    int64_t ray;       // ray index within its view
    int32_t view;      // view slot in the launch
    uint32_t steps;    // steps already taken
    uint32_t info;     // nplane / ncross bits (status cleared)
    float x[3], v[3];
    float min_r, b_axis, b;
    uint32_t pad[2];
};

// Several views for one persistent launch, passed as a __grid_constant__ parameter.
struct ViewBatch {
    int32_t nviews;
    int32_t pad;
    int64_t total_chunks;
    DevView views[kMaxViews];
};

struct Scratch {
    WorkQueue* q;
    int2* band;         // (ray index, view slot) of FP64 band rays
    PromoEntry* promo;  // promoted FP32 states
};

struct LaunchCfg {
    int block;   // 128, 256 or 512
    int grid;    // persistent blocks
    int chunk;   // rays per work chunk
    int refill;  // idle lanes that trigger a refill (1..32)
};

cudaError_t launch_march_one(const DevView& v, const Scratch& s, bool mixed, const LaunchCfg& c, cudaStream_t st);
cudaError_t launch_march_multi(const ViewBatch& b, const Scratch& s, bool mixed, const LaunchCfg& c,
                               cudaStream_t st);
cudaError_t launch_march_fp64_one(const DevView& v, const Scratch& s, int grid, cudaStream_t st);
cudaError_t launch_march_fp64_multi(const ViewBatch& b, const Scratch& s, int grid, cudaStream_t st);
// Max resident blocks per SM of the FP32 march kernel for a block size (occupancy API).
int march_blocks_per_sm(int block, bool multi, bool mixed);

}  // namespace bhr
