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
    unsigned long long surr_rays;    // rays answered by the surrogate
    unsigned long long fb_count;     // rays the surrogate sent to the integrator
    unsigned long long capture_disagree;  // surrogate capture flag disagreed with b vs sqrt(27)
    unsigned long long mlp_queries;  // network queries of surrogate rays (exit + crossings)
    unsigned long long mlp_rows;     // network rows evaluated (32 per batch, padding included)
    unsigned long long view_t_end[kMaxViews];  // globaltimer when a view's last ray finished
};

// An FP32 ray state handed to the FP64 pass (mixed precision). 48 bytes.
struct PromoEntry {
    int32_t ray;       // ray index within its view
    int32_t view;      // view slot in the launch
    uint32_t steps;    // steps already taken
    uint32_t info;     // nplane / ncross bits (status cleared)
    float x[3], v[3];
    float min_r;
    uint32_t pad;
};

// Several views sharing one rule, for one persistent launch (a __grid_constant__ parameter).
struct ViewBatch {
    int32_t nviews;
    int32_t pad;
    int64_t total_chunks;
    Rule rule;
    DevView views[kMaxViews];
};

struct Scratch {
    WorkQueue* q;
    int2* band;         // (ray index, view slot) of FP64 band rays
    PromoEntry* promo;  // promoted FP32 states
};

// Compiled specialisations of the loop body (lensing on, no far mode).
enum : int { kVariantGeneric = 0, kVariantConfigThin = 1, kVariantShaderThin = 2, kVariantCpuNone = 3 };

struct LaunchCfg {
    int block;    // 256 or 512
    int grid;     // persistent blocks
    int chunk;    // rays per work chunk
    int refill;   // idle lanes that trigger a refill (1..32)
    int variant;  // kVariant*
};

int rule_variant(const Rule& r);
cudaError_t launch_march_one(const DevView& v, const Rule& r, const Scratch& s, bool mixed, const LaunchCfg& c,
                             cudaStream_t st);
cudaError_t launch_march_multi(const ViewBatch& b, const Scratch& s, bool mixed, const LaunchCfg& c,
                               cudaStream_t st);
cudaError_t launch_march_fp64_one(const DevView& v, const Rule& r, const Scratch& s, int grid, cudaStream_t st);
cudaError_t launch_march_fp64_multi(const ViewBatch& b, const Scratch& s, int grid, cudaStream_t st);
// The FP32 march over a list of pixel indices of one view (512 threads per block, c.grid blocks).
cudaError_t launch_march_list(const DevView& v, const Rule& r, const Scratch& s, const int* list,
                              const unsigned long long* list_len, const LaunchCfg& c, cudaStream_t st);
// The FP32 march over per-view pixel lists of several views sharing one rule; view v's list
// starts at list + views[v].list_off and its length is qv[2v].fb_count. c.block: 64 or 512.
cudaError_t launch_march_multi_list(const ViewBatch& b, const Scratch& s, const int* list, const WorkQueue* qv,
                                    const LaunchCfg& c, cudaStream_t st);
// Lens table of a camera at cam_r (lens.cu): the reference's RK4 construction, or (closed_form)
// every texel from the closed-form orbit. table: BHR_LENS_PHIS x BHR_LENS_RAYS floats on the device.
cudaError_t launch_lens_table(float cam_r, int closed_form, float* table, cudaStream_t st);
double lens_alpha_crit(double r);
float lens_alpha_host(float u, float ac);
// Max resident blocks per SM of an FP32 march kernel (occupancy API).
int march_blocks_per_sm(int block, int variant, bool multi, bool mixed);
// Sets a kernel's dynamic shared-memory limit (dyn_smem bytes) and, with max_carveout, its
// preference for the largest shared-memory carveout, once per kernel and device (the runtime
// keeps function attributes per device context). A kernel that runs beside the surrogate pass
// must prefer the same carveout: an SM changes its L1 / shared split only when idle, so a
// co-resident block configured for less shared memory keeps the pass's blocks off that SM.
cudaError_t prefer_max_smem(const void* fn, int dyn_smem, bool max_carveout);

}  // namespace bhr
