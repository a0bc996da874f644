// bhr_trace_noalloc: the mixed-precision single-view trace for callers that cannot allocate
// device memory.
//
// bhr_create allocates its work memory with cudaMalloc. Some callers cannot do that: a render
// loop that must not stall (cudaMalloc and cudaFree synchronise the device), a host
// application whose memory pool already owns all device memory and hands plugins only their
// input and output buffers, or code recording a CUDA graph, where allocation is not allowed.
// This entry point needs no context and allocates nothing. Its work memory (the work-queue
// counters and the FP64 hand-off queues of the mixed-precision march) is one file-scope
// device array, g_noalloc_scratch, sized for kNoAllocMaxRays rays per call. Every GPU that
// loads the library holds that array (about 15 MB) until the process exits.
//
// The array is shared by every call on a device and keeps the last call's contents. Each call
// clears the counters that must start at zero on its own stream before the kernels run.
// Calls that overlap on the GPU (different streams, or several host threads) race on the
// array; calls on one stream are ordered and safe.
//
// Host code must not pass the array's name to a kernel: on the host that name is only a
// stand-in, not a device address. The first call on each device, with that device current,
// resolves the address with cudaGetSymbolAddress (which may load the module, so make that
// first call before any stream capture) and keeps it for later calls, together with the
// identity of the device's context (cuCtxGetId). A cudaDeviceReset destroys the context and
// the array with it; the next call sees a new context identity and resolves the address again,
// so that call, too, should come before any stream capture.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "bhr.h"
#include "host_views.h"
#include "kernels.cuh"

namespace {

constexpr int64_t kNoAllocMaxRays = 262144;  // rays per call (e.g. 512x512 or 640x360)
constexpr int kMaxDevices = 64;

struct NoAllocScratch {
    bhr::WorkQueue q;                        // counters: cleared at the start of every call
    int2 band[kNoAllocMaxRays];              // FP64 band rays (ray, view slot)
    bhr::PromoEntry promo[kNoAllocMaxRays];  // FP32 states handed to the FP64 pass
};

static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

struct DeviceSetup {
    bool ready = false;
    NoAllocScratch* scratch = nullptr;  // device address of g_noalloc_scratch on this device
    unsigned long long ctx_id = 0;      // the context the address belongs to
    int sms = 0;
};

std::mutex g_mu;
DeviceSetup g_dev[kMaxDevices];

// cuCtxGetId from the driver through the runtime (no link against libcuda): the unique identity
// of the calling thread's current context.
using CtxGetId = CUresult (*)(CUcontext, unsigned long long*);
CtxGetId g_ctx_get_id = nullptr;

int fail(int code, const std::string& msg) {
    bhr::set_last_error(msg);
    return code;
}

// Once per device (and again after a cudaDeviceReset gave it a new context), with that device
// current: resolve the scratch address and read the SM count.
int setup_device(int dev, DeviceSetup* out) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (dev < 0 || dev >= kMaxDevices) return fail(BHR_ERR_INVALID_ARG, "bhr_trace_noalloc: device ordinal out of range");
    // make the device's primary context current (cudaSetDevice initialises it; no allocation)
    cudaError_t se = cudaSetDevice(dev);
    if (se != cudaSuccess) return fail(BHR_ERR_CUDA, std::string("bhr_trace_noalloc: cudaSetDevice: ") + cudaGetErrorString(se));
    if (!g_ctx_get_id) {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult qr{};
        se = cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &qr);
        if (se != cudaSuccess || qr != cudaDriverEntryPointSuccess || !fn)
            return fail(BHR_ERR_CUDA, "bhr_trace_noalloc: the driver has no cuCtxGetId");
        g_ctx_get_id = reinterpret_cast<CtxGetId>(fn);
    }
    unsigned long long ctx_id = 0;
    if (g_ctx_get_id(nullptr, &ctx_id) != CUDA_SUCCESS)
        return fail(BHR_ERR_CUDA, "bhr_trace_noalloc: no current context on the device");
    DeviceSetup& d = g_dev[dev];
    if (d.ready && d.ctx_id != ctx_id) d.ready = false;  // the device was reset: the old address is gone
    if (!d.ready) {
        int major = 0, minor = 0, sms = 0;
        cudaError_t e = cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess)
            return fail(BHR_ERR_CUDA, std::string("bhr_trace_noalloc: device query: ") + cudaGetErrorString(e));
        if (major * 10 + minor != 103)
            return fail(BHR_ERR_UNSUPPORTED, "bhr_trace_noalloc: this library is built for sm_103a only");
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr)
            return fail(BHR_ERR_CUDA, std::string("bhr_trace_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        d.scratch = static_cast<NoAllocScratch*>(p);
        d.ctx_id = ctx_id;
        d.sms = sms;
        d.ready = true;
    }
    *out = d;
    return BHR_OK;
}

}  // namespace

extern "C" int bhr_trace_noalloc(const bhr_view* view, bhr_hit* out_dev, void* cuda_stream) {
    if (!view || !out_dev) return fail(BHR_ERR_INVALID_ARG, "bhr_trace_noalloc: view or output is NULL");
    std::string msg;
    const int rc = bhr::host::check_view(*view, 0, &msg);
    if (rc != BHR_OK) return fail(rc, "bhr_trace_noalloc: " + msg);
    if (reinterpret_cast<uintptr_t>(out_dev) % 16 != 0)
        return fail(BHR_ERR_INVALID_ARG, "bhr_trace_noalloc: the output buffer must be 16-byte aligned");
    const int64_t rays = int64_t(view->width) * view->height;
    if (rays > kNoAllocMaxRays)
        return fail(BHR_ERR_INVALID_ARG,
                    "bhr_trace_noalloc: the view has " + std::to_string(rays) +
                        " rays; the static work memory holds at most " + std::to_string(kNoAllocMaxRays) +
                        " rays per call (split the view, or use bhr_create + bhr_trace)");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(BHR_ERR_CUDA, std::string("bhr_trace_noalloc: ") + cudaGetErrorString(e));
    DeviceSetup d;
    const int src = setup_device(dev, &d);
    if (src != BHR_OK) return src;

    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    const bhr::Scratch sc{&d.scratch->q, d.scratch->band, d.scratch->promo};
    e = cudaMemsetAsync(sc.q, 0, sizeof(bhr::WorkQueue), st);
    if (e != cudaSuccess) return fail(BHR_ERR_CUDA, std::string("bhr_trace_noalloc: clear: ") + cudaGetErrorString(e));
    const bhr::DevView dv = bhr::host::make_dev_view(*view, out_dev);
    const bhr::Rule rule = bhr::host::make_rule(*view);
    bhr::LaunchCfg cfg{};
    cfg.block = 512;
    cfg.variant = bhr::rule_variant(rule);
    cfg.grid = d.sms * std::max(1, bhr::march_blocks_per_sm(cfg.block, cfg.variant, false, true));
    cfg.chunk = 64;
    cfg.refill = 8;
    e = bhr::launch_march_one(dv, rule, sc, true, cfg, st);
    if (e == cudaSuccess) e = bhr::launch_march_fp64_one(dv, rule, sc, d.sms * 8, st);
    if (e != cudaSuccess) return fail(BHR_ERR_CUDA, std::string("bhr_trace_noalloc: launch: ") + cudaGetErrorString(e));
    return BHR_OK;
}
