// Host side of the C ABI (include/bhr.h): context, argument checks, the Settings / Camera /
// setTraceUniforms mirror, and the launch sequence of a trace.
//
// Host float arithmetic here is built with -ffp-contract=off so the per-view constants match
// the reference's own float computation on both x86-64 and aarch64.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "bhr.h"
#include "host_views.h"
#include "kernels.cuh"
#include "bodies.cuh"
#include "shade.cuh"
#include "surrogate.cuh"
#include "vol.cuh"

// Device scratch of a trace: one work queue per launch batch, and the FP64 queues of MIXED.
struct TraceScratch {
    bhr::WorkQueue* q = nullptr;
    int nq = 0;
    int2* band = nullptr;
    bhr::PromoEntry* promo = nullptr;
    int64_t rays = 0;  // capacity of band / promo in rays
    void release() {
        if (q) cudaFree(q);
        if (band) cudaFree(band);
        if (promo) cudaFree(promo);
        q = nullptr;
        band = nullptr;
        promo = nullptr;
        nq = 0;
        rays = 0;
    }
};

struct bhr_ctx {
    int device = 0;
    int sms = 0;
    bhr_launch_shape shape{512, 0, 64, 8, 32, 0.0f};  // launch shape of the FP32 march
    TraceScratch scr;
    // bhr_trace_host: device staging (two halves) and two streams, created on first use
    bhr_hit* staging = nullptr;
    int64_t staging_rays = 0;  // rays per half
    cudaStream_t hstream[2] = {nullptr, nullptr};
    cudaStream_t last_stream = nullptr;
    int last_batches = 0;
    std::vector<std::pair<int, int>> last_slots;  // (work queue, view slot) per view of the last trace
    int last_nviews = 0;
    bool have_last = false;
    std::map<std::string, bhr_launch_shape> tuned;  // autotuner results by workload signature
    // shading: the blackbody table and the disk's noise volume, made on first use
    float4* lut = nullptr;
    uint16_t* noise = nullptr;
    uint4* noise8 = nullptr;  // the volume's per-texel neighbourhoods, as the samplers read it
    uint32_t noise_seed = 0;
    bool noise_ready = false;
    // per-view launches of bhr_shade / bhr_trace_volumetric alternate between two side streams,
    // forked from and joined back to the caller's stream (made on first use)
    cudaStream_t fan[2] = {nullptr, nullptr};
    cudaEvent_t fan_fork = nullptr, fan_join[2] = {nullptr, nullptr};
    // the learned orbit surrogate that serves BHR_METHOD_SURROGATE (bound, not owned)
    bhr_surrogate* surr = nullptr;
    std::string err;
};

// A batch of views traced by one instantiated CUDA graph (bhr_plan_*).
struct bhr_plan {
    bhr_ctx* ctx = nullptr;
    std::vector<bhr_view> views;
    std::vector<bhr_hit*> out;
    int precision = BHR_PREC_FP32;
    bhr_launch_shape shape{};
    TraceScratch scr;  // the plan's own: the graph holds these addresses
    cudaStream_t cap = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int batches = 0;
    std::vector<std::pair<int, int>> slots;
    cudaStream_t last_stream = nullptr;
    bool launched = false;
};

namespace {

std::mutex g_err_mu;
std::string g_err;  // last error without a context

int fail(bhr_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    std::lock_guard<std::mutex> lk(g_err_mu);
    g_err = msg;
    return code;
}

int cuda_fail(bhr_ctx* c, cudaError_t e, const char* what) {
    return fail(c, BHR_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

int check_view(bhr_ctx* c, const bhr_view& v, int k) {
    std::string msg;
    const int rc = bhr::host::check_view(v, k, &msg);
    return rc == BHR_OK ? BHR_OK : fail(c, rc, msg);
}

using bhr::host::make_dev_view;
using bhr::host::make_rule;
using bhr::host::shader_r_esc_min;

bool same_rule(const bhr::Rule& a, const bhr::Rule& b) { return std::memcmp(&a, &b, sizeof a) == 0; }

int ensure_scratch(bhr_ctx* c, TraceScratch& scr, int nbatches, int64_t rays, bool mixed) {
    if (nbatches > scr.nq) {
        if (scr.q) cudaFree(scr.q);
        scr.q = nullptr;
        scr.nq = 0;
        cudaError_t e = cudaMalloc(&scr.q, sizeof(bhr::WorkQueue) * size_t(nbatches));
        if (e != cudaSuccess) return fail(c, BHR_ERR_OOM, std::string("work queue: ") + cudaGetErrorString(e));
        scr.nq = nbatches;
    }
    if (mixed && rays > scr.rays) {
        if (scr.band) cudaFree(scr.band);
        if (scr.promo) cudaFree(scr.promo);
        scr.band = nullptr;
        scr.promo = nullptr;
        scr.rays = 0;
        cudaError_t e = cudaMalloc(&scr.band, sizeof(int2) * size_t(rays));
        if (e == cudaSuccess) e = cudaMalloc(&scr.promo, sizeof(bhr::PromoEntry) * size_t(rays));
        if (e != cudaSuccess) return fail(c, BHR_ERR_OOM, std::string("FP64 queue: ") + cudaGetErrorString(e));
        scr.rays = rays;
    }
    return BHR_OK;
}

int check_shape(bhr_ctx* c, const bhr_launch_shape& s) {
    if (s.block_size != 256 && s.block_size != 512)
        return fail(c, BHR_ERR_INVALID_ARG, "launch shape: block_size must be 256 or 512");
    if (s.blocks_per_sm < 0 || s.chunk < 0 || s.refill < 0 || s.refill > 32)
        return fail(c, BHR_ERR_INVALID_ARG, "launch shape: blocks_per_sm, chunk >= 0 and refill in 0..32");
    if (s.tile_w != 0 && s.tile_w != 32 && s.tile_w != 16 && s.tile_w != 8)
        return fail(c, BHR_ERR_INVALID_ARG, "launch shape: tile_w must be 32, 16 or 8");
    return BHR_OK;
}

bhr::LaunchCfg make_cfg(const bhr_ctx* c, const bhr_launch_shape& sh, int variant, bool multi, bool mixed) {
    bhr::LaunchCfg cfg{};
    cfg.block = sh.block_size;
    cfg.variant = variant;
    const int fit = std::max(1, bhr::march_blocks_per_sm(cfg.block, variant, multi, mixed));
    const int bps = sh.blocks_per_sm > 0 ? std::min(sh.blocks_per_sm, fit) : fit;
    cfg.grid = c->sms * bps;
    cfg.refill = std::max(1, std::min(sh.refill > 0 ? sh.refill : 8, 32));
    cfg.chunk = (std::max(32, sh.chunk > 0 ? sh.chunk : 64) + 31) / 32 * 32;
    return cfg;
}

int tile_of(const bhr_launch_shape& sh) { return sh.tile_w == 16 || sh.tile_w == 8 ? sh.tile_w : 32; }

int validate(bhr_ctx* c, const char* who, const bhr_view* views, int nviews, bhr_hit* const* out, int precision,
             int64_t* rays_out) {
    if (!views || nviews <= 0 || !out) return fail(c, BHR_ERR_INVALID_ARG, std::string(who) + ": no views or outputs");
    if (precision != BHR_PREC_FP32 && precision != BHR_PREC_MIXED)
        return fail(c, BHR_ERR_INVALID_ARG, std::string(who) + ": unknown precision");
    int64_t rays = 0;
    for (int k = 0; k < nviews; ++k) {
        const int rc = check_view(c, views[k], k);
        if (rc != BHR_OK) return rc;
        if (!out[k]) return fail(c, BHR_ERR_INVALID_ARG, std::string(who) + ": output buffer " + std::to_string(k) + " is NULL");
        if (reinterpret_cast<uintptr_t>(out[k]) % 16 != 0)
            return fail(c, BHR_ERR_INVALID_ARG, std::string(who) + ": output buffers must be 16-byte aligned");
        rays += int64_t(views[k].width) * views[k].height;
    }
    *rays_out = rays;
    return BHR_OK;
}

// Launch sequence of one trace (views already validated): views grouped by rule, one
// persistent launch per group and per kMaxViews views, each with its own work queue.
// Stream-ordered; captures cleanly into a graph (no host synchronisation, no allocation
// once `scr` is large enough).
int run_trace(bhr_ctx* c, const bhr_launch_shape& shape, TraceScratch& scr, const bhr_view* views, int nviews,
              bhr_hit* const* out_dev, int precision, int64_t rays, cudaStream_t st,
              std::vector<std::pair<int, int>>* slots_out, int* batches_out) {
    const bool mixed = precision == BHR_PREC_MIXED;
    std::vector<bhr::Rule> rules;
    std::vector<std::vector<int>> groups;
    for (int k = 0; k < nviews; ++k) {
        const bhr::Rule r = make_rule(views[k]);
        size_t g = 0;
        while (g < rules.size() && !same_rule(rules[g], r)) ++g;
        if (g == rules.size()) {
            rules.push_back(r);
            groups.emplace_back();
        }
        groups[g].push_back(k);
    }
    int nb = 0;
    for (const auto& g : groups) nb += int((g.size() + bhr::kMaxViews - 1) / bhr::kMaxViews);
    int rc = ensure_scratch(c, scr, nb, rays, mixed);
    const int fp64_grid = c->sms * 8;
    const int tile = tile_of(shape);
    int bi = 0;
    std::vector<std::pair<int, int>> slots(size_t(nviews), {0, 0});
    for (size_t g = 0; rc == BHR_OK && g < groups.size(); ++g) {
        const bhr::Rule& rule = rules[g];
        const int variant = bhr::rule_variant(rule);
        const std::vector<int>& members = groups[g];
        for (size_t m0 = 0; rc == BHR_OK && m0 < members.size(); m0 += bhr::kMaxViews, ++bi) {
            bhr::Scratch sc{scr.q + bi, scr.band, scr.promo};
            cudaError_t e = cudaMemsetAsync(sc.q, 0, sizeof(bhr::WorkQueue), st);
            if (e != cudaSuccess) {
                rc = cuda_fail(c, e, "trace: cudaMemsetAsync");
                break;
            }
            const size_t nv = std::min<size_t>(bhr::kMaxViews, members.size() - m0);
            if (nviews == 1) {
                const bhr::DevView dv = make_dev_view(views[0], out_dev[0], tile);
                e = bhr::launch_march_one(dv, rule, sc, mixed, make_cfg(c, shape, variant, false, mixed), st);
                if (e == cudaSuccess && mixed) e = bhr::launch_march_fp64_one(dv, rule, sc, fp64_grid, st);
            } else {
                static thread_local bhr::ViewBatch b;  // ~12 KB, passed by value as a kernel parameter
                const bhr::LaunchCfg cfg = make_cfg(c, shape, variant, true, mixed);
                b.nviews = int(nv);
                b.rule = rule;
                int64_t chunk_acc = 0;
                for (size_t k = 0; k < nv; ++k) {
                    const int vi = members[m0 + k];
                    slots[size_t(vi)] = {bi, int(k)};
                    b.views[k] = make_dev_view(views[vi], out_dev[vi], tile);
                    b.views[k].chunk_start = chunk_acc;
                    chunk_acc += (b.views[k].work + cfg.chunk - 1) / cfg.chunk;
                }
                b.total_chunks = chunk_acc;
                e = bhr::launch_march_multi(b, sc, mixed, cfg, st);
                if (e == cudaSuccess && mixed) e = bhr::launch_march_fp64_multi(b, sc, fp64_grid, st);
            }
            if (e != cudaSuccess) rc = cuda_fail(c, e, "trace: kernel launch");
        }
    }
    if (rc == BHR_OK) {
        if (slots_out) *slots_out = std::move(slots);
        if (batches_out) *batches_out = nb;
    }
    return rc;
}

int read_queues(bhr_ctx* c, const TraceScratch& scr, int batches, cudaStream_t st, std::vector<bhr::WorkQueue>* qs,
                const char* who) {
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(c->device);
    cudaError_t e = cudaStreamSynchronize(st);
    qs->resize(size_t(batches));
    if (e == cudaSuccess)
        e = cudaMemcpy(qs->data(), scr.q, sizeof(bhr::WorkQueue) * qs->size(), cudaMemcpyDeviceToHost);
    cudaSetDevice(prev);
    return e == cudaSuccess ? BHR_OK : cuda_fail(c, e, who);
}

void sum_stats(const std::vector<bhr::WorkQueue>& qs, int64_t rays, bhr_stats* s) {
    std::memset(s, 0, sizeof *s);
    s->rays = uint64_t(rays);
    for (const auto& q : qs) {
        s->steps += q.steps;
        s->fp64_rays += q.fp64_rays;
        s->fp64_steps += q.fp64_steps;
        s->nonfinite += q.nonfinite;
    }
}

void view_times(const std::vector<bhr::WorkQueue>& qs, const std::vector<std::pair<int, int>>& slots, double* ms,
                int nviews) {
    for (int k = 0; k < nviews; ++k) {
        const bhr::WorkQueue& q = qs[size_t(slots[size_t(k)].first)];
        const int s = slots[size_t(k)].second;
        ms[k] = q.view_t_end[s] >= q.t_start ? double(q.view_t_end[s] - q.t_start) * 1e-6 : -1.0;
    }
}

}  // namespace

void bhr::set_last_error(const std::string& msg) { fail(nullptr, BHR_ERR_INVALID_ARG, msg); }

extern "C" {

int bhr_abi_version(void) { return BHR_ABI_VERSION; }

const char* bhr_last_error(const bhr_ctx* ctx) {
    if (ctx) return ctx->err.c_str();
    std::lock_guard<std::mutex> lk(g_err_mu);
    return g_err.c_str();
}

int bhr_create(bhr_ctx** out, const bhr_options* opts) {
    if (!out) return fail(nullptr, BHR_ERR_INVALID_ARG, "bhr_create: ctx pointer is NULL");
    *out = nullptr;
    bhr_ctx* c = new (std::nothrow) bhr_ctx();
    if (!c) return fail(nullptr, BHR_ERR_OOM, "bhr_create: out of host memory");
    c->device = opts ? opts->device : 0;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        delete c;
        return fail(nullptr, BHR_ERR_CUDA, std::string("bhr_create: no CUDA device: ") + cudaGetErrorString(e));
    }
    if (c->device < 0 || c->device >= ndev) {
        delete c;
        return fail(nullptr, BHR_ERR_INVALID_ARG, "bhr_create: device ordinal out of range");
    }
    cudaDeviceProp prop{};
    e = cudaGetDeviceProperties(&prop, c->device);
    if (e != cudaSuccess) {
        delete c;
        return cuda_fail(nullptr, e, "bhr_create: cudaGetDeviceProperties");
    }
    if (prop.major * 10 + prop.minor != 103) {
        delete c;
        char buf[160];
        std::snprintf(buf, sizeof buf, "bhr_create: device %d is sm_%d%d; this library is built for sm_103a only",
                      c->device, prop.major, prop.minor);
        return fail(nullptr, BHR_ERR_UNSUPPORTED, buf);
    }
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(c->device);
    c->sms = prop.multiProcessorCount;
    if (opts) {
        bhr_launch_shape sh = c->shape;
        if (opts->block_size != 0) sh.block_size = opts->block_size;
        if (opts->chunk > 0) sh.chunk = opts->chunk;
        if (opts->refill > 0) sh.refill = opts->refill;
        if (opts->blocks_per_sm > 0) sh.blocks_per_sm = opts->blocks_per_sm;
        if (opts->tile_w != 0) sh.tile_w = opts->tile_w;
        if (check_shape(nullptr, sh) != BHR_OK) {
            cudaSetDevice(prev);
            delete c;
            return BHR_ERR_INVALID_ARG;
        }
        c->shape = sh;
    }
    const int rc = ensure_scratch(c, c->scr, 1, 0, false);
    cudaSetDevice(prev);
    if (rc != BHR_OK) {
        delete c;
        return rc;
    }
    *out = c;
    return BHR_OK;
}

int bhr_destroy(bhr_ctx* c) {
    if (!c) return BHR_OK;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(c->device);
    c->scr.release();
    if (c->staging) cudaFree(c->staging);
    if (c->lut) cudaFree(c->lut);
    if (c->noise) cudaFree(c->noise);
    if (c->noise8) cudaFree(c->noise8);
    for (cudaStream_t& st : c->hstream)
        if (st) cudaStreamDestroy(st);
    for (cudaEvent_t& e : c->fan_join)
        if (e) cudaEventDestroy(e);
    if (c->fan_fork) cudaEventDestroy(c->fan_fork);
    for (cudaStream_t& st : c->fan)
        if (st) cudaStreamDestroy(st);
    cudaSetDevice(prev);
    delete c;
    return BHR_OK;
}

int bhr_view_init(bhr_view* v, int term_mode) {
    if (!v) return fail(nullptr, BHR_ERR_INVALID_ARG, "bhr_view_init: view is NULL");
    if (term_mode < BHR_TERM_SHADER || term_mode > BHR_TERM_CPU)
        return fail(nullptr, BHR_ERR_INVALID_ARG, "bhr_view_init: unknown term_mode");
    std::memset(v, 0, sizeof *v);
    // Settings defaults (Settings.h:19-37,82); the disk mode is thin (volumetric is out of scope)
    v->width = 1920;
    v->height = 1080;
    v->max_steps = 450;
    v->step_scale = 0.05f;
    v->disk_step = 0.18f;
    v->disk_inner = 6.0f;
    v->disk_outer = 20.0f;
    v->disk_thickness = 0.035f;
    v->disk_mode = BHR_DISK_THIN;
    v->lensing = 1;
    v->far_mode = 0;
    v->term_mode = term_mode;
    bhr_view_set_fov(v, 60.0f);
    // default pose: the "Interstellar shot" bookmark (Camera.cpp:54-55)
    const double pos[3] = {0.0, 2.6, 24.9}, tgt[3] = {0.0, 0.0, 0.0};
    bhr_view_look_at(v, pos, tgt);
    v->escape_r = 1000.0f;
    v->promote_band = 1e-2f;
    v->promote_r = 2.5f;
    switch (term_mode) {
        case BHR_TERM_SHADER:  // R_HORIZON + 0.02 (blackhole.frag:144), ESC_TOL (geodesic.glsl:8)
            v->capture_r = 2.0f + 0.02f;
            v->esc_tol = 0.01f;
            v->r_esc_min = shader_r_esc_min(v->disk_outer);
            v->ds_floor = 0.02f;
            break;
        case BHR_TERM_CONFIG:
            v->capture_r = 2.0001f;
            v->esc_tol = 0.01f;
            v->r_esc_min = shader_r_esc_min(v->disk_outer);
            v->ds_floor = 0.02f;
            break;
        case BHR_TERM_CPU:  // trace() defaults (Geodesic.h:107-108,119)
            v->max_steps = 200000;
            v->step_scale = 0.005f;
            v->capture_r = 2.01f;
            v->esc_tol = 1e-4f;
            v->r_esc_min = 30.0f;
            v->ds_floor = 1e-4f;
            v->disk_mode = BHR_DISK_NONE;
            break;
    }
    return BHR_OK;
}

int bhr_view_apply_preset(bhr_view* v, int preset) {
    if (!v) return fail(nullptr, BHR_ERR_INVALID_ARG, "bhr_view_apply_preset: view is NULL");
    switch (preset) {  // Settings::applyPreset (Settings.cpp:12-35)
        case 0: v->max_steps = 200; v->step_scale = 0.10f; v->disk_step = 0.35f; break;
        case 1: v->max_steps = 300; v->step_scale = 0.07f; v->disk_step = 0.30f; break;
        case 2: v->max_steps = 450; v->step_scale = 0.05f; v->disk_step = 0.18f; break;
        case 3: v->max_steps = 700; v->step_scale = 0.035f; v->disk_step = 0.10f; break;
        default: return fail(nullptr, BHR_ERR_INVALID_ARG, "bhr_view_apply_preset: preset must be 0..3");
    }
    return BHR_OK;
}

int bhr_view_set_fov(bhr_view* v, float fov_deg) {
    if (!v || !(fov_deg > 0.0f) || !(fov_deg < 180.0f))
        return fail(nullptr, BHR_ERR_INVALID_ARG, "bhr_view_set_fov: fov must be in (0, 180) degrees");
    // Renderer.cpp:246: std::tan(glm::radians(s.fovDeg) * 0.5f)
    const float rad = fov_deg * 0.01745329251994329576923690768489f;
    v->tan_half_fov = std::tan(rad * 0.5f);
    return BHR_OK;
}

int bhr_look_rotation(const double from[3], const double target[3], const float up_in[3], float q_out[4]) {
    if (!from || !target || !q_out) return fail(nullptr, BHR_ERR_INVALID_ARG, "bhr_look_rotation: NULL argument");
    // Camera.cpp:12-23 lookRotation(from, target, up), camera looking down -Z
    const double fd[3] = {target[0] - from[0], target[1] - from[1], target[2] - from[2]};
    const double len = std::sqrt(fd[0] * fd[0] + fd[1] * fd[1] + fd[2] * fd[2]);
    float f[3] = {0.0f, 0.0f, -1.0f};
    if (len > 0.0)
        for (int k = 0; k < 3; ++k) f[k] = float(fd[k] / len);
    float u[3] = {0.0f, 1.0f, 0.0f};
    if (up_in)
        for (int k = 0; k < 3; ++k) u[k] = up_in[k];
    const float ul = std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    if (!(ul > 0.0f)) return fail(nullptr, BHR_ERR_INVALID_ARG, "bhr_look_rotation: up vector is zero");
    const float un[3] = {u[0] * (1.0f / ul), u[1] * (1.0f / ul), u[2] * (1.0f / ul)};
    if (std::fabs(f[0] * un[0] + f[1] * un[1] + f[2] * un[2]) > 0.999f) {
        u[0] = 0.0f; u[1] = 0.0f; u[2] = -1.0f;
    }
    float r[3] = {f[1] * u[2] - u[1] * f[2], f[2] * u[0] - u[2] * f[0], f[0] * u[1] - u[0] * f[1]};
    const float rl = 1.0f / std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    for (float& e : r) e *= rl;
    const float uu[3] = {r[1] * f[2] - f[1] * r[2], r[2] * f[0] - f[2] * r[0], r[0] * f[1] - f[0] * r[1]};
    // m = mat3(r, uu, -f): column-major m[col][row]
    const float m[3][3] = {{r[0], r[1], r[2]}, {uu[0], uu[1], uu[2]}, {-f[0], -f[1], -f[2]}};
    // rotation matrix -> unit quaternion by the largest-component method (Shepperd 1978)
    const float t[4] = {m[0][0] + m[1][1] + m[2][2], m[0][0] - m[1][1] - m[2][2], m[1][1] - m[0][0] - m[2][2],
                        m[2][2] - m[0][0] - m[1][1]};
    int big = 0;
    for (int k = 1; k < 4; ++k)
        if (t[k] > t[big]) big = k;
    const float bv = std::sqrt(t[big] + 1.0f) * 0.5f;
    const float mult = 0.25f / bv;
    float qw, qx, qy, qz;
    switch (big) {
        case 0: qw = bv; qx = (m[1][2] - m[2][1]) * mult; qy = (m[2][0] - m[0][2]) * mult; qz = (m[0][1] - m[1][0]) * mult; break;
        case 1: qw = (m[1][2] - m[2][1]) * mult; qx = bv; qy = (m[0][1] + m[1][0]) * mult; qz = (m[2][0] + m[0][2]) * mult; break;
        case 2: qw = (m[2][0] - m[0][2]) * mult; qx = (m[0][1] + m[1][0]) * mult; qy = bv; qz = (m[1][2] + m[2][1]) * mult; break;
        default: qw = (m[0][1] - m[1][0]) * mult; qx = (m[2][0] + m[0][2]) * mult; qy = (m[1][2] + m[2][1]) * mult; qz = bv; break;
    }
    const float qn = 1.0f / std::sqrt(qw * qw + qx * qx + qy * qy + qz * qz);
    q_out[0] = qw * qn;
    q_out[1] = qx * qn;
    q_out[2] = qy * qn;
    q_out[3] = qz * qn;
    return BHR_OK;
}

int bhr_view_set_pose(bhr_view* v, const double pos[3], const float q[4]) {
    if (!v || !pos || !q) return fail(nullptr, BHR_ERR_INVALID_ARG, "bhr_view_set_pose: NULL argument");
    // uCamBasis = mat3_cast(orientation), columns right, up, back (Camera.cpp:67, Renderer.cpp:250)
    const float qw = q[0], qx = q[1], qy = q[2], qz = q[3];
    const float xx = qx * qx, yy = qy * qy, zz = qz * qz, xz = qx * qz, xy = qx * qy, yz = qy * qz;
    const float wx = qw * qx, wy = qw * qy, wz = qw * qz;
    float* B = v->cam_basis;
    B[0] = 1.0f - 2.0f * (yy + zz); B[1] = 2.0f * (xy + wz);        B[2] = 2.0f * (xz - wy);
    B[3] = 2.0f * (xy - wz);        B[4] = 1.0f - 2.0f * (xx + zz); B[5] = 2.0f * (yz + wx);
    B[6] = 2.0f * (xz + wy);        B[7] = 2.0f * (yz - wx);        B[8] = 1.0f - 2.0f * (xx + yy);
    // uCamPos = vec3(Camera::position()) (Renderer.cpp:249)
    for (int k = 0; k < 3; ++k) v->cam_pos[k] = float(pos[k]);
    return BHR_OK;
}

int bhr_view_look_at(bhr_view* v, const double pos[3], const double target[3]) {
    if (!v || !pos || !target) return fail(nullptr, BHR_ERR_INVALID_ARG, "bhr_view_look_at: NULL argument");
    float q[4];
    const int rc = bhr_look_rotation(pos, target, nullptr, q);
    return rc == BHR_OK ? bhr_view_set_pose(v, pos, q) : rc;
}

int bhr_view_orbit_pose(bhr_view* v, double r, double incl, double azim) {
    if (!v || !(r > 0.0)) return fail(nullptr, BHR_ERR_INVALID_ARG, "bhr_view_orbit_pose: bad argument");
    const double pos[3] = {r * std::sin(incl) * std::sin(azim), r * std::cos(incl), r * std::sin(incl) * std::cos(azim)};
    const double tgt[3] = {0.0, 0.0, 0.0};
    return bhr_view_look_at(v, pos, tgt);
}

int64_t bhr_view_rays(const bhr_view* v) {
    if (!v || v->width <= 0 || v->height <= 0) return 0;
    return int64_t(v->width) * v->height;
}

int bhr_trace(bhr_ctx* c, const bhr_view* views, int nviews, bhr_hit* const* out_dev, int precision, int method,
              void* cuda_stream) {
    if (!c) return fail(nullptr, BHR_ERR_INVALID_ARG, "bhr_trace: ctx is NULL");
    if (method != BHR_METHOD_PLAIN && method != BHR_METHOD_SURROGATE)
        return fail(c, BHR_ERR_INVALID_ARG, "bhr_trace: unknown method");
    int64_t rays = 0;
    int rc = validate(c, "bhr_trace", views, nviews, out_dev, precision, &rays);
    if (rc != BHR_OK) return rc;
    // BHR_METHOD_SURROGATE: the views the bound surrogate answers go through it (with its own
    // fallback march for the rays it declines), the others through the plain march below
    std::vector<bhr_view> plain_views;
    std::vector<bhr_hit*> plain_out;
    if (method == BHR_METHOD_SURROGATE) {
        if (!c->surr)
            return fail(c, BHR_ERR_NOT_READY, "bhr_trace: no surrogate is bound to the context (bhr_ctx_set_surrogate)");
        if (precision != BHR_PREC_FP32)
            return fail(c, BHR_ERR_UNSUPPORTED, "bhr_trace: the surrogate path runs in BHR_PREC_FP32");
        std::vector<bhr_view> sv;
        std::vector<bhr_hit*> so;
        const bhr::surr::Norm nm = bhr::surr::norm_of(c->surr);
        for (int k = 0; k < nviews; ++k) {
            std::string why;
            const bool s_ok = bhr::surr::supports_view(nm, views[k], &why);
            (s_ok ? sv : plain_views).push_back(views[k]);
            (s_ok ? so : plain_out).push_back(out_dev[k]);
        }
        if (!sv.empty()) {
            const int src = bhr_surrogate_trace(c->surr, sv.data(), int(sv.size()), so.data(), cuda_stream);
            if (src != BHR_OK) return fail(c, src, std::string("bhr_trace: ") + bhr_last_error(nullptr));
        }
        if (plain_views.empty()) {  // no plain march ran: bhr_trace_stats has nothing of this trace to report
            c->have_last = false;
            return BHR_OK;
        }
        views = plain_views.data();
        out_dev = plain_out.data();
        nviews = int(plain_views.size());
        rays = 0;
        for (const bhr_view& v : plain_views) rays += int64_t(v.width) * v.height;
    }
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(c->device);
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    std::vector<std::pair<int, int>> slots;
    int nb = 0;
    rc = run_trace(c, c->shape, c->scr, views, nviews, out_dev, precision, rays, st, &slots, &nb);
    if (rc == BHR_OK) {
        c->last_stream = st;
        c->last_batches = nb;
        c->last_nviews = nviews;
        c->last_slots = std::move(slots);
        c->have_last = true;
    }
    cudaSetDevice(prev);
    return rc;
}

int bhr_ctx_set_surrogate(bhr_ctx* c, bhr_surrogate* s) {
    if (!c) return fail(nullptr, BHR_ERR_INVALID_ARG, "bhr_ctx_set_surrogate: ctx is NULL");
    if (s && bhr::surr::device_of(s) != c->device)
        return fail(c, BHR_ERR_INVALID_ARG, "bhr_ctx_set_surrogate: the surrogate lives on another device");
    c->surr = s;
    return BHR_OK;
}

int bhr_trace_host(bhr_ctx* c, const bhr_view* views, int nviews, bhr_hit* const* out_host, int precision,
                   int method) {
    if (!c) return fail(nullptr, BHR_ERR_INVALID_ARG, "bhr_trace_host: ctx is NULL");
    if (!views || nviews <= 0 || !out_host) return fail(c, BHR_ERR_INVALID_ARG, "bhr_trace_host: no views or outputs");
    int64_t biggest = 0;
    for (int k = 0; k < nviews; ++k) {
        const int rc = check_view(c, views[k], k);
        if (rc != BHR_OK) return rc;
        if (!out_host[k]) return fail(c, BHR_ERR_INVALID_ARG, "bhr_trace_host: output buffer is NULL");
        biggest = std::max(biggest, int64_t(views[k].width) * views[k].height);
    }
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(c->device);
    int rc = BHR_OK;
    // groups of views, each traced in one launch into one staging half while the other half's
    // records travel to the host on the other stream
    const int64_t half = std::max<int64_t>(biggest, int64_t(1) << 22);
    if (half > c->staging_rays) {
        if (c->staging) cudaFree(c->staging);
        c->staging = nullptr;
        c->staging_rays = 0;
        cudaError_t e = cudaMalloc(&c->staging, sizeof(bhr_hit) * size_t(2 * half));
        if (e != cudaSuccess) rc = fail(c, BHR_ERR_OOM, std::string("bhr_trace_host staging: ") + cudaGetErrorString(e));
        else c->staging_rays = half;
    }
    for (int k = 0; rc == BHR_OK && k < 2; ++k)
        if (!c->hstream[k] && cudaStreamCreateWithFlags(&c->hstream[k], cudaStreamNonBlocking) != cudaSuccess)
            rc = fail(c, BHR_ERR_CUDA, "bhr_trace_host: cannot create streams");
    std::vector<bhr_hit*> dst;
    int g = 0;
    for (int k0 = 0; rc == BHR_OK && k0 < nviews; ++g) {
        // views that fit one staging half, at most kMaxViews
        int k1 = k0;
        int64_t acc = 0;
        while (k1 < nviews && k1 - k0 < bhr::kMaxViews) {
            const int64_t n = int64_t(views[k1].width) * views[k1].height;
            if (acc + n > c->staging_rays && k1 > k0) break;
            acc += n;
            ++k1;
        }
        cudaStream_t st = c->hstream[g & 1];
        bhr_hit* base = c->staging + (g & 1) * c->staging_rays;
        dst.clear();
        int64_t off = 0;
        for (int k = k0; k < k1; ++k) {
            dst.push_back(base + off);
            off += int64_t(views[k].width) * views[k].height;
        }
        rc = bhr_trace(c, views + k0, k1 - k0, dst.data(), precision, method, st);
        off = 0;
        for (int k = k0; rc == BHR_OK && k < k1; ++k) {
            const int64_t n = int64_t(views[k].width) * views[k].height;
            cudaError_t e = cudaMemcpyAsync(out_host[k], base + off, sizeof(bhr_hit) * size_t(n),
                                            cudaMemcpyDeviceToHost, st);
            if (e != cudaSuccess) rc = cuda_fail(c, e, "bhr_trace_host: copy to host");
            off += n;
        }
        k0 = k1;
    }
    for (cudaStream_t st : c->hstream) {
        if (!st) continue;
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess && rc == BHR_OK) rc = cuda_fail(c, e, "bhr_trace_host: synchronize");
    }
    cudaSetDevice(prev);
    return rc;
}

int bhr_trace_stats(bhr_ctx* c, bhr_stats* s) {
    if (!c || !s) return fail(c, BHR_ERR_INVALID_ARG, "bhr_trace_stats: NULL argument");
    std::memset(s, 0, sizeof *s);
    if (!c->have_last)
        return fail(c, BHR_ERR_NOT_READY, "bhr_trace_stats: no plain march on this context yet (a trace answered "
                                          "wholly by the surrogate reports through bhr_surrogate_trace_stats)");
    std::vector<bhr::WorkQueue> qs;
    const int rc = read_queues(c, c->scr, c->last_batches, c->last_stream, &qs, "bhr_trace_stats");
    if (rc != BHR_OK) return rc;
    sum_stats(qs, 0, s);
    return BHR_OK;
}

int bhr_trace_view_times(bhr_ctx* c, double* ms, int nviews) {
    if (!c || !ms || nviews <= 0) return fail(c, BHR_ERR_INVALID_ARG, "bhr_trace_view_times: bad argument");
    if (!c->have_last || c->last_nviews != nviews || nviews == 1)
        return fail(c, BHR_ERR_NOT_READY, "bhr_trace_view_times: needs the last trace to be a multi-view trace");
    std::vector<bhr::WorkQueue> qs;
    const int rc = read_queues(c, c->scr, c->last_batches, c->last_stream, &qs, "bhr_trace_view_times");
    if (rc != BHR_OK) return rc;
    view_times(qs, c->last_slots, ms, nviews);
    return BHR_OK;
}

// ---------------------------------------------------------------------------------------
// lens table

int bhr_lens_table(bhr_ctx* c, float cam_r, int method, float* table, void* cuda_stream) {
    if (!c || !table) return fail(c, BHR_ERR_INVALID_ARG, "bhr_lens_table: NULL argument");
    if (!(cam_r > 2.01f) || !std::isfinite(cam_r))
        return fail(c, BHR_ERR_INVALID_ARG, "bhr_lens_table: cam_r must be finite and outside r = 2.01");
    if (method != BHR_METHOD_PLAIN && method != BHR_METHOD_SURROGATE)
        return fail(c, BHR_ERR_INVALID_ARG, "bhr_lens_table: unknown method");
    if (method == BHR_METHOD_SURROGATE && !(cam_r > 3.0f))
        return fail(c, BHR_ERR_UNSUPPORTED, "bhr_lens_table: the closed form needs a camera outside the photon sphere");
    if (reinterpret_cast<uintptr_t>(table) % 16 != 0)
        return fail(c, BHR_ERR_INVALID_ARG, "bhr_lens_table: table must be 16-byte aligned");
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(c->device);
    const cudaError_t e =
        bhr::launch_lens_table(cam_r, method == BHR_METHOD_SURROGATE, table, static_cast<cudaStream_t>(cuda_stream));
    cudaSetDevice(prev);
    return e == cudaSuccess ? BHR_OK : cuda_fail(c, e, "bhr_lens_table");
}

float bhr_lens_alpha(float u, float alpha_crit) { return bhr::lens_alpha_host(u, alpha_crit); }

// ---------------------------------------------------------------------------------------
// shading

int bhr_shade_default_params(bhr_shade_params* p) {
    if (!p) return fail(nullptr, BHR_ERR_INVALID_ARG, "bhr_shade_default_params: NULL argument");
    std::memset(p, 0, sizeof *p);
    // Settings defaults (Settings.h:32-55) at full disk fade, DiskTextures.cpp:106 noise seed
    p->disk_density = 1.0f;
    p->disk_opacity = 2.0f;
    p->disk_peak_temp = 6000.0f;
    p->disk_brightness = 5.5f;
    p->disk_noise_scale = 1.0f;
    p->disk_noise_strength = 0.85f;
    p->disk_time = 0.0f;
    p->disk_warmth = 0.4f;
    p->disk_inflow = 0.0f;
    p->doppler_strength = 0.0f;
    p->sky_brightness = 1.0f;
    p->star_density = 1.0f;
    p->star_brightness = 1.0f;
    p->shadow_overlay = 0;
    p->noise_seed = 7u;
    return BHR_OK;
}

int bhr_blackbody_lut(float* out) {
    if (!out) return fail(nullptr, BHR_ERR_INVALID_ARG, "bhr_blackbody_lut: NULL argument");
    bhr::blackbody_lut_host(out);
    return BHR_OK;
}

namespace {

// The arguments both body marches check; `volumetric` selects which disk modes are accepted.
int check_body_march(bhr_ctx* c, const char* at, const bhr_view* view, const bhr_body* bodies, int nbodies,
                     const bhr_hit* hits, const bhr_body_hit* body_out, bool volumetric) {
    const std::string who(at);
    if (!c || !view || !hits || !body_out || nbodies < 0 || (nbodies > 0 && !bodies))
        return fail(c, BHR_ERR_INVALID_ARG, who + ": NULL argument");
    if (nbodies > BHR_MAX_BODIES)
        return fail(c, BHR_ERR_INVALID_ARG, who + ": at most BHR_MAX_BODIES (32) bodies per view");
    const bhr_view& v = *view;
    if (v.width <= 0 || v.height <= 0 || v.max_steps < 0)
        return fail(c, BHR_ERR_INVALID_ARG, who + ": width and height must be positive, max_steps >= 0");
    if (volumetric && v.disk_mode != BHR_DISK_VOLUMETRIC)
        return fail(c, BHR_ERR_INVALID_ARG, who + ": disk_mode must be BHR_DISK_VOLUMETRIC (bhr_trace_bodies marches the others)");
    if (!volumetric && v.disk_mode != BHR_DISK_NONE && v.disk_mode != BHR_DISK_THIN)
        return fail(c, BHR_ERR_UNSUPPORTED, who + ": the volumetric disk is marched with bodies by bhr_trace_bodies_volumetric");
    if (volumetric && (!(v.disk_step > 0.0f) || !(v.disk_thickness > 0.0f)))
        return fail(c, BHR_ERR_INVALID_ARG, who + ": disk_step and disk_thickness must be positive");
    if (v.term_mode != BHR_TERM_SHADER && v.term_mode != BHR_TERM_CONFIG)
        return fail(c, BHR_ERR_UNSUPPORTED, who + ": bodies are marched under the SHADER or CONFIG rule");
    if (reinterpret_cast<uintptr_t>(hits) % 16 != 0 || reinterpret_cast<uintptr_t>(body_out) % 16 != 0)
        return fail(c, BHR_ERR_INVALID_ARG, who + ": buffers must be 16-byte aligned");
    for (int k = 0; k < nbodies; ++k)
        if (!(bodies[k].pos_radius[3] > 0.0f))
            return fail(c, BHR_ERR_INVALID_ARG, who + ": body " + std::to_string(k) + " has no positive radius");
    return BHR_OK;
}

bhr::BodyArgs body_args(const bhr_view& v, const bhr_body* bodies, int nbodies, bhr_hit* hits, bhr_body_hit* body_out) {
    bhr::BodyArgs a{};
    a.view = bhr::host::make_dev_view(v, hits);
    a.rule = bhr::host::make_rule(v);
    a.nbodies = nbodies;
    a.body_out = body_out;
    for (int k = 0; k < nbodies; ++k) a.bodies[k] = bodies[k];
    return a;
}

}  // namespace

int bhr_trace_bodies(bhr_ctx* c, const bhr_view* view, const bhr_body* bodies, int nbodies, bhr_hit* hits,
                     bhr_body_hit* body_out, void* cuda_stream) {
    const int rc = check_body_march(c, "bhr_trace_bodies", view, bodies, nbodies, hits, body_out, false);
    if (rc != BHR_OK) return rc;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(c->device);
    const bhr::BodyArgs a = body_args(*view, bodies, nbodies, hits, body_out);
    const cudaError_t e = bhr::launch_march_bodies(a, false, static_cast<cudaStream_t>(cuda_stream));
    cudaSetDevice(prev);
    return e == cudaSuccess ? BHR_OK : cuda_fail(c, e, "bhr_trace_bodies");
}

int bhr_noise_bake(bhr_ctx* c, uint32_t seed, uint16_t* out, void* cuda_stream) {
    if (!c || !out) return fail(c, BHR_ERR_INVALID_ARG, "bhr_noise_bake: NULL argument");
    if (reinterpret_cast<uintptr_t>(out) % 16 != 0)
        return fail(c, BHR_ERR_INVALID_ARG, "bhr_noise_bake: out must be 16-byte aligned");
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(c->device);
    const cudaError_t e = bhr::launch_noise_bake(seed, out, static_cast<cudaStream_t>(cuda_stream));
    cudaSetDevice(prev);
    return e == cudaSuccess ? BHR_OK : cuda_fail(c, e, "bhr_noise_bake");
}

namespace {

// Per-view launches spread over the context's two side streams: open() forks them from the
// caller's stream, lane(k) is view k's stream, close() joins them back, so that one view's last
// partial wave overlaps the next view's first. With one view everything stays on `st`.
struct Fan {
    bhr_ctx* c = nullptr;
    cudaStream_t st = nullptr;
    bool on = false;
    cudaError_t open(bhr_ctx* ctx, cudaStream_t s, int nviews) {
        c = ctx;
        st = s;
        on = nviews > 1;
        if (!on) return cudaSuccess;
        cudaError_t e = cudaSuccess;
        for (int k = 0; e == cudaSuccess && k < 2; ++k)
            if (!c->fan[k]) e = cudaStreamCreateWithFlags(&c->fan[k], cudaStreamNonBlocking);
        if (e == cudaSuccess && !c->fan_fork) e = cudaEventCreateWithFlags(&c->fan_fork, cudaEventDisableTiming);
        for (int k = 0; e == cudaSuccess && k < 2; ++k)
            if (!c->fan_join[k]) e = cudaEventCreateWithFlags(&c->fan_join[k], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventRecord(c->fan_fork, st);
        for (int k = 0; e == cudaSuccess && k < 2; ++k) e = cudaStreamWaitEvent(c->fan[k], c->fan_fork, 0);
        if (e != cudaSuccess) on = false;
        return e;
    }
    cudaStream_t lane(int k) const { return on ? c->fan[k & 1] : st; }
    cudaError_t close() {
        if (!on) return cudaSuccess;
        cudaError_t e = cudaSuccess;
        for (int k = 0; e == cudaSuccess && k < 2; ++k) {
            e = cudaEventRecord(c->fan_join[k], c->fan[k]);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(st, c->fan_join[k], 0);
        }
        on = false;
        return e;
    }
};

// The blackbody table and the noise volume of `seed`, complete before the call returns.
int ensure_shade_resources(bhr_ctx* c, uint32_t seed, cudaStream_t st) {
    if (!c->lut) {
        std::vector<float> host(size_t(BHR_BLACKBODY_LUT) * 4);
        bhr::blackbody_lut_host(host.data());
        cudaError_t e = cudaMalloc(&c->lut, host.size() * sizeof(float));
        if (e != cudaSuccess) {
            c->lut = nullptr;
            return cuda_fail(c, e, "bhr_shade: blackbody table");
        }
        e = cudaMemcpy(c->lut, host.data(), host.size() * sizeof(float), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_fail(c, e, "bhr_shade: blackbody table");
    }
    if (!c->noise || !c->noise8) {
        const size_t texels = size_t(BHR_NOISE_SIZE) * BHR_NOISE_SIZE * BHR_NOISE_SIZE;
        cudaError_t e = c->noise ? cudaSuccess : cudaMalloc(&c->noise, texels * 2);
        if (e != cudaSuccess) {
            c->noise = nullptr;
            return cuda_fail(c, e, "bhr_shade: noise volume");
        }
        e = cudaMalloc(&c->noise8, texels * sizeof(uint4));
        if (e != cudaSuccess) {
            c->noise8 = nullptr;
            return cuda_fail(c, e, "bhr_shade: noise neighbourhoods");
        }
        c->noise_ready = false;
    }
    if (!c->noise_ready || c->noise_seed != seed) {
        cudaError_t e = bhr::launch_noise_bake(seed, c->noise, st);
        if (e == cudaSuccess) e = bhr::launch_noise_expand(c->noise, c->noise8, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return cuda_fail(c, e, "bhr_shade: noise bake");
        c->noise_seed = seed;
        c->noise_ready = true;
    }
    return BHR_OK;
}

// The volumetric disk's look for a march: the shading parameters, the view's thickness and the
// context's textures (ensure_shade_resources first).
bhr::DiskLook disk_look(const bhr_ctx* c, const bhr_shade_params& p, const bhr_view& v) {
    bhr::DiskLook L{};
    L.p = p;
    L.ln_1000 = std::log(1000.0f);
    L.ln_40000 = std::log(40000.0f);
    L.thick = v.disk_thickness;
    L.noise8 = c->noise8;
    L.lut = c->lut;
    return L;
}

}  // namespace

int bhr_shade(bhr_ctx* c, const bhr_view* views, int nviews, const bhr_hit* const* hits, const bhr_shade_params* p,
              float* const* rgba, void* cuda_stream) {
    if (!c || !views || nviews <= 0 || !hits || !p || !rgba)
        return fail(c, BHR_ERR_INVALID_ARG, "bhr_shade: NULL argument or no views");
    for (int k = 0; k < nviews; ++k) {
        const bhr_view& v = views[k];
        const std::string at = "bhr_shade: view " + std::to_string(k);
        if (v.width <= 0 || v.height <= 0) return fail(c, BHR_ERR_INVALID_ARG, at + ": width and height must be positive");
        if (!hits[k] || !rgba[k]) return fail(c, BHR_ERR_INVALID_ARG, at + ": NULL buffer");
        if (reinterpret_cast<uintptr_t>(hits[k]) % 16 != 0 || reinterpret_cast<uintptr_t>(rgba[k]) % 16 != 0)
            return fail(c, BHR_ERR_INVALID_ARG, at + ": buffers must be 16-byte aligned");
    }
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(c->device);
    const cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    int rc = ensure_shade_resources(c, p->noise_seed, st);
    Fan fan;
    if (rc == BHR_OK) {
        const cudaError_t e = fan.open(c, st, nviews);
        if (e != cudaSuccess) rc = cuda_fail(c, e, "bhr_shade: side streams");
    }
    for (int k = 0; k < nviews && rc == BHR_OK; ++k) {
        const bhr_view& v = views[k];
        bhr::ShadeArgs a{};
        for (int i = 0; i < 3; ++i) a.cam[i] = v.cam_pos[i];
        for (int i = 0; i < 9; ++i) a.basis[i] = v.cam_basis[i];
        a.tan_half = v.tan_half_fov;
        a.jitter[0] = v.jitter[0];
        a.jitter[1] = v.jitter[1];
        a.width = v.width;
        a.height = v.height;
        a.disk_inner = v.disk_inner;
        a.disk_outer = v.disk_outer;
        a.disk_thin = v.disk_mode == BHR_DISK_THIN;
        a.volumetric = v.disk_mode == BHR_DISK_VOLUMETRIC;
        a.far_mode = v.far_mode;
        a.lensing = (v.lensing != 0 && v.far_mode == 0) ? 1 : 0;
        a.p = *p;
        a.ln_1000 = std::log(1000.0f);
        a.ln_40000 = std::log(40000.0f);
        a.ln_3000 = std::log(3000.0f);
        a.ln_22000 = std::log(22000.0f);
        a.hits = hits[k];
        a.out = reinterpret_cast<float4*>(rgba[k]);
        a.noise8 = c->noise8;
        a.lut = c->lut;
        const cudaError_t e = bhr::launch_shade(a, fan.lane(k));
        if (e != cudaSuccess) rc = cuda_fail(c, e, "bhr_shade: kernel launch");
    }
    {
        const cudaError_t e = fan.close();
        if (e != cudaSuccess && rc == BHR_OK) rc = cuda_fail(c, e, "bhr_shade: side streams");
    }
    cudaSetDevice(prev);
    return rc;
}

int bhr_shade_bodies(bhr_ctx* c, const bhr_view* view, const bhr_hit* hits, const bhr_body_hit* body,
                     const bhr_body* bodies, int nbodies, const bhr_shade_params* p, float* rgba, void* cuda_stream) {
    if (!c || !view || !hits || !body || !p || !rgba || nbodies < 0 || (nbodies > 0 && !bodies))
        return fail(c, BHR_ERR_INVALID_ARG, "bhr_shade_bodies: NULL argument");
    if (nbodies > BHR_MAX_BODIES)
        return fail(c, BHR_ERR_INVALID_ARG, "bhr_shade_bodies: at most BHR_MAX_BODIES (32) bodies per view");
    const bhr_view& v = *view;
    if (v.width <= 0 || v.height <= 0) return fail(c, BHR_ERR_INVALID_ARG, "bhr_shade_bodies: width and height must be positive");
    if (reinterpret_cast<uintptr_t>(hits) % 16 != 0 || reinterpret_cast<uintptr_t>(body) % 16 != 0 ||
        reinterpret_cast<uintptr_t>(rgba) % 16 != 0)
        return fail(c, BHR_ERR_INVALID_ARG, "bhr_shade_bodies: buffers must be 16-byte aligned");
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(c->device);
    const cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    int rc = ensure_shade_resources(c, p->noise_seed, st);
    if (rc == BHR_OK) {
        bhr::ShadeArgs a{};
        for (int i = 0; i < 3; ++i) a.cam[i] = v.cam_pos[i];
        for (int i = 0; i < 9; ++i) a.basis[i] = v.cam_basis[i];
        a.tan_half = v.tan_half_fov;
        a.jitter[0] = v.jitter[0];
        a.jitter[1] = v.jitter[1];
        a.width = v.width;
        a.height = v.height;
        a.disk_inner = v.disk_inner;
        a.disk_outer = v.disk_outer;
        a.disk_thin = v.disk_mode == BHR_DISK_THIN;
        a.volumetric = v.disk_mode == BHR_DISK_VOLUMETRIC;
        a.far_mode = v.far_mode;
        a.lensing = (v.lensing != 0 && v.far_mode == 0) ? 1 : 0;
        a.p = *p;
        a.ln_1000 = std::log(1000.0f);
        a.ln_40000 = std::log(40000.0f);
        a.ln_3000 = std::log(3000.0f);
        a.ln_22000 = std::log(22000.0f);
        a.hits = hits;
        a.out = reinterpret_cast<float4*>(rgba);
        a.noise8 = c->noise8;
        a.lut = c->lut;
        bhr::BodyShadeArgs b{};
        b.bh = body;
        b.nbodies = nbodies;
        for (int k = 0; k < nbodies; ++k) b.bodies[k] = bodies[k];
        const cudaError_t e = bhr::launch_shade_bodies(a, b, st);
        if (e != cudaSuccess) rc = cuda_fail(c, e, "bhr_shade_bodies: kernel launch");
    }
    cudaSetDevice(prev);
    return rc;
}

int bhr_trace_volumetric(bhr_ctx* c, const bhr_view* views, int nviews, bhr_hit* const* hits, const bhr_shade_params* p,
                         float* const* rgbt, void* cuda_stream) {
    if (!c || !views || nviews <= 0 || !hits || !p || !rgbt)
        return fail(c, BHR_ERR_INVALID_ARG, "bhr_trace_volumetric: NULL argument or no views");
    for (int k = 0; k < nviews; ++k) {
        const bhr_view& v = views[k];
        const std::string at = "bhr_trace_volumetric: view " + std::to_string(k);
        if (v.width <= 0 || v.height <= 0 || v.max_steps < 0)
            return fail(c, BHR_ERR_INVALID_ARG, at + ": width and height must be positive, max_steps >= 0");
        if (v.disk_mode != BHR_DISK_VOLUMETRIC)
            return fail(c, BHR_ERR_INVALID_ARG, at + ": disk_mode must be BHR_DISK_VOLUMETRIC (bhr_trace marches the others)");
        if (v.term_mode != BHR_TERM_SHADER && v.term_mode != BHR_TERM_CONFIG)
            return fail(c, BHR_ERR_UNSUPPORTED, at + ": the volumetric disk is marched under the SHADER or CONFIG rule");
        if (!(v.disk_step > 0.0f) || !(v.disk_thickness > 0.0f))
            return fail(c, BHR_ERR_INVALID_ARG, at + ": disk_step and disk_thickness must be positive");
        if (!hits[k] || !rgbt[k]) return fail(c, BHR_ERR_INVALID_ARG, at + ": NULL buffer");
        if (reinterpret_cast<uintptr_t>(hits[k]) % 16 != 0 || reinterpret_cast<uintptr_t>(rgbt[k]) % 16 != 0)
            return fail(c, BHR_ERR_INVALID_ARG, at + ": buffers must be 16-byte aligned");
    }
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(c->device);
    const cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    int rc = ensure_shade_resources(c, p->noise_seed, st);
    Fan fan;
    if (rc == BHR_OK) {
        const cudaError_t e = fan.open(c, st, nviews);
        if (e != cudaSuccess) rc = cuda_fail(c, e, "bhr_trace_volumetric: side streams");
    }
    for (int k = 0; k < nviews && rc == BHR_OK; ++k) {
        bhr::VolArgs a{};
        a.view = bhr::host::make_dev_view(views[k], hits[k]);
        a.rule = bhr::host::make_rule(views[k]);
        a.look = disk_look(c, *p, views[k]);
        a.rgbt = reinterpret_cast<float4*>(rgbt[k]);
        const cudaError_t e = bhr::launch_march_vol(a, fan.lane(k));
        if (e != cudaSuccess) rc = cuda_fail(c, e, "bhr_trace_volumetric: kernel launch");
    }
    {
        const cudaError_t e = fan.close();
        if (e != cudaSuccess && rc == BHR_OK) rc = cuda_fail(c, e, "bhr_trace_volumetric: side streams");
    }
    cudaSetDevice(prev);
    return rc;
}

int bhr_trace_bodies_volumetric(bhr_ctx* c, const bhr_view* view, const bhr_body* bodies, int nbodies,
                                const bhr_shade_params* p, bhr_hit* hits, bhr_body_hit* body_out, float* rgbt,
                                void* cuda_stream) {
    int rc = check_body_march(c, "bhr_trace_bodies_volumetric", view, bodies, nbodies, hits, body_out, true);
    if (rc != BHR_OK) return rc;
    if (!p || !rgbt) return fail(c, BHR_ERR_INVALID_ARG, "bhr_trace_bodies_volumetric: NULL argument");
    if (reinterpret_cast<uintptr_t>(rgbt) % 16 != 0)
        return fail(c, BHR_ERR_INVALID_ARG, "bhr_trace_bodies_volumetric: buffers must be 16-byte aligned");
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(c->device);
    const cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    rc = ensure_shade_resources(c, p->noise_seed, st);
    if (rc == BHR_OK) {
        bhr::BodyArgs a = body_args(*view, bodies, nbodies, hits, body_out);
        a.look = disk_look(c, *p, *view);
        a.rgbt = reinterpret_cast<float4*>(rgbt);
        const cudaError_t e = bhr::launch_march_bodies(a, true, st);
        if (e != cudaSuccess) rc = cuda_fail(c, e, "bhr_trace_bodies_volumetric");
    }
    cudaSetDevice(prev);
    return rc;
}

double bhr_shadow_angular_radius(double r) { return bhr::lens_alpha_crit(r); }

// ---------------------------------------------------------------------------------------
// launch shapes and the autotuner

int bhr_get_launch_shape(const bhr_ctx* c, bhr_launch_shape* sh) {
    if (!c || !sh) return fail(nullptr, BHR_ERR_INVALID_ARG, "bhr_get_launch_shape: NULL argument");
    *sh = c->shape;
    return BHR_OK;
}

int bhr_set_launch_shape(bhr_ctx* c, const bhr_launch_shape* sh) {
    if (!c || !sh) return fail(c, BHR_ERR_INVALID_ARG, "bhr_set_launch_shape: NULL argument");
    const int rc = check_shape(c, *sh);
    if (rc != BHR_OK) return rc;
    c->shape = *sh;
    if (c->shape.tile_w == 0) c->shape.tile_w = 32;
    return BHR_OK;
}

namespace {

std::string signature(const bhr_view* views, int nviews, int precision) {
    std::string k = "p" + std::to_string(precision);
    for (int i = 0; i < nviews; ++i) {
        const bhr_view& v = views[i];
        char buf[96];
        std::snprintf(buf, sizeof buf, "|%dx%d:%d:%d%d%d%d", v.width, v.height, v.max_steps, v.term_mode, v.disk_mode,
                      v.lensing, v.far_mode);
        k += buf;
    }
    return k;
}

// Median time of `reps` traces with shape `sh` after one warm-up (synchronous, stream st).
int time_shape(bhr_ctx* c, const bhr_launch_shape& sh, const bhr_view* views, int nviews, bhr_hit* const* out,
               int precision, int64_t rays, int reps, cudaStream_t st, cudaEvent_t e0, cudaEvent_t e1, float* ms) {
    std::vector<float> t;
    for (int r = 0; r <= reps; ++r) {
        cudaEventRecord(e0, st);
        int rc = run_trace(c, sh, c->scr, views, nviews, out, precision, rays, st, nullptr, nullptr);
        if (rc != BHR_OK) return rc;
        cudaEventRecord(e1, st);
        cudaError_t e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) return cuda_fail(c, e, "bhr_autotune");
        float x = 0.f;
        cudaEventElapsedTime(&x, e0, e1);
        if (r > 0) t.push_back(x);
    }
    std::sort(t.begin(), t.end());
    *ms = t[t.size() / 2];
    return BHR_OK;
}

}  // namespace

int bhr_autotune(bhr_ctx* c, const bhr_view* views, int nviews, bhr_hit* const* out_dev, int precision, int reps,
                 bhr_launch_shape* best) {
    if (!c) return fail(nullptr, BHR_ERR_INVALID_ARG, "bhr_autotune: ctx is NULL");
    int64_t rays = 0;
    int rc = validate(c, "bhr_autotune", views, nviews, out_dev, precision, &rays);
    if (rc != BHR_OK) return rc;
    reps = std::max(1, std::min(reps, 20));
    const std::string key = signature(views, nviews, precision);
    auto hit = c->tuned.find(key);
    if (hit != c->tuned.end()) {
        c->shape = hit->second;
        if (best) *best = hit->second;
        return BHR_OK;
    }
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(c->device);
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e != cudaSuccess) rc = cuda_fail(c, e, "bhr_autotune: stream / events");
    bhr_launch_shape top{512, 0, 64, 8, 32, 0.0f};
    float top_ms = 1e30f;
    auto trial = [&](bhr_launch_shape sh) {
        if (rc != BHR_OK) return;
        float ms = 0.f;
        rc = time_shape(c, sh, views, nviews, out_dev, precision, rays, reps, st, e0, e1, &ms);
        if (rc == BHR_OK && ms < top_ms) {
            top_ms = ms;
            sh.ms = ms;
            top = sh;
        }
    };
    // stage 1: block size x chunk (rows, refill 8)
    for (int block : {256, 512})
        for (int chunk : {32, 64, 128, 256}) trial(bhr_launch_shape{block, 0, chunk, 8, 32, 0.0f});
    // stage 2: refill threshold
    const bhr_launch_shape s1 = top;
    for (int refill : {4, 16, 24}) trial(bhr_launch_shape{s1.block_size, 0, s1.chunk, refill, 32, 0.0f});
    // stage 3: pixel tiles
    const bhr_launch_shape s2 = top;
    for (int tile : {16, 8}) trial(bhr_launch_shape{s2.block_size, 0, s2.chunk, s2.refill, tile, 0.0f});
    // stage 4: fewer resident blocks (less contention for the work queue and L1)
    const bhr_launch_shape s3 = top;
    if (rc == BHR_OK) {
        const int variant = bhr::rule_variant(make_rule(views[0]));
        const int fit = bhr::march_blocks_per_sm(s3.block_size, variant, nviews > 1, precision == BHR_PREC_MIXED);
        if (fit > 1) trial(bhr_launch_shape{s3.block_size, fit - 1, s3.chunk, s3.refill, s3.tile_w, 0.0f});
    }
    if (st) cudaStreamDestroy(st);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaSetDevice(prev);
    if (rc != BHR_OK) return rc;
    c->shape = top;
    c->tuned[key] = top;
    if (best) *best = top;
    return BHR_OK;
}

// ---------------------------------------------------------------------------------------
// plans

namespace {

int plan_capture(bhr_plan* p, cudaGraph_t* g) {
    bhr_ctx* c = p->ctx;
    int64_t rays = 0;
    for (const bhr_view& v : p->views) rays += int64_t(v.width) * v.height;
    cudaError_t e = cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(c, e, "bhr_plan: begin capture");
    int rc = run_trace(c, p->shape, p->scr, p->views.data(), int(p->views.size()), p->out.data(), p->precision, rays,
                       p->cap, &p->slots, &p->batches);
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(p->cap, &graph);
    if (rc != BHR_OK) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (e != cudaSuccess) return cuda_fail(c, e, "bhr_plan: end capture");
    *g = graph;
    return BHR_OK;
}

}  // namespace

int bhr_plan_create(bhr_ctx* c, const bhr_view* views, int nviews, bhr_hit* const* out_dev, int precision,
                    int autotune, bhr_plan** out) {
    if (!c || !out) return fail(c, BHR_ERR_INVALID_ARG, "bhr_plan_create: NULL argument");
    *out = nullptr;
    int64_t rays = 0;
    int rc = validate(c, "bhr_plan_create", views, nviews, out_dev, precision, &rays);
    if (rc != BHR_OK) return rc;
    if (autotune) {
        rc = bhr_autotune(c, views, nviews, out_dev, precision, 3, nullptr);
        if (rc != BHR_OK) return rc;
    }
    bhr_plan* p = new (std::nothrow) bhr_plan();
    if (!p) return fail(c, BHR_ERR_OOM, "bhr_plan_create: out of host memory");
    p->ctx = c;
    p->views.assign(views, views + nviews);
    p->out.assign(out_dev, out_dev + nviews);
    p->precision = precision;
    p->shape = c->shape;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(c->device);
    cudaError_t e = cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking);
    if (e != cudaSuccess) rc = cuda_fail(c, e, "bhr_plan_create: stream");
    // one eager trace on the plan's own scratch: allocates it, sets kernel attributes and
    // checks every launch before anything is captured
    if (rc == BHR_OK)
        rc = run_trace(c, p->shape, p->scr, views, nviews, out_dev, precision, rays, p->cap, &p->slots, &p->batches);
    if (rc == BHR_OK) {
        e = cudaStreamSynchronize(p->cap);
        if (e != cudaSuccess) rc = cuda_fail(c, e, "bhr_plan_create: first trace");
    }
    if (rc == BHR_OK) rc = plan_capture(p, &p->graph);
    if (rc == BHR_OK) {
        e = cudaGraphInstantiate(&p->exec, p->graph, 0);
        if (e != cudaSuccess) rc = cuda_fail(c, e, "bhr_plan_create: instantiate");
    }
    cudaSetDevice(prev);
    if (rc != BHR_OK) {
        bhr_plan_destroy(p);
        return rc;
    }
    *out = p;
    return BHR_OK;
}

int bhr_plan_update(bhr_plan* p, const bhr_view* views, int nviews) {
    if (!p) return fail(nullptr, BHR_ERR_INVALID_ARG, "bhr_plan_update: plan is NULL");
    bhr_ctx* c = p->ctx;
    if (!views || nviews != int(p->views.size()))
        return fail(c, BHR_ERR_INVALID_ARG, "bhr_plan_update: the view count must stay the same");
    for (int k = 0; k < nviews; ++k) {
        const int rc = check_view(c, views[k], k);
        if (rc != BHR_OK) return rc;
        const bhr_view& o = p->views[size_t(k)];
        if (views[k].width != o.width || views[k].height != o.height ||
            !same_rule(make_rule(views[k]), make_rule(o)))
            return fail(c, BHR_ERR_INVALID_ARG, "bhr_plan_update: view " + std::to_string(k) +
                                                    " changes its size or rule; create a new plan");
    }
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(c->device);
    const std::vector<bhr_view> old = p->views;
    p->views.assign(views, views + nviews);
    cudaGraph_t g = nullptr;
    int rc = plan_capture(p, &g);
    if (rc == BHR_OK) {
        cudaGraphExecUpdateResultInfo info{};
        cudaError_t e = cudaGraphExecUpdate(p->exec, g, &info);
        if (e != cudaSuccess) {
            // topology changed (should not happen for same sizes and rules): instantiate afresh
            cudaGetLastError();
            cudaGraphExec_t x = nullptr;
            e = cudaGraphInstantiate(&x, g, 0);
            if (e == cudaSuccess) {
                cudaGraphExecDestroy(p->exec);
                p->exec = x;
            } else {
                rc = cuda_fail(c, e, "bhr_plan_update: instantiate");
            }
        }
    }
    if (rc == BHR_OK) {
        if (p->graph) cudaGraphDestroy(p->graph);
        p->graph = g;
    } else {
        if (g) cudaGraphDestroy(g);
        p->views = old;
    }
    cudaSetDevice(prev);
    return rc;
}

int bhr_plan_launch(bhr_plan* p, void* cuda_stream) {
    if (!p || !p->exec) return fail(nullptr, BHR_ERR_INVALID_ARG, "bhr_plan_launch: plan is NULL or empty");
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(p->ctx->device);
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    cudaError_t e = cudaGraphLaunch(p->exec, st);
    cudaSetDevice(prev);
    if (e != cudaSuccess) return cuda_fail(p->ctx, e, "bhr_plan_launch");
    p->last_stream = st;
    p->launched = true;
    return BHR_OK;
}

int bhr_plan_launch_shape(const bhr_plan* p, bhr_launch_shape* sh) {
    if (!p || !sh) return fail(nullptr, BHR_ERR_INVALID_ARG, "bhr_plan_launch_shape: NULL argument");
    *sh = p->shape;
    return BHR_OK;
}

int bhr_plan_stats(bhr_plan* p, bhr_stats* s) {
    if (!p || !s) return fail(nullptr, BHR_ERR_INVALID_ARG, "bhr_plan_stats: NULL argument");
    if (!p->launched) return fail(p->ctx, BHR_ERR_NOT_READY, "bhr_plan_stats: the plan was not launched yet");
    std::vector<bhr::WorkQueue> qs;
    const int rc = read_queues(p->ctx, p->scr, p->batches, p->last_stream, &qs, "bhr_plan_stats");
    if (rc != BHR_OK) return rc;
    int64_t rays = 0;
    for (const bhr_view& v : p->views) rays += int64_t(v.width) * v.height;
    sum_stats(qs, rays, s);
    return BHR_OK;
}

int bhr_plan_view_times(bhr_plan* p, double* ms, int nviews) {
    if (!p || !ms || nviews != int(p->views.size()))
        return fail(p ? p->ctx : nullptr, BHR_ERR_INVALID_ARG, "bhr_plan_view_times: bad argument");
    if (!p->launched || nviews == 1)
        return fail(p->ctx, BHR_ERR_NOT_READY, "bhr_plan_view_times: needs a launched multi-view plan");
    std::vector<bhr::WorkQueue> qs;
    const int rc = read_queues(p->ctx, p->scr, p->batches, p->last_stream, &qs, "bhr_plan_view_times");
    if (rc != BHR_OK) return rc;
    view_times(qs, p->slots, ms, nviews);
    return BHR_OK;
}

int bhr_plan_destroy(bhr_plan* p) {
    if (!p) return BHR_OK;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(p->ctx->device);
    if (p->launched && p->last_stream) cudaStreamSynchronize(p->last_stream);
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    if (p->cap) {
        cudaStreamSynchronize(p->cap);
        cudaStreamDestroy(p->cap);
    }
    p->scr.release();
    cudaSetDevice(prev);
    delete p;
    return BHR_OK;
}

}  // extern "C"
