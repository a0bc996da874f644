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
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "bhr.h"
#include "host_views.h"
#include "kernels.cuh"

struct bhr_ctx {
    int device = 0;
    int sms = 0;
    int block = 512;        // threads per block of the FP32 march
    int blocks_per_sm = 0;  // 0: as many as fit
    int chunk = 64;         // rays per work chunk
    int refill = 8;         // idle lanes that trigger a refill
    bhr::WorkQueue* q = nullptr;  // one per batch slot
    int nq = 0;
    int2* band = nullptr;
    bhr::PromoEntry* promo = nullptr;
    int64_t scratch_rays = 0;  // capacity of band / promo in rays
    // bhr_trace_host: device staging (two halves) and two streams, created on first use
    bhr_hit* staging = nullptr;
    int64_t staging_rays = 0;  // rays per half
    cudaStream_t hstream[2] = {nullptr, nullptr};
    cudaStream_t last_stream = nullptr;
    int last_batches = 0;
    std::vector<std::pair<int, int>> last_slots;  // (work queue, view slot) per view of the last trace
    int last_nviews = 0;
    bool have_last = false;
    std::string err;
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

int ensure_scratch(bhr_ctx* c, int nbatches, int64_t rays, bool mixed) {
    if (nbatches > c->nq) {
        if (c->q) cudaFree(c->q);
        c->q = nullptr;
        c->nq = 0;
        cudaError_t e = cudaMalloc(&c->q, sizeof(bhr::WorkQueue) * size_t(nbatches));
        if (e != cudaSuccess) return fail(c, BHR_ERR_OOM, std::string("work queue: ") + cudaGetErrorString(e));
        c->nq = nbatches;
    }
    if (mixed && rays > c->scratch_rays) {
        if (c->band) cudaFree(c->band);
        if (c->promo) cudaFree(c->promo);
        c->band = nullptr;
        c->promo = nullptr;
        c->scratch_rays = 0;
        cudaError_t e = cudaMalloc(&c->band, sizeof(int2) * size_t(rays));
        if (e == cudaSuccess) e = cudaMalloc(&c->promo, sizeof(bhr::PromoEntry) * size_t(rays));
        if (e != cudaSuccess) return fail(c, BHR_ERR_OOM, std::string("FP64 queue: ") + cudaGetErrorString(e));
        c->scratch_rays = rays;
    }
    return BHR_OK;
}

bhr::LaunchCfg make_cfg(const bhr_ctx* c, int variant, bool multi, bool mixed) {
    bhr::LaunchCfg cfg{};
    cfg.block = c->block;
    cfg.variant = variant;
    const int fit = std::max(1, bhr::march_blocks_per_sm(cfg.block, variant, multi, mixed));
    const int bps = c->blocks_per_sm > 0 ? std::min(c->blocks_per_sm, fit) : fit;
    cfg.grid = c->sms * bps;
    cfg.refill = std::max(1, std::min(c->refill, 32));
    cfg.chunk = std::max(32, c->chunk);
    return cfg;
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
        if (opts->block_size == 256 || opts->block_size == 512) {
            c->block = opts->block_size;
        } else if (opts->block_size != 0) {
            cudaSetDevice(prev);
            delete c;
            return fail(nullptr, BHR_ERR_INVALID_ARG, "bhr_create: block_size must be 0, 256 or 512");
        }
        if (opts->chunk > 0) c->chunk = opts->chunk;
        if (opts->refill > 0) c->refill = opts->refill;
        if (opts->blocks_per_sm > 0) c->blocks_per_sm = opts->blocks_per_sm;
    }
    const int rc = ensure_scratch(c, 1, 0, false);
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
    if (c->q) cudaFree(c->q);
    if (c->band) cudaFree(c->band);
    if (c->promo) cudaFree(c->promo);
    if (c->staging) cudaFree(c->staging);
    for (cudaStream_t& st : c->hstream)
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

int bhr_view_look_at(bhr_view* v, const double pos[3], const double target[3]) {
    if (!v || !pos || !target) return fail(nullptr, BHR_ERR_INVALID_ARG, "bhr_view_look_at: NULL argument");
    // Camera.cpp:12-23 lookRotation(from, target, up = (0,1,0)), then basis() = mat3_cast(quat)
    const double fd[3] = {target[0] - pos[0], target[1] - pos[1], target[2] - pos[2]};
    const double len = std::sqrt(fd[0] * fd[0] + fd[1] * fd[1] + fd[2] * fd[2]);
    float f[3] = {0.0f, 0.0f, -1.0f};
    if (len > 0.0)
        for (int k = 0; k < 3; ++k) f[k] = float(fd[k] / len);
    float u[3] = {0.0f, 1.0f, 0.0f};
    if (std::fabs(f[0] * u[0] + f[1] * u[1] + f[2] * u[2]) > 0.999f) {
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
    qw *= qn; qx *= qn; qy *= qn; qz *= qn;
    // quaternion -> rotation matrix (columns right, up, back)
    const float xx = qx * qx, yy = qy * qy, zz = qz * qz, xz = qx * qz, xy = qx * qy, yz = qy * qz;
    const float wx = qw * qx, wy = qw * qy, wz = qw * qz;
    float* B = v->cam_basis;
    B[0] = 1.0f - 2.0f * (yy + zz); B[1] = 2.0f * (xy + wz);        B[2] = 2.0f * (xz - wy);
    B[3] = 2.0f * (xy - wz);        B[4] = 1.0f - 2.0f * (xx + zz); B[5] = 2.0f * (yz + wx);
    B[6] = 2.0f * (xz + wy);        B[7] = 2.0f * (yz - wx);        B[8] = 1.0f - 2.0f * (xx + yy);
    // uCamPos = vec3(Camera::position())
    for (int k = 0; k < 3; ++k) v->cam_pos[k] = float(pos[k]);
    return BHR_OK;
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
    if (!views || nviews <= 0 || !out_dev) return fail(c, BHR_ERR_INVALID_ARG, "bhr_trace: no views or outputs");
    if (precision != BHR_PREC_FP32 && precision != BHR_PREC_MIXED)
        return fail(c, BHR_ERR_INVALID_ARG, "bhr_trace: unknown precision");
    if (method != BHR_METHOD_PLAIN && method != BHR_METHOD_SURROGATE)
        return fail(c, BHR_ERR_INVALID_ARG, "bhr_trace: unknown method");
    if (method == BHR_METHOD_SURROGATE)
        return fail(c, BHR_ERR_NOT_READY, "bhr_trace: the surrogate runs through bhr_surrogate_trace");
    int64_t rays = 0;
    for (int k = 0; k < nviews; ++k) {
        const int rc = check_view(c, views[k], k);
        if (rc != BHR_OK) return rc;
        if (!out_dev[k]) return fail(c, BHR_ERR_INVALID_ARG, "bhr_trace: output buffer " + std::to_string(k) + " is NULL");
        if (reinterpret_cast<uintptr_t>(out_dev[k]) % 16 != 0)
            return fail(c, BHR_ERR_INVALID_ARG, "bhr_trace: output buffers must be 16-byte aligned");
        rays += int64_t(views[k].width) * views[k].height;
    }
    const bool mixed = precision == BHR_PREC_MIXED;
    // group views by rule (one launch per group and per kMaxViews views)
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
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(c->device);
    int rc = ensure_scratch(c, nb, rays, mixed);
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    const int fp64_grid = c->sms * 8;
    int bi = 0;
    std::vector<std::pair<int, int>> slots(size_t(nviews), {0, 0});
    for (size_t g = 0; rc == BHR_OK && g < groups.size(); ++g) {
        const bhr::Rule& rule = rules[g];
        const int variant = bhr::rule_variant(rule);
        const std::vector<int>& members = groups[g];
        for (size_t m0 = 0; rc == BHR_OK && m0 < members.size(); m0 += bhr::kMaxViews, ++bi) {
            bhr::Scratch sc{c->q + bi, c->band, c->promo};
            cudaError_t e = cudaMemsetAsync(sc.q, 0, sizeof(bhr::WorkQueue), st);
            if (e != cudaSuccess) {
                rc = cuda_fail(c, e, "bhr_trace: cudaMemsetAsync");
                break;
            }
            const size_t nv = std::min<size_t>(bhr::kMaxViews, members.size() - m0);
            if (nviews == 1) {
                const bhr::DevView dv = make_dev_view(views[0], out_dev[0]);
                e = bhr::launch_march_one(dv, rule, sc, mixed, make_cfg(c, variant, false, mixed), st);
                if (e == cudaSuccess && mixed) e = bhr::launch_march_fp64_one(dv, rule, sc, fp64_grid, st);
            } else {
                static thread_local bhr::ViewBatch b;  // ~12 KB, passed by value as a kernel parameter
                const bhr::LaunchCfg cfg = make_cfg(c, variant, true, mixed);
                b.nviews = int(nv);
                b.rule = rule;
                int64_t chunk_acc = 0;
                for (size_t k = 0; k < nv; ++k) {
                    const int vi = members[m0 + k];
                    slots[size_t(vi)] = {bi, int(k)};
                    b.views[k] = make_dev_view(views[vi], out_dev[vi]);
                    b.views[k].chunk_start = chunk_acc;
                    chunk_acc += (b.views[k].nrays + cfg.chunk - 1) / cfg.chunk;
                }
                b.total_chunks = chunk_acc;
                e = bhr::launch_march_multi(b, sc, mixed, cfg, st);
                if (e == cudaSuccess && mixed) e = bhr::launch_march_fp64_multi(b, sc, fp64_grid, st);
            }
            if (e != cudaSuccess) rc = cuda_fail(c, e, "bhr_trace: kernel launch");
        }
    }
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
    if (!c->have_last) return fail(c, BHR_ERR_NOT_READY, "bhr_trace_stats: no trace on this context yet");
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(c->device);
    cudaError_t e = cudaStreamSynchronize(c->last_stream);
    std::vector<bhr::WorkQueue> qs(size_t(c->last_batches));
    if (e == cudaSuccess)
        e = cudaMemcpy(qs.data(), c->q, sizeof(bhr::WorkQueue) * qs.size(), cudaMemcpyDeviceToHost);
    cudaSetDevice(prev);
    if (e != cudaSuccess) return cuda_fail(c, e, "bhr_trace_stats");
    for (const auto& q : qs) {
        s->steps += q.steps;
        s->fp64_rays += q.fp64_rays;
        s->fp64_steps += q.fp64_steps;
        s->nonfinite += q.nonfinite;
    }
    return BHR_OK;
}

int bhr_trace_view_times(bhr_ctx* c, double* ms, int nviews) {
    if (!c || !ms || nviews <= 0) return fail(c, BHR_ERR_INVALID_ARG, "bhr_trace_view_times: bad argument");
    if (!c->have_last || c->last_nviews != nviews || nviews == 1)
        return fail(c, BHR_ERR_NOT_READY, "bhr_trace_view_times: needs the last trace to be a multi-view trace");
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(c->device);
    cudaError_t e = cudaStreamSynchronize(c->last_stream);
    std::vector<bhr::WorkQueue> qs(size_t(c->last_batches));
    if (e == cudaSuccess)
        e = cudaMemcpy(qs.data(), c->q, sizeof(bhr::WorkQueue) * qs.size(), cudaMemcpyDeviceToHost);
    cudaSetDevice(prev);
    if (e != cudaSuccess) return cuda_fail(c, e, "bhr_trace_view_times");
    for (int k = 0; k < nviews; ++k) {
        const bhr::WorkQueue& q = qs[size_t(c->last_slots[size_t(k)].first)];
        const int s = c->last_slots[size_t(k)].second;
        ms[k] = q.view_t_end[s] >= q.t_start ? double(q.view_t_end[s] - q.t_start) * 1e-6 : -1.0;
    }
    return BHR_OK;
}

}  // extern "C"
