// View validation and the host-side view/rule conversion shared by the C ABI entry points.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>

#include "bhr.h"
#include "march.cuh"

namespace bhr {
namespace host {

inline bool finite3f(const float* a) { return std::isfinite(a[0]) && std::isfinite(a[1]) && std::isfinite(a[2]); }

// blackhole.frag:89: rEscMin = max(uDiskOuter * 1.25, 12.0)
inline float shader_r_esc_min(float disk_outer) { return std::max(disk_outer * 1.25f, 12.0f); }

// BHR_OK, or an error code with its message in *msg.
inline int check_view(const bhr_view& v, int k, std::string* msg) {
    auto bad = [&](const char* what) {
        *msg = "view " + std::to_string(k) + ": " + what;
        return BHR_ERR_INVALID_ARG;
    };
    if (v.width <= 0 || v.height <= 0) return bad("width and height must be positive");
    if (int64_t(v.width) * v.height > int64_t(INT32_MAX)) return bad("width * height exceeds 2^31 - 1 rays");
    if (v.max_steps < 0) return bad("max_steps must be >= 0");
    if (v.disk_mode == BHR_DISK_VOLUMETRIC)
    {
        *msg = "view " + std::to_string(k) + ": volumetric disk is not supported";
        return BHR_ERR_UNSUPPORTED;
    }
    if (v.disk_mode != BHR_DISK_NONE && v.disk_mode != BHR_DISK_THIN) return bad("unknown disk_mode");
    if (v.term_mode < BHR_TERM_SHADER || v.term_mode > BHR_TERM_CPU) return bad("unknown term_mode");
    if (!finite3f(v.cam_pos)) return bad("camera position is not finite");
    for (float e : v.cam_basis)
        if (!std::isfinite(e)) return bad("camera basis is not finite");
    if (!(v.tan_half_fov > 0.0f) || !std::isfinite(v.tan_half_fov)) return bad("tan_half_fov must be positive");
    if (!(v.step_scale > 0.0f) || !(v.ds_floor >= 0.0f)) return bad("step_scale must be > 0 and ds_floor >= 0");
    const float rc = std::sqrt(v.cam_pos[0] * v.cam_pos[0] + v.cam_pos[1] * v.cam_pos[1] + v.cam_pos[2] * v.cam_pos[2]);
    if (!(rc > 0.0f)) return bad("camera at the origin");
    return BHR_OK;
}

// setTraceUniforms (Renderer.cpp:242-356) + the per-ray constants of blackhole.frag:77-89 that
// depend only on the view, in float with the reference's operation order.
// tile_w: pixel width of the tile a warp's 32 consecutive work items cover (32, 16 or 8).
inline DevView make_dev_view(const bhr_view& v, bhr_hit* out, int tile_w = 32) {
    DevView d{};
    for (int k = 0; k < 3; ++k) d.cam[k] = v.cam_pos[k];
    for (int k = 0; k < 9; ++k) d.basis[k] = v.cam_basis[k];
    d.tan_half = v.tan_half_fov;
    d.jitter[0] = v.jitter[0];
    d.jitter[1] = v.jitter[1];
    d.width = v.width;
    d.height = v.height;
    d.max_steps = v.max_steps;
    d.aspect = float(v.width) / float(v.height);
    const float* p = v.cam_pos;
    d.rcam = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
    for (int k = 0; k < 3; ++k) d.rhat[k] = p[k] / d.rcam;
    d.lapse = std::sqrt(std::max(1.0f - 2.0f / d.rcam, 0.0f));
    d.baxis_scale = 1.0f / std::sqrt(std::max(1.0f - 2.0f / d.rcam, 1e-6f));
    d.two_over_r3 = 2.0f / (d.rcam * d.rcam * d.rcam);
    d.step_scale = v.step_scale;
    d.disk_step = v.disk_step;
    for (int k = 0; k < 3; ++k) d.cam_d[k] = double(v.cam_pos[k]);
    d.chunk_start = 0;
    d.nrays = int64_t(v.width) * v.height;
    d.tile_shift = tile_w == 16 ? 4 : (tile_w == 8 ? 3 : 5);
    if (d.tile_shift == 5) {
        d.tiles_x = 0;
        d.work = d.nrays;
    } else {
        const int tw = 1 << d.tile_shift, th = 32 >> d.tile_shift;
        d.tiles_x = (v.width + tw - 1) / tw;
        d.work = int64_t(d.tiles_x) * ((v.height + th - 1) / th) * 32;
    }
    d.out = out;
    return d;
}

// The launch-wide constants of a view: termination rule and disk geometry.
inline Rule make_rule(const bhr_view& v) {
    Rule r{};
    r.capture_r = v.capture_r;
    r.escape_r = v.escape_r;
    r.esc_tol = v.esc_tol;
    r.r_esc_min = v.term_mode == BHR_TERM_SHADER ? shader_r_esc_min(v.disk_outer) : v.r_esc_min;
    r.ds_floor = v.ds_floor;
    r.slab = 2.5f * v.disk_thickness;
    const float lo = v.disk_inner - 1.0f, hi = v.disk_outer + 1.0f;
    r.rcyl_lo2 = lo > 0.0f ? lo * lo : -1.0f;
    r.rcyl_hi2 = hi > 0.0f ? hi * hi : -1.0f;
    r.disk_inner = v.disk_inner;
    r.disk_outer = v.disk_outer;
    r.promote_r = v.promote_r;
    r.promote_band = v.promote_band;
    r.term_mode = v.term_mode;
    r.disk_mode = v.disk_mode;
    r.lensing = (v.lensing != 0 && v.far_mode == 0) ? 1 : 0;
    r.far_mode = v.far_mode != 0 ? 1 : 0;
    return r;
}

}  // namespace host

// Records msg as the last error reported by bhr_last_error(NULL) (defined in api.cu).
void set_last_error(const std::string& msg);

}  // namespace bhr
