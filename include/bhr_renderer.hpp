// bhr_renderer.hpp - C++ host interface of the GB300 tracer, shaped like the reference
// renderer's call surface for the traced path:
//
//   reference (DeepjotG/BlackHoleRender)            here
//   bhs::Settings trace fields (src/Settings.h)      bhr::Settings
//   bhs::Settings::applyPreset (Settings.cpp:12-35)  bhr::Settings::applyPreset
//   bhs::Camera pose, lookAt, basis (Camera.h)       bhr::Camera
//   bhs::FrameInput{camera, settings, windowW/H,     bhr::FrameInput (the fields the trace reads)
//     farMode} (src/Renderer.h:24-53)
//   bhs::Renderer::init / shutdown / render          bhr::Renderer::init / shutdown / render
//     (src/Renderer.h:58-61)
//   Renderer::setTraceUniforms (Renderer.cpp:242-356) bhr::Renderer::makeView, makeShadeParams
//   the frame's colour (blackhole.frag's fragColor)  bhr::Renderer::renderImage (bhr_shade)
//   (no counterpart: the learned orbit surrogate)    Settings::surrogate, Renderer::loadSurrogate
//
// render() traces the frame into hit records the Renderer owns (as the reference's renderer
// owns its targets, Renderer.cpp:125-145); renderTo() writes caller-owned device records on a
// caller stream; renderHost() returns host records; renderImage() traces and shades the frame
// into a float4 image the Renderer owns (the sky cube's term left to the caller, its weight in
// alpha). The internal resolution follows
// Renderer::render (Renderer.cpp:667-669): max(16, lround(window * clamp(renderScale, 0.1, 2)))
// (the reference's dynamic-resolution factor is a frame-time controller of the GL pipeline
// and is not part of this path). Errors follow the reference's convention: a bool result and
// a log line (logError, src/Log.h:23-28), never an exception across the library boundary.
//
// Header-only over the C ABI in bhr.h; link with -lbhr -lcudart.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <functional>
#include <string>
#include <vector>

#include "bhr.h"

namespace bhr {

enum DiskMode : int { DISK_NONE = 0, DISK_THIN = 1, DISK_VOLUMETRIC = 2 };
enum Preset : int { PRESET_LOW = 0, PRESET_MEDIUM = 1, PRESET_HIGH = 2, PRESET_ULTRA = 3, PRESET_CUSTOM = 4 };

// The traced fields of the reference's Settings (those it marks BHS_TRACE, Settings.cpp:76-88),
// with its defaults: the volumetric disk at the High preset.
struct Settings {
    int preset = PRESET_HIGH;
    float renderScale = 1.0f;
    int maxSteps = 450;
    float stepScale = 0.05f;
    float diskStep = 0.18f;
    int diskMode = DISK_VOLUMETRIC;
    bool lensing = true;
    float diskInner = 6.0f;
    float diskOuter = 20.0f;
    float diskThickness = 0.035f;
    float fovDeg = 60.0f;
    // shading fields (Settings.h:32-55)
    float dopplerStrength = 0.0f;
    float diskDensity = 1.0f;
    float diskOpacity = 2.0f;
    float diskPeakTemp = 6000.0f;
    float diskBrightness = 5.5f;
    float diskNoiseScale = 1.0f;
    float diskNoiseStrength = 0.85f;
    float diskWarmth = 0.4f;
    float starDensity = 1.0f;
    float starBrightness = 1.0f;
    float skyBrightness = 1.0f;
    bool showShadowOverlay = false;
    // GB300 addition, no field of the reference: trace with the learned orbit surrogate
    // (Renderer::loadSurrogate) where it answers, the plain march elsewhere.
    bool surrogate = false;

    // Quality presets (Settings.cpp:12-35); PRESET_CUSTOM leaves the fields alone.
    void applyPreset(int p) {
        preset = p;
        switch (p) {
            case PRESET_LOW: maxSteps = 200; stepScale = 0.10f; diskStep = 0.35f; break;
            case PRESET_MEDIUM: maxSteps = 300; stepScale = 0.07f; diskStep = 0.30f; break;
            case PRESET_HIGH: maxSteps = 450; stepScale = 0.05f; diskStep = 0.18f; break;
            case PRESET_ULTRA: maxSteps = 700; stepScale = 0.035f; diskStep = 0.10f; break;
            default: break;
        }
    }
};

struct Vec3d {
    double x = 0.0, y = 0.0, z = 0.0;
};
struct Quat {  // unit quaternion, GLM order of meaning (w, x, y, z)
    float w = 1.0f, x = 0.0f, y = 0.0f, z = 0.0f;
};

// Camera pose in the renderer frame (hole at the origin, +Y up the spin axis, lengths in M),
// position in double as in the reference. The flight controls of bhs::Camera are UI, not
// part of this path.
class Camera {
public:
    Camera() { lookAt(Vec3d{0.0, 0.0, 0.0}); }  // the "Interstellar shot" bookmark (Camera.cpp:54-55)

    void lookAt(const Vec3d& target, const float up[3] = nullptr) {
        const double p[3] = {pos_.x, pos_.y, pos_.z}, t[3] = {target.x, target.y, target.z};
        float q[4];
        if (bhr_look_rotation(p, t, up, q) == BHR_OK) orient_ = Quat{q[0], q[1], q[2], q[3]};
    }
    void setPose(const Vec3d& pos, const Quat& orient) {
        pos_ = pos;
        orient_ = orient;
    }
    void setPosition(const Vec3d& pos) { pos_ = pos; }
    Vec3d position() const { return pos_; }
    Quat orientation() const { return orient_; }
    double radius() const { return std::sqrt(pos_.x * pos_.x + pos_.y * pos_.y + pos_.z * pos_.z); }
    // columns right, up, back (column-major 3x3, as glm::mat3_cast)
    void basis(float out[9]) const {
        bhr_view v{};
        const double p[3] = {pos_.x, pos_.y, pos_.z};
        const float q[4] = {orient_.w, orient_.x, orient_.y, orient_.z};
        bhr_view_set_pose(&v, p, q);
        std::copy(v.cam_basis, v.cam_basis + 9, out);
    }

private:
    Vec3d pos_{0.0, 2.6, 24.9};
    Quat orient_{};
};

// The fields of the reference's FrameInput that the traced path reads.
struct FrameInput {
    const Camera* camera = nullptr;
    const Settings* settings = nullptr;
    int windowW = 0, windowH = 0;
    bool farMode = false;            // camera far from the hole: straight rays (App.cpp:506)
    int termMode = BHR_TERM_SHADER;  // BHR_TERM_*: the shader's own rule by default
    float jitter[2] = {0.0f, 0.0f};  // sub-pixel offset of accumulated frames (0 for parity)
    float diskTime = 0.0f;           // disk flow clock in M, [0, 60) (App.cpp:458-459)
    float diskFade = 1.0f;           // steady disk's fade (1 = shown; <= 0.01 = not marched)
    float time = 0.0f;               // seconds since start (uTime: clouds and stars of bodies)
    const std::vector<bhr_body>* bodies = nullptr;  // packBodies output (Renderer.h:43): the BHS_BODIES variant
};

class Renderer {
public:
    using LogFn = std::function<void(const std::string&)>;

    Renderer() = default;
    Renderer(const Renderer&) = delete;
    Renderer& operator=(const Renderer&) = delete;
    ~Renderer() { shutdown(); }

    void setLogger(LogFn fn) { log_ = std::move(fn); }

    bool init(int device = 0, const bhr_options* opts = nullptr) {
        if (ctx_) return true;
        bhr_options o{};
        if (opts) o = *opts;
        o.device = device;
        if (bhr_create(&ctx_, &o) != BHR_OK) return logError("bhr_create", nullptr);
        device_ = device;
        return true;
    }

    // Loads a surrogate checkpoint (bhr_surrogate_save) onto the Renderer's device and binds it
    // to the context; frames whose Settings ask for the surrogate then trace with it.
    bool loadSurrogate(const char* path) {
        if (!ctx_ && !init(device_)) return false;
        if (!surr_ && bhr_surrogate_create(&surr_, device_, nullptr, 1) != BHR_OK)
            return logError("loadSurrogate: create", nullptr);
        if (bhr_surrogate_load(surr_, path) != BHR_OK) return logError("loadSurrogate", nullptr);
        if (bhr_ctx_set_surrogate(ctx_, surr_) != BHR_OK) return logError("loadSurrogate", ctx_);
        return true;
    }
    bhr_surrogate* surrogate() const { return surr_; }

    void shutdown() {
        if (ctx_) bhr_ctx_set_surrogate(ctx_, nullptr);
        if (surr_) {
            bhr_surrogate_destroy(surr_);
            surr_ = nullptr;
        }
        if (body_hits_) {
            cudaFree(body_hits_);
            body_hits_ = nullptr;
            body_capacity_ = 0;
        }
        if (image_) {
            cudaFree(image_);
            image_ = nullptr;
            image_capacity_ = 0;
        }
        if (records_) {
            cudaFree(records_);
            records_ = nullptr;
            capacity_ = 0;
        }
        if (ctx_) {
            bhr_destroy(ctx_);
            ctx_ = nullptr;
        }
    }

    // The internal trace resolution of a frame (Renderer.cpp:667-669 with dynamic scale 1).
    static void internalSize(const FrameInput& in, int* w, int* h) {
        const float scale = std::clamp(in.settings ? in.settings->renderScale : 1.0f, 0.1f, 2.0f);
        *w = std::max(16, static_cast<int>(std::lround(in.windowW * scale)));
        *h = std::max(16, static_cast<int>(std::lround(in.windowH * scale)));
    }

    // setTraceUniforms (Renderer.cpp:242-356) for the traced fields: FrameInput -> bhr_view.
    static bool makeView(const FrameInput& in, bhr_view* v) {
        if (!in.camera || !in.settings || !v || in.windowW <= 0 || in.windowH <= 0) return false;
        const Settings& s = *in.settings;
        if (bhr_view_init(v, in.termMode) != BHR_OK) return false;
        internalSize(in, &v->width, &v->height);
        if (bhr_view_set_fov(v, s.fovDeg) != BHR_OK) return false;
        const Vec3d p = in.camera->position();
        const Quat q = in.camera->orientation();
        const double pos[3] = {p.x, p.y, p.z};
        const float quat[4] = {q.w, q.x, q.y, q.z};
        bhr_view_set_pose(v, pos, quat);
        v->jitter[0] = in.jitter[0];
        v->jitter[1] = in.jitter[1];
        if (in.termMode != BHR_TERM_CPU) {
            v->max_steps = s.maxSteps;
            v->step_scale = s.stepScale;
            v->disk_step = s.diskStep;
            v->disk_mode = s.diskMode;
        }
        v->disk_inner = s.diskInner;
        v->disk_outer = s.diskOuter;
        v->disk_thickness = s.diskThickness;
        v->lensing = s.lensing ? 1 : 0;
        v->far_mode = in.farMode ? 1 : 0;
        if (in.diskFade <= 0.01f) v->disk_mode = BHR_DISK_NONE;  // the faded disk is not marched (Renderer.cpp:327)
        if (in.termMode == BHR_TERM_SHADER)  // rEscMin = max(1.25 r_out, 12) (blackhole.frag:89)
            v->r_esc_min = std::max(1.25f * s.diskOuter, 12.0f);
        return true;
    }

    // The shading uniforms of setTraceUniforms (Renderer.cpp:316-346) for the steady disk: its
    // opacity and brightness scaled by the fade.
    static bool makeShadeParams(const FrameInput& in, bhr_shade_params* p) {
        if (!in.settings || !p || bhr_shade_default_params(p) != BHR_OK) return false;
        const Settings& s = *in.settings;
        const float strength = std::clamp(in.diskFade, 0.0f, 1.0f);
        p->disk_density = s.diskDensity;
        p->disk_opacity = s.diskOpacity * strength;
        p->disk_peak_temp = s.diskPeakTemp;
        p->disk_brightness = s.diskBrightness * strength;
        p->disk_noise_scale = s.diskNoiseScale;
        p->disk_noise_strength = s.diskNoiseStrength;
        p->disk_time = in.diskTime;
        p->disk_warmth = s.diskWarmth;
        p->disk_inflow = 0.0f;
        p->doppler_strength = s.dopplerStrength;
        p->sky_brightness = s.skyBrightness;
        p->star_density = s.starDensity;
        p->star_brightness = s.starBrightness;
        p->shadow_overlay = s.showShadowOverlay ? 1 : 0;
        p->time = in.time;
        return true;
    }

    // Traces a frame into the Renderer's own device records (hits(), internal size). With the
    // volumetric disk the march also gathers the disk's light into image() (rgb, transmittance),
    // which renderImage() completes; the volumetric march is FP32.
    bool render(const FrameInput& in, int precision = BHR_PREC_FP32) {
        if (!ctx_ && !init(device_)) return false;
        bhr_view v{};
        if (!makeView(in, &v)) return logError("render: incomplete FrameInput", nullptr);
        const size_t n = size_t(v.width) * size_t(v.height);
        if (n > capacity_) {
            if (records_) cudaFree(records_);
            records_ = nullptr;
            capacity_ = 0;
            if (cudaMalloc(&records_, n * sizeof(bhr_hit)) != cudaSuccess)
                return logError("render: cannot allocate the hit records", nullptr);
            capacity_ = n;
        }
        width_ = v.width;
        height_ = v.height;
        bhr_hit* const outs[1] = {records_};
        const int nb = in.bodies ? int(in.bodies->size()) : 0;
        if (nb > 0) {  // the BHS_BODIES variant (Renderer.cpp:359-366)
            if (n > body_capacity_) {
                if (body_hits_) cudaFree(body_hits_);
                body_hits_ = nullptr;
                body_capacity_ = 0;
                if (cudaMalloc(&body_hits_, n * sizeof(bhr_body_hit)) != cudaSuccess)
                    return logError("render: cannot allocate the body records", nullptr);
                body_capacity_ = n;
            }
            if (v.disk_mode == BHR_DISK_VOLUMETRIC) {  // the disk's light gathered into image()
                bhr_shade_params p{};
                if (!makeShadeParams(in, &p) || !ensureImage(n)) return logError("render: volumetric disk", nullptr);
                if (bhr_trace_bodies_volumetric(ctx_, &v, in.bodies->data(), nb, &p, records_, body_hits_, image_,
                                                nullptr) != BHR_OK)
                    return logError("render", ctx_);
                return true;
            }
            if (bhr_trace_bodies(ctx_, &v, in.bodies->data(), nb, records_, body_hits_, nullptr) != BHR_OK)
                return logError("render", ctx_);
            return true;
        }
        if (v.disk_mode == BHR_DISK_VOLUMETRIC) {
            bhr_shade_params p{};
            if (!makeShadeParams(in, &p) || !ensureImage(n)) return logError("render: volumetric disk", nullptr);
            float* const rgbt[1] = {image_};
            if (bhr_trace_volumetric(ctx_, &v, 1, outs, &p, rgbt, nullptr) != BHR_OK) return logError("render", ctx_);
            return true;
        }
        if (bhr_trace(ctx_, &v, 1, outs, precision, method(in), nullptr) != BHR_OK) return logError("render", ctx_);
        return true;
    }

    // Traces into caller-owned device records (at least internalSize() pixels) on `stream`;
    // the volumetric disk also needs rgbt_dev (as many float4).
    bool renderTo(const FrameInput& in, bhr_hit* out_dev, cudaStream_t stream, int precision = BHR_PREC_FP32,
                  float* rgbt_dev = nullptr) {
        if (!ctx_ && !init(device_)) return false;
        bhr_view v{};
        if (!makeView(in, &v)) return logError("renderTo: incomplete FrameInput", nullptr);
        bhr_hit* const outs[1] = {out_dev};
        if (v.disk_mode == BHR_DISK_VOLUMETRIC) {
            bhr_shade_params p{};
            if (!rgbt_dev || !makeShadeParams(in, &p))
                return logError("renderTo: the volumetric disk needs an rgbt buffer", nullptr);
            float* const rgbt[1] = {rgbt_dev};
            if (bhr_trace_volumetric(ctx_, &v, 1, outs, &p, rgbt, stream) != BHR_OK) return logError("renderTo", ctx_);
            return true;
        }
        if (bhr_trace(ctx_, &v, 1, outs, precision, method(in), stream) != BHR_OK) return logError("renderTo", ctx_);
        return true;
    }

    // Traces a frame and returns its records in host memory (synchronous).
    bool renderHost(const FrameInput& in, std::vector<bhr_hit>& out, int precision = BHR_PREC_FP32) {
        if (!ctx_ && !init(device_)) return false;
        bhr_view v{};
        if (!makeView(in, &v)) return logError("renderHost: incomplete FrameInput", nullptr);
        out.resize(size_t(v.width) * size_t(v.height));
        if (v.disk_mode == BHR_DISK_VOLUMETRIC) {  // device march, then one copy
            if (!render(in, precision)) return false;
            if (cudaMemcpy(out.data(), records_, out.size() * sizeof(bhr_hit), cudaMemcpyDeviceToHost) != cudaSuccess)
                return logError("renderHost: copy", nullptr);
            return true;
        }
        bhr_hit* const outs[1] = {out.data()};
        if (bhr_trace_host(ctx_, &v, 1, outs, precision, method(in)) != BHR_OK) return logError("renderHost", ctx_);
        return true;
    }

    // Traces and shades a frame: image() holds width() x height() float4 (linear rgb without
    // the sky cube's term, alpha = that term's weight), row 0 at the bottom.
    bool renderImage(const FrameInput& in, int precision = BHR_PREC_FP32) {
        if (!render(in, precision)) return false;
        bhr_view v{};
        bhr_shade_params p{};
        if (!makeView(in, &v) || !makeShadeParams(in, &p)) return logError("renderImage: incomplete FrameInput", nullptr);
        if (!ensureImage(size_t(v.width) * size_t(v.height))) return false;
        if (in.bodies && !in.bodies->empty()) {
            if (bhr_shade_bodies(ctx_, &v, records_, body_hits_, in.bodies->data(), int(in.bodies->size()), &p, image_,
                                 nullptr) != BHR_OK)
                return logError("renderImage", ctx_);
            return true;
        }
        const bhr_hit* const hits[1] = {records_};
        float* const outs[1] = {image_};
        if (bhr_shade(ctx_, &v, 1, hits, &p, outs, nullptr) != BHR_OK) return logError("renderImage", ctx_);
        return true;
    }

    const bhr_hit* hits() const { return records_; }  // device records of the last render()
    const float* image() const { return image_; }      // device float4 image of the last renderImage()
    const bhr_body_hit* bodyHits() const { return body_hits_; }  // device body records of the last render() with bodies
    int width() const { return width_; }
    int height() const { return height_; }
    bhr_ctx* context() const { return ctx_; }

private:
    static int method(const FrameInput& in) {
        return in.settings && in.settings->surrogate ? BHR_METHOD_SURROGATE : BHR_METHOD_PLAIN;
    }

    bool ensureImage(size_t n) {
        if (n <= image_capacity_) return true;
        if (image_) cudaFree(image_);
        image_ = nullptr;
        image_capacity_ = 0;
        if (cudaMalloc(&image_, n * 4 * sizeof(float)) != cudaSuccess)
            return logError("cannot allocate the image", nullptr);
        image_capacity_ = n;
        return true;
    }

    bool logError(const char* what, const bhr_ctx* c) {
        const char* m = bhr_last_error(c);
        const std::string line = std::string("bhr: ") + what + (m && *m ? std::string(": ") + m : std::string());
        if (log_) log_(line);
        else std::fprintf(stderr, "%s\n", line.c_str());
        return false;
    }

    bhr_ctx* ctx_ = nullptr;
    bhr_surrogate* surr_ = nullptr;
    int device_ = 0;
    bhr_hit* records_ = nullptr;
    size_t capacity_ = 0;
    float* image_ = nullptr;
    size_t image_capacity_ = 0;
    bhr_body_hit* body_hits_ = nullptr;
    size_t body_capacity_ = 0;
    int width_ = 0, height_ = 0;
    LogFn log_;
};

}  // namespace bhr
