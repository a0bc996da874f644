// Checks of the C++ host interface (include/bhr_renderer.hpp), in the style of the reference's
// tests/geodesic_tests.cpp: host-only checks always; with `--gpu <file>` also a traced frame
// (the 256x144 view at r = 30, inclination 85 deg, 200 steps) through Renderer::render,
// renderTo and renderHost, whose records are written to <file> for the oracle comparison the
// Python test driver makes; with `--surrogate <checkpoint>` also a 480x270 frame of the same
// camera through the learned surrogate under the shader's rule (<file>.surrogate).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "bhr_renderer.hpp"

static int g_failures = 0;
static int g_checks = 0;

#define CHECK(cond, msg)                                                    \
    do {                                                                    \
        ++g_checks;                                                         \
        if (cond) {                                                         \
            std::printf("  ok    %s\n", msg);                               \
        } else {                                                            \
            ++g_failures;                                                   \
            std::printf("  FAIL  %s   (%s:%d)\n", msg, __FILE__, __LINE__); \
        }                                                                   \
    } while (0)

static bhr::Camera orbitCamera(double r, double incl, double az) {
    bhr::Camera c;
    c.setPosition(bhr::Vec3d{r * std::sin(incl) * std::sin(az), r * std::cos(incl), r * std::sin(incl) * std::cos(az)});
    c.lookAt(bhr::Vec3d{0.0, 0.0, 0.0});
    return c;
}

static void testPresets() {
    std::printf("quality presets (Settings::applyPreset)\n");
    const int steps[4] = {200, 300, 450, 700};
    const float scale[4] = {0.10f, 0.07f, 0.05f, 0.035f};
    const float disk[4] = {0.35f, 0.30f, 0.18f, 0.10f};
    for (int p = 0; p < 4; ++p) {
        bhr::Settings s;
        s.applyPreset(p);
        char msg[96];
        std::snprintf(msg, sizeof msg, "preset %d: %d steps, step scale %.3f, disk step %.2f", p, steps[p], scale[p], disk[p]);
        CHECK(s.maxSteps == steps[p] && s.stepScale == scale[p] && s.diskStep == disk[p], msg);
    }
    bhr::Settings s;
    s.maxSteps = 123;
    s.applyPreset(bhr::PRESET_CUSTOM);
    CHECK(s.maxSteps == 123, "custom preset keeps the fields");
}

static void testCameraBasis() {
    std::printf("camera basis (lookRotation, mat3_cast)\n");
    bhr::Camera c;  // default bookmark: (0, 2.6, 24.9) looking at the hole
    float B[9];
    c.basis(B);
    double orth = 0.0;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            double d = 0.0;
            for (int k = 0; k < 3; ++k) d += double(B[3 * a + k]) * B[3 * b + k];
            orth = std::max(orth, std::fabs(d - (a == b ? 1.0 : 0.0)));
        }
    char msg[128];
    std::snprintf(msg, sizeof msg, "columns orthonormal (max error %.1e)", orth);
    CHECK(orth < 1e-6, msg);
    const bhr::Vec3d p = c.position();
    const double r = c.radius();
    const double back_dot = (B[6] * p.x + B[7] * p.y + B[8] * p.z) / r;  // back column points away from the hole
    std::snprintf(msg, sizeof msg, "back column = position / r (cos %.8f)", back_dot);
    CHECK(back_dot > 1.0 - 1e-6, msg);
    CHECK(std::fabs(B[1]) < 1e-6, "right column is horizontal (roll 0)");
    CHECK(B[4] > 0.0f, "up column points up");
    // top-down bookmark: looking along -Y with up (0,1,0) takes the (0,0,-1) fallback (Camera.cpp:17)
    bhr::Camera top;
    top.setPosition(bhr::Vec3d{0.0, 32.0, 0.001});
    top.lookAt(bhr::Vec3d{0.0, 0.0, 0.0});
    top.basis(B);
    bool finite = true;
    for (float e : B) finite = finite && std::isfinite(e);
    CHECK(finite && B[7] > 0.99f, "top-down view: finite basis, back column along +Y");
}

static void testFrameToView() {
    std::printf("FrameInput -> bhr_view (setTraceUniforms)\n");
    bhr::Settings s;
    s.applyPreset(bhr::PRESET_LOW);
    s.renderScale = 0.5f;
    s.diskOuter = 24.0f;
    const bhr::Camera cam = orbitCamera(30.0, 85.0 * M_PI / 180.0, 0.0);
    bhr::FrameInput in;
    in.camera = &cam;
    in.settings = &s;
    in.windowW = 1920;
    in.windowH = 1080;
    bhr_view v{};
    CHECK(bhr::Renderer::makeView(in, &v), "complete input converts");
    CHECK(v.width == 960 && v.height == 540, "internal size = lround(window * renderScale)");
    CHECK(v.max_steps == 200 && v.step_scale == 0.10f && v.disk_step == 0.35f, "preset fields carried");
    CHECK(std::fabs(v.tan_half_fov - std::tan(60.0f * 0.01745329252f * 0.5f)) < 1e-7f, "tan(fov/2) as Renderer.cpp:246");
    CHECK(v.r_esc_min == 30.0f, "shader rEscMin = max(1.25 r_out, 12)");
    CHECK(v.disk_mode == BHR_DISK_VOLUMETRIC && v.lensing == 1 && v.far_mode == 0, "disk (the default, volumetric), lensing and far mode carried");
    CHECK(std::fabs(v.cam_pos[1] - float(30.0 * std::cos(85.0 * M_PI / 180.0))) < 1e-5f, "camera position carried");
    s.renderScale = 0.001f;
    bhr::Renderer::makeView(in, &v);
    CHECK(v.width == 192 && v.height == 108, "renderScale clamps at 0.1");
    in.windowW = 10;
    in.windowH = 10;
    s.renderScale = 1.0f;
    bhr::Renderer::makeView(in, &v);
    CHECK(v.width == 16 && v.height == 16, "internal size at least 16");
    bhr::FrameInput bad;
    CHECK(!bhr::Renderer::makeView(bad, &v), "missing camera / settings is refused");
}

static void testErrors() {
    std::printf("error reporting (bool + log line, no exceptions)\n");
    bhr_view v{};
    bhr_view_init(&v, BHR_TERM_SHADER);
    v.width = 0;
    bhr_hit* outs[1] = {nullptr};
    CHECK(bhr_trace(nullptr, &v, 1, outs, BHR_PREC_FP32, BHR_METHOD_PLAIN, nullptr) == BHR_ERR_INVALID_ARG,
          "bhr_trace without a context is an argument error");
    CHECK(std::strlen(bhr_last_error(nullptr)) > 0, "the error has a message");
    CHECK(bhr_view_apply_preset(&v, 9) == BHR_ERR_INVALID_ARG, "unknown preset is refused");
    CHECK(bhr_view_set_fov(&v, 190.0f) == BHR_ERR_INVALID_ARG, "fov >= 180 is refused");
}

static void testShadeParams() {
    std::printf("shading uniforms\n");
    bhr::Settings s;
    const bhr::Camera cam = orbitCamera(30.0, 85.0 * M_PI / 180.0, 0.0);
    bhr::FrameInput in;
    in.camera = &cam;
    in.settings = &s;
    in.windowW = 64;
    in.windowH = 36;
    in.diskTime = 12.5f;
    bhr_shade_params p{};
    CHECK(bhr::Renderer::makeShadeParams(in, &p), "complete input converts");
    CHECK(p.disk_opacity == 2.0f && p.disk_brightness == 5.5f && p.disk_peak_temp == 6000.0f && p.noise_seed == 7u,
          "Settings defaults at full fade, noise seed 7");
    CHECK(p.disk_time == 12.5f && p.shadow_overlay == 0, "disk clock and overlay carried");
    bhr::FrameInput faded = in;
    faded.diskFade = 0.0f;
    bhr_view fv{};
    CHECK(bhr::Renderer::makeView(faded, &fv) && fv.disk_mode == BHR_DISK_NONE, "a faded disk is not marched");
    CHECK(bhr::Renderer::makeShadeParams(faded, &p) && p.disk_opacity == 0.0f && p.disk_brightness == 0.0f,
          "a faded disk neither absorbs nor shines");
    faded.diskFade = 0.25f;
    CHECK(bhr::Renderer::makeShadeParams(faded, &p) && p.disk_opacity == 0.5f, "opacity scales with the fade");
}

static int testGpu(const char* path, const char* surrogate_path) {
    std::printf("traced frame (256x144, r=30, inclination 85 deg, 200 steps)\n");
    std::string logged;
    bhr::Renderer R;
    R.setLogger([&](const std::string& m) { logged = m; });
    if (!R.init(0)) {
        std::printf("  FAIL  init: %s\n", logged.c_str());
        return 1;
    }
    bhr::Settings s;
    s.applyPreset(bhr::PRESET_LOW);
    s.diskMode = bhr::DISK_THIN;
    const bhr::Camera cam = orbitCamera(30.0, 85.0 * M_PI / 180.0, 0.0);
    bhr::FrameInput in;
    in.camera = &cam;
    in.settings = &s;
    in.windowW = 256;
    in.windowH = 144;
    in.termMode = BHR_TERM_CONFIG;
    CHECK(R.render(in), "render");
    CHECK(R.width() == 256 && R.height() == 144, "records at the internal size");
    const size_t n = 256 * 144;
    std::vector<bhr_hit> a(n), b, c(n);
    CHECK(cudaMemcpy(a.data(), R.hits(), n * sizeof(bhr_hit), cudaMemcpyDeviceToHost) == cudaSuccess, "read back");
    CHECK(R.renderHost(in, b), "renderHost");
    bhr_hit* d = nullptr;
    cudaMalloc(&d, n * sizeof(bhr_hit));
    cudaStream_t st;
    cudaStreamCreate(&st);
    CHECK(R.renderTo(in, d, st), "renderTo on a stream");
    cudaStreamSynchronize(st);
    cudaMemcpy(c.data(), d, n * sizeof(bhr_hit), cudaMemcpyDeviceToHost);
    cudaFree(d);
    cudaStreamDestroy(st);
    CHECK(b.size() == n && std::memcmp(a.data(), b.data(), n * sizeof(bhr_hit)) == 0, "renderHost = render");
    CHECK(std::memcmp(a.data(), c.data(), n * sizeof(bhr_hit)) == 0, "renderTo = render");
    int esc = 0, cap = 0, disk = 0;
    for (const bhr_hit& h : a) {
        esc += h.status == BHR_STATUS_ESCAPED;
        cap += h.status == BHR_STATUS_CAPTURED;
        disk += h.ncross > 0;
    }
    char msg[128];
    std::snprintf(msg, sizeof msg, "escaped %d, captured %d, disk %d of %zu", esc, cap, disk, n);
    CHECK(esc > 0 && cap > 0 && disk > 0 && esc + cap <= int(n), msg);
    bhr::FrameInput bad = in;
    bad.windowW = 0;
    CHECK(!R.render(bad) && !logged.empty(), "bad input: false and a log line");
    FILE* f = std::fopen(path, "wb");
    const bool wrote = f && std::fwrite(a.data(), sizeof(bhr_hit), n, f) == n;
    if (f) std::fclose(f);
    CHECK(wrote, "records written");
    // the frame's colour: traced and shaded; written beside the records for the parity check
    CHECK(R.renderImage(in), "renderImage");
    std::vector<float> img(n * 4);
    CHECK(cudaMemcpy(img.data(), R.image(), img.size() * sizeof(float), cudaMemcpyDeviceToHost) == cudaSuccess,
          "read back the image");
    int lit = 0;
    for (size_t k = 0; k < n; ++k) lit += img[4 * k] + img[4 * k + 1] + img[4 * k + 2] > 0.0f;
    std::snprintf(msg, sizeof msg, "%d of %zu pixels lit", lit, n);
    CHECK(lit > int(n / 2), msg);
    const std::string ipath = std::string(path) + ".rgba";
    FILE* g = std::fopen(ipath.c_str(), "wb");
    const bool wrote_img = g && std::fwrite(img.data(), sizeof(float), img.size(), g) == img.size();
    if (g) std::fclose(g);
    CHECK(wrote_img, "image written");
    // the reference's default disk: volumetric, its light gathered by the march
    bhr::Settings sv;
    sv.applyPreset(bhr::PRESET_LOW);
    CHECK(sv.diskMode == bhr::DISK_VOLUMETRIC, "the default disk is volumetric (Settings.h:22)");
    bhr::FrameInput iv = in;
    iv.settings = &sv;
    CHECK(R.renderImage(iv), "renderImage with the volumetric disk");
    std::vector<bhr_hit> hv(n);
    std::vector<float> imv(n * 4);
    cudaMemcpy(hv.data(), R.hits(), n * sizeof(bhr_hit), cudaMemcpyDeviceToHost);
    cudaMemcpy(imv.data(), R.image(), imv.size() * sizeof(float), cudaMemcpyDeviceToHost);
    int vlit = 0, vcross = 0;
    for (size_t k = 0; k < n; ++k) {
        vlit += imv[4 * k] + imv[4 * k + 1] + imv[4 * k + 2] > 0.0f;
        vcross += hv[k].ncross;
    }
    std::snprintf(msg, sizeof msg, "%d of %zu pixels lit, no crossing slots (%d)", vlit, n, vcross);
    CHECK(vlit > int(n / 2) && vcross == 0, msg);
    std::vector<bhr_hit> hh;
    CHECK(R.renderHost(iv, hh) && hh.size() == n && std::memcmp(hh.data(), hv.data(), n * sizeof(bhr_hit)) == 0,
          "renderHost = render with the volumetric disk");
    CHECK(!R.renderTo(iv, nullptr, nullptr) && !logged.empty(), "renderTo without an rgbt buffer is refused");
    // bodies (the BHS_BODIES variant): a planet straight ahead stops the central rays
    std::vector<bhr_body> bodies(1);
    bhr_body& pl = bodies[0];
    std::memset(&pl, 0, sizeof pl);
    const bhr::Vec3d cp = cam.position();
    const double cr = std::sqrt(cp.x * cp.x + cp.y * cp.y + cp.z * cp.z);
    const double fr = 1.0 - 6.0 / cr;
    const float pos[3] = {float(cp.x * fr), float(cp.y * fr), float(cp.z * fr)};
    for (int k = 0; k < 3; ++k) {
        pl.pos_radius[k] = pos[k];
        pl.rel_pos[k] = float(pos[k] - (k == 0 ? cp.x : k == 1 ? cp.y : cp.z));
    }
    pl.pos_radius[3] = 0.8f;
    pl.look[0] = 4.0f;  // the earth-like look
    pl.look[1] = 7.0f;
    pl.tint[0] = pl.tint[1] = pl.tint[2] = 1.0f;
    pl.light[1] = 1.0f;
    pl.light[3] = 1.0f;
    pl.light_color[0] = pl.light_color[1] = pl.light_color[2] = 1.0f;
    pl.axis[1] = 1.0f;
    pl.ring[3] = 1.0f;
    bhr::FrameInput ib = in;
    ib.bodies = &bodies;
    ib.time = 5.0f;
    CHECK(R.renderImage(ib), "renderImage with a body");
    std::vector<bhr_hit> hb(n);
    std::vector<bhr_body_hit> bb(n);
    cudaMemcpy(hb.data(), R.hits(), n * sizeof(bhr_hit), cudaMemcpyDeviceToHost);
    cudaMemcpy(bb.data(), R.bodyHits(), n * sizeof(bhr_body_hit), cudaMemcpyDeviceToHost);
    int onb = 0;
    for (size_t k = 0; k < n; ++k) onb += hb[k].status == BHR_STATUS_BODY && bb[k].body == 0;
    const size_t mid = (in.windowH / 2) * size_t(in.windowW) + in.windowW / 2;
    std::snprintf(msg, sizeof msg, "%d pixels on the planet, the centre among them", onb);
    CHECK(onb > 50 && hb[mid].status == BHR_STATUS_BODY, msg);
    // the same planet with the volumetric disk (the default disk): marched through the disk's
    // volume, then shaded in place over the light the march gathered
    bhr::FrameInput ibv = ib;
    ibv.settings = &sv;
    CHECK(R.renderImage(ibv), "renderImage with a body and the volumetric disk");
    cudaMemcpy(hb.data(), R.hits(), n * sizeof(bhr_hit), cudaMemcpyDeviceToHost);
    cudaMemcpy(bb.data(), R.bodyHits(), n * sizeof(bhr_body_hit), cudaMemcpyDeviceToHost);
    std::vector<float> imb(n * 4);
    cudaMemcpy(imb.data(), R.image(), imb.size() * sizeof(float), cudaMemcpyDeviceToHost);
    int onv = 0, litv = 0;
    for (size_t k = 0; k < n; ++k) {
        const bool on = hb[k].status == BHR_STATUS_BODY && bb[k].body == 0;
        onv += on;
        litv += on && imb[4 * k] + imb[4 * k + 1] + imb[4 * k + 2] > 0.0f && imb[4 * k + 3] == 0.0f;
    }
    std::snprintf(msg, sizeof msg, "volumetric disk: %d pixels on the planet, %d of them lit without sky", onv, litv);
    CHECK(onv > 50 && hb[mid].status == BHR_STATUS_BODY && litv > onv / 2, msg);
    if (surrogate_path) {
        // the learned orbit surrogate under the shader's own rule (the default termMode), thin disk
        bhr::Settings ss;
        ss.applyPreset(bhr::PRESET_HIGH);
        ss.diskMode = bhr::DISK_THIN;
        ss.surrogate = true;
        bhr::FrameInput is = in;
        is.settings = &ss;
        is.windowW = 480;
        is.windowH = 270;
        is.termMode = BHR_TERM_SHADER;
        logged.clear();
        CHECK(!R.render(is) && !logged.empty(), "the surrogate before one is loaded: false and a log line");
        CHECK(R.loadSurrogate(surrogate_path), "loadSurrogate");
        CHECK(R.render(is), "render with the surrogate (shader rule)");
        const size_t ns = size_t(is.windowW) * is.windowH;
        std::vector<bhr_hit> hs(ns);
        cudaMemcpy(hs.data(), R.hits(), ns * sizeof(bhr_hit), cudaMemcpyDeviceToHost);
        size_t by_surr = 0;
        for (const bhr_hit& h : hs) by_surr += (h.flags & BHR_FLAG_SURROGATE) != 0;
        std::snprintf(msg, sizeof msg, "%zu of %zu rays answered by the surrogate", by_surr, ns);
        CHECK(by_surr > ns * 99 / 100, msg);
        std::vector<bhr_hit> hh2;
        CHECK(R.renderHost(is, hh2) && hh2.size() == ns && std::memcmp(hh2.data(), hs.data(), ns * sizeof(bhr_hit)) == 0,
              "renderHost = render with the surrogate");
        const std::string spath = std::string(path) + ".surrogate";
        FILE* h = std::fopen(spath.c_str(), "wb");
        const bool wrote_s = h && std::fwrite(hs.data(), sizeof(bhr_hit), ns, h) == ns;
        if (h) std::fclose(h);
        CHECK(wrote_s, "surrogate records written");
    }
    R.shutdown();
    return 0;
}

int main(int argc, char** argv) {
    testPresets();
    testCameraBasis();
    testFrameToView();
    testErrors();
    testShadeParams();
    if (argc >= 3 && std::strcmp(argv[1], "--gpu") == 0)
        testGpu(argv[2], argc == 5 && std::strcmp(argv[3], "--surrogate") == 0 ? argv[4] : nullptr);
    std::printf("\n%d checks, %d failures\n", g_checks, g_failures);
    return g_failures == 0 ? 0 : 1;
}
