// C entry points of the CPU oracle (liboracle.so) -- TEST INFRASTRUCTURE ONLY.
// Loaded by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg through ctypes;
// never by the product library. The march itself is oracle/march.hpp.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "march.hpp"
#include "lens.hpp"
#include "shade.hpp"
#include "bodies.hpp"

using namespace oracle;

namespace {

template <class F>
void parallel_for(int64_t n, int nthreads, int64_t grain, F&& fn) {
    if (nthreads <= 1 || n <= grain) {
        for (int64_t k = 0; k < n; ++k) fn(k);
        return;
    }
    std::atomic<int64_t> next{0};
    std::vector<std::thread> pool;
    pool.reserve(nthreads);
    for (int t = 0; t < nthreads; ++t) {
        pool.emplace_back([&] {
            for (;;) {
                const int64_t b = next.fetch_add(grain);
                if (b >= n) break;
                const int64_t e = std::min(n, b + grain);
                for (int64_t k = b; k < e; ++k) fn(k);
            }
        });
    }
    for (auto& th : pool) th.join();
}

bool view_ok(const bhr_view* v) {
    return v && v->width > 0 && v->height > 0 && v->max_steps >= 0 && v->disk_mode != BHR_DISK_VOLUMETRIC;
}

// The volumetric disk's sub-sample (oracle/shade.hpp vol_disk_step) in float, as the shader.
struct VolumeSampler {
    const oracle::shade::Tex* tx;
    const bhr_shade_params* P;
    float r_in, r_out, thick, rcam;
    template <class T> void operator()(const V3<T>& p, T rm, T sub, Result<T>& res) const {
        oracle::shade::vol_disk_step(*tx, *P, r_in, r_out, thick, oracle::shade::F3{float(p.x), float(p.y), float(p.z)},
                                     float(rm), float(sub), float(res.b_axis), rcam, res.col, res.trans);
    }
};

// The body-aware march of the listed pixels (idx = j * width + i; every pixel when idx is NULL)
// with the disk sampler `vol` (NoVolume, or VolumeSampler for the volumetric disk, which also
// fills rgbt[4k..4k+3] with the gathered colour and transmittance).
template <class Vol>
int trace_bodies_impl(const bhr_view* v, const bhr_body* bodies, int nb, const int64_t* idx, int64_t n, bhr_hit* out,
                      bhr_body_hit* bout, const Vol& vol, float* rgbt, int nthreads, int fp64) {
    const int64_t npix = static_cast<int64_t>(v->width) * v->height;
    if (idx) {
        for (int64_t k = 0; k < n; ++k)
            if (idx[k] < 0 || idx[k] >= npix) return BHR_ERR_INVALID_ARG;
    } else if (n != npix) {
        return BHR_ERR_INVALID_ARG;
    }
    auto one = [&](auto R, int64_t k) {
        using T = decltype(R.step_scale);
        const int64_t px = idx ? idx[k] : k;
        const int i = static_cast<int>(px % v->width), j = static_cast<int>(px / v->width);
        const V3<T> cam{T(v->cam_pos[0]), T(v->cam_pos[1]), T(v->cam_pos[2])};
        BodyMarch<T> bm;
        bm.b = bodies;
        bm.n = nb;
        const Result<T> r = march(R, cam, primaryRay<T>(*v, i, j), vol, bm);
        toHit(r, out + k);
        bhr_body_hit& o = bout[k];
        o = bhr_body_hit{};
        // the loop-head near-field hit records only the body (blackhole.frag:147-149)
        o.body = r.status == BHR_STATUS_BODY ? (bm.hit >= 0 ? bm.hit : bm.near_idx) : -1;
        o.t = float(bm.hit_t);
        o.ro[0] = float(bm.hit_ro.x), o.ro[1] = float(bm.hit_ro.y), o.ro[2] = float(bm.hit_ro.z);
        o.rd[0] = float(bm.hit_rd.x), o.rd[1] = float(bm.hit_rd.y), o.rd[2] = float(bm.hit_rd.z);
        o.x[0] = float(r.x.x), o.x[1] = float(r.x.y), o.x[2] = float(r.x.z);
        o.near_mask = bm.near_mask;
        o.near_idx = bm.near_idx;
        o.near_t = float(bm.near_t);
        o.travelled = float(bm.travelled);
        if (rgbt) {
            for (int c = 0; c < 3; ++c) rgbt[4 * k + c] = r.col[c];
            rgbt[4 * k + 3] = r.trans;
        }
    };
    if (fp64) {
        const Rule<double> R = Rule<double>::from_view(*v);
        parallel_for(n, nthreads, 64, [&](int64_t k) { one(R, k); });
    } else {
        const Rule<float> R = Rule<float>::from_view(*v);
        parallel_for(n, nthreads, 64, [&](int64_t k) { one(R, k); });
    }
    return BHR_OK;
}

template <class T>
void trace_one(const bhr_view& w, const Rule<T>& R, int64_t idx, bhr_hit* out) {
    const int i = static_cast<int>(idx % w.width);
    const int j = static_cast<int>(idx / w.width);
    toHit(marchPixel<T>(w, R, i, j), out);
}

}  // namespace

extern "C" {

// Traces every pixel of a view (row-major, row 0 at the bottom) into host memory.
int oracle_trace_view(const bhr_view* v, bhr_hit* out, int nthreads, int fp64) {
    if (!view_ok(v) || !out) return BHR_ERR_INVALID_ARG;
    const int64_t n = static_cast<int64_t>(v->width) * v->height;
    if (fp64) {
        const Rule<double> R = Rule<double>::from_view(*v);
        parallel_for(n, nthreads, 256, [&](int64_t k) { trace_one<double>(*v, R, k, out + k); });
    } else {
        const Rule<float> R = Rule<float>::from_view(*v);
        parallel_for(n, nthreads, 256, [&](int64_t k) { trace_one<float>(*v, R, k, out + k); });
    }
    return BHR_OK;
}

// Traces the listed pixel indices (idx = j * width + i); out[k] belongs to idx[k].
int oracle_trace_pixels(const bhr_view* v, const int64_t* idx, int64_t n, bhr_hit* out, int nthreads, int fp64) {
    if (!view_ok(v) || !idx || !out || n < 0) return BHR_ERR_INVALID_ARG;
    const int64_t npix = static_cast<int64_t>(v->width) * v->height;
    for (int64_t k = 0; k < n; ++k)
        if (idx[k] < 0 || idx[k] >= npix) return BHR_ERR_INVALID_ARG;
    if (fp64) {
        const Rule<double> R = Rule<double>::from_view(*v);
        parallel_for(n, nthreads, 64, [&](int64_t k) { trace_one<double>(*v, R, idx[k], out + k); });
    } else {
        const Rule<float> R = Rule<float>::from_view(*v);
        parallel_for(n, nthreads, 64, [&](int64_t k) { trace_one<float>(*v, R, idx[k], out + k); });
    }
    return BHR_OK;
}

// Primary ray directions of the listed pixels in double (blackhole.frag:68-72 in FP64).
int oracle_primary_rays(const bhr_view* v, const int64_t* idx, int64_t n, double* dirs) {
    if (!view_ok(v) || !idx || !dirs) return BHR_ERR_INVALID_ARG;
    for (int64_t k = 0; k < n; ++k) {
        const V3<double> d = primaryRay<double>(*v, static_cast<int>(idx[k] % v->width),
                                                static_cast<int>(idx[k] / v->width));
        dirs[3 * k] = d.x;
        dirs[3 * k + 1] = d.y;
        dirs[3 * k + 2] = d.z;
    }
    return BHR_OK;
}

// One ray from a double camera position and direction under the rule of `rule` (its pose,
// size and pixel fields are ignored). state_out (may be NULL) gets the final x, v and dir
// in double: x[3], v[3], dir[3].
int oracle_march_ray(const bhr_view* rule, const double cam[3], const double dir[3], int fp64, bhr_hit* out,
                     double* state_out) {
    if (!rule || !cam || !dir || !out) return BHR_ERR_INVALID_ARG;
    if (fp64) {
        const Rule<double> R = Rule<double>::from_view(*rule);
        const Result<double> r = march(R, V3<double>{cam[0], cam[1], cam[2]}, V3<double>{dir[0], dir[1], dir[2]});
        toHit(r, out);
        if (state_out) {
            const double s[9] = {r.x.x, r.x.y, r.x.z, r.v.x, r.v.y, r.v.z, r.dir.x, r.dir.y, r.dir.z};
            std::memcpy(state_out, s, sizeof s);
        }
    } else {
        const Rule<float> R = Rule<float>::from_view(*rule);
        const Result<float> r = march(R, V3<float>{float(cam[0]), float(cam[1]), float(cam[2])},
                                      V3<float>{float(dir[0]), float(dir[1]), float(dir[2])});
        toHit(r, out);
        if (state_out) {
            const double s[9] = {r.x.x, r.x.y, r.x.z, r.v.x, r.v.y, r.v.z, r.dir.x, r.dir.y, r.dir.z};
            std::memcpy(state_out, s, sizeof s);
        }
    }
    return BHR_OK;
}

// Geodesic.h:107-140 trace(camPos, dir, maxSteps, stepScale, escTol, rEscMin) with the
// reference's double constants (capture below 2 + 0.01, ds floor 1e-4, no disk).
// out9: final x[3], v[3], dir[3]; out_int: status, steps, equatorCrossings; out_minr: minR.
int oracle_cpu_trace(const double cam[3], const double dir[3], int max_steps, double step_scale, double esc_tol,
                     double r_esc_min, double* out9, int* out_int, double* out_minr) {
    if (!cam || !dir || !out9 || !out_int || !out_minr) return BHR_ERR_INVALID_ARG;
    Rule<double> R;
    R.term_mode = BHR_TERM_CPU;
    R.max_steps = max_steps;
    R.disk_mode = BHR_DISK_NONE;
    R.lensing = true;
    R.far_mode = false;
    R.step_scale = step_scale;
    R.capture_r = 2.0 + 0.01;
    R.esc_tol = esc_tol;
    R.r_esc_min = r_esc_min;
    R.ds_floor = 1e-4;
    const Result<double> r = march(R, V3<double>{cam[0], cam[1], cam[2]}, V3<double>{dir[0], dir[1], dir[2]});
    // TraceResult::dir is zero unless the ray escaped (Geodesic.h:99)
    const bool esc = r.status == BHR_STATUS_ESCAPED;
    const double s[9] = {r.x.x, r.x.y, r.x.z, r.v.x, r.v.y, r.v.z,
                         esc ? r.dir.x : 0.0, esc ? r.dir.y : 0.0, esc ? r.dir.z : 0.0};
    std::memcpy(out9, s, sizeof s);
    // TraceResult::Status: Escaped 0, Captured 1, MaxSteps 2
    out_int[0] = r.status == BHR_STATUS_ESCAPED ? 0 : (r.status == BHR_STATUS_CAPTURED ? 1 : 2);
    out_int[1] = r.steps;
    out_int[2] = r.nplane;
    *out_minr = r.min_r;
    return BHR_OK;
}

// Single components in double, for pinning against the reference's own functions:
// rk4Step (geodesic.glsl:16-23 / Geodesic.h:27-34) in place on x, v;
// initialVelocity (geodesic.glsl:27-34 / Geodesic.h:40-47);
// farFieldDirection (geodesic.glsl:43-53 / Geodesic.h:65-75).
void oracle_rk4_step(double x[3], double v[3], double h2, double dt) {
    V3<double> X{x[0], x[1], x[2]}, V{v[0], v[1], v[2]};
    rk4Step(X, V, h2, dt);
    x[0] = X.x, x[1] = X.y, x[2] = X.z;
    v[0] = V.x, v[1] = V.y, v[2] = V.z;
}
void oracle_initial_velocity(const double cam[3], const double dir[3], double out[3]) {
    const V3<double> r = initialVelocity(V3<double>{cam[0], cam[1], cam[2]}, V3<double>{dir[0], dir[1], dir[2]});
    out[0] = r.x, out[1] = r.y, out[2] = r.z;
}
void oracle_far_field(const double x[3], const double v[3], double h2, double out[3]) {
    const V3<double> r = farFieldDirection(V3<double>{x[0], x[1], x[2]}, V3<double>{v[0], v[1], v[2]}, h2);
    out[0] = r.x, out[1] = r.y, out[2] = r.z;
}

// The lens table of a camera at cam_r (gas_lens.comp): 1024 x 1024 floats, table[j * 1024 + i],
// alpha_crit = the shadow's angular radius at cam_r (the reference passes it as a float uniform).
int oracle_lens_table(float cam_r, float alpha_crit, float* table, int nthreads, int fp64) {
    if (!table || !(cam_r > 2.0f)) return BHR_ERR_INVALID_ARG;
    if (fp64)
        parallel_for(oracle::kLensRays, nthreads, 1, [&](int64_t i) {
            oracle::lensRay<double>(int(i), double(cam_r), double(alpha_crit), table);
        });
    else
        parallel_for(oracle::kLensRays, nthreads, 1, [&](int64_t i) {
            oracle::lensRay<float>(int(i), cam_r, alpha_crit, table);
        });
    return BHR_OK;
}

// The disk's noise volume (noise_bake.comp) as IEEE half values, texel (x, y, z) at (z N + y) N + x.
int oracle_noise_bake(uint32_t seed, uint16_t* out, int nthreads) {
    if (!out) return BHR_ERR_INVALID_ARG;
    const int N = oracle::shade::kNoiseN;
    parallel_for(int64_t(N) * N, nthreads, 16, [&](int64_t zy) {
        const int z = int(zy / N), y = int(zy % N);
        for (int x = 0; x < N; ++x)
            out[zy * N + x] = oracle::shade::to_half(oracle::shade::noise_texel(x, y, z, seed));
    });
    return BHR_OK;
}

// The blackbody table (DiskTextures::bakeBlackbodyLut): BHR_BLACKBODY_LUT x 4 floats.
int oracle_blackbody_lut(float* out) {
    if (!out) return BHR_ERR_INVALID_ARG;
    oracle::shade::blackbody_lut(out);
    return BHR_OK;
}

// Shades one view from its hit records with the given noise volume and table; rgba gets
// width x height x 4 floats.
int oracle_shade_view(const bhr_view* v, const bhr_hit* hits, const bhr_shade_params* p, const uint16_t* noise,
                      const float* lut, float* rgba, int nthreads) {
    if (!v || !hits || !p || !noise || !lut || !rgba || v->width <= 0 || v->height <= 0) return BHR_ERR_INVALID_ARG;
    const oracle::shade::Tex tx{noise, lut};
    parallel_for(v->height, nthreads, 1, [&](int64_t j) { oracle::shade::shade_view(tx, *p, *v, hits, rgba, j, j + 1); });
    return BHR_OK;
}

// Single components, for known-answer tests: the shader's redshiftFactor (disk.glsl:36-41) and
// the CIE XYZ of a blackbody at T (the table's integral, DiskTextures.cpp:32-41).
float oracle_redshift_factor(float r, float b_axis, float rcam) { return oracle::shade::redshift_factor(r, b_axis, rcam); }
void oracle_blackbody_xyz(double T, double out[3]) { oracle::shade::xyz_of(T, out[0], out[1], out[2]); }
uint16_t oracle_to_half(float x) { return oracle::shade::to_half(x); }
void oracle_pcg3d(const uint32_t in[3], uint32_t out[3]) {
    const oracle::shade::U3 h = oracle::shade::pcg3d({in[0], in[1], in[2]});
    out[0] = h.x, out[1] = h.y, out[2] = h.z;
}

// The volumetric disk's march of every pixel of a view: records, and rgbt[4 k] = the colour the
// march gathered and the transmittance left (blackhole.frag:217-234).
// The volumetric march of the listed pixels (idx = j * width + i; every pixel when idx is NULL):
// out[k] and rgbt[4k..4k+3] belong to idx[k].
int oracle_trace_volumetric_pixels(const bhr_view* v, const bhr_shade_params* p, const uint16_t* noise,
                                   const float* lut, const int64_t* idx, int64_t n, bhr_hit* out, float* rgbt,
                                   int nthreads, int fp64) {
    if (!v || !p || !noise || !lut || !out || !rgbt || v->width <= 0 || v->height <= 0 || v->max_steps < 0 ||
        v->disk_mode != BHR_DISK_VOLUMETRIC || n < 0)
        return BHR_ERR_INVALID_ARG;
    const int64_t npix = static_cast<int64_t>(v->width) * v->height;
    if (idx) {
        for (int64_t k = 0; k < n; ++k)
            if (idx[k] < 0 || idx[k] >= npix) return BHR_ERR_INVALID_ARG;
    } else if (n != npix) {
        return BHR_ERR_INVALID_ARG;
    }
    const oracle::shade::Tex tx{noise, lut};
    const float cx = v->cam_pos[0], cy = v->cam_pos[1], cz = v->cam_pos[2];
    const VolumeSampler vs{&tx, p, v->disk_inner, v->disk_outer, v->disk_thickness, std::sqrt(cx * cx + cy * cy + cz * cz)};
    auto one = [&](auto R, int64_t k) {
        using T = decltype(R.step_scale);
        const int64_t px = idx ? idx[k] : k;
        const int i = static_cast<int>(px % v->width), j = static_cast<int>(px / v->width);
        const V3<T> cam{T(v->cam_pos[0]), T(v->cam_pos[1]), T(v->cam_pos[2])};
        const Result<T> r = march(R, cam, primaryRay<T>(*v, i, j), vs);
        toHit(r, out + k);
        for (int c = 0; c < 3; ++c) rgbt[4 * k + c] = r.col[c];
        rgbt[4 * k + 3] = r.trans;
    };
    if (fp64) {
        const Rule<double> R = Rule<double>::from_view(*v);
        parallel_for(n, nthreads, 64, [&](int64_t k) { one(R, k); });
    } else {
        const Rule<float> R = Rule<float>::from_view(*v);
        parallel_for(n, nthreads, 64, [&](int64_t k) { one(R, k); });
    }
    return BHR_OK;
}

int oracle_trace_volumetric(const bhr_view* v, const bhr_shade_params* p, const uint16_t* noise, const float* lut,
                            bhr_hit* out, float* rgbt, int nthreads, int fp64) {
    if (!v || v->width <= 0 || v->height <= 0) return BHR_ERR_INVALID_ARG;
    return oracle_trace_volumetric_pixels(v, p, noise, lut, nullptr, static_cast<int64_t>(v->width) * v->height, out,
                                          rgbt, nthreads, fp64);
}

// Shades a volumetric view: the records and the march's rgbt from oracle_trace_volumetric.
int oracle_shade_volumetric(const bhr_view* v, const bhr_hit* hits, const float* rgbt, const bhr_shade_params* p,
                            const uint16_t* noise, const float* lut, float* rgba, int nthreads) {
    if (!v || !hits || !rgbt || !p || !noise || !lut || !rgba || v->width <= 0 || v->height <= 0 ||
        v->disk_mode != BHR_DISK_VOLUMETRIC)
        return BHR_ERR_INVALID_ARG;
    const oracle::shade::Tex tx{noise, lut};
    parallel_for(v->height, nthreads, 1,
                 [&](int64_t j) { oracle::shade::shade_view(tx, *p, *v, hits, rgba, j, j + 1, rgbt); });
    return BHR_OK;
}

// The body-aware march (BHS_BODIES 1) of every pixel of a view: records, and per pixel what the
// shading after the loop needs (bhr_body_hit).
// idx: the listed pixels (j * width + i), out[k] / bout[k] belonging to idx[k]; NULL: every pixel.
int oracle_trace_bodies_pixels(const bhr_view* v, const bhr_body* bodies, int nb, const int64_t* idx, int64_t n,
                               bhr_hit* out, bhr_body_hit* bout, int nthreads, int fp64) {
    if (!view_ok(v) || nb < 0 || nb > BHR_MAX_BODIES || (nb > 0 && !bodies) || !out || !bout || n < 0)
        return BHR_ERR_INVALID_ARG;
    return trace_bodies_impl(v, bodies, nb, idx, n, out, bout, NoVolume{}, nullptr, nthreads, fp64);
}

int oracle_trace_bodies(const bhr_view* v, const bhr_body* bodies, int nb, bhr_hit* out, bhr_body_hit* bout,
                        int nthreads, int fp64) {
    if (!view_ok(v)) return BHR_ERR_INVALID_ARG;
    return oracle_trace_bodies_pixels(v, bodies, nb, nullptr, static_cast<int64_t>(v->width) * v->height, out, bout,
                                      nthreads, fp64);
}

// The body-aware march with the volumetric disk (BHS_BODIES 1, DISK_VOLUMETRIC) of the listed
// pixels (every pixel when idx is NULL): records, body records, and rgbt[4k..4k+3] = the colour
// the march gathered and the transmittance left.
int oracle_trace_bodies_volumetric_pixels(const bhr_view* v, const bhr_body* bodies, int nb, const bhr_shade_params* p,
                                          const uint16_t* noise, const float* lut, const int64_t* idx, int64_t n,
                                          bhr_hit* out, bhr_body_hit* bout, float* rgbt, int nthreads, int fp64) {
    if (!v || v->width <= 0 || v->height <= 0 || v->max_steps < 0 || v->disk_mode != BHR_DISK_VOLUMETRIC || nb < 0 ||
        nb > BHR_MAX_BODIES || (nb > 0 && !bodies) || !p || !noise || !lut || !out || !bout || !rgbt || n < 0)
        return BHR_ERR_INVALID_ARG;
    const oracle::shade::Tex tx{noise, lut};
    const float cx = v->cam_pos[0], cy = v->cam_pos[1], cz = v->cam_pos[2];
    const VolumeSampler vs{&tx, p, v->disk_inner, v->disk_outer, v->disk_thickness, std::sqrt(cx * cx + cy * cy + cz * cz)};
    return trace_bodies_impl(v, bodies, nb, idx, n, out, bout, vs, rgbt, nthreads, fp64);
}

int oracle_trace_bodies_volumetric(const bhr_view* v, const bhr_body* bodies, int nb, const bhr_shade_params* p,
                                   const uint16_t* noise, const float* lut, bhr_hit* out, bhr_body_hit* bout,
                                   float* rgbt, int nthreads, int fp64) {
    if (!v || v->width <= 0 || v->height <= 0) return BHR_ERR_INVALID_ARG;
    return oracle_trace_bodies_volumetric_pixels(v, bodies, nb, p, noise, lut, nullptr,
                                                 static_cast<int64_t>(v->width) * v->height, out, bout, rgbt, nthreads,
                                                 fp64);
}

// Shades a view marched with bodies and the volumetric disk: records, body records, the bodies
// and the march's rgbt.
int oracle_shade_bodies_volumetric(const bhr_view* v, const bhr_hit* hits, const bhr_body_hit* bh, const bhr_body* bodies,
                                   int nb, const float* rgbt, const bhr_shade_params* p, const uint16_t* noise,
                                   const float* lut, float* rgba, int nthreads) {
    if (!v || !hits || !bh || (nb > 0 && !bodies) || nb < 0 || nb > BHR_MAX_BODIES || !rgbt || !p || !noise || !lut ||
        !rgba || v->width <= 0 || v->height <= 0 || v->disk_mode != BHR_DISK_VOLUMETRIC)
        return BHR_ERR_INVALID_ARG;
    const oracle::shade::Tex tx{noise, lut};
    const float cx = v->cam_pos[0], cy = v->cam_pos[1], cz = v->cam_pos[2];
    const oracle::body::BodyPost post{&tx, bodies, nb, bh, v, std::sqrt(cx * cx + cy * cy + cz * cz),
                                      2.0f * v->tan_half_fov / float(v->height), p->time};
    parallel_for(v->height, nthreads, 1,
                 [&](int64_t j) { oracle::shade::shade_view(tx, *p, *v, hits, rgba, j, j + 1, rgbt, post); });
    return BHR_OK;
}

// Shades a view marched with bodies: its records, body records and the bodies.
int oracle_shade_bodies(const bhr_view* v, const bhr_hit* hits, const bhr_body_hit* bh, const bhr_body* bodies, int nb,
                        const bhr_shade_params* p, const uint16_t* noise, const float* lut, float* rgba, int nthreads) {
    if (!v || !hits || !bh || (nb > 0 && !bodies) || nb < 0 || nb > BHR_MAX_BODIES || !p || !noise || !lut || !rgba ||
        v->width <= 0 || v->height <= 0 || v->disk_mode == BHR_DISK_VOLUMETRIC)
        return BHR_ERR_INVALID_ARG;
    const oracle::shade::Tex tx{noise, lut};
    const float cx = v->cam_pos[0], cy = v->cam_pos[1], cz = v->cam_pos[2];
    const oracle::body::BodyPost post{&tx, bodies, nb, bh, v, std::sqrt(cx * cx + cy * cy + cz * cz),
                                      2.0f * v->tan_half_fov / float(v->height), p->time};
    parallel_for(v->height, nthreads, 1,
                 [&](int64_t j) { oracle::shade::shade_view(tx, *p, *v, hits, rgba, j, j + 1, nullptr, post); });
    return BHR_OK;
}

// A view of a benchmark configuration built without the product library, so that the CPU arm of
// the benchmark maps the oracle alone: the uniforms a camera on the sphere of radius r at
// inclination incl and azimuth azim (looking at the hole, roll 0) gives, with the Settings
// defaults (src/Settings.h:19-37), a preset (Settings::applyPreset, src/Settings.cpp:12-35,
// -1 = none), uTanHalfFov (src/Renderer.cpp:246) and the camera basis of lookRotation
// (src/Camera.cpp:12-23: glm::quat_cast by the largest component, then glm::mat3_cast,
// Camera.cpp:67). Float arithmetic in the reference's order, so the bytes equal the library's
// bhr_view_init + bhr_view_apply_preset + bhr_view_set_fov + bhr_view_orbit_pose.
int oracle_orbit_view(bhr_view* v, int term_mode, int preset, int width, int height, float fov_deg, double r,
                      double incl, double azim) {
    if (!v || term_mode < BHR_TERM_SHADER || term_mode > BHR_TERM_CPU || width <= 0 || height <= 0 || !(r > 0.0) ||
        !(fov_deg > 0.0f) || !(fov_deg < 180.0f) || preset < -1 || preset > 3)
        return -1;
    std::memset(v, 0, sizeof *v);
    v->width = width;
    v->height = height;
    v->max_steps = 450;
    v->step_scale = 0.05f;
    v->disk_step = 0.18f;
    v->disk_inner = 6.0f;
    v->disk_outer = 20.0f;
    v->disk_thickness = 0.035f;
    v->disk_mode = BHR_DISK_THIN;
    v->lensing = 1;
    v->term_mode = term_mode;
    v->escape_r = 1000.0f;
    v->promote_band = 1e-2f;
    v->promote_r = 2.5f;
    if (term_mode == BHR_TERM_CPU) {  // trace() defaults (Geodesic.h:107-108,119)
        v->max_steps = 200000;
        v->step_scale = 0.005f;
        v->capture_r = 2.01f;
        v->esc_tol = 1e-4f;
        v->r_esc_min = 30.0f;
        v->ds_floor = 1e-4f;
        v->disk_mode = BHR_DISK_NONE;
    } else {  // R_HORIZON + 0.02 (frag:144) or the configurations' 2.0001; ESC_TOL; rEscMin (frag:89)
        v->capture_r = term_mode == BHR_TERM_SHADER ? 2.0f + 0.02f : 2.0001f;
        v->esc_tol = 0.01f;
        v->r_esc_min = std::max(v->disk_outer * 1.25f, 12.0f);
        v->ds_floor = 0.02f;
    }
    static const int kSteps[4] = {200, 300, 450, 700};
    static const float kScale[4] = {0.10f, 0.07f, 0.05f, 0.035f}, kDisk[4] = {0.35f, 0.30f, 0.18f, 0.10f};
    if (preset >= 0) {
        v->max_steps = kSteps[preset];
        v->step_scale = kScale[preset];
        v->disk_step = kDisk[preset];
    }
    v->tan_half_fov = std::tan(fov_deg * 0.01745329251994329576923690768489f * 0.5f);
    // lookRotation(pos, 0, up = +Y)
    const double pos[3] = {r * std::sin(incl) * std::sin(azim), r * std::cos(incl), r * std::sin(incl) * std::cos(azim)};
    const double len = std::sqrt(pos[0] * pos[0] + pos[1] * pos[1] + pos[2] * pos[2]);
    float f[3];  // (target - from) / |target - from|: 0.0 - pos keeps the sign of a zero component
    for (int k = 0; k < 3; ++k) f[k] = float((0.0 - pos[k]) / len);
    float u[3] = {0.0f, 1.0f, 0.0f};
    if (std::fabs(f[1]) > 0.999f) {  // dot(f, normalize(up)) with up = +Y
        u[0] = 0.0f;
        u[1] = 0.0f;
        u[2] = -1.0f;
    }
    float rt[3] = {f[1] * u[2] - u[1] * f[2], f[2] * u[0] - u[2] * f[0], f[0] * u[1] - u[0] * f[1]};
    const float rinv = 1.0f / std::sqrt(rt[0] * rt[0] + rt[1] * rt[1] + rt[2] * rt[2]);
    for (float& e : rt) e *= rinv;
    const float up[3] = {rt[1] * f[2] - f[1] * rt[2], rt[2] * f[0] - f[2] * rt[0], rt[0] * f[1] - f[0] * rt[1]};
    const float m[3][3] = {{rt[0], rt[1], rt[2]}, {up[0], up[1], up[2]}, {-f[0], -f[1], -f[2]}};  // m[col][row]
    const float t[4] = {m[0][0] + m[1][1] + m[2][2], m[0][0] - m[1][1] - m[2][2], m[1][1] - m[0][0] - m[2][2],
                        m[2][2] - m[0][0] - m[1][1]};
    int big = 0;
    for (int k = 1; k < 4; ++k)
        if (t[k] > t[big]) big = k;
    const float bv = std::sqrt(t[big] + 1.0f) * 0.5f, mult = 0.25f / bv;
    float q[4];  // w, x, y, z
    if (big == 0) {
        q[0] = bv; q[1] = (m[1][2] - m[2][1]) * mult; q[2] = (m[2][0] - m[0][2]) * mult; q[3] = (m[0][1] - m[1][0]) * mult;
    } else if (big == 1) {
        q[0] = (m[1][2] - m[2][1]) * mult; q[1] = bv; q[2] = (m[0][1] + m[1][0]) * mult; q[3] = (m[2][0] + m[0][2]) * mult;
    } else if (big == 2) {
        q[0] = (m[2][0] - m[0][2]) * mult; q[1] = (m[0][1] + m[1][0]) * mult; q[2] = bv; q[3] = (m[1][2] + m[2][1]) * mult;
    } else {
        q[0] = (m[0][1] - m[1][0]) * mult; q[1] = (m[2][0] + m[0][2]) * mult; q[2] = (m[1][2] + m[2][1]) * mult; q[3] = bv;
    }
    const float qn = 1.0f / std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
    for (float& e : q) e *= qn;
    // glm::mat3_cast(q): columns right, up, back
    const float qw = q[0], qx = q[1], qy = q[2], qz = q[3];
    const float xx = qx * qx, yy = qy * qy, zz = qz * qz, xz = qx * qz, xy = qx * qy, yz = qy * qz;
    const float wx = qw * qx, wy = qw * qy, wz = qw * qz;
    float* B = v->cam_basis;
    B[0] = 1.0f - 2.0f * (yy + zz); B[1] = 2.0f * (xy + wz);        B[2] = 2.0f * (xz - wy);
    B[3] = 2.0f * (xy - wz);        B[4] = 1.0f - 2.0f * (xx + zz); B[5] = 2.0f * (yz + wx);
    B[6] = 2.0f * (xz + wy);        B[7] = 2.0f * (yz - wx);        B[8] = 1.0f - 2.0f * (xx + yy);
    for (int k = 0; k < 3; ++k) v->cam_pos[k] = float(pos[k]);
    return 0;
}

int oracle_hit_size(void) { return static_cast<int>(sizeof(bhr_hit)); }
int oracle_view_size(void) { return static_cast<int>(sizeof(bhr_view)); }

}  // extern "C"
