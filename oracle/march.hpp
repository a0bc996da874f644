// CPU restatement of the reference's per-pixel march -- TEST INFRASTRUCTURE ONLY.
//
// This is the oracle the CUDA kernels are checked against. It is never linked into the
// product library (blackholerender_gb300/libbhr.so); only tests/, __graft_entry__.smoke()
// and bench.py's CPU-baseline leg load it.
//
// It restates, line by line and templated on the arithmetic type T (double = the FP64 oracle,
// float = the FP32 behaviour check):
//   shaders/geodesic.glsl:10-53       geoAccel, rk4Step, initialVelocity,
//                                     impactParameterAboutAxis, farFieldDirection
//   shaders/common.glsl:7-14          R_HORIZON, B_CRIT, disk modes
//   shaders/disk.glsl:24,113-116      slab half-height, crossing radius/azimuth + range test
//   shaders/blackhole.frag:67-93      ray generation and per-ray constants
//   shaders/blackhole.frag:138-216,252  march loop (variant BHS_BODIES 0, BHS_GAS 0, thin disk)
//   shaders/blackhole.frag:169-181,217-234  volumetric disk: the 6 diskStep clamp in the slab,
//                                     Hermite sub-samples of each RK4 segment, opacity stop
//                                     (the sample itself is the caller's `vol`, oracle/shade.hpp)
//   shaders/blackhole.frag:101-121,146-150,182-190,236-250  bodies (BHS_BODIES 1): near-field
//                                     straight test, step clamps, chord intersections (`bod`)
//   src/physics/Geodesic.h:107-140    trace(), the CPU mirror's loop (BHR_TERM_CPU)
// Vector formulas follow GLM/GLSL definitions (dot = (x+y)+z, normalize = v * (1/sqrt(dot)),
// mix(a,b,t) = a*(1-t) + b*t) so the double path reproduces the reference's CPU code bit for
// bit when built with -ffp-contract=off.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <limits>

#include "bhr.h"

namespace oracle {

template <class T>
struct V3 {
    T x, y, z;
};
template <class T> inline V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> inline V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> inline V3<T> operator-(V3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> inline V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> inline V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> inline V3<T> operator/(V3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <class T> inline T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> inline T length(V3<T> a) { return std::sqrt(dot(a, a)); }
template <class T> inline V3<T> normalize(V3<T> a) { return a * (T(1) / std::sqrt(dot(a, a))); }
template <class T> inline V3<T> cross(V3<T> a, V3<T> b) {
    return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}

// geodesic.glsl:10-14 / Geodesic.h:21-25
template <class T> inline V3<T> geoAccel(V3<T> x, T h2) {
    const T r2 = dot(x, x);
    const T r = std::sqrt(r2);
    return x * (T(-3) * h2 / (r2 * r2 * r));
}

// geodesic.glsl:16-23 / Geodesic.h:27-34
template <class T> inline void rk4Step(V3<T>& x, V3<T>& v, T h2, T dt) {
    const T hdt = T(0.5) * dt;
    const V3<T> k1v = geoAccel(x, h2), k1x = v;
    const V3<T> k2v = geoAccel(x + hdt * k1x, h2), k2x = v + hdt * k1v;
    const V3<T> k3v = geoAccel(x + hdt * k2x, h2), k3x = v + hdt * k2v;
    const V3<T> k4v = geoAccel(x + dt * k3x, h2), k4x = v + dt * k3v;
    const T s = dt / T(6);
    x = x + s * (k1x + T(2) * k2x + T(2) * k3x + k4x);
    v = v + s * (k1v + T(2) * k2v + T(2) * k3v + k4v);
}

// geodesic.glsl:27-34 / Geodesic.h:40-47
template <class T> inline V3<T> initialVelocity(V3<T> camPos, V3<T> dir) {
    const T r = length(camPos);
    const V3<T> rhat = camPos / r;
    const T nr = dot(dir, rhat);
    const V3<T> nperp = dir - nr * rhat;
    const T f = std::sqrt(std::max(T(1) - T(2) / r, T(0)));
    return normalize(nr * f * rhat + nperp);
}

// geodesic.glsl:37-40 (shader form: inversesqrt(max(1 - 2/r, 1e-6)), axis = +Y)
template <class T> inline T impactParameterAboutY(V3<T> camPos, V3<T> dir) {
    const T r = length(camPos);
    const V3<T> c = cross(camPos, dir);
    return -c.y * (T(1) / std::sqrt(std::max(T(1) - T(2) / r, T(1e-6))));
}

// geodesic.glsl:43-53 / Geodesic.h:65-75
template <class T> inline V3<T> farFieldDirection(V3<T> x, V3<T> v, T h2) {
    const T vlen = length(v);
    const V3<T> vh = v / vlen;
    const T r = length(x);
    const T p = dot(x, vh);
    const V3<T> bvec = x - p * vh;
    const T s = std::clamp(p / r, T(0), T(1));
    const T r3 = r * r * r;
    const V3<T> dv = -(h2 / vlen) * (vh / r3 + bvec * ((T(2) + s) / (r3 * r * (T(1) + s) * (T(1) + s))));
    return normalize(v + dv);
}

// Termination and step rule constants of one view, in the arithmetic type T.
template <class T>
struct Rule {
    int term_mode = BHR_TERM_SHADER;
    int max_steps = 450;
    int disk_mode = BHR_DISK_THIN;
    bool lensing = true;
    bool far_mode = false;
    T step_scale = T(0.05), disk_step = T(0.18);
    T disk_inner = T(6), disk_outer = T(20), disk_thickness = T(0.035);
    T capture_r = T(2.02f), escape_r = T(1000), esc_tol = T(0.01f), r_esc_min = T(25), ds_floor = T(0.02f);

    static Rule from_view(const bhr_view& w) {
        Rule r;
        r.term_mode = w.term_mode;
        r.max_steps = w.max_steps;
        r.disk_mode = w.disk_mode;
        r.lensing = w.lensing != 0;
        r.far_mode = w.far_mode != 0;
        r.step_scale = T(w.step_scale);
        r.disk_step = T(w.disk_step);
        r.disk_inner = T(w.disk_inner);
        r.disk_outer = T(w.disk_outer);
        r.disk_thickness = T(w.disk_thickness);
        r.capture_r = T(w.capture_r);
        r.escape_r = T(w.escape_r);
        r.esc_tol = T(w.esc_tol);
        // blackhole.frag:89 derives rEscMin from uDiskOuter; the CPU mirror takes it as an argument
        r.r_esc_min = w.term_mode == BHR_TERM_SHADER ? T(std::max(w.disk_outer * 1.25f, 12.0f)) : T(w.r_esc_min);
        r.ds_floor = T(w.ds_floor);
        return r;
    }
};

template <class T>
struct Result {
    int status = 0;
    int steps = 0;
    int ncross = 0;
    int nplane = 0;
    bool nonfinite = false;
    V3<T> dir{0, 0, 0};
    T b = 0, b_axis = 0;
    T min_r = std::numeric_limits<T>::infinity();
    T cross_r[3] = {0, 0, 0};
    T cross_phi[3] = {0, 0, 0};
    V3<T> x{0, 0, 0}, v{0, 0, 0};  // final state (for tests)
    float col[3] = {0.0f, 0.0f, 0.0f};  // volumetric disk: emission gathered front to back
    float trans = 1.0f;                 // and the transmittance left
};

// Sub-samples per segment are bounded: inside the slab ds <= 6 diskStep, so a finite segment
// needs at most 7; the bound only stops a non-finite segment from looping.
constexpr int kMaxSubSamples = 64;

struct NoVolume {
    template <class... A> void operator()(A&&...) const {}
};

// The march without bodies (BHS_BODIES 0).
template <class T> struct NoBodies {
    void setup(const V3<T>&, const V3<T>&, const V3<T>&, bool, T) {}
    bool reached_near() const { return false; }
    T clamp(const V3<T>&, T ds) const { return ds; }
    void advance(T) {}
    bool chord(const V3<T>&, const V3<T>&, T) { return false; }
};

// shaders/bodies.glsl:34-44 raySphere: nearest hit in (tMin, tMax), -1 if none
template <class T> inline T raySphere(V3<T> ro, V3<T> rd, V3<T> c, T r, T tMin, T tMax) {
    const V3<T> oc = ro - c;
    const T b = dot(oc, rd);
    const T cc = dot(oc, oc) - r * r;
    const T disc = b * b - cc;
    if (disc < T(0)) return T(-1);
    const T s = std::sqrt(disc);
    T t = -b - s;
    if (t <= tMin) t = -b + s;  // inside the sphere
    return (t > tMin && t < tMax) ? t : T(-1);
}

// The bodies of one view in the march (blackhole.frag:101-121 setup, :146-150 the near-field
// hit at the loop head, :182-190 step clamps, :236-250 the chord test after each step).
template <class T> struct BodyMarch {
    const bhr_body* b = nullptr;
    int n = 0;
    V3<T> rd_near{0, 0, 0};
    uint32_t near_mask = 0;
    int near_idx = -1;
    T near_t = T(1e30), near_tol = T(0), travelled = T(0);
    int hit = -1;
    V3<T> hit_ro{0, 0, 0}, hit_rd{0, 0, 0};
    T hit_t = T(0);

    static V3<T> xyz(const float* q) { return V3<T>{T(q[0]), T(q[1]), T(q[2])}; }

    void setup(const V3<T>& cam, const V3<T>& v, const V3<T>& dir, bool lensing, T h2) {
        const T rcam = length(cam);
        rd_near = lensing ? normalize(v) : dir;
        const T a_cam = lensing ? T(3) * h2 / std::max(rcam * rcam * rcam * rcam, T(1e-30)) : T(0);
        for (int k = 0; k < n; ++k) {
            const V3<T> rel = xyz(b[k].rel_pos);
            const T R = T(b[k].pos_radius[3]);
            const T t_straight = lensing ? std::sqrt(T(0.02) * R / std::max(a_cam, T(1e-30))) : T(1e30);
            if (length(rel) + std::max(R, T(b[k].ring[1])) < t_straight) near_mask |= 1u << k;
            const T t = raySphere(V3<T>{0, 0, 0}, rd_near, rel, R, T(0), std::min(t_straight, near_t));
            if (t > T(0)) {
                near_t = t;
                near_idx = k;
            }
        }
        near_tol = std::max(T(2e-6) * rcam, T(1e-9));
    }
    bool reached_near() const { return near_idx >= 0 && travelled + near_tol >= near_t; }
    T clamp(const V3<T>& x, T ds) const {
        if (near_idx >= 0) ds = std::min(ds, std::max(near_t - travelled, near_tol));
        for (int k = 0; k < n; ++k) {
            if (near_mask & (1u << k)) continue;
            const T R = T(b[k].pos_radius[3]);
            ds = std::min(ds, std::max(T(0.5) * (length(x - xyz(b[k].pos_radius)) - R), T(0.25) * R));
        }
        return ds;
    }
    void advance(T seg) { travelled += seg; }
    bool chord(const V3<T>& x0, const V3<T>& x, T seg) {
        if (n == 0 || !(seg > T(0))) return false;
        const V3<T> sd = (x - x0) / seg;
        T best = seg;
        for (int k = 0; k < n; ++k) {
            if (near_mask & (1u << k)) continue;
            const T t = raySphere(x0, sd, xyz(b[k].pos_radius), T(b[k].pos_radius[3]), T(0), best);
            if (t > T(0)) {
                best = t;
                hit = k;
                hit_ro = x0;
                hit_rd = sd;
                hit_t = t;
            }
        }
        return hit >= 0;
    }
};

// blackhole.frag:68-72: primary ray of pixel (i, j), row 0 at the bottom.
template <class T> inline V3<T> primaryRay(const bhr_view& w, int i, int j) {
    const T pxx = T(i) + T(0.5) + T(w.jitter[0]);
    const T pxy = T(j) + T(0.5) + T(w.jitter[1]);
    const T ndcx = pxx / T(w.width) * T(2) - T(1);
    const T ndcy = pxy / T(w.height) * T(2) - T(1);
    const T aspect = T(w.width) / T(w.height);
    const T th = T(w.tan_half_fov);
    const V3<T> dc = normalize(V3<T>{ndcx * th * aspect, ndcy * th, T(-1)});
    const float* B = w.cam_basis;  // column-major
    const V3<T> d{T(B[0]) * dc.x + T(B[3]) * dc.y + T(B[6]) * dc.z,
                  T(B[1]) * dc.x + T(B[4]) * dc.y + T(B[7]) * dc.z,
                  T(B[2]) * dc.x + T(B[5]) * dc.y + T(B[8]) * dc.z};
    return normalize(d);
}

template <class T> inline bool finite3(V3<T> a) {
    return std::isfinite(a.x) && std::isfinite(a.y) && std::isfinite(a.z);
}

// blackhole.frag:77-93 (setup) + :138-253 (march), or Geodesic.h:107-140 for BHR_TERM_CPU.
// For BHR_DISK_VOLUMETRIC, vol(p, r_cyl, sub, res) shades one sub-sample of a segment in the
// slab into res.col / res.trans (volumetricDiskStep).
template <class T, class Vol, class Bod> Result<T> march(const Rule<T>& R, V3<T> camPos, V3<T> dir, const Vol& vol, Bod& bod) {
    Result<T> res;
    const bool lensing = R.lensing && !R.far_mode;
    V3<T> x = camPos;
    V3<T> v = dir;
    T h2 = 0, h = 0;
    if (lensing) {
        v = initialVelocity(camPos, dir);
        const V3<T> hv = cross(x, v);
        h2 = dot(hv, hv);
        h = std::sqrt(h2);
    }
    res.b_axis = impactParameterAboutY(camPos, dir);
    // impact parameter b = h / |v_inf|, |v_inf|^2 = |v|^2 - 2 h^2 / r^3 (energy integral of
    // x'' = -3 h^2 x / r^5); equals Geodesic.h:50-54 impactParameter = r sin(alpha) / sqrt(1 - 2/r)
    if (lensing) {
        const T rc = length(camPos);
        res.b = h / std::sqrt(dot(v, v) - T(2) * h2 / (rc * rc * rc));
    }
    bod.setup(camPos, v, dir, lensing, h2);
    const bool shader_rule = R.term_mode != BHR_TERM_CPU;
    const T farMul = shader_rule ? std::clamp((h - T(6)) / T(3), T(1), T(3)) : T(1);
    const T slab = T(2.5) * R.disk_thickness;  // diskSlabHalfHeight(r) = slab * r (disk.glsl:24)
    int status = 0;
    V3<T> escDir = dir;
    int steps = 0;
    if (R.far_mode) {
        status = BHR_STATUS_ESCAPED;
        escDir = dir;
    } else {
        for (int i = 0; i < R.max_steps; ++i) {
            const T r = length(x);
            res.min_r = std::min(res.min_r, r);
            if (r < R.capture_r) {
                status = BHR_STATUS_CAPTURED;
                break;
            }
            const T vlen = length(v);
            if (bod.reached_near()) {  // reached the near-field body (blackhole.frag:146-150)
                status = BHR_STATUS_BODY;
                break;
            }
            if (dot(x, v) > T(0)) {
                bool esc = false;
                if (R.term_mode == BHR_TERM_CONFIG) {
                    esc = r > R.escape_r;
                } else if (r > R.r_esc_min) {
                    const T b = h / vlen;
                    esc = !lensing || T(0.75) * b * b * b / (r * r * r * r) < R.esc_tol;
                }
                if (esc) {
                    escDir = lensing ? farFieldDirection(x, v, h2) : normalize(v);
                    status = BHR_STATUS_ESCAPED;
                    break;
                }
            }
            T ds;
            bool near_disk = false;
            if (shader_rule) {
                ds = std::max(R.step_scale * r * farMul, R.ds_floor);
                if (R.disk_mode != BHR_DISK_NONE) {
                    const T rcyl = std::sqrt(x.x * x.x + x.z * x.z);
                    if (rcyl > R.disk_inner - T(1) && rcyl < R.disk_outer + T(1)) {
                        const T outside = std::fabs(x.y) - slab * rcyl;
                        if (outside > T(0)) {
                            ds = std::min(ds, std::max(R.disk_step, outside / (std::fabs(v.y) / vlen + slab)));
                        } else {
                            near_disk = true;  // inside the slab: sub-sampled below (blackhole.frag:173-175)
                            if (R.disk_mode == BHR_DISK_VOLUMETRIC) ds = std::min(ds, T(6) * R.disk_step);
                        }
                    }
                }
            } else {
                ds = std::max(R.step_scale * r, R.ds_floor);
            }
            ds = bod.clamp(x, ds);  // blackhole.frag:184-190
            const T dt = ds / vlen;
            const V3<T> x0 = x, v0 = v;
            if (lensing)
                rk4Step(x, v, h2, dt);
            else
                x = x + v * dt;
            steps = i + 1;
            const T seg = length(x - x0);
            bod.advance(seg);
            if ((x.y > T(0)) != (x0.y > T(0))) {
                if (res.nplane < 255) ++res.nplane;
                if (R.disk_mode == BHR_DISK_THIN) {
                    const T f = x0.y / (x0.y - x.y);
                    const V3<T> hit = x0 * (T(1) - f) + x * f;
                    const T rh = std::sqrt(hit.x * hit.x + hit.z * hit.z);
                    if (rh >= R.disk_inner && rh <= R.disk_outer && res.ncross < 3) {
                        res.cross_r[res.ncross] = rh;
                        res.cross_phi[res.ncross] = std::atan2(hit.z, hit.x);
                        ++res.ncross;
                    }
                }
            }
            if (R.disk_mode == BHR_DISK_VOLUMETRIC && near_disk) {
                // blackhole.frag:217-233: samples along the cubic Hermite interpolant of the segment
                const T nf = std::ceil(seg / R.disk_step);
                const int n = std::isfinite(nf) ? std::min(std::max(1, int(std::min(nf, T(kMaxSubSamples)))), kMaxSubSamples) : 1;
                const T sub = seg / T(n);
                const V3<T> m0 = dt * v0, m1 = dt * v;
                for (int k = 0; k < n; ++k) {
                    const T t = (T(k) + T(0.5)) / T(n);
                    const T t2 = t * t, t3 = t2 * t;
                    const V3<T> p = (T(2) * t3 - T(3) * t2 + T(1)) * x0 + (t3 - T(2) * t2 + t) * m0 +
                                    (T(-2) * t3 + T(3) * t2) * x + (t3 - t2) * m1;
                    const T rm = std::sqrt(p.x * p.x + p.z * p.z);
                    if (rm > R.disk_inner - T(0.5) && rm < R.disk_outer && std::fabs(p.y) < slab * rm)
                        vol(p, rm, sub, res);
                    if (res.trans < 0.004f) break;
                }
            }
            if (res.trans < 0.004f) {  // blackhole.frag:234
                status = BHR_STATUS_OPAQUE;
                break;
            }
            if (bod.chord(x0, x, seg)) {  // blackhole.frag:236-250
                status = BHR_STATUS_BODY;
                break;
            }
            if (!finite3(x) || !finite3(v)) {
                res.nonfinite = true;
                break;
            }
        }
        if (status == 0) status = BHR_STATUS_BUDGET;
    }
    res.status = status;
    res.steps = steps;
    res.dir = escDir;
    res.x = x;
    res.v = v;
    return res;
}

template <class T, class Vol> Result<T> march(const Rule<T>& R, V3<T> camPos, V3<T> dir, const Vol& vol) {
    NoBodies<T> none;
    return march(R, camPos, dir, vol, none);
}

template <class T> Result<T> march(const Rule<T>& R, V3<T> camPos, V3<T> dir) {
    return march(R, camPos, dir, NoVolume{});
}

template <class T> inline void toHit(const Result<T>& r, bhr_hit* o) {
    *o = bhr_hit{};
    o->status = static_cast<uint8_t>(r.status);
    o->ncross = static_cast<uint8_t>(r.ncross);
    o->flags = r.nonfinite ? BHR_FLAG_NONFINITE : 0;
    o->nplane = static_cast<uint8_t>(r.nplane);
    o->steps = static_cast<uint32_t>(r.steps);
    if (r.status == BHR_STATUS_ESCAPED) {  // dir is zero unless the ray escaped
        o->dir[0] = static_cast<float>(r.dir.x);
        o->dir[1] = static_cast<float>(r.dir.y);
        o->dir[2] = static_cast<float>(r.dir.z);
    }
    o->b_axis = static_cast<float>(r.b_axis);
    o->b = static_cast<float>(r.b);
    o->min_r = std::isfinite(r.min_r) ? static_cast<float>(r.min_r) : 0.0f;
    for (int k = 0; k < 3; ++k) {
        o->cross_r[k] = static_cast<float>(r.cross_r[k]);
        o->cross_phi[k] = static_cast<float>(r.cross_phi[k]);
    }
}

template <class T> inline Result<T> marchPixel(const bhr_view& w, const Rule<T>& R, int i, int j) {
    const V3<T> cam{T(w.cam_pos[0]), T(w.cam_pos[1]), T(w.cam_pos[2])};
    return march(R, cam, primaryRay<T>(w, i, j));
}

}  // namespace oracle
