// Device-side Schwarzschild march, templated on the arithmetic type (float for the bulk,
// double for the mixed-precision band). Follows the reference shader:
//   shaders/geodesic.glsl:10-53   geoAccel, rk4Step, initialVelocity, bAxis, farFieldDirection
//   shaders/blackhole.frag:68-93  ray generation, per-ray constants (h, bAxis, farMul)
//   shaders/blackhole.frag:142-216 the loop body: horizon test, escape test, step size with the
//                                 disk-slab clamp, RK4 step, thin-disk plane crossing
//   src/physics/Geodesic.h:107-140 the CPU mirror's rule (BHR_TERM_CPU)
// Arithmetic is rearranged for the SFU budget: one rsqrt per acceleration (r^-5 =
// rsqrt(r2)^5), |v| and r from rsqrt, divisions only off the common path.
#pragma once
#include <cstdint>

#include "bhr.h"

namespace bhr {

// Per-view constants, precomputed on the host (api.cpp: make_dev_view) in float with the
// reference's operation order, so every lane sees the uniforms blackhole.frag sees.
struct DevView {
    float cam[3];        // uCamPos
    float basis[9];      // uCamBasis, column-major
    float tan_half;      // uTanHalfFov
    float jitter[2];
    int32_t width, height;
    int32_t max_steps;
    float aspect;        // uResolution.x / uResolution.y
    float rcam;          // length(uCamPos)
    float rhat[3];       // uCamPos / rcam
    float lapse;         // sqrt(max(1 - 2/rcam, 0))          initialVelocity
    float baxis_scale;   // inversesqrt(max(1 - 2/rcam, 1e-6))  impactParameterAboutAxis
    float step_scale, disk_step, disk_inner, disk_outer;
    float slab;          // 2.5 * disk_thickness (diskSlabHalfHeight(r) = slab * r)
    float rcyl_lo2;      // (disk_inner - 1)^2, or -1 when disk_inner - 1 <= 0
    float rcyl_hi2;      // (disk_outer + 1)^2
    float capture_r, escape_r, esc_tol, r_esc_min, ds_floor;
    float promote_band, promote_r;
    int32_t disk_mode, lensing, far_mode, term_mode;
    double cam_d[3];     // the same float uniforms promoted, for the FP64 path
    int64_t chunk_start; // first work chunk of this view (batched launches)
    int64_t nrays;       // width * height
    bhr_hit* out;        // device hit buffer of this view
};

template <class T> struct M;
template <> struct M<float> {
    static __device__ __forceinline__ float rsqrt(float x) { return rsqrtf(x); }
    static __device__ __forceinline__ float sqrt(float x) { return sqrtf(x); }
    static __device__ __forceinline__ float rcp(float x) { return __frcp_rn(x); }
    static __device__ __forceinline__ float fmax(float a, float b) { return fmaxf(a, b); }
    static __device__ __forceinline__ float fmin(float a, float b) { return fminf(a, b); }
    static __device__ __forceinline__ float fabs(float a) { return fabsf(a); }
    static __device__ __forceinline__ float atan2(float y, float x) { return atan2f(y, x); }
    static __device__ __forceinline__ bool finite(float a) { return isfinite(a); }
};
template <> struct M<double> {
    static __device__ __forceinline__ double rsqrt(double x) { return ::rsqrt(x); }
    static __device__ __forceinline__ double sqrt(double x) { return ::sqrt(x); }
    static __device__ __forceinline__ double rcp(double x) { return 1.0 / x; }
    static __device__ __forceinline__ double fmax(double a, double b) { return ::fmax(a, b); }
    static __device__ __forceinline__ double fmin(double a, double b) { return ::fmin(a, b); }
    static __device__ __forceinline__ double fabs(double a) { return ::fabs(a); }
    static __device__ __forceinline__ double atan2(double y, double x) { return ::atan2(y, x); }
    static __device__ __forceinline__ bool finite(double a) { return isfinite(a); }
};

template <class T> struct V3 { T x, y, z; };
template <class T> __device__ __forceinline__ T dot3(const V3<T>& a, const V3<T>& b) {
    return a.x * b.x + a.y * b.y + a.z * b.z;
}

// State a lane needs to start a ray (x starts at the camera). Produced in bulk by
// setup_ray, parked in the warp's shared-memory pool, taken by idle lanes.
template <class T> struct RayInit {
    V3<T> v;     // initialVelocity(camPos, dir) (or dir when lensing is off)
    T h2;        // |x × v|^2
    T ssf;       // step_scale * farMul (shader rule) or step_scale (CPU rule)
    T b_axis;    // impactParameterAboutAxis(camPos, dir, +Y)
    T b;         // h / |v|
};

// blackhole.frag:68-93 for pixel (i, j) of view w, in arithmetic type T.
template <class T>
__device__ __forceinline__ RayInit<T> setup_ray(const DevView& w, int i, int j, V3<T>* dir_out) {
    const T pxx = T(i) + T(0.5) + T(w.jitter[0]);
    const T pxy = T(j) + T(0.5) + T(w.jitter[1]);
    const T ndcx = pxx / T(w.width) * T(2) - T(1);
    const T ndcy = pxy / T(w.height) * T(2) - T(1);
    const T th = T(w.tan_half);
    V3<T> dc{ndcx * th * T(w.aspect), ndcy * th, T(-1)};
    T inv = M<T>::rsqrt(dot3(dc, dc));
    dc = {dc.x * inv, dc.y * inv, dc.z * inv};
    V3<T> d{T(w.basis[0]) * dc.x + T(w.basis[3]) * dc.y + T(w.basis[6]) * dc.z,
            T(w.basis[1]) * dc.x + T(w.basis[4]) * dc.y + T(w.basis[7]) * dc.z,
            T(w.basis[2]) * dc.x + T(w.basis[5]) * dc.y + T(w.basis[8]) * dc.z};
    inv = M<T>::rsqrt(dot3(d, d));
    d = {d.x * inv, d.y * inv, d.z * inv};
    *dir_out = d;
    V3<T> cam;
    if constexpr (sizeof(T) == 8) cam = {w.cam_d[0], w.cam_d[1], w.cam_d[2]};
    else cam = {w.cam[0], w.cam[1], w.cam[2]};
    RayInit<T> o;
    const bool lensing = w.lensing != 0 && w.far_mode == 0;
    // impactParameterAboutAxis: -dot(cross(cam, dir), +Y) * inversesqrt(max(1-2/r, 1e-6))
    T baxis_scale;
    if constexpr (sizeof(T) == 8) {
        const double r = ::sqrt(dot3(cam, cam));
        baxis_scale = 1.0 / ::sqrt(::fmax(1.0 - 2.0 / r, 1e-6));
    } else {
        baxis_scale = w.baxis_scale;
    }
    o.b_axis = -(cam.z * d.x - d.z * cam.x) * baxis_scale;
    if (lensing) {
        // initialVelocity (geodesic.glsl:27-34)
        V3<T> rh;
        T lapse;
        if constexpr (sizeof(T) == 8) {
            const double r = ::sqrt(dot3(cam, cam));
            rh = {cam.x / r, cam.y / r, cam.z / r};
            lapse = ::sqrt(::fmax(1.0 - 2.0 / r, 0.0));
        } else {
            rh = {w.rhat[0], w.rhat[1], w.rhat[2]};
            lapse = w.lapse;
        }
        const T nr = dot3(d, rh);
        const T nrf = nr * lapse - nr;  // v = nr*f*rhat + (d - nr*rhat) = d + (nr*f - nr)*rhat
        V3<T> v{d.x + nrf * rh.x, d.y + nrf * rh.y, d.z + nrf * rh.z};
        inv = M<T>::rsqrt(dot3(v, v));
        v = {v.x * inv, v.y * inv, v.z * inv};
        const V3<T> hv{cam.y * v.z - v.y * cam.z, cam.z * v.x - v.z * cam.x, cam.x * v.y - v.x * cam.y};
        o.v = v;
        o.h2 = dot3(hv, hv);
        const T h = M<T>::sqrt(o.h2);
        o.b = h * M<T>::rsqrt(dot3(v, v));
        T far_mul = T(1);
        if (w.term_mode != BHR_TERM_CPU) far_mul = M<T>::fmin(M<T>::fmax((h - T(6)) / T(3), T(1)), T(3));
        o.ssf = T(w.step_scale) * far_mul;
    } else {
        o.v = d;
        o.h2 = T(0);
        o.b = T(0);
        o.ssf = T(w.step_scale);
    }
    return o;
}

// geodesic.glsl:43-53 farFieldDirection (first-order remaining deflection), normalised.
template <class T>
__device__ __forceinline__ V3<T> far_field_dir(const V3<T>& x, const V3<T>& v, T h2) {
    const T vi = M<T>::rsqrt(dot3(v, v));
    const T vlen_inv = vi;
    const V3<T> vh{v.x * vi, v.y * vi, v.z * vi};
    const T ri = M<T>::rsqrt(dot3(x, x));
    const T p = dot3(x, vh);
    const V3<T> bv{x.x - p * vh.x, x.y - p * vh.y, x.z - p * vh.z};
    const T s = M<T>::fmin(M<T>::fmax(p * ri, T(0)), T(1));
    const T ri3 = ri * ri * ri;
    const T ops = T(1) + s;
    const T c2 = (T(2) + s) * ri3 * ri / (ops * ops);
    const T k = -h2 * vlen_inv;
    V3<T> o{v.x + k * (vh.x * ri3 + bv.x * c2), v.y + k * (vh.y * ri3 + bv.y * c2),
            v.z + k * (vh.z * ri3 + bv.z * c2)};
    const T oi = M<T>::rsqrt(dot3(o, o));
    return {o.x * oi, o.y * oi, o.z * oi};
}

// Live state of one ray in a lane.
template <class T> struct RayState {
    V3<T> x, v;
    T h2, ssf;
    T min_r;
    uint32_t steps;
    uint32_t info;  // bits 0-7 nplane, 8-9 ncross, 12-15 status (0 marching)
};

enum : uint32_t { kStatusShift = 12, kNcrossShift = 8, kPromote = 4 };

// One march iteration (blackhole.frag:143-216) for an active ray. Returns true when the
// ray stopped at the loop head this iteration (status set in info). Crossings inside
// [disk_inner, disk_outer] are written straight into the ray's own hit record `rec`.
template <class T, bool kMixed>
__device__ __forceinline__ bool march_step(const DevView& w, RayState<T>& s, bhr_hit* rec) {
    if (w.far_mode != 0) {  // blackhole.frag:138-140: no march, escDir = dir
        s.info |= uint32_t(BHR_STATUS_ESCAPED) << kStatusShift;
        return true;
    }
    // loop head `i < uMaxSteps` comes before the horizon test (blackhole.frag:142-144)
    if (s.steps >= uint32_t(w.max_steps)) {
        s.info |= uint32_t(BHR_STATUS_BUDGET) << kStatusShift;
        return true;
    }
    const T r2 = dot3(s.x, s.x);
    const T ri = M<T>::rsqrt(r2);
    const T r = r2 * ri;
    s.min_r = M<T>::fmin(s.min_r, r);
    if (r < T(w.capture_r)) {
        s.info |= uint32_t(BHR_STATUS_CAPTURED) << kStatusShift;
        return true;
    }
    if constexpr (kMixed) {
        if (r < T(w.promote_r)) {
            s.info |= uint32_t(kPromote) << kStatusShift;
            return true;
        }
    }
    const T v2 = dot3(s.v, s.v);
    const T vi = M<T>::rsqrt(v2);
    const bool lensing = w.lensing != 0;
    if (dot3(s.x, s.v) > T(0)) {
        bool esc = false;
        if (w.term_mode == BHR_TERM_CONFIG) {
            esc = r > T(w.escape_r);
        } else if (r > T(w.r_esc_min)) {
            // 0.75 b^3 / r^4 < tol with b = h / |v|  ->  0.75 (h vi)^3 ri^4 < tol
            const T bh = M<T>::sqrt(s.h2) * vi;
            const T ri2 = ri * ri;
            esc = !lensing || T(0.75) * bh * bh * bh * (ri2 * ri2) < T(w.esc_tol);
        }
        if (esc) {
            s.info |= uint32_t(BHR_STATUS_ESCAPED) << kStatusShift;
            return true;
        }
    }
    T ds = M<T>::fmax(s.ssf * r, T(w.ds_floor));
    if (w.term_mode != BHR_TERM_CPU && w.disk_mode != BHR_DISK_NONE) {
        const T rc2 = s.x.x * s.x.x + s.x.z * s.x.z;
        if (rc2 > T(w.rcyl_lo2) && rc2 < T(w.rcyl_hi2)) {
            const T slab = T(w.slab);
            const T outside = M<T>::fabs(s.x.y) - slab * M<T>::sqrt(rc2);
            if (outside > T(0))
                ds = M<T>::fmin(ds, M<T>::fmax(T(w.disk_step), outside / (M<T>::fabs(s.v.y) * vi + slab)));
        }
    }
    const T dt = ds * vi;
    const T y0 = s.x.y;
    V3<T> x0 = s.x;
    if (lensing) {
        // rk4Step (geodesic.glsl:16-23); acceleration -3 h2 x / r^5
        const T hdt = T(0.5) * dt;
        const T m3h2 = T(-3) * s.h2;
        const V3<T> x = s.x, v = s.v;
        T ri2 = ri * ri;
        T a = m3h2 * (ri2 * ri2 * ri);
        const V3<T> k1v{x.x * a, x.y * a, x.z * a};
        V3<T> sx = v;                       // running sum of k*x (k1x = v)
        V3<T> sv = k1v;                     // running sum of k*v
        V3<T> xs{x.x + hdt * v.x, x.y + hdt * v.y, x.z + hdt * v.z};
        V3<T> vs{v.x + hdt * k1v.x, v.y + hdt * k1v.y, v.z + hdt * k1v.z};  // k2x
        T q = M<T>::rsqrt(dot3(xs, xs));
        T q2 = q * q;
        a = m3h2 * (q2 * q2 * q);
        V3<T> kv{xs.x * a, xs.y * a, xs.z * a};  // k2v
        sx = {sx.x + T(2) * vs.x, sx.y + T(2) * vs.y, sx.z + T(2) * vs.z};
        sv = {sv.x + T(2) * kv.x, sv.y + T(2) * kv.y, sv.z + T(2) * kv.z};
        xs = {x.x + hdt * vs.x, x.y + hdt * vs.y, x.z + hdt * vs.z};
        vs = {v.x + hdt * kv.x, v.y + hdt * kv.y, v.z + hdt * kv.z};  // k3x
        q = M<T>::rsqrt(dot3(xs, xs));
        q2 = q * q;
        a = m3h2 * (q2 * q2 * q);
        kv = {xs.x * a, xs.y * a, xs.z * a};  // k3v
        sx = {sx.x + T(2) * vs.x, sx.y + T(2) * vs.y, sx.z + T(2) * vs.z};
        sv = {sv.x + T(2) * kv.x, sv.y + T(2) * kv.y, sv.z + T(2) * kv.z};
        xs = {x.x + dt * vs.x, x.y + dt * vs.y, x.z + dt * vs.z};
        vs = {v.x + dt * kv.x, v.y + dt * kv.y, v.z + dt * kv.z};  // k4x
        q = M<T>::rsqrt(dot3(xs, xs));
        q2 = q * q;
        a = m3h2 * (q2 * q2 * q);
        kv = {xs.x * a, xs.y * a, xs.z * a};  // k4v
        sx = {sx.x + vs.x, sx.y + vs.y, sx.z + vs.z};
        sv = {sv.x + kv.x, sv.y + kv.y, sv.z + kv.z};
        const T s6 = dt * T(1.0 / 6.0);
        s.x = {x.x + s6 * sx.x, x.y + s6 * sx.y, x.z + s6 * sx.z};
        s.v = {v.x + s6 * sv.x, v.y + s6 * sv.y, v.z + s6 * sv.z};
    } else {
        s.x = {s.x.x + s.v.x * dt, s.x.y + s.v.y * dt, s.x.z + s.v.z * dt};
    }
    s.steps += 1;
    if ((s.x.y > T(0)) != (y0 > T(0))) {
        if ((s.info & 0xffu) < 255u) s.info += 1u;
        if (w.disk_mode == BHR_DISK_THIN) {
            // blackhole.frag:211-213: f = y0 / (y0 - y), hit = mix(x0, x, f); disk.glsl:114-116
            const T f = y0 / (y0 - s.x.y);
            const T g = T(1) - f;
            const T hx = x0.x * g + s.x.x * f;
            const T hz = x0.z * g + s.x.z * f;
            const T rh = M<T>::sqrt(hx * hx + hz * hz);
            const uint32_t nc = (s.info >> kNcrossShift) & 3u;
            if (rh >= T(w.disk_inner) && rh <= T(w.disk_outer) && nc < 3u) {
                rec->cross_r[nc] = float(rh);
                rec->cross_phi[nc] = float(M<T>::atan2(hz, hx));
                s.info += 1u << kNcrossShift;
            }
        }
    }
    if (!(M<T>::finite(s.x.x) && M<T>::finite(s.x.y) && M<T>::finite(s.x.z) && M<T>::finite(s.v.x) &&
          M<T>::finite(s.v.y) && M<T>::finite(s.v.z))) {
        s.info |= (uint32_t(BHR_STATUS_BUDGET) << kStatusShift) | (1u << 16);  // bit 16: non-finite
        return true;
    }
    return false;
}

}  // namespace bhr
