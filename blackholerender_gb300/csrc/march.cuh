// Device-side Schwarzschild march, templated on the arithmetic type (float for the bulk,
// double for the mixed-precision band) and specialised at compile time on the termination
// rule and disk mode. Follows the reference shader:
//   shaders/geodesic.glsl:10-53   geoAccel, rk4Step, initialVelocity, bAxis, farFieldDirection
//   shaders/blackhole.frag:68-93  ray generation, per-ray constants (h, bAxis, farMul)
//   shaders/blackhole.frag:142-216 the loop body: horizon test, escape test, step size with the
//                                 disk-slab clamp, RK4 step, thin-disk plane crossing
//   src/physics/Geodesic.h:107-140 the CPU mirror's rule (BHR_TERM_CPU)
// The kernel is issue-bound, so the arithmetic is arranged for few instructions: one rsqrt
// per acceleration (r^-5 = rsqrt(r2)^5), r and |v| from rsqrt, the RK4 stage slopes folded
// into FMAs (k_v = a x is never formed), divisions and square roots off the common path.
#pragma once
#include <cstdint>

#include "bhr.h"

namespace bhr {

// Constants shared by every view of one launch (termination rule, disk geometry).
struct Rule {
    float capture_r;   // horizon test radius
    float escape_r;    // CONFIG escape radius
    float esc_tol;     // tolerance escape
    float r_esc_min;   // tolerance escape lower radius
    float ds_floor;    // smallest step
    float slab;        // 2.5 * disk_thickness (diskSlabHalfHeight(r) = slab * r, disk.glsl:24)
    float rcyl_lo2;    // (disk_inner - 1)^2, or -1 when disk_inner - 1 <= 0
    float rcyl_hi2;    // (disk_outer + 1)^2
    float disk_inner, disk_outer;
    float promote_r, promote_band;  // mixed precision
    int32_t term_mode, disk_mode, lensing, far_mode;
};

// Per-view geometry, precomputed on the host (api.cu: make_dev_view) in float with the
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
    float step_scale, disk_step;
    float two_over_r3;   // 2 / rcam^3 (impact parameter from h)
    int32_t tile_shift;  // a warp's 32 consecutive work items cover a (1 << tile_shift) x (32 >> tile_shift)
                         // pixel tile; 5 = plain row-major order (work item = pixel index)
    int32_t tiles_x;     // tiles per pixel row (tile_shift < 5)
    double cam_d[3];     // the same float uniforms promoted, for the FP64 path
    int64_t chunk_start; // first work chunk of this view (multi-view launches)
    int64_t nrays;       // width * height
    int64_t work;        // work items: nrays, or tiles * 32 (tile_shift < 5; edge tiles padded)
    bhr_hit* out;        // device hit buffer of this view
    int64_t list_off;    // offset of this view's pixel list (list launches)
};

template <class T> struct M;
template <> struct M<float> {
    static __device__ __forceinline__ float rsqrt(float x) { return rsqrtf(x); }
    static __device__ __forceinline__ float sqrt(float x) { return sqrtf(x); }
    static __device__ __forceinline__ float fdiv(float a, float b) { return __fdividef(a, b); }
    static __device__ __forceinline__ float fmax(float a, float b) { return fmaxf(a, b); }
    static __device__ __forceinline__ float fmin(float a, float b) { return fminf(a, b); }
    static __device__ __forceinline__ float fabs(float a) { return fabsf(a); }
    static __device__ __forceinline__ float atan2(float y, float x) { return atan2f(y, x); }
};
template <> struct M<double> {
    static __device__ __forceinline__ double rsqrt(double x) { return ::rsqrt(x); }
    static __device__ __forceinline__ double sqrt(double x) { return ::sqrt(x); }
    static __device__ __forceinline__ double fdiv(double a, double b) { return a / b; }
    static __device__ __forceinline__ double fmax(double a, double b) { return ::fmax(a, b); }
    static __device__ __forceinline__ double fmin(double a, double b) { return ::fmin(a, b); }
    static __device__ __forceinline__ double fabs(double a) { return ::fabs(a); }
    static __device__ __forceinline__ double atan2(double y, double x) { return ::atan2(y, x); }
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
    T b;         // impact parameter h / |v_inf|
};

// The unit direction of pixel (i, j) of view w (blackhole.frag:68-72), in arithmetic type T.
template <class T>
__device__ __forceinline__ V3<T> pixel_dir(const DevView& w, int i, int j) {
    const T pxx = T(i) + T(0.5) + T(w.jitter[0]);
    const T pxy = T(j) + T(0.5) + T(w.jitter[1]);
    const T ndcx = pxx / T(w.width) * T(2) - T(1);
    const T ndcy = pxy / T(w.height) * T(2) - T(1);
    const T th = T(w.tan_half);
    // uResolution.x / uResolution.y: float in the shader, double on the FP64 path (near the
    // photon sphere a 1e-8 change of direction moves the exit direction by ~1e-3 rad)
    const T aspect = sizeof(T) == 8 ? T(w.width) / T(w.height) : T(w.aspect);
    V3<T> dc{ndcx * th * aspect, ndcy * th, T(-1)};
    T inv = M<T>::rsqrt(dot3(dc, dc));
    dc = {dc.x * inv, dc.y * inv, dc.z * inv};
    V3<T> d{T(w.basis[0]) * dc.x + T(w.basis[3]) * dc.y + T(w.basis[6]) * dc.z,
            T(w.basis[1]) * dc.x + T(w.basis[4]) * dc.y + T(w.basis[7]) * dc.z,
            T(w.basis[2]) * dc.x + T(w.basis[5]) * dc.y + T(w.basis[8]) * dc.z};
    inv = M<T>::rsqrt(dot3(d, d));
    return {d.x * inv, d.y * inv, d.z * inv};
}

// blackhole.frag:68-93 for pixel (i, j) of view w, in arithmetic type T.
template <class T>
__device__ __forceinline__ RayInit<T> setup_ray(const DevView& w, const Rule& R, int i, int j) {
    const V3<T> d = pixel_dir<T>(w, i, j);
    V3<T> cam;
    T baxis_scale, lapse;
    V3<T> rh;
    if constexpr (sizeof(T) == 8) {
        cam = {w.cam_d[0], w.cam_d[1], w.cam_d[2]};
        const double r = ::sqrt(dot3(cam, cam));
        baxis_scale = 1.0 / ::sqrt(::fmax(1.0 - 2.0 / r, 1e-6));
        rh = {cam.x / r, cam.y / r, cam.z / r};
        lapse = ::sqrt(::fmax(1.0 - 2.0 / r, 0.0));
    } else {
        cam = {w.cam[0], w.cam[1], w.cam[2]};
        baxis_scale = w.baxis_scale;
        rh = {w.rhat[0], w.rhat[1], w.rhat[2]};
        lapse = w.lapse;
    }
    RayInit<T> o;
    // impactParameterAboutAxis: -dot(cross(cam, dir), +Y) * inversesqrt(max(1-2/r, 1e-6))
    o.b_axis = -(cam.z * d.x - d.z * cam.x) * baxis_scale;
    if (R.lensing) {
        // initialVelocity (geodesic.glsl:27-34): v = normalize(nr f rhat + (d - nr rhat))
        const T nr = dot3(d, rh);
        const T nrf = nr * lapse - nr;
        V3<T> v{d.x + nrf * rh.x, d.y + nrf * rh.y, d.z + nrf * rh.z};
        const T inv = M<T>::rsqrt(dot3(v, v));
        v = {v.x * inv, v.y * inv, v.z * inv};
        const V3<T> hv{cam.y * v.z - v.y * cam.z, cam.z * v.x - v.z * cam.x, cam.x * v.y - v.x * cam.y};
        o.v = v;
        o.h2 = dot3(hv, hv);
        const T h = M<T>::sqrt(o.h2);
        // b = h / |v_inf| with |v_inf|^2 = |v|^2 - 2 h2 / r^3 (Geodesic.h:50-54 impactParameter)
        T two_over_r3;
        if constexpr (sizeof(T) == 8) {
            const double r = ::sqrt(dot3(cam, cam));
            two_over_r3 = 2.0 / (r * r * r);
        } else {
            two_over_r3 = w.two_over_r3;
        }
        o.b = h * M<T>::rsqrt(dot3(v, v) - o.h2 * two_over_r3);
        T far_mul = T(1);
        if (R.term_mode != BHR_TERM_CPU) far_mul = M<T>::fmin(M<T>::fmax((h - T(6)) / T(3), T(1)), T(3));
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
    const V3<T> vh{v.x * vi, v.y * vi, v.z * vi};
    const T ri = M<T>::rsqrt(dot3(x, x));
    const T p = dot3(x, vh);
    const V3<T> bv{x.x - p * vh.x, x.y - p * vh.y, x.z - p * vh.z};
    const T s = M<T>::fmin(M<T>::fmax(p * ri, T(0)), T(1));
    const T ri3 = ri * ri * ri;
    const T ops = T(1) + s;
    const T c2 = M<T>::fdiv((T(2) + s) * ri3 * ri, ops * ops);
    const T k = -h2 * vi;
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

// rk4Step (geodesic.glsl:16-23) for x'' = a(x) = k(x) x, k(x) = -3 h2 / r^5, with ri = 1/|x|
// already known. With h = dt/2 and c_j = h k(x_j) the stages are x2 = x + h v, x3 = x2 + h c1 x1,
// x4 = x + dt v + dt c2 x2, and the update collapses to
//   x' = x + (dt v + (dt/3)(c1 x1 + c2 x2 + c3 x3))
//   v' = v + (1/3)(c1 x1 + 2 c2 x2 + 2 c3 x3 + c4 x4)
// (algebraically the reference's k-sums; no slope vector is formed, one rounding onto x).
template <class T>
__device__ __forceinline__ void rk4_update(V3<T>& xs, V3<T>& vs, T h2, T dt, T ri) {
    const T hdt = T(0.5) * dt;
    const T hm = hdt * (T(-3) * h2);
    const V3<T> x = xs, v = vs;
    T q2 = ri * ri;
    const T c1 = hm * ri * (q2 * q2);
    const V3<T> x2{x.x + hdt * v.x, x.y + hdt * v.y, x.z + hdt * v.z};
    const V3<T> q1{c1 * x.x, c1 * x.y, c1 * x.z};                      // c1 x1
    T q = M<T>::rsqrt(dot3(x2, x2));
    q2 = q * q;
    const T c2 = hm * q * (q2 * q2);
    V3<T> P{c2 * x2.x, c2 * x2.y, c2 * x2.z};                          // c2 x2
    const T g = hdt * c1;
    const V3<T> x3{x2.x + g * x.x, x2.y + g * x.y, x2.z + g * x.z};
    q = M<T>::rsqrt(dot3(x3, x3));
    q2 = q * q;
    const T c3 = hm * q * (q2 * q2);
    P = {P.x + c3 * x3.x, P.y + c3 * x3.y, P.z + c3 * x3.z};           // + c3 x3
    const V3<T> dv{dt * v.x, dt * v.y, dt * v.z};
    const T e = dt * c2;
    const V3<T> x4{x2.x + hdt * v.x + e * x2.x, x2.y + hdt * v.y + e * x2.y, x2.z + hdt * v.z + e * x2.z};
    q = M<T>::rsqrt(dot3(x4, x4));
    q2 = q * q;
    const T c4 = hm * q * (q2 * q2);
    const V3<T> W{q1.x + P.x, q1.y + P.y, q1.z + P.z};
    const T dt3 = dt * T(1.0 / 3.0);
    xs = {x.x + (dv.x + dt3 * W.x), x.y + (dv.y + dt3 * W.y), x.z + (dv.z + dt3 * W.z)};
    const V3<T> U{W.x + P.x + c4 * x4.x, W.y + P.y + c4 * x4.y, W.z + P.z + c4 * x4.z};
    const T third = T(1.0 / 3.0);
    vs = {v.x + third * U.x, v.y + third * U.y, v.z + third * U.z};
}

// Compile-time variant of the loop body: kTerm = BHR_TERM_* or -1 (rule read at run time,
// with lensing and far mode); kDisk = BHR_DISK_NONE / BHR_DISK_THIN or -1.
template <int kTerm, int kDisk>
struct Variant {
    static constexpr bool generic = kTerm < 0 || kDisk < 0;
};

// One march iteration (blackhole.frag:143-216) for an active ray. Returns true when the ray
// stopped at the loop head this iteration (status set in s.info). Crossings inside
// [disk_inner, disk_outer] are written straight into the ray's own hit record `rec`.
template <class T, int kTerm, int kDisk, bool kMixed>
__device__ __forceinline__ bool march_step(const Rule& R, int max_steps, T disk_step, RayState<T>& s,
                                           bhr_hit* rec) {
    constexpr bool kGen = Variant<kTerm, kDisk>::generic;
    const int term = kGen ? R.term_mode : kTerm;
    const int disk = kGen ? R.disk_mode : kDisk;
    const bool lensing = kGen ? (R.lensing != 0) : true;
    if (kGen && R.far_mode) {  // blackhole.frag:138-140: no march, escDir = dir
        s.info |= uint32_t(BHR_STATUS_ESCAPED) << kStatusShift;
        return true;
    }
    // loop head `i < uMaxSteps` comes before the horizon test (blackhole.frag:142-144)
    if (s.steps >= uint32_t(max_steps)) {
        s.info |= uint32_t(BHR_STATUS_BUDGET) << kStatusShift;
        return true;
    }
    const T r2 = dot3(s.x, s.x);
    const T v2 = dot3(s.v, s.v);
    const T ri = M<T>::rsqrt(r2);
    const T vi = M<T>::rsqrt(v2);
    const T r = r2 * ri;
    s.min_r = M<T>::fmin(s.min_r, r);
    if (r < T(R.capture_r)) {
        s.info |= uint32_t(BHR_STATUS_CAPTURED) << kStatusShift;
        return true;
    }
    if constexpr (kMixed) {
        if (r < T(R.promote_r)) {
            s.info |= uint32_t(kPromote) << kStatusShift;
            return true;
        }
    }
    if (dot3(s.x, s.v) > T(0)) {
        bool esc;
        if (term == BHR_TERM_CONFIG) {
            esc = r > T(R.escape_r);
        } else {
            // 0.75 b^3 / r^4 < tol with b = h / |v|  ->  0.75 (h vi)^3 ri^4 < tol
            esc = false;
            if (r > T(R.r_esc_min)) {
                const T bh = M<T>::sqrt(s.h2) * vi;
                const T ri2 = ri * ri;
                esc = !lensing || T(0.75) * bh * bh * bh * (ri2 * ri2) < T(R.esc_tol);
            }
        }
        if (esc) {
            s.info |= uint32_t(BHR_STATUS_ESCAPED) << kStatusShift;
            return true;
        }
    }
    T ds = M<T>::fmax(s.ssf * r, T(R.ds_floor));
    if (term != BHR_TERM_CPU && disk != BHR_DISK_NONE) {
        const T rc2 = s.x.x * s.x.x + s.x.z * s.x.z;
        if (rc2 > T(R.rcyl_lo2) && rc2 < T(R.rcyl_hi2)) {
            const T slab = T(R.slab);
            const T outside = M<T>::fabs(s.x.y) - slab * (rc2 * M<T>::rsqrt(rc2));
            if (outside > T(0))  // land on the slab boundary (blackhole.frag:177-179)
                ds = M<T>::fmin(ds, M<T>::fmax(disk_step, M<T>::fdiv(outside, M<T>::fabs(s.v.y) * vi + slab)));
        }
    }
    const T dt = ds * vi;
    const V3<T> x0 = s.x;
    if (lensing) {
        rk4_update(s.x, s.v, s.h2, dt, ri);
    } else {
        s.x = {s.x.x + s.v.x * dt, s.x.y + s.v.y * dt, s.x.z + s.v.z * dt};
    }
    s.steps += 1;
    if ((s.x.y > T(0)) != (x0.y > T(0))) {
        if ((s.info & 0xffu) < 255u) s.info += 1u;
        if (disk == BHR_DISK_THIN) {
            // blackhole.frag:211-213: f = y0 / (y0 - y), hit = mix(x0, x, f); disk.glsl:114-116
            const T f = x0.y / (x0.y - s.x.y);
            const T g = T(1) - f;
            const T hx = x0.x * g + s.x.x * f;
            const T hz = x0.z * g + s.x.z * f;
            const T rh = M<T>::sqrt(hx * hx + hz * hz);
            const uint32_t nc = (s.info >> kNcrossShift) & 3u;
            if (rh >= T(R.disk_inner) && rh <= T(R.disk_outer) && nc < 3u) {
                rec->cross_r[nc] = float(rh);
                rec->cross_phi[nc] = float(M<T>::atan2(hz, hx));
                s.info += 1u << kNcrossShift;
            }
        }
    }
    return false;
}

}  // namespace bhr
