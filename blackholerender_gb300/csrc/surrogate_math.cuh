// Closed-form orbit skeleton of the learned surrogate (device, templated on float/double).
//
// Every ray lies in the plane through the hole spanned by the camera position and the initial
// velocity. In that plane u = 1/r obeys the first integral of the Binet equation u'' + u = 3u^2,
// the orbit shape of x'' = -3 h^2 x / r^5 (shaders/geodesic.glsl:3-5, src/physics/Geodesic.h:4-6):
//     (du/dphi)^2 = P(u) = 2u^3 - u^2 + 1/b^2 = 2 (u - u1)(u - u2)(u - u3).
// For b > sqrt(27) the roots are real, u1 < 0 < u2 < u3, and an ingoing ray turns at u2. The
// polar angle swept between u = a and the turning point is
//     I(a) = sqrt(2) sqrt(u2 - a) R_F((a - u1)(u3 - u2), (u2 - u1)(u3 - u2), (u3 - a)(u2 - u1))
// (Carlson's symmetric elliptic integral; B. C. Carlson, Numer. Algorithms 10 (1995), the
// duplication theorem and its Taylor series). The surrogate evaluates R_F with kBaseDup
// duplication steps only (one more near the photon sphere, base_sweep): that cheap baseline is
// what the network corrects.
//
// Position along an ingoing-then-outgoing orbit is the signed coordinate
//     sigma = -sqrt((u2 - u) / (u2 - uc))   ingoing leg  (camera -1 .. turning point 0)
//     sigma = +sqrt((u2 - u) / u2)          outgoing leg (turning point 0 .. infinity 1)
// in which the polar angle is smooth across the turning point.
#pragma once
#include <cstdint>

namespace bhr {
namespace orbit {

constexpr int kBaseDup = 1;  // R_F duplication steps of the baseline

// Arithmetic of the closed form. The double path (training targets) is exact IEEE. The float
// path (inference) uses the SFU's approximate square root and reciprocal (PTX sqrt.approx /
// rcp.approx, a few units in the last place): the baseline it feeds is corrected by the network,
// whose residual is three orders of magnitude larger, and the Newton iterations correct their
// own update errors.
template <class T> struct FM;
template <> struct FM<double> {
    static __host__ __device__ __forceinline__ double sqrt(double x) { return ::sqrt(x); }
    static __host__ __device__ __forceinline__ double rcp(double x) { return 1.0 / x; }
    static __host__ __device__ __forceinline__ double div(double a, double b) { return a / b; }
    static __host__ __device__ __forceinline__ double div_sqrt(double a, double b) { return a / ::sqrt(b); }
    static __host__ __device__ __forceinline__ double cbrt(double x) { return ::cbrt(x); }
};
template <> struct FM<float> {
    static __host__ __device__ __forceinline__ float sqrt(float x) {
#ifdef __CUDA_ARCH__
        float y;
        asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
        return y;
#else
        return ::sqrtf(x);
#endif
    }
    static __host__ __device__ __forceinline__ float rcp(float x) {
#ifdef __CUDA_ARCH__
        float y;
        asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
        return y;
#else
        return 1.0f / x;
#endif
    }
    static __host__ __device__ __forceinline__ float div(float a, float b) { return a * rcp(b); }
    static __host__ __device__ __forceinline__ float cbrt(float x) { return ::cbrtf(x); }
    static __host__ __device__ __forceinline__ float div_sqrt(float a, float b) {
#ifdef __CUDA_ARCH__
        float y;
        asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(b));
        return a * y;
#else
        return a / ::sqrtf(b);
#endif
    }
};
template <class T> __host__ __device__ __forceinline__ T tsqrt(T x) { return FM<T>::sqrt(x); }

template <class T> struct Roots {
    T u1, u2, u3;
    T d32;  // u3 - u2, formed without cancellation
    bool ok;
};

// Roots of 2u^3 - u^2 + 1/b^2 for b = sqrt(27) (1 + beta), beta > 0.
// Near the critical orbit (beta < 0.1), around its double root u = 1/3: with u = 1/3 + w,
// w^2 (1 + 2w) = D, D = 1/27 - 1/b^2 = beta (2 + beta) / (27 (1 + beta)^2); Newton from +-sqrt(D).
// Elsewhere the trigonometric solution of the cubic with theta = 2 asin(sqrt(27)/b), written in
// products of sines so that no root is a difference of nearly equal terms:
//   u2 = 2/3 sin(theta/6) sin(2pi/3 - theta/6),  u3 = 2/3 cos(theta/6 + pi/6) cos(theta/6 - pi/6),
//   u3 - u2 = sin((pi - theta)/3) / sqrt(3).
// sin(theta/6) comes from Newton on the triple-angle identity, so no library trigonometry is used.
template <class T, int kIters>
__host__ __device__ __forceinline__ Roots<T> roots(T beta) {
    Roots<T> r;
    r.ok = beta > T(0);
    if (beta >= T(0.1)) {
        // a = theta / 6 = asin(sqrt(27)/b) / 3 from sin(3a) = 3s - 4s^3 = y, s = sin(a) <= 0.371
        // (Newton; f' = 3 - 12 s^2 >= 1.35 here), then products of s and c = cos(a):
        //   u2 = s (sqrt(3) c + s) / 3,  u3 = (3 c^2 - s^2) / 6 ... written without cancellation,
        //   u3 - u2 = (sqrt(3) (c^2 - s^2) - 2 s c) / 3 / sqrt(3) * sqrt(3)   (sin(pi/3 - 2a) / sqrt(3))
        const T y = FM<T>::rcp(T(1) + beta);
        // first guess from the series of the inverse, s = y/3 + 4 y^3/81 + 16 y^5/729 + ... (within
        // 5% at beta = 0.1); Newton then reaches FP32 precision in 3 steps and FP64 in 5
        const T y2 = y * y;
        T sa = y * (T(1.0 / 3.0) + y2 * (T(4.0 / 81.0) + y2 * T(16.0 / 729.0)));
        constexpr int kNewton = sizeof(T) == 4 ? 3 : 5;
#pragma unroll 1
        for (int k = 0; k < kNewton; ++k) sa -= FM<T>::div(T(3) * sa - T(4) * sa * sa * sa - y, T(3) - T(12) * sa * sa);
        const T ca = tsqrt<T>(T(1) - sa * sa);
        const T r3 = T(1.7320508075688772);
        // u2 = 2/3 sin(a) sin(2pi/3 - a) = 2/3 s (r3/2 c + s/2)
        r.u2 = T(1.0 / 3.0) * sa * (r3 * ca + sa);
        // u3 = 2/3 cos(a + pi/6) cos(a - pi/6) = 2/3 ((r3/2 c)^2 - (s/2)^2)
        r.u3 = T(1.0 / 6.0) * (T(3) * ca * ca - sa * sa);
        r.u1 = T(0.5) - r.u2 - r.u3;
        // u3 - u2 = sin(pi/3 - 2a) / sqrt(3) = (r3/2 cos 2a - 1/2 sin 2a) / r3
        const T c2a = ca * ca - sa * sa, s2a = T(2) * sa * ca;
        r.d32 = (T(0.5) * c2a - T(0.5) / r3 * s2a);
        return r;
    }
    const T ob = T(1) + beta;
    const T D = FM<T>::div(beta * (T(2) + beta), T(27) * ob * ob);
    const T sd = tsqrt<T>(D > T(0) ? D : T(0));
    T wp = sd, wm = -sd;
#pragma unroll
    for (int k = 0; k < kIters; ++k) {
        wp -= FM<T>::div(wp * wp * (T(1) + T(2) * wp) - D, wp * (T(2) + T(6) * wp));
        wm -= FM<T>::div(wm * wm * (T(1) + T(2) * wm) - D, wm * (T(2) + T(6) * wm));
    }
    r.u2 = T(1) / T(3) + wm;
    r.u3 = T(1) / T(3) + wp;
    r.u1 = T(0.5) - r.u2 - r.u3;
    r.d32 = wp - wm;
    return r;
}

// Carlson R_F(x, y, z) with N duplication steps and the fifth-order Taylor series.
template <class T, int N>
__host__ __device__ __forceinline__ T rf(T x, T y, T z) {
#pragma unroll 1
    for (int k = 0; k < N; ++k) {
        const T sx = tsqrt<T>(x), sy = tsqrt<T>(y), sz = tsqrt<T>(z);
        const T lam = sx * sy + sy * sz + sz * sx;
        x = T(0.25) * (x + lam);
        y = T(0.25) * (y + lam);
        z = T(0.25) * (z + lam);
    }
    const T A = (x + y + z) * T(1.0 / 3.0);
    const T iA = FM<T>::rcp(A);
    const T X = T(1) - x * iA, Y = T(1) - y * iA, Z = -(X + Y);
    const T E2 = X * Y - Z * Z, E3 = X * Y * Z;
    const T s = T(1) - E2 * T(0.1) + E3 * T(1.0 / 14.0) + E2 * E2 * T(1.0 / 24.0) - T(3.0 / 44.0) * E2 * E3;
    return FM<T>::div_sqrt(s, A);
}

// I(a): polar angle between u = a and the turning point u2 (a <= u2).
template <class T, int N>
__host__ __device__ __forceinline__ T sweep_to_turn(T a, const Roots<T>& R) {
    const T da = R.u2 - a;
    const T X = (a - R.u1) * R.d32;
    const T Y = (R.u2 - R.u1) * R.d32;
    const T Z = (R.u3 - a) * (R.u2 - R.u1);
    return T(1.4142135623730951) * tsqrt<T>(da > T(0) ? da : T(0)) * rf<T, N>(X, Y, Z);
}

// The baseline the network corrects. With one duplication step the closed form's error grows
// towards the photon sphere (to ~0.07 rad), beyond what a BF16 network resolves to 1e-4 rad;
// there a second step (error ~4^-6 of the first) is blended in: weight 1 for beta < kBlendLo,
// 0 for beta > kBlendHi, smoothstep between, so the residual the network learns stays smooth.
constexpr double kBlendLo = 0.002, kBlendHi = 0.02;

template <class T>
__host__ __device__ __forceinline__ T base_blend(T beta) {
    T x = (T(kBlendHi) - beta) * T(1.0 / (kBlendHi - kBlendLo));
    x = x < T(0) ? T(0) : (x > T(1) ? T(1) : x);
    return x * x * (T(3) - T(2) * x);
}

template <class T>
__host__ __device__ __forceinline__ T base_sweep(T a, const Roots<T>& R, T blend) {
    const T I1 = sweep_to_turn<T, kBaseDup>(a, R);
    if (!(blend > T(0))) return I1;
    return I1 + blend * (sweep_to_turn<T, kBaseDup + 1>(a, R) - I1);
}

// The closed form a surrogate variant evaluates: kNet (the learned path) the cheap baseline the
// network corrects (base_sweep); otherwise the converged closed form, R_F with kClosedDup
// duplication steps everywhere (error below 1e-8 rad on these orbits, no network).
constexpr int kClosedDup = 3;
template <bool kNet> struct Baseline {
    template <class T>
    static __host__ __device__ __forceinline__ T sweep(T a, const Roots<T>& R, T beta) {
        if constexpr (kNet) return base_sweep<T>(a, R, base_blend<T>(beta));
        else return sweep_to_turn<T, kClosedDup>(a, R);
    }
};

// u at orbit coordinate sigma (see the file comment).
template <class T>
__host__ __device__ __forceinline__ T u_of_sigma(T sigma, T uc, const Roots<T>& R) {
    const T s2 = sigma * sigma;
    return sigma < T(0) ? R.u2 - s2 * (R.u2 - uc) : R.u2 - s2 * R.u2;
}

// sigma of the exit radius u_e on the outgoing leg.
template <class T>
__host__ __device__ __forceinline__ T sigma_exit(T ue, const Roots<T>& R) {
    const T q = (R.u2 - ue) / R.u2;
    return tsqrt<T>(q > T(0) ? q : T(0));
}

// The exit u of the tolerance escape (the SHADER and CPU rules, blackhole.frag:151-155,
// Geodesic.h:125-129) in the continuum limit of the march's steps: the escape test passes on the
// outgoing leg once r > r_esc_min and 0.75 b'^3 / r^4 < tol, where b' = h / |v| is taken with
// the current speed. The energy integral of x'' = -3 h^2 x / r^5 gives |v|^2 = |v_inf|^2 +
// 2 h^2 u^3, so b' = b / sqrt(1 + 2 b^2 u^3). Along the outgoing leg the estimate falls
// monotonically (its log-derivative in r is (9 q / (1 + 2 q) - 4) / r with q = b^2 u^3 =
// u2 / (1 - 2 u2) <= 1 at the turning point and less beyond it), so the test first passes at
// u_e = min(1 / r_esc_min, u_tol, u2): never before the turning point, where x.v turns positive.
// u_tol solves u^4 = c^4 (1 + 2 b^2 u^3)^(3/2), c = (tol / (0.75 b^3))^(1/4), by fixed-point
// iteration from c; the iteration contracts by 9 q / (4 (1 + 2 q)), below 0.06 here (q < 0.03 at
// u_tol for b <= 60 and tol <= 0.01), so five iterations reach float precision.
template <class T>
__host__ __device__ __forceinline__ T exit_u_tol(T b, T tol, T u_esc_min, T u2) {
    const T c = tsqrt<T>(tsqrt<T>(FM<T>::div(tol, T(0.75) * b * b * b)));
    const T b2 = b * b;
    T u = c;
#pragma unroll 1
    for (int k = 0; k < 5; ++k) {
        const T w = T(1) + T(2) * b2 * u * u * u;
        u = c * tsqrt<T>(tsqrt<T>(tsqrt<T>(w * w * w)));  // c w^(3/8)
    }
    u = u < u_esc_min ? u : u_esc_min;
    return u < u2 ? u : u2;
}

// Baseline polar angle from the camera to orbit coordinate sigma: Ic -+ I(u(sigma)).
template <class T, int N>
__host__ __device__ __forceinline__ T phi_base(T sigma, T uc, T Ic, const Roots<T>& R) {
    const T I = sweep_to_turn<T, N>(u_of_sigma(sigma, uc, R), R);
    return sigma < T(0) ? Ic - I : Ic + I;
}

// sqrt(P(u)) = |du/dphi| on the orbit.
template <class T>
__host__ __device__ __forceinline__ T dudphi(T u, const Roots<T>& R) {
    const T p = T(2) * (u - R.u1) * (R.u2 - u) * (R.u3 - u);
    return tsqrt<T>(p > T(0) ? p : T(0));
}

// One duplication step of R_F(x, y, z), with sqrt(y) given.
template <class T>
__host__ __device__ __forceinline__ void rf_dup(T& x, T& y, T& z, T sy) {
    const T sx = tsqrt<T>(x), sz = tsqrt<T>(z);
    const T lam = sx * sy + sy * sz + sz * sx;
    x = T(0.25) * (x + lam);
    y = T(0.25) * (y + lam);
    z = T(0.25) * (z + lam);
}
// R_F after its duplication steps: the fifth-order series at the mean of (x, y, z), as rf.
template <class T>
__host__ __device__ __forceinline__ T rf_tail(T x, T y, T z) {
    const T A = (x + y + z) * T(1.0 / 3.0);
    const T iA = FM<T>::rcp(A);
    const T X = T(1) - x * iA, Y = T(1) - y * iA, Z = -(X + Y);
    const T E2 = X * Y - Z * Z, E3 = X * Y * Z;
    const T s = T(1) - E2 * T(0.1) + E3 * T(1.0 / 14.0) + E2 * E2 * T(1.0 / 24.0) - T(3.0 / 44.0) * E2 * E3;
    return FM<T>::div_sqrt(s, A);
}

// Solves I(u) = target for u in [0, u2] on a variant's closed form (Baseline<kNet>::sweep), by
// Newton in s = sqrt(u2 - u) as invert_sweep below, with the sweep written for it: in
// I = sqrt(2) s R_F((u - u1) d32, (u2 - u1) d32, (u3 - u)(u2 - u1)) the factor sqrt(u2 - u) is s,
// the middle argument and its square root are the same at every u, the first guess is the slope
// at the turning point, sqrt(2) R_F(y, y, y) = sqrt(2 / y), and the learned variant's second
// duplication step (its blend near the photon sphere) continues from the first.
template <class T, int kIters, bool kNet>
__host__ __device__ __forceinline__ T invert_sweep_v(T target, const Roots<T>& R, T beta) {
    const T d21 = R.u2 - R.u1;
    const T Y = d21 * R.d32;
    const T sY = tsqrt<T>(Y);
    const T smax = tsqrt<T>(R.u2);
    T s = target * sY * T(0.70710678118654752);
    s = s < T(0) ? T(0) : (s > smax ? smax : s);
    const T blend = kNet ? base_blend<T>(beta) : T(0);
#pragma unroll 1
    for (int k = 0; k < kIters; ++k) {
        const T u = R.u2 - s * s;
        T x = (u - R.u1) * R.d32, y = Y, z = (R.u3 - u) * d21;
        rf_dup<T>(x, y, z, sY);
        T rfv;
        if constexpr (kNet) {
            static_assert(kBaseDup == 1, "the learned baseline takes one duplication step, two in its blend");
            rfv = rf_tail<T>(x, y, z);
            if (blend > T(0)) {
                rf_dup<T>(x, y, z, tsqrt<T>(y));
                rfv += blend * (rf_tail<T>(x, y, z) - rfv);
            }
        } else {
#pragma unroll
            for (int d = 1; d < kClosedDup; ++d) rf_dup<T>(x, y, z, tsqrt<T>(y));
            rfv = rf_tail<T>(x, y, z);
        }
        const T f = T(1.4142135623730951) * s * rfv - target;
        s -= f * T(0.5) * tsqrt<T>(T(2) * (u - R.u1) * (R.u3 - u));
        s = s < T(0) ? T(0) : (s > smax ? smax : s);
    }
    return R.u2 - s * s;
}

// Solves I(u) = target for u in [0, u2] on the baseline (base_sweep), by Newton in
// s = sqrt(u2 - u), where dI/ds = 2 / sqrt(2 (u - u1)(u3 - u)) is smooth through the turning point.
template <class T, int kIters>
__host__ __device__ __forceinline__ T invert_sweep(T target, const Roots<T>& R, T blend) {
    // I(s) ~ s * sqrt(2) R_F at the turning point for the first guess
    const T X0 = (R.u2 - R.u1) * R.d32;
    const T Z0 = R.d32 * (R.u2 - R.u1);
    const T slope0 = T(1.4142135623730951) * rf<T, kBaseDup>(X0, X0, Z0);
    const T smax = tsqrt<T>(R.u2);
    T s = FM<T>::div(target, slope0);
    s = s < T(0) ? T(0) : (s > smax ? smax : s);
#pragma unroll 1
    for (int k = 0; k < kIters; ++k) {
        const T u = R.u2 - s * s;
        const T f = base_sweep<T>(u, R, blend) - target;
        // dI/ds = 2 / sqrt(2 (u - u1)(u3 - u)): the step is f / (dI/ds)
        s -= f * T(0.5) * tsqrt<T>(T(2) * (u - R.u1) * (R.u3 - u));
        s = s < T(0) ? T(0) : (s > smax ? smax : s);
    }
    return R.u2 - s * s;
}

// ---- captured orbits (b < sqrt(27)): P(u) = 2 (u - u1)((u - p)^2 + q^2) has one real root
// u1 < 0 and u rises from the camera to the horizon without turning. With A^2 = (p - u1)^2 + q^2,
// w = u - u1 and cos(theta) = (A - w) / (A + w), the substitution of Byrd & Friedman (1971, 239.00)
// gives int du / sqrt(P) = F(theta, k) / sqrt(2 A), k^2 = (A + p - u1) / (2 A), the incomplete
// elliptic integral of the first kind F(theta, k) = sin(theta) R_F(cos^2, 1 - k^2 sin^2, 1)
// for theta <= pi/2 and 2 K(k) - F(pi - theta, k) beyond.
template <class T> struct CapOrbit {
    T u1, A, k2, K;  // real root, A, k^2, K(k) = R_F(0, 1 - k^2, 1)
    T c;             // 1 / b^2
};

template <class T, int N>
__host__ __device__ __forceinline__ CapOrbit<T> cap_orbit(T beta) {
    CapOrbit<T> o;
    const T ob = T(1) + beta;
    o.c = FM<T>::rcp(T(27) * ob * ob);
    // the real root of 2u^3 - u^2 + c: Newton from -cbrt(c/2), where the cubic is -u^2 < 0; the
    // cubic is increasing and concave for u < 0, so the iterates rise monotonically to the root
    T u = -FM<T>::cbrt(T(0.5) * o.c);
#pragma unroll 1
    for (int k = 0; k < 6; ++k) u -= FM<T>::div(T(2) * u * u * u - u * u + o.c, T(6) * u * u - T(2) * u);
    o.u1 = u;
    const T p = T(0.5) * (T(0.5) - u);                               // the roots sum to 1/2
    const T A2 = -FM<T>::div(o.c, T(2) * u) - T(2) * p * u + u * u;  // (p - u1)^2 + q^2, p^2 + q^2 = -c / (2 u1)
    o.A = tsqrt<T>(A2);
    o.k2 = FM<T>::div(o.A + p - u, T(2) * o.A);
    o.K = rf<T, N>(T(0), T(1) - o.k2, T(1));
    return o;
}

// F(theta(u), k) of the captured orbit.
template <class T, int N>
__host__ __device__ __forceinline__ T cap_F(T u, const CapOrbit<T>& o) {
    const T w = u - o.u1;
    const T apw = o.A + w;
    const T cth = FM<T>::div(o.A - w, apw);
    const T sth = T(2) * tsqrt<T>(o.A * w) * FM<T>::rcp(apw);
    const T f0 = sth * rf<T, N>(cth * cth, T(1) - o.k2 * sth * sth, T(1));
    return cth < T(0) ? T(2) * o.K - f0 : f0;
}

// Arctangent in float for the surrogate's per-ray angles: range reduction to a = min / max of
// |y|, |x| in [0, 1] (atan(1/a) = pi/2 - atan(a)), then atan(a) = a + a s Q(s), s = a^2, with Q of
// degree 7 fitted to (atan(a) - a) / (a s) by least squares weighted by a s on 4000 Chebyshev
// nodes of [0, 1] (a near-minimax fit; its float evaluation stays within 7e-8 rad of atan,
// checked against numpy's arctan by tests/test_cpu_surrogate_math.py, which reads these constants).
// atan(a) for a in [0, 1]
__host__ __device__ __forceinline__ float atan_unit(float a) {
    const float s = a * a;
    // Q(s) = c0 + c1 s + ... + c7 s^7, Horner from c7
    float q = 0.002599463565275073f;
    q = q * s + -0.015040560625493526f;
    q = q * s + 0.04097096249461174f;
    q = q * s + -0.07353820651769638f;
    q = q * s + 0.1056785061955452f;
    q = q * s + -0.1418442726135254f;
    q = q * s + 0.19990207254886627f;
    q = q * s + -0.33332979679107666f;
    return a + a * s * q;
}
// atan(y / x) in [-pi/2, pi/2]
__host__ __device__ __forceinline__ float atan_ratio(float y, float x) {
    const float ax = x < 0.f ? -x : x, ay = y < 0.f ? -y : y;
    const float mx = ax > ay ? ax : ay, mn = ax > ay ? ay : ax;
    float r = mx > 0.f ? atan_unit(FM<float>::div(mn, mx)) : 0.f;
    if (ay > ax) r = 1.57079632679489662f - r;
    return (x < 0.f) != (y < 0.f) ? -r : r;
}
// atan2(y, x) in (-pi, pi]
__host__ __device__ __forceinline__ float atan2_fast(float y, float x) {
    const float r = atan_ratio(y, x);
    if (x >= 0.f) return r;
    return y >= 0.f ? r + 3.14159265358979f : r - 3.14159265358979f;
}

// Monotone transform of b / sqrt(27): t = sign(beta) ln(1 + |beta| / eps).
template <class T>
__host__ __device__ __forceinline__ T b_transform(T beta, T eps) {
    const T a = beta < T(0) ? -beta : beta;
    const T t = log1p(a / eps);
    return beta < T(0) ? -t : t;
}

}  // namespace orbit
}  // namespace bhr
