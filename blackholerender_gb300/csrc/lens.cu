// Lens table of the star-disruption particle renderer (shaders/gas_lens.comp, gas_lens.glsl):
// for a camera at radius r_cam, a fan of 1024 rays in one plane through the hole, at local angles
// alpha from the hole's direction (0) to straight away (pi), crowded at the shadow's edge; texel
// (ray i, angle j) holds log r of ray i once it has swept phi_j = j 2 pi / 1023 around the hole,
// log 2 after capture, log 2e5 after escape. table[j * 1024 + i].
//
// Two builders:
//   k_lens_integrate: the reference's own construction, one ray per thread, RK4 with
//     ds = (r < 8 ? 0.004 : 0.01) r and log r linear in r between steps (gas_lens.comp:22-40).
//     Near the shadow's edge rays wind for up to 20,000 steps, so the launch lasts as long as its
//     slowest ray, one thread's sequential chain.
//   k_lens_closed: every texel independently from the closed-form orbit: the Carlson R_F form of
//     the polar angle (escaping orbits, Newton in s = sqrt(u2 - u) through the turning point)
//     or the one-real-root elliptic form (captured orbits), one thread per texel. No step rule:
//     it is the orbit the integrator converges to (cameras outside the photon sphere).
#include <cuda_runtime.h>

#include "bhr.h"
#include "march.cuh"
#include "surrogate_math.cuh"

namespace bhr {

namespace {

constexpr int kRays = BHR_LENS_RAYS, kPhis = BHR_LENS_PHIS;
constexpr float kRMax = 2.0e5f;        // LENS_RMAX
constexpr float kTwoPi = 6.28318530717959f;
constexpr float kPi = 3.14159265358979f;

// gas_lens.glsl:13-17 lensAlpha (LENS_P = 3)
__host__ __device__ __forceinline__ float lens_alpha(float u, float ac) {
    const float uc = ac / kPi;
    if (u < uc) {
        const float q = (uc - u) / uc;
        return ac - ac * (q * q * q);
    }
    const float q = (u - uc) / (1.0f - uc);
    return ac + (kPi - ac) * (q * q * q);
}

__global__ void __launch_bounds__(64) k_lens_integrate(float cam_r, float ac, float* __restrict__ table) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kRays) return;
    const float a = lens_alpha((float(i) + 0.5f) / float(kRays), ac);
    float sa, ca;
    sincosf(a, &sa, &ca);
    // initialVelocity((r, 0, 0), (-cos a, sin a, 0)) (geodesic.glsl:27-34), camera on +X
    const float f = sqrtf(fmaxf(1.0f - 2.0f / cam_r, 0.0f));
    V3<float> v{-ca * f, sa, 0.f};
    const float vi0 = rsqrtf(dot3(v, v));
    v = {v.x * vi0, v.y * vi0, 0.f};
    V3<float> x{cam_r, 0.f, 0.f};
    const float h = cam_r * v.y;
    const float h2 = h * h;
    const float dphi_j = kTwoPi / float(kPhis - 1);
    const float logH = logf(2.0f);
    table[i] = logf(cam_r);
    int j = 1;
    float phi = 0.f, r = cam_r;
    for (int s = 0; s < 20000 && j < kPhis; ++s) {
        const float ds = (r < 8.0f ? 0.004f : 0.01f) * r;
        const V3<float> x0 = x;
        const float r0 = r;
        rk4_update(x, v, h2, ds * rsqrtf(dot3(v, v)), 1.0f / r);
        r = sqrtf(dot3(x, x));
        const float dphi = atan2f(x0.x * x.y - x0.y * x.x, x0.x * x.x + x0.y * x.y);
        const float phi1 = phi + dphi;
        for (; j < kPhis && float(j) * dphi_j <= phi1; ++j) {
            const float t = fminf(fmaxf((float(j) * dphi_j - phi) / fmaxf(dphi, 1e-12f), 0.f), 1.f);
            table[size_t(j) * kRays + i] = fmaxf(logf(r0 * (1.0f - t) + r * t), logH);
        }
        phi = phi1;
        if (r < 2.01f || (r > kRMax && dot3(x, v) > 0.f)) break;
    }
    const float fill = r < 10.0f ? logH : logf(kRMax);
    for (; j < kPhis; ++j) table[size_t(j) * kRays + i] = fill;
}

constexpr int kDup = 4;  // R_F duplication steps: converged in FP32

// u on an escaping orbit where the sweep from the turning point equals T (Newton in s).
__device__ __forceinline__ float invert_exact(float T, const orbit::Roots<float>& R) {
    const float smax = sqrtf(R.u2);
    float s = fminf(fmaxf(T / (1.41421356f * orbit::rf<float, kDup>((R.u2 - R.u1) * R.d32, (R.u2 - R.u1) * R.d32,
                                                                   R.d32 * (R.u2 - R.u1))), 0.f), smax);
#pragma unroll 1
    for (int k = 0; k < 8; ++k) {
        const float u = R.u2 - s * s;
        const float fv = orbit::sweep_to_turn<float, kDup>(u, R) - T;
        s = fminf(fmaxf(s - fv * 0.5f * sqrtf(2.0f * (u - R.u1) * (R.u3 - u)), 0.f), smax);
    }
    return R.u2 - s * s;
}

// One block of 256 threads per fan ray, 4 angles per thread.
__global__ void __launch_bounds__(256) k_lens_closed(float cam_r, float ac, float* __restrict__ table) {
    const int i = blockIdx.x;
    const float a = lens_alpha((float(i) + 0.5f) / float(kRays), ac);
    // impact parameter b = r sin(alpha) / sqrt(1 - 2/r) (Geodesic.h:50-54), in FP64: near the
    // shadow's edge the fan is dense in b
    const double rd = double(cam_r);
    const double b = rd * ::sin(double(a)) / ::sqrt(1.0 - 2.0 / rd);
    const float beta = float(b * (1.0 / 5.196152422706632) - 1.0);
    const bool ingoing = cosf(a) > 0.f;
    const float uc = 1.0f / cam_r;
    const float ue = 1.0f / kRMax, uh = 1.0f / 2.01f;
    const float logH = logf(2.0f), logMax = logf(kRMax);
    const float dphi_j = kTwoPi / float(kPhis - 1);
    if (threadIdx.x == 0) table[i] = logf(cam_r);
    if (beta > 0.f) {
        const orbit::Roots<float> R = orbit::roots<float, 8>(beta);
        const float Ic = orbit::sweep_to_turn<float, kDup>(uc, R);
        const float Ie = orbit::sweep_to_turn<float, kDup>(ue, R);
        // ingoing: camera -> turning point (Ic) -> r_max (Ic + Ie); outgoing: camera -> r_max (Ie - Ic)
        const float phi_end = ingoing ? Ic + Ie : Ie - Ic;
        for (int j = 1 + threadIdx.x; j < kPhis; j += blockDim.x) {
            const float ph = float(j) * dphi_j;
            float val = logMax;
            if (ph <= phi_end) {
                const float T = ingoing ? fabsf(Ic - ph) : Ic + ph;
                val = fmaxf(-logf(invert_exact(T, R)), logH);
            }
            table[size_t(j) * kRays + i] = val;
        }
    } else {
        const orbit::CapOrbit<float> C = orbit::cap_orbit<float, kDup>(beta);
        const float s2a = rsqrtf(2.0f * C.A);
        const float Fc = orbit::cap_F<float, kDup>(uc, C);
        // ingoing: u rises from uc to the capture radius; outgoing: u falls to 1 / r_max
        const float u_end = ingoing ? uh : ue;
        const float phi_end = fabsf(orbit::cap_F<float, kDup>(u_end, C) - Fc) * s2a;
        const float sgn = ingoing ? 1.f : -1.f;
        for (int j = 1 + threadIdx.x; j < kPhis; j += blockDim.x) {
            const float ph = float(j) * dphi_j;
            float val = ingoing ? logH : logMax;
            if (ph <= phi_end) {
                // Newton on sgn (F(u) - Fc) / sqrt(2A) = ph with dphi/du = sgn / sqrt(P(u))
                const float lo = fminf(uc, u_end), hi = fmaxf(uc, u_end);
                float u = uc + (u_end - uc) * (ph / phi_end);
#pragma unroll 1
                for (int k = 0; k < 10; ++k) {
                    const float fv = sgn * (orbit::cap_F<float, kDup>(u, C) - Fc) * s2a - ph;
                    const float P = fmaxf(2.0f * u * u * u - u * u + C.c, 0.f);
                    u = fminf(fmaxf(u - sgn * fv * sqrtf(P), lo), hi);
                }
                val = fmaxf(-logf(u), logH);
            }
            table[size_t(j) * kRays + i] = val;
        }
    }
}

}  // namespace

// the shadow's angular radius at r for a static observer (Geodesic.h:78-82), in double
double lens_alpha_crit(double r) {
    const double s = ::fmin(1.0, 5.196152422706632 / r * ::sqrt(::fmax(1.0 - 2.0 / r, 0.0)));
    const double a = ::asin(s);
    return r >= 3.0 ? a : 3.14159265358979323846 - a;
}

float lens_alpha_host(float u, float ac) { return lens_alpha(u, ac); }

cudaError_t launch_lens_table(float cam_r, int closed_form, float* table, cudaStream_t st) {
    const float ac = float(lens_alpha_crit(double(cam_r)));  // the reference's float uniform
    if (closed_form)
        k_lens_closed<<<kRays, 256, 0, st>>>(cam_r, ac, table);
    else
        k_lens_integrate<<<kRays / 64, 64, 0, st>>>(cam_r, ac, table);
    return cudaGetLastError();
}

}  // namespace bhr
