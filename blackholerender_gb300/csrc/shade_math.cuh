// Device shading math shared by the shading consumer (shade.cu) and the volumetric disk march
// (vol.cu): hashing, the noise volume and blackbody table lookups, and the disk's emission
// models (disk.glsl, blackbody.glsl, common.glsl). Float arithmetic in the GLSL formula order.
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "bhr.h"

namespace bhr {
namespace shading {

constexpr int kN = BHR_NOISE_SIZE, kLut = BHR_BLACKBODY_LUT;
constexpr float kPi = 3.14159265358979f, kTwoPi = 6.28318530717959f;

struct F3 { float x, y, z; };
__device__ __forceinline__ F3 add(F3 a, F3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ F3 sub(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ F3 scale(F3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ F3 divs(F3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ float dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ F3 cross(F3 a, F3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ float len(F3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ F3 normalize(F3 a) { return divs(a, len(a)); }
__device__ __forceinline__ float mixf(float x, float y, float a) { return x * (1.0f - a) + y * a; }  // GLSL mix
__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
__device__ __forceinline__ float smoothstep(float e0, float e1, float x) {
    const float t = clampf((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}

// exp, log and pow of the shading: the SFU approximations, as GLSL's exp / log / pow compile to
// on the GPU (a few ulp; the noise bake uses none of them and stays exact)
__device__ __forceinline__ float gexp(float x) { return __expf(x); }
__device__ __forceinline__ float glog(float x) { return __logf(x); }
__device__ __forceinline__ float gpow(float x, float y) { return __powf(x, y); }

// common.glsl:16-22 pcg3d, the three lanes updated in sequence
__device__ __forceinline__ uint3 pcg3d(uint3 v) {
    v.x = v.x * 1664525u + 1013904223u;
    v.y = v.y * 1664525u + 1013904223u;
    v.z = v.z * 1664525u + 1013904223u;
    v.x += v.y * v.z;
    v.y += v.z * v.x;
    v.z += v.x * v.y;
    v.x ^= v.x >> 16;
    v.y ^= v.y >> 16;
    v.z ^= v.z >> 16;
    v.x += v.y * v.z;
    v.y += v.z * v.x;
    v.z += v.x * v.y;
    return v;
}

// common.glsl:33-39 grad3: a unit gradient from the hashed lattice point
__device__ __forceinline__ F3 grad3(int cx, int cy, int cz, uint32_t salt) {
    const uint3 h = pcg3d(make_uint3(uint32_t(cx) + salt, uint32_t(cy) + (salt * 3u + 11u), uint32_t(cz) + (salt * 7u + 29u)));
    const float s = 1.0f / 4294967296.0f;
    const F3 g{float(h.x) * s * 2.0f - 1.0f, float(h.y) * s * 2.0f - 1.0f, float(h.z) * s * 2.0f - 1.0f};
    return scale(g, 1.0f / sqrtf(fmaxf(dot(g, g), 1e-8f)));
}

struct Tex {
    const uint4* noise8;  // per texel its 2x2x2 REPEAT neighbourhood, eight halves (k_noise_expand)
    const float4* lut;  // shared memory
    float ln_1000, ln_40000;
};

// blackbody.glsl:7-16: log-temperature lookup, linear filter, clamp to edge; Wien-tail fade
__device__ __forceinline__ float4 blackbody(const Tex& tx, float T) {
    const float Tc = clampf(T, 1000.0f, 40000.0f);
    const float t = (glog(Tc) - tx.ln_1000) / (tx.ln_40000 - tx.ln_1000);
    const float u = t * float(kLut) - 0.5f;
    const float fl = floorf(u);
    const float a = u - fl;
    const int i0 = min(max(int(fl), 0), kLut - 1), i1 = min(max(int(fl) + 1, 0), kLut - 1);
    const float4 p = tx.lut[i0], q = tx.lut[i1];
    float4 o{mixf(p.x, q.x, a), mixf(p.y, q.y, a), mixf(p.z, q.z, a), mixf(p.w, q.w, a)};
    const float under = clampf(T / 1000.0f, 0.0f, 1.0f);
    o.w *= under * under * under * under * under * under;
    return o;
}

__device__ __forceinline__ float2 half2_bits(uint32_t u) {
    return __half22float2(*reinterpret_cast<const __half2*>(&u));
}

// texture(uNoise3d, c).r: trilinear, REPEAT
__device__ inline float noise_sample(const Tex& tx, F3 c) {
    const float ux = c.x * float(kN) - 0.5f, uy = c.y * float(kN) - 0.5f, uz = c.z * float(kN) - 0.5f;
    const float fx = floorf(ux), fy = floorf(uy), fz = floorf(uz);
    const float ax = ux - fx, ay = uy - fy, az = uz - fz;
    // REPEAT: the wrap of a power-of-two size is a mask (two's complement for negative texels)
    const int x0 = int(fx) & (kN - 1), y0 = int(fy) & (kN - 1), z0 = int(fz) & (kN - 1);
    // one 16-byte load: (x0, x1) pairs at (y0, z0), (y1, z0), (y0, z1), (y1, z1)
    const uint4 q = __ldg(tx.noise8 + (size_t(z0) * kN + y0) * kN + x0);
    const float2 p00 = half2_bits(q.x), p10 = half2_bits(q.y), p01 = half2_bits(q.z), p11 = half2_bits(q.w);
    const float c00 = mixf(p00.x, p00.y, ax);
    const float c10 = mixf(p10.x, p10.y, ax);
    const float c01 = mixf(p01.x, p01.y, ax);
    const float c11 = mixf(p11.x, p11.y, ax);
    return mixf(mixf(c00, c10, ay), mixf(c01, c11, ay), az);
}

__device__ __forceinline__ float glsl_mod(float x, float y) { return x - y * floorf(x / y); }

// The constants of a view that diskNoise and the redshift recompute per sample in the shader:
// the flow clock's two phases and cross-fade, the azimuthal repeat, the camera's lapse.
struct DiskConsts {
    float t1, t2, w2, k, lapse_cam;
};
__device__ __forceinline__ DiskConsts disk_consts(const bhr_shade_params& P, float rcam) {
    DiskConsts C;
    const float t = P.disk_time;
    const float Pd = 60.0f;
    C.t1 = glsl_mod(t, Pd);
    C.t2 = glsl_mod(t + 0.5f * Pd, Pd);
    C.w2 = fabsf(2.0f * C.t1 / Pd - 1.0f);
    const float rep = fmaxf(1.0f, floorf(2.0f * P.disk_noise_scale + 0.5f));
    C.k = rep / kTwoPi;
    C.lapse_cam = sqrtf(fmaxf(1.0f - 2.0f / rcam, 1e-4f));
    return C;
}

// x^y and its parts for x >= 0 as the SFU computes it, 2^(y log2 x) (0 at x = 0 for y > 0);
// several powers of one base share its log2
__device__ __forceinline__ float lg2a(float x) {
    float y;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float ex2a(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// disk.glsl:45-63 diskNoise: two phase-shifted copies of the flow-advected noise, cross-faded;
// omega = keplerOmega(r) = r^-1.5
__device__ __forceinline__ float disk_noise(const Tex& tx, const bhr_shade_params& P, const DiskConsts& C, float r,
                                            float phi, float y_over_h, float omega) {
    const float lr = glog(r) * 3.2f * P.disk_noise_scale;
    const float yy = y_over_h * 0.35f;
    const F3 c1{(phi + omega * C.t1) * C.k, lr + P.disk_inflow * omega * C.t1, yy};
    const F3 c2{(phi + omega * C.t2) * C.k, lr + 0.37f + P.disk_inflow * omega * C.t2, yy + 0.61f};
    return mixf(noise_sample(tx, c1), noise_sample(tx, c2), C.w2);
}

// thinDiskSample (disk.glsl:113-129) at a recorded crossing: radiance (rgb) and alpha
__device__ inline float4 thin_disk_sample(const Tex& tx, const bhr_shade_params& P, const DiskConsts& C, float r_in,
                                          float r_out, float r, float phi, float b_axis) {
    if (r < r_in || r > r_out) return make_float4(0.f, 0.f, 0.f, 0.f);
    const float omega = gpow(r, -1.5f);
    const float n = disk_noise(tx, P, C, r, phi, 0.0f, omega);
    const float f = smoothstep(0.32f, 0.78f, n);
    const float pattern = mixf(1.0f, mixf(0.08f, 1.4f, f), P.disk_noise_strength);
    const float emit = mixf(1.0f, mixf(0.22f, 1.35f, f * f), P.disk_noise_strength);
    // diskRadialProfile (disk.glsl:81-85)
    const float inner = smoothstep(r_in, r_in + 0.25f, r);
    const float outer = 1.0f - smoothstep(r_out * 0.55f, r_out, r);
    const float radial = inner * outer * gpow(r_in / fmaxf(r, r_in), 1.2f);
    const float dens = P.disk_density * radial * pattern;
    // diskTempProfile (disk.glsl:26-30)
    const float x = r_in / fmaxf(r, r_in);
    const float prof = gpow(x, 0.75f) * gpow(fmaxf(1.0f - sqrtf(x), 0.0f), 0.25f) / 0.48796f;
    const float T = P.disk_peak_temp * prof * mixf(1.0f, 0.85f + 0.3f * emit, 0.5f);
    // redshiftFactor (disk.glsl:36-41)
    const float ut = 1.0f / sqrtf(fmaxf(1.0f - 3.0f / r, 0.02f));
    const float lapse = C.lapse_cam;
    const float g_phys = 1.0f / (lapse * ut * fmaxf(1.0f - omega * b_axis, 0.05f));
    const float g = mixf(1.0f, g_phys, P.doppler_strength);
    const float4 bb = blackbody(tx, T * g);
    // opticalDepthScale (disk.glsl:67-71)
    const float lapse_em = sqrtf(fmaxf(1.0f - 2.0f / r, 1e-4f));
    const float ods = mixf(1.0f, lapse_em / (g_phys * lapse), P.doppler_strength);
    const float alpha = 1.0f - gexp(-dens * P.disk_opacity * 0.6f * ods);
    // diskTint (disk.glsl:21)
    const float w = P.disk_warmth;
    const float s = bb.w * P.disk_brightness * emit;
    return make_float4(bb.x * mixf(1.0f, 1.0f, w) * s, bb.y * mixf(1.0f, 0.80f, w) * s, bb.z * mixf(1.0f, 0.58f, w) * s,
                       alpha);
}

// volumetricDiskStep (disk.glsl:88-110) with diskDensity (:88-99): emission and absorption of
// one march segment of length ds centred at p (r = |p.xz|), front to back into col / trans.
// The radial profile is taken first: where it is zero the sample adds nothing (dens < 1e-4).
__device__ inline void vol_disk_step(const Tex& tx, const bhr_shade_params& P, const DiskConsts& C, float r_in,
                                     float r_out, float thick, F3 p, float r, float ds, float b_axis, F3& col,
                                     float& trans) {
    const float inner = smoothstep(r_in, r_in + 0.25f, r);
    const float outer = 1.0f - smoothstep(r_out * 0.55f, r_out, r);
    if (inner * outer == 0.0f) return;
    const float x = r_in / fmaxf(r, r_in);
    const float lx = lg2a(x);                     // x^1.2, x^0.75, x^0.6 share log2 x
    const float radial = inner * outer * ex2a(1.2f * lx);
    const float omega = ex2a(-1.5f * lg2a(r));    // keplerOmega(r)
    const float H = fmaxf(thick * r, 1e-3f);
    const float yh = p.y / H;
    const float vert = gexp(-yh * yh);
    const float phi = atan2f(p.z, p.x);
    const float n = disk_noise(tx, P, C, r, phi, yh, omega);
    const float f = smoothstep(0.32f, 0.78f, n);
    const float pattern = mixf(1.0f, mixf(0.08f, 1.4f, f), P.disk_noise_strength);
    const float emit = mixf(1.0f, mixf(0.22f, 1.35f, f * f), P.disk_noise_strength);
    const float puff = 1.0f + 0.6f * smoothstep(r_out * 0.4f, r_out, r) * (n - 0.5f);
    const float dens = P.disk_density * radial * vert * pattern * fmaxf(puff, 0.0f);
    if (dens < 1e-4f) return;
    const float prof = ex2a(0.75f * lx) * ex2a(0.25f * lg2a(fmaxf(1.0f - sqrtf(x), 0.0f))) / 0.48796f;
    const float T = P.disk_peak_temp * prof * mixf(1.0f, 0.85f + 0.3f * emit, 0.5f);
    const float ut = 1.0f / sqrtf(fmaxf(1.0f - 3.0f / r, 0.02f));
    const float lapse = C.lapse_cam;
    const float g_phys = 1.0f / (lapse * ut * fmaxf(1.0f - omega * b_axis, 0.05f));
    const float g = mixf(1.0f, g_phys, P.doppler_strength);
    const float4 bb = blackbody(tx, T * g);
    const float inward = ex2a(0.6f * lx);
    const float w = P.disk_warmth;
    const float s = bb.w * P.disk_brightness * emit * inward;
    const F3 source{bb.x * mixf(1.0f, 1.0f, w) * s, bb.y * mixf(1.0f, 0.80f, w) * s, bb.z * mixf(1.0f, 0.58f, w) * s};
    const float lapse_em = sqrtf(fmaxf(1.0f - 2.0f / r, 1e-4f));
    const float absorb = dens * P.disk_opacity * mixf(1.0f, lapse_em / (g_phys * lapse), P.doppler_strength);
    const float a = 1.0f - gexp(-absorb * ds);
    col = F3{col.x + trans * source.x * a, col.y + trans * source.y * a, col.z + trans * source.z * a};
    trans *= 1.0f - a;
}

}  // namespace shading
}  // namespace bhr
