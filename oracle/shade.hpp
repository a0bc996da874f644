// CPU restatement of the renderer's shading of a traced pixel -- TEST INFRASTRUCTURE ONLY.
//
// Everything the fragment shader does with the march's result when the disk is thin and no
// bodies, gas or universe sky are on screen, in FP32 like the shader:
//   shaders/common.glsl:16-22,33-39,58-77   pcg3d, hash3u, grad3, pgnoise3 (periodic gradient noise)
//   shaders/noise_bake.comp:9-26            the 128^3 fbm + ridge noise volume, stored as R16F
//   src/DiskTextures.cpp:13-41,65-91        the blackbody LUT (CIE 1931 lobe fits x Planck, in double)
//   shaders/blackbody.glsl:7-16             blackbody(T): LUT lookup + Wien-tail fade
//   shaders/disk.glsl:21-48,81-85,113-129   diskTint, diskTempProfile, redshiftFactor, diskNoise,
//                                           opticalDepthScale, diskRadialProfile, thinDiskSample
//   shaders/disk.glsl:88-110                diskDensity, volumetricDiskStep (one slab sub-sample)
//   shaders/blackhole.frag:209-216,234      front-to-back compositing of the crossings, opacity stop
//   shaders/blackhole.frag:297-310          screen-space derivatives of escDir, mixed-quad rule
//   shaders/sky.glsl:26-48,54-103,105-118   makeFootprint, starLayer, sampleSky (without the cube)
//   shaders/blackhole.frag:354-359,377-379  shadow overlay, NaN clear, clamp at 0
//   shaders/geodesic.glsl:56-60             shadowAngularRadius
// GL's texture filtering is restated with exact (not 8-bit) weights: texel centres at
// (i + 0.5) / N, REPEAT for the noise volume and CLAMP_TO_EDGE for the LUT.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>

#include "bhr.h"

namespace oracle {
namespace shade {

constexpr int kNoiseN = BHR_NOISE_SIZE, kLutN = BHR_BLACKBODY_LUT;
constexpr float kPi = 3.14159265358979f, kTwoPi = 6.28318530717959f;

struct F3 { float x, y, z; };
inline F3 operator+(F3 a, F3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline F3 operator-(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline F3 operator*(F3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline F3 mul(F3 a, F3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline float dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline F3 cross(F3 a, F3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline float length(F3 a) { return std::sqrt(dot(a, a)); }
inline F3 divs(F3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline F3 normalize(F3 a) { return divs(a, length(a)); }
inline float mixf(float x, float y, float a) { return x * (1.0f - a) + y * a; }  // GLSL mix
// min / max as fminf / fmaxf (and the GPU's FMNMX): a NaN operand yields the other one
inline float clampf(float x, float lo, float hi) { return std::fmin(std::fmax(x, lo), hi); }
inline float smoothstep(float e0, float e1, float x) {
    const float t = clampf((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}

// ---------------------------------------------------------------- hashing and noise
struct U3 { uint32_t x, y, z; };
inline U3 pcg3d(U3 v) {
    v.x = v.x * 1664525u + 1013904223u;
    v.y = v.y * 1664525u + 1013904223u;
    v.z = v.z * 1664525u + 1013904223u;
    v.x += v.y * v.z; v.y += v.z * v.x; v.z += v.x * v.y;
    v.x ^= v.x >> 16u; v.y ^= v.y >> 16u; v.z ^= v.z >> 16u;
    v.x += v.y * v.z; v.y += v.z * v.x; v.z += v.x * v.y;
    return v;
}
inline F3 grad3(int cx, int cy, int cz, uint32_t salt) {
    const U3 h = pcg3d({uint32_t(cx) + salt, uint32_t(cy) + (salt * 3u + 11u), uint32_t(cz) + (salt * 7u + 29u)});
    const float s = 1.0f / 4294967296.0f;
    const F3 g{float(h.x) * s * 2.0f - 1.0f, float(h.y) * s * 2.0f - 1.0f, float(h.z) * s * 2.0f - 1.0f};
    return g * (1.0f / std::sqrt(std::fmax(dot(g, g), 1e-8f)));
}
inline float pgnoise3(F3 p, int period, uint32_t salt) {
    const F3 i{std::floor(p.x), std::floor(p.y), std::floor(p.z)};
    const F3 f = p - i;
    auto fade = [](float t) { return t * t * t * (t * (t * 6.0f - 15.0f) + 10.0f); };
    const F3 u{fade(f.x), fade(f.y), fade(f.z)};
    const int c[3] = {int(i.x), int(i.y), int(i.z)};
    int c0[3], c1[3];
    for (int k = 0; k < 3; ++k) {
        c0[k] = ((c[k] % period) + period) % period;
        c1[k] = ((c[k] + 1) % period + period) % period;
    }
    auto corner = [&](int ox, int oy, int oz) {
        const F3 g = grad3(ox ? c1[0] : c0[0], oy ? c1[1] : c0[1], oz ? c1[2] : c0[2], salt);
        return dot(g, f - F3{float(ox), float(oy), float(oz)});
    };
    const float nx00 = mixf(corner(0, 0, 0), corner(1, 0, 0), u.x), nx10 = mixf(corner(0, 1, 0), corner(1, 1, 0), u.x);
    const float nx01 = mixf(corner(0, 0, 1), corner(1, 0, 1), u.x), nx11 = mixf(corner(0, 1, 1), corner(1, 1, 1), u.x);
    return 1.4f * mixf(mixf(nx00, nx10, u.y), mixf(nx01, nx11, u.y), u.z);
}

// IEEE binary16 with round-to-nearest-even (the R16F store)
inline uint16_t to_half(float x) {
    uint32_t b;
    std::memcpy(&b, &x, 4);
    const uint32_t sign = (b >> 16) & 0x8000u;
    const uint32_t a = b & 0x7fffffffu;
    if (a >= 0x7f800000u) return uint16_t(sign | 0x7c00u | (a > 0x7f800000u ? 0x200u : 0u));
    if (a >= 0x477ff000u) return uint16_t(sign | 0x7c00u);  // rounds to infinity
    if (a < 0x38800000u) {                                   // half subnormal or zero
        if (a < 0x33000000u) return uint16_t(sign);
        const uint32_t m = (a & 0x7fffffu) | 0x800000u;
        const int shift = 126 - int(a >> 23);                // 14 .. 24
        uint32_t h = m >> shift;
        const uint32_t rem = m & ((1u << shift) - 1u), half_ = 1u << (shift - 1);
        if (rem > half_ || (rem == half_ && (h & 1u))) ++h;
        return uint16_t(sign | h);
    }
    uint32_t h = ((a >> 13) - (112u << 10));
    const uint32_t rem = a & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) ++h;
    return uint16_t(sign | h);
}
inline float from_half(uint16_t h) {
    const uint32_t sign = uint32_t(h & 0x8000u) << 16;
    const uint32_t e = (h >> 10) & 0x1fu, m = h & 0x3ffu;
    float v;
    if (e == 0) v = std::ldexp(float(m), -24);
    else if (e == 31) v = m ? NAN : INFINITY;
    else v = std::ldexp(float(m | 0x400u), int(e) - 25);
    uint32_t b;
    std::memcpy(&b, &v, 4);
    b |= sign;
    std::memcpy(&v, &b, 4);
    return v;
}

// noise_bake.comp: texel (x, y, z) of the volume, index (z N + y) N + x
inline float noise_texel(int x, int y, int z, uint32_t seed) {
    const F3 uvw{(float(x) + 0.5f) / float(kNoiseN), (float(y) + 0.5f) / float(kNoiseN), (float(z) + 0.5f) / float(kNoiseN)};
    float sum = 0.0f, amp = 0.55f, norm = 0.0f;
    int period = 4;
    for (int o = 0; o < 6; ++o) {
        sum += amp * pgnoise3(uvw * float(period), period, seed + uint32_t(o) * 131u);
        norm += amp;
        amp *= 0.55f;
        period *= 2;
    }
    float n = clampf(0.5f + 0.5f * (sum / norm) * 1.6f, 0.0f, 1.0f);
    const float ridge = 1.0f - std::fabs(pgnoise3(uvw * 8.0f, 8, seed + 977u));
    n = mixf(n, n * ridge * 1.3f, 0.35f);
    return n;
}

// ---------------------------------------------------------------- blackbody LUT (double, as the CPU bake)
inline double lobe(double l, double mu, double s1, double s2) {
    const double t = (l - mu) / (l < mu ? s1 : s2);
    return std::exp(-0.5 * t * t);
}
inline void cie_xyz(double l, double& x, double& y, double& z) {
    x = 1.056 * lobe(l, 599.8, 37.9, 31.0) + 0.362 * lobe(l, 442.0, 16.0, 26.7) - 0.065 * lobe(l, 501.1, 20.4, 26.2);
    y = 0.821 * lobe(l, 568.8, 46.9, 40.5) + 0.286 * lobe(l, 530.9, 16.3, 31.1);
    z = 1.217 * lobe(l, 437.0, 11.8, 36.0) + 0.681 * lobe(l, 459.0, 26.0, 13.8);
}
inline double planck(double l_nm, double T) {
    const double h = 6.62607015e-34, c = 2.99792458e8, k = 1.380649e-23;
    const double l = l_nm * 1e-9;
    return (2.0 * h * c * c) / (l * l * l * l * l) / (std::exp((h * c) / (l * k * T)) - 1.0);
}
inline void xyz_of(double T, double& X, double& Y, double& Z) {
    X = Y = Z = 0.0;
    for (int l = 380; l <= 780; ++l) {
        double x, y, z;
        cie_xyz(l, x, y, z);
        const double b = planck(l, T);
        X += b * x;
        Y += b * y;
        Z += b * z;
    }
}
inline void blackbody_lut(float* out) {
    double Xr, Yr, Zr;
    xyz_of(6500.0, Xr, Yr, Zr);
    const double lo = std::log(1000.0), hi = std::log(40000.0);
    for (int i = 0; i < kLutN; ++i) {
        const double T = std::exp(lo + (hi - lo) * (double(i) / (kLutN - 1)));
        double X, Y, Z;
        xyz_of(T, X, Y, Z);
        const double r = std::fmax(3.2406 * X - 1.5372 * Y - 0.4986 * Z, 0.0);
        const double g = std::fmax(-0.9689 * X + 1.8758 * Y + 0.0415 * Z, 0.0);
        const double b = std::fmax(0.0557 * X - 0.2040 * Y + 1.0570 * Z, 0.0);
        const double lum = 0.2126 * r + 0.7152 * g + 0.0722 * b;
        const double inv = lum > 0.0 ? 1.0 / lum : 0.0;
        out[4 * i + 0] = float(r * inv);
        out[4 * i + 1] = float(g * inv);
        out[4 * i + 2] = float(b * inv);
        out[4 * i + 3] = float(Y / Yr);
    }
}

// ---------------------------------------------------------------- shading
struct Tex {
    const uint16_t* noise;  // kNoiseN^3 half
    const float* lut;       // kLutN x 4
};

struct RGBA { float r, g, b, a; };

inline RGBA blackbody(const Tex& tx, float T) {
    const float Tc = clampf(T, 1000.0f, 40000.0f);
    const float t = (std::log(Tc) - std::log(1000.0f)) / (std::log(40000.0f) - std::log(1000.0f));
    const float u = t * float(kLutN) - 0.5f;
    const float fl = std::floor(u);
    const float a = u - fl;
    const int i0 = std::min(std::max(int(fl), 0), kLutN - 1), i1 = std::min(std::max(int(fl) + 1, 0), kLutN - 1);
    const float* p = tx.lut + 4 * i0;
    const float* q = tx.lut + 4 * i1;
    RGBA o{mixf(p[0], q[0], a), mixf(p[1], q[1], a), mixf(p[2], q[2], a), mixf(p[3], q[3], a)};
    const float under = clampf(T / 1000.0f, 0.0f, 1.0f);
    o.a *= under * under * under * under * under * under;
    return o;
}

inline float noise_sample(const Tex& tx, F3 c) {
    const float N = float(kNoiseN);
    const float ux = c.x * N - 0.5f, uy = c.y * N - 0.5f, uz = c.z * N - 0.5f;
    const float fx = std::floor(ux), fy = std::floor(uy), fz = std::floor(uz);
    const float ax = ux - fx, ay = uy - fy, az = uz - fz;
    auto wrap = [](int i) { return ((i % kNoiseN) + kNoiseN) % kNoiseN; };
    const int x0 = wrap(int(fx)), y0 = wrap(int(fy)), z0 = wrap(int(fz));
    const int x1 = (x0 + 1) % kNoiseN, y1 = (y0 + 1) % kNoiseN, z1 = (z0 + 1) % kNoiseN;
    auto T = [&](int x, int y, int z) { return from_half(tx.noise[(size_t(z) * kNoiseN + y) * kNoiseN + x]); };
    const float c00 = mixf(T(x0, y0, z0), T(x1, y0, z0), ax), c10 = mixf(T(x0, y1, z0), T(x1, y1, z0), ax);
    const float c01 = mixf(T(x0, y0, z1), T(x1, y0, z1), ax), c11 = mixf(T(x0, y1, z1), T(x1, y1, z1), ax);
    return mixf(mixf(c00, c10, ay), mixf(c01, c11, ay), az);
}

inline float disk_temp_profile(float r_in, float r) {
    const float x = r_in / std::fmax(r, r_in);
    const float f = std::pow(x, 0.75f) * std::pow(std::fmax(1.0f - std::sqrt(x), 0.0f), 0.25f);
    return f / 0.48796f;
}
inline float kepler_omega(float r) { return std::pow(r, -1.5f); }
inline float redshift_factor(float r, float b_axis, float rcam) {
    const float omega = kepler_omega(r);
    const float ut = 1.0f / std::sqrt(std::fmax(1.0f - 3.0f / r, 0.02f));
    const float lapse = std::sqrt(std::fmax(1.0f - 2.0f / rcam, 1e-4f));
    return 1.0f / (lapse * ut * std::fmax(1.0f - omega * b_axis, 0.05f));
}
inline float glsl_mod(float x, float y) { return x - y * std::floor(x / y); }

inline float disk_noise(const Tex& tx, const bhr_shade_params& P, float r, float phi, float y_over_h) {
    const float omega = kepler_omega(r);
    const float t = P.disk_time;
    const float Pd = 60.0f;
    const float t1 = glsl_mod(t, Pd);
    const float t2 = glsl_mod(t + 0.5f * Pd, Pd);
    const float w2 = std::fabs(2.0f * t1 / Pd - 1.0f);
    const float rep = std::fmax(1.0f, std::floor(2.0f * P.disk_noise_scale + 0.5f));
    const float lr = std::log(r) * 3.2f * P.disk_noise_scale;
    const float yy = y_over_h * 0.35f;
    const float k = rep / kTwoPi;
    const F3 c1{(phi + omega * t1) * k, lr + P.disk_inflow * omega * t1, yy};
    const F3 c2{(phi + omega * t2) * k, lr + 0.37f + P.disk_inflow * omega * t2, yy + 0.61f};
    return mixf(noise_sample(tx, c1), noise_sample(tx, c2), w2);
}
inline float optical_depth_scale(const bhr_shade_params& P, float r, float g_phys, float rcam) {
    const float lapse_em = std::sqrt(std::fmax(1.0f - 2.0f / r, 1e-4f));
    const float lapse_cam = std::sqrt(std::fmax(1.0f - 2.0f / rcam, 1e-4f));
    return mixf(1.0f, lapse_em / (g_phys * lapse_cam), P.doppler_strength);
}
inline float disk_radial_profile(float r_in, float r_out, float r) {
    const float inner = smoothstep(r_in, r_in + 0.25f, r);
    const float outer = 1.0f - smoothstep(r_out * 0.55f, r_out, r);
    return inner * outer * std::pow(r_in / std::fmax(r, r_in), 1.2f);
}

// thinDiskSample at a recorded crossing (r = |hit.xz|, phi = atan(hit.z, hit.x))
inline RGBA thin_disk_sample(const Tex& tx, const bhr_shade_params& P, const bhr_view& v, float r, float phi,
                             float b_axis, float rcam) {
    if (r < v.disk_inner || r > v.disk_outer) return {0, 0, 0, 0};
    const float n = disk_noise(tx, P, r, phi, 0.0f);
    const float f = smoothstep(0.32f, 0.78f, n);
    const float pattern = mixf(1.0f, mixf(0.08f, 1.4f, f), P.disk_noise_strength);
    const float emit = mixf(1.0f, mixf(0.22f, 1.35f, f * f), P.disk_noise_strength);
    const float dens = P.disk_density * disk_radial_profile(v.disk_inner, v.disk_outer, r) * pattern;
    const float T = P.disk_peak_temp * disk_temp_profile(v.disk_inner, r) * mixf(1.0f, 0.85f + 0.3f * emit, 0.5f);
    const float g_phys = redshift_factor(r, b_axis, rcam);
    const float g = mixf(1.0f, g_phys, P.doppler_strength);
    const RGBA bb = blackbody(tx, T * g);
    const float alpha = 1.0f - std::exp(-dens * P.disk_opacity * 0.6f * optical_depth_scale(P, r, g_phys, rcam));
    const float tint_w = P.disk_warmth;
    const F3 tint{mixf(1.0f, 1.0f, tint_w), mixf(1.0f, 0.80f, tint_w), mixf(1.0f, 0.58f, tint_w)};
    const float s = bb.a * P.disk_brightness * emit;
    return {bb.r * tint.x * s, bb.g * tint.y * s, bb.b * tint.z * s, alpha};
}

// volumetricDiskStep (disk.glsl:101-110) with diskDensity (:88-99): one segment of length ds
// centred at p, r = |p.xz|, composited front to back into col / trans.
inline void vol_disk_step(const Tex& tx, const bhr_shade_params& P, float r_in, float r_out, float thick, F3 p, float r,
                          float ds, float b_axis, float rcam, float col[3], float& trans) {
    const float H = std::fmax(thick * r, 1e-3f);
    const float yh = p.y / H;
    const float vert = std::exp(-yh * yh);
    const float phi = std::atan2(p.z, p.x);
    const float n = disk_noise(tx, P, r, phi, yh);
    const float f = smoothstep(0.32f, 0.78f, n);
    const float pattern = mixf(1.0f, mixf(0.08f, 1.4f, f), P.disk_noise_strength);
    const float emit = mixf(1.0f, mixf(0.22f, 1.35f, f * f), P.disk_noise_strength);
    const float puff = 1.0f + 0.6f * smoothstep(r_out * 0.4f, r_out, r) * (n - 0.5f);
    const float dens = P.disk_density * disk_radial_profile(r_in, r_out, r) * vert * pattern * std::fmax(puff, 0.0f);
    if (dens < 1e-4f) return;
    const float T = P.disk_peak_temp * disk_temp_profile(r_in, r) * mixf(1.0f, 0.85f + 0.3f * emit, 0.5f);
    const float g_phys = redshift_factor(r, b_axis, rcam);
    const float g = mixf(1.0f, g_phys, P.doppler_strength);
    const RGBA bb = blackbody(tx, T * g);
    const float inward = std::pow(r_in / std::fmax(r, r_in), 0.6f);
    const float w = P.disk_warmth;
    const float s = bb.a * P.disk_brightness * emit * inward;
    const float src[3] = {bb.r * mixf(1.0f, 1.0f, w) * s, bb.g * mixf(1.0f, 0.80f, w) * s, bb.b * mixf(1.0f, 0.58f, w) * s};
    const float absorb = dens * P.disk_opacity * optical_depth_scale(P, r, g_phys, rcam);
    const float a = 1.0f - std::exp(-absorb * ds);
    for (int c = 0; c < 3; ++c) col[c] = col[c] + trans * src[c] * a;
    trans *= 1.0f - a;
}

struct Footprint {
    F3 e1, e2;
    float r11, r12, r22, gi11, gi12, gi22, det_gi, det, mu;
};
inline Footprint make_footprint(F3 d, F3 a, F3 b, float omega0) {
    Footprint f;
    const float min_axis = 1e-3f * std::sqrt(omega0);
    const float la_raw = length(a);
    const float la = std::fmax(la_raw, min_axis);
    f.e1 = la_raw > 1e-12f ? divs(a, la_raw) : normalize(cross(d, F3{1e-3f, 1.0f + 1e-3f, 1e-3f}));
    const float b1 = dot(b, f.e1);
    const F3 bp = b - f.e1 * b1;
    const float lbp_raw = length(bp);
    const float lbp = std::fmax(lbp_raw, min_axis);
    f.e2 = lbp_raw > 1e-3f * min_axis ? divs(bp, lbp_raw) : normalize(cross(d, f.e1));
    f.r11 = 1.0f / la;
    f.r12 = -b1 / (la * lbp);
    f.r22 = 1.0f / lbp;
    f.gi11 = f.r11 * f.r11 + f.r12 * f.r12;
    f.gi12 = f.r12 * f.r22;
    f.gi22 = f.r22 * f.r22;
    f.det_gi = (f.r11 * f.r22) * (f.r11 * f.r22);
    const float area = la * lbp;
    f.det = area * area;
    f.mu = std::fmin(omega0 / area, 1e4f);
    return f;
}

inline F3 star_layer(const Tex& tx, F3 d, const Footprint& fp, float N, float prob, float flux, float sig_star,
                     float omega0, uint32_t salt, float g_shift) {
    const float footprint_cells = std::pow(fp.det, 0.25f) * N;
    const float w = smoothstep(0.8f, 2.5f, footprint_cells);
    const float kMeanFlux = 9.517f;
    const RGBA bavg = blackbody(tx, 5600.0f * g_shift);
    const float aw = prob * N * N * kMeanFlux * flux * omega0;
    const F3 avg{bavg.r * aw, bavg.g * aw, bavg.b * aw};
    F3 sum{0, 0, 0};
    if (w < 1.0f) {
        const float s2 = sig_star * sig_star;
        const float px2 = 0.45f;
        const float saa = px2 + s2 * fp.gi11, sab = s2 * fp.gi12, sbb = px2 + s2 * fp.gi22;
        const float det_s = px2 * px2 + px2 * s2 * (fp.gi11 + fp.gi22) + s2 * s2 * fp.det_gi;
        const float inv_det_s = 1.0f / det_s;
        const float isaa = sbb * inv_det_s, isab = -sab * inv_det_s, isbb = saa * inv_det_s;
        const float norm = fp.mu / (kTwoPi * std::sqrt(det_s));
        const F3 p = d * N;
        const int c0[3] = {int(std::floor(p.x)), int(std::floor(p.y)), int(std::floor(p.z))};
        const float s_in = 1.0f - 0.5f / N, s_out = 1.0f + 0.5f / N;
        const float s_in2 = s_in * s_in, s_out2 = s_out * s_out;
        const float k16 = 1.0f / 65536.0f;
        const float inv_n = 1.0f / N;  // (c + u2) / N as a product, pow(x, -1) as 1 / x
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    const int c[3] = {c0[0] + dx, c0[1] + dy, c0[2] + dz};
                    const U3 h = pcg3d({uint32_t(c[0]) + salt, uint32_t(c[1]) + (salt * 7u + 1u),
                                        uint32_t(c[2]) + (salt * 13u + 2u)});
                    const float ux = float(h.x >> 16u) * k16;
                    if (ux > prob) continue;
                    const F3 u2{float(h.x & 0xffffu) * k16, float(h.y >> 16u) * k16, float(h.y & 0xffffu) * k16};
                    const float uy = float(h.z >> 16u) * k16, uz = float(h.z & 0xffffu) * k16;
                    const F3 q{(float(c[0]) + u2.x) * inv_n, (float(c[1]) + u2.y) * inv_n, (float(c[2]) + u2.z) * inv_n};
                    const float ql2 = dot(q, q);
                    if (ql2 < s_in2 || ql2 > s_out2) continue;
                    const F3 delta = q * (1.0f / std::sqrt(ql2)) - d;
                    const float d1 = dot(fp.e1, delta), d2 = dot(fp.e2, delta);
                    const float sp = fp.r11 * d1 + fp.r12 * d2;
                    const float sq = fp.r22 * d2;
                    const float e = isaa * sp * sp + 2.0f * isab * sp * sq + isbb * sq * sq;
                    if (!(e < 30.0f)) continue;
                    const float F = flux / std::fmax(uy, 2e-4f);
                    const float T = std::exp(mixf(std::log(3000.0f), std::log(22000.0f), std::pow(uz, 1.7f)));
                    const RGBA bb = blackbody(tx, T * g_shift);
                    const float k = F * norm * std::exp(-0.5f * e);
                    sum = sum + F3{mixf(1.0f, bb.r, 0.7f) * k, mixf(1.0f, bb.g, 0.7f) * k, mixf(1.0f, bb.b, 0.7f) * k};
                }
    }
    if (!std::isfinite(sum.x) || !std::isfinite(sum.y) || !std::isfinite(sum.z)) sum = {0, 0, 0};
    sum = {std::fmin(sum.x, 64.0f), std::fmin(sum.y, 64.0f), std::fmin(sum.z, 64.0f)};
    return {mixf(sum.x, avg.x, w), mixf(sum.y, avg.y, w), mixf(sum.z, avg.z, w)};
}

// Primary ray direction of pixel (i, j) in float, as the fragment shader (blackhole.frag:68-72).
inline F3 primary_dir(const bhr_view& v, int i, int j) {
    const float pxx = float(i) + 0.5f + v.jitter[0], pxy = float(j) + 0.5f + v.jitter[1];
    const float ndcx = pxx / float(v.width) * 2.0f - 1.0f, ndcy = pxy / float(v.height) * 2.0f - 1.0f;
    const float aspect = float(v.width) / float(v.height);
    const F3 dc = normalize(F3{ndcx * v.tan_half_fov * aspect, ndcy * v.tan_half_fov, -1.0f});
    const float* B = v.cam_basis;
    return normalize(F3{B[0] * dc.x + B[3] * dc.y + B[6] * dc.z, B[1] * dc.x + B[4] * dc.y + B[7] * dc.z,
                        B[2] * dc.x + B[5] * dc.y + B[8] * dc.z});
}

inline float shadow_angular_radius(float r) {
    const float s = std::fmin(1.0f, 5.19615242270663f / r * std::sqrt(std::fmax(1.0f - 2.0f / r, 0.0f)));
    const float a = std::asin(s);
    return r >= 3.0f ? a : kPi - a;
}

// Per-pixel state after the disk composite: what the derivative pass needs from a pixel.
struct PixelState {
    F3 col;
    float trans;
    int status;   // the record's status; OPAQUE once the disk blocked the ray
    bool esc;     // status == escaped and not opaque (the shader's status == 1 after the loop)
    F3 esc_dir;   // escDir (the primary direction when the ray did not escape)
    F3 dir;       // primary direction
};

// The disk's colour and transmittance in front of the sky: composited here from the thin
// disk's crossings, or, for the volumetric disk, gathered by its march (rgbt[k] = rgb, T).
inline PixelState composite_disk(const Tex& tx, const bhr_shade_params& P, const bhr_view& v, const bhr_hit& h, int i,
                                 int j, float rcam, const float* rgbt) {
    PixelState s;
    s.col = {0, 0, 0};
    s.trans = 1.0f;
    s.dir = primary_dir(v, i, j);
    bool opaque = false;
    if (v.disk_mode == BHR_DISK_VOLUMETRIC) {
        const float* q = rgbt + 4 * (int64_t(j) * v.width + i);
        s.col = {q[0], q[1], q[2]};
        s.trans = q[3];
        opaque = h.status == BHR_STATUS_OPAQUE;
    } else if (v.disk_mode == BHR_DISK_THIN) {
        for (int k = 0; k < h.ncross && k < 3; ++k) {
            const RGBA d = thin_disk_sample(tx, P, v, h.cross_r[k], h.cross_phi[k], h.b_axis, rcam);
            s.col = s.col + F3{s.trans * d.r * d.a, s.trans * d.g * d.a, s.trans * d.b * d.a};
            s.trans *= 1.0f - d.a;
            if (s.trans < 0.004f) {
                opaque = true;
                break;
            }
        }
    }
    s.esc = h.status == BHR_STATUS_ESCAPED && !opaque;
    s.status = opaque ? BHR_STATUS_OPAQUE : int(h.status);
    s.esc_dir = h.status == BHR_STATUS_ESCAPED ? F3{h.dir[0], h.dir[1], h.dir[2]} : s.dir;
    return s;
}

// No further layers after the disk (no bodies on screen).
struct NoPost {
    void operator()(PixelState&, int, int) const {}
};

// Shades every pixel of one view from its hit records; rgba[4 k + c], k = j * width + i.
// `post(state, i, j)` adds what lies behind the disk before the sky (the bodies, oracle/bodies.hpp).
template <class Post = NoPost>
inline void shade_view(const Tex& tx, const bhr_shade_params& P, const bhr_view& v, const bhr_hit* hits, float* rgba,
                       int64_t row_begin, int64_t row_end, const float* rgbt = nullptr, const Post& post = Post{}) {
    const int W = v.width, H = v.height;
    const F3 cam{v.cam_pos[0], v.cam_pos[1], v.cam_pos[2]};
    const float rcam = length(cam);
    const float tan_half = v.tan_half_fov;
    const float pixel_angle = 2.0f * tan_half / float(H);
    const float omega0 = pixel_angle * pixel_angle;
    const float g = mixf(1.0f, 1.0f / std::sqrt(std::fmax(1.0f - 2.0f / rcam, 1e-4f)), P.doppler_strength);
    const float g4 = g * g * g * g;
    auto state = [&](int i, int j) {
        PixelState s = composite_disk(tx, P, v, hits[int64_t(j) * W + i], i, j, rcam, rgbt);
        post(s, i, j);
        return s;
    };
    for (int64_t j = row_begin; j < row_end; ++j)
        for (int i = 0; i < W; ++i) {
            const PixelState s = state(i, int(j));
            F3 col = s.col;
            float alpha = 0.0f;
            if (s.esc) {
                // fine derivatives over the 2x2 quad (even-aligned); a partner outside the image
                // takes the unlensed footprint
                const int ix0 = i & ~1, iy0 = int(j) & ~1;
                const bool hx = ix0 + 1 < W, hy = iy0 + 1 < H;
                F3 ddx, ddy;
                bool mixed = !hx || !hy;
                PixelState sx0, sx1, sy0, sy1;
                if (!mixed) {
                    sx0 = (ix0 == i) ? s : state(ix0, int(j));
                    sx1 = (ix0 + 1 == i) ? s : state(ix0 + 1, int(j));
                    sy0 = (iy0 == j) ? s : state(i, iy0);
                    sy1 = (iy0 + 1 == j) ? s : state(i, iy0 + 1);
                    mixed = sx0.esc != sx1.esc || sy0.esc != sy1.esc;
                }
                if (!mixed) {
                    ddx = sx1.esc_dir - sx0.esc_dir;
                    ddy = sy1.esc_dir - sy0.esc_dir;
                } else {
                    ddx = primary_dir(v, ix0 + 1, int(j)) - primary_dir(v, ix0, int(j));
                    ddy = primary_dir(v, i, iy0 + 1) - primary_dir(v, i, iy0);
                }
                const Footprint fp = make_footprint(s.esc_dir, ddx, ddy, omega0);
                const float sb = P.star_brightness * g4;
                const F3 s1 = star_layer(tx, s.esc_dir, fp, 200.0f, 0.40f * P.star_density, 0.0045f * sb, 0.0004f, omega0,
                                         11u, g);
                const F3 s2 = star_layer(tx, s.esc_dir, fp, 48.0f, 0.25f * P.star_density, 0.06f * sb, 0.0011f, omega0,
                                         23u, g);
                const F3 sky = s1 + s2;
                col = col + F3{s.trans * sky.x, s.trans * sky.y, s.trans * sky.z};
                alpha = s.trans * (P.sky_brightness * g4);
            }
            if (P.shadow_overlay && !v.far_mode) {
                const float ang = std::acos(clampf(dot(s.dir, F3{-cam.x / rcam, -cam.y / rcam, -cam.z / rcam}), -1.0f, 1.0f));
                const float dd = std::fabs(ang - shadow_angular_radius(rcam)) / pixel_angle;
                const float k = 0.85f * (1.0f - smoothstep(0.8f, 1.8f, dd));
                col = {mixf(col.x, 0.1f, k), mixf(col.y, 1.0f, k), mixf(col.z, 0.2f, k)};
                alpha *= 1.0f - k;
            }
            if (!std::isfinite(col.x) || !std::isfinite(col.y) || !std::isfinite(col.z)) {
                col = {0, 0, 0};
                alpha = 0.0f;
            }
            float* o = rgba + 4 * (int64_t(j) * W + i);
            o[0] = std::fmax(col.x, 0.0f);
            o[1] = std::fmax(col.y, 0.0f);
            o[2] = std::fmax(col.z, 0.0f);
            o[3] = alpha;
        }
}

}  // namespace shade
}  // namespace oracle
