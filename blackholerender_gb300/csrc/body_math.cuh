// Device shading of bodies (planets and stars), used by the shading consumer for views marched
// with bodies:
//   common.glsl:24-57,78-88   hash3u, gnoise3, fbm3
//   bodies.glsl:28,47-221     lodFade, bodyLocal, ridged, craters, lookAtmoColor, planetClouds,
//                             planetSurface (nine looks)
//   bodies.glsl:224-361       shadeBodySurface, ringSample, traceBody, bodyHalo
//   blackhole.frag:41-62      composite, nearestBodyStraight
// FP32 in the GLSL formula order; sin / cos are the accurate library functions (their arguments
// reach tens of radians), exp and pow the SFU approximations as elsewhere in the shading.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "bhr.h"
#include "shade_math.cuh"

namespace bhr {
namespace shading {

__device__ __forceinline__ F3 mix3(F3 a, F3 b, float t) { return {mixf(a.x, b.x, t), mixf(a.y, b.y, t), mixf(a.z, b.z, t)}; }
__device__ __forceinline__ F3 mul3(F3 a, F3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ F3 add_s(F3 a, float s) { return {a.x + s, a.y + s, a.z + s}; }
__device__ __forceinline__ F3 xyz4(const float* q) { return {q[0], q[1], q[2]}; }

// common.glsl:24 hash3u
__device__ __forceinline__ F3 hash3u(uint32_t x, uint32_t y, uint32_t z) {
    const uint3 h = pcg3d(make_uint3(x, y, z));
    const float s = 1.0f / 4294967296.0f;
    return {float(h.x) * s, float(h.y) * s, float(h.z) * s};
}

// common.glsl:41-57 gnoise3: gradient noise on the unbounded lattice
__device__ inline float gnoise3(F3 p, uint32_t salt) {
    const float ix = floorf(p.x), iy = floorf(p.y), iz = floorf(p.z);
    const F3 f{p.x - ix, p.y - iy, p.z - iz};
    auto fade = [](float t) { return t * t * t * (t * (t * 6.0f - 15.0f) + 10.0f); };
    const F3 u{fade(f.x), fade(f.y), fade(f.z)};
    const int cx = int(ix), cy = int(iy), cz = int(iz);
    float n[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int ox = k & 1, oy = (k >> 1) & 1, oz = k >> 2;
        const F3 g = grad3(cx + ox, cy + oy, cz + oz, salt);
        n[k] = dot(g, F3{f.x - float(ox), f.y - float(oy), f.z - float(oz)});
    }
    const float nx00 = mixf(n[0], n[1], u.x), nx10 = mixf(n[2], n[3], u.x);
    const float nx01 = mixf(n[4], n[5], u.x), nx11 = mixf(n[6], n[7], u.x);
    return 1.4f * mixf(mixf(nx00, nx10, u.y), mixf(nx01, nx11, u.y), u.z);
}

// common.glsl:78-88 fbm3
__device__ inline float fbm3(F3 p, int octaves, float gain, uint32_t salt) {
    float sum = 0.0f, amp = 0.5f, norm = 0.0f;
    for (int i = 0; i < octaves; ++i) {
        sum += amp * gnoise3(p, salt + uint32_t(i) * 101u);
        norm += amp;
        amp *= gain;
        p = F3{p.x * 2.02f + 17.3f, p.y * 2.02f + 9.1f, p.z * 2.02f + 31.7f};
    }
    return sum / norm;
}

// bodies.glsl:28 lodFade: detail of `frequency` per radius fades once unresolved
__device__ __forceinline__ float lod_fade(float frequency, float lod) { return 1.0f - smoothstep(0.25f, 1.0f, frequency * lod); }

// bodies.glsl:47-55 bodyLocal: the normal in body coordinates (y along the spin axis)
__device__ inline F3 body_local(const bhr_body& b, F3 n) {
    const F3 ax = normalize(xyz4(b.axis));
    const F3 ref = fabsf(ax.y) < 0.95f ? F3{0.0f, 1.0f, 0.0f} : F3{1.0f, 0.0f, 0.0f};
    const F3 e1 = normalize(cross(ref, ax));
    const F3 e2 = cross(ax, e1);
    const float ca = cosf(b.look[3]), sa = sinf(b.look[3]);
    const F3 u = add(scale(e1, ca), scale(e2, sa));
    const F3 v = add(scale(scale(e1, -1.0f), sa), scale(e2, ca));
    return {dot(n, u), dot(n, ax), dot(n, v)};
}

// bodies.glsl:57-66 ridged
__device__ inline float ridged(F3 p, int oct, uint32_t salt) {
    float s = 0.0f, a = 0.5f, nrm = 0.0f;
    for (int i = 0; i < oct; ++i) {
        s += a * (1.0f - fabsf(gnoise3(p, salt + uint32_t(i) * 17u)));
        nrm += a;
        a *= 0.5f;
        p = F3{p.x * 2.03f + 7.1f, p.y * 2.03f + 7.1f, p.z * 2.03f + 7.1f};
    }
    return s / nrm;
}

// bodies.glsl:69-89 craters: (floor 0..1, rim)
__device__ inline float2 craters(F3 p, float scale_, uint32_t salt) {
    const F3 q = scale(p, scale_);
    const float ix = floorf(q.x), iy = floorf(q.y), iz = floorf(q.z);
    float2 best = make_float2(0.0f, 0.0f);
    for (int z = -1; z <= 1; ++z)
        for (int y = -1; y <= 1; ++y)
            for (int x = -1; x <= 1; ++x) {
                const F3 c{ix + float(x), iy + float(y), iz + float(z)};
                const F3 h = hash3u(uint32_t(int(c.x)) + salt, uint32_t(int(c.y)) + salt * 3u, uint32_t(int(c.z)) + salt * 7u);
                if (h.x > 0.45f) continue;
                const F3 center = add(c, h);
                const float rad = 0.15f + 0.35f * h.y;
                const float d = len(sub(q, center)) / rad;
                if (d < 1.25f) {
                    const float floorv = 1.0f - smoothstep(0.7f, 1.0f, d);
                    const float rim = smoothstep(0.75f, 1.0f, d) * (1.0f - smoothstep(1.0f, 1.25f, d));
                    best = make_float2(fmaxf(best.x, floorv), fmaxf(best.y, rim));
                }
            }
    return best;
}

enum : int { kRocky = 0, kDesert = 1, kOcean = 2, kIce = 3, kEarth = 4, kGasWarm = 5, kGasCold = 6, kCloudy = 7, kLava = 8 };

// bodies.glsl:91-101 lookAtmoColor
__device__ inline F3 look_atmo_color(int look) {
    if (look == kOcean) return {0.35f, 0.6f, 1.0f};
    if (look == kIce) return {0.6f, 0.78f, 1.0f};
    if (look == kDesert) return {1.0f, 0.62f, 0.42f};
    if (look == kRocky) return {0.0f, 0.0f, 0.0f};
    if (look == kEarth) return {0.35f, 0.58f, 1.0f};
    if (look == kCloudy) return {1.0f, 0.88f, 0.6f};
    if (look == kGasWarm) return {1.0f, 0.85f, 0.65f};
    if (look == kGasCold) return {0.55f, 0.85f, 1.0f};
    return {1.0f, 0.45f, 0.2f};
}

struct Surface {
    F3 albedo, emission;
    float specular, roughness;
    F3 atmo;
};

// bodies.glsl:113-119 planetClouds: fbm through a domain warp, drifting with the clock
__device__ inline float planet_clouds(F3 p, uint32_t seed, float scale_, float time) {
    const float a = time * 0.004f;
    const float ca = cosf(a), sa = sinf(a);
    const F3 q{ca * p.x - sa * p.z, p.y, sa * p.x + ca * p.z};
    const F3 q17 = scale(q, 1.7f);
    const F3 w{fbm3(q17, 3, 0.5f, seed + 21u), fbm3(add_s(q17, 4.1f), 3, 0.5f, seed + 22u),
               fbm3(add_s(q17, 8.3f), 3, 0.5f, seed + 23u)};
    return fbm3(add(scale(q, scale_), scale(w, 1.4f)), 6, 0.55f, seed + 8u);
}

// bodies.glsl:121-221 planetSurface
__device__ inline Surface planet_surface(const bhr_body& b, F3 n, float lod, float time) {
    const F3 p = body_local(b, n);
    const int look = int(b.look[0] + 0.5f);
    const uint32_t seed = uint32_t(b.look[1]);
    const float lat = p.y;
    Surface s;
    s.emission = {0.0f, 0.0f, 0.0f};
    s.specular = 0.0f;
    s.roughness = 0.8f;
    s.atmo = {0.4f, 0.6f, 1.0f};
    if (look == kOcean) {
        const float swell = gnoise3(add_s(F3{p.x * 2.0f, p.y * 6.0f, p.z * 2.0f}, float(seed)), seed);
        const float bands = 0.5f + 0.5f * sinf(p.x * 14.0f + 3.0f * swell) * lod_fade(14.0f / 6.283f, lod);
        const float detail = fbm3(scale(p, 9.0f), 4, 0.5f, seed + 3u) * lod_fade(9.0f, lod);
        s.albedo = mix3(F3{0.03f, 0.10f, 0.15f}, F3{0.16f, 0.36f, 0.42f}, smoothstep(0.55f, 0.95f, bands) * 0.8f + 0.2f * detail);
        const float foam = smoothstep(0.9f, 0.99f, bands) * smoothstep(0.0f, 0.5f, detail) * lod_fade(20.0f, lod);
        s.albedo = mix3(s.albedo, F3{0.8f, 0.8f, 0.8f}, foam * 0.6f);
        const F3 sun_local = body_local(b, normalize(xyz4(b.light)));
        const float cloud = smoothstep(0.25f, 0.7f, planet_clouds(p, seed + 9u, 4.0f, time));
        const float shade =
            smoothstep(0.25f, 0.7f, planet_clouds(normalize(add(p, scale(sun_local, 0.025f))), seed + 9u, 4.0f, time));
        s.albedo = scale(s.albedo, 1.0f - 0.4f * shade);
        s.albedo = mix3(s.albedo, F3{0.9f, 0.9f, 0.9f}, cloud * 0.55f);
        s.specular = 0.8f * (1.0f - cloud);
        s.roughness = 0.25f;
        s.atmo = {0.35f, 0.6f, 1.0f};
    } else if (look == kIce) {
        const float base = fbm3(scale(p, 3.0f), 5, 0.5f, seed);
        const float cracks = ridged(scale(p, 6.0f), 4, seed + 5u);
        const F3 ice = mix3(F3{0.78f, 0.84f, 0.9f}, F3{0.95f, 0.97f, 1.0f}, 0.5f + 0.5f * base);
        s.albedo = mix3(ice, F3{0.42f, 0.55f, 0.68f}, smoothstep(0.86f, 0.97f, cracks));
        const float cloud = smoothstep(0.35f, 0.8f, fbm3(add_s(scale(p, 5.0f), 3.0f), 4, 0.5f, seed + 2u));
        s.albedo = mix3(s.albedo, F3{0.97f, 0.97f, 0.97f}, cloud * 0.4f);
        s.specular = 0.3f;
        s.roughness = 0.5f;
        s.atmo = {0.6f, 0.78f, 1.0f};
    } else if (look == kDesert) {
        const float big = fbm3(scale(p, 2.5f), 5, 0.55f, seed);
        const float dunes =
            0.5f + 0.5f * sinf(dot(p, F3{40.0f, 13.0f, 27.0f}) + 8.0f * fbm3(scale(p, 6.0f), 3, 0.5f, seed + 1u)) * lod_fade(8.0f, lod);
        const F3 sand = mix3(F3{0.62f, 0.40f, 0.24f}, F3{0.86f, 0.66f, 0.44f}, 0.5f + 0.5f * big);
        s.albedo = scale(sand, 0.85f + 0.15f * dunes);
        const float2 cr = craters(p, 7.0f, seed + 4u);
        s.albedo = scale(s.albedo, 1.0f - 0.25f * cr.x + 0.15f * cr.y);
        s.albedo = mix3(s.albedo, F3{0.92f, 0.9f, 0.88f}, smoothstep(0.82f, 0.92f, fabsf(lat)));
        s.atmo = {1.0f, 0.62f, 0.42f};
    } else if (look == kRocky) {
        const float base = fbm3(scale(p, 3.0f), 5, 0.5f, seed);
        s.albedo = scale(F3{0.32f, 0.30f, 0.29f}, 0.8f + 0.4f * base);
        const float2 c1 = craters(p, 6.0f, seed + 1u), c2 = craters(p, 17.0f, seed + 2u);
        s.albedo = scale(s.albedo, 1.0f - 0.3f * fmaxf(c1.x, c2.x) + 0.25f * fmaxf(c1.y, c2.y));
        s.atmo = {0.0f, 0.0f, 0.0f};
    } else if (look == kEarth) {
        const float land = fbm3(scale(p, 2.2f), 6, 0.55f, seed);
        const float coast = smoothstep(0.02f, 0.08f, land);
        const float dry = fbm3(add_s(scale(p, 4.0f), 17.0f), 4, 0.5f, seed + 1u);
        const F3 ground = mix3(F3{0.10f, 0.22f, 0.07f}, F3{0.42f, 0.35f, 0.22f},
                               smoothstep(-0.2f, 0.4f, dry + 0.6f * (1.0f - fabsf(lat) * 1.6f)));
        s.albedo = mix3(F3{0.015f, 0.05f, 0.13f}, ground, coast);
        s.albedo = mix3(s.albedo, F3{0.92f, 0.94f, 0.97f}, smoothstep(0.78f, 0.86f, fabsf(lat) + 0.08f * land));
        const F3 sun_local = body_local(b, normalize(xyz4(b.light)));
        const float cloud = smoothstep(0.1f, 0.6f, planet_clouds(p, seed, 3.5f, time));
        const float shade = smoothstep(0.1f, 0.6f, planet_clouds(normalize(add(p, scale(sun_local, 0.025f))), seed, 3.5f, time));
        s.albedo = scale(s.albedo, 1.0f - 0.45f * shade);
        s.albedo = mix3(s.albedo, F3{0.95f, 0.95f, 0.95f}, cloud * 0.8f);
        s.specular = 0.7f * (1.0f - coast) * (1.0f - cloud);
        s.roughness = 0.3f;
        s.atmo = {0.35f, 0.58f, 1.0f};
    } else if (look == kCloudy) {
        const float w = fbm3(scale(p, 3.0f), 5, 0.5f, seed);
        const float bands = 0.5f + 0.5f * sinf(lat * 9.0f + 3.0f * w);
        s.albedo = mix3(F3{0.80f, 0.72f, 0.52f}, F3{0.95f, 0.90f, 0.75f}, bands);
        s.atmo = {1.0f, 0.88f, 0.6f};
    } else if (look == kGasWarm || look == kGasCold) {
        const F3 q = add(p, scale(F3{fbm3(scale(p, 3.0f), 4, 0.5f, seed), 0.0f, fbm3(add_s(scale(p, 3.0f), 9.0f), 4, 0.5f, seed + 1u)},
                                  0.12f));
        const float turb = fbm3(F3{q.x * 6.0f, q.y * 30.0f, q.z * 6.0f}, 5, 0.55f, seed + 2u);
        const float bands = 0.5f + 0.5f * sinf(q.y * 26.0f + 2.5f * turb) * lod_fade(26.0f / 6.283f, lod);
        if (look == kGasWarm) {
            s.albedo = mix3(F3{0.62f, 0.42f, 0.26f}, F3{0.93f, 0.86f, 0.74f}, bands);
            const float sx = p.x - 0.6f, sy = (p.y + 0.35f) * 1.8f;
            const float spot = 1.0f - smoothstep(0.08f, 0.16f, sqrtf(sx * sx + sy * sy));
            s.albedo = mix3(s.albedo, F3{0.72f, 0.32f, 0.20f}, spot * 0.8f);
            s.atmo = {1.0f, 0.85f, 0.65f};
        } else {
            s.albedo = mix3(F3{0.42f, 0.70f, 0.80f}, F3{0.62f, 0.86f, 0.92f}, bands * 0.35f + 0.3f * turb);
            s.atmo = {0.55f, 0.85f, 1.0f};
        }
        s.roughness = 0.9f;
    } else {  // lava
        const float crust = fbm3(scale(p, 3.0f), 5, 0.5f, seed);
        const float cracks = ridged(scale(p, 5.0f), 5, seed + 3u);
        s.albedo = scale(F3{0.06f, 0.05f, 0.05f}, 0.7f + 0.6f * crust);
        const float glow = smoothstep(0.82f, 0.96f, cracks);
        s.emission = scale(scale(F3{1.0f, 0.35f, 0.05f}, glow), 2.5f);
        s.atmo = {1.0f, 0.45f, 0.2f};
    }
    s.albedo = mul3(s.albedo, xyz4(b.tint));
    return s;
}

__device__ __forceinline__ F3 rgb3(float4 c) { return {c.x, c.y, c.z}; }
__device__ __forceinline__ float max3(F3 c) { return fmaxf(c.x, fmaxf(c.y, c.z)); }

// bodies.glsl:224-292 shadeBodySurface: radiance leaving the surface towards the viewer
__device__ inline F3 shade_body_surface(const Tex& tx, const bhr_body& b, F3 n, F3 view_dir, float lod, float time) {
    if (b.rel_pos[3] > 0.5f) {
        const float mu = fmaxf(dot(n, scale(view_dir, -1.0f)), 0.0f);
        const F3 p = body_local(b, n);
        const uint32_t seed = uint32_t(b.look[1]);
        const float teff = b.light_color[3];
        if (b.tint[3] > 0.0f) {  // an exploding photosphere
            const float turb = b.tint[3], ph = b.ring[2];
            const F3 q = scale(p, fmaxf(b.look[2], 1.0f));
            const F3 q6 = scale(q, 0.6f);
            const F3 warp{fbm3(add(q6, F3{0.0f, 0.0f, ph}), 2, 0.5f, seed + 11u), fbm3(add(q6, F3{5.2f, 1.3f, ph}), 2, 0.5f, seed + 13u),
                          fbm3(add(q6, F3{9.1f, 4.7f, ph}), 2, 0.5f, seed + 17u)};
            const float plume = fbm3(add(add(q, scale(warp, 1.8f)), F3{0.0f, 0.7f * ph, 0.0f}), 4, 0.55f, seed);
            const float heads = smoothstep(-0.05f, 0.45f, plume);
            const float lanes = 1.0f - smoothstep(-0.45f, -0.05f, plume);
            const float limb_x = 0.25f + 0.75f * gpow(mu, 0.6f);
            const float t_local_x = teff * (0.8f + 0.2f * gpow(mu, 0.4f)) * mixf(1.0f, 0.86f + 0.26f * heads - 0.08f * lanes, turb);
            const float ix = b.light[3] * limb_x * mixf(1.0f, (0.5f + 0.9f * heads) * (1.0f - 0.5f * lanes), turb);
            const F3 base_x = rgb3(blackbody(tx, teff));
            return scale(rgb3(blackbody(tx, t_local_x)), ix / fmaxf(max3(base_x), 1e-3f));
        }
        const float cool = clampf((7500.0f - teff) / 2500.0f, 0.0f, 1.0f);
        const float freq = b.look[2] > 0.0f ? b.look[2] : 70.0f;
        const float tt = time * 0.02f;
        const float g1 = fbm3(add(scale(p, freq), F3{0.0f, tt, 0.0f}), 3, 0.55f, seed);
        const float lanes = smoothstep(0.0f, 0.35f, fabsf(g1));
        const float gran = mixf(1.0f, mixf(1.0f, 0.78f + 0.3f * lanes, 0.35f + 0.65f * cool), lod_fade(freq, lod));
        const float sg = fbm3(add_s(scale(p, 6.0f), tt * 0.2f), 2, 0.5f, seed + 7u);
        const float spot_n = fbm3(add_s(scale(p, 3.5f), 13.1f), 3, 0.5f, seed + 3u);
        const float spot = cool * smoothstep(0.40f, 0.52f, spot_n);
        const float umbra = cool * smoothstep(0.50f, 0.58f, spot_n);
        const float limb = 0.32f + 0.68f * gpow(mu, 0.55f);
        const float faculae = (1.0f - mu) * smoothstep(0.2f, 0.5f, sg) * 0.25f * cool;
        const float t_local = teff * (0.84f + 0.16f * gpow(mu, 0.4f)) * (1.0f - 0.2f * spot - 0.2f * umbra) * (0.98f + 0.04f * sg);
        const float I = b.light[3] * limb * gran * (1.0f - 0.5f * spot - 0.4f * umbra) * (1.0f + faculae);
        if (b.look[2] < 0.0f) return scale(rgb3(blackbody(tx, t_local)), I * blackbody(tx, teff).w);
        const F3 base = rgb3(blackbody(tx, teff));
        return scale(rgb3(blackbody(tx, t_local)), I / fmaxf(max3(base), 1e-3f));
    }
    const Surface s = planet_surface(b, n, lod, time);
    const F3 L = normalize(xyz4(b.light));
    const float ndl = dot(n, L);
    const float atmo = b.look[2];
    const float wrap = mixf(fmaxf(ndl, 0.0f), clampf((ndl + 0.25f) / 1.25f, 0.0f, 1.0f), clampf(atmo, 0.0f, 1.0f));
    const F3 irr = scale(xyz4(b.light_color), b.light[3]);
    F3 col = add(add(scale(mul3(s.albedo, irr), wrap), scale(mul3(s.albedo, irr), 0.015f)), s.emission);
    if (s.specular > 0.0f && ndl > 0.0f) {
        const F3 h = normalize(sub(L, view_dir));
        const float shininess = mixf(400.0f, 20.0f, s.roughness);
        col = add(col, scale(scale(scale(scale(irr, s.specular), gpow(fmaxf(dot(n, h), 0.0f), shininess)), ndl), 0.6f));
    }
    if (atmo > 0.0f) {
        const float rim = gpow(1.0f - fmaxf(dot(n, scale(view_dir, -1.0f)), 0.0f), 3.0f);
        col = add(col, scale(scale(scale(scale(mul3(s.atmo, irr), rim), atmo), 0.6f), clampf(ndl + 0.35f, 0.0f, 1.0f)));
    }
    return col;
}

// bodies.glsl:34-44 raySphere
__device__ __forceinline__ float ray_sphere3(F3 ro, F3 rd, F3 c, float r, float t_min, float t_max) {
    const F3 oc = sub(ro, c);
    const float b = dot(oc, rd);
    const float cc = dot(oc, oc) - r * r;
    const float disc = b * b - cc;
    if (disc < 0.0f) return -1.0f;
    const float s = sqrtf(disc);
    float t = -b - s;
    if (t <= t_min) t = -b + s;
    return (t > t_min && t < t_max) ? t : -1.0f;
}

// bodies.glsl:294-317 ringSample: colour (rgb) and opacity (w) of the ring plane along the ray
__device__ inline float4 ring_sample(const bhr_body& b, F3 c, F3 ro, F3 rd, float t_max, float& t_ring) {
    t_ring = -1.0f;
    const float4 none = make_float4(0.f, 0.f, 0.f, 0.f);
    if (b.ring[1] <= 0.0f) return none;
    const F3 ax = normalize(xyz4(b.axis));
    const float denom = dot(rd, ax);
    if (fabsf(denom) < 1e-6f) return none;
    const float t = dot(sub(c, ro), ax) / denom;
    if (t <= 0.0f || t >= t_max) return none;
    const F3 q = sub(add(ro, scale(rd, t)), c);
    const float rr = len(q);
    if (rr < b.ring[0] || rr > b.ring[1]) return none;
    const float u = (rr - b.ring[0]) / (b.ring[1] - b.ring[0]);
    float dens = 0.55f + 0.45f * gnoise3(F3{u * 60.0f, 0.0f, 0.0f}, 77u);
    dens *= smoothstep(0.0f, 0.04f, u) * (1.0f - smoothstep(0.96f, 1.0f, u));
    dens *= 1.0f - 0.85f * (1.0f - smoothstep(0.55f, 0.57f, u)) * smoothstep(0.52f, 0.54f, u);
    const F3 L = normalize(xyz4(b.light));
    const float sh = ray_sphere3(q, L, F3{0.f, 0.f, 0.f}, b.pos_radius[3], 0.0f, 1e30f) > 0.0f ? 0.1f : 1.0f;
    const F3 col = scale(scale(scale(mul3(mul3(F3{0.80f, 0.72f, 0.58f}, xyz4(b.tint)), xyz4(b.light_color)), b.light[3]),
                               0.3f + 0.7f * fabsf(dot(L, ax))),
                         sh);
    t_ring = t;
    return make_float4(col.x, col.y, col.z, clampf(dens, 0.0f, 0.95f));
}

// bodies.glsl:319-341 traceBody: sphere and rings along a straight ray; footprint = radians per pixel
__device__ inline float4 trace_body(const Tex& tx, const bhr_body& b, F3 c, F3 ro, F3 rd, float t_max, float& t_hit,
                                    float footprint, float time) {
    const float R = b.pos_radius[3];
    const float ts = ray_sphere3(ro, rd, c, R, 0.0f, t_max);
    float tr;
    const float4 ring = ring_sample(b, c, ro, rd, ts > 0.0f ? ts : t_max, tr);
    float4 res = make_float4(0.f, 0.f, 0.f, 0.f);
    t_hit = -1.0f;
    if (ts > 0.0f) {
        const F3 n = normalize(sub(add(ro, scale(rd, ts)), c));
        const float lod = footprint * ts / R / fmaxf(dot(n, scale(rd, -1.0f)), 0.08f);
        const float op = clampf(b.ring[3], 0.0f, 1.0f);
        const F3 sc = scale(shade_body_surface(tx, b, n, rd, lod, time), op);
        res = make_float4(sc.x, sc.y, sc.z, op);
        t_hit = ts;
    }
    if (tr > 0.0f) {
        res = make_float4(ring.x * ring.w + res.x * (1.0f - ring.w), ring.y * ring.w + res.y * (1.0f - ring.w),
                          ring.z * ring.w + res.z * (1.0f - ring.w), ring.w + res.w * (1.0f - ring.w));
        t_hit = t_hit > 0.0f ? fminf(t_hit, tr) : tr;
    }
    return res;
}

// bodies.glsl:343-361 bodyHalo: the glow around a star or an airy planet the ray just missed
__device__ inline F3 body_halo(const Tex& tx, const bhr_body& b, F3 c, F3 ro, F3 rd, float t_max) {
    const float R = b.pos_radius[3];
    const F3 oc = sub(c, ro);
    const float t = clampf(dot(oc, rd), 0.0f, t_max);
    const float d = len(sub(add(ro, scale(rd, t)), c));
    if (d < R) return {0.f, 0.f, 0.f};
    const float x = (d - R) / R;
    if (b.rel_pos[3] > 0.5f) {
        const float4 bb = blackbody(tx, b.light_color[3]);
        return scale(scale(scale(rgb3(bb), b.light[3]), 0.25f), gexp(-x * 6.0f));
    }
    const float atmo = b.look[2];
    if (atmo <= 0.0f) return {0.f, 0.f, 0.f};
    const F3 L = normalize(xyz4(b.light));
    const F3 to_point = normalize(sub(add(ro, scale(rd, t)), c));
    const float lit = clampf(dot(to_point, L) + 0.3f, 0.0f, 1.0f);
    return scale(scale(scale(scale(scale(mul3(look_atmo_color(int(b.look[0] + 0.5f)), xyz4(b.light_color)), b.light[3]), atmo),
                             lit),
                       0.5f),
                 gexp(-x * 40.0f));
}

// blackhole.frag:50-62 nearestBodyStraight
__device__ inline float4 nearest_body_straight(const Tex& tx, const bhr_body* bodies, int nb, F3 ro, F3 rd, bool camera_frame,
                                               uint32_t skip, float t_max, float footprint, float time) {
    float best_t = t_max;
    float4 best = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int k = 0; k < nb; ++k) {
        if (skip & (1u << k)) continue;
        const F3 c = camera_frame ? xyz4(bodies[k].rel_pos) : xyz4(bodies[k].pos_radius);
        {  // the sphere and its ring lie within ext of c: a ray passing wider, or a body behind the
           // origin seen from outside, is missed by both tests below. The slack (1e-6 |oc|^2) is
           // above both computations' FP32 rounding, so no hit is culled.
            const F3 oc = sub(c, ro);
            const float oo = dot(oc, oc), tc = dot(oc, rd);
            const float ext = fmaxf(bodies[k].pos_radius[3], bodies[k].ring[1]);
            const float lim = fmaf(ext, ext, fmaf(1e-6f, oo, 1e-6f));
            if (oo - tc * tc > lim || (tc < 0.0f && oo > lim)) continue;
        }
        float t_hit;
        const float4 col = trace_body(tx, bodies[k], c, ro, rd, best_t, t_hit, footprint, time);
        if (t_hit > 0.0f && t_hit < best_t) {
            best_t = t_hit;
            best = col;
        }
    }
    return best;
}

// blackhole.frag:43-47 composite: true once the ray is fully blocked
__device__ __forceinline__ bool composite_layer(float4 l, F3& col, float& trans) {
    col = add(col, scale(F3{l.x, l.y, l.z}, trans));
    trans *= 1.0f - clampf(l.w, 0.0f, 1.0f);
    return trans < 0.004f;
}

// blackhole.frag:255-296: after the march, the hit body (opaque, or turning transparent and
// letting the ray on along its chord), the straight stretches beyond the escape point, and the
// halos of the bodies the ray just missed. status / esc_dir / col / trans are updated in place.
__device__ inline void shade_bodies_after_march(const Tex& tx, const bhr_body* bodies, int nb, const bhr_body_hit& bh,
                                                bool far_mode, float rcam, F3 dir, F3 rd_near, float footprint, float time,
                                                int& status, F3& esc_dir, F3& col, float& trans) {
    const uint32_t near_mask = bh.near_mask;
    uint32_t seen = 0;
    if (status == BHR_STATUS_BODY && bh.body >= 0) {
        const bhr_body& bd = bodies[bh.body];
        F3 ro = xyz4(bh.ro), rd = xyz4(bh.rd), c = xyz4(bd.pos_radius);
        float t = bh.t;
        const float near_tol = fmaxf(2e-6f * rcam, 1e-9f);
        if (bh.body == bh.near_idx && bh.travelled + near_tol >= bh.near_t) {
            ro = F3{0.f, 0.f, 0.f};
            rd = rd_near;
            c = xyz4(bd.rel_pos);
            t = bh.near_t;
        }
        const F3 n = normalize(sub(add(ro, scale(rd, t)), c));
        const float lod = footprint * t / bd.pos_radius[3] / fmaxf(dot(n, scale(rd, -1.0f)), 0.08f);
        const float op = clampf(bd.ring[3], 0.0f, 1.0f);
        col = add(col, scale(shade_body_surface(tx, bd, n, rd, lod, time), trans * op));
        trans *= 1.0f - op;
        if (trans > 0.004f) {
            status = BHR_STATUS_ESCAPED;
            esc_dir = rd;
            seen = 1u << bh.body;
        } else {
            trans = 0.0f;
        }
    }
    if (status == BHR_STATUS_ESCAPED) {
        float4 layer = far_mode ? nearest_body_straight(tx, bodies, nb, F3{0.f, 0.f, 0.f}, dir, true, seen, 1e30f, footprint, time)
                                : nearest_body_straight(tx, bodies, nb, F3{0.f, 0.f, 0.f}, rd_near, true, ~near_mask | seen, 1e30f,
                                                        footprint, time);
        if (!far_mode && layer.w <= 0.0f)
            layer = nearest_body_straight(tx, bodies, nb, xyz4(bh.x), esc_dir, false, near_mask | seen, 1e30f, footprint, time);
        if (composite_layer(layer, col, trans)) status = BHR_STATUS_BODY;
    }
    if (status != BHR_STATUS_BODY) {
        F3 halo{0.f, 0.f, 0.f};
        for (int k = 0; k < nb; ++k) {
            if (!far_mode && (near_mask & (1u << k)) == 0u) continue;
            halo = add(halo, body_halo(tx, bodies[k], xyz4(bodies[k].rel_pos), F3{0.f, 0.f, 0.f}, far_mode ? dir : rd_near, 1e30f));
        }
        col = add(col, scale(halo, trans));
    }
}

}  // namespace shading
}  // namespace bhr
