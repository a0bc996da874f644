// CPU restatement of the shading of bodies (planets and stars) -- TEST INFRASTRUCTURE ONLY.
//
//   shaders/common.glsl:24-57,78-88     hash3u, gnoise3 (gradient noise), fbm3
//   shaders/bodies.glsl:28,47-223       lodFade, bodyLocal, ridged, craters, lookAtmoColor,
//                                       planetClouds, planetSurface (nine looks)
//   shaders/bodies.glsl:224-292         shadeBodySurface (stars: granulation, spots, limb; an
//                                       exploding photosphere; planets: wrap light, specular, rim)
//   shaders/bodies.glsl:294-361         ringSample, traceBody, bodyHalo
//   shaders/blackhole.frag:41-62        composite, nearestBodyStraight
//   shaders/blackhole.frag:255-296      after the march: the hit body, the straight stretches
//                                       and the halos of the bodies the ray just missed
// FP32 like the shader, in the GLSL formula order. The footprint that fades unresolved surface
// detail (gSurfaceLod) is passed as `lod`.
#pragma once
#include <cmath>
#include <cstdint>

#include "march.hpp"
#include "shade.hpp"

namespace oracle {
namespace body {

using shade::F3;
using shade::clampf;
using shade::cross;
using shade::divs;
using shade::dot;
using shade::length;
using shade::mixf;
using shade::normalize;
using shade::smoothstep;

inline F3 mix3(F3 a, F3 b, float t) { return {mixf(a.x, b.x, t), mixf(a.y, b.y, t), mixf(a.z, b.z, t)}; }
inline F3 mul3(F3 a, F3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline F3 add_s(F3 a, float s) { return {a.x + s, a.y + s, a.z + s}; }
inline F3 xyz(const float* q) { return {q[0], q[1], q[2]}; }

// common.glsl:24 hash3u
inline F3 hash3u(uint32_t x, uint32_t y, uint32_t z) {
    const shade::U3 h = shade::pcg3d({x, y, z});
    const float s = 1.0f / 4294967296.0f;
    return {float(h.x) * s, float(h.y) * s, float(h.z) * s};
}

// common.glsl:41-57 gnoise3: gradient noise on the unbounded lattice
inline float gnoise3(F3 p, uint32_t salt) {
    const F3 i{std::floor(p.x), std::floor(p.y), std::floor(p.z)};
    const F3 f = p - i;
    auto fade = [](float t) { return t * t * t * (t * (t * 6.0f - 15.0f) + 10.0f); };
    const F3 u{fade(f.x), fade(f.y), fade(f.z)};
    const int c[3] = {int(i.x), int(i.y), int(i.z)};
    auto corner = [&](int ox, int oy, int oz) {
        const F3 g = shade::grad3(c[0] + ox, c[1] + oy, c[2] + oz, salt);
        return dot(g, f - F3{float(ox), float(oy), float(oz)});
    };
    const float nx00 = mixf(corner(0, 0, 0), corner(1, 0, 0), u.x), nx10 = mixf(corner(0, 1, 0), corner(1, 1, 0), u.x);
    const float nx01 = mixf(corner(0, 0, 1), corner(1, 0, 1), u.x), nx11 = mixf(corner(0, 1, 1), corner(1, 1, 1), u.x);
    return 1.4f * mixf(mixf(nx00, nx10, u.y), mixf(nx01, nx11, u.y), u.z);
}

// common.glsl:78-88 fbm3
inline float fbm3(F3 p, int octaves, float gain, uint32_t salt) {
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
inline float lod_fade(float frequency, float lod) { return 1.0f - smoothstep(0.25f, 1.0f, frequency * lod); }

// bodies.glsl:47-55 bodyLocal: the normal in body coordinates (y along the spin axis)
inline F3 body_local(const bhr_body& b, F3 n) {
    const F3 ax = normalize(xyz(b.axis));
    const F3 ref = std::fabs(ax.y) < 0.95f ? F3{0.0f, 1.0f, 0.0f} : F3{1.0f, 0.0f, 0.0f};
    const F3 e1 = normalize(cross(ref, ax));
    const F3 e2 = cross(ax, e1);
    const float ca = std::cos(b.look[3]), sa = std::sin(b.look[3]);
    const F3 u = e1 * ca + e2 * sa;
    const F3 v = (e1 * -1.0f) * sa + e2 * ca;
    return {dot(n, u), dot(n, ax), dot(n, v)};
}

// bodies.glsl:57-66 ridged
inline float ridged(F3 p, int oct, uint32_t salt) {
    float s = 0.0f, a = 0.5f, nrm = 0.0f;
    for (int i = 0; i < oct; ++i) {
        s += a * (1.0f - std::fabs(gnoise3(p, salt + uint32_t(i) * 17u)));
        nrm += a;
        a *= 0.5f;
        p = F3{p.x * 2.03f + 7.1f, p.y * 2.03f + 7.1f, p.z * 2.03f + 7.1f};
    }
    return s / nrm;
}

// bodies.glsl:69-89 craters: (floor 0..1, rim)
struct V2 {
    float x, y;
};
inline V2 craters(F3 p, float scale, uint32_t salt) {
    const F3 q = p * scale;
    const F3 i{std::floor(q.x), std::floor(q.y), std::floor(q.z)};
    V2 best{0.0f, 0.0f};
    for (int z = -1; z <= 1; ++z)
        for (int y = -1; y <= 1; ++y)
            for (int x = -1; x <= 1; ++x) {
                const F3 c{i.x + float(x), i.y + float(y), i.z + float(z)};
                const F3 h = hash3u(uint32_t(int(c.x)) + salt, uint32_t(int(c.y)) + salt * 3u, uint32_t(int(c.z)) + salt * 7u);
                if (h.x > 0.45f) continue;
                const F3 center = c + h;
                const float rad = 0.15f + 0.35f * h.y;
                const float d = length(q - center) / rad;
                if (d < 1.25f) {
                    const float floorv = 1.0f - smoothstep(0.7f, 1.0f, d);
                    const float rim = smoothstep(0.75f, 1.0f, d) * (1.0f - smoothstep(1.0f, 1.25f, d));
                    best = V2{std::fmax(best.x, floorv), std::fmax(best.y, rim)};
                }
            }
    return best;
}

enum : int { kRocky = 0, kDesert = 1, kOcean = 2, kIce = 3, kEarth = 4, kGasWarm = 5, kGasCold = 6, kCloudy = 7, kLava = 8 };

// bodies.glsl:91-101 lookAtmoColor
inline F3 look_atmo_color(int look) {
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
inline float planet_clouds(F3 p, uint32_t seed, float scale, float time) {
    const float a = time * 0.004f;
    const float ca = std::cos(a), sa = std::sin(a);
    const F3 q{ca * p.x - sa * p.z, p.y, sa * p.x + ca * p.z};
    const F3 q17 = q * 1.7f;
    const F3 w{fbm3(q17, 3, 0.5f, seed + 21u), fbm3(add_s(q17, 4.1f), 3, 0.5f, seed + 22u),
               fbm3(add_s(q17, 8.3f), 3, 0.5f, seed + 23u)};
    return fbm3(q * scale + w * 1.4f, 6, 0.55f, seed + 8u);
}

// bodies.glsl:121-221 planetSurface
inline Surface planet_surface(const bhr_body& b, F3 n, float lod, float time) {
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
        const float bands = 0.5f + 0.5f * std::sin(p.x * 14.0f + 3.0f * swell) * lod_fade(14.0f / 6.283f, lod);
        const float detail = fbm3(p * 9.0f, 4, 0.5f, seed + 3u) * lod_fade(9.0f, lod);
        const F3 deep{0.03f, 0.10f, 0.15f}, crest{0.16f, 0.36f, 0.42f};
        s.albedo = mix3(deep, crest, smoothstep(0.55f, 0.95f, bands) * 0.8f + 0.2f * detail);
        const float foam = smoothstep(0.9f, 0.99f, bands) * smoothstep(0.0f, 0.5f, detail) * lod_fade(20.0f, lod);
        s.albedo = mix3(s.albedo, F3{0.8f, 0.8f, 0.8f}, foam * 0.6f);
        const F3 sun_local = body_local(b, normalize(xyz(b.light)));
        const float cloud = smoothstep(0.25f, 0.7f, planet_clouds(p, seed + 9u, 4.0f, time));
        const float shade = smoothstep(0.25f, 0.7f, planet_clouds(normalize(p + sun_local * 0.025f), seed + 9u, 4.0f, time));
        s.albedo = s.albedo * (1.0f - 0.4f * shade);
        s.albedo = mix3(s.albedo, F3{0.9f, 0.9f, 0.9f}, cloud * 0.55f);
        s.specular = 0.8f * (1.0f - cloud);
        s.roughness = 0.25f;
        s.atmo = {0.35f, 0.6f, 1.0f};
    } else if (look == kIce) {
        const float base = fbm3(p * 3.0f, 5, 0.5f, seed);
        const float cracks = ridged(p * 6.0f, 4, seed + 5u);
        const F3 ice = mix3(F3{0.78f, 0.84f, 0.9f}, F3{0.95f, 0.97f, 1.0f}, 0.5f + 0.5f * base);
        s.albedo = mix3(ice, F3{0.42f, 0.55f, 0.68f}, smoothstep(0.86f, 0.97f, cracks));
        const float cloud = smoothstep(0.35f, 0.8f, fbm3(add_s(p * 5.0f, 3.0f), 4, 0.5f, seed + 2u));
        s.albedo = mix3(s.albedo, F3{0.97f, 0.97f, 0.97f}, cloud * 0.4f);
        s.specular = 0.3f;
        s.roughness = 0.5f;
        s.atmo = {0.6f, 0.78f, 1.0f};
    } else if (look == kDesert) {
        const float big = fbm3(p * 2.5f, 5, 0.55f, seed);
        const float dunes = 0.5f + 0.5f * std::sin(dot(p, F3{40.0f, 13.0f, 27.0f}) + 8.0f * fbm3(p * 6.0f, 3, 0.5f, seed + 1u)) *
                                       lod_fade(8.0f, lod);
        const F3 sand = mix3(F3{0.62f, 0.40f, 0.24f}, F3{0.86f, 0.66f, 0.44f}, 0.5f + 0.5f * big);
        s.albedo = sand * (0.85f + 0.15f * dunes);
        const V2 cr = craters(p, 7.0f, seed + 4u);
        s.albedo = s.albedo * (1.0f - 0.25f * cr.x + 0.15f * cr.y);
        s.albedo = mix3(s.albedo, F3{0.92f, 0.9f, 0.88f}, smoothstep(0.82f, 0.92f, std::fabs(lat)));
        s.atmo = {1.0f, 0.62f, 0.42f};
    } else if (look == kRocky) {
        const float base = fbm3(p * 3.0f, 5, 0.5f, seed);
        s.albedo = F3{0.32f, 0.30f, 0.29f} * (0.8f + 0.4f * base);
        const V2 c1 = craters(p, 6.0f, seed + 1u), c2 = craters(p, 17.0f, seed + 2u);
        s.albedo = s.albedo * (1.0f - 0.3f * std::fmax(c1.x, c2.x) + 0.25f * std::fmax(c1.y, c2.y));
        s.atmo = {0.0f, 0.0f, 0.0f};
    } else if (look == kEarth) {
        const float land = fbm3(p * 2.2f, 6, 0.55f, seed);
        const float coast = smoothstep(0.02f, 0.08f, land);
        const F3 ocean{0.015f, 0.05f, 0.13f};
        const float dry = fbm3(add_s(p * 4.0f, 17.0f), 4, 0.5f, seed + 1u);
        const F3 ground = mix3(F3{0.10f, 0.22f, 0.07f}, F3{0.42f, 0.35f, 0.22f},
                               smoothstep(-0.2f, 0.4f, dry + 0.6f * (1.0f - std::fabs(lat) * 1.6f)));
        s.albedo = mix3(ocean, ground, coast);
        s.albedo = mix3(s.albedo, F3{0.92f, 0.94f, 0.97f}, smoothstep(0.78f, 0.86f, std::fabs(lat) + 0.08f * land));
        const F3 sun_local = body_local(b, normalize(xyz(b.light)));
        const float cloud = smoothstep(0.1f, 0.6f, planet_clouds(p, seed, 3.5f, time));
        const float shade = smoothstep(0.1f, 0.6f, planet_clouds(normalize(p + sun_local * 0.025f), seed, 3.5f, time));
        s.albedo = s.albedo * (1.0f - 0.45f * shade);
        s.albedo = mix3(s.albedo, F3{0.95f, 0.95f, 0.95f}, cloud * 0.8f);
        s.specular = 0.7f * (1.0f - coast) * (1.0f - cloud);
        s.roughness = 0.3f;
        s.atmo = {0.35f, 0.58f, 1.0f};
    } else if (look == kCloudy) {
        const float w = fbm3(p * 3.0f, 5, 0.5f, seed);
        const float bands = 0.5f + 0.5f * std::sin(lat * 9.0f + 3.0f * w);
        s.albedo = mix3(F3{0.80f, 0.72f, 0.52f}, F3{0.95f, 0.90f, 0.75f}, bands);
        s.atmo = {1.0f, 0.88f, 0.6f};
    } else if (look == kGasWarm || look == kGasCold) {
        const F3 q = p + F3{fbm3(p * 3.0f, 4, 0.5f, seed), 0.0f, fbm3(add_s(p * 3.0f, 9.0f), 4, 0.5f, seed + 1u)} * 0.12f;
        const float turb = fbm3(F3{q.x * 6.0f, q.y * 30.0f, q.z * 6.0f}, 5, 0.55f, seed + 2u);
        const float bands = 0.5f + 0.5f * std::sin(q.y * 26.0f + 2.5f * turb) * lod_fade(26.0f / 6.283f, lod);
        if (look == kGasWarm) {
            s.albedo = mix3(F3{0.62f, 0.42f, 0.26f}, F3{0.93f, 0.86f, 0.74f}, bands);
            const float sx = p.x - 0.6f, sy = (p.y + 0.35f) * 1.8f;
            const float spot = 1.0f - smoothstep(0.08f, 0.16f, std::sqrt(sx * sx + sy * sy));
            s.albedo = mix3(s.albedo, F3{0.72f, 0.32f, 0.20f}, spot * 0.8f);
            s.atmo = {1.0f, 0.85f, 0.65f};
        } else {
            s.albedo = mix3(F3{0.42f, 0.70f, 0.80f}, F3{0.62f, 0.86f, 0.92f}, bands * 0.35f + 0.3f * turb);
            s.atmo = {0.55f, 0.85f, 1.0f};
        }
        s.roughness = 0.9f;
    } else {  // lava
        const float crust = fbm3(p * 3.0f, 5, 0.5f, seed);
        const float cracks = ridged(p * 5.0f, 5, seed + 3u);
        s.albedo = F3{0.06f, 0.05f, 0.05f} * (0.7f + 0.6f * crust);
        const float glow = smoothstep(0.82f, 0.96f, cracks);
        s.emission = F3{1.0f, 0.35f, 0.05f} * glow * 2.5f;
        s.atmo = {1.0f, 0.45f, 0.2f};
    }
    s.albedo = mul3(s.albedo, xyz(b.tint));
    return s;
}

inline F3 rgb(const shade::RGBA& c) { return {c.r, c.g, c.b}; }
inline float max3(F3 c) { return std::fmax(c.x, std::fmax(c.y, c.z)); }

// bodies.glsl:224-292 shadeBodySurface: radiance leaving the surface towards the viewer
inline F3 shade_body_surface(const shade::Tex& tx, const bhr_body& b, F3 n, F3 view_dir, float lod, float time) {
    if (b.rel_pos[3] > 0.5f) {
        const float mu = std::fmax(dot(n, view_dir * -1.0f), 0.0f);
        const F3 p = body_local(b, n);
        const uint32_t seed = uint32_t(b.look[1]);
        const float teff = b.light_color[3];
        if (b.tint[3] > 0.0f) {  // an exploding photosphere
            const float turb = b.tint[3], ph = b.ring[2];
            const F3 q = p * std::fmax(b.look[2], 1.0f);
            const F3 q6 = q * 0.6f;
            const F3 warp{fbm3(q6 + F3{0.0f, 0.0f, ph}, 2, 0.5f, seed + 11u), fbm3(q6 + F3{5.2f, 1.3f, ph}, 2, 0.5f, seed + 13u),
                          fbm3(q6 + F3{9.1f, 4.7f, ph}, 2, 0.5f, seed + 17u)};
            const float plume = fbm3(q + warp * 1.8f + F3{0.0f, 0.7f * ph, 0.0f}, 4, 0.55f, seed);
            const float heads = smoothstep(-0.05f, 0.45f, plume);
            const float lanes = 1.0f - smoothstep(-0.45f, -0.05f, plume);
            const float limb_x = 0.25f + 0.75f * std::pow(mu, 0.6f);
            const float t_local_x =
                teff * (0.8f + 0.2f * std::pow(mu, 0.4f)) * mixf(1.0f, 0.86f + 0.26f * heads - 0.08f * lanes, turb);
            const float ix = b.light[3] * limb_x * mixf(1.0f, (0.5f + 0.9f * heads) * (1.0f - 0.5f * lanes), turb);
            const F3 base_x = rgb(shade::blackbody(tx, teff));
            return rgb(shade::blackbody(tx, t_local_x)) * (ix / std::fmax(max3(base_x), 1e-3f));
        }
        const float cool = clampf((7500.0f - teff) / 2500.0f, 0.0f, 1.0f);
        const float freq = b.look[2] > 0.0f ? b.look[2] : 70.0f;
        const float tt = time * 0.02f;
        const float g1 = fbm3(p * freq + F3{0.0f, tt, 0.0f}, 3, 0.55f, seed);
        const float lanes = smoothstep(0.0f, 0.35f, std::fabs(g1));
        const float gran = mixf(1.0f, mixf(1.0f, 0.78f + 0.3f * lanes, 0.35f + 0.65f * cool), lod_fade(freq, lod));
        const float sg = fbm3(add_s(p * 6.0f, tt * 0.2f), 2, 0.5f, seed + 7u);
        const float spot_n = fbm3(add_s(p * 3.5f, 13.1f), 3, 0.5f, seed + 3u);
        const float spot = cool * smoothstep(0.40f, 0.52f, spot_n);
        const float umbra = cool * smoothstep(0.50f, 0.58f, spot_n);
        const float limb = 0.32f + 0.68f * std::pow(mu, 0.55f);
        const float faculae = (1.0f - mu) * smoothstep(0.2f, 0.5f, sg) * 0.25f * cool;
        const float t_local = teff * (0.84f + 0.16f * std::pow(mu, 0.4f)) * (1.0f - 0.2f * spot - 0.2f * umbra) * (0.98f + 0.04f * sg);
        const float I = b.light[3] * limb * gran * (1.0f - 0.5f * spot - 0.4f * umbra) * (1.0f + faculae);
        if (b.look[2] < 0.0f) return rgb(shade::blackbody(tx, t_local)) * (I * shade::blackbody(tx, teff).a);
        const F3 base = rgb(shade::blackbody(tx, teff));
        return rgb(shade::blackbody(tx, t_local)) * (I / std::fmax(max3(base), 1e-3f));
    }
    const Surface s = planet_surface(b, n, lod, time);
    const F3 L = normalize(xyz(b.light));
    const float ndl = dot(n, L);
    const float atmo = b.look[2];
    const float wrap = mixf(std::fmax(ndl, 0.0f), clampf((ndl + 0.25f) / 1.25f, 0.0f, 1.0f), clampf(atmo, 0.0f, 1.0f));
    const F3 irr = xyz(b.light_color) * b.light[3];
    F3 col = mul3(s.albedo, irr) * wrap + mul3(s.albedo, irr) * 0.015f + s.emission;
    if (s.specular > 0.0f && ndl > 0.0f) {
        const F3 h = normalize(L - view_dir);
        const float shininess = mixf(400.0f, 20.0f, s.roughness);
        col = col + irr * s.specular * std::pow(std::fmax(dot(n, h), 0.0f), shininess) * ndl * 0.6f;
    }
    if (atmo > 0.0f) {
        const float rim = std::pow(1.0f - std::fmax(dot(n, view_dir * -1.0f), 0.0f), 3.0f);
        col = col + mul3(s.atmo, irr) * rim * atmo * 0.6f * clampf(ndl + 0.35f, 0.0f, 1.0f);
    }
    return col;
}

// bodies.glsl:34-44 raySphere in float
inline float ray_sphere(F3 ro, F3 rd, F3 c, float r, float t_min, float t_max) {
    const F3 oc = ro - c;
    const float b = dot(oc, rd);
    const float cc = dot(oc, oc) - r * r;
    const float disc = b * b - cc;
    if (disc < 0.0f) return -1.0f;
    const float s = std::sqrt(disc);
    float t = -b - s;
    if (t <= t_min) t = -b + s;
    return (t > t_min && t < t_max) ? t : -1.0f;
}

struct Layer {
    F3 rgb;
    float a;
};

// bodies.glsl:294-317 ringSample: colour and opacity of the ring plane along the ray
inline Layer ring_sample(const bhr_body& b, F3 c, F3 ro, F3 rd, float t_max, float& t_ring) {
    t_ring = -1.0f;
    if (b.ring[1] <= 0.0f) return {{0, 0, 0}, 0.0f};
    const F3 ax = normalize(xyz(b.axis));
    const float denom = dot(rd, ax);
    if (std::fabs(denom) < 1e-6f) return {{0, 0, 0}, 0.0f};
    const float t = dot(c - ro, ax) / denom;
    if (t <= 0.0f || t >= t_max) return {{0, 0, 0}, 0.0f};
    const F3 q = ro + rd * t - c;
    const float rr = length(q);
    if (rr < b.ring[0] || rr > b.ring[1]) return {{0, 0, 0}, 0.0f};
    const float u = (rr - b.ring[0]) / (b.ring[1] - b.ring[0]);
    float dens = 0.55f + 0.45f * gnoise3(F3{u * 60.0f, 0.0f, 0.0f}, 77u);
    dens *= smoothstep(0.0f, 0.04f, u) * (1.0f - smoothstep(0.96f, 1.0f, u));
    dens *= 1.0f - 0.85f * (1.0f - smoothstep(0.55f, 0.57f, u)) * smoothstep(0.52f, 0.54f, u);
    const F3 L = normalize(xyz(b.light));
    const float sh = ray_sphere(q, L, F3{0, 0, 0}, b.pos_radius[3], 0.0f, 1e30f) > 0.0f ? 0.1f : 1.0f;
    const F3 col = mul3(mul3(F3{0.80f, 0.72f, 0.58f}, xyz(b.tint)), xyz(b.light_color)) * b.light[3] *
                   (0.3f + 0.7f * std::fabs(dot(L, ax))) * sh;
    t_ring = t;
    return {col, clampf(dens, 0.0f, 0.95f)};
}

// bodies.glsl:319-341 traceBody: sphere and rings along a straight ray; footprint = radians per pixel
inline Layer trace_body(const shade::Tex& tx, const bhr_body& b, F3 c, F3 ro, F3 rd, float t_max, float& t_hit,
                        float footprint, float time) {
    const float R = b.pos_radius[3];
    const float ts = ray_sphere(ro, rd, c, R, 0.0f, t_max);
    float tr;
    const Layer ring = ring_sample(b, c, ro, rd, ts > 0.0f ? ts : t_max, tr);
    Layer res{{0, 0, 0}, 0.0f};
    t_hit = -1.0f;
    if (ts > 0.0f) {
        const F3 n = normalize(ro + rd * ts - c);
        const float lod = footprint * ts / R / std::fmax(dot(n, rd * -1.0f), 0.08f);
        const float op = clampf(b.ring[3], 0.0f, 1.0f);
        res = {shade_body_surface(tx, b, n, rd, lod, time) * op, op};
        t_hit = ts;
    }
    if (tr > 0.0f) {
        res.rgb = ring.rgb * ring.a + res.rgb * (1.0f - ring.a);
        res.a = ring.a + res.a * (1.0f - ring.a);
        t_hit = t_hit > 0.0f ? std::fmin(t_hit, tr) : tr;
    }
    return res;
}

// bodies.glsl:343-361 bodyHalo: the glow around a star or an airy planet the ray just missed
inline F3 body_halo(const shade::Tex& tx, const bhr_body& b, F3 c, F3 ro, F3 rd, float t_max) {
    const float R = b.pos_radius[3];
    const F3 oc = c - ro;
    const float t = clampf(dot(oc, rd), 0.0f, t_max);
    const float d = length(ro + rd * t - c);
    if (d < R) return {0, 0, 0};
    const float x = (d - R) / R;
    if (b.rel_pos[3] > 0.5f) {
        const shade::RGBA bb = shade::blackbody(tx, b.light_color[3]);
        return rgb(bb) * b.light[3] * 0.25f * std::exp(-x * 6.0f);
    }
    const float atmo = b.look[2];
    if (atmo <= 0.0f) return {0, 0, 0};
    const F3 L = normalize(xyz(b.light));
    const F3 to_point = normalize(ro + rd * t - c);
    const float lit = clampf(dot(to_point, L) + 0.3f, 0.0f, 1.0f);
    return mul3(look_atmo_color(int(b.look[0] + 0.5f)), xyz(b.light_color)) * b.light[3] * atmo * lit * 0.5f *
           std::exp(-x * 40.0f);
}

// blackhole.frag:50-62 nearestBodyStraight
inline Layer nearest_body_straight(const shade::Tex& tx, const bhr_body* bodies, int nb, F3 ro, F3 rd, bool camera_frame,
                                   uint32_t skip, float t_max, float footprint, float time) {
    float best_t = t_max;
    Layer best{{0, 0, 0}, 0.0f};
    for (int k = 0; k < nb; ++k) {
        if (skip & (1u << k)) continue;
        const F3 c = camera_frame ? xyz(bodies[k].rel_pos) : xyz(bodies[k].pos_radius);
        float t_hit;
        const Layer col = trace_body(tx, bodies[k], c, ro, rd, best_t, t_hit, footprint, time);
        if (t_hit > 0.0f && t_hit < best_t) {
            best_t = t_hit;
            best = col;
        }
    }
    return best;
}

// blackhole.frag:43-47 composite: true once the ray is fully blocked
inline bool composite(const Layer& l, F3& col, float& trans) {
    col = col + l.rgb * trans;
    trans *= 1.0f - clampf(l.a, 0.0f, 1.0f);
    return trans < 0.004f;
}

// The pixel's state after the march that the body shading reads and changes.
struct PixelBodies {
    int status;   // BHR_STATUS_*, OPAQUE once the thin disk blocked the ray
    F3 esc_dir;   // escDir
    F3 col;
    float trans;
};

// blackhole.frag:255-296: the hit body (opaque or turning transparent), the straight stretches
// beyond the escape point, the halos. dir = the pixel's direction, rd_near = the geodesic's
// initial direction, footprint = the pixel's angle.
inline void shade_bodies_after_march(const shade::Tex& tx, const bhr_body* bodies, int nb, const bhr_body_hit& bh,
                                     bool far_mode, float rcam, F3 dir, F3 rd_near, float footprint, float time,
                                     PixelBodies& s) {
    const uint32_t near_mask = bh.near_mask;
    uint32_t seen = 0;
    if (s.status == BHR_STATUS_BODY && bh.body >= 0) {
        const bhr_body& bd = bodies[bh.body];
        F3 ro = xyz(bh.ro), rd = xyz(bh.rd), c = xyz(bd.pos_radius);
        float t = bh.t;
        const float near_tol = std::fmax(2e-6f * rcam, 1e-9f);
        if (bh.body == bh.near_idx && bh.travelled + near_tol >= bh.near_t) {
            ro = {0, 0, 0};
            rd = rd_near;
            c = xyz(bd.rel_pos);
            t = bh.near_t;
        }
        const F3 n = normalize(ro + rd * t - c);
        const float lod = footprint * t / bd.pos_radius[3] / std::fmax(dot(n, rd * -1.0f), 0.08f);
        const float op = clampf(bd.ring[3], 0.0f, 1.0f);
        s.col = s.col + shade_body_surface(tx, bd, n, rd, lod, time) * (s.trans * op);
        s.trans *= 1.0f - op;
        if (s.trans > 0.004f) {
            s.status = BHR_STATUS_ESCAPED;
            s.esc_dir = rd;
            seen = 1u << bh.body;
        } else {
            s.trans = 0.0f;
        }
    }
    if (s.status == BHR_STATUS_ESCAPED) {
        Layer layer = far_mode ? nearest_body_straight(tx, bodies, nb, F3{0, 0, 0}, dir, true, seen, 1e30f, footprint, time)
                               : nearest_body_straight(tx, bodies, nb, F3{0, 0, 0}, rd_near, true, ~near_mask | seen, 1e30f,
                                                       footprint, time);
        if (!far_mode && layer.a <= 0.0f)
            layer = nearest_body_straight(tx, bodies, nb, xyz(bh.x), s.esc_dir, false, near_mask | seen, 1e30f, footprint,
                                          time);
        if (composite(layer, s.col, s.trans)) s.status = BHR_STATUS_BODY;
    }
    if (s.status != BHR_STATUS_BODY) {
        F3 halo{0, 0, 0};
        for (int k = 0; k < nb; ++k) {
            if (!far_mode && (near_mask & (1u << k)) == 0u) continue;
            halo = halo + body_halo(tx, bodies[k], xyz(bodies[k].rel_pos), F3{0, 0, 0}, far_mode ? dir : rd_near, 1e30f);
        }
        s.col = s.col + halo * s.trans;
    }
}

// The body layers of a pixel inside oracle::shade::shade_view.
struct BodyPost {
    const shade::Tex* tx;
    const bhr_body* bodies;
    int nb;
    const bhr_body_hit* bh;  // per pixel
    const bhr_view* v;
    float rcam, footprint, time;
    void operator()(shade::PixelState& s, int i, int j) const {
        const bool lensing = v->lensing != 0 && v->far_mode == 0;
        F3 rd_near = s.dir;
        if (lensing) {  // normalize(initialVelocity(uCamPos, dir)) (blackhole.frag:78,107)
            const V3<float> iv = initialVelocity(V3<float>{v->cam_pos[0], v->cam_pos[1], v->cam_pos[2]},
                                                 V3<float>{s.dir.x, s.dir.y, s.dir.z});
            rd_near = normalize(F3{iv.x, iv.y, iv.z});
        }
        PixelBodies pb{s.status, s.esc_dir, s.col, s.trans};
        shade_bodies_after_march(*tx, bodies, nb, bh[int64_t(j) * v->width + i], v->far_mode != 0, rcam, s.dir, rd_near,
                                 footprint, time, pb);
        s.status = pb.status;
        s.esc_dir = pb.esc_dir;
        s.col = pb.col;
        s.trans = pb.trans;
        s.esc = pb.status == BHR_STATUS_ESCAPED;
    }
};

}  // namespace body
}  // namespace oracle
