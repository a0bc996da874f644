// The consumer of the hit records: the fragment shader's shading of a traced pixel when the
// disk is thin and no bodies, gas or universe sky are on screen.
//   k_noise_bake  noise_bake.comp:9-26 (fbm of periodic gradient noise, common.glsl:16-77,
//                 plus a ridged octave) into a 128^3 half volume, one thread per texel
//   k_shade       per pixel: the recorded crossings shaded by thinDiskSample (disk.glsl:113-129)
//                 and composited front to back (blackhole.frag:209-216,234); the sky's analytic
//                 star layers (sky.glsl:26-118) for escaped rays, with the footprint from 2x2-quad
//                 differences of escDir (blackhole.frag:297-310); shadow overlay and NaN clear
//                 (:354-359,377-379). The sky cube's weight goes to the alpha channel.
// Block of 32 x 8 pixels in warps of 8 x 4: every 2x2 quad (even-aligned, as the rasteriser's)
// lies inside one warp, so the derivative exchange is two shuffles. The star layers run per
// warp over the union of its pixels' lattice cells. The blackbody table (4 KiB) is staged in
// shared memory; the noise volume (4 MiB) is read through L1/L2.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>

#include "bhr.h"
#include "shade.cuh"
#include "body_math.cuh"
#include "shade_math.cuh"

namespace bhr {

namespace {

using namespace shading;
constexpr int kBX = 32, kBY = 8;

__device__ __forceinline__ float fade(float t) { return t * t * t * (t * (t * 6.0f - 15.0f) + 10.0f); }

// common.glsl:58-77 pgnoise3: gradient noise whose lattice wraps every `period` cells
__device__ float pgnoise3(F3 p, int period, uint32_t salt) {
    const float ix = floorf(p.x), iy = floorf(p.y), iz = floorf(p.z);
    const F3 f{p.x - ix, p.y - iy, p.z - iz};
    const F3 u{fade(f.x), fade(f.y), fade(f.z)};
    const int c[3] = {int(ix), int(iy), int(iz)};
    int c0[3], c1[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        c0[k] = ((c[k] % period) + period) % period;
        c1[k] = ((c[k] + 1) % period + period) % period;
    }
    float n[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int ox = k & 1, oy = (k >> 1) & 1, oz = k >> 2;
        const F3 g = grad3(ox ? c1[0] : c0[0], oy ? c1[1] : c0[1], oz ? c1[2] : c0[2], salt);
        n[k] = dot(g, F3{f.x - float(ox), f.y - float(oy), f.z - float(oz)});
    }
    const float nx00 = mixf(n[0], n[1], u.x), nx10 = mixf(n[2], n[3], u.x);
    const float nx01 = mixf(n[4], n[5], u.x), nx11 = mixf(n[6], n[7], u.x);
    return 1.4f * mixf(mixf(nx00, nx10, u.y), mixf(nx01, nx11, u.y), u.z);
}

__global__ void __launch_bounds__(256) k_noise_bake(uint32_t seed, uint16_t* __restrict__ out) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= kN * kN * kN) return;
    const int x = idx % kN, y = (idx / kN) % kN, z = idx / (kN * kN);
    const F3 uvw{(float(x) + 0.5f) / float(kN), (float(y) + 0.5f) / float(kN), (float(z) + 0.5f) / float(kN)};
    float sum = 0.0f, amp = 0.55f, norm = 0.0f;
    int period = 4;
#pragma unroll 1
    for (int o = 0; o < 6; ++o) {
        sum += amp * pgnoise3(scale(uvw, float(period)), period, seed + uint32_t(o) * 131u);
        norm += amp;
        amp *= 0.55f;
        period *= 2;
    }
    float n = clampf(0.5f + 0.5f * (sum / norm) * 1.6f, 0.0f, 1.0f);
    const float ridge = 1.0f - fabsf(pgnoise3(scale(uvw, 8.0f), 8, seed + 977u));
    n = mixf(n, n * ridge * 1.3f, 0.35f);
    out[idx] = __half_as_ushort(__float2half_rn(n));  // the R16F store
}

// The baked volume's 2x2x2 REPEAT neighbourhood of every texel, as the sampler reads it: word 0
// = (x, x+1) at (y, z), word 1 at (y+1, z), word 2 at (y, z+1), word 3 at (y+1, z+1); the lower
// half of each word is x.
__global__ void __launch_bounds__(256) k_noise_expand(const uint16_t* __restrict__ v, uint4* __restrict__ out) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= kN * kN * kN) return;
    const int x = idx % kN, y = (idx / kN) % kN, z = idx / (kN * kN);
    const int x1 = (x + 1) & (kN - 1), y1 = (y + 1) & (kN - 1), z1 = (z + 1) & (kN - 1);
    auto pair = [&](int yy, int zz) {
        const size_t row = (size_t(zz) * kN + yy) * kN;
        return uint32_t(v[row + x]) | (uint32_t(v[row + x1]) << 16);
    };
    out[idx] = make_uint4(pair(y, z), pair(y1, z), pair(y, z1), pair(y1, z1));
}

// ---------------------------------------------------------------- shading

struct Footprint {
    F3 e1, e2;
    float r11, r12, r22, gi11, gi12, gi22, det_gi, det, mu;
};

// sky.glsl:26-48 makeFootprint (QR of the screen-to-sky Jacobian [a b])
__device__ Footprint make_footprint(F3 d, F3 a, F3 b, float omega0) {
    Footprint f;
    const float min_axis = 1e-3f * sqrtf(omega0);
    const float la_raw = len(a);
    const float la = fmaxf(la_raw, min_axis);
    f.e1 = la_raw > 1e-12f ? divs(a, la_raw) : normalize(cross(d, F3{1e-3f, 1.0f + 1e-3f, 1e-3f}));
    const float b1 = dot(b, f.e1);
    const F3 bp = sub(b, scale(f.e1, b1));
    const float lbp_raw = len(bp);
    const float lbp = fmaxf(lbp_raw, min_axis);
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
    f.mu = fminf(omega0 / area, 1e4f);
    return f;
}

// One star of a layer, as starLayer finds it in lattice cell c (sky.glsl:79-92): the unit
// direction q / |q|, flux F and colour sc. Lane-independent: computed once per warp.
struct StarSlot {
    float qx, qy, qz, F, r, g, b;
    int cx, cy, cz;
};

struct Layer {
    float N, inv_n, prob, flux, s_in2, s_out2, cull_lo, cull_hi;
    uint32_t salt, sy, sz;
};

__device__ __forceinline__ Layer make_layer(float N, float prob, float flux, uint32_t salt) {
    Layer L;
    L.N = N;
    L.inv_n = 1.0f / N;
    L.prob = prob;
    L.flux = flux;
    const float s_in = 1.0f - 0.5f / N, s_out = 1.0f + 0.5f / N;
    L.s_in2 = s_in * s_in;
    L.s_out2 = s_out * s_out;
    // a cell whose cube [c, c + 1) / N misses the shell holds no star: skipped before hashing
    // (conservative, with a relative margin of 1e-4)
    L.cull_lo = L.s_out2 * 1.0001f;
    L.cull_hi = L.s_in2 * 0.9999f;
    L.salt = salt;
    L.sy = salt * 7u + 1u;
    L.sz = salt * 13u + 2u;
    return L;
}

// The star of cell (cx, cy, cz), if it is lit (ux <= prob) and on the shell.
__device__ bool star_of_cell(const Tex& tx, const ShadeArgs& A, const Layer& L, float g_shift, int cx, int cy, int cz,
                             StarSlot& st) {
    const float lx = float(cx) * L.inv_n, ly = float(cy) * L.inv_n, lz = float(cz) * L.inv_n;
    const float hx = lx + L.inv_n, hy = ly + L.inv_n, hz = lz + L.inv_n;
    const float nx = fminf(fmaxf(0.0f, lx), hx), ny = fminf(fmaxf(0.0f, ly), hy), nz = fminf(fmaxf(0.0f, lz), hz);
    const float fx = fmaxf(lx * lx, hx * hx), fy = fmaxf(ly * ly, hy * hy), fz = fmaxf(lz * lz, hz * hz);
    if (nx * nx + ny * ny + nz * nz > L.cull_lo || fx + fy + fz < L.cull_hi) return false;
    const uint3 h = pcg3d(make_uint3(uint32_t(cx) + L.salt, uint32_t(cy) + L.sy, uint32_t(cz) + L.sz));
    const float k16 = 1.0f / 65536.0f;
    const float ux = float(h.x >> 16) * k16;
    if (ux > L.prob) return false;
    const float q0 = (float(cx) + float(h.x & 0xffffu) * k16) * L.inv_n;
    const float q1 = (float(cy) + float(h.y >> 16) * k16) * L.inv_n;
    const float q2 = (float(cz) + float(h.y & 0xffffu) * k16) * L.inv_n;
    const float ql2 = q0 * q0 + q1 * q1 + q2 * q2;
    if (ql2 < L.s_in2 || ql2 > L.s_out2) return false;
    const float iq = 1.0f / sqrtf(ql2);
    const float uy = float(h.z >> 16) * k16, uz = float(h.z & 0xffffu) * k16;
    st.qx = q0 * iq;
    st.qy = q1 * iq;
    st.qz = q2 * iq;
    st.F = L.flux / fmaxf(uy, 2e-4f);  // flux * pow(max(u.y, 2e-4), -1)
    const float T = gexp(mixf(A.ln_3000, A.ln_22000, gpow(uz, 1.7f)));
    const float4 bb = blackbody(tx, T * g_shift);
    st.r = mixf(1.0f, bb.x, 0.7f);
    st.g = mixf(1.0f, bb.y, 0.7f);
    st.b = mixf(1.0f, bb.z, 0.7f);
    st.cx = cx;
    st.cy = cy;
    st.cz = cz;
    return true;
}

// A pixel's per-layer constants: the covariance of its star Gaussians (sky.glsl:66-73).
struct LanePart {
    float isaa, isab, isbb, norm;
    F3 d;
    const Footprint* fp;
};

__device__ __forceinline__ void star_add(const StarSlot& t, const LanePart& P, F3& sum) {
    const F3 delta{t.qx - P.d.x, t.qy - P.d.y, t.qz - P.d.z};
    const float d1 = dot(P.fp->e1, delta), d2 = dot(P.fp->e2, delta);
    const float sp = P.fp->r11 * d1 + P.fp->r12 * d2;
    const float sq = P.fp->r22 * d2;
    const float e = P.isaa * sp * sp + 2.0f * P.isab * sp * sq + P.isbb * sq * sq;
    if (!(e < 30.0f)) return;  // also skips NaN
    const float k = t.F * P.norm * gexp(-0.5f * e);
    sum = add(sum, F3{t.r * k, t.g * k, t.b * k});
}

constexpr int kMaxBox = 1024;  // union boxes of up to this many cells are scanned by the warp

// warp-wide min / max by xor butterflies (every lane gets the result)
__device__ __forceinline__ int warp_min(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ int warp_max(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// sky.glsl:54-103 starLayer for the 32 pixels of a warp (all lanes call it; `active` lanes
// are escaped pixels). A pixel's stars come from the 27 cells around c0 = floor(d N), summed in
// the order z, y, x of the cell. The warp scans the union box of its pixels' cells in that same
// lexicographic order, 32 cells at a time: each lane hashes one cell, the lit stars on the
// shell are compacted into shared memory, then every lane adds those inside its own 27 cells.
// A pixel therefore sums exactly the stars, in exactly the order, of its own loop. Warps whose
// box is larger (directions spread wide near the photon ring) run the per-pixel loop.
__device__ F3 star_layer_warp(const Tex& tx, const ShadeArgs& A, bool active, F3 d, const Footprint& fp,
                              const Layer& L, float sig_star, float omega0, float g_shift, StarSlot* list) {
    const int lane = threadIdx.x & 31;
    float w = 1.0f;
    F3 avg{0.f, 0.f, 0.f};
    LanePart P{0.f, 0.f, 0.f, 0.f, d, &fp};
    int c0x = 0, c0y = 0, c0z = 0;
    bool loop = false;
    if (active) {
        const float footprint_cells = gpow(fp.det, 0.25f) * L.N;
        w = smoothstep(0.8f, 2.5f, footprint_cells);
        const float4 bavg = blackbody(tx, 5600.0f * g_shift);
        const float aw = L.prob * L.N * L.N * 9.517f * L.flux * omega0;
        avg = F3{bavg.x * aw, bavg.y * aw, bavg.z * aw};
        loop = w < 1.0f;
        if (loop) {
            const float s2 = sig_star * sig_star;
            const float px2 = 0.45f;
            const float saa = px2 + s2 * fp.gi11, sab = s2 * fp.gi12, sbb = px2 + s2 * fp.gi22;
            const float det_s = px2 * px2 + px2 * s2 * (fp.gi11 + fp.gi22) + s2 * s2 * fp.det_gi;
            const float inv_det_s = 1.0f / det_s;
            P.isaa = sbb * inv_det_s;
            P.isab = -sab * inv_det_s;
            P.isbb = saa * inv_det_s;
            P.norm = fp.mu / (kTwoPi * sqrtf(det_s));
            c0x = int(floorf(d.x * L.N));
            c0y = int(floorf(d.y * L.N));
            c0z = int(floorf(d.z * L.N));
        }
    }
    F3 sum{0.f, 0.f, 0.f};
    const unsigned any_loop = __ballot_sync(0xffffffffu, loop);
    if (any_loop != 0u) {
        const int bx = warp_min(loop ? c0x - 1 : INT_MAX);
        const int by = warp_min(loop ? c0y - 1 : INT_MAX);
        const int bz = warp_min(loop ? c0z - 1 : INT_MAX);
        const int ex = warp_max(loop ? c0x + 1 : INT_MIN);
        const int ey = warp_max(loop ? c0y + 1 : INT_MIN);
        const int ez = warp_max(loop ? c0z + 1 : INT_MIN);
        const long long nx = (long long)ex - bx + 1, ny = (long long)ey - by + 1, nz = (long long)ez - bz + 1;
        if (nx * ny * nz <= kMaxBox) {
            const int vol = int(nx * ny * nz), sx = int(nx), sxy = int(nx * ny);
            for (int base = 0; base < vol; base += 32) {
                const int cell = base + lane;
                StarSlot st;
                bool star = false;
                if (cell < vol)
                    star = star_of_cell(tx, A, L, g_shift, bx + cell % sx, by + (cell % sxy) / sx, bz + cell / sxy, st);
                const unsigned m = __ballot_sync(0xffffffffu, star);
                if (star) list[__popc(m & ((1u << lane) - 1u))] = st;
                __syncwarp();
                const int n = __popc(m);
                if (loop) {
                    for (int s = 0; s < n; ++s) {
                        const StarSlot t = list[s];
                        if (abs(t.cx - c0x) <= 1 && abs(t.cy - c0y) <= 1 && abs(t.cz - c0z) <= 1) star_add(t, P, sum);
                    }
                }
                __syncwarp();
            }
        } else if (loop) {
#pragma unroll 1
            for (int cell = 0; cell < 27; ++cell) {
                StarSlot t;
                if (star_of_cell(tx, A, L, g_shift, c0x + cell % 3 - 1, c0y + (cell / 3) % 3 - 1, c0z + cell / 9 - 1, t))
                    star_add(t, P, sum);
            }
        }
    }
    if (!isfinite(sum.x) || !isfinite(sum.y) || !isfinite(sum.z)) sum = F3{0.f, 0.f, 0.f};
    sum = F3{fminf(sum.x, 64.0f), fminf(sum.y, 64.0f), fminf(sum.z, 64.0f)};
    return F3{mixf(sum.x, avg.x, w), mixf(sum.y, avg.y, w), mixf(sum.z, avg.z, w)};
}

// blackhole.frag:68-72 primary direction of pixel (i, j), any i, j (quad partners outside the
// image included)
__device__ __forceinline__ F3 primary_dir(const ShadeArgs& A, int i, int j) {
    const float pxx = float(i) + 0.5f + A.jitter[0], pxy = float(j) + 0.5f + A.jitter[1];
    const float ndcx = pxx / float(A.width) * 2.0f - 1.0f, ndcy = pxy / float(A.height) * 2.0f - 1.0f;
    const float aspect = float(A.width) / float(A.height);
    const F3 dc = normalize(F3{ndcx * A.tan_half * aspect, ndcy * A.tan_half, -1.0f});
    const float* B = A.basis;
    return normalize(F3{B[0] * dc.x + B[3] * dc.y + B[6] * dc.z, B[1] * dc.x + B[4] * dc.y + B[7] * dc.z,
                        B[2] * dc.x + B[5] * dc.y + B[8] * dc.z});
}

// Fine derivative over the quad: v(odd) - v(even) along the axis whose partner is lane ^ mask.
__device__ __forceinline__ F3 quad_diff(F3 v, int lane, int mask) {
    const F3 o{__shfl_xor_sync(0xffffffffu, v.x, mask), __shfl_xor_sync(0xffffffffu, v.y, mask),
               __shfl_xor_sync(0xffffffffu, v.z, mask)};
    return (lane & mask) ? sub(v, o) : sub(o, v);
}

// A block is 4 x 2 warps, a warp 8 x 4 pixels (lane = 8 y + x): the 2x2 quads of the
// rasteriser (even-aligned) sit inside a warp, with partners at lane ^ 1 (x) and lane ^ 8 (y).
// blackhole.frag:78,107 rdNear = normalize(initialVelocity(uCamPos, dir)) (dir when lensing is off)
__device__ __forceinline__ F3 rd_near_of(F3 cam, float rcam, F3 d, bool lensing) {
    if (!lensing) return d;
    const F3 rhat = divs(cam, rcam);
    const float nr = dot(d, rhat);
    const F3 nperp = sub(d, scale(rhat, nr));
    const float f = sqrtf(fmaxf(1.0f - 2.0f / rcam, 0.0f));
    const F3 w = add(scale(rhat, nr * f), nperp);
    const F3 v = scale(w, 1.0f / sqrtf(dot(w, w)));
    return normalize(v);
}

// The shading of one block. With kBodies, the body records and bodies of B add what lies
// behind the disk before the sky (blackhole.frag:255-296).
template <bool kBodies>
__device__ __forceinline__ void shade_block(const ShadeArgs& A, const BodyShadeArgs* B) {
    __shared__ float4 s_lut[kLut];
    __shared__ StarSlot s_star[kBX * kBY / 32][32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int k = tid; k < kLut; k += kBX * kBY) s_lut[k] = A.lut[k];
    const Tex tx{A.noise8, s_lut, A.ln_1000, A.ln_40000};
    const int i = blockIdx.x * kBX + (warp & 3) * 8 + (lane & 7);
    const int j = blockIdx.y * kBY + (warp >> 2) * 4 + (lane >> 3);
    const bool in = i < A.width && j < A.height;
    const bhr_shade_params& P = A.p;
    const F3 cam{A.cam[0], A.cam[1], A.cam[2]};
    const float rcam = len(cam);
    const DiskConsts C = disk_consts(P, rcam);
    const F3 dir = primary_dir(A, i, j);
    const float pixel_angle = 2.0f * A.tan_half / float(A.height);
    __syncthreads();  // the table is staged

    F3 col{0.f, 0.f, 0.f};
    float trans = 1.0f;
    bool esc = false;
    F3 esc_dir = dir;
    if (in) {
        const int64_t k_pix = int64_t(j) * A.width + i;
        const float4* rec = reinterpret_cast<const float4*>(A.hits + k_pix);
        const float4 w0 = __ldg(rec), w1 = __ldg(rec + 1);
        const uint32_t head = __float_as_uint(w0.x);
        const int status = int(head & 0xffu), ncross = int((head >> 8) & 0xffu);
        bool opaque = false;
        if (A.volumetric) {  // the volumetric march gathered the disk's light along the ray
            const float4 m = A.out[k_pix];
            col = F3{m.x, m.y, m.z};
            trans = m.w;
            opaque = status == BHR_STATUS_OPAQUE;
        } else if (A.disk_thin && ncross > 0) {
            const float4 w2 = __ldg(rec + 2), w3 = __ldg(rec + 3);
            const float cr[3] = {w2.z, w2.w, w3.x}, cp[3] = {w3.y, w3.z, w3.w};
            const float b_axis = w2.x;
            for (int k = 0; k < ncross && k < 3; ++k) {
                const float4 dk = thin_disk_sample(tx, P, C, A.disk_inner, A.disk_outer, cr[k], cp[k], b_axis);
                col = add(col, F3{trans * dk.x * dk.w, trans * dk.y * dk.w, trans * dk.z * dk.w});
                trans *= 1.0f - dk.w;
                if (trans < 0.004f) {
                    opaque = true;
                    break;
                }
            }
        }
        if (status == BHR_STATUS_ESCAPED) esc_dir = F3{w0.z, w0.w, w1.x};
        int st = opaque ? int(BHR_STATUS_OPAQUE) : status;
        if constexpr (kBodies) {
            const bhr_body_hit bh = B->bh[k_pix];
            const F3 rdn = rd_near_of(cam, rcam, dir, A.lensing != 0);
            shade_bodies_after_march(tx, B->bodies, B->nbodies, bh, A.far_mode != 0, rcam, dir, rdn, pixel_angle, P.time, st,
                                     esc_dir, col, trans);
        }
        esc = st == BHR_STATUS_ESCAPED;
    }
    // blackhole.frag:297-306: derivatives of escDir; the unlensed footprint where a quad mixes
    // escaped and other pixels (a partner outside the image counts as not escaped)
    // (both shuffles run in every lane: a short-circuit || would leave lanes out of the second
    // full-mask shuffle, which is undefined)
    const int e = esc ? 1 : 0;
    const int ex = __shfl_xor_sync(0xffffffffu, e, 1);
    const int ey = __shfl_xor_sync(0xffffffffu, e, 8);
    const bool mixed = ex != e || ey != e;
    const F3 ddx_l = quad_diff(esc_dir, lane, 1), ddy_l = quad_diff(esc_dir, lane, 8);
    const F3 ddx_0 = quad_diff(dir, lane, 1), ddy_0 = quad_diff(dir, lane, 8);
    const F3 ddx = mixed ? ddx_0 : ddx_l, ddy = mixed ? ddy_0 : ddy_l;

    const float omega0 = pixel_angle * pixel_angle;
    const float g = mixf(1.0f, 1.0f / sqrtf(fmaxf(1.0f - 2.0f / rcam, 1e-4f)), P.doppler_strength);
    const float g4 = g * g * g * g;
    Footprint fp{};
    if (esc) fp = make_footprint(esc_dir, ddx, ddy, omega0);
    const float sb = P.star_brightness * g4;
    StarSlot* list = s_star[warp];
    const F3 s1 = star_layer_warp(tx, A, esc, esc_dir, fp, make_layer(200.0f, 0.40f * P.star_density, 0.0045f * sb, 11u),
                                  0.0004f, omega0, g, list);
    const F3 s2 = star_layer_warp(tx, A, esc, esc_dir, fp, make_layer(48.0f, 0.25f * P.star_density, 0.06f * sb, 23u),
                                  0.0011f, omega0, g, list);
    if (!in) return;
    float alpha = 0.0f;
    if (esc) {
        const F3 sky = add(s1, s2);
        col = add(col, F3{trans * sky.x, trans * sky.y, trans * sky.z});
        alpha = trans * (P.sky_brightness * g4);
    }
    if (P.shadow_overlay && !A.far_mode) {
        const float ang = acosf(clampf(dot(dir, F3{-cam.x / rcam, -cam.y / rcam, -cam.z / rcam}), -1.0f, 1.0f));
        // shadowAngularRadius (geodesic.glsl:56-60)
        const float s = fminf(1.0f, 5.19615242270663f / rcam * sqrtf(fmaxf(1.0f - 2.0f / rcam, 0.0f)));
        const float a = asinf(s);
        const float edge = rcam >= 3.0f ? a : kPi - a;
        const float dd = fabsf(ang - edge) / pixel_angle;
        const float k = 0.85f * (1.0f - smoothstep(0.8f, 1.8f, dd));
        col = F3{mixf(col.x, 0.1f, k), mixf(col.y, 1.0f, k), mixf(col.z, 0.2f, k)};
        alpha *= 1.0f - k;
    }
    if (!isfinite(col.x) || !isfinite(col.y) || !isfinite(col.z)) {
        col = F3{0.f, 0.f, 0.f};
        alpha = 0.0f;
    }
    A.out[int64_t(j) * A.width + i] = make_float4(fmaxf(col.x, 0.0f), fmaxf(col.y, 0.0f), fmaxf(col.z, 0.0f), alpha);
}

__global__ void __launch_bounds__(kBX * kBY) k_shade(const __grid_constant__ ShadeArgs A) { shade_block<false>(A, nullptr); }

__global__ void __launch_bounds__(kBX * kBY) k_shade_bodies(const __grid_constant__ ShadeArgs A,
                                                            const __grid_constant__ BodyShadeArgs B) {
    shade_block<true>(A, &B);
}

// ---------------------------------------------------------------- blackbody table (host, double)

double lobe(double l, double mu, double s1, double s2) {
    const double t = (l - mu) / (l < mu ? s1 : s2);
    return std::exp(-0.5 * t * t);
}

// CIE 1931 2-degree colour matching functions as the multi-lobe Gaussian fits of Wyman, Sloan
// and Shirley (2013), times Planck's law, summed over 380..780 nm in 1 nm steps
void tristimulus(double T, double& X, double& Y, double& Z) {
    const double h = 6.62607015e-34, c = 2.99792458e8, kb = 1.380649e-23;
    X = Y = Z = 0.0;
    for (int nm = 380; nm <= 780; ++nm) {
        const double l = double(nm);
        const double x = 1.056 * lobe(l, 599.8, 37.9, 31.0) + 0.362 * lobe(l, 442.0, 16.0, 26.7) -
                         0.065 * lobe(l, 501.1, 20.4, 26.2);
        const double y = 0.821 * lobe(l, 568.8, 46.9, 40.5) + 0.286 * lobe(l, 530.9, 16.3, 31.1);
        const double z = 1.217 * lobe(l, 437.0, 11.8, 36.0) + 0.681 * lobe(l, 459.0, 26.0, 13.8);
        const double lm = l * 1e-9;
        const double b = (2.0 * h * c * c) / (lm * lm * lm * lm * lm) / (std::exp((h * c) / (lm * kb * T)) - 1.0);
        X += b * x;
        Y += b * y;
        Z += b * z;
    }
}

}  // namespace

void blackbody_lut_host(float* out) {
    double Xr, Yr, Zr;
    tristimulus(6500.0, Xr, Yr, Zr);
    const double lo = std::log(1000.0), hi = std::log(40000.0);
    for (int i = 0; i < kLut; ++i) {
        const double T = std::exp(lo + (hi - lo) * (double(i) / (kLut - 1)));
        double X, Y, Z;
        tristimulus(T, X, Y, Z);
        // XYZ -> linear sRGB (D65), negative lobes clipped, normalised to luminance 1
        const double r = std::max(3.2406 * X - 1.5372 * Y - 0.4986 * Z, 0.0);
        const double g = std::max(-0.9689 * X + 1.8758 * Y + 0.0415 * Z, 0.0);
        const double b = std::max(0.0557 * X - 0.2040 * Y + 1.0570 * Z, 0.0);
        const double lum = 0.2126 * r + 0.7152 * g + 0.0722 * b;
        const double inv = lum > 0.0 ? 1.0 / lum : 0.0;
        out[4 * i + 0] = float(r * inv);
        out[4 * i + 1] = float(g * inv);
        out[4 * i + 2] = float(b * inv);
        out[4 * i + 3] = float(Y / Yr);
    }
}

cudaError_t launch_noise_bake(uint32_t seed, uint16_t* out, cudaStream_t st) {
    const int n = kN * kN * kN;
    k_noise_bake<<<(n + 255) / 256, 256, 0, st>>>(seed, out);
    return cudaGetLastError();
}

cudaError_t launch_noise_expand(const uint16_t* vol, uint4* out, cudaStream_t st) {
    const int n = kN * kN * kN;
    k_noise_expand<<<(n + 255) / 256, 256, 0, st>>>(vol, out);
    return cudaGetLastError();
}

cudaError_t launch_shade(const ShadeArgs& a, cudaStream_t st) {
    const dim3 grid((a.width + kBX - 1) / kBX, (a.height + kBY - 1) / kBY);
    k_shade<<<grid, kBX * kBY, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_shade_bodies(const ShadeArgs& a, const BodyShadeArgs& b, cudaStream_t st) {
    const dim3 grid((a.width + kBX - 1) / kBX, (a.height + kBY - 1) / kBY);
    k_shade_bodies<<<grid, kBX * kBY, 0, st>>>(a, b);
    return cudaGetLastError();
}

}  // namespace bhr
