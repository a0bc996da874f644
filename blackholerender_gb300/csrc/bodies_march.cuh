// The body-aware march (blackhole.frag's BHS_BODIES 1 variant): the plain march, or the
// volumetric disk's march (vol.cu), plus spheres it can hit.
//   setup   (:101-121)  near-field bodies: a straight camera-relative ray along the geodesic's
//                       initial direction is exact while the geodesic has not bent away, for
//                       t < sqrt(0.02 R / |x''|); bodies wholly inside that stretch are settled
//                       there (near_mask) and the nearest hit among them is remembered
//   loop head (:146-150) the ray has travelled to the near-field hit: status BODY
//   step size (:184-190) land on the near-field hit; short steps near the other bodies
//   after the step (:236-250) the step's straight chord against the other bodies
// Shading the hit is the consumer's (bhr_shade_bodies); the march records where it happened.
// With the volumetric disk (kVol) the steps in the slab are clamped to 6 diskStep and sampled
// (:173-175,217-233) before the ray can turn opaque (:234) and before the step's chord is tested
// against the bodies, so a body behind the disk keeps the light gathered in front of it.
// One ray per thread, warps of 8 x 4 pixels; the bodies are kernel parameters (constant bank,
// read warp-uniformly). FP32, like the shader.
//
// Clearance: each ray keeps a lower bound on its distance to the surface of every body the two
// loops test. A step's chord shortens it by at most the chord's length (triangle inequality), so
// the loops run only on steps where a body could shorten the step (within 2 ds) or be reached by
// the chord; the other steps skip them. The bound carries a relative margin of 1e-5 against
// FP32 rounding, so a skipped loop is one in which every body would have failed its own
// squared-distance test: the records are the same bits as with the loops run on every step.
//
// The kernel is a template included by two translation units: bodies.cu instantiates the thin
// or no-disk march, bodies_vol.cu the volumetric one, built with the volumetric march's fast
// divide and square root (vol.cu's flags) for the disk's samples.
#pragma once
#include <cuda_runtime.h>

#include <cmath>

#include "bhr.h"
#include "bodies.cuh"
#include "march.cuh"

namespace bhr {

namespace {

__device__ __forceinline__ V3<float> xyz(const float* q) { return V3<float>{q[0], q[1], q[2]}; }
__device__ __forceinline__ float len3(const V3<float>& a) { return sqrtf(dot3(a, a)); }

// shaders/bodies.glsl:34-44 raySphere: nearest hit in (tMin, tMax), -1 if none
__device__ __forceinline__ float ray_sphere(V3<float> ro, V3<float> rd, V3<float> c, float r, float t_min, float t_max) {
    const V3<float> oc{ro.x - c.x, ro.y - c.y, ro.z - c.z};
    const float b = dot3(oc, rd);
    const float cc = dot3(oc, oc) - r * r;
    const float disc = b * b - cc;
    if (disc < 0.f) return -1.f;
    const float s = sqrtf(disc);
    float t = -b - s;
    if (t <= t_min) t = -b + s;
    return (t > t_min && t < t_max) ? t : -1.f;
}

// The volumetric variant asks for three blocks per SM: 80 registers (a 4-byte spill) in place of
// 100 and two blocks, 13% faster on the 16-pose body gallery
template <bool kVol>
__global__ void __launch_bounds__(256, kVol ? 3 : 1) k_march_bodies(const __grid_constant__ BodyArgs A) {
    __shared__ float4 s_lut[kVol ? BHR_BLACKBODY_LUT : 1];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if constexpr (kVol) {
        for (int k = tid; k < BHR_BLACKBODY_LUT; k += 256) s_lut[k] = A.look.lut[k];
        __syncthreads();
    }
    const DevView& w = A.view;
    const int i = blockIdx.x * 32 + (warp & 3) * 8 + (lane & 7);
    const int j = blockIdx.y * 8 + (warp >> 2) * 4 + (lane >> 3);
    if (i >= w.width || j >= w.height) return;
    const Rule& R = A.rule;
    const RayInit<float> ri = setup_ray<float>(w, R, i, j);
    const int64_t k = int64_t(j) * w.width + i;
    bhr_hit* rec = w.out + k;
    const bool lensing = R.lensing != 0;
    const int nb = A.nbodies;

    // ---- near-field bodies (blackhole.frag:107-121)
    V3<float> v = ri.v;
    V3<float> rd_near = v;
    if (lensing) {
        const float vl = len3(v);
        rd_near = {v.x / vl, v.y / vl, v.z / vl};
    }
    const float rcam = w.rcam;
    const float a_cam = lensing ? 3.0f * ri.h2 / fmaxf(rcam * rcam * rcam * rcam, 1e-30f) : 0.0f;
    uint32_t near_mask = 0;
    int near_idx = -1;
    float near_t = 1e30f;
    for (int b = 0; b < nb; ++b) {
        const bhr_body& B = A.bodies[b];
        const V3<float> rel = xyz(B.rel_pos);
        const float Rb = B.pos_radius[3];
        const float t_straight = lensing ? sqrtf(0.02f * Rb / fmaxf(a_cam, 1e-30f)) : 1e30f;
        if (len3(rel) + fmaxf(Rb, B.ring[1]) < t_straight) near_mask |= 1u << b;
        const float t = ray_sphere(V3<float>{0.f, 0.f, 0.f}, rd_near, rel, Rb, 0.f, fminf(t_straight, near_t));
        if (t > 0.f) {
            near_t = t;
            near_idx = b;
        }
    }
    const float near_tol = fmaxf(2e-6f * rcam, 1e-9f);

    V3<float> x{w.cam[0], w.cam[1], w.cam[2]};
    const float h2 = ri.h2;
    float min_r = INFINITY, travelled = 0.f;
    uint32_t steps = 0, nplane = 0, ncross = 0, status = 0;
    float cr[3] = {0.f, 0.f, 0.f}, cp[3] = {0.f, 0.f, 0.f};
    int hit = -1;
    V3<float> hit_ro{0.f, 0.f, 0.f}, hit_rd{0.f, 0.f, 0.f};
    float hit_t = 0.f;
    const bool thin = !kVol && R.disk_mode == BHR_DISK_THIN;
    const shading::Tex tx{A.look.noise8, s_lut, A.look.ln_1000, A.look.ln_40000};
    const shading::DiskConsts C = shading::disk_consts(A.look.p, rcam);
    shading::F3 col{0.f, 0.f, 0.f};
    float trans = 1.0f;
    float clear = -1.f;  // lower bound of |x - c| - R over the bodies the loops test; < 0: unknown
    if (R.far_mode) {
        status = BHR_STATUS_ESCAPED;
    } else {
        for (;;) {
            if (steps >= uint32_t(w.max_steps)) {
                status = BHR_STATUS_BUDGET;
                break;
            }
            const float r2 = dot3(x, x), v2 = dot3(v, v);
            const float rinv = rsqrtf(r2), vi = rsqrtf(v2);
            const float r = r2 * rinv;
            min_r = fminf(min_r, r);
            if (r < R.capture_r) {
                status = BHR_STATUS_CAPTURED;
                break;
            }
            if (near_idx >= 0 && travelled + near_tol >= near_t) {  // reached the near-field body
                hit = near_idx;
                status = BHR_STATUS_BODY;
                break;
            }
            if (dot3(x, v) > 0.f) {
                bool esc;
                if (R.term_mode == BHR_TERM_CONFIG) {
                    esc = r > R.escape_r;
                } else {
                    esc = false;
                    if (r > R.r_esc_min) {
                        const float bh = sqrtf(h2) * vi;
                        const float ri2 = rinv * rinv;
                        esc = !lensing || 0.75f * bh * bh * bh * (ri2 * ri2) < R.esc_tol;
                    }
                }
                if (esc) {
                    status = BHR_STATUS_ESCAPED;
                    break;
                }
            }
            float ds = fmaxf(ri.ssf * r, R.ds_floor);
            bool near_disk = false;
            if (kVol || thin) {
                const float rc2 = x.x * x.x + x.z * x.z;
                if (rc2 > R.rcyl_lo2 && rc2 < R.rcyl_hi2) {
                    const float outside = fabsf(x.y) - R.slab * (rc2 * rsqrtf(rc2));
                    if (outside > 0.f) {
                        ds = fminf(ds, fmaxf(w.disk_step, __fdividef(outside, fabsf(v.y) * vi + R.slab)));
                    } else if (kVol) {  // inside the slab: sub-sampled after the step
                        near_disk = true;
                        ds = fminf(ds, 6.0f * w.disk_step);
                    }
                }
            }
            // land on the near-field hit; short steps near the other bodies (:184-190)
            if (near_idx >= 0) ds = fminf(ds, fmaxf(near_t - travelled, near_tol));
            if (clear < 2.00002f * ds) {  // a body may be within 2 ds: the loop, and a fresh bound
                clear = INFINITY;
                for (int b = 0; b < nb; ++b) {
                    if (near_mask & (1u << b)) continue;
                    const float* pr = A.bodies[b].pos_radius;
                    const V3<float> d{x.x - pr[0], x.y - pr[1], x.z - pr[2]};
                    const float dd = dot3(d, d);
                    const float dist = sqrtf(dd);
                    clear = fminf(clear, fmaf(dist, 0.99999f, -pr[3]));
                    // a body farther than 2 ds + R cannot shorten the step
                    const float reach = 2.0f * ds + pr[3];
                    if (dd >= reach * reach) continue;
                    ds = fminf(ds, fmaxf(0.5f * (dist - pr[3]), 0.25f * pr[3]));
                }
            }
            const float dt = ds * vi;
            const V3<float> x0 = x, v0 = v;
            if (lensing) {
                rk4_update(x, v, h2, dt, rinv);
            } else {
                x = {x.x + v.x * dt, x.y + v.y * dt, x.z + v.z * dt};
            }
            steps += 1;
            const V3<float> dx{x.x - x0.x, x.y - x0.y, x.z - x0.z};
            const float seg = len3(dx);
            travelled += seg;
            if ((x.y > 0.f) != (x0.y > 0.f)) {
                if (nplane < 255u) ++nplane;
                if (thin) {
                    const float f = x0.y / (x0.y - x.y);
                    const float g = 1.0f - f;
                    const float hx = x0.x * g + x.x * f, hz = x0.z * g + x.z * f;
                    const float rh = sqrtf(hx * hx + hz * hz);
                    if (rh >= R.disk_inner && rh <= R.disk_outer && ncross < 3u) {
                        cr[ncross] = rh;
                        cp[ncross] = atan2f(hz, hx);
                        ++ncross;
                    }
                }
            }
            if (kVol && near_disk) {
                vol_segment(tx, A.look, C, R, w.disk_step, ri.b_axis, x0, v0, x, v, dt, seg, col, trans);
                if (trans < 0.004f) {  // blackhole.frag:234, before the chord test
                    status = BHR_STATUS_OPAQUE;
                    break;
                }
            }
            // the step's chord against the bodies not settled by the near-field test (:236-250);
            // a chord shorter than the clearance at its start reaches no body
            if (nb > 0 && seg > 0.f && 1.00001f * seg >= clear) {
                const V3<float> sd{dx.x / seg, dx.y / seg, dx.z / seg};
                float best = seg;
                for (int b = 0; b < nb; ++b) {
                    if (near_mask & (1u << b)) continue;
                    const float* pr = A.bodies[b].pos_radius;
                    // a sphere farther from the chord's start than its length plus R is out of reach
                    const V3<float> d{x0.x - pr[0], x0.y - pr[1], x0.z - pr[2]};
                    const float reach = seg + pr[3];
                    if (dot3(d, d) > reach * reach) continue;
                    const float t = ray_sphere(x0, sd, xyz(pr), pr[3], 0.f, best);
                    if (t > 0.f) {
                        best = t;
                        hit = b;
                        hit_ro = x0;
                        hit_rd = sd;
                        hit_t = t;
                    }
                }
                if (hit >= 0) {
                    status = BHR_STATUS_BODY;
                    break;
                }
            }
            clear = fmaf(clear, 0.999999f, -1.0001f * seg);  // over-subtracts more than it rounds
        }
    }
    const bool nonfinite = !isfinite(dot3(x, x) + dot3(v, v));
    float3 d = make_float3(0.f, 0.f, 0.f);
    if (status == BHR_STATUS_ESCAPED) {
        if (lensing) {
            const V3<float> o = far_field_dir(x, v, h2);
            d = make_float3(o.x, o.y, o.z);
        } else {
            const float vin = rsqrtf(dot3(v, v));
            d = make_float3(v.x * vin, v.y * vin, v.z * vin);
        }
    }
    const uint32_t w0 = status | (ncross << 8) | ((nonfinite ? uint32_t(BHR_FLAG_NONFINITE) : 0u) << 16) | (nplane << 24);
    float4* p = reinterpret_cast<float4*>(rec);
    p[0] = make_float4(__uint_as_float(w0), __uint_as_float(steps), d.x, d.y);
    p[1] = make_float4(d.z, isfinite(min_r) ? min_r : 0.f, 0.f, 0.f);
    p[2] = make_float4(ri.b_axis, ri.b, cr[0], cr[1]);
    p[3] = make_float4(cr[2], cp[0], cp[1], cp[2]);
    float4* q = reinterpret_cast<float4*>(A.body_out + k);
    q[0] = make_float4(__int_as_float(status == BHR_STATUS_BODY ? hit : -1), hit_t, hit_ro.x, hit_ro.y);
    q[1] = make_float4(hit_ro.z, hit_rd.x, hit_rd.y, hit_rd.z);
    q[2] = make_float4(x.x, x.y, x.z, __uint_as_float(near_mask));
    q[3] = make_float4(__int_as_float(near_idx), near_t, travelled, 0.f);
    if constexpr (kVol) A.rgbt[k] = make_float4(col.x, col.y, col.z, trans);
}

}  // namespace

}  // namespace bhr
