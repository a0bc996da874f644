// The volumetric disk march (the reference's default High-preset disk): blackhole.frag's loop
// with uDiskMode == DISK_VOLUMETRIC. Inside the disk slab the step is clamped to 6 diskStep
// (:173-175), and every step in the slab samples the cubic Hermite interpolant of its RK4
// segment at n = ceil(seg / diskStep) points (:217-233). Each sample in the disk's volume adds
// emission and absorption (volumetricDiskStep, disk.glsl:88-110) front to back; the ray turns
// opaque once the transmittance falls below 0.004 (:234). The colour depends on the path, so the
// march carries it: rgbt[pixel] = (gathered rgb, transmittance), beside the hit record.
//
// One ray per thread, warps of 8 x 4 pixels (neighbouring rays cross the slab together), the
// blackbody table in shared memory, the noise volume read through L1/L2. FP32, like the shader.
#include <cuda_runtime.h>

#include <cmath>

#include "bhr.h"
#include "march.cuh"
#include "shade_math.cuh"
#include "vol.cuh"

namespace bhr {

namespace {

using shading::F3;

__global__ void __launch_bounds__(256) k_march_vol(const __grid_constant__ VolArgs A) {
    __shared__ float4 s_lut[BHR_BLACKBODY_LUT];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int k = tid; k < BHR_BLACKBODY_LUT; k += 256) s_lut[k] = A.look.lut[k];
    __syncthreads();
    const DevView& w = A.view;
    const int i = blockIdx.x * 32 + (warp & 3) * 8 + (lane & 7);
    const int j = blockIdx.y * 8 + (warp >> 2) * 4 + (lane >> 3);
    if (i >= w.width || j >= w.height) return;
    const Rule& R = A.rule;
    const shading::Tex tx{A.look.noise8, s_lut, A.look.ln_1000, A.look.ln_40000};
    const RayInit<float> ri = setup_ray<float>(w, R, i, j);
    const int64_t k = int64_t(j) * w.width + i;
    bhr_hit* rec = w.out + k;

    V3<float> x{w.cam[0], w.cam[1], w.cam[2]}, v = ri.v;
    const float h2 = ri.h2;
    float min_r = INFINITY;
    uint32_t steps = 0, nplane = 0, status = 0;
    F3 col{0.f, 0.f, 0.f};
    float trans = 1.0f;
    const bool lensing = R.lensing != 0;
    const float b_axis = ri.b_axis;
    const shading::DiskConsts C = shading::disk_consts(A.look.p, w.rcam);
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
            // step size with the slab clamp; inside the slab the volumetric clamp (blackhole.frag:169-181)
            float ds = fmaxf(ri.ssf * r, R.ds_floor);
            bool near_disk = false;
            const float rc2 = x.x * x.x + x.z * x.z;
            if (rc2 > R.rcyl_lo2 && rc2 < R.rcyl_hi2) {
                const float outside = fabsf(x.y) - R.slab * (rc2 * rsqrtf(rc2));
                if (outside > 0.f) {
                    ds = fminf(ds, fmaxf(w.disk_step, __fdividef(outside, fabsf(v.y) * vi + R.slab)));
                } else {
                    near_disk = true;
                    ds = fminf(ds, 6.0f * w.disk_step);
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
            if ((x.y > 0.f) != (x0.y > 0.f) && nplane < 255u) ++nplane;
            if (near_disk) {
                const V3<float> dx{x.x - x0.x, x.y - x0.y, x.z - x0.z};
                vol_segment(tx, A.look, C, R, w.disk_step, b_axis, x0, v0, x, v, dt, sqrtf(dot3(dx, dx)), col, trans);
                if (trans < 0.004f) {  // blackhole.frag:234
                    status = BHR_STATUS_OPAQUE;
                    break;
                }
            }
        }
    }
    const bool nonfinite = !isfinite(dot3(x, x) + dot3(v, v));
    float3 d = make_float3(0.f, 0.f, 0.f);
    if (status == BHR_STATUS_ESCAPED) {
        if (lensing) {
            const V3<float> o = far_field_dir(x, v, h2);
            d = make_float3(o.x, o.y, o.z);
        } else {
            const float vi = rsqrtf(dot3(v, v));
            d = make_float3(v.x * vi, v.y * vi, v.z * vi);
        }
    }
    const uint32_t w0 = status | ((nonfinite ? uint32_t(BHR_FLAG_NONFINITE) : 0u) << 16) | (nplane << 24);
    float4* p = reinterpret_cast<float4*>(rec);
    p[0] = make_float4(__uint_as_float(w0), __uint_as_float(steps), d.x, d.y);
    p[1] = make_float4(d.z, isfinite(min_r) ? min_r : 0.f, 0.f, 0.f);
    p[2] = make_float4(b_axis, ri.b, 0.f, 0.f);
    p[3] = make_float4(0.f, 0.f, 0.f, 0.f);
    A.rgbt[k] = make_float4(col.x, col.y, col.z, trans);
}

}  // namespace

cudaError_t launch_march_vol(const VolArgs& a, cudaStream_t st) {
    const dim3 grid((a.view.width + 31) / 32, (a.view.height + 7) / 8);
    k_march_vol<<<grid, 256, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace bhr
