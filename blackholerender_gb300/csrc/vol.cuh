// Launch arguments of the volumetric disk march (vol.cu), filled by the C ABI (api.cu), and the
// disk's sub-sampling of one RK4 segment, shared by that march and the body-aware one (bodies.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "bhr.h"
#include "march.cuh"
#include "shade_math.cuh"

namespace bhr {

// The volumetric disk's look and the textures it samples.
struct DiskLook {
    bhr_shade_params p;      // the disk's look (density, opacity, temperature, noise, Doppler)
    float ln_1000, ln_40000; // logf of the blackbody table's range, from the host's libm
    float thick;             // uDiskThickness (H / r)
    const uint4* noise8;     // BHR_NOISE_SIZE^3 texel neighbourhoods (launch_noise_expand)
    const float4* lut;       // BHR_BLACKBODY_LUT entries
};

struct VolArgs {
    DevView view;            // geometry of the view; view.out = its hit records
    Rule rule;               // termination rule and slab geometry
    DiskLook look;
    float4* rgbt;            // per pixel: gathered rgb, transmittance
};

cudaError_t launch_march_vol(const VolArgs& a, cudaStream_t st);

constexpr int kMaxSubSamples = 64;  // inside the slab ds <= 6 diskStep: a finite segment needs <= 7

// blackhole.frag:217-233: the samples of one RK4 segment inside the slab, n = ceil(seg /
// diskStep) points along the cubic Hermite interpolant of (x0, dt v0) -> (x, dt v); each point
// in the disk's volume adds emission and absorption (volumetricDiskStep, disk.glsl:88-110) front
// to back, and the samples stop once the transmittance falls below 0.004.
__device__ __forceinline__ void vol_segment(const shading::Tex& tx, const DiskLook& L, const shading::DiskConsts& C,
                                            const Rule& R, float disk_step, float b_axis, const V3<float>& x0,
                                            const V3<float>& v0, const V3<float>& x, const V3<float>& v, float dt,
                                            float seg, shading::F3& col, float& trans) {
    const float nf = ceilf(seg / disk_step);
    const int n = isfinite(nf) ? min(max(1, int(fminf(nf, float(kMaxSubSamples)))), kMaxSubSamples) : 1;
    const float sub = seg / float(n);
    const V3<float> m0{dt * v0.x, dt * v0.y, dt * v0.z}, m1{dt * v.x, dt * v.y, dt * v.z};
    for (int s = 0; s < n; ++s) {
        const float t = (float(s) + 0.5f) / float(n);
        const float t2 = t * t, t3 = t2 * t;
        const float h00 = 2.0f * t3 - 3.0f * t2 + 1.0f, h10 = t3 - 2.0f * t2 + t;
        const float h01 = -2.0f * t3 + 3.0f * t2, h11 = t3 - t2;
        const shading::F3 p{h00 * x0.x + h10 * m0.x + h01 * x.x + h11 * m1.x,
                            h00 * x0.y + h10 * m0.y + h01 * x.y + h11 * m1.y,
                            h00 * x0.z + h10 * m0.z + h01 * x.z + h11 * m1.z};
        const float rm = sqrtf(p.x * p.x + p.z * p.z);
        if (rm > R.disk_inner - 0.5f && rm < R.disk_outer && fabsf(p.y) < R.slab * rm)
            shading::vol_disk_step(tx, L.p, C, R.disk_inner, R.disk_outer, L.thick, p, rm, sub, b_axis, col, trans);
        if (trans < 0.004f) break;
    }
}

}  // namespace bhr
