// Launch arguments of the shading consumer (shade.cu), filled by the C ABI (api.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "bhr.h"

namespace bhr {

struct ShadeArgs {
    float cam[3];      // uCamPos
    float basis[9];    // uCamBasis, column-major
    float tan_half;    // uTanHalfFov
    float jitter[2];
    int32_t width, height;
    float disk_inner, disk_outer;
    int32_t disk_thin;  // uDiskMode == DISK_THIN
    int32_t volumetric; // uDiskMode == DISK_VOLUMETRIC: `out` holds the march's (rgb, transmittance)
    int32_t far_mode;
    int32_t lensing;    // uLensing and not far mode (the geodesic's initial direction for bodies)
    bhr_shade_params p;
    float ln_1000, ln_40000, ln_3000, ln_22000;  // logf of the constants, from the host's libm
    const bhr_hit* hits;
    float4* out;
    const uint4* noise8;    // BHR_NOISE_SIZE^3 texel neighbourhoods (launch_noise_expand)
    const float4* lut;      // BHR_BLACKBODY_LUT entries
};

// The bodies of a view shaded with them (bhr_shade_bodies).
struct BodyShadeArgs {
    const bhr_body_hit* bh;  // per pixel
    int32_t nbodies;
    int32_t pad;
    bhr_body bodies[BHR_MAX_BODIES];
};

cudaError_t launch_noise_bake(uint32_t seed, uint16_t* out, cudaStream_t st);
// Per texel of the baked volume, its 2x2x2 neighbourhood with REPEAT as eight halves (16 B), so
// that a trilinear sample is one load.
cudaError_t launch_noise_expand(const uint16_t* vol, uint4* out, cudaStream_t st);
cudaError_t launch_shade_bodies(const ShadeArgs& a, const BodyShadeArgs& b, cudaStream_t st);
cudaError_t launch_shade(const ShadeArgs& a, cudaStream_t st);
void blackbody_lut_host(float* out);  // BHR_BLACKBODY_LUT x 4 floats, in double like the CPU bake

}  // namespace bhr
