// Launch arguments of the volumetric disk march (vol.cu), filled by the C ABI (api.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "bhr.h"
#include "march.cuh"

namespace bhr {

struct VolArgs {
    DevView view;            // geometry of the view; view.out = its hit records
    Rule rule;               // termination rule and slab geometry
    bhr_shade_params p;      // the disk's look (density, opacity, temperature, noise, Doppler)
    float ln_1000, ln_40000; // logf of the blackbody table's range, from the host's libm
    float thick;             // uDiskThickness (H / r)
    const uint4* noise8;     // BHR_NOISE_SIZE^3 texel neighbourhoods (launch_noise_expand)
    const float4* lut;       // BHR_BLACKBODY_LUT entries
    float4* rgbt;            // per pixel: gathered rgb, transmittance
};

cudaError_t launch_march_vol(const VolArgs& a, cudaStream_t st);

}  // namespace bhr
