// Launch arguments of the body-aware march (bodies.cu), filled by the C ABI (api.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "bhr.h"
#include "march.cuh"
#include "vol.cuh"

namespace bhr {

struct BodyArgs {
    DevView view;                     // geometry of the view; view.out = its hit records
    Rule rule;                        // termination rule and slab geometry
    int32_t nbodies;
    int32_t pad;
    bhr_body_hit* body_out;           // per pixel
    DiskLook look;                    // the volumetric disk's look (volumetric views only)
    float4* rgbt;                     // volumetric views: per pixel gathered rgb, transmittance
    bhr_body bodies[BHR_MAX_BODIES];  // the reference's BodyGpu array
};

// Thin or no disk: k_march_bodies<false> (bodies.cu); the volumetric disk: <true> (bodies_vol.cu).
cudaError_t launch_march_bodies(const BodyArgs& a, bool volumetric, cudaStream_t st);
cudaError_t launch_march_bodies_vol(const BodyArgs& a, cudaStream_t st);

}  // namespace bhr
