// Launch arguments of the body-aware march (bodies.cu), filled by the C ABI (api.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "bhr.h"
#include "march.cuh"

namespace bhr {

struct BodyArgs {
    DevView view;                     // geometry of the view; view.out = its hit records
    Rule rule;                        // termination rule and slab geometry
    int32_t nbodies;
    int32_t pad;
    bhr_body_hit* body_out;           // per pixel
    bhr_body bodies[BHR_MAX_BODIES];  // the reference's BodyGpu array
};

cudaError_t launch_march_bodies(const BodyArgs& a, cudaStream_t st);

}  // namespace bhr
