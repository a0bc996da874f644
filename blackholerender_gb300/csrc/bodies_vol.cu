// The body-aware march with the volumetric disk (bodies_march.cuh, kVol), compiled with the
// volumetric march's flags: the disk's samples take the same fast divide and square root as
// k_march_vol.
#include <cuda_runtime.h>

#include "bodies.cuh"
#include "bodies_march.cuh"

namespace bhr {

cudaError_t launch_march_bodies_vol(const BodyArgs& a, cudaStream_t st) {
    const dim3 grid((a.view.width + 31) / 32, (a.view.height + 7) / 8);
    k_march_bodies<true><<<grid, 256, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace bhr
