// Launches of the body-aware march (bodies_march.cuh): the thin or no-disk variant here; the
// volumetric variant is built in bodies_vol.cu with the volumetric march's arithmetic flags.
#include <cuda_runtime.h>

#include "bodies.cuh"
#include "bodies_march.cuh"

namespace bhr {

cudaError_t launch_march_bodies(const BodyArgs& a, bool volumetric, cudaStream_t st) {
    if (volumetric) return launch_march_bodies_vol(a, st);
    const dim3 grid((a.view.width + 31) / 32, (a.view.height + 7) / 8);
    k_march_bodies<false><<<grid, 256, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace bhr
