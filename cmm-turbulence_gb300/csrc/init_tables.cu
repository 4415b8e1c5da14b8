// init_tables.cu -- random offsets of the turbulence_gaussienne initial condition.
//
// The reference draws the offset of each of its 7 x 7 negative blobs inside the
// initial-condition function, from a fresh cuRAND device generator per blob and axis:
// curand_init(seed, 0, 0), one curand() draw, offset = ((draw % 1000) - 500) / 1e5, with
// seed (mu_x + 1) mu_y^2 for x and (mu_y + 1) mu_x^2 for y
// (src/simulation/cmm-init.cu:148-160).  The 98 values depend on nothing else, so this
// library draws them once, with the same cuRAND device calls, into a table the
// initial-condition evaluators read: out[mu_x * 7 + mu_y] (x) and out[49 + mu_x * 7 + mu_y] (y).
#include <cuda_runtime.h>
#include <curand_kernel.h>

#include "kernels.hpp"

namespace cmm {

__global__ void k_gaussienne_offsets(double* __restrict__ out)
{
    const int b = threadIdx.x;
    if (b >= 2 * kGaussBlobs * kGaussBlobs) return;
    const int axis = b / (kGaussBlobs * kGaussBlobs), k = b % (kGaussBlobs * kGaussBlobs);
    const int mx = k / kGaussBlobs, my = k % kGaussBlobs;
    const unsigned long long seed = axis == 0 ? (unsigned long long)((mx + 1) * my * my)
                                              : (unsigned long long)((my + 1) * mx * mx);
    curandState_t st;
    curand_init(seed, 0, 0, &st);
    out[b] = ((double)(curand(&st) % 1000) - 500) / 100000;
}

cudaError_t launch_gaussienne_offsets(double* out, cudaStream_t s)
{
    k_gaussienne_offsets<<<1, 2 * kGaussBlobs * kGaussBlobs, 0, s>>>(out);
    return cudaGetLastError();
}

}  // namespace cmm
