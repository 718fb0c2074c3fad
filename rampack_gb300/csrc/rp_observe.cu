// Observables reduced on the device: the nematic order tensor's sums
// (NematicOrder::calculate, core/observables/NematicOrder.cpp:9-27).
#include <cuda_runtime.h>

#include <algorithm>

#include "rp_internal.cuh"

namespace rp {

namespace {

constexpr int Q_THREADS = 256;

// Per block, in a fixed order: the six sums of u_i u_j over its particles' primary axes
// (orientation column 2).  The host adds the block sums in block order, so the result does
// not depend on scheduling.
__global__ void k_axis_moments(const double *rot64, int64_t n, double *partial) {
    __shared__ double red[6][Q_THREADS];
    double m[6] = {0, 0, 0, 0, 0, 0};
    for (int64_t i = blockIdx.x * (int64_t)Q_THREADS + threadIdx.x; i < n; i += (int64_t)gridDim.x * Q_THREADS) {
        const double *r = rot64 + 9 * i;
        const double u[3] = {r[2], r[5], r[8]};
        m[0] += u[0] * u[0];
        m[1] += u[0] * u[1];
        m[2] += u[0] * u[2];
        m[3] += u[1] * u[1];
        m[4] += u[1] * u[2];
        m[5] += u[2] * u[2];
    }
    for (int k = 0; k < 6; k++) red[k][threadIdx.x] = m[k];
    __syncthreads();
    for (int w = Q_THREADS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int k = 0; k < 6; k++) red[k][threadIdx.x] += red[k][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < 6) partial[6 * blockIdx.x + threadIdx.x] = red[threadIdx.x][0];
}

}  // namespace

int axis_moment_blocks(int64_t n) { return (int)std::min<int64_t>(1024, (n + Q_THREADS - 1) / Q_THREADS); }

cudaError_t launch_axis_moments(const double *rot64, int64_t n, double *partial, cudaStream_t st) {
    k_axis_moments<<<axis_moment_blocks(n), Q_THREADS, 0, st>>>(rot64, n, partial);
    return cudaGetLastError();
}

}  // namespace rp
