// fr_fields.cu -- the reference's two field kernels that its registration never calls
// (src/fastreg/cuda/vector_fields.cu:109-136,194-225), on 3-plane FP32 fields in the
// caller's unpadded layout:
//   estimate_inverse_kernel    `sweeps` passes of psi_inv <- -psi o psi_inv, in place.
//                              A voxel's update reads only its own previous value (the
//                              gather is from psi), so each thread runs all the sweeps of
//                              its voxel in registers: one launch instead of the
//                              reference's 48 launches with a device sync after each.
//   interpolate_field_kernel   out = field o pos (the reference's interpolate_gradient)
// Both sample with the unchecked vector trilinear rule of interpolate_field
// (include/cuda/cuda_utils.hpp:86-107), one cell shared by the three components.
#include "fr_common.cuh"
#include "fr_kernels.h"

namespace frg {

__global__ void __launch_bounds__(256) estimate_inverse_kernel(const float* __restrict__ psi, float* psi_inv, int X,
                                                               int Y, int Z, int sweeps) {
    const int N = X * Y * Z, XY = X * Y;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        float p[3] = {psi_inv[i], psi_inv[N + i], psi_inv[2 * N + i]};
        for (int s = 0; s < sweeps; ++s) {
            const Cell32 cl = locate32(X, Y, Z, X, p[0], p[1], p[2]);
#pragma unroll
            for (int c = 0; c < 3; ++c) p[c] = -1.f * tri_unchecked32(psi + (long long)c * N, X, XY, N, cl);
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) psi_inv[(long long)c * N + i] = p[c];
    }
}

__global__ void __launch_bounds__(256) interpolate_field_kernel(const float* __restrict__ field,
                                                                const float* __restrict__ pos, float* __restrict__ out,
                                                                int X, int Y, int Z) {
    const int N = X * Y * Z, XY = X * Y;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const Cell32 cl = locate32(X, Y, Z, X, __ldg(pos + i), __ldg(pos + N + i), __ldg(pos + 2 * N + i));
#pragma unroll
        for (int c = 0; c < 3; ++c) out[(long long)c * N + i] = tri_unchecked32(field + (long long)c * N, X, XY, N, cl);
    }
}

}  // namespace frg
