// fr_sob.h -- the sobolev solver: SSD data term, Gaussian-smoothed (Sobolev) gradient,
// heavy-ball momentum and a compositional update of the deformation.
//
// One iteration, per voxel x of every pair (phi = positions, m = momentum):
//   W(x)   = S(phi(x))                         trilinear, cell floor clamped to dim-2
//   g(x)   = (W(x) - T(x)) * dW/dphi(x)        exact derivative of the trilinear
//            + lambda * lap(phi - x)(x)        interpolant (0 along a clamped axis);
//                                              lap = graph Laplacian over the grid's
//                                              neighbours, lambda = W_REG
//   gs     = G_sigma * g                       separable Gaussian, SMOOTH_WIDTH taps,
//                                              normalised, replicate boundary, each tap
//                                              a fused multiply-add in the order -R..R
//   m      = DAMPING * m - STEP * gs
//   phi(x) = phi(x) + m(phi(x))                trilinear gather of the new m
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include "fr_common.cuh"

namespace frg {

constexpr int kMaxSmoothWidth = 15;
constexpr int kSobTileY = 8;
static_assert(kSobTileY == kTileY, "tile extents must agree");

struct SobIterArgs {
    const Pair* pairs;
    // each kernel's own table of 32 x 8 x depth tiles: gradient, smoothing, update
    const Tile* tiles_g;
    int ntiles_g, depth_g;
    const Tile* tiles_s;
    int ntiles_s, depth_s;
    const Tile* tiles_b;
    int ntiles_b, depth_b;
    int npairs;
    long long NT;
    const float* S;
    const float* T;
    float* phi;   // positions (3 planes)
    float* m;     // momentum (3 planes)
    float* g;     // gradient (3 planes)
    float damping, step;
    float lambda;  // W_REG; the kernels take each pair's weight from Pair::w_reg
    float taps[kMaxSmoothWidth];
    int radius;
    float max_update_norm;
    int iter;
    int* stop;
    unsigned long long* keys;
    unsigned long long* trace;
    double* energy;  // [max_iter][npairs] 0.5 * sum (W - T)^2 before the update
    unsigned int* counter;
    const CUtensorMap* tmaps;  // [npairs][TM_COUNT] tensor maps (fr_kernels.h), TMA-staged variants
    unsigned int* err;         // device error word (kErrTmaTimeout: a staging wait gave up)
};

// Gaussian taps exp(-k^2 / (2 sigma^2)), k = -R..R, normalised; computed in double
// and rounded to float.
void gaussian_taps(float sigma, int width, float* taps);

size_t sob_grad_smem_bytes();  // dynamic shared memory of sob_grad_kernel
__global__ void sob_grad_kernel(SobIterArgs a);
size_t sob_grad_tma_smem_bytes();  // dynamic shared memory of sob_grad_tma_kernel
__global__ void sob_grad_tma_kernel(SobIterArgs a);
// the smoothing kernel instance for a radius and staging variant (1: TMA)
const void* sob_smooth3_fn(int radius, int variant = 0);
// box of the smoothing kernel's staged slice for radius R: x extent, rows
inline void sob_smooth_box(int R, int* wx, int* rows) {
    *wx = kTileX + 2 * ((R + 3) / 4 * 4);
    *rows = kSobTileY + 2 * R;
}
__global__ void sob_pass_b_kernel(SobIterArgs a);
__global__ void sob_pass_b_staged_kernel(SobIterArgs a);

// grids: {grad, smooth, pass_b}; variants: staging of {grad, smooth, pass_b} (1: TMA); with `ev`
// (4 events) each launch is bracketed
cudaError_t launch_sob_iter(const SobIterArgs& a, const int* grids, const int* variants, cudaStream_t s,
                            cudaEvent_t* ev = nullptr);

}  // namespace frg
