// fr_kernels.h -- kernel argument blocks and launch entry points shared between the
// kernel translation units and the C-ABI implementation (fr_api.cu).
#pragma once

#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>

#include "fr_common.cuh"

namespace frg {

// Tensor maps of one pair, in this order, for the kernels that stage through TMA (boxes
// are part of a map, so each kernel that stages a field has its own map of it).
enum TmapIndex {
    TM_LAP_PSI = 0,  // psi, 4-D (x, y, z, component), box 40 x 10 x 1 x 3 (Laplacian)
    TM_LAP_T,        // T, 3-D, box 32 x 8 x 1 (Laplacian; the sobolev gradient uses both,
                     // phi living where psi does)
    TM_SOB_G,        // the sobolev gradient g, 4-D, box (32 + 2 HX) x (8 + 2 R) x 1 x 3 for the
                     // smoothing radius R (HX = R rounded up to 4)
    TM_PA_V0,        // pass A: v (buffer 0, 1), 4-D, box 40 x 12 x 1 x 3 (2-voxel halo)
    TM_PA_V1,
    TM_PA_Q0,        // psi_inv (buffer 0, 1), 4-D, box 40 x 10 x 1 x 3
    TM_PA_Q1,
    TM_PA_R0,        // rho (buffer 0, 1), 3-D, box 40 x 10 x 1
    TM_PA_R1,
    TM_PA_S,         // S, 3-D, box 40 x 10 x 1
    TM_PB_V0,        // pass B's gathered v (buffer 0, 1), 4-D, box kGBX x kGBY x kGBZ x 3
    TM_PB_V1,
    TM_SB_M,         // the sobolev update's gathered momentum, 4-D, the same box
    TM_COUNT
};

// The box of a staged gather (pass B of either solver): columns, rows and slices of the
// gathered field copied per slice of a tile, enough for the cells of a 32 x 8 slice of a
// smooth map (the box's x origin is the cells' lowest x rounded down to a multiple of 4).
constexpr int kGBX = 48, kGBY = 12, kGBZ = 4;

// Arguments of one reference-mode iteration (all three launches take the same block).
struct RefIterArgs {
    const Pair* pairs;
    const Tile* tiles_l;  // 32 x 8 x depth_l tiles (Laplacian)
    int ntiles_l, depth_l;
    const Tile* tiles_a;  // 32 x 8 x depth_a tiles (pass A)
    int ntiles_a, depth_a;
    const Tile* tiles_b;  // 32 x 8 x depth_b tiles (pass B)
    int ntiles_b, depth_b;
    int npairs;
    long long NT;  // packed voxels (plane stride of vector fields)

    const float* S;  // source intensities (packed)
    const float* T;  // target intensities (packed)

    const float* rho;   // density, read
    const float* v;     // velocity, read
    const float* pinv;  // psi_inv, read
    float* rho_n;       // density, written
    float* v_n;         // velocity, written
    float* pinv_n;      // psi_inv, written
    float* psi;         // psi (in place)
    float4* LT;         // (-Laplacian(psi), T) interleaved: the two fields pass A gathers at psi_inv

    float alpha, f1, m2, tau, w_reg, max_update_norm;  // w_reg: W_REG (pass A uses Pair::w_reg)
    int iter;        // 1-based iteration number
    int first_iter;  // T o psi_inv is T itself on the first iteration of a call

    int* stop;                 // per pair: iteration at which it converged (0 = running)
    unsigned long long* keys;  // per pair: max-norm key of the running iteration
    unsigned long long* trace; // [max_iter][npairs] max-norm keys
    unsigned int* counter;     // last-block ticket of pass B
    const CUtensorMap* tmaps;  // [npairs][TM_COUNT] tensor maps of the TMA-staged kernels
    unsigned int* err;         // device error word (kErrTmaTimeout: a staging wait gave up)
};

size_t ref_laplacian_smem_bytes();  // dynamic shared memory of ref_laplacian_kernel
__global__ void ref_laplacian_kernel(RefIterArgs a);
size_t ref_laplacian_tma_smem_bytes();  // dynamic shared memory of ref_laplacian_tma_kernel
__global__ void ref_laplacian_tma_kernel(RefIterArgs a);
size_t ref_pass_a_smem_bytes();  // dynamic shared memory of ref_pass_a_kernel
__global__ void ref_pass_a_kernel(RefIterArgs a);
size_t ref_pass_a_tma_smem_bytes();  // dynamic shared memory of ref_pass_a_tma_kernel
__global__ void ref_pass_a_tma_kernel(RefIterArgs a);
// ref_pass_b_kernel runs 128-thread blocks on 32 x 4 tiles (its staged variant 256 on 32 x 8)
constexpr int kPassBThreads = 128, kPassBTileY = 4;
__global__ void ref_pass_b_kernel(RefIterArgs a);
size_t gather_staged_smem_bytes();  // dynamic shared memory of the staged-gather pass B kernels
__global__ void ref_pass_b_staged_kernel(RefIterArgs a);

// Caller-owned buffers of one pair (device pointers); outputs overwrite inputs in place
// exactly like FastReg::operator() (src/fastreg/fastreg.cpp:58-75).
struct PairIO {
    float* img_T;
    int16_t* lab_T;
    float* img_S;
    int16_t* lab_S;
};

// Arguments of the start-of-registration and end-of-registration kernels.
struct IoArgs {
    const Pair* pairs;
    const Tile* tiles;
    int ntiles;
    int npairs;
    long long NT;
    const PairIO* io;

    float* S;
    float* T;
    int16_t* labS;
    int16_t* labT;
    float* rho0;
    float* rho1;
    float* v0;
    float* v1;
    float* psi;
    float* pinv0;
    float* pinv1;
    float4* LT;
    float rho_init;
    int keep_state;
    int sobolev;        // sobolev solver: no rho/psi_inv, nearest-neighbour labels
    int write_outputs;  // 0: statistics only (verbose energy)

    // final stage
    const int* stop;    // per pair convergence iteration (0 = ran max_iter)
    int max_iter;
    int no_labels;
    double* tile_partials;      // [ntiles][2]: e_data, e_reg
    long long* tile_folds;      // [ntiles]
    const int* pair_tiles;      // [npairs + 1]: the first tile of each pair (tiles are ordered by pair)
    unsigned long long* dice;   // [npairs][2*256 + 1]: inter, count, out of range
    double* pair_energy;        // [npairs][2]
    long long* pair_folds;      // [npairs]
    unsigned int* counter;
};

__global__ void pack_init_kernel(IoArgs a);
__global__ void finalize_kernel(IoArgs a);

// Standalone trilinear warp of one volume (a1 of the hot path).
__global__ void warp_kernel(const float* __restrict__ pos, const float* __restrict__ img,
                            const int16_t* __restrict__ lab, float* __restrict__ out,
                            int16_t* __restrict__ out_lab, Pair P);
__global__ void warp2_kernel(const float* pos, const float* img, const int16_t* lab, float* out, int16_t* out_lab, int X,
                             int Y, int Z);
// the reference's unused field kernels (fr_fields.cu)
__global__ void estimate_inverse_kernel(const float* psi, float* psi_inv, int X, int Y, int Z, int sweeps);
__global__ void interpolate_field_kernel(const float* field, const float* pos, float* out, int X, int Y, int Z);

}  // namespace frg
