// fr_ref.cu -- reference-mode solver kernels (the accelerated PDE flow of fastreg).
//
// One iteration of estimate_psi (src/fastreg/cuda/solver.cu:329-433) is three
// launches over a packed cohort of pairs:
//   ref_laplacian_kernel  L = -Laplacian(psi) on the interior    (vector_fields.cu:275-300)
//   ref_pass_a_kernel     divergence + density, J(psi_inv) and its determinant, the
//                         potential gradient with L o psi_inv and T o psi_inv gathered
//                         on the fly, (Dv)v, the upwind velocity Laplacian, the
//                         velocity update and the psi_inv update -- all fused
//                         (solver.cu:56-289, vector_fields.cu:231-404,503-535)
//   ref_pass_b_kernel     psi += alpha * v o psi with the max-update-norm reduction
//                         and the on-device convergence test (solver.cu:230-247,
//                         reductor.cu:426-539, solver.cu:407-421)
// rho, v and psi_inv are double-buffered because pass A reads neighbours of the old
// values while writing the new ones; psi is updated in place (pass B reads psi only
// at the voxel it writes).  Boundary voxels are never written, as in the reference.
#include "fr_common.cuh"
#include "fr_kernels.h"

namespace frg {

// ----------------------------------------------------------------------------------
// L = -(sum of 6 neighbours - 6 psi), interior only
// ----------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) ref_laplacian_kernel(RefIterArgs a) {
    for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x) {
        const Tile tl = a.tiles[t];
        if (a.stop[tl.x]) continue;
        const Pair P = a.pairs[tl.x];
        const int x = tl.y + (int)(threadIdx.x & 31), y = tl.z + (int)(threadIdx.x >> 5);
        if (x < 1 || x > P.X - 2 || y < 1 || y > P.Y - 2) continue;
        const long long X = P.X, XY = (long long)P.X * P.Y;
        const int z0 = max(tl.w, 1), z1 = min(tl.w + kTileZ, P.Z - 1);
        for (int z = z0; z < z1; ++z) {
            const long long i = P.off + lin(P, x, y, z);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float* __restrict__ Q = a.psi + c * a.NT;
                float s = -6.f * __ldg(Q + i);
                s = s + __ldg(Q + i + 1);
                s = s + __ldg(Q + i - 1);
                s = s + __ldg(Q + i + X);
                s = s + __ldg(Q + i - X);
                s = s + __ldg(Q + i + XY);
                s = s + __ldg(Q + i - XY);
                a.L[c * a.NT + i] = -1.f * s;
            }
        }
    }
}

// det(Mat4f) as written in the reference (include/cuda/cuda_utils.hpp:389-396)
__device__ __forceinline__ float det_ref(const float m[3][3]) {
    float first = ((m[0][0] * m[1][1]) * m[2][2] + (m[1][0] * m[2][1]) * m[0][2]) + (m[2][0] * m[0][1]) * m[1][2];
    float second = ((m[0][2] * m[1][1]) + m[2][0]) * ((m[1][2] * m[2][1]) * m[0][0]) + (m[2][2] * m[0][1]) * m[1][0];
    return first - second;
}

// ----------------------------------------------------------------------------------
// fused pass A
// ----------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) ref_pass_a_kernel(RefIterArgs a) {
    for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x) {
        const Tile tl = a.tiles[t];
        if (a.stop[tl.x]) continue;
        const Pair P = a.pairs[tl.x];
        const int x = tl.y + (int)(threadIdx.x & 31), y = tl.z + (int)(threadIdx.x >> 5);
        if (x < 1 || x > P.X - 2 || y < 1 || y > P.Y - 2) continue;
        const long long X = P.X, XY = (long long)P.X * P.Y, NT = a.NT;
        const float* __restrict__ S = a.S + P.off;
        const float* __restrict__ T = a.T + P.off;
        const float* __restrict__ rho = a.rho + P.off;
        const float* __restrict__ vx_ = a.v + P.off;
        const float* __restrict__ vy_ = vx_ + NT;
        const float* __restrict__ vz_ = vy_ + NT;
        const float* __restrict__ pinv = a.pinv + P.off;
        const float* __restrict__ L = a.L + P.off;
        const bool dv_y = y >= 2 && y <= P.Y - 2;
        const bool dv_x = x >= 2 && x <= P.X - 3;
        const int z0 = max(tl.w, 1), z1 = min(tl.w + kTileZ, P.Z - 1);
        for (int z = z0; z < z1; ++z) {
            const long long i = lin(P, x, y, z);

            // divergence of rho*v (upwind) and the density update
            const float vx = __ldg(vx_ + i), vy = __ldg(vy_ + i), vz = __ldg(vz_ + i);
            const float p = __ldg(rho + i);
            const float t11 = (vx > 0.f) ? (-vx) * p : (-vx) * __ldg(rho + i + 1);
            const float vxm = __ldg(vx_ + i - 1);
            const float t12 = (vxm > 0.f) ? vxm * __ldg(rho + i - 1) : vxm * p;
            const float t21 = (vy > 0.f) ? (-vy) * p : (-vy) * __ldg(rho + i + X);
            const float vym = __ldg(vy_ + i - X);
            const float t22 = (vym > 0.f) ? vym * __ldg(rho + i - X) : vym * p;
            const float t31 = (vz > 0.f) ? (-vz) * p : (-vz) * __ldg(rho + i + XY);
            const float vzm = __ldg(vz_ + i - XY);
            const float t32 = (vzm > 0.f) ? vzm * __ldg(rho + i - XY) : vzm * p;
            const float div = ((((t11 + t12) + t21) + t22) + t31) + t32;
            const float rho_new = p + a.alpha * div;
            a.rho_n[P.off + i] = rho_new;

            // Jacobian of psi_inv, row r = d(psi_inv_r)/d(x, y, z)
            float M[3][3];
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                const float* __restrict__ Q = pinv + r * NT;
                M[r][0] = (__ldg(Q + i + 1) - __ldg(Q + i - 1)) * 0.5f;
                M[r][1] = (__ldg(Q + i + X) - __ldg(Q + i - X)) * 0.5f;
                M[r][2] = (__ldg(Q + i + XY) - __ldg(Q + i - XY)) * 0.5f;
            }
            const float det = det_ref(M);

            // T o psi_inv and L o psi_inv, gathered at psi_inv(x)
            const Cell cl = locate(P, __ldg(pinv + i), __ldg(pinv + NT + i), __ldg(pinv + 2 * NT + i));
            const float Tq = a.first_iter ? __ldg(T + i) : tri_unchecked(T, P, cl);
            float Lq[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) Lq[c] = tri_unchecked(L + c * NT, P, cl);

            // central-difference gradient of S and the potential gradient
            float gs[3];
            gs[0] = (__ldg(S + i + 1) - __ldg(S + i - 1)) * 0.5f;
            gs[1] = (__ldg(S + i + X) - __ldg(S + i - X)) * 0.5f;
            gs[2] = (__ldg(S + i + XY) - __ldg(S + i - XY)) * 0.5f;
            const float diff = __ldg(S + i) - Tq;
            float gU[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) gU[c] = ((diff * gs[c]) + (a.w_reg * Lq[c])) * det;

            // (Dv)v
            const float vxp_x = __ldg(vx_ + i + 1), vyp_y = __ldg(vy_ + i + X), vzp_z = __ldg(vz_ + i + XY);
            const float ax1 = ((fmaxf(vx, 0.f) * fmaxf(vx, 0.f) - fminf(vx, 0.f) * fminf(vx, 0.f)) +
                               fminf(vxp_x, 0.f) * fminf(vxp_x, 0.f)) -
                              fmaxf(vxp_x, 0.f) * fmaxf(vxp_x, 0.f);
            const float ax2 = (vy > 0.f) ? vy * (vx - __ldg(vx_ + i - X)) : vy * (__ldg(vx_ + i + X) - vx);
            const float ax3 = (vz > 0.f) ? vz * (vx - __ldg(vx_ + i - XY)) : vz * (__ldg(vx_ + i + XY) - vx);
            const float ay1 = (vx > 0.f) ? vx * (vy - __ldg(vy_ + i - 1)) : vx * (__ldg(vy_ + i + 1) - vy);
            const float ay2 = ((fmaxf(vy, 0.f) * fmaxf(vy, 0.f) - fminf(vy, 0.f) * fminf(vy, 0.f)) +
                               fminf(vyp_y, 0.f) * fminf(vyp_y, 0.f)) -
                              fmaxf(vyp_y, 0.f) * fmaxf(vyp_y, 0.f);
            const float ay3 = (vz > 0.f) ? vz * (vy - __ldg(vy_ + i - XY)) : vz * (__ldg(vy_ + i + XY) - vy);
            const float az1 = (vx > 0.f) ? vx * (vz - __ldg(vz_ + i - 1)) : vx * (__ldg(vz_ + i + 1) - vz);
            const float az2 = (vy > 0.f) ? vy * (vz - __ldg(vz_ + i - X)) : vy * (__ldg(vz_ + i + X) - vz);
            const float az3 = ((fmaxf(vz, 0.f) * fmaxf(vz, 0.f) - fminf(vz, 0.f) * fminf(vz, 0.f)) +
                               fminf(vzp_z, 0.f) * fminf(vzp_z, 0.f)) -
                              fmaxf(vzp_z, 0.f) * fmaxf(vzp_z, 0.f);
            float dvv[3];
            dvv[0] = (0.5f * ax1 + ax2) + ax3;
            dvv[1] = (ay1 + 0.5f * ay2) + ay3;
            dvv[2] = (az1 + az2) + 0.5f * az3;

            // negated upwind second differences of v (x in [2,X-3], y in [2,Y-2],
            // z in [2,Z-3]); the y and z forward branches read (+2, -1, 0) as the
            // reference does, and y+2 at y = Y-2 reads linear index i + 2X as is.
            const float vel[3] = {vx, vy, vz};
            float dv[3] = {0.f, 0.f, 0.f};
            if (dv_x && dv_y && z >= 2 && z <= P.Z - 3) {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float* __restrict__ V = vx_ + c * NT;
                    const float xx = (vx < 0.f) ? (__ldg(V + i + 2) - 2.f * __ldg(V + i + 1)) + vel[c]
                                                : (vel[c] - 2.f * __ldg(V + i - 1)) + __ldg(V + i - 2);
                    const float yy = (vy < 0.f) ? (__ldg(V + i + 2 * X) - 2.f * __ldg(V + i - X)) + vel[c]
                                                : (vel[c] - 2.f * __ldg(V + i - X)) + __ldg(V + i - 2 * X);
                    const float zz = (vz < 0.f) ? (__ldg(V + i + 2 * XY) - 2.f * __ldg(V + i - XY)) + vel[c]
                                                : (vel[c] - 2.f * __ldg(V + i - XY)) + __ldg(V + i - 2 * XY);
                    dv[c] = -1.f * ((xx + yy) + zz);
                }
            }

            // velocity update (solver.cu:198-209) and psi_inv update (solver.cu:275-277)
            const float q = a.m2 / (fabsf(rho_new) + 1e-5f);
            float vn[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float friction = a.f1 * vel[c];
                const float diffusion = a.tau * dv[c];
                const float potential = q * gU[c];
                const float acc = ((friction + dvv[c]) - diffusion) + potential;
                vn[c] = vel[c] - a.alpha * acc;
                a.v_n[c * NT + P.off + i] = vn[c];
            }
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                const float jv = ((M[r][0] * vn[0]) + (M[r][1] * vn[1])) + (M[r][2] * vn[2]);
                a.pinv_n[r * NT + P.off + i] = __ldg(pinv + r * NT + i) - a.alpha * jv;
            }
        }
    }
}

// ----------------------------------------------------------------------------------
// pass B: psi += alpha * v o psi, max update norm, convergence
// ----------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) ref_pass_b_kernel(RefIterArgs a) {
    __shared__ unsigned long long red[32];
    __shared__ bool last;
    const int tid = threadIdx.x;
    for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x) {
        const Tile tl = a.tiles[t];
        if (a.stop[tl.x]) continue;  // uniform over the block
        const Pair P = a.pairs[tl.x];
        const int x = tl.y + (int)(threadIdx.x & 31), y = tl.z + (int)(threadIdx.x >> 5);
        unsigned long long best = 0ull;
        if (x >= 1 && x <= P.X - 2 && y >= 1 && y <= P.Y - 2) {
            const long long NT = a.NT;
            const float* __restrict__ v = a.v_n + P.off;  // the velocity pass A just wrote
            float* psi = a.psi + P.off;
            const int z0 = max(tl.w, 1), z1 = min(tl.w + kTileZ, P.Z - 1);
            for (int z = z0; z < z1; ++z) {
                const long long i = lin(P, x, y, z);
                const float px = psi[i], py = psi[NT + i], pz = psi[2 * NT + i];
                const Cell cl = locate(P, px, py, pz);
                const float ux = a.alpha * tri_checked(v, P, cl);
                const float uy = a.alpha * tri_checked(v + NT, P, cl);
                const float uz = a.alpha * tri_checked(v + 2 * NT, P, cl);
                psi[i] = px + ux;
                psi[NT + i] = py + uy;
                psi[2 * NT + i] = pz + uz;
                const float nrm = norm3_rd(ux, uy, uz);
                if (nrm == nrm) {  // NaN norms never win, as in the reference's '>' test
                    const unsigned long long k = norm_key(nrm, i);
                    best = k > best ? k : best;
                }
            }
        }
        const unsigned long long bm = block_max_u64(best, red);
        if (tid == 0 && bm) atomicMax(a.keys + tl.x, bm);
    }

    // the last block to finish records this iteration and decides convergence
    __threadfence();
    __syncthreads();
    if (tid == 0) last = (atomicAdd(a.counter, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!last) return;
    __threadfence();
    for (int p = tid; p < a.npairs; p += blockDim.x) {
        if (a.stop[p]) continue;
        const unsigned long long k = atomicExch(a.keys + p, 0ull);
        a.trace[(long long)(a.iter - 1) * a.npairs + p] = k;
        const float mx = __uint_as_float((unsigned)(k >> 32));
        if (mx <= a.max_update_norm) a.stop[p] = a.iter;
    }
    if (tid == 0) *a.counter = 0u;
}

}  // namespace frg
