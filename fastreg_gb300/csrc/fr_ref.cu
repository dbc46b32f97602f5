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
        const int X = P.X, XY = P.X * P.Y;
        const int z0 = max(tl.w, 1), z1 = min(tl.w + kTileZ, P.Z - 1);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float* __restrict__ Q = a.psi + c * a.NT + P.off;
            float* Lc = a.L + c * a.NT + P.off;
            for (int z = z0; z < z1; ++z) {
                const int i = x + X * y + XY * z;
                float s = -6.f * __ldg(Q + i);
                s = s + __ldg(Q + i + 1);
                s = s + __ldg(Q + i - 1);
                s = s + __ldg(Q + i + X);
                s = s + __ldg(Q + i - X);
                s = s + __ldg(Q + i + XY);
                s = s + __ldg(Q + i - XY);
                Lc[i] = -1.f * s;
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

// entropy flux of the (Dv)v diagonal term (vector_fields.cu:376-378)
__device__ __forceinline__ float entropy_flux(float c, float n) {
    return ((fmaxf(c, 0.f) * fmaxf(c, 0.f) - fminf(c, 0.f) * fminf(c, 0.f)) + fminf(n, 0.f) * fminf(n, 0.f)) -
           fmaxf(n, 0.f) * fmaxf(n, 0.f);
}

// ----------------------------------------------------------------------------------
// fused pass A
// ----------------------------------------------------------------------------------
__global__ void __launch_bounds__(256, 3) ref_pass_a_kernel(RefIterArgs a) {
    for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x) {
        const Tile tl = a.tiles[t];
        if (a.stop[tl.x]) continue;
        const Pair P = a.pairs[tl.x];
        const int x = tl.y + (int)(threadIdx.x & 31), y = tl.z + (int)(threadIdx.x >> 5);
        if (x < 1 || x > P.X - 2 || y < 1 || y > P.Y - 2) continue;
        const int X = P.X, Y = P.Y, Z = P.Z, XY = P.X * P.Y, N = (int)P.N;
        const long long NT = a.NT;
        const float* __restrict__ S = a.S + P.off;
        const float* __restrict__ T = a.T + P.off;
        const float* __restrict__ rho = a.rho + P.off;
        const float* __restrict__ V[3] = {a.v + P.off, a.v + NT + P.off, a.v + 2 * NT + P.off};
        const float* __restrict__ Q[3] = {a.pinv + P.off, a.pinv + NT + P.off, a.pinv + 2 * NT + P.off};
        const float* __restrict__ Lp[3] = {a.L + P.off, a.L + NT + P.off, a.L + 2 * NT + P.off};
        float* rho_n = a.rho_n + P.off;
        float* Vn[3] = {a.v_n + P.off, a.v_n + NT + P.off, a.v_n + 2 * NT + P.off};
        float* Qn[3] = {a.pinv_n + P.off, a.pinv_n + NT + P.off, a.pinv_n + 2 * NT + P.off};
        const bool dv_xy = x >= 2 && x <= X - 3 && y >= 2 && y <= Y - 2;
        const int z0 = max(tl.w, 1), z1 = min(tl.w + kTileZ, Z - 1);
        for (int z = z0; z < z1; ++z) {
            const int i = x + X * y + XY * z;

            // T o psi_inv and L o psi_inv, gathered at psi_inv(x)
            const float q[3] = {__ldg(Q[0] + i), __ldg(Q[1] + i), __ldg(Q[2] + i)};
            const Cell32 cl = locate32(X, Y, Z, q[0], q[1], q[2]);
            const float Tq = a.first_iter ? __ldg(T + i) : tri_unchecked32(T, X, XY, N, cl);
            float Lq[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) Lq[c] = tri_unchecked32(Lp[c], X, XY, N, cl);

            // Jacobian of psi_inv, row r = d(psi_inv_r)/d(x, y, z), and its determinant
            float M[3][3];
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                M[r][0] = (__ldg(Q[r] + i + 1) - __ldg(Q[r] + i - 1)) * 0.5f;
                M[r][1] = (__ldg(Q[r] + i + X) - __ldg(Q[r] + i - X)) * 0.5f;
                M[r][2] = (__ldg(Q[r] + i + XY) - __ldg(Q[r] + i - XY)) * 0.5f;
            }
            const float det = det_ref(M);

            // central-difference gradient of S and the potential gradient
            const float Si = __ldg(S + i);
            const float gs[3] = {(__ldg(S + i + 1) - __ldg(S + i - 1)) * 0.5f,
                                 (__ldg(S + i + X) - __ldg(S + i - X)) * 0.5f,
                                 (__ldg(S + i + XY) - __ldg(S + i - XY)) * 0.5f};
            const float diff = Si - Tq;
            float gU[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) gU[c] = ((diff * gs[c]) + (a.w_reg * Lq[c])) * det;

            // velocity and its 6 neighbours, each loaded once
            float vc[3], vxm[3], vxp[3], vym[3], vyp[3], vzm[3], vzp[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                vc[c] = __ldg(V[c] + i);
                vxm[c] = __ldg(V[c] + i - 1);
                vxp[c] = __ldg(V[c] + i + 1);
                vym[c] = __ldg(V[c] + i - X);
                vyp[c] = __ldg(V[c] + i + X);
                vzm[c] = __ldg(V[c] + i - XY);
                vzp[c] = __ldg(V[c] + i + XY);
            }
            const float vx = vc[0], vy = vc[1], vz = vc[2];

            // divergence of rho*v (upwind) and the density update
            const float p = __ldg(rho + i);
            const float t11 = (vx > 0.f) ? (-vx) * p : (-vx) * __ldg(rho + i + 1);
            const float t12 = (vxm[0] > 0.f) ? vxm[0] * __ldg(rho + i - 1) : vxm[0] * p;
            const float t21 = (vy > 0.f) ? (-vy) * p : (-vy) * __ldg(rho + i + X);
            const float t22 = (vym[1] > 0.f) ? vym[1] * __ldg(rho + i - X) : vym[1] * p;
            const float t31 = (vz > 0.f) ? (-vz) * p : (-vz) * __ldg(rho + i + XY);
            const float t32 = (vzm[2] > 0.f) ? vzm[2] * __ldg(rho + i - XY) : vzm[2] * p;
            const float div = ((((t11 + t12) + t21) + t22) + t31) + t32;
            const float rho_new = p + a.alpha * div;
            rho_n[i] = rho_new;

            // (Dv)v: entropy scheme on the diagonal, upwind off the diagonal
            const float ax1 = entropy_flux(vx, vxp[0]);
            const float ax2 = (vy > 0.f) ? vy * (vx - vym[0]) : vy * (vyp[0] - vx);
            const float ax3 = (vz > 0.f) ? vz * (vx - vzm[0]) : vz * (vzp[0] - vx);
            const float ay1 = (vx > 0.f) ? vx * (vy - vxm[1]) : vx * (vxp[1] - vy);
            const float ay2 = entropy_flux(vy, vyp[1]);
            const float ay3 = (vz > 0.f) ? vz * (vy - vzm[1]) : vz * (vzp[1] - vy);
            const float az1 = (vx > 0.f) ? vx * (vz - vxm[2]) : vx * (vxp[2] - vz);
            const float az2 = (vy > 0.f) ? vy * (vz - vym[2]) : vy * (vyp[2] - vz);
            const float az3 = entropy_flux(vz, vzp[2]);
            const float dvv[3] = {(0.5f * ax1 + ax2) + ax3, (ay1 + 0.5f * ay2) + ay3, (az1 + az2) + 0.5f * az3};

            // negated upwind second differences of v (x in [2,X-3], y in [2,Y-2],
            // z in [2,Z-3]); the y and z forward branches read (+2, -1, 0) as the
            // reference does, and y+2 at y = Y-2 reads linear index i + 2X as is.
            float dv[3] = {0.f, 0.f, 0.f};
            if (dv_xy && z >= 2 && z <= Z - 3) {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float xx = (vx < 0.f) ? (__ldg(V[c] + i + 2) - 2.f * vxp[c]) + vc[c]
                                                : (vc[c] - 2.f * vxm[c]) + __ldg(V[c] + i - 2);
                    const float yy = (vy < 0.f) ? (__ldg(V[c] + i + 2 * X) - 2.f * vym[c]) + vc[c]
                                                : (vc[c] - 2.f * vym[c]) + __ldg(V[c] + i - 2 * X);
                    const float zz = (vz < 0.f) ? (__ldg(V[c] + i + 2 * XY) - 2.f * vzm[c]) + vc[c]
                                                : (vc[c] - 2.f * vzm[c]) + __ldg(V[c] + i - 2 * XY);
                    dv[c] = -1.f * ((xx + yy) + zz);
                }
            }

            // velocity update (solver.cu:198-209) and psi_inv update (solver.cu:275-277)
            const float qd = a.m2 / (fabsf(rho_new) + 1e-5f);
            float vn[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float friction = a.f1 * vc[c];
                const float diffusion = a.tau * dv[c];
                const float potential = qd * gU[c];
                const float acc = ((friction + dvv[c]) - diffusion) + potential;
                vn[c] = vc[c] - a.alpha * acc;
                Vn[c][i] = vn[c];
            }
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                const float jv = ((M[r][0] * vn[0]) + (M[r][1] * vn[1])) + (M[r][2] * vn[2]);
                Qn[r][i] = q[r] - a.alpha * jv;
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
            const int X = P.X, Y = P.Y, Z = P.Z, XY = P.X * P.Y;
            const long long NT = a.NT;
            // the velocity pass A just wrote
            const float* __restrict__ V[3] = {a.v_n + P.off, a.v_n + NT + P.off, a.v_n + 2 * NT + P.off};
            float* Q[3] = {a.psi + P.off, a.psi + NT + P.off, a.psi + 2 * NT + P.off};
            const int z0 = max(tl.w, 1), z1 = min(tl.w + kTileZ, P.Z - 1);
            for (int z = z0; z < z1; ++z) {
                const int i = x + X * y + XY * z;
                const float px = Q[0][i], py = Q[1][i], pz = Q[2][i];
                const Cell32 cl = locate32(X, Y, Z, px, py, pz);
                const float ux = a.alpha * tri_checked32(V[0], X, Y, Z, XY, cl);
                const float uy = a.alpha * tri_checked32(V[1], X, Y, Z, XY, cl);
                const float uz = a.alpha * tri_checked32(V[2], X, Y, Z, XY, cl);
                Q[0][i] = px + ux;
                Q[1][i] = py + uy;
                Q[2][i] = pz + uz;
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
