// fr_io.cu -- start and end of a registration, and the standalone warp.
//
//   pack_init_kernel  copies the caller's images/labels into the packed cohort arrays
//                     (Volume::initialise, src/fastreg/cuda/volume.cu:29-46) and sets
//                     psi = psi_inv = identity, v = 0, rho = rho_0
//                     (vector_fields.cu:64-79, scalar_fields.cu:53-65)
//   finalize_kernel   writes T o psi_inv and S o psi (intensity + floor-corner label)
//                     into the caller's buffers in place (solver.cu:402,435 and
//                     fastreg.cpp:3-22,71-72) and reduces the final statistics in one
//                     pass: SSD energy and regulariser energy in FP64
//                     (reductor.cpp:45-61), fold count det(I + J_u) <= 0, and the
//                     per-label Dice counts (solver.cu:9-50) on the GPU
//   warp_kernel       apply_kernel (vector_fields.cu:81-99) on its own (warp2_kernel:
//                     the same, two voxels per thread, for aligned buffers)
#include "fr_common.cuh"
#include "fr_kernels.h"

namespace frg {

__global__ void __launch_bounds__(256) pack_init_kernel(IoArgs a) {
    for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x) {
        const Tile tl = a.tiles[t];
        const Pair P = a.pairs[tl.x];
        const PairIO io = a.io[tl.x];
        const int x = tl.y + (int)(threadIdx.x & 31), y = tl.z + (int)(threadIdx.x >> 5);
        if (x >= P.X || y >= P.Y) continue;
        const long long NT = a.NT;
        const int z1 = min(tl.w + kTileZ, P.Z);
        for (int z = tl.w; z < z1; ++z) {
            const long long u = user_lin(P, x, y, z);  // caller's layout
            const long long g = P.off + lin(P, x, y, z);
            a.S[g] = io.img_S[u];
            a.T[g] = io.img_T[u];
            a.labS[g] = io.lab_S[u];
            a.labT[g] = io.lab_T[u];
            if (a.sobolev) {
                if (!a.keep_state) {
                    const float pos[3] = {(float)x, (float)y, (float)z};
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        a.v0[c * NT + g] = 0.f;
                        a.psi[c * NT + g] = pos[c];
                    }
                }
                continue;
            }
            a.rho0[g] = a.rho_init;
            a.rho1[g] = a.rho_init;
            a.LT[g] = make_float4(0.f, 0.f, 0.f, io.img_T[u]);  // the Laplacian is 0 on the boundary
            if (!a.keep_state) {
                const float pos[3] = {(float)x, (float)y, (float)z};
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    a.v0[c * NT + g] = 0.f;
                    a.v1[c * NT + g] = 0.f;
                    a.psi[c * NT + g] = pos[c];
                    a.pinv0[c * NT + g] = pos[c];
                    a.pinv1[c * NT + g] = pos[c];
                }
            } else {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    a.v1[c * NT + g] = a.v0[c * NT + g];
                    a.pinv1[c * NT + g] = a.pinv0[c * NT + g];
                }
            }
        }
    }
}

// voxel nearest to a position clamped into the grid (round half up)
__device__ __forceinline__ long long nearest_index(const Pair& P, float px, float py, float pz) {
    const float cx = fminf(fmaxf(0.f, px), (float)(P.X - 1));
    const float cy = fminf(fmaxf(0.f, py), (float)(P.Y - 1));
    const float cz = fminf(fmaxf(0.f, pz), (float)(P.Z - 1));
    const int ix = min((int)floorf(cx + 0.5f), P.X - 1);
    const int iy = min((int)floorf(cy + 0.5f), P.Y - 1);
    const int iz = min((int)floorf(cz + 0.5f), P.Z - 1);
    return lin(P, ix, iy, iz);
}

// correct determinant of I + J (fixed evaluation order, mirrored by the oracle)
__device__ __forceinline__ float det_true(const float J[3][3]) {
    const float f00 = J[0][0] + 1.f, f11 = J[1][1] + 1.f, f22 = J[2][2] + 1.f;
    const float f01 = J[0][1], f02 = J[0][2], f10 = J[1][0], f12 = J[1][2], f20 = J[2][0], f21 = J[2][1];
    const float c0 = f11 * f22 - f12 * f21;
    const float c1 = f10 * f22 - f12 * f20;
    const float c2 = f10 * f21 - f11 * f20;
    return (f00 * c0 - f01 * c1) + f02 * c2;
}

__global__ void __launch_bounds__(256) finalize_kernel(IoArgs a) {
    __shared__ double red[32];
    __shared__ unsigned int hist[2 * 256 + 1];
    __shared__ bool last;
    const int tid = threadIdx.x;
    const int nbins = 2 * 256 + 1;
    for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x) {
        const Tile tl = a.tiles[t];
        const Pair P = a.pairs[tl.x];
        const PairIO io = a.io[tl.x];
        const int done = a.stop[tl.x] ? a.stop[tl.x] : a.max_iter;
        const float* __restrict__ pinv = (done & 1) ? a.pinv1 : a.pinv0;
        for (int b = tid; b < nbins; b += blockDim.x) hist[b] = 0u;
        __syncthreads();
        const int x = tl.y + (int)(threadIdx.x & 31), y = tl.z + (int)(threadIdx.x >> 5);
        double ed = 0.0, er = 0.0;
        long long folds = 0;
        if (x < P.X && y < P.Y) {
            const long long NT = a.NT;
            const float* __restrict__ S = a.S + P.off;
            const float* __restrict__ T = a.T + P.off;
            const int16_t* __restrict__ labS = a.labS + P.off;
            const int16_t* __restrict__ labT = a.labT + P.off;
            const float* __restrict__ psi = a.psi + P.off;
            const float* __restrict__ pi = pinv + P.off;
            const int z1 = min(tl.w + kTileZ, P.Z);
            for (int z = tl.w; z < z1; ++z) {
                const long long i = lin(P, x, y, z);
                // S o psi
                const Cell cs = locate(P, __ldg(psi + i), __ldg(psi + NT + i), __ldg(psi + 2 * NT + i));
                const float ws = tri_unchecked(S, P, cs);
                // floor-corner label (reference, cuda_utils.hpp:81) or the nearest
                // voxel (sobolev solver)
                const int16_t wl = a.sobolev ? __ldg(labS + nearest_index(P, __ldg(psi + i), __ldg(psi + NT + i),
                                                                          __ldg(psi + 2 * NT + i)))
                                             : __ldg(labS + cs.base);
                // T o psi_inv
                float wt;
                int16_t wtl;
                if (done == 0 || a.sobolev) {
                    wt = __ldg(T + i);
                    wtl = __ldg(labT + i);
                } else {
                    const Cell ct = locate(P, __ldg(pi + i), __ldg(pi + NT + i), __ldg(pi + 2 * NT + i));
                    wt = tri_unchecked(T, P, ct);
                    wtl = __ldg(labT + ct.base);
                }
                if (a.write_outputs) {
                    const long long u = user_lin(P, x, y, z);  // caller's layout
                    io.img_S[u] = ws;
                    io.lab_S[u] = wl;
                    io.img_T[u] = wt;
                    io.lab_T[u] = wtl;
                }

                // data energy
                const float df = __ldg(T + i) - ws;
                ed = fma((double)df, (double)df, ed);  // df * df is exact in FP64: same bits

                // deformation Jacobian with the mirrored one-sided boundary
                int x1 = x + 1, x2 = x - 1, y1 = y + 1, y2 = y - 1, z1_ = z + 1, z2_ = z - 1;
                if (x == 0) x2 = x + 1; else if (x == P.X - 1) x1 = x - 1;
                if (y == 0) y2 = y + 1; else if (y == P.Y - 1) y1 = y - 1;
                if (z == 0) z2_ = z + 1; else if (z == P.Z - 1) z1_ = z - 1;
                const long long ix1 = lin(P, x1, y, z), ix2 = lin(P, x2, y, z);
                const long long iy1 = lin(P, x, y1, z), iy2 = lin(P, x, y2, z);
                const long long iz1 = lin(P, x, y, z1_), iz2 = lin(P, x, y, z2_);
                const float cx1[3] = {(float)x1, (float)y, (float)z}, cx2[3] = {(float)x2, (float)y, (float)z};
                const float cy1[3] = {(float)x, (float)y1, (float)z}, cy2[3] = {(float)x, (float)y2, (float)z};
                const float cz1[3] = {(float)x, (float)y, (float)z1_}, cz2[3] = {(float)x, (float)y, (float)z2_};
                float J[3][3];
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    const float* __restrict__ Q = psi + r * NT;
                    J[r][0] = ((__ldg(Q + ix1) - cx1[r]) - (__ldg(Q + ix2) - cx2[r])) * 0.5f;
                    J[r][1] = ((__ldg(Q + iy1) - cy1[r]) - (__ldg(Q + iy2) - cy2[r])) * 0.5f;
                    J[r][2] = ((__ldg(Q + iz1) - cz1[r]) - (__ldg(Q + iz2) - cz2[r])) * 0.5f;
                }
                const float r0 = (J[0][0] * J[0][0] + J[0][1] * J[0][1]) + J[0][2] * J[0][2];
                const float r1 = (J[1][0] * J[1][0] + J[1][1] * J[1][1]) + J[1][2] * J[1][2];
                const float r2 = (J[2][0] * J[2][0] + J[2][1] * J[2][1]) + J[2][2] * J[2][2];
                er += (double)((r0 + r1) + r2);
                if (det_true(J) <= 0.f) folds++;

                // Dice counts on [0, X-1) x [0, Y-1) x [0, Z-1)
                if (x < P.X - 1 && y < P.Y - 1 && z < P.Z - 1) {
                    const int la = wl, lb = __ldg(labT + i);
                    const bool ok = la >= 0 && la < a.no_labels && lb >= 0 && lb < a.no_labels;
                    if (!ok) {
                        atomicAdd(&hist[2 * 256], 1u);
                    } else {
                        atomicAdd(&hist[256 + la], 1u);
                        atomicAdd(&hist[256 + lb], 1u);
                        if (la == lb) atomicAdd(&hist[la], 1u);
                    }
                }
            }
        }
        // per-tile partials (summed per pair in tile order by the last block)
        ed = block_sum_f64(ed, red);
        er = block_sum_f64(er, red);
        double fd = block_sum_f64((double)folds, red);
        if (tid == 0) {
            a.tile_partials[2 * (long long)t] = ed;
            a.tile_partials[2 * (long long)t + 1] = er;
            a.tile_folds[t] = (long long)fd;
        }
        unsigned long long* dice = a.dice + (long long)tl.x * nbins;
        for (int b = tid; b < nbins; b += blockDim.x)
            if (hist[b]) atomicAdd(dice + b, (unsigned long long)hist[b]);
        __syncthreads();
    }

    __threadfence();
    __syncthreads();
    if (tid == 0) last = (atomicAdd(a.counter, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!last) return;
    __threadfence();
    // a pair's tiles are contiguous (the table is ordered by pair): the whole block sums
    // them, each thread a fixed strided subset in order, then a fixed shuffle tree -- the
    // same sums on every run
    for (int p = 0; p < a.npairs; ++p) {
        double ed = 0.0, er = 0.0, f = 0.0;  // fold counts stay exact in FP64 (< 2^53)
        for (int t = a.pair_tiles[p] + tid; t < a.pair_tiles[p + 1]; t += blockDim.x) {
            ed += a.tile_partials[2 * (long long)t];
            er += a.tile_partials[2 * (long long)t + 1];
            f += (double)a.tile_folds[t];
        }
        ed = block_sum_f64(ed, red);
        er = block_sum_f64(er, red);
        f = block_sum_f64(f, red);
        if (tid == 0) {
            a.pair_energy[2 * p] = 0.5 * ed;
            a.pair_energy[2 * p + 1] = 0.5 * er;
            a.pair_folds[p] = (long long)f;
        }
    }
    if (tid == 0) *a.counter = 0u;
}

__global__ void __launch_bounds__(256) warp_kernel(const float* __restrict__ pos, const float* __restrict__ img,
                                                   const int16_t* __restrict__ lab, float* __restrict__ out,
                                                   int16_t* __restrict__ out_lab, Pair P) {
    const long long N = P.N;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
         i += (long long)gridDim.x * blockDim.x) {
        const Cell cl = locate(P, __ldg(pos + i), __ldg(pos + N + i), __ldg(pos + 2 * N + i));
        out[i] = tri_unchecked(img, P, cl);
        if (out_lab) out_lab[i] = __ldg(lab + cl.base);
    }
}

// Two consecutive voxels per thread (32-bit indices): 8-byte loads of the three position
// planes, issued one grid-stride item ahead so that they are in flight with the current
// item's 16 corner and 2 label loads; an 8-byte store of the intensities and a 4-byte
// store of the labels.  Positions and outputs are touched once and go through the cache as
// streaming (evict-first) accesses, leaving L1 and L2 to the corner gathers, which
// neighbouring voxels share.  Two voxels rather than four per thread: 40 registers and 48
// warps per SM instead of 64 registers and 32 warps, 0.0306 against 0.0372 ms on the
// 182x218x182 pair.  The caller guarantees N = X*Y*Z even and below 2^31 and 8-byte
// (pos, out) / 4-byte (out_lab) aligned buffers; per voxel the arithmetic is warp_kernel's
// (corners past the last voxel, of weight 0, clamped as tri_unchecked32 does).
__global__ void __launch_bounds__(256) warp2_kernel(const float* __restrict__ pos, const float* __restrict__ img,
                                                    const int16_t* __restrict__ lab, float* __restrict__ out,
                                                    int16_t* __restrict__ out_lab, int X, int Y, int Z) {
    const int N = X * Y * Z, N2 = N >> 1, XY = X * Y, last = N - 1;
    const float2* __restrict__ p2 = reinterpret_cast<const float2*>(pos);
    const int stride = gridDim.x * blockDim.x;
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    float2 npx = make_float2(0.f, 0.f), npy = npx, npz = npx;
    if (t < N2) {  // positions are read once: streaming loads, evicted first
        npx = __ldcs(p2 + t);
        npy = __ldcs(p2 + N2 + t);
        npz = __ldcs(p2 + 2 * N2 + t);
    }
    for (; t < N2; t += stride) {
        const float2 px = npx, py = npy, pz = npz;
        if (t + stride < N2) {  // the next item's positions load while this one's corners do
            npx = __ldcs(p2 + t + stride);
            npy = __ldcs(p2 + N2 + t + stride);
            npz = __ldcs(p2 + 2 * N2 + t + stride);
        }
        const float xs[2] = {px.x, px.y}, ys[2] = {py.x, py.y}, zs[2] = {pz.x, pz.y};
        Cell32 cl[2];
        float f[2][8];
        short lb[2];
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            cl[k] = locate32(X, Y, Z, X, xs[k], ys[k], zs[k]);
            const int b = cl[k].base;
            const int o[8] = {min(b + 1 + X + XY, last), min(b + 1 + X, last), min(b + 1 + XY, last), min(b + 1, last),
                              min(b + X + XY, last),     min(b + X, last),     min(b + XY, last),     b};
#pragma unroll
            for (int j = 0; j < 8; ++j) f[k][j] = __ldg(img + o[j]);
            if (out_lab) lb[k] = __ldg(lab + b);
        }
        // the two voxels as one packed pair, each lane with its own cell: per voxel exactly trilerp
        auto p = [&](int q) { return make_float2(f[0][q], f[1][q]); };
        const float2 v = trilerp2w(p(0), p(1), p(2), p(3), p(4), p(5), p(6), p(7), make_float2(cl[0].a, cl[1].a),
                                   make_float2(cl[0].b, cl[1].b), make_float2(cl[0].c, cl[1].c));
        __stcs(reinterpret_cast<float2*>(out) + t, v);  // written once
        if (out_lab) {
            short2 l;
            l.x = lb[0];
            l.y = lb[1];
            __stcs(reinterpret_cast<short2*>(out_lab) + t, l);
        }
    }
}

}  // namespace frg
