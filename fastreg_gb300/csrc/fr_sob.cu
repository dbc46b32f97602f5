// fr_sob.cu -- kernels of the sobolev solver (see fr_sob.h for the iteration).
//
// Launches per iteration: sob_grad_kernel (W, residual, exact trilinear gradient,
// FP64 data energy), three sob_smooth_kernel passes (x, y, then z fused with the
// momentum update), sob_pass_b_kernel (compositional update, max update norm,
// on-device convergence test).
#include <cmath>

#include "fr_common.cuh"
#include "fr_sob.h"

namespace frg {

void gaussian_taps(float sigma, int width, float* taps) {
    const int R = width / 2;
    double w[kMaxSmoothWidth];
    double sum = 0.0;
    for (int k = -R; k <= R; ++k) {
        w[k + R] = std::exp(-(double)k * (double)k / (2.0 * (double)sigma * (double)sigma));
        sum += w[k + R];
    }
    for (int k = 0; k < width; ++k) taps[k] = (float)(w[k] / sum);
}

// Cell for the sobolev solver: clamp to [0, dim-1], floor clamped to dim-2 so that
// both corners of every axis are inside the grid; clamped[axis] marks positions that
// were outside [0, dim-1] (their derivative along that axis is 0).
struct SobCell {
    long long base;
    float a, b, c;
    bool in_x, in_y, in_z;
};

__device__ __forceinline__ SobCell sob_locate(const Pair& P, float px, float py, float pz) {
    SobCell s;
    const float cx = fminf(fmaxf(0.f, px), (float)(P.X - 1));
    const float cy = fminf(fmaxf(0.f, py), (float)(P.Y - 1));
    const float cz = fminf(fmaxf(0.f, pz), (float)(P.Z - 1));
    const int gx = min((int)floorf(cx), P.X - 2);
    const int gy = min((int)floorf(cy), P.Y - 2);
    const int gz = min((int)floorf(cz), P.Z - 2);
    s.a = cx - (float)gx;
    s.b = cy - (float)gy;
    s.c = cz - (float)gz;
    s.in_x = px >= 0.f && px <= (float)(P.X - 1);
    s.in_y = py >= 0.f && py <= (float)(P.Y - 1);
    s.in_z = pz >= 0.f && pz <= (float)(P.Z - 1);
    s.base = lin(P, gx, gy, gz);
    return s;
}

__global__ void __launch_bounds__(256) sob_grad_kernel(SobIterArgs a) {
    __shared__ double red[32];
    for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x) {
        const Tile tl = a.tiles[t];
        if (a.stop[tl.x]) continue;  // uniform over the block
        const Pair P = a.pairs[tl.x];
        const int x = tl.y + (int)(threadIdx.x & 31), y = tl.z + (int)(threadIdx.x >> 5);
        double e = 0.0;
        if (x < P.X && y < P.Y) {
            const long long NT = a.NT, X = P.X, XY = (long long)P.X * P.Y;
            const float* __restrict__ S = a.S + P.off;
            const float* __restrict__ T = a.T + P.off;
            const float* __restrict__ phi = a.phi + P.off;
            float* g = a.g + P.off;
            const int z1 = min(tl.w + kSobTileZ, P.Z);
            for (int z = tl.w; z < z1; ++z) {
                const long long i = lin(P, x, y, z);
                const SobCell s = sob_locate(P, __ldg(phi + i), __ldg(phi + NT + i), __ldg(phi + 2 * NT + i));
                const long long b = s.base;
                const float f000 = __ldg(S + b), f100 = __ldg(S + b + 1);
                const float f010 = __ldg(S + b + X), f110 = __ldg(S + b + 1 + X);
                const float f001 = __ldg(S + b + XY), f101 = __ldg(S + b + 1 + XY);
                const float f011 = __ldg(S + b + X + XY), f111 = __ldg(S + b + 1 + X + XY);
                const float e11 = lerpf_(f111, f110, s.c), e10 = lerpf_(f101, f100, s.c);
                const float e01 = lerpf_(f011, f010, s.c), e00 = lerpf_(f001, f000, s.c);
                const float A1 = lerpf_(e11, e10, s.b), A0 = lerpf_(e01, e00, s.b);
                const float W = lerpf_(A1, A0, s.a);
                const float dWa = s.in_x ? A1 - A0 : 0.f;
                const float dWb = s.in_y ? lerpf_(e11 - e10, e01 - e00, s.a) : 0.f;
                const float dWc = s.in_z ? lerpf_(lerpf_(f111 - f110, f101 - f100, s.b),
                                                  lerpf_(f011 - f010, f001 - f000, s.b), s.a)
                                         : 0.f;
                const float r = W - __ldg(T + i);
                g[i] = r * dWa;
                g[NT + i] = r * dWb;
                g[2 * NT + i] = r * dWc;
                e += (double)r * (double)r;
            }
        }
        e = block_sum_f64(e, red);
        if (threadIdx.x == 0) atomicAdd(a.energy + (long long)(a.iter - 1) * a.npairs + tl.x, 0.5 * e);
    }
}

// One separable pass along `axis` (0 = x, 1 = y, 2 = z) with the replicate boundary;
// with `momentum` set the result gs updates m = damping * m - step * gs instead of
// being stored.
__global__ void __launch_bounds__(256) sob_smooth_kernel(SobIterArgs a, int axis, const float* src, float* dst,
                                                         int momentum) {
    for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x) {
        const Tile tl = a.tiles[t];
        if (a.stop[tl.x]) continue;
        const Pair P = a.pairs[tl.x];
        const int x = tl.y + (int)(threadIdx.x & 31), y = tl.z + (int)(threadIdx.x >> 5);
        if (x >= P.X || y >= P.Y) continue;
        const long long NT = a.NT;
        const int R = a.radius;
        const int z1 = min(tl.w + kSobTileZ, P.Z);
        const int dim = axis == 0 ? P.X : (axis == 1 ? P.Y : P.Z);
        const long long stride = axis == 0 ? 1 : (axis == 1 ? (long long)P.X : (long long)P.X * P.Y);
        for (int z = tl.w; z < z1; ++z) {
            const long long i = lin(P, x, y, z);
            const int pos = axis == 0 ? x : (axis == 1 ? y : z);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float* __restrict__ Sp = src + c * NT + P.off;
                float acc = 0.f;
                for (int k = -R; k <= R; ++k) {
                    const int q = min(max(pos + k, 0), dim - 1);
                    acc = acc + a.taps[k + R] * __ldg(Sp + i + (long long)(q - pos) * stride);
                }
                if (momentum) {
                    float* mp = dst + c * NT + P.off;
                    mp[i] = a.damping * mp[i] - a.step * acc;
                } else {
                    dst[c * NT + P.off + i] = acc;
                }
            }
        }
    }
}

__global__ void __launch_bounds__(256) sob_pass_b_kernel(SobIterArgs a) {
    __shared__ unsigned long long red[32];
    __shared__ bool last;
    for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x) {
        const Tile tl = a.tiles[t];
        if (a.stop[tl.x]) continue;
        const Pair P = a.pairs[tl.x];
        const int x = tl.y + (int)(threadIdx.x & 31), y = tl.z + (int)(threadIdx.x >> 5);
        unsigned long long best = 0ull;
        if (x < P.X && y < P.Y) {
            const long long NT = a.NT, X = P.X, XY = (long long)P.X * P.Y;
            float* phi = a.phi + P.off;
            const float* __restrict__ m = a.m + P.off;
            const int z1 = min(tl.w + kSobTileZ, P.Z);
            for (int z = tl.w; z < z1; ++z) {
                const long long i = lin(P, x, y, z);
                const float px = phi[i], py = phi[NT + i], pz = phi[2 * NT + i];
                const SobCell s = sob_locate(P, px, py, pz);
                float u[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float* __restrict__ F = m + c * NT;
                    const long long b = s.base;
                    u[c] = lerpf_(lerpf_(lerpf_(__ldg(F + b + 1 + X + XY), __ldg(F + b + 1 + X), s.c),
                                         lerpf_(__ldg(F + b + 1 + XY), __ldg(F + b + 1), s.c), s.b),
                                  lerpf_(lerpf_(__ldg(F + b + X + XY), __ldg(F + b + X), s.c),
                                         lerpf_(__ldg(F + b + XY), __ldg(F + b), s.c), s.b),
                                  s.a);
                }
                phi[i] = px + u[0];
                phi[NT + i] = py + u[1];
                phi[2 * NT + i] = pz + u[2];
                const float nrm = norm3_rd(u[0], u[1], u[2]);
                if (nrm == nrm) {
                    const unsigned long long k = norm_key(nrm, i);
                    best = k > best ? k : best;
                }
            }
        }
        const unsigned long long bm = block_max_u64(best, red);
        if (threadIdx.x == 0 && bm) atomicMax(a.keys + tl.x, bm);
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = (atomicAdd(a.counter, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!last) return;
    __threadfence();
    for (int p = threadIdx.x; p < a.npairs; p += blockDim.x) {
        if (a.stop[p]) continue;
        const unsigned long long k = atomicExch(a.keys + p, 0ull);
        a.trace[(long long)(a.iter - 1) * a.npairs + p] = k;
        const float mx = __uint_as_float((unsigned)(k >> 32));
        if (mx <= a.max_update_norm) a.stop[p] = a.iter;
    }
    if (threadIdx.x == 0) *a.counter = 0u;
}

cudaError_t launch_sob_iter(const SobIterArgs& a, const int* grids, cudaStream_t s, cudaEvent_t* ev) {
    if (ev) cudaEventRecord(ev[0], s);
    sob_grad_kernel<<<grids[0], 256, 0, s>>>(a);
    if (ev) cudaEventRecord(ev[1], s);
    sob_smooth_kernel<<<grids[1], 256, 0, s>>>(a, 0, a.g, a.tmp, 0);
    if (ev) cudaEventRecord(ev[2], s);
    sob_smooth_kernel<<<grids[1], 256, 0, s>>>(a, 1, a.tmp, a.g, 0);
    if (ev) cudaEventRecord(ev[3], s);
    sob_smooth_kernel<<<grids[1], 256, 0, s>>>(a, 2, a.g, a.m, 1);
    if (ev) cudaEventRecord(ev[4], s);
    sob_pass_b_kernel<<<grids[2], 256, 0, s>>>(a);
    if (ev) cudaEventRecord(ev[5], s);
    return cudaGetLastError();
}

}  // namespace frg
