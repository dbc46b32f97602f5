// fr_adjoint.cu -- the differentiated sobolev registration.
//
// J(v0, lambda) = 0.5 * sum (S(phi_K) - T)^2 + 0.1 * sum |m_K|^2 after K iterations of the
// sobolev solver (fr_sob.h) started from phi_0 = identity and m_0 = v0, with the
// displacement regulariser weighted by lambda:
//   g       = (S(phi) - T) dS(phi) + lambda * lap(phi - x)
//   m'      = damping * m - step * G g
//   phi'    = phi + m'(phi)
// The reverse sweep runs hand-written adjoint kernels for each line: the compositional
// update (gather of dm'/dphi, scatter-add into m'), the momentum, the transposed
// separable Gaussian (replicate boundary), the regulariser (the graph Laplacian is
// symmetric) and the data gradient (the trilinear interpolant's gradient and Hessian).
// Forward states are checkpointed every `checkpoint_every` iterations and each segment
// is recomputed before it is reversed.  Layout: one pair, planes of N voxels.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

#include "../../include/fastreg_gb300.h"
#include "fr_common.cuh"
#include "fr_limits.h"
#include "fr_sob.h"

namespace frg {

struct AdjDims {
    int X, Y, Z, XY, N;
};

struct TriEval {
    int off[8];
    float w[8];
    float val, d[3], H01, H02, H12;
    bool in[3];
};

__device__ __forceinline__ void sob_cell(const AdjDims& D, float px, float py, float pz, int& base, float& a,
                                         float& b, float& c, bool* in) {
    const float cx = fminf(fmaxf(0.f, px), (float)(D.X - 1));
    const float cy = fminf(fmaxf(0.f, py), (float)(D.Y - 1));
    const float cz = fminf(fmaxf(0.f, pz), (float)(D.Z - 1));
    const int gx = min((int)floorf(cx), D.X - 2), gy = min((int)floorf(cy), D.Y - 2), gz = min((int)floorf(cz), D.Z - 2);
    a = cx - (float)gx;
    b = cy - (float)gy;
    c = cz - (float)gz;
    in[0] = px >= 0.f && px <= (float)(D.X - 1);
    in[1] = py >= 0.f && py <= (float)(D.Y - 1);
    in[2] = pz >= 0.f && pz <= (float)(D.Z - 1);
    base = gx + D.X * (gy + D.Y * gz);
}

// value, masked gradient and (optionally) Hessian of the trilinear interpolant of F
__device__ __forceinline__ void tri_eval(const AdjDims& D, const float* __restrict__ F, float px, float py, float pz,
                                         TriEval& t, bool hessian) {
    int b;
    float a, bb, c;
    sob_cell(D, px, py, pz, b, a, bb, c, t.in);
    const int X = D.X, XY = D.XY;
    const int off[8] = {0, 1, X, 1 + X, XY, 1 + XY, X + XY, 1 + X + XY};
    float f[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        t.off[q] = b + off[q];
        f[q] = F ? __ldg(F + b + off[q]) : 0.f;
        const float wx = (q & 1) ? a : 1.f - a, wy = (q & 2) ? bb : 1.f - bb, wz = (q & 4) ? c : 1.f - c;
        t.w[q] = wx * wy * wz;
    }
    if (!F) return;
    const float f000 = f[0], f100 = f[1], f010 = f[2], f110 = f[3], f001 = f[4], f101 = f[5], f011 = f[6],
                f111 = f[7];
    const float e11 = lerpf_(f111, f110, c), e10 = lerpf_(f101, f100, c);
    const float e01 = lerpf_(f011, f010, c), e00 = lerpf_(f001, f000, c);
    const float A1 = lerpf_(e11, e10, bb), A0 = lerpf_(e01, e00, bb);
    t.val = lerpf_(A1, A0, a);
    const float d11 = f111 - f110, d10 = f101 - f100, d01 = f011 - f010, d00 = f001 - f000;
    t.d[0] = t.in[0] ? A1 - A0 : 0.f;
    t.d[1] = t.in[1] ? lerpf_(e11 - e10, e01 - e00, a) : 0.f;
    t.d[2] = t.in[2] ? lerpf_(lerpf_(d11, d10, bb), lerpf_(d01, d00, bb), a) : 0.f;
    if (!hessian) return;
    t.H01 = (t.in[0] && t.in[1]) ? (e11 - e10) - (e01 - e00) : 0.f;
    t.H02 = (t.in[0] && t.in[2]) ? lerpf_(d11, d10, bb) - lerpf_(d01, d00, bb) : 0.f;
    t.H12 = (t.in[1] && t.in[2]) ? lerpf_(d11 - d10, d01 - d00, a) : 0.f;
}

__device__ __forceinline__ void coords(const AdjDims& D, int i, int& x, int& y, int& z) {
    z = i / D.XY;
    const int r = i - z * D.XY;
    y = r / D.X;
    x = r - y * D.X;
}

// graph Laplacian of u = phi - x (neighbours inside the grid; order -x,+x,-y,+y,-z,+z)
__device__ __forceinline__ void lap_u(const AdjDims& D, const float* __restrict__ phi, int i, int x, int y, int z,
                                      float out[3]) {
    const bool ok[6] = {x > 0, x < D.X - 1, y > 0, y < D.Y - 1, z > 0, z < D.Z - 1};
    const int off[6] = {-1, 1, -D.X, D.X, -D.XY, D.XY};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float* P = phi + (long long)c * D.N;
        const float pc = __ldg(P + i);
        float acc = 0.f;
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            if (!ok[k]) continue;
            const float delta = (k / 2 == c) ? ((k & 1) ? 1.f : -1.f) : 0.f;
            acc = acc + ((pc - __ldg(P + i + off[k])) + delta);
        }
        out[c] = acc;
    }
}

#define GRID_STRIDE(i, n) for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += gridDim.x * blockDim.x)

// Grid-stride loop over whole warps: every lane of a warp runs the same iterations (lane
// i of a warp holds voxel base + i; `act` is false past the end), so the body may use
// warp shuffles.
#define WARP_STRIDE(i, act, n)                                                                  \
    for (int i##_w = blockIdx.x * blockDim.x + (threadIdx.x & ~31); i##_w < (n);                  \
         i##_w += gridDim.x * blockDim.x)                                                        \
        for (int i = i##_w + (threadIdx.x & 31), act = i < (n), i##_once = 1; i##_once; i##_once = 0)

// Scatter-add of one cell's eight corner contributions cw[q] (q: bit 0 x, bit 1 y, bit 2 z;
// the corners of tri_eval) into F, with the corners that neighbouring lanes share added
// once: the lanes of a warp hold consecutive voxels of a row, whose cells are usually
// consecutive along x (a smooth map), so lane k's x + 1 corners are lane k + 1's x corners.
// Lane k then adds lane k - 1's x + 1 contribution to its own x one (one atomic for both),
// halving the atomics of such runs.  All 32 lanes must call it; inactive lanes pass
// act = false.
__device__ __forceinline__ void scatter_cell_warp(float* F, int b, const float cw[8], bool act, int X, int XY) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int bprev = __shfl_up_sync(full, act ? b : -4, 1);
    const bool merge = act && lane > 0 && bprev == b - 1;
    const bool next_merges = __shfl_down_sync(full, (int)merge, 1) != 0 && lane < 31;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int o = ((j & 1) ? X : 0) + ((j & 2) ? XY : 0);
        const float c0 = cw[2 * j], c1 = cw[2 * j + 1];
        const float c1prev = __shfl_up_sync(full, c1, 1);
        if (act) {
            atomicAdd(F + b + o, merge ? c0 + c1prev : c0);
            if (!next_merges) atomicAdd(F + b + 1 + o, c1);
        }
    }
}

// ---- forward (same arithmetic as the cohort kernels and the oracle) ----
__global__ void adj_fwd_grad_kernel(AdjDims D, const float* __restrict__ S, const float* __restrict__ T,
                                    const float* __restrict__ phi, float lambda, float* __restrict__ g) {
    GRID_STRIDE(i, D.N) {
        int x, y, z;
        coords(D, i, x, y, z);
        TriEval t;
        tri_eval(D, S, __ldg(phi + i), __ldg(phi + D.N + i), __ldg(phi + 2 * D.N + i), t, false);
        const float r = t.val - __ldg(T + i);
        float lap[3];
        lap_u(D, phi, i, x, y, z, lap);
#pragma unroll
        for (int c = 0; c < 3; ++c) g[(long long)c * D.N + i] = (r * t.d[c]) + (lambda * lap[c]);
    }
}

// one separable pass of radius R (fma taps, replicate boundary); momentum: dst =
// damping*dst - step*acc
template <int R>
__global__ void adj_fwd_smooth_kernel(AdjDims D, SobIterArgs a, int axis, const float* __restrict__ src, float* dst,
                                      int momentum) {
    const int dim = axis == 0 ? D.X : (axis == 1 ? D.Y : D.Z);
    const int stride = axis == 0 ? 1 : (axis == 1 ? D.X : D.XY);
    GRID_STRIDE(i, D.N) {
        int x, y, z;
        coords(D, i, x, y, z);
        const int pos = axis == 0 ? x : (axis == 1 ? y : z);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float* Sp = src + (long long)c * D.N;
            float acc = 0.f;
#pragma unroll
            for (int k = -R; k <= R; ++k) {
                const int q = min(max(pos + k, 0), dim - 1);
                acc = fmaf(a.taps[k + R], __ldg(Sp + i + (q - pos) * stride), acc);
            }
            float* dp = dst + (long long)c * D.N + i;
            *dp = momentum ? a.damping * *dp - a.step * acc : acc;
        }
    }
}

__global__ void adj_fwd_update_kernel(AdjDims D, const float* __restrict__ m, float* phi) {
    GRID_STRIDE(i, D.N) {
        const float p[3] = {phi[i], phi[D.N + i], phi[2 * D.N + i]};
        float u[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            TriEval t;
            tri_eval(D, m + (long long)c * D.N, p[0], p[1], p[2], t, false);
            u[c] = t.val;
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) phi[(long long)c * D.N + i] = p[c] + u[c];
    }
}

// ---- loss and the adjoint seeds ----
__global__ void adj_loss_kernel(AdjDims D, const float* __restrict__ S, const float* __restrict__ T,
                                const float* __restrict__ phi, const float* __restrict__ m, float* pbar, float* mbar,
                                double* loss) {
    __shared__ double red[32];
    double e = 0.0;
    GRID_STRIDE(i, D.N) {
        TriEval t;
        tri_eval(D, S, __ldg(phi + i), __ldg(phi + D.N + i), __ldg(phi + 2 * D.N + i), t, false);
        const float r = t.val - __ldg(T + i);
        e = fma(0.5 * (double)r, (double)r, e);  // (r / 2) * r is exact in FP64: same bits
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float mc = __ldg(m + (long long)c * D.N + i);
            e += 0.1 * (double)mc * (double)mc;
            pbar[(long long)c * D.N + i] = r * t.d[c];
            mbar[(long long)c * D.N + i] = 0.2f * mc;
        }
    }
    e = block_sum_f64(e, red);
    if (threadIdx.x == 0) atomicAdd(loss, e);
}

// phi' = phi + m'(phi): pbar_k = pbar + (dm'/dphi)^T pbar, mbar += scatter(w * pbar), the
// scatter warp-aggregated (scatter_cell_warp)
__global__ void adj_update_kernel(AdjDims D, const float* __restrict__ phi, const float* __restrict__ mn,
                                  const float* __restrict__ pbar, float* pbar_k, float* mbar) {
    WARP_STRIDE(i, act, D.N) {
        const int k = act ? i : 0;
        const float p[3] = {__ldg(phi + k), __ldg(phi + D.N + k), __ldg(phi + 2 * D.N + k)};
        float acc[3] = {__ldg(pbar + k), __ldg(pbar + D.N + k), __ldg(pbar + 2 * D.N + k)};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            TriEval t;
            tri_eval(D, mn + (long long)c * D.N, p[0], p[1], p[2], t, false);
            const float pb = __ldg(pbar + (long long)c * D.N + k);
#pragma unroll
            for (int j = 0; j < 3; ++j) acc[j] += pb * t.d[j];
            float cw[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) cw[q] = t.w[q] * pb;
            scatter_cell_warp(mbar + (long long)c * D.N, t.off[0], cw, act, D.X, D.XY);
        }
        if (act)
#pragma unroll
            for (int j = 0; j < 3; ++j) pbar_k[(long long)j * D.N + i] = acc[j];
    }
}

// m' = damping * m - step * gs: gsbar = -step * mbar, mbar_k = damping * mbar
__global__ void adj_momentum_kernel(AdjDims D, float damping, float step, float* mbar, float* gsbar) {
    GRID_STRIDE(i, 3 * D.N) {
        const float mb = mbar[i];
        gsbar[i] = -step * mb;
        mbar[i] = damping * mb;
    }
}

// transpose of one replicate-boundary pass of radius R, gather form: dst(y) = sum over x
// of src(x) * sum_k w_k [clamp(x + k) == y]
template <int R>
__global__ void adj_smooth_t_kernel(AdjDims D, SobIterArgs a, int axis, const float* __restrict__ src, float* dst) {
    const int dim = axis == 0 ? D.X : (axis == 1 ? D.Y : D.Z);
    const int stride = axis == 0 ? 1 : (axis == 1 ? D.X : D.XY);
    GRID_STRIDE(i, D.N) {
        int x, y, z;
        coords(D, i, x, y, z);
        const int pos = axis == 0 ? x : (axis == 1 ? y : z);
        float acc[3] = {0.f, 0.f, 0.f};
        if (pos >= R && pos <= dim - 1 - R) {
            // clamped taps land only on the first and last position: inside, the weight of
            // s = pos + j is the single tap at -j (the sum below with one nonzero term)
#pragma unroll
            for (int j = -R; j <= R; ++j) {
                const float w = a.taps[R - j];
#pragma unroll
                for (int c = 0; c < 3; ++c) acc[c] += w * __ldg(src + (long long)c * D.N + i + j * stride);
            }
        } else if (pos >= 1 && pos <= dim - 2) {
            for (int s = max(pos - R, 0); s <= min(pos + R, dim - 1); ++s) {
                const float w = a.taps[pos - s + R];
#pragma unroll
                for (int c = 0; c < 3; ++c) acc[c] += w * __ldg(src + (long long)c * D.N + i + (s - pos) * stride);
            }
        } else {
            for (int s = max(pos - R, 0); s <= min(pos + R, dim - 1); ++s) {
                float w = 0.f;
                for (int k = -R; k <= R; ++k)
                    if (min(max(s + k, 0), dim - 1) == pos) w += a.taps[k + R];
                if (w == 0.f) continue;
#pragma unroll
                for (int c = 0; c < 3; ++c) acc[c] += w * __ldg(src + (long long)c * D.N + i + (s - pos) * stride);
            }
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) dst[(long long)c * D.N + i] = acc[c];
    }
}

// g = (S(phi) - T) dS(phi) + lambda lap(phi - x): pbar_k += lambda lap^T(gbar)
// + (gbar . dS) dS + r H gbar; lambda_bar += gbar . lap
__global__ void adj_grad_kernel(AdjDims D, const float* __restrict__ S, const float* __restrict__ T,
                                const float* __restrict__ phi, float lambda, const float* __restrict__ gbar,
                                float* pbar_k, double* lbar) {
    __shared__ double red[32];
    double lb = 0.0;
    GRID_STRIDE(i, D.N) {
        int x, y, z;
        coords(D, i, x, y, z);
        float lap[3];
        lap_u(D, phi, i, x, y, z, lap);
        const float gb[3] = {__ldg(gbar + i), __ldg(gbar + D.N + i), __ldg(gbar + 2 * D.N + i)};
#pragma unroll
        for (int c = 0; c < 3; ++c) lb += (double)gb[c] * (double)lap[c];
        const bool ok[6] = {x > 0, x < D.X - 1, y > 0, y < D.Y - 1, z > 0, z < D.Z - 1};
        const int off[6] = {-1, 1, -D.X, D.X, -D.XY, D.XY};
        float add[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int k = 0; k < 6; ++k)
                if (ok[k]) add[c] += lambda * (gb[c] - __ldg(gbar + (long long)c * D.N + i + off[k]));
        TriEval t;
        tri_eval(D, S, __ldg(phi + i), __ldg(phi + D.N + i), __ldg(phi + 2 * D.N + i), t, true);
        const float r = t.val - __ldg(T + i);
        const float gd = (gb[0] * t.d[0] + gb[1] * t.d[1]) + gb[2] * t.d[2];
        const float h[3] = {gb[1] * t.H01 + gb[2] * t.H02, gb[0] * t.H01 + gb[2] * t.H12, gb[0] * t.H02 + gb[1] * t.H12};
#pragma unroll
        for (int j = 0; j < 3; ++j) pbar_k[(long long)j * D.N + i] += add[j] + (gd * t.d[j] + r * h[j]);
    }
    lb = block_sum_f64(lb, red);
    if (threadIdx.x == 0) atomicAdd(lbar, lb);
}

__global__ void adj_identity_kernel(AdjDims D, float* phi) {
    GRID_STRIDE(i, D.N) {
        int x, y, z;
        coords(D, i, x, y, z);
        phi[i] = (float)x;
        phi[D.N + i] = (float)y;
        phi[2 * D.N + i] = (float)z;
    }
}

// one separable pass (transposed: the adjoint's) with the radius as a template argument
template <int R>
void launch_smooth_r(bool transposed, int grid, cudaStream_t s, const AdjDims& D, const SobIterArgs& a, int axis,
                     const float* src, float* dst, int momentum) {
    if (transposed)
        adj_smooth_t_kernel<R><<<grid, 256, 0, s>>>(D, a, axis, src, dst);
    else
        adj_fwd_smooth_kernel<R><<<grid, 256, 0, s>>>(D, a, axis, src, dst, momentum);
}

void launch_smooth(int radius, bool transposed, int grid, cudaStream_t s, const AdjDims& D, const SobIterArgs& a,
                   int axis, const float* src, float* dst, int momentum) {
    switch (radius) {
        case 0: launch_smooth_r<0>(transposed, grid, s, D, a, axis, src, dst, momentum); break;
        case 1: launch_smooth_r<1>(transposed, grid, s, D, a, axis, src, dst, momentum); break;
        case 2: launch_smooth_r<2>(transposed, grid, s, D, a, axis, src, dst, momentum); break;
        case 3: launch_smooth_r<3>(transposed, grid, s, D, a, axis, src, dst, momentum); break;
        case 4: launch_smooth_r<4>(transposed, grid, s, D, a, axis, src, dst, momentum); break;
        case 5: launch_smooth_r<5>(transposed, grid, s, D, a, axis, src, dst, momentum); break;
        case 6: launch_smooth_r<6>(transposed, grid, s, D, a, axis, src, dst, momentum); break;
        default: launch_smooth_r<7>(transposed, grid, s, D, a, axis, src, dst, momentum); break;
    }
}

}  // namespace frg

namespace {

struct AdjBuffers {
    float* block = nullptr;
    size_t floats = 0;
};

// The device workspace of fr_sobolev_loss_grad (checkpoints, segment states and adjoint
// fields, about 40 fields of 3 N floats for 50 iterations), kept per device and reused by
// later calls that need as much or less: an unrolled registration is typically
// differentiated many times in a row (hypergradient steps), and a fresh cudaMalloc /
// cudaFree of a gigabyte per call costs milliseconds and synchronises the device.  A call
// that finds the workspace busy (another host thread's call on the same device) uses a
// private allocation instead.
std::mutex g_ws_mu;
struct Workspace {
    float* ptr = nullptr;
    size_t floats = 0;
    bool busy = false;
};
Workspace g_ws[64];

// a workspace of at least `floats` floats on device `dev`; *cached says whether it is the
// shared one (released with release_workspace) or private (freed by the caller)
float* acquire_workspace(int dev, size_t floats, bool* cached) {
    *cached = false;
    if (dev >= 0 && dev < 64) {
        std::lock_guard<std::mutex> lk(g_ws_mu);
        Workspace& w = g_ws[dev];
        if (!w.busy) {
            if (w.floats < floats) {
                if (w.ptr) cudaFree(w.ptr);
                w.ptr = nullptr;
                w.floats = 0;
                if (cudaMalloc((void**)&w.ptr, floats * sizeof(float)) == cudaSuccess)
                    w.floats = floats;
                else {
                    cudaGetLastError();
                    w.ptr = nullptr;
                }
            }
            if (w.ptr) {
                w.busy = true;
                *cached = true;
                return w.ptr;
            }
        }
    }
    float* p = nullptr;
    if (cudaMalloc((void**)&p, floats * sizeof(float)) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return p;
}

void release_workspace(int dev, float* p, bool cached) {
    if (!cached) {
        cudaFree(p);
        return;
    }
    std::lock_guard<std::mutex> lk(g_ws_mu);
    g_ws[dev].busy = false;
}

int grid_for(long long n) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long long want = (n + 255) / 256;
    return (int)std::max(1LL, std::min<long long>(want, (long long)std::max(sms, 1) * 8));
}

}  // namespace

namespace frg {
void set_global_error(const char* msg);
}

extern "C" int fr_sobolev_loss_grad(const float* d_T, const float* d_S, const int dims[3], const float* d_v0,
                                    float lambda, int iters, int checkpoint_every, float damping, float step,
                                    float smooth_sigma, int smooth_width, double* loss, float* d_grad_v0,
                                    double* grad_lambda, void* stream) {
    using namespace frg;
    set_global_error("");
    if (!d_T || !d_S || !dims || !d_v0 || !loss) {
        set_global_error("fr_sobolev_loss_grad: NULL argument");
        return FR_ERR_INVALID_ARG;
    }
    if (dims[0] < 4 || dims[1] < 4 || dims[2] < 4 || iters < 1 || checkpoint_every < 1 || smooth_width < 1 ||
        smooth_width > kMaxSmoothWidth || (smooth_width & 1) == 0 || !(smooth_sigma > 0.f)) {
        set_global_error("fr_sobolev_loss_grad: invalid size or parameter");
        return FR_ERR_INVALID_ARG;
    }
    const long long N64 = (long long)dims[0] * dims[1] * dims[2];
    if (N64 > (1LL << 30)) {
        set_global_error("fr_sobolev_loss_grad: volume too large (limit 2^30 voxels)");
        return FR_ERR_INVALID_ARG;
    }
    AdjDims D{dims[0], dims[1], dims[2], dims[0] * dims[1], (int)N64};
    const size_t N = (size_t)N64, N3 = 3 * N;
    const int K = iters, ck = std::min(checkpoint_every, iters);
    const int nck = (K + ck - 1) / ck + 1;
    cudaStream_t s = (cudaStream_t)stream;
    SobIterArgs a{};
    gaussian_taps(smooth_sigma, smooth_width, a.taps);
    a.radius = smooth_width / 2;
    a.damping = damping;
    a.step = step;
    // buffers: checkpoints (phi, m) x nck, segment states (phi_k, m_{k+1}) x ck, working phi, m,
    // g, tmp, adjoint pbar, pbar_k, mbar, gbar (+ 2 doubles)
    const size_t floats = N3 * (2 * nck + 2 * ck + 8) + 64;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        set_global_error("fr_sobolev_loss_grad: no current CUDA device");
        return FR_ERR_CUDA;
    }
    bool cached = false;
    float* blk = acquire_workspace(dev, floats, &cached);
    if (!blk) {
        set_global_error("fr_sobolev_loss_grad: device allocation failed");
        return FR_ERR_ALLOC;
    }
    float* ckpt = blk;                          // [nck][2][3N]
    float* seg = ckpt + N3 * 2 * nck;          // [ck][2][3N]
    float* phi = seg + N3 * 2 * ck;
    float* m = phi + N3;
    float* g = m + N3;
    float* tmp = g + N3;
    float* pbar = tmp + N3;
    float* pbar_k = pbar + N3;
    float* mbar = pbar_k + N3;
    float* gbar = mbar + N3;
    double* dd = (double*)(((uintptr_t)(gbar + N3) + 15) & ~(uintptr_t)15);  // loss, lambda_bar
    const int grid = grid_for(N64);
    int rc = FR_OK;
    auto fwd_step = [&]() {
        adj_fwd_grad_kernel<<<grid, 256, 0, s>>>(D, d_S, d_T, phi, lambda, g);
        launch_smooth(a.radius, false, grid, s, D, a, 0, g, tmp, 0);
        launch_smooth(a.radius, false, grid, s, D, a, 1, tmp, g, 0);
        launch_smooth(a.radius, false, grid, s, D, a, 2, g, m, 1);
        adj_fwd_update_kernel<<<grid, 256, 0, s>>>(D, m, phi);
    };
    auto copy = [&](float* dst, const float* src) {
        return cudaMemcpyAsync(dst, src, N3 * sizeof(float), cudaMemcpyDeviceToDevice, s);
    };
    do {
        if (cudaMemsetAsync(dd, 0, 2 * sizeof(double), s) != cudaSuccess) { rc = FR_ERR_CUDA; break; }
        adj_identity_kernel<<<grid, 256, 0, s>>>(D, phi);
        if (copy(m, d_v0) != cudaSuccess) { rc = FR_ERR_CUDA; break; }
        // forward with checkpoints every ck iterations
        for (int k = 0; k < K; ++k) {
            if (k % ck == 0) {
                copy(ckpt + N3 * 2 * (k / ck), phi);
                copy(ckpt + N3 * (2 * (k / ck) + 1), m);
            }
            fwd_step();
        }
        adj_loss_kernel<<<grid, 256, 0, s>>>(D, d_S, d_T, phi, m, pbar, mbar, dd);
        if (!d_grad_v0) break;
        // reverse, one segment at a time
        for (int s0 = ((K - 1) / ck) * ck; s0 >= 0; s0 -= ck) {
            const int s1 = std::min(s0 + ck, K);
            copy(phi, ckpt + N3 * 2 * (s0 / ck));
            copy(m, ckpt + N3 * (2 * (s0 / ck) + 1));
            for (int k = s0; k < s1; ++k) {
                copy(seg + N3 * 2 * (k - s0), phi);  // phi_k
                fwd_step();
                copy(seg + N3 * (2 * (k - s0) + 1), m);  // m_{k+1}
            }
            for (int k = s1 - 1; k >= s0; --k) {
                const float* phik = seg + N3 * 2 * (k - s0);
                const float* mn = seg + N3 * (2 * (k - s0) + 1);
                adj_update_kernel<<<grid, 256, 0, s>>>(D, phik, mn, pbar, pbar_k, mbar);
                adj_momentum_kernel<<<grid, 256, 0, s>>>(D, damping, step, mbar, g);
                launch_smooth(a.radius, true, grid, s, D, a, 2, g, tmp, 0);
                launch_smooth(a.radius, true, grid, s, D, a, 1, tmp, g, 0);
                launch_smooth(a.radius, true, grid, s, D, a, 0, g, gbar, 0);
                adj_grad_kernel<<<grid, 256, 0, s>>>(D, d_S, d_T, phik, lambda, gbar, pbar_k, dd + 1);
                std::swap(pbar, pbar_k);
            }
        }
        if (copy(d_grad_v0, mbar) != cudaSuccess) { rc = FR_ERR_CUDA; break; }
    } while (0);
    double host[2] = {0.0, 0.0};
    if (rc == FR_OK) {
        if (cudaGetLastError() != cudaSuccess || cudaMemcpyAsync(host, dd, sizeof host, cudaMemcpyDeviceToHost, s) !=
                                                     cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            rc = FR_ERR_CUDA;
    }
    if (rc != FR_OK) cudaStreamSynchronize(s);  // nothing may still use the workspace
    release_workspace(dev, blk, cached);
    if (rc != FR_OK) {
        cudaGetLastError();
        set_global_error("fr_sobolev_loss_grad: a CUDA call failed");
        return rc;
    }
    *loss = host[0];
    if (grad_lambda) *grad_lambda = host[1];
    return FR_OK;
}

extern "C" int fr_warp_adjoint(const float* d_pos, const float* d_img, const float* d_wbar, const int dims[3],
                               float* d_pos_bar, float* d_img_bar, void* stream);

namespace frg {
__global__ void warp_adjoint_kernel(AdjDims D, const float* __restrict__ pos, const float* __restrict__ img,
                                    const float* __restrict__ wbar, float* pos_bar, float* img_bar) {
    WARP_STRIDE(i, act, D.N) {
        const int k = act ? i : 0;
        TriEval t;
        tri_eval(D, img, __ldg(pos + k), __ldg(pos + D.N + k), __ldg(pos + 2 * D.N + k), t, false);
        const float wb = __ldg(wbar + k);
        if (pos_bar && act)
#pragma unroll
            for (int j = 0; j < 3; ++j) pos_bar[(long long)j * D.N + i] = wb * t.d[j];
        if (img_bar) {  // uniform: every lane calls the warp scatter
            float cw[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) cw[q] = t.w[q] * wb;
            scatter_cell_warp(img_bar, t.off[0], cw, act, D.X, D.XY);
        }
    }
}
}  // namespace frg

extern "C" int fr_warp_adjoint(const float* d_pos, const float* d_img, const float* d_wbar, const int dims[3],
                               float* d_pos_bar, float* d_img_bar, void* stream) {
    using namespace frg;
    set_global_error("");
    if (!d_pos || !d_img || !d_wbar || !dims || (!d_pos_bar && !d_img_bar)) {
        set_global_error("fr_warp_adjoint: NULL argument");
        return FR_ERR_INVALID_ARG;
    }
    if (dims[0] < 2 || dims[1] < 2 || dims[2] < 2 || !frg::fits_index32(dims[0], dims[1], dims[2])) {
        set_global_error("fr_warp_adjoint: invalid dims (each >= 2, N + 2 X Y + 2 X + 2 <= 2^31-1)");
        return FR_ERR_INVALID_ARG;
    }
    AdjDims D{dims[0], dims[1], dims[2], dims[0] * dims[1], dims[0] * dims[1] * dims[2]};
    cudaStream_t s = (cudaStream_t)stream;
    if (d_img_bar && cudaMemsetAsync(d_img_bar, 0, sizeof(float) * (size_t)D.N, s) != cudaSuccess) {
        cudaGetLastError();
        set_global_error("fr_warp_adjoint: memset failed");
        return FR_ERR_CUDA;
    }
    warp_adjoint_kernel<<<grid_for(D.N), 256, 0, s>>>(D, d_pos, d_img, d_wbar, d_pos_bar, d_img_bar);
    if (cudaGetLastError() != cudaSuccess) {
        set_global_error("fr_warp_adjoint: launch failed");
        return FR_ERR_CUDA;
    }
    return FR_OK;
}
