// fr_sob.cu -- kernels of the sobolev solver (see fr_sob.h for the iteration).
//
// Launches per iteration: sob_grad_kernel (W, residual, exact trilinear gradient,
// FP64 data energy), sob_smooth3_kernel (separable Gaussian along x, y, z fused with
// the momentum update), sob_pass_b_kernel (compositional update, max update norm,
// on-device convergence test).
#include <cmath>

#include "fr_common.cuh"
#include "fr_kernels.h"
#include "fr_sob.h"
#include "fr_tma.cuh"

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
    int gx, gy, gz;
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
    s.gx = gx;
    s.gy = gy;
    s.gz = gz;
    s.base = lin(P, gx, gy, gz);
    return s;
}

// W = S o phi, r = W - T, the exact trilinear gradient of the interpolant, the graph
// Laplacian of u = phi - x and the FP64 data energy.  A block owns a 32 x 8 column tile
// and marches z: phi's three components (tile rows plus a 1-voxel halo) and T are staged
// slice by slice into a shared-memory ring by 16-byte cp.async kGAhead slices ahead of the
// compute; the eight corners of S are gathered through L1.
namespace {
constexpr int kGAhead = 2;        // slices in flight ahead of the one computed
constexpr int kGS = 3 + kGAhead;  // ring slots: slices z - 1, z, z + 1 and those in flight
constexpr int kGW = kStageW, kGPlane = kGW * (kTileY + 2), kGTPlane = kTileX * kTileY;
}  // namespace

size_t sob_grad_smem_bytes() { return sizeof(float) * kGS * (3 * kGPlane + kGTPlane); }

__global__ void __launch_bounds__(256) sob_grad_kernel(SobIterArgs a) {
    extern __shared__ __align__(16) float ring[];  // phi [3][kGS][10][kGW], then T [kGS][8][32]
    float* tring = ring + 3 * kGS * kGPlane;
    __shared__ double red[32];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int t = blockIdx.x; t < a.ntiles_g; t += gridDim.x) {
        const Tile tl = a.tiles_g[t];
        if (a.stop[tl.x]) continue;  // uniform over the block
        const Pair P = a.pairs[tl.x];
        const int Y = P.Y, Z = P.Z, Xp = P.Xp, XYp = P.Xp * P.Y;  // strides of the packed arrays
        const long long NT = a.NT;
        const float* __restrict__ S = a.S + P.off;
        const float* __restrict__ Tg = a.T + P.off;
        const float* __restrict__ Fg[3] = {a.phi + P.off, a.phi + NT + P.off, a.phi + 2 * NT + P.off};
        float* G[3] = {a.g + P.off, a.g + NT + P.off, a.g + 2 * NT + P.off};
        const int x = tl.y + tx, y = tl.z + ty;
        const bool inside = x < P.X && y < Y;
        const int z0 = tl.w, z1 = min(tl.w + a.depth_g, Z);
        const int gq = stage_offset<1>(threadIdx.x, Y, Xp, tl.y, tl.z);
        // T: thread e < 64 copies chunk e & 7 of tile row e >> 3 (x0 is a multiple of 32)
        const int tr = (int)threadIdx.x >> 3, tk = (int)threadIdx.x & 7;
        const int gt = (threadIdx.x < 64 && tl.z + tr < Y && tl.y + 4 * tk < Xp) ? Xp * (tl.z + tr) + tl.y + 4 * tk
                                                                                 : -1;
        auto stage = [&](int zs, int sl) {  // slice zs of phi (and T) into slot sl
            if (zs < 0 || zs >= Z) return;
            if (gq >= 0) {
                float* dst = ring + sl * kGPlane + 4 * threadIdx.x;
                const int off = gq + XYp * zs;
#pragma unroll
                for (int c = 0; c < 3; ++c) cp_async16(dst + c * kGS * kGPlane, Fg[c] + off);
            }
            if (gt >= 0) cp_async16(tring + sl * kGTPlane + 4 * threadIdx.x, Tg + gt + XYp * zs);
        };
        double e = 0.0;
        __syncthreads();  // the previous tile is done with the ring
        // prologue: slices z0 - 1 .. z0 + 1 (one group), then one group per slice ahead
        stage(z0 - 1, 0);
        stage(z0, 1);
        stage(z0 + 1, 2);
        cp_async_commit();
#pragma unroll
        for (int k = 1; k < kGAhead; ++k) {
            if (z0 + 1 + k <= z1) stage(z0 + 1 + k, 2 + k);
            cp_async_commit();
        }
        int sm = 0;  // slot of slice z - 1 (z, z + 1 follow it in the ring)
        const int c0 = (ty + 1) * kGW + tx + kStageXO;
        for (int z = z0; z < z1; ++z) {
            cp_async_wait<kGAhead - 1>();  // slice z + 1 has landed ...
            __syncthreads();               // ... for every thread, and slice z - 2's slot is free
            {
                int sl = sm + 2 + kGAhead;  // the slot of slice z - 2
                sl = sl >= kGS ? sl - kGS : sl;
                if (z + 1 + kGAhead <= z1) stage(z + 1 + kGAhead, sl);  // reads reach z1
                cp_async_commit();
            }
            const int s0 = sm + 1 >= kGS ? sm + 1 - kGS : sm + 1;
            const int sp = s0 + 1 >= kGS ? s0 + 1 - kGS : s0 + 1;
            if (inside) {
                const int i = x + Xp * y + XYp * z;
                const float* q[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) q[c] = ring + (c * kGS + s0) * kGPlane + c0;
                const SobCell s = sob_locate(P, q[0][0], q[1][0], q[2][0]);
                const int b = (int)s.base;
                const float f000 = __ldg(S + b), f100 = __ldg(S + b + 1);
                const float f010 = __ldg(S + b + Xp), f110 = __ldg(S + b + 1 + Xp);
                const float f001 = __ldg(S + b + XYp), f101 = __ldg(S + b + 1 + XYp);
                const float f011 = __ldg(S + b + Xp + XYp), f111 = __ldg(S + b + 1 + Xp + XYp);
                // graph Laplacian of u = phi - x, neighbours inside the grid, order -x,+x,-y,+y,-z,+z
                // (shared-memory work placed between the corner loads and their use)
                const bool ok[6] = {x > 0, x < P.X - 1, y > 0, y < Y - 1, z > 0, z < Z - 1};
                float lap[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float* qc = q[c];
                    const float* qm = ring + (c * kGS + sm) * kGPlane + c0;
                    const float* qp = ring + (c * kGS + sp) * kGPlane + c0;
                    const float pc = qc[0];
                    const float nb[6] = {qc[-1], qc[1], qc[-kGW], qc[kGW], qm[0], qp[0]};
                    float acc = 0.f;
#pragma unroll
                    for (int k = 0; k < 6; ++k) {
                        if (!ok[k]) continue;
                        const float delta = (k / 2 == c) ? ((k & 1) ? 1.f : -1.f) : 0.f;
                        acc = acc + ((pc - nb[k]) + delta);
                    }
                    lap[c] = acc;
                }
                const float e11 = lerpf_(f111, f110, s.c), e10 = lerpf_(f101, f100, s.c);
                const float e01 = lerpf_(f011, f010, s.c), e00 = lerpf_(f001, f000, s.c);
                const float A1 = lerpf_(e11, e10, s.b), A0 = lerpf_(e01, e00, s.b);
                const float W = lerpf_(A1, A0, s.a);
                const float dWa = s.in_x ? A1 - A0 : 0.f;
                const float dWb = s.in_y ? lerpf_(e11 - e10, e01 - e00, s.a) : 0.f;
                const float dWc = s.in_z ? lerpf_(lerpf_(f111 - f110, f101 - f100, s.b),
                                                  lerpf_(f011 - f010, f001 - f000, s.b), s.a)
                                         : 0.f;
                const float r = W - tring[s0 * kGTPlane + ty * kTileX + tx];
                G[0][i] = (r * dWa) + (P.w_reg * lap[0]);
                G[1][i] = (r * dWb) + (P.w_reg * lap[1]);
                G[2][i] = (r * dWc) + (P.w_reg * lap[2]);
                e = fma((double)r, (double)r, e);  // r * r is exact in FP64: one DFMA, same bits
            }
            sm = s0;
        }
        cp_async_wait<0>();
        e = block_sum_f64(e, red);
        if (threadIdx.x == 0) atomicAdd(a.energy + (long long)(a.iter - 1) * a.npairs + tl.x, 0.5 * e);
    }
}

// The same gradient with TMA staging: per slice one thread copies phi's box (40 columns
// x 10 rows x 3 components: the tile and a 1-voxel halo; out-of-volume parts read as zero
// and are masked by the grid-neighbour tests) and T's 32 x 8 box with two tensor copies
// into a six-slot ring, completing on the slot's mbarrier; three slices are in flight
// ahead of the one computed.  Waits are bounded as in ref_laplacian_tma_kernel.
namespace {
constexpr int kGBAhead = 3;
constexpr int kGBS = 3 + kGBAhead;
constexpr int kGBW = 40, kGBPlane = kGBW * 10;  // phi box row and plane (floats)
constexpr int kGBTOff = 1216;                   // T box offset in a slot (floats, 128-byte aligned)
constexpr int kGBSlot = kGBTOff + kTileX * kTileY;
constexpr unsigned kGBBytes = sizeof(float) * (3 * kGBPlane + kTileX * kTileY);
static_assert(3 * kGBPlane <= kGBTOff && (kGBSlot * 4) % 128 == 0, "slot layout");
}  // namespace

size_t sob_grad_tma_smem_bytes() { return 128 + sizeof(float) * kGBS * kGBSlot + sizeof(uint64_t) * kGBS; }

__global__ void __launch_bounds__(256) sob_grad_tma_kernel(SobIterArgs a) {
    extern __shared__ __align__(128) unsigned char grad_raw[];
    float* ring = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(grad_raw) + 127) & ~uintptr_t(127));
    uint64_t* full = reinterpret_cast<uint64_t*>(ring + kGBS * kGBSlot);
    __shared__ double red[32];
    typedef SliceRing<kGBS> Ring;
    const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
    if (tid == 0) {
        for (int k = 0; k < kGBS; ++k) mbar_init(full + k, 1);
        mbar_fence_init();
    }
    __syncthreads();
    unsigned nbase = 0, issued = 0;
    bool failed = false;
    for (int t = blockIdx.x; t < a.ntiles_g && !failed; t += gridDim.x) {
        const Tile tl = a.tiles_g[t];
        if (a.stop[tl.x]) continue;  // uniform over the block
        const Pair P = a.pairs[tl.x];
        const int Y = P.Y, Z = P.Z, Xp = P.Xp, XYp = P.Xp * P.Y;
        const long long NT = a.NT;
        const float* __restrict__ S = a.S + P.off;
        float* G[3] = {a.g + P.off, a.g + NT + P.off, a.g + 2 * NT + P.off};
        const CUtensorMap* mphi = a.tmaps + (long long)tl.x * TM_COUNT + TM_LAP_PSI;
        const CUtensorMap* mT = a.tmaps + (long long)tl.x * TM_COUNT + TM_LAP_T;
        const int x = tl.y + tx, y = tl.z + ty;
        const bool inside = x < P.X && y < Y;
        const int z0 = tl.w, z1 = min(tl.w + a.depth_g, Z);
        const int nsl = z1 - z0 + 2;  // slices z0 - 1 .. z1 (outside the volume: zeros, unused)
        auto issue = [&](int j) {
            const unsigned n = nbase + (unsigned)j;
            float* dst = ring + Ring::slot(n) * kGBSlot;
            uint64_t* bar = full + Ring::slot(n);
            mbar_arrive_expect_tx(bar, kGBBytes);
            tma_load_4d(dst, mphi, tl.y - 4, tl.z - 1, z0 - 1 + j, 0, bar);
            tma_load_3d(dst + kGBTOff, mT, tl.y, tl.z, z0 - 1 + j, bar);
            ++issued;
        };
        double e = 0.0;
        __syncthreads();  // the previous tile is done with the ring
        if (tid == 0) {
            tma_prefetch_map(mphi);
            tma_prefetch_map(mT);
            for (int j = 0; j < min(nsl, kGBS); ++j) issue(j);
        }
        const int c0 = (ty + 1) * kGBW + tx + 4;
        for (int j0 = 0; j0 + 2 < nsl; ++j0) {
            bool ok = true;
            for (int j = (j0 == 0 ? 0 : j0 + 2); j <= j0 + 2; ++j)
                ok = ok && mbar_wait_bounded(full + Ring::slot(nbase + j), Ring::parity(nbase + j));
            if (__syncthreads_or(!ok)) {
                failed = true;
                break;
            }
            if (tid == 0 && j0 >= 1 && j0 - 1 + kGBS < nsl) issue(j0 - 1 + kGBS);
            if (inside) {
                const int z = z0 + j0;
                const int i = x + Xp * y + XYp * z;
                const float* qm = ring + Ring::slot(nbase + j0) * kGBSlot + c0;
                const float* q0 = ring + Ring::slot(nbase + j0 + 1) * kGBSlot;
                const float* qp = ring + Ring::slot(nbase + j0 + 2) * kGBSlot + c0;
                const SobCell s = sob_locate(P, q0[c0], q0[c0 + kGBPlane], q0[c0 + 2 * kGBPlane]);
                const int b = (int)s.base;
                const float f000 = __ldg(S + b), f100 = __ldg(S + b + 1);
                const float f010 = __ldg(S + b + Xp), f110 = __ldg(S + b + 1 + Xp);
                const float f001 = __ldg(S + b + XYp), f101 = __ldg(S + b + 1 + XYp);
                const float f011 = __ldg(S + b + Xp + XYp), f111 = __ldg(S + b + 1 + Xp + XYp);
                const bool okn[6] = {x > 0, x < P.X - 1, y > 0, y < Y - 1, z > 0, z < Z - 1};
                float lap[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float* qc = q0 + c0 + c * kGBPlane;
                    const float pc = qc[0];
                    const float nb[6] = {qc[-1], qc[1], qc[-kGBW], qc[kGBW], qm[c * kGBPlane], qp[c * kGBPlane]};
                    float acc = 0.f;
#pragma unroll
                    for (int k = 0; k < 6; ++k) {
                        if (!okn[k]) continue;
                        const float delta = (k / 2 == c) ? ((k & 1) ? 1.f : -1.f) : 0.f;
                        acc = acc + ((pc - nb[k]) + delta);
                    }
                    lap[c] = acc;
                }
                const float e11 = lerpf_(f111, f110, s.c), e10 = lerpf_(f101, f100, s.c);
                const float e01 = lerpf_(f011, f010, s.c), e00 = lerpf_(f001, f000, s.c);
                const float A1 = lerpf_(e11, e10, s.b), A0 = lerpf_(e01, e00, s.b);
                const float W = lerpf_(A1, A0, s.a);
                const float dWa = s.in_x ? A1 - A0 : 0.f;
                const float dWb = s.in_y ? lerpf_(e11 - e10, e01 - e00, s.a) : 0.f;
                const float dWc = s.in_z ? lerpf_(lerpf_(f111 - f110, f101 - f100, s.b),
                                                  lerpf_(f011 - f010, f001 - f000, s.b), s.a)
                                         : 0.f;
                const float r = W - q0[kGBTOff + ty * kTileX + tx];
                G[0][i] = (r * dWa) + (P.w_reg * lap[0]);
                G[1][i] = (r * dWb) + (P.w_reg * lap[1]);
                G[2][i] = (r * dWc) + (P.w_reg * lap[2]);
                e = fma((double)r, (double)r, e);  // r * r is exact in FP64: one DFMA, same bits
            }
        }
        nbase += (unsigned)nsl;
        if (failed) break;
        e = block_sum_f64(e, red);
        if (threadIdx.x == 0) atomicAdd(a.energy + (long long)(a.iter - 1) * a.npairs + tl.x, 0.5 * e);
    }
    if (failed && tid == 0) {
        for (unsigned n = (issued > (unsigned)kGBS ? issued - kGBS : 0u); n < issued; ++n)
            mbar_wait_bounded(full + Ring::slot(n), Ring::parity(n));
        atomicOr(a.err, kErrTmaTimeout);
    }
}

// The x pass of one staged slice: the K-tap filter along x of each of its 3 H staged rows
// (WS columns; column s holds x = x0 - HX + s) into 32 outputs per row of Gx.  Task (row rr,
// group gq) computes outputs 4 gq .. 4 gq + 3 of row rr from 1 + HX / 2 aligned 16-byte
// shared-memory loads (one load per tap and output before).  Thread e of the 256 takes
// tasks e + 256 j, whose group is e & 7 and whose offsets in a staged slice and in Gx do not
// change within a tile, so they are computed once per tile (init) rather than per slice.
// On a tile at an x edge the columns beyond the edges hold the edge column's value by the
// time the x pass reads them (fix_edges: the replicate boundary).  Each output is the chain
// acc = fma(w_q, g_q, acc), q = 0 .. K - 1.
template <int R>
struct SmoothXPass {
    static constexpr int HX = (R + 3) / 4 * 4, WS = kTileX + 2 * HX, H = kSobTileY + 2 * R, K = 2 * R + 1;
    static constexpr int NQ = 1 + HX / 2, NV = 4 * NQ;  // loads and values per task
    static constexpr int NTASK = 3 * H * (kTileX / 4), NJ = (NTASK + 255) / 256;
    static_assert(HX - R + 3 + K - 1 < NV, "a task's taps lie in its loads");
    int src[NJ];  // offset of task j's first load in a staged slice (-1: no task j)
    int dst[NJ];  // offset of its four outputs in Gx

    // row_off(rr): offset in a staged slice of the row that Gx row rr filters
    template <typename RowOff>
    __device__ __forceinline__ void init(RowOff row_off) {
        const int gq = threadIdx.x & 7;
#pragma unroll
        for (int j = 0; j < NJ; ++j) {
            const int task = threadIdx.x + 256 * j, rr = task >> 3;
            src[j] = task < NTASK ? row_off(rr) + 4 * gq : -1;
            dst[j] = rr * kTileX + 4 * gq;
        }
    }

    __device__ __forceinline__ void run(const SobIterArgs& a, const float* __restrict__ slice,
                                        float* __restrict__ gx) const {
#pragma unroll
        for (int j = 0; j < NJ; ++j) {
            if (src[j] < 0) continue;
            const float* p = slice + src[j];
            float v[NV];
#pragma unroll
            for (int u = 0; u < NQ; ++u) {
                const float4 f = *reinterpret_cast<const float4*>(p + 4 * u);
                v[4 * u] = f.x;
                v[4 * u + 1] = f.y;
                v[4 * u + 2] = f.z;
                v[4 * u + 3] = f.w;
            }
            float out[4];
#pragma unroll
            for (int o = 0; o < 4; ++o) {
                float acc = 0.f;
#pragma unroll
                for (int q = 0; q < K; ++q) acc = fmaf(a.taps[q], v[o + HX - R + q], acc);
                out[o] = acc;
            }
            *reinterpret_cast<float4*>(gx + dst[j]) = make_float4(out[0], out[1], out[2], out[3]);
        }
    }

    // The replicate boundary written into a staged slice of a tile at an x edge.  Outputs
    // outside [0, X) are never stored, so only the R staged columns beyond each edge that
    // outputs inside it read need the edge value: x = -R .. -1 take x = 0's, x = X .. X - 1 + R
    // take x = X - 1's.  One (row, side, column) item per thread, 3 H * 2 R items (252 at
    // R = 3); the other staged columns outside the volume keep whatever the copy left there
    // and reach only outputs that are discarded.  The edge columns are only read, so the
    // threads need no ordering among themselves; the block barrier that precedes the
    // slice's x pass orders the writes before it.
    __device__ __forceinline__ static void fix_edges(float* slice, int x0, int X) {
        if constexpr (R > 0) {
            constexpr int NW = 3 * H * 2 * R;
            const bool left = x0 == 0;        // x0 is a multiple of 32 and HX <= 8
            const int shi = X - 1 - x0 + HX;  // column of x = X - 1
#pragma unroll
            for (int w0 = 0; w0 < NW; w0 += 256) {
                const int w = w0 + (int)threadIdx.x;
                if (w < NW) {
                    const int rr = w / (2 * R), k = w - rr * (2 * R);
                    float* row = slice + rr * WS;
                    if (k < R) {
                        if (left) row[HX - R + k] = row[HX];
                    } else {
                        const int c = shi + 1 + (k - R);
                        if (c < WS) row[c] = row[shi];
                    }
                }
            }
            // these generic-proxy writes come before the copy that next refills the buffer
            // (a tensor copy writes through the async proxy)
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        }
    }
};

// Separable Gaussian smoothing of g along x, y and z with the replicate boundary,
// fused with the momentum update m = damping * m - step * gs.  A block owns a 32 x 8
// column tile and marches z.  Each input slice (the tile's rows plus an R halo, clamped
// into the volume; columns x0 - HX .. x0 + 31 + HX with HX = R rounded up to 4) is staged
// in shared memory by 16-byte cp.async NB slices ahead (NB = 3 buffers, 2 for wide
// kernels, so that the block stays within 48 KB of shared memory).  Per slice step one block
// barrier separates two independent halves: the x pass of the next slice (shared memory
// to a double-buffered Gx) and the y pass of this slice (Gx to a per-thread register ring
// of 2R + 1 slices that the z pass reads).  On tiles at the x edges the R columns beyond
// each edge are overwritten with the edge column in shared memory between two barriers
// before the slice's x pass (the replicate boundary; SmoothXPass::fix_edges).  Each tap is
// one fused multiply-add, acc = fma(w_k, g_k, acc), taken in the order k = -R..R for every
// axis.  Resident blocks per SM the kernel is held to: as many as its (2R + 1)-slice ring
// allows without spilling much (5 blocks are 48 registers a thread, 4 are 64, 3 are 85).
template <int R>
constexpr int kSmoothMinBlocksCp = R <= 4 ? 5 : 4;

template <int R>
__global__ void __launch_bounds__(256, kSmoothMinBlocksCp<R>) sob_smooth3_kernel(SobIterArgs a) {
    constexpr int HX = (R + 3) / 4 * 4;                // staged x halo: whole 16-byte chunks
    constexpr int WS = kTileX + 2 * HX, C = WS / 4;    // staged row: floats, chunks
    constexpr int H = kSobTileY + 2 * R, K = 2 * R + 1;
    constexpr int NB = 4 * (3 * 3 * H * WS + 2 * 3 * H * kTileX) <= 48 * 1024 ? 3 : 2;  // staging buffers
    constexpr int NF = 3 * H * C;                      // chunks of one staged slice
    constexpr int NJ = (NF + 255) / 256;               // chunks per thread
    __shared__ __align__(16) float G[NB][3][H][WS];
    __shared__ __align__(16) float Gx[2][3][H][kTileX];
    const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;

    for (int t = blockIdx.x; t < a.ntiles_s; t += gridDim.x) {
        const Tile tl = a.tiles_s[t];
        if (a.stop[tl.x]) continue;  // uniform over the block
        const Pair P = a.pairs[tl.x];
        const int X = P.X, Y = P.Y, Z = P.Z, Xp = P.Xp, XY = P.Xp * P.Y;
        const long long NT = a.NT;
        const float* __restrict__ g0 = a.g + P.off;
        float* m[3] = {a.m + P.off, a.m + NT + P.off, a.m + 2 * NT + P.off};
        const int x0 = tl.y, y0 = tl.z, zt0 = tl.w, zt1 = min(tl.w + a.depth_s, Z);
        const int nsl = (zt1 - zt0) + 2 * R;
        const bool xedge = x0 - R < 0 || x0 + kTileX - 1 + R > X - 1;  // uniform over the block

        // chunk f = tid + 256 j of a staged slice is (component c, row r, chunk k); its
        // shared-memory offset is 4 f floats and its offset inside a slice of component c
        // is fixed for the tile (-1: the chunk lies outside the padded row, never read)
        int goff[NJ];
#pragma unroll
        for (int j = 0; j < NJ; ++j) {
            const int f = tid + 256 * j;
            goff[j] = -1;
            if (f < NF) {
                const int c = f / (H * C), rem = f - c * (H * C), r = rem / C, k = rem - r * C;
                const int gy = min(max(y0 - R + r, 0), Y - 1), xs = x0 - HX + 4 * k;
                if (xs >= 0 && xs < Xp) goff[j] = Xp * gy + xs;
            }
        }
        auto stage = [&](int k) {  // staged slice k of the tile (z = zt0 - R + k, clamped)
            if (k >= nsl) return;
            const long long zoff = (long long)XY * min(max(zt0 - R + k, 0), Z - 1);
            float* dst = &G[k % NB][0][0][0];
#pragma unroll
            for (int j = 0; j < NJ; ++j) {
                const int f = tid + 256 * j;
                if (goff[j] >= 0) cp_async16(dst + 4 * f, g0 + (f / (H * C)) * NT + zoff + goff[j]);
            }
        };
        SmoothXPass<R> xp;  // staged rows are already the clamped rows
        xp.init([](int rr) { return rr * WS; });
        auto x_pass = [&](int k) {  // staged slice k -> Gx[k & 1]
            xp.run(a, &G[k % NB][0][0][0], &Gx[k & 1][0][0][0]);
        };
        // on a tile at an x edge: slice k's edge columns, after the barrier that made every
        // thread's copies of it visible, and a second barrier before its x pass (block-uniform)
        auto fix_edges = [&](int k) {
            if (!xedge) return;
            SmoothXPass<R>::fix_edges(&G[k % NB][0][0][0], x0, X);
            __syncthreads();
        };

        // this thread's column; its momentum is loaded one output slice ahead
        const int x = x0 + tx, y = y0 + ty, col = x + Xp * y;
        const bool inside = x < X && y < Y;
        float mv[3] = {0.f, 0.f, 0.f};
        if (inside)
#pragma unroll
            for (int c = 0; c < 3; ++c) mv[c] = m[c][col + XY * zt0];

        float2 ring01[K];  // the z ring of the y-pass results: components 0 and 1 packed, 2
        float ring2[K];
        // zeroed: the shift below copies every slot from the first step on, before the slots
        // near the end are filled, and a copy of an indeterminate value is undefined behaviour
        // (a build at 48 registers turned it into wrong results)
#pragma unroll
        for (int q = 0; q < K; ++q) {
            ring01[q] = make_float2(0.f, 0.f);
            ring2[q] = 0.f;
        }
        __syncthreads();  // the previous tile is done with G and Gx
#pragma unroll
        for (int k = 0; k < NB; ++k) {
            stage(k);
            cp_async_commit();
        }
        cp_async_wait<NB - 1>();  // slice 0 has landed
        __syncthreads();
        fix_edges(0);
        x_pass(0);
        for (int k = 0; k < nsl; ++k) {
            cp_async_wait<NB - 2>();  // slice k + 1 has landed (the later ones may not)
            __syncthreads();          // ... for every thread; Gx[k & 1] is complete; slice k's buffer
                                      // and Gx[(k + 1) & 1] are no longer read
            stage(k + NB);            // into slice k's buffer
            cp_async_commit();
            if (k + 1 < nsl) {
                fix_edges(k + 1);
                x_pass(k + 1);
            }
            // y pass of slice k for this thread's column, pushed into the z ring
#pragma unroll
            for (int q = 0; q < K - 1; ++q) {
                ring01[q] = ring01[q + 1];
                ring2[q] = ring2[q + 1];
            }
            {  // components 0 and 1 as one packed pair: per lane the same fused multiply-adds
                float2 acc01 = make_float2(0.f, 0.f);
                float acc2 = 0.f;
#pragma unroll
                for (int q = 0; q < K; ++q) {
                    const float w = a.taps[q];
                    acc01 = __ffma2_rn(make_float2(w, w),
                                       make_float2(Gx[k & 1][0][ty + q][tx], Gx[k & 1][1][ty + q][tx]), acc01);
                    acc2 = fmaf(w, Gx[k & 1][2][ty + q][tx], acc2);
                }
                ring01[K - 1] = acc01;
                ring2[K - 1] = acc2;
            }
            // z pass and momentum for slice zt0 + k - 2R once the ring holds its 2R + 1 slices
            const int zo = zt0 - 2 * R + k;
            if (k >= 2 * R && inside) {
                const int i = col + XY * zo;
                float2 acc01 = make_float2(0.f, 0.f);
                float acc2 = 0.f;
#pragma unroll
                for (int q = 0; q < K; ++q) {
                    const float w = a.taps[q];
                    acc01 = __ffma2_rn(make_float2(w, w), ring01[q], acc01);
                    acc2 = fmaf(w, ring2[q], acc2);
                }
                const float accs[3] = {acc01.x, acc01.y, acc2};
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float acc = accs[c];
                    const float mo = mv[c];
                    if (zo + 1 < zt1) mv[c] = m[c][i + XY];  // the next output slice's momentum
                    m[c][i] = a.damping * mo - a.step * acc;
                }
            }
        }
        cp_async_wait<0>();
    }
}

// The same smoothing with TMA staging: each input slice (3 components of the tile's rows
// plus an R halo and columns x0 - HX .. x0 + 31 + HX) is one tensor copy, issued by one
// thread NT - 1 slices ahead into a ring of NT buffers and completed on the buffer's
// mbarrier.  Rows and slices outside the volume realise the replicate boundary: a slice
// beyond an end is requested at the clamped z, and the x pass reads, for each staged row,
// the row of the clamped y (inside the box whenever the tile is inside the volume); along x,
// the R columns beyond each edge are overwritten with the edge column in shared memory
// once the slice has landed (SmoothXPass::fix_edges), so the x pass runs without selects.
// Waits are bounded as in ref_laplacian_tma_kernel.  Held to 5 resident blocks per SM up
// to R = 4 and 4 above.
template <int R>
constexpr int kSmoothMinBlocks = R <= 4 ? 5 : 4;

template <int R>
__global__ void __launch_bounds__(256, kSmoothMinBlocks<R>) sob_smooth3_tma_kernel(SobIterArgs a) {
    constexpr int HX = (R + 3) / 4 * 4;
    constexpr int WS = kTileX + 2 * HX;
    constexpr int H = kSobTileY + 2 * R, K = 2 * R + 1;
    constexpr int BOX = 3 * H * WS;                    // floats copied per slice
    constexpr int BSTRIDE = (BOX + 31) / 32 * 32;      // buffer stride: 128-byte multiple
    // buffers: as many (up to 4) as keep the block's static shared memory within 48 KB
    constexpr int NT = 4 * (4 * BSTRIDE + 2 * 3 * H * kTileX) + 32 <= 48 * 1024   ? 4
                       : 4 * (3 * BSTRIDE + 2 * 3 * H * kTileX) + 24 <= 48 * 1024 ? 3
                                                                                  : 2;
    __shared__ __align__(128) float G[NT][BSTRIDE];
    __shared__ __align__(16) float Gx[2][3][H][kTileX];
    __shared__ __align__(8) uint64_t full[NT];
    typedef SliceRing<NT> Ring;
    const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
    if (tid == 0) {
        for (int k = 0; k < NT; ++k) mbar_init(full + k, 1);
        mbar_fence_init();
    }
    __syncthreads();
    unsigned nbase = 0, issued = 0;
    bool failed = false;

    for (int t = blockIdx.x; t < a.ntiles_s && !failed; t += gridDim.x) {
        const Tile tl = a.tiles_s[t];
        if (a.stop[tl.x]) continue;  // uniform over the block
        const Pair P = a.pairs[tl.x];
        const int X = P.X, Y = P.Y, Z = P.Z, Xp = P.Xp, XY = P.Xp * P.Y;
        const long long NTv = a.NT;
        float* m[3] = {a.m + P.off, a.m + NTv + P.off, a.m + 2 * NTv + P.off};
        const CUtensorMap* mg = a.tmaps + (long long)tl.x * TM_COUNT + TM_SOB_G;
        const int x0 = tl.y, y0 = tl.z, zt0 = tl.w, zt1 = min(tl.w + a.depth_s, Z);
        const int nsl = (zt1 - zt0) + 2 * R;
        const bool xedge = x0 - R < 0 || x0 + kTileX - 1 + R > X - 1;  // uniform over the block
        auto issue = [&](int k) {  // staged slice k of the tile (z = zt0 - R + k, clamped)
            const unsigned n = nbase + (unsigned)k;
            uint64_t* bar = full + Ring::slot(n);
            mbar_arrive_expect_tx(bar, sizeof(float) * BOX);
            tma_load_4d(&G[Ring::slot(n)][0], mg, x0 - HX, y0 - R, min(max(zt0 - R + k, 0), Z - 1), 0, bar);
            ++issued;
        };
        SmoothXPass<R> xp;  // staged row rr holds row r of component c; the filter reads the clamped row
        xp.init([&](int rr) {
            const int c = rr / H, r = rr - c * H;
            const int rs = min(max(y0 - R + r, 0), Y - 1) - (y0 - R);
            return (c * H + rs) * WS;
        });
        auto x_pass = [&](int k) {  // staged slice k -> Gx[k & 1] (its edge columns already fixed)
            xp.run(a, &G[Ring::slot(nbase + (unsigned)k)][0], &Gx[k & 1][0][0][0]);
        };
        auto fix_edges = [&](int k) {  // after slice k has landed, before the barrier that precedes its x pass
            if (xedge) SmoothXPass<R>::fix_edges(&G[Ring::slot(nbase + (unsigned)k)][0], x0, X);
        };
        auto wait = [&](int k) {
            return mbar_wait_bounded(full + Ring::slot(nbase + (unsigned)k), Ring::parity(nbase + (unsigned)k));
        };

        const int x = x0 + tx, y = y0 + ty, col = x + Xp * y;
        const bool inside = x < X && y < Y;
        float mv[3] = {0.f, 0.f, 0.f};
        if (inside)
#pragma unroll
            for (int c = 0; c < 3; ++c) mv[c] = m[c][col + XY * zt0];

        float2 ring01[K];  // the z ring of the y-pass results: components 0 and 1 packed, 2
        float ring2[K];
        // zeroed: the shift below copies every slot from the first step on, before the slots
        // near the end are filled, and a copy of an indeterminate value is undefined behaviour
        // (a build at 48 registers turned it into wrong results)
#pragma unroll
        for (int q = 0; q < K; ++q) {
            ring01[q] = make_float2(0.f, 0.f);
            ring2[q] = 0.f;
        }
        __syncthreads();  // the previous tile is done with G and Gx
        if (tid == 0) {
            tma_prefetch_map(mg);
            for (int k = 0; k < min(NT, nsl); ++k) issue(k);
        }
        const bool ok0 = wait(0);  // slice 0 has landed
        if (ok0) fix_edges(0);
        if (__syncthreads_or(!ok0)) {
            failed = true;
            break;
        }
        x_pass(0);
        for (int k = 0; k < nsl; ++k) {
            const bool ok = k + 1 < nsl ? wait(k + 1) : true;  // slice k + 1 has landed
            if (ok && k + 1 < nsl) fix_edges(k + 1);           // nobody reads its buffer before the barrier
            // every thread is past step k - 1: Gx[k & 1] is complete, slice k's buffer and
            // Gx[(k + 1) & 1] are no longer read, slice k + 1's edge columns are written; and
            // the block agrees on the waits
            if (__syncthreads_or(!ok)) {
                failed = true;
                break;
            }
            if (tid == 0 && k + NT < nsl) issue(k + NT);  // into slice k's buffer
            if (k + 1 < nsl) x_pass(k + 1);
#pragma unroll
            for (int q = 0; q < K - 1; ++q) {
                ring01[q] = ring01[q + 1];
                ring2[q] = ring2[q + 1];
            }
            {  // components 0 and 1 as one packed pair: per lane the same fused multiply-adds
                float2 acc01 = make_float2(0.f, 0.f);
                float acc2 = 0.f;
#pragma unroll
                for (int q = 0; q < K; ++q) {
                    const float w = a.taps[q];
                    acc01 = __ffma2_rn(make_float2(w, w),
                                       make_float2(Gx[k & 1][0][ty + q][tx], Gx[k & 1][1][ty + q][tx]), acc01);
                    acc2 = fmaf(w, Gx[k & 1][2][ty + q][tx], acc2);
                }
                ring01[K - 1] = acc01;
                ring2[K - 1] = acc2;
            }
            const int zo = zt0 - 2 * R + k;
            if (k >= 2 * R && inside) {
                const int i = col + XY * zo;
                float2 acc01 = make_float2(0.f, 0.f);
                float acc2 = 0.f;
#pragma unroll
                for (int q = 0; q < K; ++q) {
                    const float w = a.taps[q];
                    acc01 = __ffma2_rn(make_float2(w, w), ring01[q], acc01);
                    acc2 = fmaf(w, ring2[q], acc2);
                }
                const float accs[3] = {acc01.x, acc01.y, acc2};
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float acc = accs[c];
                    const float mo = mv[c];
                    if (zo + 1 < zt1) mv[c] = m[c][i + XY];
                    m[c][i] = a.damping * mo - a.step * acc;
                }
            }
        }
        nbase += (unsigned)nsl;
    }
    if (failed && tid == 0) {
        for (unsigned n = (issued > (unsigned)NT ? issued - NT : 0u); n < issued; ++n)
            mbar_wait_bounded(full + Ring::slot(n), Ring::parity(n));
        atomicOr(a.err, kErrTmaTimeout);
    }
}

// phi += m o phi with the max update norm.  Held to 48 registers for 5 resident blocks
// per SM (0.098 against 0.101 ms with 63 registers and 4 blocks): the kernel waits on its
// corner loads, and more resident warps keep more of them in flight.
__global__ void __launch_bounds__(256, 5) sob_pass_b_kernel(SobIterArgs a) {
    __shared__ unsigned long long red[32];
    __shared__ bool last;
    for (int t = blockIdx.x; t < a.ntiles_b; t += gridDim.x) {
        const Tile tl = a.tiles_b[t];
        if (a.stop[tl.x]) continue;
        const Pair P = a.pairs[tl.x];
        const int x = tl.y + (int)(threadIdx.x & 31), y = tl.z + (int)(threadIdx.x >> 5);
        unsigned long long best = 0ull;
        if (x < P.X && y < P.Y) {
            const long long NT = a.NT;
            const int X = P.Xp, XY = P.Xp * P.Y;  // strides of the packed arrays
            float* phi[3] = {a.phi + P.off, a.phi + NT + P.off, a.phi + 2 * NT + P.off};
            const float* __restrict__ mc[3] = {a.m + P.off, a.m + NT + P.off, a.m + 2 * NT + P.off};
            const int z1 = min(tl.w + a.depth_b, P.Z);
            int i = x + X * y + XY * tl.w;
            // phi of the next slice is loaded while this slice's gathers are in flight
            float nx = phi[0][i], ny = phi[1][i], nz = phi[2][i];
            for (int z = tl.w; z < z1; ++z, i += XY) {
                const float px = nx, py = ny, pz = nz;
                if (z + 1 < z1) {
                    nx = phi[0][i + XY];
                    ny = phi[1][i + XY];
                    nz = phi[2][i + XY];
                }
                const SobCell s = sob_locate(P, px, py, pz);
                {  // L2 prefetch: the m rows the next slice's cell adds (phi is smooth, so that
                   // cell is about this one plus a slice) and phi two slices on
                    const int N = (int)P.N, o0 = min((int)s.base + 2 * XY, N - 1);
                    const int o1 = min((int)s.base + 2 * XY + X, N - 1);
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        prefetch_l2(mc[c] + o0);
                        prefetch_l2(mc[c] + o1);
                    }
                    if (z + 2 < P.Z)
#pragma unroll
                        for (int c = 0; c < 3; ++c) prefetch_l2(phi[c] + i + 2 * XY);
                }
                float u[3];
                {  // components 0 and 1 interpolated as one packed pair (trilerp3)
                    const int b = (int)s.base;
                    float f[3][8];
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const float* __restrict__ F = mc[c];
                        f[c][0] = __ldg(F + b + 1 + X + XY);
                        f[c][1] = __ldg(F + b + 1 + X);
                        f[c][2] = __ldg(F + b + 1 + XY);
                        f[c][3] = __ldg(F + b + 1);
                        f[c][4] = __ldg(F + b + X + XY);
                        f[c][5] = __ldg(F + b + X);
                        f[c][6] = __ldg(F + b + XY);
                        f[c][7] = __ldg(F + b);
                    }
                    trilerp3(f, s.a, s.b, s.c, u);
                }
                phi[0][i] = px + u[0];
                phi[1][i] = py + u[1];
                phi[2][i] = pz + u[2];
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

// The compositional update with the gathered neighbourhood of m staged in shared memory,
// as ref_pass_b_staged_kernel does for v: per slice the block reduces its cells' bounding
// box and, when it fits kGBX x kGBY x kGBZ, one tensor copy brings that box of m's three
// components into one of two buffers while the previous slice is gathered.  The sobolev
// cell's floor is clamped to dim - 2, so every corner is inside the grid; slices whose
// cells do not fit gather from global memory as sob_pass_b_kernel does, with the same
// arithmetic.  Waits are bounded as in ref_pass_b_staged_kernel.
__global__ void __launch_bounds__(256, 4) sob_pass_b_staged_kernel(SobIterArgs a) {
    constexpr int kPlane = kGBX * kGBY * kGBZ;
    constexpr unsigned kBytes = sizeof(float) * 3 * kPlane;
    extern __shared__ __align__(128) unsigned char sb_raw[];
    float* box = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(sb_raw) + 127) & ~uintptr_t(127));
    uint64_t* full = reinterpret_cast<uint64_t*>(box + 2 * 3 * kPlane);
    __shared__ unsigned long long red[32];
    __shared__ bool last;
    __shared__ CellBoxSets cb;
    const int tid = threadIdx.x;
    if (tid == 0) {
        mbar_init(full, 1);
        mbar_init(full + 1, 1);
        mbar_fence_init();
        for (int k = 0; k < 3; ++k) cellbox_clear(cb, k);
    }
    __syncthreads();
    unsigned g = 0, nbox = 0;
    bool failed = false, wait_failed = false;
    for (int t = blockIdx.x; t < a.ntiles_b && !failed; t += gridDim.x) {
        const Tile tl = a.tiles_b[t];
        if (a.stop[tl.x]) continue;
        const Pair P = a.pairs[tl.x];
        const int x = tl.y + (int)(tid & 31), y = tl.z + (int)(tid >> 5);
        const bool col = x < P.X && y < P.Y;
        const long long NT = a.NT;
        const int X = P.Xp, XY = P.Xp * P.Y;  // strides of the packed arrays
        float* phi[3] = {a.phi + P.off, a.phi + NT + P.off, a.phi + 2 * NT + P.off};
        const float* __restrict__ mc[3] = {a.m + P.off, a.m + NT + P.off, a.m + 2 * NT + P.off};
        const CUtensorMap* mm = a.tmaps + (long long)tl.x * TM_COUNT + TM_SB_M;
        const int z0 = tl.w, z1 = min(tl.w + a.depth_b, P.Z);
        unsigned long long best = 0ull;
        int i = x + X * y + XY * z0;
        float px = 0.f, py = 0.f, pz = 0.f;
        SobCell cl{};
        if (col) {
            px = phi[0][i];
            py = phi[1][i];
            pz = phi[2][i];
            cl = sob_locate(P, px, py, pz);
        }
        auto plan = [&](unsigned set, int o[3]) -> bool {
            int lo[3], hi[3];
            if (!cellbox_read(cb, (int)set, lo, hi)) return false;
            o[0] = lo[0] & ~3;
            o[1] = lo[1];
            o[2] = lo[2];
            const bool fits = hi[0] + 1 - o[0] < kGBX && hi[1] + 1 - o[1] < kGBY && hi[2] + 1 - o[2] < kGBZ;
            if (fits && tid == 0) {
                uint64_t* bar = full + (nbox & 1);
                mbar_arrive_expect_tx(bar, kBytes);
                tma_load_4d(box + (nbox & 1) * 3 * kPlane, mm, o[0], o[1], o[2], 0, bar);
            }
            return fits;
        };
        ++g;
        cellbox_add(cb, (int)(g % 3), col, cl.gx, cl.gy, cl.gz);
        if (__syncthreads_or(wait_failed)) {
            failed = true;
            break;
        }
        if (tid == 0) cellbox_clear(cb, (int)((g - 1) % 3));
        int org[3] = {0, 0, 0};
        bool staged = plan(g % 3, org);
        unsigned mybox = nbox;
        if (staged) ++nbox;
        for (int z = z0; z < z1; ++z, i += XY) {
            const float cx = px, cy = py, cz = pz;
            const SobCell c = cl;
            const bool cur_staged = staged;
            const unsigned cur_box = mybox;
            const int o0 = org[0], o1 = org[1], o2 = org[2];
            const bool nact = col && z + 1 < z1;
            if (nact) {
                px = phi[0][i + XY];
                py = phi[1][i + XY];
                pz = phi[2][i + XY];
                cl = sob_locate(P, px, py, pz);
            }
            ++g;
            cellbox_add(cb, (int)(g % 3), nact, cl.gx, cl.gy, cl.gz);
            if (__syncthreads_or(wait_failed)) {
                failed = true;
                break;
            }
            if (tid == 0) cellbox_clear(cb, (int)((g - 1) % 3));
            staged = plan(g % 3, org);
            mybox = nbox;
            if (staged) ++nbox;
            if (!col) continue;
            float u[3];
            if (cur_staged) {
                if (!mbar_wait_bounded(full + (cur_box & 1), (cur_box >> 1) & 1)) wait_failed = true;
                const float* b0 =
                    box + (cur_box & 1) * 3 * kPlane + ((c.gz - o2) * kGBY + (c.gy - o1)) * kGBX + (c.gx - o0);
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const float* f = b0 + k * kPlane;
                    constexpr int SX = 1, SY = kGBX, SZ = kGBX * kGBY;
                    u[k] = lerpf_(lerpf_(lerpf_(f[SX + SY + SZ], f[SX + SY], c.c), lerpf_(f[SX + SZ], f[SX], c.c), c.b),
                                  lerpf_(lerpf_(f[SY + SZ], f[SY], c.c), lerpf_(f[SZ], f[0], c.c), c.b), c.a);
                }
            } else {
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const float* __restrict__ F = mc[k];
                    const int b = (int)c.base;
                    u[k] = lerpf_(lerpf_(lerpf_(__ldg(F + b + 1 + X + XY), __ldg(F + b + 1 + X), c.c),
                                         lerpf_(__ldg(F + b + 1 + XY), __ldg(F + b + 1), c.c), c.b),
                                  lerpf_(lerpf_(__ldg(F + b + X + XY), __ldg(F + b + X), c.c),
                                         lerpf_(__ldg(F + b + XY), __ldg(F + b), c.c), c.b),
                                  c.a);
                }
            }
            phi[0][i] = cx + u[0];
            phi[1][i] = cy + u[1];
            phi[2][i] = cz + u[2];
            const float nrm = norm3_rd(u[0], u[1], u[2]);
            if (nrm == nrm) {
                const unsigned long long k = norm_key(nrm, i);
                best = k > best ? k : best;
            }
        }
        if (failed) break;
        const unsigned long long bm = block_max_u64(best, red);
        if (tid == 0 && bm) atomicMax(a.keys + tl.x, bm);
    }
    if (failed) {
        if (tid == 0) {
            for (unsigned n = (nbox > 2u ? nbox - 2u : 0u); n < nbox; ++n)
                mbar_wait_bounded(full + (n & 1), (n >> 1) & 1);
            atomicOr(a.err, kErrTmaTimeout);
        }
        return;
    }
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

cudaError_t launch_sob_iter(const SobIterArgs& a, const int* grids, const int* variants, cudaStream_t s,
                            cudaEvent_t* ev) {
    if (ev) cudaEventRecord(ev[0], s);
    if (variants[0])
        sob_grad_tma_kernel<<<grids[0], 256, sob_grad_tma_smem_bytes(), s>>>(a);
    else
        sob_grad_kernel<<<grids[0], 256, sob_grad_smem_bytes(), s>>>(a);
    if (ev) cudaEventRecord(ev[1], s);
    {
        void* args[1] = {const_cast<SobIterArgs*>(&a)};
        cudaLaunchKernel(sob_smooth3_fn(a.radius, variants[1]), dim3(grids[1]), dim3(256), args, 0, s);
    }
    if (ev) cudaEventRecord(ev[2], s);
    if (variants[2])
        sob_pass_b_staged_kernel<<<grids[2], 256, gather_staged_smem_bytes(), s>>>(a);
    else
        sob_pass_b_kernel<<<grids[2], 256, 0, s>>>(a);
    if (ev) cudaEventRecord(ev[3], s);
    return cudaGetLastError();
}

const void* sob_smooth3_fn(int radius, int variant) {
    if (variant) {
        switch (radius) {
            case 0: return (const void*)sob_smooth3_tma_kernel<0>;
            case 1: return (const void*)sob_smooth3_tma_kernel<1>;
            case 2: return (const void*)sob_smooth3_tma_kernel<2>;
            case 3: return (const void*)sob_smooth3_tma_kernel<3>;
            case 4: return (const void*)sob_smooth3_tma_kernel<4>;
            case 5: return (const void*)sob_smooth3_tma_kernel<5>;
            case 6: return (const void*)sob_smooth3_tma_kernel<6>;
            default: return (const void*)sob_smooth3_tma_kernel<7>;
        }
    }
    switch (radius) {
        case 0: return (const void*)sob_smooth3_kernel<0>;
        case 1: return (const void*)sob_smooth3_kernel<1>;
        case 2: return (const void*)sob_smooth3_kernel<2>;
        case 3: return (const void*)sob_smooth3_kernel<3>;
        case 4: return (const void*)sob_smooth3_kernel<4>;
        case 5: return (const void*)sob_smooth3_kernel<5>;
        case 6: return (const void*)sob_smooth3_kernel<6>;
        default: return (const void*)sob_smooth3_kernel<7>;
    }
}

}  // namespace frg
