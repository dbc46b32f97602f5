// fr_common.cuh -- shared device-side types and helpers of the fastreg GB300 kernels.
//
// Layout in HBM (all pairs of a cohort packed into one allocation per field):
//   scalar field  f[off_p + i]                    i = x + Xp*(y + Y*z), x fastest
//   vector field  f[c*NT + off_p + i], c = 0,1,2  three planes (SoA), NT = packed voxels
// Xp is X rounded up to a multiple of 4 (rows start on 16-byte boundaries); the pad
// columns are zero and never written.  off_p, the voxel offset of pair p, is a
// multiple of 32 (128 B).  The caller's buffers keep the reference's unpadded layout
// x + X*(y + Y*z); pack_init_kernel and finalize_kernel convert.
//
// Arithmetic contract (mirrored by the CPU oracle): the library is compiled with
// --fmad=false, so a*b+c is never contracted; the only fused multiply-adds are the
// explicit fmaf() calls of lerp (include/cuda/cuda_utils.hpp:43-46 of the reference).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace frg {

// One registration pair inside a packed cohort.
struct Pair {
    int X, Y, Z;
    int Xp;         // row pitch in the packed arrays (X rounded up to a multiple of 4)
    long long off;  // voxel offset into the packed arrays
    long long N;    // Xp*Y*Z: the pair's extent in the packed arrays
    float w_reg;    // regularisation weight of this pair (W_REG unless set per pair)
    int pad_;
};

// A tile of work: pair index and the tile origin (x0, y0, z0).
typedef int4 Tile;

constexpr int kTileX = 32;  // threads along x (one warp per row)
constexpr int kTileY = 8;   // rows per block
constexpr int kTileZ = 16;  // slices marched by each thread
// The solver kernels walk their own tile tables of 32 x 8 x depth tiles; the depth of
// each table and the kernel's blocks per SM are chosen on the host (fr_api.cu: defaults,
// or the autotuner's choice for the cohort's size class).

__device__ __forceinline__ long long lin(const Pair& P, int x, int y, int z) {
    return (long long)x + (long long)P.Xp * ((long long)y + (long long)P.Y * z);
}

// index of (x, y, z) in the caller's unpadded layout
__device__ __forceinline__ long long user_lin(const Pair& P, int x, int y, int z) {
    return (long long)x + (long long)P.X * ((long long)y + (long long)P.Y * z);
}

// lerp(v0, v1, t) = fma(t, v0, fma(-t, v1, v1))
__device__ __forceinline__ float lerpf_(float v0, float v1, float t) { return fmaf(t, v0, fmaf(-t, v1, v1)); }

// Sample cell: clamp to [0, dim-1], floor corner, fractional weights
// (interpolate_intensity / interpolate_field, include/cuda/cuda_utils.hpp:60-136).
struct Cell {
    long long base;  // linear index of the floor corner
    int gx, gy, gz;
    float a, b, c;
};

__device__ __forceinline__ Cell locate(const Pair& P, float px, float py, float pz) {
    Cell cl;
    float cx = fminf(fmaxf(0.f, px), (float)(P.X - 1));
    float cy = fminf(fmaxf(0.f, py), (float)(P.Y - 1));
    float cz = fminf(fmaxf(0.f, pz), (float)(P.Z - 1));
    cl.gx = (int)floorf(cx);
    cl.gy = (int)floorf(cy);
    cl.gz = (int)floorf(cz);
    cl.a = cx - (float)cl.gx;
    cl.b = cy - (float)cl.gy;
    cl.c = cz - (float)cl.gz;
    cl.base = lin(P, cl.gx, cl.gy, cl.gz);
    return cl;
}

// Trilinear sample with the unchecked corner addressing of the reference's
// Volume/VectorField operator(): the +1 corner of a cell on the upper face aliases
// to the next row/slice (weight 0 there); an index past the last voxel is clamped.
// F points at the pair's plane (already offset by off_p).
__device__ __forceinline__ float tri_unchecked(const float* __restrict__ F, const Pair& P, const Cell& cl) {
    const long long X = P.Xp, XY = (long long)P.Xp * P.Y, last = P.N - 1;
    const long long b = cl.base;
    auto at = [&](long long d) -> float {
        long long j = b + d;
        return __ldg(F + (j < last ? j : last));
    };
    float f111 = at(1 + X + XY), f110 = at(1 + X), f101 = at(1 + XY), f100 = at(1);
    float f011 = at(X + XY), f010 = at(X), f001 = at(XY), f000 = __ldg(F + b);
    return lerpf_(lerpf_(lerpf_(f111, f110, cl.c), lerpf_(f101, f100, cl.c), cl.b),
                  lerpf_(lerpf_(f011, f010, cl.c), lerpf_(f001, f000, cl.c), cl.b), cl.a);
}

// Trilinear sample with get_global_idx addressing (include/cuda/cuda_utils.hpp:31-37,
// 109-136): a corner outside the grid reads element 0 of the field.
__device__ __forceinline__ float tri_checked(const float* __restrict__ F, const Pair& P, const Cell& cl) {
    const long long X = P.Xp, XY = (long long)P.Xp * P.Y;
    const long long b = cl.base;
    const bool ox = cl.gx + 1 < P.X, oy = cl.gy + 1 < P.Y, oz = cl.gz + 1 < P.Z;
    const float f0 = __ldg(F);
    float f000 = __ldg(F + b);
    float f100 = ox ? __ldg(F + b + 1) : f0;
    float f010 = oy ? __ldg(F + b + X) : f0;
    float f001 = oz ? __ldg(F + b + XY) : f0;
    float f110 = (ox && oy) ? __ldg(F + b + 1 + X) : f0;
    float f101 = (ox && oz) ? __ldg(F + b + 1 + XY) : f0;
    float f011 = (oy && oz) ? __ldg(F + b + X + XY) : f0;
    float f111 = (ox && oy && oz) ? __ldg(F + b + 1 + X + XY) : f0;
    return lerpf_(lerpf_(lerpf_(f111, f110, cl.c), lerpf_(f101, f100, cl.c), cl.b),
                  lerpf_(lerpf_(f011, f010, cl.c), lerpf_(f001, f000, cl.c), cl.b), cl.a);
}

// ---- 32-bit variants used inside one pair (N < 2^31) ----

struct Cell32 {
    int base;  // linear index of the floor corner inside the pair
    int gx, gy, gz;
    float a, b, c;
};

// X, Y, Z: grid extents; Xp: row pitch of the array the cell indexes
__device__ __forceinline__ Cell32 locate32(int X, int Y, int Z, int Xp, float px, float py, float pz) {
    Cell32 cl;
    const float cx = fminf(fmaxf(0.f, px), (float)(X - 1));
    const float cy = fminf(fmaxf(0.f, py), (float)(Y - 1));
    const float cz = fminf(fmaxf(0.f, pz), (float)(Z - 1));
    cl.gx = (int)floorf(cx);
    cl.gy = (int)floorf(cy);
    cl.gz = (int)floorf(cz);
    cl.a = cx - (float)cl.gx;
    cl.b = cy - (float)cl.gy;
    cl.c = cz - (float)cl.gz;
    cl.base = cl.gx + Xp * (cl.gy + Y * cl.gz);
    return cl;
}

__device__ __forceinline__ float trilerp(float f111, float f110, float f101, float f100, float f011, float f010,
                                         float f001, float f000, float a, float b, float c) {
    return lerpf_(lerpf_(lerpf_(f111, f110, c), lerpf_(f101, f100, c), b),
                  lerpf_(lerpf_(f011, f010, c), lerpf_(f001, f000, c), b), a);
}

// Two lerps as one packed FP32 pair: per lane exactly lerpf_(v0, v1, t) (both fused
// multiply-adds of a lane are the lane's own, rounded once each).  nt = -t, passed in so
// that a cell's negated weights are formed once.
__device__ __forceinline__ float2 lerp2_(float2 v0, float2 v1, float2 t, float2 nt) {
    return __ffma2_rn(t, v0, __ffma2_rn(nt, v1, v1));
}

// two trilerps as one packed pair, each lane with its own corner values and weights
__device__ __forceinline__ float2 trilerp2w(float2 f111, float2 f110, float2 f101, float2 f100, float2 f011,
                                            float2 f010, float2 f001, float2 f000, float2 ta, float2 tb, float2 tc) {
    const float2 na = make_float2(-ta.x, -ta.y), nb = make_float2(-tb.x, -tb.y), nc = make_float2(-tc.x, -tc.y);
    return lerp2_(lerp2_(lerp2_(f111, f110, tc, nc), lerp2_(f101, f100, tc, nc), tb, nb),
                  lerp2_(lerp2_(f011, f010, tc, nc), lerp2_(f001, f000, tc, nc), tb, nb), ta, na);
}

// trilerp of two fields at one cell as one packed pair (lane 0: field 0, lane 1: field 1)
__device__ __forceinline__ float2 trilerp2(float2 f111, float2 f110, float2 f101, float2 f100, float2 f011,
                                           float2 f010, float2 f001, float2 f000, float a, float b, float c) {
    return trilerp2w(f111, f110, f101, f100, f011, f010, f001, f000, make_float2(a, a), make_float2(b, b),
                     make_float2(c, c));
}

// trilerp of three fields' corners f[k][0..7] (order 111, 110, 101, 100, 011, 010, 001, 000)
// at one cell: fields 0 and 1 as one packed pair, field 2 alone; per field exactly trilerp
__device__ __forceinline__ void trilerp3(const float f[3][8], float a, float b, float c, float out[3]) {
    auto p = [&](int q) { return make_float2(f[0][q], f[1][q]); };
    const float2 r = trilerp2(p(0), p(1), p(2), p(3), p(4), p(5), p(6), p(7), a, b, c);
    out[0] = r.x;
    out[1] = r.y;
    out[2] = trilerp(f[2][0], f[2][1], f[2][2], f[2][3], f[2][4], f[2][5], f[2][6], f[2][7], a, b, c);
}

// tri_unchecked with 32-bit indices: corners past the last voxel (only possible when
// the cell touches the end of the array) are clamped on a slow path.  X, XY, N are the
// strides and extent of the array (pitched for the packed arrays).
__device__ __forceinline__ float tri_unchecked32(const float* __restrict__ F, int X, int XY, int N, const Cell32& cl) {
    const int b = cl.base;
    if (b + 1 + X + XY <= N - 1) {
        return trilerp(__ldg(F + b + 1 + X + XY), __ldg(F + b + 1 + X), __ldg(F + b + 1 + XY), __ldg(F + b + 1),
                       __ldg(F + b + X + XY), __ldg(F + b + X), __ldg(F + b + XY), __ldg(F + b), cl.a, cl.b, cl.c);
    }
    const int last = N - 1;
    return trilerp(__ldg(F + min(b + 1 + X + XY, last)), __ldg(F + min(b + 1 + X, last)),
                   __ldg(F + min(b + 1 + XY, last)), __ldg(F + min(b + 1, last)), __ldg(F + min(b + X + XY, last)),
                   __ldg(F + min(b + X, last)), __ldg(F + min(b + XY, last)), __ldg(F + b), cl.a, cl.b, cl.c);
}

// The three components of a vector field (planes F0, F1, F2) at one cell with
// tri_checked32's addressing; components 0 and 1 interpolated as one packed pair.
__device__ __forceinline__ void tri_checked32_3(const float* __restrict__ F0, const float* __restrict__ F1,
                                                const float* __restrict__ F2, int X, int Y, int Z, int Xp, int XYp,
                                                const Cell32& cl, float out[3]) {
    const int b = cl.base;
    const bool ox = cl.gx + 1 < X, oy = cl.gy + 1 < Y, oz = cl.gz + 1 < Z;
    const float* const F[3] = {F0, F1, F2};
    float f[3][8];
    if (ox && oy && oz) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            f[k][0] = __ldg(F[k] + b + 1 + Xp + XYp);
            f[k][1] = __ldg(F[k] + b + 1 + Xp);
            f[k][2] = __ldg(F[k] + b + 1 + XYp);
            f[k][3] = __ldg(F[k] + b + 1);
            f[k][4] = __ldg(F[k] + b + Xp + XYp);
            f[k][5] = __ldg(F[k] + b + Xp);
            f[k][6] = __ldg(F[k] + b + XYp);
            f[k][7] = __ldg(F[k] + b);
        }
    } else {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float f0 = __ldg(F[k]);
            f[k][0] = (ox && oy && oz) ? __ldg(F[k] + b + 1 + Xp + XYp) : f0;
            f[k][1] = (ox && oy) ? __ldg(F[k] + b + 1 + Xp) : f0;
            f[k][2] = (ox && oz) ? __ldg(F[k] + b + 1 + XYp) : f0;
            f[k][3] = ox ? __ldg(F[k] + b + 1) : f0;
            f[k][4] = (oy && oz) ? __ldg(F[k] + b + Xp + XYp) : f0;
            f[k][5] = oy ? __ldg(F[k] + b + Xp) : f0;
            f[k][6] = oz ? __ldg(F[k] + b + XYp) : f0;
            f[k][7] = __ldg(F[k] + b);
        }
    }
    trilerp3(f, cl.a, cl.b, cl.c, out);
}

// tri_checked with 32-bit indices: corners outside the grid read element 0.  X, Y, Z:
// grid extents; Xp, XYp: strides of the array.
__device__ __forceinline__ float tri_checked32(const float* __restrict__ F, int X, int Y, int Z, int Xp, int XYp,
                                               const Cell32& cl) {
    const int b = cl.base;
    const bool ox = cl.gx + 1 < X, oy = cl.gy + 1 < Y, oz = cl.gz + 1 < Z;
    if (ox && oy && oz) {
        return trilerp(__ldg(F + b + 1 + Xp + XYp), __ldg(F + b + 1 + Xp), __ldg(F + b + 1 + XYp), __ldg(F + b + 1),
                       __ldg(F + b + Xp + XYp), __ldg(F + b + Xp), __ldg(F + b + XYp), __ldg(F + b), cl.a, cl.b,
                       cl.c);
    }
    const float f0 = __ldg(F);
    return trilerp((ox && oy && oz) ? __ldg(F + b + 1 + Xp + XYp) : f0, (ox && oy) ? __ldg(F + b + 1 + Xp) : f0,
                   (ox && oz) ? __ldg(F + b + 1 + XYp) : f0, ox ? __ldg(F + b + 1) : f0,
                   (oy && oz) ? __ldg(F + b + Xp + XYp) : f0, oy ? __ldg(F + b + Xp) : f0,
                   oz ? __ldg(F + b + XYp) : f0, __ldg(F + b), cl.a, cl.b, cl.c);
}

__device__ __forceinline__ float4 lerp4_(float4 v0, float4 v1, float t) {
    return make_float4(lerpf_(v0.x, v1.x, t), lerpf_(v0.y, v1.y, t), lerpf_(v0.z, v1.z, t), lerpf_(v0.w, v1.w, t));
}

// tri_unchecked32 on an interleaved 4-channel field (one 16-byte load per corner)
__device__ __forceinline__ float4 tri_unchecked32_f4(const float4* __restrict__ F, int X, int XY, int N,
                                                     const Cell32& cl) {
    const int b = cl.base;
    int o111 = b + 1 + X + XY, o110 = b + 1 + X, o101 = b + 1 + XY, o100 = b + 1;
    int o011 = b + X + XY, o010 = b + X, o001 = b + XY;
    if (o111 > N - 1) {
        const int last = N - 1;
        o111 = min(o111, last);
        o110 = min(o110, last);
        o101 = min(o101, last);
        o100 = min(o100, last);
        o011 = min(o011, last);
        o010 = min(o010, last);
        o001 = min(o001, last);
    }
    const float4 f111 = __ldg(F + o111), f110 = __ldg(F + o110), f101 = __ldg(F + o101), f100 = __ldg(F + o100);
    const float4 f011 = __ldg(F + o011), f010 = __ldg(F + o010), f001 = __ldg(F + o001), f000 = __ldg(F + b);
    // channels (x, y) and (z, w) as packed pairs: per channel the lerp4_ arithmetic
    auto lo = [](float4 v) { return make_float2(v.x, v.y); };
    auto hi = [](float4 v) { return make_float2(v.z, v.w); };
    const float2 r0 = trilerp2(lo(f111), lo(f110), lo(f101), lo(f100), lo(f011), lo(f010), lo(f001), lo(f000), cl.a,
                               cl.b, cl.c);
    const float2 r1 = trilerp2(hi(f111), hi(f110), hi(f101), hi(f100), hi(f011), hi(f010), hi(f001), hi(f000), cl.a,
                               cl.b, cl.c);
    return make_float4(r0.x, r0.y, r1.x, r1.y);
}

// Hint that the 128-byte line holding *p will be read soon: it is fetched into L2 with
// no register written and nothing waited for (p must point into an allocation).
__device__ __forceinline__ void prefetch_l2(const void* p) {
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// ---- asynchronous global -> shared copies (cp.async, 4 bytes each) ----
__device__ __forceinline__ void cp_async4(float* smem, const float* gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
// 16-byte copy that bypasses L1; both addresses 16-byte aligned
__device__ __forceinline__ void cp_async16(float* smem, const float* gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int Pending>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(Pending) : "memory");
}

// ---- slices of a 32 x 8 column tile staged in shared memory ----
// A staged slice of a plane with y halo H is 8 + 2H rows (y0 - H .. y0 + 7 + H) of
// kStageChunks aligned 16-byte chunks (columns x0 - 4 .. x0 + 35; column x0 + tx sits at
// row offset tx + kStageXO).  Thread e copies chunk e of every slice and component of the
// tile: its shared-memory offset is 4e floats, and its offset inside a slice, fixed for
// the tile, is returned here (-1: no chunk, or the chunk lies outside the padded volume,
// where no voxel of the tile reads).
constexpr int kStageXO = 4, kStageW = kTileX + 2 * kStageXO, kStageChunks = kStageW / 4;
template <int H>
__device__ __forceinline__ int stage_offset(int e, int Y, int Xp, int x0, int y0) {
    constexpr int R = kTileY + 2 * H;
    static_assert(R * kStageChunks <= 256, "one chunk per thread of a 256-thread block");
    if (e >= R * kStageChunks) return -1;
    const int r = e / kStageChunks, k = e - r * kStageChunks;
    const int y = y0 - H + r, x = x0 - kStageXO + 4 * k;
    if (y < 0 || y >= Y || x < 0 || x >= Xp) return -1;
    return Xp * y + x;
}

// sqrt rounded toward -inf (reference norm(), include/cuda/cuda_utils.hpp:251-253)
__device__ __forceinline__ float norm3_rd(float x, float y, float z) {
    return __fsqrt_rd((x * x + y * y) + z * z);
}

// (norm, index) packed so that a larger key means a larger norm and, for equal
// norms, a lower linear index.  norm >= 0, so its IEEE bits order like the value.
__device__ __forceinline__ unsigned long long norm_key(float nrm, long long idx) {
    return ((unsigned long long)__float_as_uint(nrm) << 32) | (unsigned long long)(0xffffffffu - (unsigned)idx);
}

// Block-wide max of a 64-bit key; every thread must call it.  Returns the block max
// in thread 0.
__device__ __forceinline__ unsigned long long block_max_u64(unsigned long long k, unsigned long long* smem) {
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long other = __shfl_xor_sync(0xffffffffu, k, o);
        k = other > k ? other : k;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) smem[warp] = k;
    __syncthreads();
    const int nw = blockDim.x >> 5;
    if (warp == 0) {
        k = lane < nw ? smem[lane] : 0ull;
        for (int o = 16; o > 0; o >>= 1) {
            unsigned long long other = __shfl_xor_sync(0xffffffffu, k, o);
            k = other > k ? other : k;
        }
    }
    __syncthreads();
    return k;
}

__device__ __forceinline__ double block_sum_f64(double v, double* smem) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) smem[warp] = v;
    __syncthreads();
    const int nw = blockDim.x >> 5;
    if (warp == 0) {
        v = lane < nw ? smem[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    }
    __syncthreads();
    return v;
}

}  // namespace frg
