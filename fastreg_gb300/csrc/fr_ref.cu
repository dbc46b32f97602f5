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
#include "fr_tma.cuh"

namespace frg {

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
//
// A block owns a 32 x 8 column tile and marches z.  Every stencil operand is staged in
// shared-memory ring buffers by 16-byte cp.async one slice ahead of the compute: v with
// a 2-voxel halo over a 5-slice window, and psi_inv, rho and S with a 1-voxel halo over a
// 3-slice window (one ring of five components), so the stencil reads are shared-memory
// loads and the global traffic is one coalesced pass per field.  T o psi_inv and
// L o psi_inv are gathered from the interleaved LT field (eight 16-byte loads per voxel).
// The LT rows of the next slice's cell and the rho/S slice three steps ahead are
// prefetched into L2 (the kernel is latency-bound).
// ----------------------------------------------------------------------------------
namespace {
// prefetch distance: slices in flight ahead of the one being computed
constexpr int kAhead = 1;
// Staged rows cover x0 - 4 .. x0 + 35 (stage_offset): column x0 + tx sits at row offset
// tx + kXO.  v has a 2-row y halo, psi_inv a 1-row one.
constexpr int kXO = kStageXO;
constexpr int kVH = 2, kVW = kTileX + 2 * kXO, kVR = kTileY + 2 * kVH, kVS = 5 + kAhead;  // v: halo, width, rows, slots
constexpr int kQH = 1, kQW = kTileX + 2 * kXO, kQR = kTileY + 2 * kQH, kQS = 3 + kAhead;  // psi_inv
constexpr int kVPlane = kVW * kVR, kQPlane = kQW * kQR;
constexpr int kQC = 5;  // the psi_inv ring also holds rho and S (same halo and window)
constexpr int kPassASmemFloats = 3 * kVS * kVPlane + kQC * kQS * kQPlane;  // v x3, psi_inv x3, rho, S
constexpr size_t kPassASmemBytes = sizeof(float) * kPassASmemFloats;

struct PassASmem {
    float* v;  // [3][kVS][kVR][kVW]
    float* q;  // [kQC][kQS][kQR][kQW]: psi_inv x, y, z, rho, S
};

}  // namespace

size_t ref_pass_a_smem_bytes() { return kPassASmemBytes; }

// ----------------------------------------------------------------------------------
// LT = (-(sum of 6 neighbours - 6 psi), T) on the interior; the boundary keeps the
// (0, 0, 0, T) that pack_init_kernel wrote
//
// A block owns a 32 x 8 column tile and marches z.  psi's three components (tile rows
// plus a 1-voxel halo, the psi_inv ring's geometry) and T are staged slice by slice into
// a shared-memory ring by 16-byte cp.async three slices ahead of the compute, so each
// slice of psi is fetched once per tile instead of once per stencil tap (11% faster than
// 7-point reads through L1; one slice ahead or T read per voxel gained nothing).
// ----------------------------------------------------------------------------------
namespace {
constexpr int kLAhead = 3;        // slices in flight ahead of the one computed
constexpr int kLS = 3 + kLAhead;  // ring slots: slices z - 1, z, z + 1 and those in flight
constexpr bool kLStageT = true;   // T staged with psi (else read per voxel)
constexpr int kTPlane = kTileX * kTileY;
}

size_t ref_laplacian_smem_bytes() { return sizeof(float) * kLS * (3 * kQPlane + (kLStageT ? kTPlane : 0)); }

__global__ void __launch_bounds__(256) ref_laplacian_kernel(RefIterArgs a) {
    extern __shared__ __align__(16) float ring[];  // psi [3][kLS][kQR][kQW], then T [kLS][8][32]
    float* tring = ring + 3 * kLS * kQPlane;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int t = blockIdx.x; t < a.ntiles_l; t += gridDim.x) {
        const Tile tl = a.tiles_l[t];
        if (a.stop[tl.x]) continue;  // uniform over the block
        const Pair P = a.pairs[tl.x];
        const int X = P.X, Y = P.Y, Z = P.Z, Xp = P.Xp, XYp = P.Xp * P.Y;  // strides of the packed arrays
        const int zs0 = max(tl.w, 1), zs1 = min(tl.w + a.depth_l, Z - 1);
        if (zs0 >= zs1 || tl.y + kTileX <= 1 || tl.z + kTileY <= 1 || tl.y >= X - 1 || tl.z >= Y - 1) continue;
        const long long NT = a.NT;
        const float* __restrict__ Qg[3] = {a.psi + P.off, a.psi + NT + P.off, a.psi + 2 * NT + P.off};
        const float* __restrict__ Tg = a.T + P.off;
        float4* LT = a.LT + P.off;
        const int x = tl.y + tx, y = tl.z + ty;
        const bool active = x >= 1 && x <= X - 2 && y >= 1 && y <= Y - 2;
        const int g = stage_offset<1>(threadIdx.x, Y, Xp, tl.y, tl.z);
        // T: thread e < 64 copies chunk e & 7 of tile row e >> 3 (x0 is a multiple of 32)
        const int tr = (int)threadIdx.x >> 3, tk = (int)threadIdx.x & 7;
        const int gt = (kLStageT && threadIdx.x < 64 && tl.z + tr < Y && tl.y + 4 * tk < Xp)
                           ? Xp * (tl.z + tr) + tl.y + 4 * tk : -1;
        auto stage = [&](int zs, int sl) {  // slice zs of psi's three components (and T) into slot sl
            if (g >= 0) {
                float* dst = ring + sl * kQPlane + 4 * threadIdx.x;
                const int off = g + XYp * zs;
#pragma unroll
                for (int c = 0; c < 3; ++c) cp_async16(dst + c * kLS * kQPlane, Qg[c] + off);
            }
            if (kLStageT && gt >= 0) cp_async16(tring + sl * kTPlane + 4 * threadIdx.x, Tg + gt + XYp * zs);
        };
        __syncthreads();  // the previous tile is done with the ring
        // prologue: slices zs0 - 1 .. zs0 + 1 (one group), then one group per slice ahead
        stage(zs0 - 1, 0);
        stage(zs0, 1);
        stage(zs0 + 1, 2);
        cp_async_commit();
#pragma unroll
        for (int k = 1; k < kLAhead; ++k) {
            if (zs0 + 1 + k <= zs1) stage(zs0 + 1 + k, 2 + k);
            cp_async_commit();
        }
        int sm = 0;  // slot of slice z - 1 (z, z + 1 follow it in the ring)
        const int c0 = (ty + 1) * kQW + tx + kXO;
        for (int z = zs0; z < zs1; ++z) {
            cp_async_wait<kLAhead - 1>();  // slice z + 1 has landed ...
            __syncthreads();               // ... for every thread, and slice z - 2's slot is free
            {
                int sl = sm + 2 + kLAhead;  // the slot of slice z - 2
                sl = sl >= kLS ? sl - kLS : sl;
                if (z + 1 + kLAhead <= zs1) stage(z + 1 + kLAhead, sl);  // reads reach zs1
                cp_async_commit();
            }
            const int s0 = sm + 1 >= kLS ? sm + 1 - kLS : sm + 1;
            const int sp = s0 + 1 >= kLS ? s0 + 1 - kLS : s0 + 1;
            if (active) {
                const int i = x + Xp * y + XYp * z;
                float l[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float* q = ring + (c * kLS + s0) * kQPlane + c0;
                    const float* qm = ring + (c * kLS + sm) * kQPlane + c0;
                    const float* qp = ring + (c * kLS + sp) * kQPlane + c0;
                    float s = -6.f * q[0];
                    s = s + q[1];
                    s = s + q[-1];
                    s = s + q[kQW];
                    s = s + q[-kQW];
                    s = s + qp[0];
                    s = s + qm[0];
                    l[c] = -1.f * s;
                }
                const float tv = kLStageT ? tring[s0 * kTPlane + ty * kTileX + tx] : __ldg(Tg + i);
                LT[i] = make_float4(l[0], l[1], l[2], tv);
            }
            sm = s0;
        }
        cp_async_wait<0>();
    }
}

// ----------------------------------------------------------------------------------
// The same Laplacian with TMA staging.  Per slice, one thread issues two tensor copies
// into the slot's shared memory -- psi's box of 40 columns x 10 rows x 3 components (the
// tile plus a 1-voxel halo, x0 - 4 .. x0 + 35, y0 - 1 .. y0 + 8; out-of-volume parts read
// as zero and are never used) and T's 32 x 8 box -- completing on the slot's mbarrier; no
// other thread computes an address or issues a copy.  A six-slot ring keeps three slices
// ahead of the one computed (slices z - 1, z, z + 1 are read), and one block barrier per
// slice frees the slot of slice z - 2 for the next copy.  Every wait is bounded (about a
// second); a block that gives up sets the device error word, waits (bounded) for its own
// copies in flight and returns.
// ----------------------------------------------------------------------------------
namespace {
constexpr int kTLAhead = 3;
constexpr int kTLS = 3 + kTLAhead;                      // ring slots
constexpr int kTQW = 40, kTQR = 10, kTQPlane = kTQW * kTQR;  // psi box: row, rows, plane (floats)
constexpr int kTTOff = 1216;                            // T box offset in a slot (floats, 128-byte aligned)
constexpr int kTSlot = kTTOff + kTileX * kTileY;        // slot stride: 1472 floats = 5888 bytes
constexpr unsigned kTLBytes = sizeof(float) * (3 * kTQPlane + kTileX * kTileY);  // copied per slice
static_assert(3 * kTQPlane <= kTTOff && (kTTOff * 4) % 128 == 0 && (kTSlot * 4) % 128 == 0, "slot layout");
}  // namespace

size_t ref_laplacian_tma_smem_bytes() { return 128 + sizeof(float) * kTLS * kTSlot + sizeof(uint64_t) * kTLS; }

__global__ void __launch_bounds__(256) ref_laplacian_tma_kernel(RefIterArgs a) {
    extern __shared__ __align__(128) unsigned char lap_raw[];
    float* ring = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(lap_raw) + 127) & ~uintptr_t(127));
    uint64_t* full = reinterpret_cast<uint64_t*>(ring + kTLS * kTSlot);
    typedef SliceRing<kTLS> Ring;
    const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
    if (tid == 0) {
        for (int k = 0; k < kTLS; ++k) mbar_init(full + k, 1);
        mbar_fence_init();
    }
    __syncthreads();
    // The block's slices go through the ring in one sequence n = 0, 1, 2, ... across its
    // tiles (slot n % kTLS, the (n / kTLS)-th fill of that slot), issued by thread 0 and
    // waited for by every thread in the same order; both walk it with counters instead of
    // dividing: the next slot to issue (islot), the next slot to wait for (wslot), and per
    // slot the parity of its next completion (bit k of wph).
    unsigned issued = 0;  // slices issued so far (thread 0's count)
    int islot = 0, wslot = 0;
    unsigned wph = 0u;
    bool failed = false;
    for (int t = blockIdx.x; t < a.ntiles_l && !failed; t += gridDim.x) {
        const Tile tl = a.tiles_l[t];
        if (a.stop[tl.x]) continue;  // uniform over the block
        const Pair P = a.pairs[tl.x];
        const int X = P.X, Y = P.Y, Z = P.Z, Xp = P.Xp, XYp = P.Xp * P.Y;
        const int zs0 = max(tl.w, 1), zs1 = min(tl.w + a.depth_l, Z - 1);
        if (zs0 >= zs1 || tl.y + kTileX <= 1 || tl.z + kTileY <= 1 || tl.y >= X - 1 || tl.z >= Y - 1) continue;
        const CUtensorMap* mpsi = a.tmaps + (long long)tl.x * TM_COUNT + TM_LAP_PSI;
        const CUtensorMap* mT = a.tmaps + (long long)tl.x * TM_COUNT + TM_LAP_T;
        float4* LT = a.LT + P.off;
        const int x = tl.y + tx, y = tl.z + ty;
        const bool active = x >= 1 && x <= X - 2 && y >= 1 && y <= Y - 2;
        const int nsl = zs1 - zs0 + 2;  // slices zs0 - 1 .. zs1, all issued and all waited for
        auto issue = [&](int j) {       // slice zs0 - 1 + j of the tile (thread 0)
            float* dst = ring + islot * kTSlot;
            uint64_t* bar = full + islot;
            mbar_arrive_expect_tx(bar, kTLBytes);
            tma_load_4d(dst, mpsi, tl.y - 4, tl.z - 1, zs0 - 1 + j, 0, bar);
            tma_load_3d(dst + kTTOff, mT, tl.y, tl.z, zs0 - 1 + j, bar);
            islot = islot + 1 == kTLS ? 0 : islot + 1;
            ++issued;
        };
        auto wait_next = [&]() {  // the next slice of the sequence has landed
            const bool ok = mbar_wait_bounded(full + wslot, (wph >> wslot) & 1u);
            wph ^= 1u << wslot;
            wslot = wslot + 1 == kTLS ? 0 : wslot + 1;
            return ok;
        };
        __syncthreads();  // the previous tile is done with the ring
        if (tid == 0) {
            tma_prefetch_map(mpsi);
            tma_prefetch_map(mT);
            for (int j = 0; j < min(nsl, kTLS); ++j) issue(j);
        }
        const int c0 = (ty + 1) * kTQW + tx + 4;
        int sm = 0, s0 = 0, sp = 0;  // slots of slices j0, j0 + 1 and j0 + 2 of the tile
        for (int j0 = 0; j0 + 2 < nsl; ++j0) {
            // slices j0, j0 + 1 and j0 + 2 of the tile are read; j0 + 2 is the newest
            bool ok;
            if (j0 == 0) {
                sm = wslot;
                ok = wait_next();
                s0 = wslot;
                ok = wait_next() && ok;
                sp = wslot;
                ok = wait_next() && ok;
            } else {
                sm = s0;
                s0 = sp;
                sp = wslot;
                ok = wait_next();
            }
            // every thread is past step j0 - 1 (the slot of slice j0 - 1 is free), and the
            // block agrees on whether any wait gave up
            if (__syncthreads_or(!ok)) {
                failed = true;
                break;
            }
            if (tid == 0 && j0 >= 1 && j0 - 1 + kTLS < nsl) issue(j0 - 1 + kTLS);
            if (active) {
                const int z = zs0 + j0;
                const float* qm = ring + sm * kTSlot + c0;
                const float* q0 = ring + s0 * kTSlot;
                const float* qp = ring + sp * kTSlot + c0;
                float l[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float* q = q0 + c0 + c * kTQPlane;
                    float s = -6.f * q[0];
                    s = s + q[1];
                    s = s + q[-1];
                    s = s + q[kTQW];
                    s = s + q[-kTQW];
                    s = s + qp[c * kTQPlane];
                    s = s + qm[c * kTQPlane];
                    l[c] = -1.f * s;
                }
                const float tv = q0[kTTOff + ty * kTileX + tx];
                LT[x + Xp * y + XYp * z] = make_float4(l[0], l[1], l[2], tv);
            }
        }
    }
    if (failed && tid == 0) {
        // the copies this block issued and nobody waited for: wait for them (bounded)
        // before the block's shared memory goes away, then report
        for (unsigned n = (issued > (unsigned)kTLS ? issued - kTLS : 0u); n < issued; ++n)
            mbar_wait_bounded(full + Ring::slot(n), Ring::parity(n));
        atomicOr(a.err, kErrTmaTimeout);
    }
}

// One voxel of pass A (i = x + Xp (y + Y z), an interior voxel).  vb[k]: this thread's
// column in the staged slice z - 2 + k of v (component c at + c VC); qb[k]: in the staged
// slice z - 1 + k of psi_inv (component c at + c QC), rho (at + QR) and S (at + QS); RW is
// the staged row length.  The arithmetic is the reference's, operation for operation.
template <int VC, int QC, int QR, int QS, int RW>
__device__ __forceinline__ void pass_a_voxel(const RefIterArgs& a, const Pair& P, int X, int Y, int Z, int N, int Xp,
                                             int XYp, int y, int z, int i, bool dv_xy, const float* const vb[5],
                                             const float* const qb[3], const float4* __restrict__ LT,
                                             const float* __restrict__ Tg, const float* __restrict__ Sg,
                                             const float* __restrict__ Rg, const float* __restrict__ const* Vg,
                                             float* rho_n,
                                             float* const* Vn, float* const* Qn) {
    auto V = [&](int k, int c) { return vb[k] + c * VC; };
    auto Q = [&](int k, int c) { return qb[k] + (c < 3 ? c * QC : (c == 3 ? QR : QS)); };
    // T o psi_inv and L o psi_inv, gathered at psi_inv(x)
    const float q[3] = {Q(1, 0)[0], Q(1, 1)[0], Q(1, 2)[0]};
    const Cell32 cl = locate32(X, Y, Z, Xp, q[0], q[1], q[2]);
    const float4 lt = tri_unchecked32_f4(LT, Xp, XYp, N, cl);
    // psi_inv is smooth: the cell of slice z + 1 is about this one plus a slice, so
    // the rows it adds (two slices above the floor corner) are fetched into L2 now
    prefetch_l2(LT + min(cl.base + 2 * XYp, N - 1));
    prefetch_l2(LT + min(cl.base + 2 * XYp + Xp, N - 1));

    // Jacobian of psi_inv, row r = d(psi_inv_r)/d(x, y, z), and its determinant
    float M[3][3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        M[r][0] = (Q(1, r)[1] - Q(1, r)[-1]) * 0.5f;
        M[r][1] = (Q(1, r)[RW] - Q(1, r)[-RW]) * 0.5f;
        M[r][2] = (Q(2, r)[0] - Q(0, r)[0]) * 0.5f;
    }
    const float det = det_ref(M);

    // central-difference gradient of S and the potential gradient
    // rho and S are read through L1 (their 7-point stencils stay in cache)
    const float Si = Q(1, 4)[0];
    if (z + 3 < Z) {  // the S and rho slice this column reads three steps on
        prefetch_l2(Sg + i + 3 * XYp);
        prefetch_l2(Rg + i + 3 * XYp);
    }
    const float gs[3] = {(Q(1, 4)[1] - Q(1, 4)[-1]) * 0.5f,
                         (Q(1, 4)[RW] - Q(1, 4)[-RW]) * 0.5f,
                         (Q(2, 4)[0] - Q(0, 4)[0]) * 0.5f};

    // velocity and its 6 neighbours (vb[2] is slice z)
    float vc[3], vxm[3], vxp[3], vym[3], vyp[3], vzm[3], vzp[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        vc[c] = V(2, c)[0];
        vxm[c] = V(2, c)[-1];
        vxp[c] = V(2, c)[1];
        vym[c] = V(2, c)[-RW];
        vyp[c] = V(2, c)[RW];
        vzm[c] = V(1, c)[0];
        vzp[c] = V(3, c)[0];
    }
    const float vx = vc[0], vy = vc[1], vz = vc[2];

    // divergence of rho*v (upwind) and the density update
    const float* rb = Q(1, 3);
    const float p = rb[0];
    const float t11 = (vx > 0.f) ? (-vx) * p : (-vx) * rb[1];
    const float t12 = (vxm[0] > 0.f) ? vxm[0] * rb[-1] : vxm[0] * p;
    const float t21 = (vy > 0.f) ? (-vy) * p : (-vy) * rb[RW];
    const float t22 = (vym[1] > 0.f) ? vym[1] * rb[-RW] : vym[1] * p;
    const float t31 = (vz > 0.f) ? (-vz) * p : (-vz) * Q(2, 3)[0];
    const float t32 = (vzm[2] > 0.f) ? vzm[2] * Q(0, 3)[0] : vzm[2] * p;
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
    const float dvv[3] = {(0.5f * ax1 + ax2) + ax3, (ay1 + 0.5f * ay2) + ay3,
                          (az1 + az2) + 0.5f * az3};

    // negated upwind second differences of v (x in [2,X-3], y in [2,Y-2],
    // z in [2,Z-3]); the y and z forward branches read (+2, -1, 0) as the
    // reference does; y+2 at y = Y-2 reads index i + 2 rows (voxel (x, 0, z+1))
    // from global memory, as the reference's unchecked read does
    float dv[3] = {0.f, 0.f, 0.f};
    if (dv_xy && z >= 2 && z <= Z - 3) {
        const bool y_edge = y + 2 > Y - 1;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float xx = (vx < 0.f) ? (V(2, c)[2] - 2.f * vxp[c]) + vc[c]
                                        : (vc[c] - 2.f * vxm[c]) + V(2, c)[-2];
            const float vyp2 = y_edge ? __ldg(Vg[c] + i + 2 * Xp) : V(2, c)[2 * RW];
            const float yy = (vy < 0.f) ? (vyp2 - 2.f * vym[c]) + vc[c]
                                        : (vc[c] - 2.f * vym[c]) + V(2, c)[-2 * RW];
            const float zz = (vz < 0.f) ? (V(4, c)[0] - 2.f * vzm[c]) + vc[c]
                                        : (vc[c] - 2.f * vzm[c]) + V(0, c)[0];
            dv[c] = -1.f * ((xx + yy) + zz);
        }
    }

    // the potential gradient, from the gathered (L, T) o psi_inv: used as late as the
    // arithmetic allows, so that the work above overlaps the gather's latency
    const float Tq = a.first_iter ? __ldg(Tg + i) : lt.w;
    const float Lq[3] = {lt.x, lt.y, lt.z};
    const float diff = Si - Tq;
    float gU[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) gU[c] = ((diff * gs[c]) + (P.w_reg * Lq[c])) * det;

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

__global__ void __launch_bounds__(256, 3) ref_pass_a_kernel(RefIterArgs a) {
    extern __shared__ __align__(16) float smem[];
    PassASmem sm;
    sm.v = smem;
    sm.q = sm.v + 3 * kVS * kVPlane;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;

    for (int t = blockIdx.x; t < a.ntiles_a; t += gridDim.x) {
        const Tile tl = a.tiles_a[t];
        if (a.stop[tl.x]) continue;  // uniform over the block
        const Pair P = a.pairs[tl.x];
        const int X = P.X, Y = P.Y, Z = P.Z, N = (int)P.N;
        const int Xp = P.Xp, XYp = P.Xp * P.Y;  // strides of the packed arrays
        const int zs0 = max(tl.w, 1), zs1 = min(tl.w + a.depth_a, Z - 1);
        if (zs0 >= zs1 || tl.y + kTileX <= 1 || tl.z + kTileY <= 1 || tl.y >= X - 1 || tl.z >= Y - 1) continue;
        const long long NT = a.NT;
        const float* __restrict__ Vg[3] = {a.v + P.off, a.v + NT + P.off, a.v + 2 * NT + P.off};
        const float* __restrict__ Qg[3] = {a.pinv + P.off, a.pinv + NT + P.off, a.pinv + 2 * NT + P.off};
        const float* __restrict__ Rg = a.rho + P.off;
        const float* __restrict__ Sg = a.S + P.off;
        const float* __restrict__ Tg = a.T + P.off;
        const float4* __restrict__ LT = a.LT + P.off;
        float* rho_n = a.rho_n + P.off;
        float* Vn[3] = {a.v_n + P.off, a.v_n + NT + P.off, a.v_n + 2 * NT + P.off};
        float* Qn[3] = {a.pinv_n + P.off, a.pinv_n + NT + P.off, a.pinv_n + 2 * NT + P.off};
        const int x0 = tl.y, y0 = tl.z;
        const int x = x0 + tx, y = y0 + ty;
        const bool active = x >= 1 && x <= X - 2 && y >= 1 && y <= Y - 2;
        const bool dv_xy = x >= 2 && x <= X - 3 && y >= 2 && y <= Y - 2;

        auto vslot = [](int zs) { return ((zs % kVS) + kVS) % kVS; };
        auto qslot = [](int zs) { return ((zs % kQS) + kQS) % kQS; };
        const int gv = stage_offset<kVH>(threadIdx.x, Y, Xp, x0, y0);
        const int gq = stage_offset<kQH>(threadIdx.x, Y, Xp, x0, y0);
        auto stage_v_at = [&](int zs, int sl) {  // slice zs of v's three components into slot sl
            if (gv < 0 || zs < 0 || zs >= Z) return;
            float* dst = sm.v + sl * kVPlane + 4 * threadIdx.x;
            const int off = gv + XYp * zs;
#pragma unroll
            for (int c = 0; c < 3; ++c) cp_async16(dst + c * kVS * kVPlane, Vg[c] + off);
        };
        auto stage_v = [&](int zs) { stage_v_at(zs, vslot(zs)); };
        auto stage_q_at = [&](int zs, int sl) {  // slice zs of psi_inv's three components, rho and S
            if (gq < 0 || zs < 0 || zs >= Z) return;
            float* dst = sm.q + sl * kQPlane + 4 * threadIdx.x;
            const int off = gq + XYp * zs;
#pragma unroll
            for (int c = 0; c < 3; ++c) cp_async16(dst + c * kQS * kQPlane, Qg[c] + off);
            cp_async16(dst + 3 * kQS * kQPlane, Rg + off);
            cp_async16(dst + 4 * kQS * kQPlane, Sg + off);
        };
        auto stage_q = [&](int zs) { stage_q_at(zs, qslot(zs)); };

        __syncthreads();  // the previous tile is done with the ring buffers
        // prologue: everything slice zs0 needs, then what each of the next kAhead - 1
        // slices adds (one commit group per slice)
        for (int zs = zs0 - 2; zs <= zs0 + 2; ++zs) stage_v(zs);
        for (int zs = zs0 - 1; zs <= zs0 + 1; ++zs) stage_q(zs);
        cp_async_commit();
#pragma unroll
        for (int k = 1; k < kAhead; ++k) {
            if (zs0 + 2 + k <= zs1 + 1) stage_v(zs0 + 2 + k);
            if (zs0 + 1 + k <= zs1) stage_q(zs0 + 1 + k);
            cp_async_commit();
        }

        // this thread's column in the staged slices z - 2 .. z + 2 of v and z - 1 .. z + 1 of
        // psi_inv/rho/S, rotated by one slice per step; with one slice in flight, the slice
        // staged at step z (z + 3 of v, z + 2 of psi_inv) goes into the slot of slice z - 3 /
        // z - 2, and that slot is the newest one read at step z + 1
        static_assert(kAhead == 1 && kVS == 6 && kQS == 4, "the slot rotation below assumes these rings");
        const int vc0 = (ty + kVH) * kVW + tx + kXO;
        const int qc0 = (ty + kQH) * kQW + tx + kXO;
        const float* vb[5];
        const float* qb[3];
#pragma unroll
        for (int k = 0; k < 5; ++k) vb[k] = sm.v + vslot(zs0 - 2 + k) * kVPlane + vc0;
#pragma unroll
        for (int k = 0; k < 3; ++k) qb[k] = sm.q + qslot(zs0 - 1 + k) * kQPlane + qc0;
        int sv = vslot(zs0 - 3), sq = qslot(zs0 - 2);  // the slots step zs0 stages into
        for (int z = zs0; z < zs1; ++z) {
            cp_async_wait<kAhead - 1>();  // slice z's group has landed (the newer ones may not)
            __syncthreads();              // ... for every thread, and slice z - 3 / z - 2 is no longer read
            // prefetch what slice z + 1 adds, into the slots of slices z - 3 (v) and z - 2
            if (z + 3 <= zs1 + 1) stage_v_at(z + 3, sv);  // the last slice reads v up to zs1 + 1
            if (z + 2 <= zs1) stage_q_at(z + 2, sq);      // and psi_inv up to zs1
            cp_async_commit();
            if (active) {
                const int i = x + Xp * y + XYp * z;
                pass_a_voxel<kVS * kVPlane, kQS * kQPlane, 3 * kQS * kQPlane, 4 * kQS * kQPlane, kVW>(
                    a, P, X, Y, Z, N, Xp, XYp, y, z, i, dv_xy, vb, qb, LT, Tg, Sg, Rg, Vg, rho_n, Vn, Qn);
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) vb[k] = vb[k + 1];
            vb[4] = sm.v + sv * kVPlane + vc0;
            qb[0] = qb[1];
            qb[1] = qb[2];
            qb[2] = sm.q + sq * kQPlane + qc0;
            sv = sv + 1 == kVS ? 0 : sv + 1;
            sq = (sq + 1) & 3;
        }
        cp_async_wait<0>();
    }
}

// ----------------------------------------------------------------------------------
// Pass A with TMA staging.  Per slice, one thread issues four tensor copies: v's box of 40
// columns x 12 rows x 3 components (2-voxel halo) into the v ring, and psi_inv's 40 x 10 x
// 3 box, rho's and S's 40 x 10 boxes into one slot of the psi_inv ring; each ring slot
// completes on its own mbarrier.  The v ring holds the 5 slices z - 2 .. z + 2 and the
// psi_inv ring the 3 slices z - 1 .. z + 1 that slice z reads, each with one more slice in
// flight; one block barrier per slice frees the slots of slices z - 3 / z - 2 for the next
// copies.  Out-of-volume parts of a box read as zero and are never used (the stencils
// that reach them are masked, as in the cp.async kernel).  Waits are bounded as in
// ref_laplacian_tma_kernel.  The voxel arithmetic is pass_a_voxel, shared with
// ref_pass_a_kernel.
// ----------------------------------------------------------------------------------
namespace {
constexpr int kPVS = 6, kPQS = 4;                 // ring slots: v (5 + 1), psi_inv/rho/S (3 + 1)
constexpr int kPW = 40;                           // staged row: columns x0 - 4 .. x0 + 35
constexpr int kPVPlane = kPW * 12, kPVSlot = 3 * kPVPlane;  // 1440 floats = 5760 bytes
constexpr int kPQPlane = kPW * 10;
constexpr int kPQR = 1216, kPQSo = 1632, kPQSlot = 2048;    // rho, S offsets; slot (floats)
constexpr unsigned kPVBytes = sizeof(float) * kPVSlot;
constexpr unsigned kPQBytes = sizeof(float) * (3 * kPQPlane + 2 * kPQPlane);
static_assert((kPVSlot * 4) % 128 == 0 && (kPQR * 4) % 128 == 0 && (kPQSo * 4) % 128 == 0 &&
                  3 * kPQPlane <= kPQR && kPQR + kPQPlane <= kPQSo && kPQSo + kPQPlane <= kPQSlot,
              "slot layout");
}  // namespace

size_t ref_pass_a_tma_smem_bytes() {
    return 128 + sizeof(float) * (kPVS * kPVSlot + kPQS * kPQSlot) + sizeof(uint64_t) * (kPVS + kPQS);
}

__global__ void __launch_bounds__(256, 3) ref_pass_a_tma_kernel(RefIterArgs a) {
    extern __shared__ __align__(128) unsigned char pa_raw[];
    float* vring = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(pa_raw) + 127) & ~uintptr_t(127));
    float* qring = vring + kPVS * kPVSlot;
    uint64_t* fullv = reinterpret_cast<uint64_t*>(qring + kPQS * kPQSlot);
    uint64_t* fullq = fullv + kPVS;
    typedef SliceRing<kPVS> VRing;
    typedef SliceRing<kPQS> QRing;
    const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
    if (tid == 0) {
        for (int k = 0; k < kPVS; ++k) mbar_init(fullv + k, 1);
        for (int k = 0; k < kPQS; ++k) mbar_init(fullq + k, 1);
        mbar_fence_init();
    }
    __syncthreads();
    const int src = (a.iter - 1) & 1;  // the buffers this iteration reads
    unsigned nbv = 0, nbq = 0, iv = 0, iq = 0;  // fills before this tile; fills issued (thread 0)
    bool failed = false;
    for (int t = blockIdx.x; t < a.ntiles_a && !failed; t += gridDim.x) {
        const Tile tl = a.tiles_a[t];
        if (a.stop[tl.x]) continue;  // uniform over the block
        const Pair P = a.pairs[tl.x];
        const int X = P.X, Y = P.Y, Z = P.Z, N = (int)P.N;
        const int Xp = P.Xp, XYp = P.Xp * P.Y;
        const int zs0 = max(tl.w, 1), zs1 = min(tl.w + a.depth_a, Z - 1);
        if (zs0 >= zs1 || tl.y + kTileX <= 1 || tl.z + kTileY <= 1 || tl.y >= X - 1 || tl.z >= Y - 1) continue;
        const long long NT = a.NT;
        const float* __restrict__ Vg[3] = {a.v + P.off, a.v + NT + P.off, a.v + 2 * NT + P.off};
        const float* __restrict__ Rg = a.rho + P.off;
        const float* __restrict__ Sg = a.S + P.off;
        const float* __restrict__ Tg = a.T + P.off;
        const float4* __restrict__ LT = a.LT + P.off;
        float* rho_n = a.rho_n + P.off;
        float* Vn[3] = {a.v_n + P.off, a.v_n + NT + P.off, a.v_n + 2 * NT + P.off};
        float* Qn[3] = {a.pinv_n + P.off, a.pinv_n + NT + P.off, a.pinv_n + 2 * NT + P.off};
        const int pair = tl.x;
        const int x0 = tl.y, y0 = tl.z;
        const int x = x0 + tx, y = y0 + ty;
        const bool active = x >= 1 && x <= X - 2 && y >= 1 && y <= Y - 2;
        const bool dv_xy = x >= 2 && x <= X - 3 && y >= 2 && y <= Y - 2;
        const int nsteps = zs1 - zs0;
        const int nv = nsteps + 4, nq = nsteps + 2;  // v slices zs0 - 2 .. zs1 + 1; psi_inv zs0 - 1 .. zs1
        // the copies (thread 0 only); the maps' addresses are formed where they are used
        auto issue_v = [&](int f) {
            const unsigned n = nbv + (unsigned)f;
            uint64_t* bar = fullv + VRing::slot(n);
            const CUtensorMap* mv = a.tmaps + (long long)pair * TM_COUNT + TM_PA_V0 + src;
            mbar_arrive_expect_tx(bar, kPVBytes);
            tma_load_4d(vring + VRing::slot(n) * kPVSlot, mv, x0 - 4, y0 - 2, zs0 - 2 + f, 0, bar);
            ++iv;
        };
        auto issue_q = [&](int f) {
            const unsigned n = nbq + (unsigned)f;
            uint64_t* bar = fullq + QRing::slot(n);
            float* dst = qring + QRing::slot(n) * kPQSlot;
            const CUtensorMap* maps = a.tmaps + (long long)pair * TM_COUNT;
            const int z = zs0 - 1 + f;
            mbar_arrive_expect_tx(bar, kPQBytes);
            tma_load_4d(dst, maps + TM_PA_Q0 + src, x0 - 4, y0 - 1, z, 0, bar);
            tma_load_3d(dst + kPQR, maps + TM_PA_R0 + src, x0 - 4, y0 - 1, z, bar);
            tma_load_3d(dst + kPQSo, maps + TM_PA_S, x0 - 4, y0 - 1, z, bar);
            ++iq;
        };
        __syncthreads();  // the previous tile is done with the rings
        if (tid == 0) {
            for (int f = 0; f < min(nv, kPVS); ++f) issue_v(f);
            for (int f = 0; f < min(nq, kPQS); ++f) issue_q(f);
        }
        const int vc0 = (ty + 2) * kPW + tx + 4;
        const int qc0 = (ty + 1) * kPW + tx + 4;
        for (int j0 = 0; j0 < nsteps; ++j0) {
            // slice z = zs0 + j0 reads v fills j0 .. j0 + 4 and psi_inv fills j0 .. j0 + 2
            bool ok = true;
            for (int f = (j0 == 0 ? 0 : j0 + 4); f <= j0 + 4; ++f)
                ok = ok && mbar_wait_bounded(fullv + VRing::slot(nbv + f), VRing::parity(nbv + f));
            for (int f = (j0 == 0 ? 0 : j0 + 2); f <= j0 + 2; ++f)
                ok = ok && mbar_wait_bounded(fullq + QRing::slot(nbq + f), QRing::parity(nbq + f));
            // every thread is past slice z - 1: the slots of v fill j0 - 1 and psi_inv fill
            // j0 - 1 are free; the block agrees on whether any wait gave up
            if (__syncthreads_or(!ok)) {
                failed = true;
                break;
            }
            if (tid == 0 && j0 >= 1) {
                if (j0 - 1 + kPVS < nv) issue_v(j0 - 1 + kPVS);
                if (j0 - 1 + kPQS < nq) issue_q(j0 - 1 + kPQS);
            }
            if (active) {
                const int z = zs0 + j0;
                const int i = x + Xp * y + XYp * z;
                const float* vb[5];
#pragma unroll
                for (int k = 0; k < 5; ++k) vb[k] = vring + VRing::slot(nbv + j0 + k) * kPVSlot + vc0;
                const float* qb[3];
#pragma unroll
                for (int k = 0; k < 3; ++k) qb[k] = qring + QRing::slot(nbq + j0 + k) * kPQSlot + qc0;
                pass_a_voxel<kPVPlane, kPQPlane, kPQR, kPQSo, kPW>(a, P, X, Y, Z, N, Xp, XYp, y, z, i, dv_xy, vb, qb,
                                                                   LT, Tg, Sg, Rg, Vg, rho_n, Vn, Qn);
            }
        }
        nbv += (unsigned)nv;  // every fill of the tile has been waited for
        nbq += (unsigned)nq;
    }
    if (failed && tid == 0) {
        for (unsigned n = (iv > (unsigned)kPVS ? iv - kPVS : 0u); n < iv; ++n)
            mbar_wait_bounded(fullv + VRing::slot(n), VRing::parity(n));
        for (unsigned n = (iq > (unsigned)kPQS ? iq - kPQS : 0u); n < iq; ++n)
            mbar_wait_bounded(fullq + QRing::slot(n), QRing::parity(n));
        atomicOr(a.err, kErrTmaTimeout);
    }
}

// ----------------------------------------------------------------------------------
// pass B: psi += alpha * v o psi, max update norm, convergence
//
// One thread per column of a 32 x 4 tile (128-thread blocks): the kernel waits on its
// gathers, and 9 blocks of 128 threads at 56 registers hold 36 warps per SM where 256-thread
// blocks held 32 (at 64 registers; at 48, for 5 blocks of 256, it spills).
// ----------------------------------------------------------------------------------
__global__ void __launch_bounds__(kPassBThreads, 9) ref_pass_b_kernel(RefIterArgs a) {
    __shared__ unsigned long long red[32];
    __shared__ bool last;
    const int tid = threadIdx.x;
    for (int t = blockIdx.x; t < a.ntiles_b; t += gridDim.x) {
        const Tile tl = a.tiles_b[t];
        if (a.stop[tl.x]) continue;  // uniform over the block
        const Pair P = a.pairs[tl.x];
        const int x = tl.y + (int)(threadIdx.x & 31), y = tl.z + (int)(threadIdx.x >> 5);
        unsigned long long best = 0ull;
        if (x >= 1 && x <= P.X - 2 && y >= 1 && y <= P.Y - 2) {
            const int X = P.X, Y = P.Y, Z = P.Z, Xp = P.Xp, XYp = P.Xp * P.Y;
            const long long NT = a.NT;
            // the velocity pass A just wrote
            const float* __restrict__ V[3] = {a.v_n + P.off, a.v_n + NT + P.off, a.v_n + 2 * NT + P.off};
            float* Q[3] = {a.psi + P.off, a.psi + NT + P.off, a.psi + 2 * NT + P.off};
            const int z0 = max(tl.w, 1), z1 = min(tl.w + a.depth_b, P.Z - 1);
            int i = x + Xp * y + XYp * z0;
            // psi of the next slice is loaded while this slice's gathers are in flight
            float nx = 0.f, ny = 0.f, nz = 0.f;
            if (z0 < z1) {
                nx = Q[0][i];
                ny = Q[1][i];
                nz = Q[2][i];
            }
            for (int z = z0; z < z1; ++z, i += XYp) {
                const float px = nx, py = ny, pz = nz;
                if (z + 1 < z1) {
                    nx = Q[0][i + XYp];
                    ny = Q[1][i + XYp];
                    nz = Q[2][i + XYp];
                }
                const Cell32 cl = locate32(X, Y, Z, Xp, px, py, pz);
                float vp[3];
                tri_checked32_3(V[0], V[1], V[2], X, Y, Z, Xp, XYp, cl, vp);
                const float ux = a.alpha * vp[0];
                const float uy = a.alpha * vp[1];
                const float uz = a.alpha * vp[2];
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


// ----------------------------------------------------------------------------------
// Pass B with the gathered neighbourhood staged in shared memory.  Per slice of its tile
// the block reduces the bounding box of its voxels' cells (cellbox_add) and, when the
// cells fit a kGBX x kGBY x kGBZ box, one thread copies that box of v's three components
// with one tensor copy; the corners are then read from shared memory.  The copy of slice
// z + 1's box is issued while slice z is gathered (two buffers), and the slice's one block
// barrier both publishes the next box and frees the buffer of slice z - 1.  Voxels whose
// cell has a corner outside the grid (they read element 0, as get_global_idx does) and
// slices whose cells do not fit the box gather from global memory as ref_pass_b_kernel
// does; the arithmetic is the same.  Waits are bounded (about a second); a block that gives
// up sets the device error word.
// ----------------------------------------------------------------------------------
namespace {
constexpr int kGBPlane = kGBX * kGBY * kGBZ;  // one component of a box (floats)
constexpr unsigned kGBBytes = sizeof(float) * 3 * kGBPlane;
}  // namespace

size_t gather_staged_smem_bytes() { return 128 + 2 * (size_t)kGBBytes + 2 * sizeof(uint64_t); }

__global__ void __launch_bounds__(256, 4) ref_pass_b_staged_kernel(RefIterArgs a) {
    extern __shared__ __align__(128) unsigned char gb_raw[];
    float* box = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(gb_raw) + 127) & ~uintptr_t(127));
    uint64_t* full = reinterpret_cast<uint64_t*>(box + 2 * 3 * kGBPlane);
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
    const int dst = a.iter & 1;  // the velocity buffer pass A just wrote
    unsigned g = 0;       // slices reduced by this block (cell-box set g % 3)
    unsigned nbox = 0;    // boxes issued by this block (buffer nbox & 1, parity (nbox >> 1) & 1)
    bool failed = false, wait_failed = false;
    for (int t = blockIdx.x; t < a.ntiles_b && !failed; t += gridDim.x) {
        const Tile tl = a.tiles_b[t];
        if (a.stop[tl.x]) continue;  // uniform over the block
        const Pair P = a.pairs[tl.x];
        const int x = tl.y + (int)(tid & 31), y = tl.z + (int)(tid >> 5);
        const int X = P.X, Y = P.Y, Z = P.Z, Xp = P.Xp, XYp = P.Xp * P.Y;
        const bool col = x >= 1 && x <= X - 2 && y >= 1 && y <= Y - 2;
        const long long NT = a.NT;
        const float* __restrict__ V[3] = {a.v_n + P.off, a.v_n + NT + P.off, a.v_n + 2 * NT + P.off};
        float* Q[3] = {a.psi + P.off, a.psi + NT + P.off, a.psi + 2 * NT + P.off};
        const CUtensorMap* mv = a.tmaps + (long long)tl.x * TM_COUNT + TM_PB_V0 + dst;
        const int z0 = max(tl.w, 1), z1 = min(tl.w + a.depth_b, Z - 1);
        unsigned long long best = 0ull;
        // the slice being prepared: positions, cell, and whether its box was issued (and where)
        float px = 0.f, py = 0.f, pz = 0.f;
        Cell32 cl{};
        int i = x + Xp * y + XYp * z0;
        if (col && z0 < z1) {
            px = Q[0][i];
            py = Q[1][i];
            pz = Q[2][i];
            cl = locate32(X, Y, Z, Xp, px, py, pz);
        }
        // box of a reduced slice: issue it when it fits (uniform decision); returns the box
        // origin in o[] and whether it was issued
        auto plan = [&](unsigned set, int zz, int o[3]) -> bool {
            int lo[3], hi[3];
            if (!cellbox_read(cb, (int)set, lo, hi)) return false;
            o[0] = lo[0] & ~3;
            o[1] = lo[1];
            o[2] = lo[2];
            const bool fits = hi[0] + 1 - o[0] < kGBX && hi[1] + 1 - o[1] < kGBY && hi[2] + 1 - o[2] < kGBZ;
            if (fits && tid == 0) {
                uint64_t* bar = full + (nbox & 1);
                mbar_arrive_expect_tx(bar, kGBBytes);
                tma_load_4d(box + (nbox & 1) * 3 * kGBPlane, mv, o[0], o[1], o[2], 0, bar);
            }
            return fits;
        };
        // prologue: the first slice's box (a fresh set: the previous tile's last one may
        // still be read by slower threads)
        ++g;
        cellbox_add(cb, (int)(g % 3), col && z0 < z1, cl.gx, cl.gy, cl.gz);
        if (__syncthreads_or(wait_failed)) {
            failed = true;
            break;
        }
        if (tid == 0) cellbox_clear(cb, (int)((g - 1) % 3));
        int org[3] = {0, 0, 0};
        bool staged = plan(g % 3, z0, org);
        unsigned mybox = nbox;
        if (staged) ++nbox;
        for (int z = z0; z < z1; ++z, i += XYp) {
            // this slice's state
            const float cx = px, cy = py, cz = pz;
            const Cell32 c = cl;
            const bool cur_staged = staged;
            const unsigned cur_box = mybox;
            const int o0 = org[0], o1 = org[1], o2 = org[2];
            // the next slice's positions and cell, its box reduced and issued
            const bool nact = col && z + 1 < z1;
            if (nact) {
                px = Q[0][i + XYp];
                py = Q[1][i + XYp];
                pz = Q[2][i + XYp];
                cl = locate32(X, Y, Z, Xp, px, py, pz);
            }
            ++g;
            cellbox_add(cb, (int)(g % 3), nact, cl.gx, cl.gy, cl.gz);
            // every thread is past slice z - 1 (its buffer is free), the next box is
            // reduced, and the block agrees on whether a wait gave up
            if (__syncthreads_or(wait_failed)) {
                failed = true;
                break;
            }
            if (tid == 0) cellbox_clear(cb, (int)((g - 1) % 3));
            staged = plan(g % 3, z + 1, org);
            mybox = nbox;
            if (staged) ++nbox;
            if (!col) continue;
            float u[3];
            const bool inside = c.gx + 1 < X && c.gy + 1 < Y && c.gz + 1 < Z;
            if (cur_staged && inside) {
                if (!mbar_wait_bounded(full + (cur_box & 1), (cur_box >> 1) & 1)) wait_failed = true;
                const float* b0 = box + (cur_box & 1) * 3 * kGBPlane + ((c.gz - o2) * kGBY + (c.gy - o1)) * kGBX +
                                  (c.gx - o0);
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const float* f = b0 + k * kGBPlane;
                    constexpr int SX = 1, SY = kGBX, SZ = kGBX * kGBY;
                    u[k] = a.alpha * trilerp(f[SX + SY + SZ], f[SX + SY], f[SX + SZ], f[SX], f[SY + SZ], f[SY],
                                             f[SZ], f[0], c.a, c.b, c.c);
                }
            } else {
                if (cur_staged && !mbar_wait_bounded(full + (cur_box & 1), (cur_box >> 1) & 1)) wait_failed = true;
#pragma unroll
                for (int k = 0; k < 3; ++k) u[k] = a.alpha * tri_checked32(V[k], X, Y, Z, Xp, XYp, c);
            }
            Q[0][i] = cx + u[0];
            Q[1][i] = cy + u[1];
            Q[2][i] = cz + u[2];
            const float nrm = norm3_rd(u[0], u[1], u[2]);
            if (nrm == nrm) {  // NaN norms never win, as in the reference's '>' test
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
        return;  // the iteration's record is left to the blocks that finished
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
