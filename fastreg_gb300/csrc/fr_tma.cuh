// fr_tma.cuh -- tensor-memory-accelerator (TMA) staging: bulk tensor copies of a box of a
// field into shared memory, completed on an mbarrier.
//
// One elected thread of a block issues a whole box (tile rows plus halo, of one slice,
// all components of a field at once) with a single cp.async.bulk.tensor; the copy lands
// in shared memory and signals the slot's mbarrier with its byte count.  Consumers wait
// on the barrier's phase parity.  Every wait here is bounded: after about a second of
// device time it gives up and reports failure, and the kernel then records an error word
// for the host instead of hanging.
//
// Tensor maps (CUtensorMap, 128 bytes, 64-byte aligned) are encoded on the host per pair
// and per field (fr_api.cu) and live in device memory; a kernel passes their generic
// address to the copy.  They cover this GPU's own memory only; no multicast is used.
#pragma once

#include <cuda.h>
#include <cstdint>

namespace frg {

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// make barrier initialisation visible to the async (TMA) proxy
__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// this thread arrives and the phase also waits for `bytes` of copies
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Wait for the phase of parity `parity` to complete; false if it has not after about
// 2^31 clock cycles (about a second at the GB300's clocks).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    for (;;) {
        for (int k = 0; k < 64; ++k)
            if (mbar_try_wait(bar, parity)) return true;
        if (clock64() - t0 > (1LL << 31)) return false;
    }
}

// 3-D / 4-D tiled tensor copies, global -> this block's shared memory, completing on `bar`.
// The innermost coordinate x times the element size must be a multiple of 16 bytes.
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_u32(dst)),
        "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, int x, int y, int z, int w,
                                            uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5}], [%6];" ::"r"(smem_u32(dst)),
        "l"(map), "r"(x), "r"(y), "r"(z), "r"(w), "r"(smem_u32(bar))
        : "memory");
}

// fetch a tensor map's descriptor ahead of its first use
__device__ __forceinline__ void tma_prefetch_map(const CUtensorMap* map) {
    asm volatile("prefetch.tensormap [%0];" ::"l"(map) : "memory");
}

// A ring of `S` slots filled in order by one producer thread: slice n of the block's
// stream of slices goes to slot n % S, and the k-th fill of a slot completes phase k of its
// barrier (parity k & 1).
template <int S>
struct SliceRing {
    __device__ __forceinline__ static int slot(unsigned n) { return (int)(n % S); }
    __device__ __forceinline__ static unsigned parity(unsigned n) { return (n / S) & 1u; }
};

// Codes of the device error word (RefIterArgs::err, SobIterArgs::err).
constexpr unsigned kErrTmaTimeout = 1u;

// ---- a slice's source neighbourhood: the bounding box of the block's trilinear cells ----
// The gathers of the update kernels read, per voxel, the eight corners of the cell that
// holds its sample position.  The map is smooth, so the cells of one slice of a 32 x 8
// tile lie in a small box of the gathered field; the box is copied into shared memory by
// one tensor copy and the corners are read from there.  The box of slice j is reduced
// over the block into set j % 3 of a CellBoxSets (min of gx, gy, gz and of their
// negations): redux.sync per warp, one shared-memory atomicMin per warp and value, and
// one block barrier, after which every thread reads it.  Three sets rotate so that one
// barrier per slice suffices: set j % 3 is cleared by thread 0 after barrier j + 1 (all
// threads have read it) and refilled after barrier j + 2.
struct CellBoxSets {
    int v[3][6];
};
constexpr int kCellBoxEmpty = 0x7fffffff;

__device__ __forceinline__ void cellbox_clear(CellBoxSets& s, int set) {
    for (int k = 0; k < 6; ++k) s.v[set][k] = kCellBoxEmpty;
}

// every thread of the block calls it; act: this thread has a cell in the slice
__device__ __forceinline__ void cellbox_add(CellBoxSets& s, int set, bool act, int gx, int gy, int gz) {
    const unsigned full = 0xffffffffu;
    int r[6] = {act ? gx : kCellBoxEmpty,  act ? gy : kCellBoxEmpty,  act ? gz : kCellBoxEmpty,
                act ? -gx : kCellBoxEmpty, act ? -gy : kCellBoxEmpty, act ? -gz : kCellBoxEmpty};
#pragma unroll
    for (int k = 0; k < 6; ++k) r[k] = __reduce_min_sync(full, r[k]);
    if ((threadIdx.x & 31) == 0 && r[0] != kCellBoxEmpty)
#pragma unroll
        for (int k = 0; k < 6; ++k) atomicMin(&s.v[set][k], r[k]);
}

// after the barrier: the box of set `set`, cells' floor corners gx in [lo[0], hi[0]] etc.;
// false if the slice had no cell
__device__ __forceinline__ bool cellbox_read(const CellBoxSets& s, int set, int lo[3], int hi[3]) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        lo[k] = s.v[set][k];
        hi[k] = -s.v[set][3 + k];
    }
    return lo[0] != kCellBoxEmpty;
}

}  // namespace frg
