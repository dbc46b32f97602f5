// fr_limits.h -- when a volume may be addressed with 32-bit voxel indices.
//
// The 32-bit kernels (the solver kernels inside one pair, warp2_kernel) form corner and
// prefetch offsets from a cell's floor corner b <= N - 1 by adding up to two slices, a
// row and one voxel (b + 1 + X + XY for the far corner of a cell, b + 2 XY + X for the
// rows the next slice's cell adds), and only then clamp them to the last voxel.  Those
// sums must not overflow an int, so a volume of pitch Xp and Y rows per slice takes the
// 32-bit path only when N + 2 XY + 2 Xp + 2 <= 2^31 - 1 (N = Xp * Y * Z).  Header-only,
// plain C++: the host code includes it, and a CPU test compiles it on its own.
#pragma once

namespace frg {

constexpr long long kIndex32Max = 0x7fffffffLL;

inline bool fits_index32(long long Xp, long long Y, long long Z) {
    if (Xp < 1 || Y < 1 || Z < 1) return false;
    const long long XY = Xp * Y;
    if (XY > kIndex32Max) return false;
    const long long N = XY * Z;
    if (N / Z != XY || N > kIndex32Max) return false;
    return N + 2 * XY + 2 * Xp + 2 <= kIndex32Max;
}

}  // namespace frg
