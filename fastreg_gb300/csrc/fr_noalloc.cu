// fr_noalloc.cu -- registration statistics for callers that cannot allocate device memory.
//
// fr_stats_noalloc computes, for one registered pair, the same statistics that
// fr_get_stats reports after fr_register (the reference's Reductor::energy,
// reductor.cpp:45-62, and Dice, solver.cu:9-50, plus the fold count), from buffers
// the caller already holds.  Some callers cannot call cudaMalloc at that point: a
// process whose device memory is handed out by another framework's pool, a
// real-time pipeline that forbids allocation after start-up, or code running where
// an allocation would synchronise the device.  For them the per-block partial sums
// and the Dice bins live in one file-scope __device__ array, g_stats_scratch, of a
// fixed size (FR_NOALLOC_SCRATCH_BYTES = 28,712 bytes).  The function allocates
// nothing.  Its first call on a device looks up the array's device address; with CUDA's
// lazy module loading that lookup loads this file's module onto the device (which may
// allocate device memory once), so callers make that first call at start-up.  The array
// then stays on the device until the process exits; the address is kept per device and
// is not looked up again, so the function is not for use after cudaDeviceReset.
//
// The array is shared by every call: each call clears what must start at zero, and
// calls whose work overlaps on the GPU (different streams, or different host
// threads on one device) race on it and must be serialised by the caller.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>

#include "../../include/fastreg_gb300.h"
#include "fr_common.cuh"

namespace frg {

constexpr int kStatsBlocks = 1024;  // fixed grid: one partial slot per block
constexpr int kStatsBins = 2 * 256 + 1;

struct StatsScratch {
    double e_data[kStatsBlocks];
    double e_reg[kStatsBlocks];
    long long folds[kStatsBlocks];
    unsigned long long dice[kStatsBins];  // inter[256], count[256], out of range
    double result_e[2];
    long long result_folds;
    unsigned int counter;
};

static_assert(sizeof(StatsScratch) == FR_NOALLOC_SCRATCH_BYTES, "scratch size is part of the C ABI");

static __device__ __align__(256) StatsScratch g_stats_scratch;

__device__ __forceinline__ float det_true_na(const float J[3][3]) {
    const float f00 = J[0][0] + 1.f, f11 = J[1][1] + 1.f, f22 = J[2][2] + 1.f;
    const float f01 = J[0][1], f02 = J[0][2], f10 = J[1][0], f12 = J[1][2], f20 = J[2][0], f21 = J[2][1];
    const float c0 = f11 * f22 - f12 * f21;
    const float c1 = f10 * f22 - f12 * f20;
    const float c2 = f10 * f21 - f11 * f20;
    return (f00 * c0 - f01 * c1) + f02 * c2;
}

__global__ void __launch_bounds__(256) stats_noalloc_kernel(const float* __restrict__ T,
                                                            const int16_t* __restrict__ labT,
                                                            const float* __restrict__ wS,
                                                            const int16_t* __restrict__ wlabS,
                                                            const float* __restrict__ psi, int X, int Y, int Z,
                                                            int no_labels, StatsScratch* scr) {
    __shared__ double red[32];
    __shared__ unsigned int hist[kStatsBins];
    __shared__ bool last;
    const int tid = threadIdx.x;
    for (int b = tid; b < kStatsBins; b += blockDim.x) hist[b] = 0u;
    __syncthreads();
    const long long N = (long long)X * Y * Z, XY = (long long)X * Y;
    double ed = 0.0, er = 0.0;
    long long folds = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + tid; i < N; i += (long long)gridDim.x * blockDim.x) {
        const int z = (int)(i / XY), y = (int)((i - z * XY) / X), x = (int)(i - z * XY - (long long)y * X);
        const float df = __ldg(T + i) - __ldg(wS + i);
        ed = fma((double)df, (double)df, ed);  // df * df is exact in FP64: same bits
        // deformation Jacobian with the mirrored one-sided boundary (vector_fields.cu:537-585)
        int x1 = x + 1, x2 = x - 1, y1 = y + 1, y2 = y - 1, z1 = z + 1, z2 = z - 1;
        if (x == 0) x2 = x + 1; else if (x == X - 1) x1 = x - 1;
        if (y == 0) y2 = y + 1; else if (y == Y - 1) y1 = y - 1;
        if (z == 0) z2 = z + 1; else if (z == Z - 1) z1 = z - 1;
        const long long ix1 = x1 + X * (y + (long long)Y * z), ix2 = x2 + X * (y + (long long)Y * z);
        const long long iy1 = x + X * (y1 + (long long)Y * z), iy2 = x + X * (y2 + (long long)Y * z);
        const long long iz1 = x + X * (y + (long long)Y * z1), iz2 = x + X * (y + (long long)Y * z2);
        const float cx1[3] = {(float)x1, (float)y, (float)z}, cx2[3] = {(float)x2, (float)y, (float)z};
        const float cy1[3] = {(float)x, (float)y1, (float)z}, cy2[3] = {(float)x, (float)y2, (float)z};
        const float cz1[3] = {(float)x, (float)y, (float)z1}, cz2[3] = {(float)x, (float)y, (float)z2};
        float J[3][3];
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            const float* __restrict__ Q = psi + r * N;
            J[r][0] = ((__ldg(Q + ix1) - cx1[r]) - (__ldg(Q + ix2) - cx2[r])) * 0.5f;
            J[r][1] = ((__ldg(Q + iy1) - cy1[r]) - (__ldg(Q + iy2) - cy2[r])) * 0.5f;
            J[r][2] = ((__ldg(Q + iz1) - cz1[r]) - (__ldg(Q + iz2) - cz2[r])) * 0.5f;
        }
        const float r0 = (J[0][0] * J[0][0] + J[0][1] * J[0][1]) + J[0][2] * J[0][2];
        const float r1 = (J[1][0] * J[1][0] + J[1][1] * J[1][1]) + J[1][2] * J[1][2];
        const float r2 = (J[2][0] * J[2][0] + J[2][1] * J[2][1]) + J[2][2] * J[2][2];
        er += (double)((r0 + r1) + r2);
        if (det_true_na(J) <= 0.f) folds++;
        if (x < X - 1 && y < Y - 1 && z < Z - 1) {
            const int la = __ldg(wlabS + i), lb = __ldg(labT + i);
            if (la < 0 || la >= no_labels || lb < 0 || lb >= no_labels) {
                atomicAdd(&hist[2 * 256], 1u);
            } else {
                atomicAdd(&hist[256 + la], 1u);
                atomicAdd(&hist[256 + lb], 1u);
                if (la == lb) atomicAdd(&hist[la], 1u);
            }
        }
    }
    ed = block_sum_f64(ed, red);
    er = block_sum_f64(er, red);
    const double fd = block_sum_f64((double)folds, red);
    if (tid == 0) {
        scr->e_data[blockIdx.x] = ed;
        scr->e_reg[blockIdx.x] = er;
        scr->folds[blockIdx.x] = (long long)fd;
    }
    for (int b = tid; b < kStatsBins; b += blockDim.x)
        if (hist[b]) atomicAdd(scr->dice + b, (unsigned long long)hist[b]);
    __threadfence();
    __syncthreads();
    if (tid == 0) last = (atomicAdd(&scr->counter, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!last || tid != 0) return;
    __threadfence();
    double se = 0.0, sr = 0.0;
    long long sf = 0;
    for (int b = 0; b < (int)gridDim.x; ++b) {  // fixed order: the same bits on every call
        se += scr->e_data[b];
        sr += scr->e_reg[b];
        sf += scr->folds[b];
    }
    scr->result_e[0] = 0.5 * se;
    scr->result_e[1] = 0.5 * sr;
    scr->result_folds = sf;
    scr->counter = 0u;
}

// message for fr_last_error(NULL), defined with the rest of the C ABI (fr_api.cu)
void set_global_error(const char* msg);

namespace {

std::mutex g_scratch_mutex;
void* g_scratch_ptr[64] = {nullptr};

int na_fail(int code, const char* msg) {
    set_global_error(msg);
    return code;
}

}  // namespace

}  // namespace frg

extern "C" int fr_stats_noalloc(const float* d_T, const int16_t* d_labT, const float* d_warped_S,
                                const int16_t* d_warped_labS, const float* d_psi, const int dims[3], int no_labels,
                                float w_reg, fr_stats* out, void* stream) {
    using namespace frg;
    set_global_error("");
    if (!d_T || !d_labT || !d_warped_S || !d_warped_labS || !d_psi || !dims || !out)
        return na_fail(FR_ERR_INVALID_ARG, "fr_stats_noalloc: NULL argument");
    if (dims[0] < 2 || dims[1] < 2 || dims[2] < 2)
        return na_fail(FR_ERR_INVALID_ARG, "fr_stats_noalloc: every dimension must be >= 2");
    const long long N = (long long)dims[0] * dims[1] * dims[2];
    if (N > (long long)FR_NOALLOC_MAX_VOXELS)
        return na_fail(FR_ERR_INVALID_ARG, "fr_stats_noalloc: volume larger than FR_NOALLOC_MAX_VOXELS");
    if (no_labels < 1 || no_labels > FR_MAX_LABELS)
        return na_fail(FR_ERR_INVALID_ARG, "fr_stats_noalloc: no_labels outside [1, FR_MAX_LABELS]");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return na_fail(FR_ERR_CUDA, "fr_stats_noalloc: no current CUDA device");
    }
    // set-up, once per device, with that device current: the device address of the
    // scratch array (its host-side name is only a stand-in, not a device address)
    StatsScratch* scr = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_scratch_mutex);
        if (!g_scratch_ptr[dev]) {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_stats_scratch);
            if (e != cudaSuccess || !p) {
                cudaGetLastError();
                return na_fail(FR_ERR_CUDA, "fr_stats_noalloc: cudaGetSymbolAddress failed");
            }
            g_scratch_ptr[dev] = p;
        }
        scr = (StatsScratch*)g_scratch_ptr[dev];
    }
    cudaStream_t s = (cudaStream_t)stream;
    // the array keeps the previous call's contents: clear the bins and the ticket
    if (cudaMemsetAsync(scr->dice, 0, sizeof(scr->dice), s) != cudaSuccess ||
        cudaMemsetAsync(&scr->counter, 0, sizeof(scr->counter), s) != cudaSuccess) {
        cudaGetLastError();
        return na_fail(FR_ERR_CUDA, "fr_stats_noalloc: clearing the scratch failed");
    }
    const long long want = (N + 255) / 256;
    const int grid = (int)(want < kStatsBlocks ? want : kStatsBlocks);
    stats_noalloc_kernel<<<grid, 256, 0, s>>>(d_T, d_labT, d_warped_S, d_warped_labS, d_psi, dims[0], dims[1],
                                              dims[2], no_labels, scr);
    if (cudaGetLastError() != cudaSuccess) return na_fail(FR_ERR_CUDA, "fr_stats_noalloc: kernel launch failed");
    double e[2];
    long long folds = 0;
    unsigned long long dice[kStatsBins];
    if (cudaMemcpyAsync(e, scr->result_e, sizeof e, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(&folds, &scr->result_folds, sizeof folds, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(dice, scr->dice, sizeof dice, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        cudaGetLastError();
        return na_fail(FR_ERR_CUDA, "fr_stats_noalloc: reading the results failed");
    }
    std::memset(out, 0, sizeof(*out));
    out->e_data = e[0];
    out->e_reg = e[1];
    out->energy = e[0] + (double)w_reg * e[1];
    out->folds = folds;
    out->no_labels = no_labels;
    double num = 0.0, den = 0.0;
    for (int l = 0; l < FR_MAX_LABELS; ++l) {
        out->dice_inter[l] = (int64_t)dice[l];
        out->dice_count[l] = (int64_t)dice[256 + l];
        out->dice[l] = dice[256 + l] ? 2.0 * (double)dice[l] / (double)dice[256 + l] : NAN;
        if (l >= 1 && l < no_labels) {
            num += (double)dice[l];
            den += (double)dice[256 + l];
        }
    }
    out->dice_all = den > 0 ? 2.0 * num / den : NAN;
    out->dice_out_of_range = (int64_t)dice[2 * 256];
    return FR_OK;
}
