// fr_selftest.cu -- the failure path of the TMA-staged kernels, exercised on the GPU.
//
// The staged kernels wait on their ring slots' mbarriers with a bound of about 2^31 clock
// cycles (mbar_wait_bounded); a block whose wait gives up agrees with the rest of the
// block on it (__syncthreads_or), sets the device error word and returns, and the host
// reports FR_ERR_CUDA.  fr_selftest_wait_limit runs exactly that path on a barrier armed
// for bytes that no copy will deliver (a flag that nothing sets): nothing faults, traps or
// hangs, the wait simply runs out.
#include <cuda_runtime.h>

#include <chrono>

#include "../../include/fastreg_gb300.h"
#include "fr_tma.cuh"

namespace frg {
void set_global_error(const char* msg);

__global__ void __launch_bounds__(256) selftest_wait_kernel(unsigned int* err, long long* cycles) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_fence_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) mbar_arrive_expect_tx(&bar, 16);  // 16 bytes that never arrive
    const long long t0 = clock64();
    const bool ok = mbar_wait_bounded(&bar, 0);
    if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) {
            atomicOr(err, kErrTmaTimeout);
            *cycles = clock64() - t0;
        }
    }
}
}  // namespace frg

extern "C" int fr_selftest_wait_limit(double* seconds, void* stream) {
    using namespace frg;
    set_global_error("");
    cudaStream_t s = (cudaStream_t)stream;
    unsigned int* d_err = nullptr;
    long long* d_cycles = nullptr;
    if (cudaMalloc((void**)&d_err, 64) != cudaSuccess) {
        cudaGetLastError();
        set_global_error("fr_selftest_wait_limit: device allocation failed");
        return FR_ERR_ALLOC;
    }
    d_cycles = (long long*)(d_err + 4);
    int rc = FR_OK;
    unsigned int err = 0;
    long long cycles = 0;
    const auto t0 = std::chrono::steady_clock::now();
    if (cudaMemsetAsync(d_err, 0, 64, s) != cudaSuccess) rc = FR_ERR_CUDA;
    if (rc == FR_OK) {
        selftest_wait_kernel<<<1, 256, 0, s>>>(d_err, d_cycles);
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpyAsync(&err, d_err, sizeof err, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaMemcpyAsync(&cycles, d_cycles, sizeof cycles, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            rc = FR_ERR_CUDA;
    }
    const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    cudaFree(d_err);
    if (rc != FR_OK) {
        cudaGetLastError();
        set_global_error("fr_selftest_wait_limit: a CUDA call failed");
        return rc;
    }
    if (seconds) *seconds = dt;
    if (!(err & kErrTmaTimeout) || cycles < (1LL << 31)) {
        set_global_error("fr_selftest_wait_limit: the wait did not give up as designed");
        return FR_ERR_STATE;
    }
    return FR_OK;
}
