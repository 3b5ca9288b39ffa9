// Device check of the integer-pipe binary64 additions and multiply
// (fortran-to-cuda_gb300/csrc/kernels/soft_fp64.cuh) against the GPU's own
// DADD and DMUL, bit for bit (NaN results only need to be NaN on both sides).
// Built by tests/test_soft_fp64_gpu.py into a temporary shared library.
#include <cuda_runtime.h>
#include <cstdint>

#include "soft_fp64.cuh"
#include "cases.h"

namespace {

__global__ void check_kernel(int op, int dist, uint64_t seed, uint64_t n, unsigned long long *bad) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
        uint64_t ia, ib;
        soft_cases::pair(dist, seed, i, &ia, &ib);
        const double a = __longlong_as_double((long long)ia), b = __longlong_as_double((long long)ib);
        const double got = op == 0 ? f2c::add_rn_int(a, b) : op == 1 ? f2c::mul_rn_int(a, b) : f2c::add_rn_near(a, b);
        const double want = op == 1 ? __dmul_rn(a, b) : __dadd_rn(a, b);
        const bool both_nan = got != got && want != want;
        if (!both_nan && __double_as_longlong(got) != __double_as_longlong(want)) atomicAdd(bad, 1ull);
    }
}

} // namespace

// Mismatch count of `n` pairs of distribution `dist` (cases.h) for op 0 (add),
// 1 (multiply) or 2 (the nearby-exponent add); -1 on a CUDA error.
extern "C" long long soft_fp64_device_check(int op, int dist, unsigned long long seed, unsigned long long n) {
    unsigned long long *bad = nullptr, host = 0;
    if (cudaMalloc(&bad, sizeof host) != cudaSuccess) return -1;
    long long out = -1;
    if (cudaMemset(bad, 0, sizeof host) == cudaSuccess) {
        check_kernel<<<152 * 8, 256>>>(op, dist, seed, n, bad);
        if (cudaGetLastError() == cudaSuccess && cudaMemcpy(&host, bad, sizeof host, cudaMemcpyDeviceToHost) == cudaSuccess)
            out = (long long)host;
    }
    cudaFree(bad);
    return out;
}
