// Live measurement of the FP64 arithmetic rate of the current GPU: the second
// roofline of the advection templates, which on GB300 are bound by the FP64
// pipe before HBM. Each thread runs eight independent chains of
// fma.rn.f64 / add.rn.f64 / mul.rn.f64 in registers and stores one value.
#include <cuda_runtime.h>

#include <cstdint>

namespace {

__device__ __forceinline__ double ptx_fma(double a, double b, double c) {
    double d;
    asm volatile("fma.rn.f64 %0, %1, %2, %3;" : "=d"(d) : "d"(a), "d"(b), "d"(c));
    return d;
}
__device__ __forceinline__ double ptx_add(double a, double b) {
    double d;
    asm volatile("add.rn.f64 %0, %1, %2;" : "=d"(d) : "d"(a), "d"(b));
    return d;
}

template <int OP>
__global__ void __launch_bounds__(256) fp64_chains(double *out, int iters, double b) {
    double x[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) x[c] = threadIdx.x + c;
    for (int n = 0; n < iters; ++n) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
#pragma unroll
            for (int c = 0; c < 8; ++c) x[c] = OP == 0 ? ptx_add(x[c], b) : ptx_fma(x[c], b, 0.5);
        }
    }
    double acc = 0.0;
#pragma unroll
    for (int c = 0; c < 8; ++c) acc += x[c];
    out[blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

} // namespace

// Measures FP64 instructions per second (one lane-op per instruction per
// thread) for add.rn.f64 (op 0) and fma.rn.f64 (op 1). Uses `scratch`, a
// device buffer of at least blocks*256 doubles supplied by the caller, where
// blocks = 8 x the SM count. Synchronous; returns 0 on success.
extern "C" int f2c_fp64_rate_v1(int op, double *scratch, size_t scratch_elems, double *ops_per_second) {
    int device = 0, sms = 0;
    if (cudaGetDevice(&device) != cudaSuccess) return 6;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 6;
    const int blocks = 8 * sms, threads = 256, iters = 1000;
    if (!scratch || !ops_per_second || scratch_elems < (size_t)blocks * threads) return 1;
    cudaEvent_t start, stop;
    if (cudaEventCreate(&start) != cudaSuccess) return 6;
    if (cudaEventCreate(&stop) != cudaSuccess) {
        cudaEventDestroy(start);
        return 6;
    }
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(start, 0);
        if (op == 0) fp64_chains<0><<<blocks, threads>>>(scratch, iters, 1.0000001);
        else fp64_chains<1><<<blocks, threads>>>(scratch, iters, 1.0000001);
        cudaEventRecord(stop, 0);
        cudaEventSynchronize(stop);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, start, stop);
        if (rep > 0 && ms < best) best = ms;
    }
    cudaEventDestroy(start);
    cudaEventDestroy(stop);
    if (cudaGetLastError() != cudaSuccess) return 6;
    *ops_per_second = (double)blocks * threads * iters * 32.0 / (best * 1e-3);
    return 0;
}
