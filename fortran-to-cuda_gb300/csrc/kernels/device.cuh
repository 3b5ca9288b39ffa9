// Per-device facts and one-time kernel configuration.
//
// A process may drive several GPUs in turn. Launch shapes that depend on the
// SM count, and kernel attributes such as the dynamic shared-memory limit,
// belong to a device, so they are looked up and applied once per device
// ordinal (with that device current), never once per process.
#pragma once
#include <cuda_runtime.h>

#include <atomic>

namespace f2c {

constexpr int kMaxDeviceOrdinals = 64;
constexpr int kDefaultSMs = 152;  // GB300; used only when the device cannot be asked

// SM count of the current device (cached per ordinal).
inline int current_sm_count() {
    static std::atomic<int> cache[kMaxDeviceOrdinals];
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess || device < 0) return kDefaultSMs;
    if (device < kMaxDeviceOrdinals) {
        const int known = cache[device].load(std::memory_order_relaxed);
        if (known > 0) return known;
    }
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || sms < 1)
        return kDefaultSMs;
    if (device < kMaxDeviceOrdinals) cache[device].store(sms, std::memory_order_relaxed);
    return sms;
}

// Sets `function`'s dynamic shared-memory limit to `bytes` on the current
// device, once per device ordinal for each distinct `done` record (one record
// per kernel instantiation). Returns the status of the attribute call.
inline cudaError_t configure_shared_once(std::atomic<unsigned long long> &done, const void *function, int bytes) {
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return e;
    const bool cacheable = device >= 0 && device < kMaxDeviceOrdinals;
    const unsigned long long bit = cacheable ? (1ULL << device) : 0ULL;
    if (cacheable && (done.load(std::memory_order_acquire) & bit)) return cudaSuccess;
    e = cudaFuncSetAttribute(function, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess && cacheable) done.fetch_or(bit, std::memory_order_release);
    return e;
}

} // namespace f2c
