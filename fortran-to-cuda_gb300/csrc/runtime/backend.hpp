// Device operations of the residency runtime, behind one small interface with
// two implementations chosen at compile time:
//
//  * the CUDA backend (default): stream-ordered allocations (cudaMallocAsync),
//    pitched rectangle copies, kernel launches and CUDA graphs on the
//    context's own non-blocking stream, host arrays pinned in place;
//  * the CPU test backend (F2C_RUNTIME_CPU_BACKEND): "device" memory is host
//    memory and a kernel function is a host function `void f(void **args)`,
//    so every coherence, queue and graph-cache rule can be tested on a machine
//    without a GPU.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "regions.hpp"

#ifndef F2C_RUNTIME_CPU_BACKEND
#include <cuda_runtime.h>
#endif

namespace f2c::rt {

struct LaunchSpec {
    const void *function = nullptr;
    unsigned grid[3] = {1, 1, 1}, block[3] = {1, 1, 1};
    size_t shared_bytes = 0;
    std::vector<void *> arguments; // pointers to argument values
};

// Copy geometry of one array: extents and element size; a box is copied as
// contiguous runs (the leading dimensions the box spans fully) or as 2-D
// pitched copies when the first dimension is partial.
struct CopyPlan {
    int rank;
    size_t elem;
    size_t extents[kMaxRank];
};

template <typename F>
void for_each_run(const CopyPlan &plan, const Box &box, F &&f) {
    // f(offset_elements, width_elements, rows, row_pitch_elements)
    const int r = plan.rank;
    int full = 0;
    while (full < r && box.lo[full] == 0 && box.hi[full] == plan.extents[full]) ++full;
    size_t inner = 1;
    for (int d = 0; d < full; ++d) inner *= plan.extents[d];
    size_t stride[kMaxRank];
    stride[0] = 1;
    for (int d = 1; d < r; ++d) stride[d] = stride[d - 1] * plan.extents[d - 1];
    if (full == r) {
        f(0, inner, 1, inner);
        return;
    }
    // dimension `full` is the first partial one
    size_t width, rows, pitch;
    int outer_start;
    if (full > 0) {
        width = inner * (box.hi[full] - box.lo[full]);
        rows = 1;
        pitch = width;
        outer_start = full + 1;
    } else {
        width = box.hi[0] - box.lo[0];
        if (r >= 2) {
            rows = box.hi[1] - box.lo[1];
            pitch = plan.extents[0];
            outer_start = 2;
        } else {
            rows = 1;
            pitch = width;
            outer_start = 1;
        }
    }
    size_t idx[kMaxRank];
    for (int d = outer_start; d < r; ++d) idx[d] = box.lo[d];
    while (true) {
        size_t off = 0;
        if (full > 0) off += box.lo[full] * stride[full];
        else {
            off += box.lo[0];
            if (r >= 2) off += box.lo[1] * stride[1];
        }
        for (int d = outer_start; d < r; ++d) off += idx[d] * stride[d];
        f(off, width, rows, pitch);
        int d = outer_start;
        for (; d < r; ++d) {
            if (++idx[d] < box.hi[d]) break;
            idx[d] = box.lo[d];
        }
        if (d == r) break;
    }
}

#ifdef F2C_RUNTIME_CPU_BACKEND

using Stream = void *;
struct Backend {
    static constexpr bool cpu = true;
    static std::string last_error() { return "cpu backend"; }
    static bool select(int) { return true; }
    static int current() { return 0; }
    static bool make_stream(Stream *s) {
        *s = nullptr;
        return true;
    }
    static void destroy_stream(Stream) {}
    static bool alloc(void **p, size_t bytes, Stream) {
        if (std::getenv("F2C_TEST_FAIL_ALLOC")) return false;
        // F2C_TEST_FAIL_ALLOC_AFTER=n: the allocations after the first n fail (counted while it is set)
        static int granted = 0;
        if (const char *after = std::getenv("F2C_TEST_FAIL_ALLOC_AFTER")) {
            if (granted >= std::atoi(after)) return false;
            ++granted;
        } else {
            granted = 0;
        }
        *p = std::malloc(bytes ? bytes : 1);
        return *p != nullptr;
    }
    static void free(void *p, Stream) { std::free(p); }
    // `bytes` contiguous bytes between the host array and its device copy.
    static bool linear(void *dst, const void *src, size_t bytes, bool, const void *, Stream) {
        std::memcpy(dst, src, bytes);
        return true;
    }
    static bool copy(void *dst, const void *src, const CopyPlan &plan, const Box &box, bool, Stream) {
        for_each_run(plan, box, [&](size_t off, size_t width, size_t rows, size_t pitch) {
            for (size_t r = 0; r < rows; ++r)
                std::memcpy(static_cast<char *>(dst) + (off + r * pitch) * plan.elem,
                            static_cast<const char *>(src) + (off + r * pitch) * plan.elem, width * plan.elem);
        });
        return true;
    }
    static bool sync(Stream) { return !std::getenv("F2C_TEST_FAIL_WAIT"); }
    // A scratch arena cannot be allocated (tests only).
    static bool scratch_alloc_fails() { return std::getenv("F2C_TEST_FAIL_SCRATCH_ALLOC") != nullptr; }
    // An external provider's effects fail to commit after it ran (tests only).
    static bool external_commit_fails() { return std::getenv("F2C_TEST_FAIL_EXTERNAL_COMMIT") != nullptr; }
    // Completion events. Work here is synchronous, but an event reads as pending
    // until it is waited for, so that the runtime's bookkeeping of what is still
    // in flight is exercised as on a device.
    using Event = int;
    static bool make_event(Event *e) {
        *e = 1;
        return true;
    }
    static void destroy_event(Event) {}
    static bool record(Event, Stream) { return true; }
    // Timing events: work here is synchronous, every interval reads as zero.
    static bool make_timing_event(Event *e) {
        *e = 1;
        return true;
    }
    static bool elapsed(Event, Event, float *ms) {
        *ms = 0.0f;
        return true;
    }
    static bool query(Event) { return false; }
    static bool wait_event(Event) { return !std::getenv("F2C_TEST_FAIL_WAIT"); }
    // Host arrays are never pinned here, unless a test asks for the mapped
    // case (F2C_TEST_MAPPED): then the "device-usable" address is the array.
    static int pin(void *p, size_t, void **mapped) {
        if (!std::getenv("F2C_TEST_MAPPED")) return 0;
        *mapped = p;
        return 1;
    }
    static void unpin(void *) {}
    // Work is synchronous: every stream is already joined.
    static bool join(Stream, Stream) { return true; }
    // A 16 GiB device with 12 GiB free, or the free bytes a test states (F2C_TEST_FREE_BYTES).
    static bool memory_info(size_t *free_bytes, size_t *total) {
        *total = size_t(16) << 30;
        const char *stated = std::getenv("F2C_TEST_FREE_BYTES");
        *free_bytes = stated ? (size_t)std::strtoull(stated, nullptr, 10) : size_t(12) << 30;
        return true;
    }
    static bool launch(const LaunchSpec &k, Stream) {
        if (std::getenv("F2C_TEST_FAIL_LAUNCH")) return false;
        auto fn = reinterpret_cast<void (*)(void **)>(const_cast<void *>(k.function));
        fn(const_cast<void **>(k.arguments.data()));
        return true;
    }
    // Graphs: on the CPU backend a graph is the node count; the runtime's cached
    // launch records (with their current arguments) are run in order.
    struct Graph {
        size_t nodes = 0;
    };
    static bool graph_build(Graph **g, const std::vector<LaunchSpec> &nodes) {
        if (std::getenv("F2C_TEST_FAIL_GRAPH_CREATE")) return false;
        *g = new Graph{nodes.size()};
        return true;
    }
    static bool graph_update(Graph *, size_t, const LaunchSpec &) { return !std::getenv("F2C_TEST_FAIL_GRAPH_UPDATE"); }
    static bool graph_launch(Graph *g, const std::vector<LaunchSpec> &specs, Stream s) {
        if (specs.size() != g->nodes) return false;
        for (const auto &k : specs)
            if (!launch(k, s)) return false;
        return true;
    }
    static void graph_destroy(Graph *g) { delete g; }
};

#else

using Stream = cudaStream_t;
struct Backend {
    static constexpr bool cpu = false;
    static thread_local std::string error;
    static std::string last_error() { return error; }
    static bool ok(cudaError_t e) {
        if (e == cudaSuccess) return true;
        error = cudaGetErrorString(e);
        return false;
    }
    static bool select(int device) { return ok(cudaSetDevice(device)); }
    static int current() {
        int d = 0;
        cudaGetDevice(&d);
        return d;
    }
    static bool make_stream(Stream *s) { return ok(cudaStreamCreateWithFlags(s, cudaStreamNonBlocking)); }
    static void destroy_stream(Stream s) {
        if (s) cudaStreamDestroy(s);
    }
    static bool alloc(void **p, size_t bytes, Stream s) { return ok(cudaMallocAsync(p, bytes ? bytes : 256, s)); }
    static void free(void *p, Stream s) {
        if (p) cudaFreeAsync(p, s);
    }
    // One contiguous host<->device copy. A large copy whose host start is not on
    // a 2 MiB boundary goes as a head up to that boundary and an aligned body:
    // with uploads and downloads running at once, a copy from a misaligned host
    // start moves about 116 GB/s each way on GB300 and an aligned one 171 GB/s.
    static bool contiguous(char *d, const char *sp, size_t bytes, cudaMemcpyKind kind, const char *host, Stream s) {
        constexpr size_t kAlign = size_t(2) << 20;
        const size_t head = (kAlign - reinterpret_cast<uintptr_t>(host) % kAlign) % kAlign;
        if (bytes < 4 * kAlign || head == 0) return ok(cudaMemcpyAsync(d, sp, bytes, kind, s));
        return ok(cudaMemcpyAsync(d, sp, head, kind, s)) && ok(cudaMemcpyAsync(d + head, sp + head, bytes - head, kind, s));
    }
    static bool linear(void *dst, const void *src, size_t bytes, bool to_device, const void *host, Stream s) {
        return contiguous(static_cast<char *>(dst), static_cast<const char *>(src), bytes,
                          to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost, static_cast<const char *>(host),
                          s);
    }
    static bool copy(void *dst, const void *src, const CopyPlan &plan, const Box &box, bool to_device, Stream s) {
        const cudaMemcpyKind kind = to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost;
        const bool full_rows = box.lo[0] == 0 && box.hi[0] == plan.extents[0];
        const bool full_planes = full_rows && box.lo[1] == 0 && box.hi[1] == plan.extents[1];
        if (plan.rank == 3 && !full_planes) {
            // one strided 3-D copy per box (host and device share the layout)
            cudaMemcpy3DParms p{};
            const size_t pitch = plan.extents[0] * plan.elem;
            p.srcPtr = make_cudaPitchedPtr(const_cast<void *>(src), pitch, plan.extents[0], plan.extents[1]);
            p.dstPtr = make_cudaPitchedPtr(dst, pitch, plan.extents[0], plan.extents[1]);
            p.srcPos = make_cudaPos(box.lo[0] * plan.elem, box.lo[1], box.lo[2]);
            p.dstPos = p.srcPos;
            p.extent = make_cudaExtent((box.hi[0] - box.lo[0]) * plan.elem, box.hi[1] - box.lo[1], box.hi[2] - box.lo[2]);
            p.kind = kind;
            return ok(cudaMemcpy3DAsync(&p, s));
        }
        bool good = true;
        for_each_run(plan, box, [&](size_t off, size_t width, size_t rows, size_t pitch) {
            if (!good) return;
            char *d = static_cast<char *>(dst) + off * plan.elem;
            const char *sp = static_cast<const char *>(src) + off * plan.elem;
            if (rows == 1)
                good = contiguous(d, sp, width * plan.elem, kind, to_device ? sp : d, s);
            else
                good = ok(cudaMemcpy2DAsync(d, pitch * plan.elem, sp, pitch * plan.elem, width * plan.elem, rows, kind,
                                            s));
        });
        return good;
    }
    static bool sync(Stream s) { return ok(cudaStreamSynchronize(s)); }
    static bool external_commit_fails() { return false; }
    static bool scratch_alloc_fails() { return false; }
    using Event = cudaEvent_t;
    static bool make_event(Event *e) { return ok(cudaEventCreateWithFlags(e, cudaEventDisableTiming)); }
    static void destroy_event(Event e) {
        if (e) cudaEventDestroy(e);
    }
    static bool record(Event e, Stream s) { return ok(cudaEventRecord(e, s)); }
    static bool make_timing_event(Event *e) { return ok(cudaEventCreate(e)); }
    // Milliseconds between two completed timing events (the later one is waited for).
    static bool elapsed(Event a, Event b, float *ms) { return ok(cudaEventSynchronize(b)) && ok(cudaEventElapsedTime(ms, a, b)); }
    // Complete or not; a failure of the work shows at the wait. "Not ready" is an
    // answer, not an error: should it be left as the last error, it is cleared so
    // that no later launch check reads it.
    static bool query(Event e) {
        const cudaError_t r = cudaEventQuery(e);
        if (r == cudaErrorNotReady && cudaPeekAtLastError() == cudaErrorNotReady) (void)cudaGetLastError();
        return r == cudaSuccess;
    }
    static bool wait_event(Event e) { return ok(cudaEventSynchronize(e)); }
    // `waiter` runs its later work after everything queued so far on `signaller`.
    static bool join(Stream waiter, Stream signaller) {
        cudaEvent_t e;
        if (!ok(cudaEventCreateWithFlags(&e, cudaEventDisableTiming))) return false;
        const bool good = ok(cudaEventRecord(e, signaller)) && ok(cudaStreamWaitEvent(waiter, e, 0));
        cudaEventDestroy(e);
        return good;
    }
    // Whether the host byte at `p` is page-locked memory that CUDA knows (the
    // caller's cudaHostAlloc or cudaHostRegister).
    static bool page_locked(const void *p) {
        cudaPointerAttributes attr{};
        if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        return attr.type == cudaMemoryTypeHost;
    }
    // Pin a host array in place and map it into the device address space;
    // `mapped` receives the address a kernel uses to reach it over NVLink-C2C.
    // Returns 1 when this call pinned it (unpin it later), 2 when the caller's
    // memory was page-locked already (its first and last bytes; leave it
    // pinned), 0 when it could not be pinned.
    static int pin(void *p, size_t bytes, void **mapped) {
        int how = 1;
        if (page_locked(p) && page_locked(static_cast<const char *>(p) + bytes - 1)) {
            how = 2;
        } else {
            const cudaError_t r = cudaHostRegister(p, bytes, cudaHostRegisterMapped | cudaHostRegisterPortable);
            if (r != cudaSuccess) {
                cudaGetLastError();
                return 0;
            }
        }
        if (cudaHostGetDevicePointer(mapped, p, 0) != cudaSuccess) {
            cudaGetLastError();
            *mapped = nullptr;
        }
        return how;
    }
    static void unpin(void *p) {
        if (cudaHostUnregister(p) != cudaSuccess) cudaGetLastError();
    }
    static bool memory_info(size_t *free_bytes, size_t *total) { return ok(cudaMemGetInfo(free_bytes, total)); }
    static cudaKernelNodeParams params(const LaunchSpec &k) {
        cudaKernelNodeParams p{};
        p.func = const_cast<void *>(k.function);
        p.gridDim = dim3(k.grid[0], k.grid[1], k.grid[2]);
        p.blockDim = dim3(k.block[0], k.block[1], k.block[2]);
        p.sharedMemBytes = (unsigned)k.shared_bytes;
        p.kernelParams = const_cast<void **>(k.arguments.data());
        p.extra = nullptr;
        return p;
    }
    static bool launch(const LaunchSpec &k, Stream s) {
        return ok(cudaLaunchKernel(k.function, dim3(k.grid[0], k.grid[1], k.grid[2]),
                                   dim3(k.block[0], k.block[1], k.block[2]), const_cast<void **>(k.arguments.data()),
                                   k.shared_bytes, s));
    }
    struct Graph {
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        std::vector<cudaGraphNode_t> nodes;
    };
    static bool graph_build(Graph **out, const std::vector<LaunchSpec> &nodes) {
        auto *g = new Graph;
        if (!ok(cudaGraphCreate(&g->graph, 0))) {
            delete g;
            return false;
        }
        cudaGraphNode_t prev = nullptr;
        for (const auto &k : nodes) {
            cudaGraphNode_t node;
            const cudaKernelNodeParams p = params(k);
            if (!ok(cudaGraphAddKernelNode(&node, g->graph, prev ? &prev : nullptr, prev ? 1 : 0, &p))) {
                graph_destroy(g);
                return false;
            }
            g->nodes.push_back(node);
            prev = node;
        }
        if (!ok(cudaGraphInstantiate(&g->exec, g->graph, 0))) {
            graph_destroy(g);
            return false;
        }
        *out = g;
        return true;
    }
    static bool graph_update(Graph *g, size_t node, const LaunchSpec &k) {
        const cudaKernelNodeParams p = params(k);
        return ok(cudaGraphExecKernelNodeSetParams(g->exec, g->nodes[node], &p));
    }
    static bool graph_launch(Graph *g, const std::vector<LaunchSpec> &, Stream s) { return ok(cudaGraphLaunch(g->exec, s)); }
    static void graph_destroy(Graph *g) {
        if (!g) return;
        if (g->exec) cudaGraphExecDestroy(g->exec);
        if (g->graph) cudaGraphDestroy(g->graph);
        delete g;
    }
};

#endif

} // namespace f2c::rt
