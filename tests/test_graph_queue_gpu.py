"""The task queue and checked graph groups of the runtime with real kernels on the GPU.

The CPU scenarios of the queue (tests/test_runtime_abi.py) run test kernels as
host functions; here a CUDA client written against include/scoped_runtime.h
passes the addresses of its own ``__global__`` functions, so the CUDA
backend's graph construction, parameter updates, replays and direct launches
run for real. The behaviours follow the reference's CUDA suites
(compiler/tests/test_scoped_graph_replay_cuda.py:241-262: replay, rebinding,
topology change, long groups; test_scoped_graph_queue_cuda.py:333-341: the
deferred queue). An external provider's kernel on the runtime's stream is ordered before
the publication that follows it (test_scoped_domains_cuda.py:267-300), and
host work waits only for the device work it conflicts with, checked against a
kernel delayed by a bounded spin (test_scoped_host_completion_cuda.py), and
sparse sections move exactly through real pitched copies
(test_scoped_direct_copy_cuda.py). The
client checks every value it reads back and prints the runtime's statistics
as one JSON line per scenario.
"""

import json
import subprocess
from pathlib import Path

import pytest

from compiler import native

pytestmark = pytest.mark.gpu

CLIENT = r"""
#include <cstdio>
#include <cstring>
#include <string>
#include <cuda_runtime.h>
#include "scoped_runtime.h"

#define CHECK(x)                                                                                 \
    do {                                                                                         \
        const int status_ = (x);                                                                 \
        if (status_) {                                                                           \
            std::fprintf(stderr, "%s: status %d: %s\n", #x, status_, fort_scope_error());        \
            return 1;                                                                            \
        }                                                                                        \
    } while (0)

constexpr int N = 1024;

__global__ void axpy(double *x, int n, double a, double b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = x[i] * a + b;
}
__global__ void produce(const double *a, double *b, int n, double add) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = a[i] + add;
}
__global__ void consume(const double *b, double *out, int n, double factor) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = factor * b[i];
}
__global__ void alternate(const double *b, double *out, int n, double factor) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = factor * b[i] + 1.0;
}

struct Array {
    double host[N];
    fort_buffer_t handle = 0;
    double *device = nullptr;
};

static size_t g_extent[1] = {N};
static int64_t g_lower[1] = {1};

static int add_array(fort_scope_t ctx, Array &a, uint64_t identity, bool initialized) {
    fort_scope_layout layout{1, FORT_SCOPE_REAL64, 8, a.host, g_extent, g_lower, 1};
    CHECK(fort_scope_register(ctx, identity, 1, &layout, initialized ? 1 : 0, &a.handle));
    CHECK(fort_scope_device_reserve_v1(ctx, a.handle, reinterpret_cast<void **>(&a.device)));
    return 0;
}

static fort_scope_access whole(uint32_t flags) {
    fort_scope_access acc;
    std::memset(&acc, 0, sizeof acc);
    acc.flags = flags;
    return acc;
}

static fort_scope_kernel_v1 kernel(const void *fn, void *const *args, size_t count) {
    fort_scope_kernel_v1 k;
    std::memset(&k, 0, sizeof k);
    k.version = 1;
    k.function = fn;
    k.grid[0] = N / 256; k.grid[1] = k.grid[2] = 1;
    k.block[0] = 256; k.block[1] = k.block[2] = 1;
    k.arguments = args;
    k.argument_count = count;
    return k;
}

static int observe(fort_scope_t ctx, fort_buffer_t h) { return fort_scope_observe_v1(ctx, &h, 1); }

static void print_stats(fort_scope_t ctx, const char *scenario) {
    fort_scope_graph_stats_v1 g{};
    fort_scope_graph_queue_stats_v1 q{};
    fort_scope_stats s{};
    fort_scope_graph_stats_get_v1(ctx, &g);
    fort_scope_graph_queue_stats_get_v1(ctx, &q);
    fort_scope_stats_get(ctx, &s);
    std::printf("{\"scenario\": \"%s\", \"creations\": %llu, \"instantiations\": %llu, \"rebuilds\": %llu, "
                "\"submissions\": %llu, \"replays\": %llu, \"parameter_updates\": %llu, \"live_graphs\": %llu, "
                "\"accepted_tasks\": %llu, \"direct_submissions\": %llu, \"pending_tasks\": %llu, "
                "\"uploads\": %llu, \"downloads\": %llu}\n",
                scenario, (unsigned long long)g.creations, (unsigned long long)g.instantiations,
                (unsigned long long)g.rebuilds, (unsigned long long)g.submissions, (unsigned long long)g.replays,
                (unsigned long long)g.parameter_updates, (unsigned long long)g.live_graphs,
                (unsigned long long)q.accepted_tasks, (unsigned long long)q.direct_submissions,
                (unsigned long long)q.pending_tasks, (unsigned long long)s.uploads, (unsigned long long)s.downloads);
}

static int expect(const Array &a, double (*value)(int), const char *what) {
    for (int i = 0; i < N; ++i)
        if (a.host[i] != value(i)) {
            std::fprintf(stderr, "%s: element %d is %.17g, expected %.17g\n", what, i, a.host[i], value(i));
            return 1;
        }
    return 0;
}

// four queued axpy steps, each flushed: the first runs directly, the second instantiates, the rest replay
static int queue_replay() {
    fort_scope_t ctx = 0;
    CHECK(fort_scope_create(0, &ctx));
    static Array x;
    for (int i = 0; i < N; ++i) x.host[i] = 1.0 + i;
    if (add_array(ctx, x, 1, true)) return 1;
    int n = N;
    double a = 2.0, b = 0.0;
    void *args[4] = {&x.device, &n, &a, &b};
    const size_t sizes[4] = {sizeof(double *), sizeof(int), sizeof(double), sizeof(double)};
    fort_scope_plan_binding bind{x.handle, whole(FORT_SCOPE_READ_ALL | FORT_SCOPE_WRITE_ALL)};
    for (int step = 0; step < 4; ++step) {
        b = step;  // argument values are copied when the task is accepted
        fort_scope_graph_task_v1 task{kernel((const void *)axpy, args, 4), &bind, 1};
        CHECK(fort_scope_graph_enqueue_v1(ctx, 7, &task, sizes));
        CHECK(fort_scope_graph_flush_v1(ctx));
    }
    CHECK(observe(ctx, x.handle));
    print_stats(ctx, "queue");
    CHECK(fort_scope_close(ctx));
    return expect(x, [](int i) { return ((((1.0 + i) * 2 + 0) * 2 + 1) * 2 + 2) * 2 + 3; }, "queue");
}

// a checked group (producer then consumer) executed four times with a new factor each time, then once with
// another consumer: replays with parameter updates, and a new graph for the new sequence
static int group_replay() {
    fort_scope_t ctx = 0;
    CHECK(fort_scope_create(0, &ctx));
    static Array a, b, out;
    for (int i = 0; i < N; ++i) a.host[i] = 0.5 * i;
    if (add_array(ctx, a, 1, true) || add_array(ctx, b, 2, false) || add_array(ctx, out, 3, false)) return 1;
    int n = N;
    double add = 2.0, factor = 1.0;
    void *produce_args[4] = {&a.device, &b.device, &n, &add};
    void *consume_args[4] = {&b.device, &out.device, &n, &factor};
    fort_scope_plan_binding producer[2] = {{a.handle, whole(FORT_SCOPE_READ_ALL)},
                                           {b.handle, whole(FORT_SCOPE_WRITE_ALL | FORT_SCOPE_OVERWRITE_ALL)}};
    fort_scope_plan_binding consumer[2] = {{b.handle, whole(FORT_SCOPE_READ_ALL)},
                                           {out.handle, whole(FORT_SCOPE_WRITE_ALL | FORT_SCOPE_OVERWRITE_ALL)}};
    for (int round = 1; round <= 4; ++round) {
        factor = round;
        fort_scope_graph_task_v1 tasks[2] = {{kernel((const void *)produce, produce_args, 4), producer, 2},
                                             {kernel((const void *)consume, consume_args, 4), consumer, 2}};
        CHECK(fort_scope_graph_execute_v1(ctx, 21, tasks, 2));
    }
    CHECK(observe(ctx, out.handle));
    if (expect(out, [](int i) { return 4.0 * (0.5 * i + 2.0); }, "group")) return 1;
    print_stats(ctx, "group");
    factor = 10.0;
    fort_scope_graph_task_v1 other[2] = {{kernel((const void *)produce, produce_args, 4), producer, 2},
                                         {kernel((const void *)alternate, consume_args, 4), consumer, 2}};
    CHECK(fort_scope_graph_execute_v1(ctx, 22, other, 2));
    CHECK(fort_scope_graph_execute_v1(ctx, 22, other, 2));
    CHECK(observe(ctx, out.handle));
    if (expect(out, [](int i) { return 10.0 * (0.5 * i + 2.0) + 1.0; }, "topology")) return 1;
    print_stats(ctx, "topology");
    CHECK(fort_scope_close(ctx));
    return 0;
}

// queued tasks that are cancelled never run and leave the array as it was
static int cancel() {
    fort_scope_t ctx = 0;
    CHECK(fort_scope_create(0, &ctx));
    static Array x;
    for (int i = 0; i < N; ++i) x.host[i] = 3.0 * i;
    if (add_array(ctx, x, 1, true)) return 1;
    int n = N;
    double a = 5.0, b = 7.0;
    void *args[4] = {&x.device, &n, &a, &b};
    const size_t sizes[4] = {sizeof(double *), sizeof(int), sizeof(double), sizeof(double)};
    fort_scope_plan_binding bind{x.handle, whole(FORT_SCOPE_READ_ALL | FORT_SCOPE_WRITE_ALL)};
    for (int k = 0; k < 3; ++k) {
        fort_scope_graph_task_v1 task{kernel((const void *)axpy, args, 4), &bind, 1};
        CHECK(fort_scope_graph_enqueue_v1(ctx, 9, &task, sizes));
    }
    CHECK(fort_scope_graph_queue_cancel_v1(ctx));
    CHECK(fort_scope_graph_flush_v1(ctx));
    CHECK(observe(ctx, x.handle));
    print_stats(ctx, "cancel");
    CHECK(fort_scope_close(ctx));
    return expect(x, [](int i) { return 3.0 * i; }, "cancel");
}

// a long chain of queued tasks goes as one submission, in order
static int long_chain() {
    fort_scope_t ctx = 0;
    CHECK(fort_scope_create(0, &ctx));
    static Array x;
    for (int i = 0; i < N; ++i) x.host[i] = i;
    if (add_array(ctx, x, 1, true)) return 1;
    int n = N;
    double a = 1.0, b = 0.0;
    void *args[4] = {&x.device, &n, &a, &b};
    const size_t sizes[4] = {sizeof(double *), sizeof(int), sizeof(double), sizeof(double)};
    fort_scope_plan_binding bind{x.handle, whole(FORT_SCOPE_READ_ALL | FORT_SCOPE_WRITE_ALL)};
    for (int k = 0; k < 64; ++k) {
        b = k;
        fort_scope_graph_task_v1 task{kernel((const void *)axpy, args, 4), &bind, 1};
        CHECK(fort_scope_graph_enqueue_v1(ctx, 5, &task, sizes));
    }
    CHECK(observe(ctx, x.handle));  // host access drains the queue
    print_stats(ctx, "long");
    CHECK(fort_scope_close(ctx));
    return expect(x, [](int i) { return i + 63.0 * 64.0 / 2.0; }, "long");
}

// an external provider's kernel, slowed down by a bounded spin on the clock, runs on the stream the runtime
// hands it: the publication that follows must wait for it
__global__ void slow_double(const double *a, double *b, int n, long long delay) {
    const long long start = clock64();
    while (clock64() - start < delay) {
    }
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = 2.0 * a[i];
}

static int provider(void *user, const fort_scope_external_view_v1 *views, size_t count, void *stream, int *started) {
    if (count != 2 || !views[0].device || !views[1].device || views[1].bytes != N * sizeof(double)) return 1;
    const long long delay = *static_cast<const long long *>(user);
    slow_double<<<N / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const double *>(views[0].device), static_cast<double *>(views[1].device), N, delay);
    *started = 1;
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

static int external() {
    fort_scope_t ctx = 0;
    CHECK(fort_scope_create(0, &ctx));
    static Array a, b;
    for (int i = 0; i < N; ++i) a.host[i] = 0.25 * i;
    if (add_array(ctx, a, 1, true)) return 1;
    fort_scope_layout layout{1, FORT_SCOPE_REAL64, 8, b.host, g_extent, g_lower, 1};
    CHECK(fort_scope_register(ctx, 2, 1, &layout, 0, &b.handle));
    fort_scope_external_binding_v1 bindings[2];
    std::memset(bindings, 0, sizeof bindings);
    bindings[0].buffer = a.handle;
    bindings[0].access = whole(FORT_SCOPE_READ_ALL);
    bindings[1].buffer = b.handle;
    bindings[1].access = whole(FORT_SCOPE_WRITE_ALL | FORT_SCOPE_OVERWRITE_ALL);
    for (auto &x : bindings) {
        x.type = FORT_SCOPE_REAL64;
        x.rank = 1;
        x.element_bytes = 8;
    }
    fort_scope_external_call_v1 call;
    std::memset(&call, 0, sizeof call);
    call.version = FORT_SCOPE_EXTERNAL_ABI_VERSION;
    call.bindings = bindings;
    call.binding_count = 2;
    long long delay = 4000000;  // about 2 ms of clock cycles
    fort_scope_external_report_v1 report{};
    CHECK(fort_scope_external_execute_v1(ctx, &call, provider, &delay, &report));
    if (report.status != 0 || !report.started || !report.committed) {
        std::fprintf(stderr, "report: status %d started %u committed %u\n", report.status, report.started,
                     report.committed);
        return 1;
    }
    CHECK(observe(ctx, b.handle));  // reads what the provider's kernel wrote, after it finished
    if (expect(b, [](int i) { return 0.5 * i; }, "external")) return 1;
    print_stats(ctx, "external");
    CHECK(fort_scope_close(ctx));
    return 0;
}

// a device write delayed by about 40 ms of clock cycles (a bounded spin), on the context's stream
__global__ void delayed_fill(double *out, int n, double value, long long cycles) {
    const long long start = clock64();
    while (clock64() - start < cycles) {
    }
    for (int i = 0; i < n; ++i) out[i] = value;
}

static int completion() {
    fort_scope_t ctx = 0;
    CHECK(fort_scope_create(0, &ctx));
    static Array a, x;
    for (int i = 0; i < N; ++i) {
        a.host[i] = 0.0;
        x.host[i] = 10.0 + i;
    }
    fort_scope_layout la{1, FORT_SCOPE_REAL64, 8, a.host, g_extent, g_lower, 1};
    fort_scope_layout lx{1, FORT_SCOPE_REAL64, 8, x.host, g_extent, g_lower, 1};
    CHECK(fort_scope_register(ctx, 1, 1, &la, 1, &a.handle));
    CHECK(fort_scope_register(ctx, 2, 1, &lx, 1, &x.handle));
    int previous = 0;
    void *raw = nullptr;
    CHECK(fort_scope_gpu_enter(ctx, &previous, &raw));
    cudaStream_t stream = static_cast<cudaStream_t>(raw);
    int khz = 0;
    if (cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, 0) != cudaSuccess || khz <= 0) return 1;
    const long long cycles = static_cast<long long>(khz) * 40;
    fort_scope_access write = whole(FORT_SCOPE_WRITE_ALL | FORT_SCOPE_OVERWRITE_ALL);
    double *pa = nullptr;
    CHECK(fort_scope_device_begin(ctx, a.handle, &write, reinterpret_cast<void **>(&pa)));
    delayed_fill<<<1, 1, 0, stream>>>(pa, N, 1.0, cycles);
    if (cudaGetLastError() != cudaSuccess) return 1;
    CHECK(fort_scope_note_launch(ctx));
    CHECK(fort_scope_device_end(ctx, a.handle));
    cudaEvent_t marker;
    if (cudaEventCreateWithFlags(&marker, cudaEventDisableTiming) != cudaSuccess) return 1;
    if (cudaEventRecord(marker, stream) != cudaSuccess) return 1;
    fort_scope_stats before{}, after{};
    CHECK(fort_scope_stats_get(ctx, &before));
    // host work on an array the pending kernel does not touch returns at once
    fort_scope_access rw = whole(FORT_SCOPE_READ_ALL | FORT_SCOPE_WRITE_ALL);
    CHECK(fort_scope_host_begin(ctx, x.handle, &rw));
    x.host[0] = 99.0;
    CHECK(fort_scope_host_end(ctx, x.handle));
    const bool pending = cudaEventQuery(marker) == cudaErrorNotReady;
    cudaGetLastError();
    CHECK(fort_scope_stats_get(ctx, &after));
    fort_scope_completion_stats_v1 cs{};
    CHECK(fort_scope_completion_stats_get_v1(ctx, &cs));
    // host work on the array it writes waits for it
    fort_scope_access read = whole(FORT_SCOPE_READ_ALL);
    CHECK(fort_scope_host_begin(ctx, a.handle, &read));
    const bool seen = a.host[0] == 1.0 && a.host[N - 1] == 1.0;
    CHECK(fort_scope_host_end(ctx, a.handle));
    const bool done = cudaEventQuery(marker) == cudaSuccess;
    cudaEventDestroy(marker);
    std::printf("{\"scenario\": \"completion\", \"pending_after_independent\": %s, \"independent_waits\": %llu, "
                "\"independent_host_tasks\": %llu, \"dependent_saw_kernel\": %s, \"done_after_dependent\": %s}\n",
                pending ? "true" : "false", (unsigned long long)(after.waits - before.waits),
                (unsigned long long)cs.independent_host_tasks, seen ? "true" : "false", done ? "true" : "false");
    CHECK(fort_scope_gpu_leave(ctx, previous));
    CHECK(fort_scope_close(ctx));
    return 0;
}

// exact sparse transfers through real DMA: the halo of a 134 x 70 x 70 array moves as its six faces, stripes
// one byte wide of a byte array move as twenty pitched copies, and mirrors that both hold the values survive
// interleaved read-only use without transfers
constexpr size_t EX = 134, EY = 70, EZ = 70, EN = EX * EY * EZ;
__global__ void fill_index(double *p) {
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < EN) p[i] = 1000000.0 + i;
}
__global__ void fill_bytes(unsigned char *p, size_t n) {
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) p[i] = i % 251 + 1;
}
static bool in_halo(size_t x, size_t y, size_t z) { return x < 3 || x >= 131 || y < 3 || y >= 67 || z < 2 || z >= 68; }

static int exact_faces() {
    static double host[EN], got[EN];
    for (size_t i = 0; i < EN; ++i) host[i] = -7.0;
    fort_scope_t ctx = 0;
    fort_buffer_t b = 0;
    CHECK(fort_scope_create(0, &ctx));
    size_t shape[3] = {EX, EY, EZ};
    int64_t lower[3] = {-10, 2, -100};
    fort_scope_layout layout{3, FORT_SCOPE_REAL64, 8, host, shape, lower, 1};
    CHECK(fort_scope_register(ctx, 1, 1, &layout, 1, &b));
    int previous = 0;
    void *raw = nullptr;
    CHECK(fort_scope_gpu_enter(ctx, &previous, &raw));
    cudaStream_t stream = static_cast<cudaStream_t>(raw);
    fort_scope_access write_all = whole(FORT_SCOPE_WRITE_ALL | FORT_SCOPE_OVERWRITE_ALL);
    double *device = nullptr;
    CHECK(fort_scope_device_begin(ctx, b, &write_all, reinterpret_cast<void **>(&device)));
    fill_index<<<(EN + 255) / 256, 256, 0, stream>>>(device);
    if (cudaGetLastError() != cudaSuccess) return 1;
    CHECK(fort_scope_note_launch(ctx));
    CHECK(fort_scope_device_end(ctx, b));
    size_t lo[3] = {3, 3, 2}, hi[3] = {131, 67, 68};
    fort_scope_section interior{lo, hi};
    fort_scope_access overwrite{0, 0, nullptr, 1, &interior, 1, &interior};
    CHECK(fort_scope_host_begin(ctx, b, &overwrite));
    for (size_t z = 2; z < 68; ++z)
        for (size_t y = 3; y < 67; ++y)
            for (size_t x = 3; x < 131; ++x) host[x + EX * (y + EY * z)] = -42.0;
    CHECK(fort_scope_host_end(ctx, b));
    CHECK(observe(ctx, b));
    fort_scope_stats first{}, mirrored{}, after{}, before{}, uploaded{};
    CHECK(fort_scope_stats_get(ctx, &first));
    const size_t face_bytes = (EN - size_t(128) * 64 * 66) * sizeof(double);
    int bad = 0;
    for (size_t z = 0; z < EZ; ++z)
        for (size_t y = 0; y < EY; ++y)
            for (size_t x = 0; x < EX; ++x) {
                const size_t i = x + EX * (y + EY * z);
                bad += host[i] != (in_halo(x, y, z) ? 1000000.0 + i : -42.0);
            }
    fort_scope_access read_all = whole(FORT_SCOPE_READ_ALL);
    CHECK(fort_scope_device_begin(ctx, b, &read_all, reinterpret_cast<void **>(&device)));
    CHECK(fort_scope_device_end(ctx, b));
    CHECK(fort_scope_wait(ctx));
    CHECK(fort_scope_stats_get(ctx, &mirrored));
    for (int n = 0; n < 20; ++n) {
        CHECK(fort_scope_host_begin(ctx, b, &read_all));
        CHECK(fort_scope_host_end(ctx, b));
        CHECK(fort_scope_device_begin(ctx, b, &read_all, reinterpret_cast<void **>(&device)));
        CHECK(fort_scope_device_end(ctx, b));
    }
    CHECK(fort_scope_stats_get(ctx, &after));
    size_t lows[6][3] = {{0, 0, 0}, {131, 0, 0}, {3, 0, 0}, {3, 67, 0}, {3, 3, 0}, {3, 3, 68}};
    size_t highs[6][3] = {{3, EY, EZ}, {EX, EY, EZ}, {131, 3, EZ}, {131, EY, EZ}, {131, 67, 2}, {131, 67, EZ}};
    fort_scope_section faces[6];
    for (int n = 0; n < 6; ++n) faces[n] = {lows[n], highs[n]};
    fort_scope_access halo_write{0, 0, nullptr, 6, faces, 6, faces};
    CHECK(fort_scope_host_begin(ctx, b, &halo_write));
    for (size_t z = 0; z < EZ; ++z)
        for (size_t y = 0; y < EY; ++y)
            for (size_t x = 0; x < EX; ++x)
                if (in_halo(x, y, z)) host[x + EX * (y + EY * z)] = 2000000.0 + (x + EX * (y + EY * z));
    CHECK(fort_scope_host_end(ctx, b));
    CHECK(fort_scope_stats_get(ctx, &before));
    CHECK(fort_scope_device_begin(ctx, b, &read_all, reinterpret_cast<void **>(&device)));
    CHECK(fort_scope_device_end(ctx, b));
    CHECK(fort_scope_wait(ctx));
    CHECK(fort_scope_stats_get(ctx, &uploaded));
    if (cudaMemcpy(got, device, sizeof got, cudaMemcpyDeviceToHost) != cudaSuccess) return 1;
    for (size_t i = 0; i < EN; ++i) bad += got[i] != host[i];
    CHECK(fort_scope_gpu_leave(ctx, previous));
    CHECK(fort_scope_close(ctx));
    std::printf("{\"scenario\": \"faces\", \"bad\": %d, \"downloads\": %llu, \"download_bytes\": %llu, "
                "\"face_bytes\": %zu, \"interleaved_transfers\": %llu, \"uploads\": %llu, \"upload_bytes\": %llu}\n",
                bad, (unsigned long long)first.downloads, (unsigned long long)first.download_bytes, face_bytes,
                (unsigned long long)(after.uploads - mirrored.uploads + after.downloads - mirrored.downloads),
                (unsigned long long)(uploaded.uploads - before.uploads),
                (unsigned long long)(uploaded.upload_bytes - before.upload_bytes));
    return 0;
}

static int byte_stripes() {
    constexpr size_t a = 135, b = 71, d = 71, n = a * b * d;
    static unsigned char host[n], got[n];
    std::memset(host, 0, sizeof host);
    fort_scope_t ctx = 0;
    fort_buffer_t buffer = 0;
    CHECK(fort_scope_create(0, &ctx));
    size_t shape[3] = {a, b, d};
    int64_t lower[3] = {-5, -9, 100};
    fort_scope_layout layout{3, FORT_SCOPE_BYTES, 1, host, shape, lower, 1};
    CHECK(fort_scope_register(ctx, 1, 1, &layout, 1, &buffer));
    int previous = 0;
    void *raw = nullptr;
    CHECK(fort_scope_gpu_enter(ctx, &previous, &raw));
    cudaStream_t stream = static_cast<cudaStream_t>(raw);
    fort_scope_access overwrite_all = whole(FORT_SCOPE_WRITE_ALL | FORT_SCOPE_OVERWRITE_ALL);
    unsigned char *device = nullptr;
    CHECK(fort_scope_device_begin(ctx, buffer, &overwrite_all, reinterpret_cast<void **>(&device)));
    fill_bytes<<<(n + 255) / 256, 256, 0, stream>>>(device, n);
    if (cudaGetLastError() != cudaSuccess) return 1;
    CHECK(fort_scope_note_launch(ctx));
    CHECK(fort_scope_device_end(ctx, buffer));
    size_t lo[20][3], hi[20][3];
    fort_scope_section sections[20];
    for (size_t k = 0; k < 20; ++k) {
        lo[k][0] = k * 6 + 1;
        lo[k][1] = lo[k][2] = 0;
        hi[k][0] = k * 6 + 2;
        hi[k][1] = b;
        hi[k][2] = d;
        sections[k] = {lo[k], hi[k]};
    }
    fort_scope_access reads{0, 20, sections, 0, nullptr, 0, nullptr};
    CHECK(fort_scope_host_begin(ctx, buffer, &reads));
    CHECK(fort_scope_host_end(ctx, buffer));
    int bad = 0;
    auto selected = [&](size_t i) { const size_t x = i % a; return x >= 1 && x <= 115 && (x - 1) % 6 == 0; };
    for (size_t i = 0; i < n; ++i) bad += host[i] != (selected(i) ? i % 251 + 1 : 0);
    fort_scope_stats first{}, last{};
    CHECK(fort_scope_stats_get(ctx, &first));
    fort_scope_access writes{0, 0, nullptr, 20, sections, 20, sections};
    CHECK(fort_scope_host_begin(ctx, buffer, &writes));
    for (size_t i = 0; i < n; ++i)
        if (selected(i)) host[i] = 255 - i % 251;
    CHECK(fort_scope_host_end(ctx, buffer));
    CHECK(fort_scope_device_begin(ctx, buffer, &reads, reinterpret_cast<void **>(&device)));
    CHECK(fort_scope_device_end(ctx, buffer));
    CHECK(fort_scope_wait(ctx));
    if (cudaMemcpy(got, device, n, cudaMemcpyDeviceToHost) != cudaSuccess) return 1;
    for (size_t i = 0; i < n; ++i) bad += got[i] != (selected(i) ? 255 - i % 251 : i % 251 + 1);
    CHECK(fort_scope_stats_get(ctx, &last));
    CHECK(fort_scope_gpu_leave(ctx, previous));
    CHECK(fort_scope_close(ctx));
    std::printf("{\"scenario\": \"stripes\", \"bad\": %d, \"downloads\": %llu, \"download_bytes\": %llu, "
                "\"uploads\": %llu, \"upload_bytes\": %llu, \"stripe_bytes\": %zu}\n",
                bad, (unsigned long long)first.downloads, (unsigned long long)first.download_bytes,
                (unsigned long long)last.uploads, (unsigned long long)last.upload_bytes, 20 * b * d);
    return 0;
}

int main(int argc, char **argv) {
    const std::string mode = argc > 1 ? argv[1] : "";
    if (mode == "faces") return exact_faces();
    if (mode == "stripes") return byte_stripes();
    if (mode == "completion") return completion();
    if (mode == "external") return external();
    if (mode == "queue") return queue_replay();
    if (mode == "group") return group_replay();
    if (mode == "cancel") return cancel();
    if (mode == "long") return long_chain();
    return 2;
}
"""


@pytest.fixture(scope="module")
def client(tmp_path_factory):
    library = native.build()
    directory = tmp_path_factory.mktemp("graph_client")
    source = directory / "client.cu"
    source.write_text(CLIENT)
    exe = directory / "client"
    built = subprocess.run([native.nvcc(), *native.ARCH, "-std=c++17", "-O2", "-cudart", "shared",
                            f"-I{native.INCLUDE}", str(source), "-o", str(exe), str(library),
                            f"-Xlinker=-rpath,{library.parent}"], capture_output=True, text=True)
    assert built.returncode == 0, built.stderr
    return exe


def _run(client: Path, mode: str, **env):
    import os

    run = subprocess.run([str(client), mode], capture_output=True, text=True, timeout=120,
                         env={**os.environ, **env})
    assert run.returncode == 0, run.stdout + run.stderr
    return {r["scenario"]: r for r in map(json.loads, run.stdout.splitlines())}


def test_queued_steps_replay_one_graph_with_new_parameters(client):
    q = _run(client, "queue")["queue"]
    assert (q["creations"], q["instantiations"], q["replays"], q["parameter_updates"]) == (1, 1, 2, 2)
    assert (q["accepted_tasks"], q["direct_submissions"], q["pending_tasks"]) == (4, 1, 0)
    assert (q["uploads"], q["downloads"]) == (1, 1)


def test_a_checked_group_replays_and_a_new_sequence_gets_its_own_graph(client):
    runs = _run(client, "group")
    group, topology = runs["group"], runs["topology"]
    assert group["creations"] == group["instantiations"] == 1
    assert group["replays"] >= 2 and group["parameter_updates"] >= 2
    assert topology["creations"] == group["creations"] + 1
    assert topology["live_graphs"] == 2


def test_cancelled_tasks_never_run(client):
    c = _run(client, "cancel")["cancel"]
    assert (c["accepted_tasks"], c["pending_tasks"], c["submissions"]) == (3, 0, 0)


def test_a_long_chain_goes_in_one_submission(client):
    chain = _run(client, "long")["long"]
    assert chain["accepted_tasks"] == 64 and chain["pending_tasks"] == 0
    assert chain["submissions"] == 1


def test_an_external_providers_kernel_is_ordered_before_the_publication(client):
    """The provider launches a deliberately slow kernel on the stream the runtime hands it; observing its output
    right after the call returns still sees every value it wrote (reference:
    test_scoped_domains_cuda.py:267-300, actual stream ordering)."""
    e = _run(client, "external")["external"]
    assert e["downloads"] == 1 and e["uploads"] == 1


def test_host_work_waits_only_for_the_device_work_it_conflicts_with(client):
    """While a kernel delayed by about 40 ms writes one array, host work on another array returns at once with no
    wait; host work on the written array waits for the kernel and sees its values (reference:
    test_scoped_host_completion_cuda.py:197-203, the independent scenario)."""
    r = _run(client, "completion")["completion"]
    assert r["pending_after_independent"] and r["independent_waits"] == 0 and r["independent_host_tasks"] >= 1
    assert r["dependent_saw_kernel"] and r["done_after_dependent"]


def test_sparse_sections_move_exactly_through_real_copies(client):
    """The halo of a 134 x 70 x 70 array (lower bounds -10, 2, -100) comes home as its six faces and goes back as
    six uploads of exactly those bytes; mirrors that both hold the values survive twenty interleaved read-only
    uses without a transfer; twenty byte stripes one element wide move as twenty pitched copies each way.
    Arrays are kept as device mirrors here (no in-place use of the host array), as the reference's direct
    transport keeps them (reference: test_scoped_direct_copy_cuda.py:111-118)."""
    faces = _run(client, "faces", FORT_SCOPE_HOST_IN_PLACE="0")["faces"]
    assert faces["bad"] == 0
    assert (faces["downloads"], faces["download_bytes"]) == (6, faces["face_bytes"])
    assert faces["interleaved_transfers"] == 0
    assert (faces["uploads"], faces["upload_bytes"]) == (6, faces["face_bytes"])
    stripes = _run(client, "stripes", FORT_SCOPE_HOST_IN_PLACE="0")["stripes"]
    assert stripes["bad"] == 0
    assert (stripes["downloads"], stripes["download_bytes"]) == (20, stripes["stripe_bytes"])
    assert (stripes["uploads"], stripes["upload_bytes"]) == (20, stripes["stripe_bytes"])


def test_closing_reports_the_graphs_it_destroyed(client):
    """With tracing on, closing the context reports its graph and queue statistics as evidence records: complete,
    no graph left alive, every graph created also destroyed (reference: test_scoped_graph_replay_cuda.py:241-258)."""
    import os

    run = subprocess.run([str(client), "group"], capture_output=True, text=True, timeout=120,
                         env={**os.environ, "FORT_RUNTIME_TRACE": "1"})
    assert run.returncode == 0, run.stdout + run.stderr
    records = [json.loads(line.removeprefix("FORT_SCOPED evidence ")) for line in run.stderr.splitlines()
               if line.startswith("FORT_SCOPED evidence ")]
    (graphs,) = [r for r in records if r["event"] == "graph_statistics"]
    assert graphs["complete"] and graphs["live_graphs"] == 0
    assert graphs["creations"] == graphs["destructions"] == 2
    assert run.stderr.count("FORT_SCOPED graph_submit ") == graphs["instantiations"] + graphs["replays"]

