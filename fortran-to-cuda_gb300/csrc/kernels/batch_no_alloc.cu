// Batched advection step that allocates nothing (f2c_batch_step_static_v1, include/f2c_batch.h).
//
// f2c_batch_step_v1 keeps its instance descriptors, tile queue and work
// counter in a device workspace the caller allocates. Some callers cannot
// allocate device memory when they want to step an ensemble: their device
// memory is already fully handed to another allocator (a caching allocator,
// or a residency budget sized to the whole device), or they run a
// time-stepping loop in which the device-wide synchronisation that cudaFree
// implies is not acceptable. This entry keeps the same scratch in a fixed
// array that the library itself holds in device memory, so such a caller only
// passes its fields.
//
// The array is a file-scope __device__ variable: every GPU that loads the
// library holds its kNoAllocScratchBytes until the process exits, and every
// call on a device shares (and overwrites) that device's array. Calls that
// overlap on the GPU, or come from several host threads at once, race on it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>

#include "../../../include/f2c_batch.h"
#include "advection_faces.cuh"

namespace f2c {
int fail(int status, const std::string &message);
int check_grid(const f2c_grid_v1 *g);
int check_mode(const f2c_grid_v1 *g, int mode);

namespace {

struct NoAllocItem {
    int instance;
    short tile_x, tile_y;
    int k0, k1;
};
static_assert(sizeof(NoAllocItem) == 16, "item layout");

constexpr size_t kAlignment = 256;
constexpr size_t round_up(size_t v) { return (v + kAlignment - 1) / kAlignment * kAlignment; }
constexpr size_t kCounterBytes = kAlignment;
constexpr size_t kDescriptorBytes = round_up(sizeof(AdvArgs) * F2C_BATCH_NO_ALLOC_MAX_INSTANCES);
constexpr size_t kNoAllocScratchBytes =
    kCounterBytes + kDescriptorBytes + sizeof(NoAllocItem) * (size_t)F2C_BATCH_NO_ALLOC_MAX_ITEMS;
static_assert(kNoAllocScratchBytes <= F2C_BATCH_NO_ALLOC_SCRATCH_BYTES, "stated scratch size");

// The scratch: [work counter | instance descriptors | tile queue].
static __device__ __align__(256) unsigned char g_no_alloc_scratch[F2C_BATCH_NO_ALLOC_SCRATCH_BYTES];

// Device address of the array per device ordinal, found once per device with that device current.
constexpr int kMaxDevices = 64;
void *g_scratch_address[kMaxDevices] = {};

// Host staging, also static: a pageable copy source is consumed before cudaMemcpyAsync returns.
AdvArgs g_descriptors[F2C_BATCH_NO_ALLOC_MAX_INSTANCES];
NoAllocItem g_items[F2C_BATCH_NO_ALLOC_MAX_ITEMS];

template <int NS, int MASK>
__global__ void __launch_bounds__(kFaceThreads, kFaceCtasPerSM) no_alloc_batched_kernel(unsigned char *scratch,
                                                                                 int nitems) {
    extern __shared__ double smem[];
    __shared__ int slot;
    unsigned *counter = reinterpret_cast<unsigned *>(scratch);
    const AdvArgs *instances = reinterpret_cast<const AdvArgs *>(scratch + kCounterBytes);
    const NoAllocItem *items = reinterpret_cast<const NoAllocItem *>(scratch + kCounterBytes + kDescriptorBytes);
    for (;;) {
        if (threadIdx.x == 0 && threadIdx.y == 0) slot = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int n = slot;
        __syncthreads();
        if (n >= nitems) return;
        const NoAllocItem it = items[n];
        faces_tile<NS, MASK>(instances[it.instance], it.tile_x, it.tile_y, it.k0, it.k1, smem);
    }
}

struct NoAllocKernel {
    const void *fn;
    size_t smem;
    cudaError_t status;  // of the shared-memory limit set on the current device
};

// The kernel's dynamic shared-memory limit is a property of each device: set once per device ordinal.
template <int NS, int MASK>
NoAllocKernel no_alloc_kernel() {
    static std::atomic<unsigned long long> configured{0};
    const cudaError_t e = configure_shared_once(configured, (const void *)no_alloc_batched_kernel<NS, MASK>,
                                                (int)FaceSmem<NS, MASK>::bytes);
    return {(const void *)no_alloc_batched_kernel<NS, MASK>, FaceSmem<NS, MASK>::bytes, e};
}

template <int MASK>
NoAllocKernel no_alloc_kernel_ns(int ns) {
    switch (ns) {
    case 0: return no_alloc_kernel<0, MASK>();
    case 1: return no_alloc_kernel<1, MASK>();
    case 2: return no_alloc_kernel<2, MASK>();
    case 3: return no_alloc_kernel<3, MASK>();
    default: return no_alloc_kernel<4, MASK>();
    }
}

NoAllocKernel no_alloc_kernel_for(int ns, int mask) {
    switch (mask) {
    case 1: return no_alloc_kernel_ns<1>(ns);
    case 2: return no_alloc_kernel_ns<2>(ns);
    case 4: return no_alloc_kernel_ns<4>(ns);
    case 0: return no_alloc_kernel_ns<0>(ns);
    default: return no_alloc_kernel_ns<7>(ns);
    }
}

// Set-up, once per device and with that device current: the device address of the array.
int scratch_address(void **out) {
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return fail(6, std::string("no current device: ") + cudaGetErrorString(e));
    if (device < 0 || device >= kMaxDevices) return fail(1, "device ordinal beyond the no-allocation table");
    if (!g_scratch_address[device]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_no_alloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(6, std::string("cannot find the no-allocation scratch: ") + cudaGetErrorString(e));
        g_scratch_address[device] = p;
    }
    *out = g_scratch_address[device];
    return 0;
}

}  // namespace
}  // namespace f2c

using namespace f2c;

extern "C" int f2c_batch_step_static_v1(const f2c_grid_v1 *grids, const f2c_fields_v1 *fields, const int32_t *kz,
                                        int32_t count, void *stream) {
    if (!grids || !fields || count <= 0) return fail(1, "empty batch");
    if (count > F2C_BATCH_NO_ALLOC_MAX_INSTANCES)
        return fail(1, "batch has more instances than the no-allocation maximum (F2C_BATCH_NO_ALLOC_MAX_INSTANCES)");
    int ns = -1, mask = -1;
    size_t nitems = 0;
    for (int n = 0; n < count; ++n) {
        if (int s = check_grid(&grids[n])) return s;
        const f2c_fields_v1 &f = fields[n];
        if (!f.u || !f.v || !f.w) return fail(1, "batch instance without velocities");
        if (f.nscalar < 0 || f.nscalar > F2C_MAX_SCALARS) return fail(1, "scalar count out of range");
        const int m = (f.ut ? 1 : 0) | (f.vt ? 2 : 0) | (f.wt ? 4 : 0);
        if (n == 0) {
            ns = f.nscalar;
            mask = m;
        } else if (f.nscalar != ns || m != mask || f.mode != fields[0].mode) {
            return fail(1, "batch instances differ in scalars, outputs or mode");
        }
        if (kz && kz[n] < 0) return fail(1, "negative z-chunk depth");
        if (int s = check_mode(&grids[n], f.mode)) return s;
        if (f.mode == F2C_ADVANCE_FILLED) return fail(1, "the no-allocation step takes the tendency or advance mode");
        const int c = kz && kz[n] > 0 ? kz[n] : kFaceKZ;
        const f2c_grid_v1 &g = grids[n];
        const long long tx = (g.nx + kFaceTX - 1) / kFaceTX, ty = (g.ny + kFaceTY - 1) / kFaceTY;
        if (tx > 32767 || ty > 32767) return fail(1, "instance too wide for the tile queue");
        nitems += (size_t)(tx * ty * ((g.nz + c - 1) / c));
        if (nitems > (size_t)F2C_BATCH_NO_ALLOC_MAX_ITEMS)
            return fail(1, "batch has more work items than the no-allocation maximum (F2C_BATCH_NO_ALLOC_MAX_ITEMS)");
    }
    if (mask != 7 && mask != 1 && mask != 2 && mask != 4 && mask != 0) mask = 7;
    if (mask == 0 && ns == 0) return fail(1, "batch computes nothing");
    void *scratch = nullptr;
    if (int s = scratch_address(&scratch)) return s;
    // descriptors and the queue, staged in static host arrays
    size_t at = 0;
    for (int n = 0; n < count; ++n) {
        const f2c_fields_v1 &f = fields[n];
        const f2c_grid_v1 &g = grids[n];
        AdvArgs &a = g_descriptors[n];
        std::memset(&a, 0, sizeof a);
        a.u = f.u; a.v = f.v; a.w = f.w;
        a.out[0] = f.ut; a.out[1] = f.vt; a.out[2] = f.wt;
        a.nscalar = f.nscalar;
        for (int s = 0; s < f.nscalar; ++s) {
            if (!f.s[s]) return fail(1, "null scalar input");
            a.s[s] = f.s[s];
            a.st[s] = f.st[s];
        }
        a.mode = f.mode;
        a.dt = f.dt;
        a.nx = (int)g.nx; a.ny = (int)g.ny; a.nz = (int)g.nz; a.h = (int)g.halo;
        a.sx = g.sx;
        a.plane = g.sx * g.sy;
        a.c = make_coefficients(g.dx, g.dy, g.dz);
        a.f = make_fast_coefficients(g.dx, g.dy, g.dz, a.mode, a.dt);
        const int c = kz && kz[n] > 0 ? kz[n] : kFaceKZ;
        const int tx = (int)((g.nx + kFaceTX - 1) / kFaceTX), ty = (int)((g.ny + kFaceTY - 1) / kFaceTY);
        for (int k0 = 0; k0 < g.nz; k0 += c)
            for (int y = 0; y < ty; ++y)
                for (int x = 0; x < tx; ++x)
                    g_items[at++] = {n, (short)x, (short)y, k0, (int)std::min<int64_t>(k0 + c, g.nz)};
    }
    // largest items first; ties in queue order (std::sort works in place)
    auto cost = [&](const NoAllocItem &it) {
        const f2c_grid_v1 &g = grids[it.instance];
        const long long w = std::min<long long>(kFaceTX, g.nx - (long long)it.tile_x * kFaceTX);
        const long long h = std::min<long long>(kFaceTY, g.ny - (long long)it.tile_y * kFaceTY);
        return w * h * (it.k1 - it.k0);
    };
    std::sort(g_items, g_items + at, [&](const NoAllocItem &a, const NoAllocItem &b) {
        const long long ca = cost(a), cb = cost(b);
        if (ca != cb) return ca > cb;
        if (a.instance != b.instance) return a.instance < b.instance;
        if (a.k0 != b.k0) return a.k0 < b.k0;
        if (a.tile_y != b.tile_y) return a.tile_y < b.tile_y;
        return a.tile_x < b.tile_x;
    });
    const cudaStream_t st = static_cast<cudaStream_t>(stream);
    unsigned char *base = static_cast<unsigned char *>(scratch);
    cudaError_t e = cudaMemcpyAsync(base + kCounterBytes, g_descriptors, sizeof(AdvArgs) * (size_t)count,
                                    cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(base + kCounterBytes + kDescriptorBytes, g_items, sizeof(NoAllocItem) * at,
                            cudaMemcpyHostToDevice, st);
    // the counter keeps the previous call's value: start from zero
    if (e == cudaSuccess) e = cudaMemsetAsync(base, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return fail(6, std::string("no-allocation batch staging: ") + cudaGetErrorString(e));
    const NoAllocKernel k = no_alloc_kernel_for(ns, mask);
    if (k.status != cudaSuccess)
        return fail(6, std::string("no-allocation batch kernel set-up: ") + cudaGetErrorString(k.status));
    const int sms = current_sm_count();
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k.fn, kFaceThreads, k.smem);
    if (e != cudaSuccess || per_sm < 1) return fail(6, "no-allocation batch kernel does not fit on an SM");
    const unsigned ctas = (unsigned)std::min<size_t>((size_t)sms * per_sm, at);
    int items = (int)at;
    void *args[] = {(void *)&base, (void *)&items};
    e = cudaLaunchKernel(k.fn, dim3(ctas), dim3(kFaceTX, kFaceTY + 1, 1), args, k.smem, st);
    if (e != cudaSuccess) return fail(6, std::string("no-allocation batch launch: ") + cudaGetErrorString(e));
    return 0;
}
