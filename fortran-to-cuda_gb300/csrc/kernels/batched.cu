// Persistent batched advection over a flattened tile queue (include/f2c_batch.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../../include/f2c_batch.h"
#include "advection_fast.cuh"
#include "advection_faces.cuh"

namespace f2c {
int fail(int status, const std::string &message);
int check_grid(const f2c_grid_v1 *g);
int check_mode(const f2c_grid_v1 *g, int mode);

struct BatchItem {
    int instance;
    short tile_x, tile_y;
    int k0, k1;
};
static_assert(sizeof(BatchItem) == 16, "batch item layout");

struct BatchHeader {
    unsigned counter;
    unsigned pad[63];
};

namespace {

constexpr size_t kAlign = 256;
size_t align_up(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

// The tile's instance arguments, copied into shared memory by the whole CTA
// (as 8-byte words) so that the tile reads its coefficients and pointers
// from shared memory rather than through global loads of the instance table.
static_assert(sizeof(AdvArgs) % 8 == 0 && alignof(AdvArgs) == 8, "instance arguments copied as 8-byte words");
__device__ __forceinline__ void stage_args(AdvArgs *dst, const AdvArgs *src) {
    const unsigned long long *from = reinterpret_cast<const unsigned long long *>(src);
    unsigned long long *to = reinterpret_cast<unsigned long long *>(dst);
    const int threads = blockDim.x * blockDim.y;
    for (int w = threadIdx.y * blockDim.x + threadIdx.x; w < (int)(sizeof(AdvArgs) / 8); w += threads) to[w] = from[w];
}

template <int NS, int MASK>
__global__ void __launch_bounds__(kFaceThreads, kFaceCtasPerSM)
    advection_batched_kernel(const AdvArgs *__restrict__ instances, const BatchItem *__restrict__ items, int nitems,
                             unsigned *counter) {
    extern __shared__ double smem[];
    __shared__ int slot;
    __shared__ AdvArgs args;
    for (;;) {
        if (threadIdx.x == 0 && threadIdx.y == 0) slot = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int n = slot;
        __syncthreads();  // every thread has read the slot (and left the previous tile) before the next one
        if (n >= nitems) return;
        const BatchItem it = items[n];
        stage_args(&args, instances + it.instance);
        __syncthreads();
        faces_tile<NS, MASK>(args, it.tile_x, it.tile_y, it.k0, it.k1, smem);
    }
}

// The same persistent loop over the fast-fp tile (advection_fast.cuh), tiles of 32 x TY points: TY + 1
// warps per CTA; small tiles run more CTAs per SM (the register budget at 96 per thread).

template <int NS, int MASK, int TY>
__global__ void __launch_bounds__(fast_threads<TY>(), fast_ctas_per_sm<TY>())
    advection_batched_fast_kernel(const AdvArgs *__restrict__ instances, const BatchItem *__restrict__ items,
                                  int nitems, unsigned *counter) {
    __shared__ double smem[FastSmem<TY>::doubles];
    __shared__ int slot;
    __shared__ AdvArgs args;
    for (;;) {
        if (threadIdx.x == 0 && threadIdx.y == 0) slot = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int n = slot;
        __syncthreads();  // every thread has read the slot (and left the previous tile) before the next one
        if (n >= nitems) return;
        const BatchItem it = items[n];
        stage_args(&args, instances + it.instance);
        __syncthreads();
        fast_tile<NS, MASK, TY>(args, it.tile_x, it.tile_y, it.k0, it.k1, smem);
    }
}

struct Kernel {
    const void *fn;
    size_t smem;
    cudaError_t status;
};

template <int NS, int MASK>
Kernel kernel_of(bool fast, int rows) {
    if (fast) {
        switch (rows) {
        case 4: return {(const void *)advection_batched_fast_kernel<NS, MASK, 4>, 0, cudaSuccess};
        case 16: return {(const void *)advection_batched_fast_kernel<NS, MASK, 16>, 0, cudaSuccess};
        default: return {(const void *)advection_batched_fast_kernel<NS, MASK, 8>, 0, cudaSuccess};
        }
    }
    static std::atomic<unsigned long long> configured{0};
    const cudaError_t e = configure_shared_once(configured, (const void *)advection_batched_kernel<NS, MASK>,
                                                (int)FaceSmem<NS, MASK>::bytes);
    return {(const void *)advection_batched_kernel<NS, MASK>, FaceSmem<NS, MASK>::bytes, e};
}

template <int MASK>
Kernel kernel_for_ns(int ns, bool fast, int rows) {
    switch (ns) {
    case 0: return kernel_of<0, MASK>(fast, rows);
    case 1: return kernel_of<1, MASK>(fast, rows);
    case 2: return kernel_of<2, MASK>(fast, rows);
    case 3: return kernel_of<3, MASK>(fast, rows);
    default: return kernel_of<4, MASK>(fast, rows);
    }
}

Kernel kernel_for(int ns, int mask, bool fast, int rows) {
    switch (mask) {
    case 7 | kFillMask: return kernel_for_ns<7 | kFillMask>(ns, fast, rows);
    case 1: return kernel_for_ns<1>(ns, fast, rows);
    case 2: return kernel_for_ns<2>(ns, fast, rows);
    case 4: return kernel_for_ns<4>(ns, fast, rows);
    case 0: return kernel_for_ns<0>(ns, fast, rows);
    default: return kernel_for_ns<7>(ns, fast, rows);
    }
}

// Tile rows of a plan (the fast-fp kernel's tile height; 8 for plans of the strict kernel).
int plan_rows(const f2c_batch_plan_v1 *plan) {
    const int r = (int)((plan->reserved >> 8) & 0xffu);
    return r ? r : kFaceTY;
}

int chunk(const int32_t *kz, int n) { return kz && kz[n] > 0 ? kz[n] : kFaceKZ; }

size_t item_count(const f2c_grid_v1 *grids, const int32_t *kz, int count, int rows) {
    size_t items = 0;
    for (int n = 0; n < count; ++n) {
        const f2c_grid_v1 &g = grids[n];
        const int c = chunk(kz, n);
        items += (size_t)((g.nx + kFaceTX - 1) / kFaceTX) * ((g.ny + rows - 1) / rows) * ((g.nz + c - 1) / c);
    }
    return items;
}

bool rows_ok(int rows) { return rows == 4 || rows == 8 || rows == 16; }

}  // namespace
}  // namespace f2c

using namespace f2c;

extern "C" size_t f2c_batch_workspace_bytes_rows_v1(const f2c_grid_v1 *grids, const int32_t *kz, int32_t count,
                                                    int32_t tile_rows) {
    if (!grids || count <= 0 || !rows_ok(tile_rows)) return 0;
    return align_up(sizeof(BatchHeader)) + align_up(sizeof(AdvArgs) * (size_t)count) +
           align_up(sizeof(BatchItem) * item_count(grids, kz, count, tile_rows));
}

extern "C" size_t f2c_batch_workspace_bytes_v1(const f2c_grid_v1 *grids, const int32_t *kz, int32_t count) {
    return f2c_batch_workspace_bytes_rows_v1(grids, kz, count, kFaceTY);
}

namespace f2c {
namespace {
// Descriptors and the flattened item queue of a batch, built and checked on the host.
struct Built {
    std::vector<AdvArgs> descs;
    std::vector<BatchItem> items;
    int ns = -1, mask = -1, rows = kFaceTY;
    bool halo_ok = true; // every instance admits the boundary fill (nz > halo, nx and ny >= halo)
};

int build(const f2c_grid_v1 *grids, const f2c_fields_v1 *fields, const int32_t *kz, int32_t count, int rows,
          Built &out) {
    if (!grids || !fields || count <= 0) return fail(1, "empty batch");
    if (!rows_ok(rows)) return fail(1, "tile rows must be 4, 8 or 16");
    out.rows = rows;
    std::vector<AdvArgs> &descs = out.descs;
    descs.assign((size_t)count, AdvArgs{});
    int ns = -1, mask = -1;
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
        AdvArgs &a = descs[(size_t)n];
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
        const f2c_grid_v1 &g = grids[n];
        a.nx = (int)g.nx; a.ny = (int)g.ny; a.nz = (int)g.nz; a.h = (int)g.halo;
        a.sx = g.sx;
        a.plane = g.sx * g.sy;
        a.c = make_coefficients(g.dx, g.dy, g.dz);
        a.f = make_fast_coefficients(g.dx, g.dy, g.dz, a.mode, a.dt);
        if (g.nz < g.halo + 1 || g.nx < g.halo || g.ny < g.halo) out.halo_ok = false;
    }
    if (mask != 7 && mask != 1 && mask != 2 && mask != 4 && mask != 0) mask = 7;
    if (mask == 0 && ns == 0) return fail(1, "batch computes nothing");
    if (fields[0].mode == F2C_ADVANCE_FILLED) {
        if (mask != 7) return fail(1, "a filled advance needs the U, V and W outputs");
        mask = 7 | kFillMask;
    }
    // the flattened queue: full-depth items first (largest first), then the partial ones
    std::vector<BatchItem> &items = out.items;
    items.clear();
    items.reserve(item_count(grids, kz, count, rows));
    for (int n = 0; n < count; ++n) {
        const f2c_grid_v1 &g = grids[n];
        const int c = chunk(kz, n);
        const int tx = (int)((g.nx + kFaceTX - 1) / kFaceTX), ty = (int)((g.ny + rows - 1) / rows);
        if (tx > 32767 || ty > 32767) return fail(1, "instance too wide for the tile queue");
        for (int k0 = 0; k0 < g.nz; k0 += c)
            for (int y = 0; y < ty; ++y)
                for (int x = 0; x < tx; ++x)
                    items.push_back({n, (short)x, (short)y, k0, (int)std::min<int64_t>(k0 + c, g.nz)});
    }
    auto cost = [&](const BatchItem &it) {
        const f2c_grid_v1 &g = grids[it.instance];
        const long long w = std::min<long long>(kFaceTX, g.nx - (long long)it.tile_x * kFaceTX);
        const long long h = std::min<long long>(rows, g.ny - (long long)it.tile_y * rows);
        return w * h * (it.k1 - it.k0);
    };
    std::stable_sort(items.begin(), items.end(),
                     [&](const BatchItem &a, const BatchItem &b) { return cost(a) > cost(b); });
    out.ns = ns;
    out.mask = mask;
    return 0;
}

size_t descs_offset() { return align_up(sizeof(BatchHeader)); }
size_t items_offset(int count) { return descs_offset() + align_up(sizeof(AdvArgs) * (size_t)count); }

// The plan of a built batch whose descriptors and items are (being) copied into `workspace`.
int finish(const Built &b, int32_t count, void *workspace, size_t workspace_bytes, f2c_batch_plan_v1 *plan) {
    // the persistent grid is sized for the smaller occupancy of the kernels that can run the plan (either
    // numerical contract for 8-row tiles, since F2C_BATCH_FAST_FP may be set after preparation; the fast-fp
    // kernel alone for 4- and 16-row tiles)
    const int sms = current_sm_count();
    int per_sm = 1 << 30;
    for (const bool fast : {false, true}) {
        if (!fast && b.rows != kFaceTY) continue;
        const Kernel k = kernel_for(b.ns, b.mask, fast, b.rows);
        if (k.status != cudaSuccess) return fail(6, std::string("batch kernel set-up: ") + cudaGetErrorString(k.status));
        int n = 0;
        const int threads = kFaceTX * (b.rows + 1);
        const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k.fn, threads, k.smem);
        if (e != cudaSuccess || n < 1) return fail(6, "batch kernel does not fit on an SM");
        per_sm = std::min(per_sm, n);
    }
    plan->workspace = workspace;
    plan->workspace_bytes = workspace_bytes;
    plan->count = count;
    plan->nscalar = b.ns;
    plan->mask = b.mask;
    plan->items = (int32_t)b.items.size();
    plan->ctas = (uint32_t)std::min<size_t>((size_t)sms * per_sm, b.items.size());
    plan->reserved = (b.halo_ok ? F2C_BATCH_HALO_OK : 0u) | (b.rows != kFaceTY ? F2C_BATCH_FAST_FP : 0u) |
                     ((uint32_t)b.rows << 8);
    return 0;
}

// Halo fill of every instance's outputs: one warp per (instance, field, row) unit,
// instances found by a binary search over their first units (shared memory).
constexpr int kBatchHaloThreads = 256;
constexpr int kBatchHaloMaxInstances = 4096;

__global__ void __launch_bounds__(kBatchHaloThreads) batch_halo_kernel(const AdvArgs *__restrict__ inst, int count,
                                                                      int nfields) {
    extern __shared__ long long first[]; // first[n]: first unit of instance n; first[count]: all units
    for (int n = threadIdx.x; n < count; n += blockDim.x) {
        const AdvArgs &a = inst[n];
        first[n + 1] = (long long)(a.ny + 2 * a.h) * (a.nz + 2 * a.h) * nfields;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        first[0] = 0;
        for (int n = 1; n <= count; ++n) first[n] += first[n - 1];
    }
    __syncthreads();
    const long long total = first[count];
    const int lane = threadIdx.x & 31, warps = blockDim.x >> 5;
    for (long long u = (long long)blockIdx.x * warps + (threadIdx.x >> 5); u < total;
         u += (long long)gridDim.x * warps) {
        int lo = 0, hi = count - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (first[mid] <= u) lo = mid;
            else hi = mid - 1;
        }
        const AdvArgs &a = inst[lo];
        const int ey = a.ny + 2 * a.h;
        const long long rows = (long long)ey * (a.nz + 2 * a.h);
        const long long local = u - first[lo];
        const int fidx = (int)(local / rows);
        const long long row = local - (long long)fidx * rows;
        double *f = fidx < 3 ? a.out[fidx] : a.st[fidx - 3];
        if (!f) continue;
        halo_row(f, fidx == 2 ? 1 : 0, a.nx, a.ny, a.nz, a.h, a.sx, a.plane, (int)(row % ey), (int)(row / ey), lane,
                 32);
    }
}
}  // namespace
}  // namespace f2c

extern "C" int f2c_batch_prepare_rows_v1(const f2c_grid_v1 *grids, const f2c_fields_v1 *fields, const int32_t *kz,
                                         int32_t count, int32_t tile_rows, void *workspace, size_t workspace_bytes,
                                         void *staging, void *stream, f2c_batch_plan_v1 *plan) {
    if (!grids || !fields || count <= 0 || !plan) return fail(1, "empty batch");
    if (!workspace) return fail(1, "null batch workspace");
    if (!rows_ok(tile_rows)) return fail(1, "tile rows must be 4, 8 or 16");
    if (workspace_bytes < f2c_batch_workspace_bytes_rows_v1(grids, kz, count, tile_rows))
        return fail(4, "batch workspace too small");
    Built b;
    if (int s = build(grids, fields, kz, count, tile_rows, b)) return s;
    char *base = static_cast<char *>(workspace);
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t descs = descs_offset(), items = items_offset(count);
    cudaError_t e;
    if (staging) {  // through the caller's host staging, without waiting
        char *host = static_cast<char *>(staging);
        std::memcpy(host + descs, b.descs.data(), sizeof(AdvArgs) * b.descs.size());
        std::memcpy(host + items, b.items.data(), sizeof(BatchItem) * b.items.size());
        const size_t bytes = items + sizeof(BatchItem) * b.items.size() - descs;
        e = cudaMemcpyAsync(base + descs, host + descs, bytes, cudaMemcpyHostToDevice, s);
    } else {
        e = cudaMemcpyAsync(base + descs, b.descs.data(), sizeof(AdvArgs) * b.descs.size(), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(base + items, b.items.data(), sizeof(BatchItem) * b.items.size(),
                                cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    }
    if (e != cudaSuccess) return fail(6, std::string("batch prepare: ") + cudaGetErrorString(e));
    return finish(b, count, workspace, workspace_bytes, plan);
}

extern "C" int f2c_batch_prepare_v1(const f2c_grid_v1 *grids, const f2c_fields_v1 *fields, const int32_t *kz,
                                    int32_t count, void *workspace, size_t workspace_bytes, void *stream,
                                    f2c_batch_plan_v1 *plan) {
    if (!grids || !fields || count <= 0 || !plan) return fail(1, "empty batch");
    if (!workspace) return fail(1, "null batch workspace");
    return f2c_batch_prepare_rows_v1(grids, fields, kz, count, kFaceTY, workspace, workspace_bytes, nullptr, stream,
                                     plan);
}

extern "C" int f2c_batch_prepare_async_v1(const f2c_grid_v1 *grids, const f2c_fields_v1 *fields, const int32_t *kz,
                                          int32_t count, void *workspace, size_t workspace_bytes, void *staging,
                                          void *stream, f2c_batch_plan_v1 *plan) {
    if (!grids || !fields || count <= 0 || !plan) return fail(1, "empty batch");
    if (!workspace || !staging) return fail(1, "null batch workspace or staging");
    return f2c_batch_prepare_rows_v1(grids, fields, kz, count, kFaceTY, workspace, workspace_bytes, staging, stream,
                                     plan);
}

extern "C" int f2c_batch_halo_v1(const f2c_batch_plan_v1 *plan, void *stream) {
    if (!plan || !plan->workspace || plan->count <= 0) return fail(1, "batch plan not prepared");
    if (plan->count > kBatchHaloMaxInstances) return fail(1, "batch halo fill takes at most 4096 instances");
    if (!(plan->reserved & F2C_BATCH_HALO_OK)) return fail(1, "halo fill needs nz > halo, nx >= halo and ny >= halo in every instance");
    const AdvArgs *descs = reinterpret_cast<const AdvArgs *>(static_cast<char *>(plan->workspace) + descs_offset());
    const int sms = current_sm_count();
    const int count = plan->count, nfields = 3 + plan->nscalar;
    const size_t shared = sizeof(long long) * (size_t)(count + 1);
    batch_halo_kernel<<<(unsigned)(sms > 0 ? sms * 8 : 1216), kBatchHaloThreads, shared,
                        static_cast<cudaStream_t>(stream)>>>(descs, count, nfields);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(6, std::string("batch halo launch: ") + cudaGetErrorString(e));
    return 0;
}

extern "C" int f2c_batch_step_v1(const f2c_batch_plan_v1 *plan, void *stream) {
    if (!plan || !plan->workspace || plan->items <= 0) return fail(1, "batch plan not prepared");
    const int rows = plan_rows(plan);
    const bool fast = (plan->reserved & F2C_BATCH_FAST_FP) != 0;
    if (!rows_ok(rows)) return fail(1, "batch plan with unknown tile rows");
    if (!fast && rows != kFaceTY) return fail(1, "tiles of 4 or 16 rows run only the fast-fp kernel");
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    char *base = static_cast<char *>(plan->workspace);
    unsigned *counter = reinterpret_cast<unsigned *>(base);
    const AdvArgs *descs = reinterpret_cast<const AdvArgs *>(base + descs_offset());
    const BatchItem *items = reinterpret_cast<const BatchItem *>(base + items_offset(plan->count));
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) return fail(6, std::string("batch counter reset: ") + cudaGetErrorString(e));
    const Kernel k = kernel_for(plan->nscalar, plan->mask, fast, rows);
    if (k.status != cudaSuccess) return fail(6, std::string("batch kernel set-up: ") + cudaGetErrorString(k.status));
    int nitems = plan->items;
    void *args[] = {(void *)&descs, (void *)&items, (void *)&nitems, (void *)&counter};
    e = cudaLaunchKernel(k.fn, dim3(plan->ctas), dim3(kFaceTX, rows + 1, 1), args, k.smem, s);
    if (e != cudaSuccess) return fail(6, std::string("batch launch: ") + cudaGetErrorString(e));
    return 0;
}

extern "C" int f2c_batch_graph_create_v1(const f2c_batch_plan_v1 *plan, void **graph) {
    if (!plan || !graph) return fail(1, "null plan or graph output");
    *graph = nullptr;
    cudaStream_t capture = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&capture, cudaStreamNonBlocking);
    if (e != cudaSuccess) return fail(6, std::string("batch graph stream: ") + cudaGetErrorString(e));
    e = cudaStreamBeginCapture(capture, cudaStreamCaptureModeThreadLocal);
    int status = e == cudaSuccess ? f2c_batch_step_v1(plan, capture) : 6;
    cudaGraph_t g = nullptr;
    const cudaError_t end = e == cudaSuccess ? cudaStreamEndCapture(capture, &g) : e;
    cudaGraphExec_t exec = nullptr;
    if (status == 0 && end == cudaSuccess) {
        e = cudaGraphInstantiate(&exec, g, 0);
        if (e != cudaSuccess) status = fail(6, std::string("batch graph instantiation: ") + cudaGetErrorString(e));
    } else if (status == 0) {
        status = fail(6, std::string("batch graph capture: ") + cudaGetErrorString(end));
    }
    if (g) cudaGraphDestroy(g);
    cudaStreamDestroy(capture);
    if (status == 0) *graph = exec;
    return status;
}

extern "C" int f2c_batch_graph_launch_v1(void *graph, void *stream) {
    if (!graph) return fail(1, "null batch graph");
    const cudaError_t e = cudaGraphLaunch(static_cast<cudaGraphExec_t>(graph), static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(6, std::string("batch graph launch: ") + cudaGetErrorString(e));
    return 0;
}

extern "C" int f2c_batch_graph_destroy_v1(void *graph) {
    if (graph) cudaGraphExecDestroy(static_cast<cudaGraphExec_t>(graph));
    return 0;
}
