// Device kernels of the advection templates: the fused z-marching tendency
// kernel and the single-pass boundary fill.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "advection_point.cuh"

namespace f2c {

constexpr int kMaxScalars = 4;
constexpr int kMaxHaloFields = 16;

struct AdvArgs {
    const double *u, *v, *w;
    double *out[3];
    const double *s[kMaxScalars];
    double *st[kMaxScalars];
    int nscalar, mode;
    double dt;
    int nx, ny, nz, h;
    int kz;  // levels per z-chunk of the face-sharing kernel
    long long sx, plane;
    Coefficients c;
    FastCoefficients f;  // the factored (fast-fp) kernel's coefficients, for this mode and dt
};

struct HaloArgs {
    double *f[kMaxHaloFields];
    int kind[kMaxHaloFields];
    int count;
    int nx, ny, nz, h;
    long long sx, plane;
};

// Bit 8 of a fused kernel's MASK template argument: the outputs are stored with their ghost images
// (F2C_ADVANCE_FILLED); used with all three velocity outputs (MASK 7 | kFillMask).
constexpr int kFillMask = 8;

__device__ __forceinline__ void store_result(double *out, const double *in, long long p, double t, int mode,
                                             double dt) {
    if (mode == 0) {
        out[p] = t;
    } else {
        out[p] = __ldg(in + p) + dt * t;
    }
}

// Output mode F2C_ADVANCE_FILLED: the new value v of interior point (i, j, k)
// is stored with every ghost the boundary fill (halo_row) would copy from it,
// so that the step needs no fill launch: periodic images in x and y, and in z
// the mirror (kind 0) or, for W (kind 1), the zero wall faces at levels h-1
// and h+nz-1 (written by the points of interior levels 0 and nz-1) and the
// sign-flipped mirrors beyond. Every ghost has exactly one source point, and
// the values are those the fill copies, so the result equals an advance step
// followed by f2c_halo_fill_v1 bit for bit. Needs nx >= h, ny >= h, nz > h.
__device__ __forceinline__ void store_filled(double *f, int kind, const AdvArgs &a, int i, int j, int k, double v) {
    const int h = a.h, nx = a.nx, ny = a.ny, nz = a.nz;
    // x and y targets: the point's own column and row and their periodic images (-1: none)
    const int x0 = i + h, x1 = i < h ? i + h + nx : -1, x2 = i >= nx - h ? i + h - nx : -1;
    const int y0 = j + h, y1 = j < h ? j + h + ny : -1, y2 = j >= ny - h ? j + h - ny : -1;
    const long long sx = a.sx, plane = a.plane;
    auto level = [&](int z, double val) {
        double *base = f + plane * z;
        auto row = [&](int y) {
            if (y < 0) return;
            double *r = base + sx * y;
            r[x0] = val;
            if (x1 >= 0) r[x1] = val;
            if (x2 >= 0) r[x2] = val;
        };
        row(y0);
        row(y1);
        row(y2);
    };
    if (kind == 0) {
        level(k + h, v);
        if (k < h) level(h - 1 - k, v);
        if (k >= nz - h) level(h + 2 * nz - 1 - k, v);
    } else {
        level(k + h, k == nz - 1 ? 0.0 : v);
        if (k == 0) level(h - 1, 0.0);
        if (k <= h - 2) level(h - 2 - k, -v);
        if (k >= nz - 1 - h && k <= nz - 2) level(h + 2 * nz - 2 - k, -v);
    }
}

// store_result, or for F2C_ADVANCE_FILLED the advanced value with its ghost images.
__device__ __forceinline__ void store_point(double *out, const double *in, long long p, double t, const AdvArgs &a,
                                            int kind, int i, int j, int k) {
    if (a.mode == 2) {
        store_filled(out, kind, a, i, j, k, __ldg(in + p) + a.dt * t);
    } else {
        store_result(out, in, p, t, a.mode, a.dt);
    }
}

// The same with the fill chosen at compile time (the face-sharing kernels' MASK bit 8, kFillMask): kernels
// without it keep their register budget.
template <bool FILL>
__device__ __forceinline__ void store_point_t(double *out, const double *in, long long p, double t, const AdvArgs &a,
                                              int kind, int i, int j, int k) {
    if (FILL) {
        store_filled(out, kind, a, i, j, k, __ldg(in + p) + a.dt * t);
    } else {
        store_result(out, in, p, t, a.mode, a.dt);
    }
}

// Direct z-marching kernel: one thread per (i, j) column of a BX x BY tile,
// marching KZ levels. Every value is read through the read-only path; the
// per-point expressions are those of advection_point.cuh.
template <int BX, int BY, int KZ>
__global__ void __launch_bounds__(BX *BY) advection_direct_kernel(const AdvArgs a) {
    const int i = blockIdx.x * BX + threadIdx.x;
    const int j = blockIdx.y * BY + threadIdx.y;
    if (i >= a.nx || j >= a.ny) return;
    const int k0 = blockIdx.z * KZ;
    const int k1 = min(k0 + KZ, a.nz);
    const double *__restrict__ U = a.u;
    const double *__restrict__ V = a.v;
    const double *__restrict__ W = a.w;
    const long long sx = a.sx, plane = a.plane;
    long long p = (long long)(i + a.h) + sx * (long long)(j + a.h) + plane * (long long)(k0 + a.h);
#define F2C_AT(A, di, dj, dk) __ldg((A) + p + (di) + (dj)*sx + (dk)*plane)
    for (int k = k0; k < k1; ++k, p += plane) {
        if (a.out[0]) store_point(a.out[0], U, p, F2C_CDU_POINT(F2C_AT, a.c), a, 0, i, j, k);
        if (a.out[1]) store_point(a.out[1], V, p, F2C_CDV_POINT(F2C_AT, a.c), a, 0, i, j, k);
        if (a.out[2]) store_point(a.out[2], W, p, F2C_CDW_POINT(F2C_AT, a.c), a, 1, i, j, k);
#pragma unroll
        for (int n = 0; n < kMaxScalars; ++n) {
            if (n < a.nscalar && a.st[n]) {
                const double *__restrict__ S = a.s[n];
                store_point(a.st[n], S, p, F2C_SCALAR_POINT(F2C_AT, S, a.c), a, 0, i, j, k);
            }
        }
    }
#undef F2C_AT
}

// Boundary fill in one pass: every ghost value is read from the interior point
// that the ordered fill (periodic x, then y over the whole x extent, then the
// vertical walls over whole planes) would copy into it. Periodic maps compose,
// and each vertical mirror source is an interior, non-wall level (nz > halo),
// so no ghost reads another ghost and the pass order is free.
//
// halo_row fills the ghosts of row (j, k) of one field (kind 0: periodic x/y,
// mirrored z; kind 1: the W rule, zero walls at h-1 and h+nz-1 and sign-flipped
// mirrors beyond); threads `lane` = 0.. stride `lanes` across the row. A row
// inside the interior in j and k has only its 2h x-ghosts to fill.
__device__ __forceinline__ void halo_row(double *__restrict__ f, int kind, int nx, int ny, int nz, int h, long long sx,
                                         long long plane, int j, int k, int lane, int lanes) {
    const int ex = nx + 2 * h;
    const bool jin = j >= h && j < h + ny;
    const bool kwall = kind == 1 && (k == h - 1 || k == h + nz - 1);
    const bool kin = k >= h && k < h + nz && !kwall;
    const int jj = j < h ? j + ny : (j >= h + ny ? j - ny : j);
    int kk = k;
    double sign = 1.0;
    if (kind == 0) {
        if (k < h) kk = 2 * h - 1 - k;
        else if (k >= h + nz) kk = 2 * (h + nz) - 1 - k;
    } else if (!kwall) {
        if (k < h - 1) { kk = 2 * (h - 1) - k; sign = -1.0; }
        else if (k >= h + nz) { kk = 2 * (h + nz - 1) - k; sign = -1.0; }
    }
    const long long dst_row = sx * (long long)j + plane * (long long)k;
    const long long src_row = sx * (long long)jj + plane * (long long)kk;
    if (jin && kin) {
        for (int t = lane; t < 2 * h; t += lanes) {
            const int i = t < h ? t : nx + t;
            const int ii = i < h ? i + nx : i - nx;
            f[dst_row + i] = f[src_row + ii];
        }
        return;
    }
    for (int i = lane; i < ex; i += lanes) {
        if (kwall) {
            f[dst_row + i] = 0.0;
            continue;
        }
        const int ii = i < h ? i + nx : (i >= h + nx ? i - nx : i);
        const double v = f[src_row + ii];
        f[dst_row + i] = sign < 0.0 ? -v : v;
    }
}

static __global__ void __launch_bounds__(256) halo_fill_kernel(const HaloArgs a) {
    const int ey = a.ny + 2 * a.h, ez = a.nz + 2 * a.h;
    const long long row = blockIdx.x;          // j + ey*k
    const int fidx = blockIdx.y;
    const int j = (int)(row % ey), k = (int)(row / ey);
    if (k >= ez || fidx >= a.count) return;
    halo_row(a.f[fidx], a.kind[fidx], a.nx, a.ny, a.nz, a.h, a.sx, a.plane, j, k, threadIdx.x, blockDim.x);
}

inline cudaError_t launch_advection(const AdvArgs &a, cudaStream_t stream) {
    constexpr int BX = 32, BY = 8, KZ = 16;
    const dim3 block(BX, BY, 1);
    const dim3 grid((a.nx + BX - 1) / BX, (a.ny + BY - 1) / BY, (a.nz + KZ - 1) / KZ);
    advection_direct_kernel<BX, BY, KZ><<<grid, block, 0, stream>>>(a);
    return cudaGetLastError();
}

inline cudaError_t launch_halo(const HaloArgs &a, cudaStream_t stream) {
    const long long rows = (long long)(a.ny + 2 * a.h) * (a.nz + 2 * a.h);
    if (rows > 0x7fffffffLL) return cudaErrorInvalidValue;
    const int ex = a.nx + 2 * a.h;
    const int threads = ex >= 256 ? 256 : ((ex + 31) / 32) * 32;
    halo_fill_kernel<<<dim3((unsigned)rows, (unsigned)a.count, 1), dim3(threads, 1, 1), 0, stream>>>(a);
    return cudaGetLastError();
}

} // namespace f2c
