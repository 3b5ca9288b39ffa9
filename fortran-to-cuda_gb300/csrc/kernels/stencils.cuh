// Generality stencils on the same z-march / 2-D tile machinery as the
// advection templates, FP64 with the reference grouping (bit-identical to the
// oracle):
//   diffusion7: compiler/tests/apps/box/stepper.f90:8-30
//       b = a + dt*nu*((a(i-1)+a(i+1)+a(j-1)+a(j+1)+a(k-1)+a(k+1) - 6*a)/(dx*dx))
//   jacobi5:    compiler/tests/apps/relax/relax.f90:28-33
//       v = 0.25*(u(i-1)+u(i+1)+u(j-1)+u(j+1))
//   yee2d:      2-D TM leapfrog (this project's form; no reference source in the mount)
//       Hx -= ch*(Ez(j+1)-Ez); Hy += ch*(Ez(i+1)-Ez); then Ez += ce*((Hy-Hy(i-1)) - (Hx-Hx(j-1)))
// Dirichlet-zero boundaries are ghost values kept at zero; no kernel writes a ghost.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "soft_fp64.cuh"

// The products below run on the integer pipes (mul_rn_int: the correctly
// rounded product, the same bits as DMUL), leaving the FP64 pipe, which bounds
// these stencils, to the additions.
namespace f2c {

// x * 2^e for an exact power-of-two factor, on the integer pipe when the
// result stays normal (the same bits as the correctly rounded product);
// the FP64 multiply otherwise.
// The multiplication for the rare operands the exponent shift cannot take. Out
// of line, so that the common path issues no FP64 instruction (an inline
// fallback is evaluated alongside and costs one FP64 multiply per point).
static __device__ __noinline__ double scale_by(double x, double factor) { return x * factor; }

__device__ __forceinline__ double scale_pow2(double x, int e, double factor) {
    const long long b = __double_as_longlong(x);
    const int ex = (int)((unsigned long long)b >> 52) & 0x7ff;
    const int r = ex + e;
    if (ex != 0 && ex != 0x7ff && r >= 1 && r <= 0x7fe) return __longlong_as_double(b + ((long long)e << 52));
    return scale_by(x, factor);
}

struct DiffusionArgs {
    const double *a;
    double *b;
    double dtnu;      // dt*nu, formed on the host exactly as the source does
    double dx2;       // dx*dx
    int dx2_pow2;     // dx*dx is 2^dx2_exp: the division is an exact scaling
    int dx2_exp;
    int nx, ny, nz, h;
    long long sx, plane;
};

constexpr int kDiffBX = 32, kDiffBY = 8, kDiffKZ = 32;

static __global__ void __launch_bounds__(kDiffBX *kDiffBY) diffusion7_kernel(const DiffusionArgs p) {
    const int i = blockIdx.x * kDiffBX + threadIdx.x;
    const int j = blockIdx.y * kDiffBY + threadIdx.y;
    if (i >= p.nx || j >= p.ny) return;
    const int k0 = blockIdx.z * kDiffKZ;
    const int k1 = min(k0 + kDiffKZ, p.nz);
    const double *__restrict__ A = p.a;
    const long long sx = p.sx, plane = p.plane;
    long long q = (long long)(i + p.h) + sx * (long long)(j + p.h) + plane * (long long)(k0 + p.h);
    double below = __ldg(A + q - plane), centre = __ldg(A + q);
    for (int k = k0; k < k1; ++k, q += plane) {
        const double above = __ldg(A + q + plane);
        const double sum = __ldg(A + q - 1) + __ldg(A + q + 1) + __ldg(A + q - sx) + __ldg(A + q + sx) + below + above;
        const double num = sum - mul_rn_int(6.0, centre);
        const double lap = p.dx2_pow2 ? scale_pow2(num, -p.dx2_exp, 1.0 / p.dx2) : num / p.dx2;
        p.b[q] = centre + mul_rn_int(p.dtnu, lap);
        below = centre;
        centre = above;
    }
}

struct JacobiArgs {
    const double *u;
    double *v;
    int nx, ny, h;
    long long sx;
};

constexpr int kJacBX = 64, kJacBY = 4, kJacJY = 8;  // each thread does kJacJY rows

static __global__ void __launch_bounds__(kJacBX *kJacBY) jacobi5_kernel(const JacobiArgs p) {
    const int i = blockIdx.x * kJacBX + threadIdx.x;
    const int j0 = (blockIdx.y * kJacBY + threadIdx.y) * kJacJY;
    if (i >= p.nx) return;
    const double *__restrict__ U = p.u;
    const long long sx = p.sx;
    long long q = (long long)(i + p.h) + sx * (long long)(j0 + p.h);
    const int j1 = min(j0 + kJacJY, p.ny);
    double south = j0 < p.ny ? __ldg(U + q - sx) : 0.0;
    double centre = j0 < p.ny ? __ldg(U + q) : 0.0;
    for (int j = j0; j < j1; ++j, q += sx) {
        const double north = __ldg(U + q + sx);
        const double sum = __ldg(U + q - 1) + __ldg(U + q + 1) + south + north;
        p.v[q] = scale_pow2(sum, -2, 0.25);
        south = centre;
        centre = north;
    }
}

struct YeeArgs {
    double *ez, *hx, *hy;
    double ch, ce;
    int nx, ny, h;
    long long sx;
};

constexpr int kYeeBX = 64, kYeeBY = 4;

static __global__ void __launch_bounds__(kYeeBX *kYeeBY) yee_h_kernel(const YeeArgs p) {
    const int i = blockIdx.x * kYeeBX + threadIdx.x;
    const int j = blockIdx.y * kYeeBY + threadIdx.y;
    if (i >= p.nx || j >= p.ny) return;
    const long long q = (long long)(i + p.h) + p.sx * (long long)(j + p.h);
    const double e = __ldg(p.ez + q);
    p.hx[q] = p.hx[q] - mul_rn_int(p.ch, __ldg(p.ez + q + p.sx) - e);
    p.hy[q] = p.hy[q] + mul_rn_int(p.ch, __ldg(p.ez + q + 1) - e);
}

static __global__ void __launch_bounds__(kYeeBX *kYeeBY) yee_e_kernel(const YeeArgs p) {
    const int i = blockIdx.x * kYeeBX + threadIdx.x;
    const int j = blockIdx.y * kYeeBY + threadIdx.y;
    if (i >= p.nx || j >= p.ny) return;
    const long long q = (long long)(i + p.h) + p.sx * (long long)(j + p.h);
    p.ez[q] = p.ez[q] + mul_rn_int(p.ce, (__ldg(p.hy + q) - __ldg(p.hy + q - 1)) - (__ldg(p.hx + q) - __ldg(p.hx + q - p.sx)));
}

inline dim3 diffusion_grid(const DiffusionArgs &p) {
    return dim3((p.nx + kDiffBX - 1) / kDiffBX, (p.ny + kDiffBY - 1) / kDiffBY, (p.nz + kDiffKZ - 1) / kDiffKZ);
}
inline dim3 jacobi_grid(const JacobiArgs &p) {
    return dim3((p.nx + kJacBX - 1) / kJacBX, (p.ny + kJacBY * kJacJY - 1) / (kJacBY * kJacJY), 1);
}
inline dim3 yee_grid(const YeeArgs &p) { return dim3((p.nx + kYeeBX - 1) / kYeeBX, (p.ny + kYeeBY - 1) / kYeeBY, 1); }

// Exponent e with x == 2^e exactly, or a flag that x is not a power of two.
inline bool power_of_two(double x, int *e) {
    if (!(x > 0.0)) return false;
    int k = 0;
    double m = x;
    while (m >= 2.0 && k < 1100) { m *= 0.5; ++k; }
    while (m < 1.0 && k > -1100) { m *= 2.0; --k; }
    if (m != 1.0) return false;
    *e = k;
    return true;
}

} // namespace f2c
