// Per-procedure templates: one launch per reference procedure of the
// MomentumAdvection modules, for callers that run them one at a time:
//   set       benchmarks/cdu/src/cdu.f90:12-27    out(interior) = val
//   multiply  cdu.f90:30-45                       out(interior) = out * val
//   CDUdiv    cdu.f90:48-76                       out = -div           (CDVdiv, CDWdiv likewise)
//   CDUadv    cdu.f90:79-106                      out = out - adv      (CDVadv, CDWadv likewise)
// Each runs the same expressions as the fused kernels (advection_point.cuh),
// so the four-launch sequence set, div, adv, multiply(0.5) gives the fused
// result bit for bit.
#pragma once
#include <cuda_runtime.h>

#include "advection_point.cuh"

namespace f2c {

enum ProcedureOp : int {
    kOpSet = 0,
    kOpMultiply = 1,
    kOpCduDiv = 2,
    kOpCduAdv = 3,
    kOpCdvDiv = 4,
    kOpCdvAdv = 5,
    kOpCdwDiv = 6,
    kOpCdwAdv = 7,
};

struct ProcedureArgs {
    double *out;
    const double *u, *v, *w;
    double value;
    int nx, ny, nz, h;
    long long sx, plane;
    Coefficients c;
};

constexpr int kProcBX = 32, kProcBY = 8, kProcKZ = 16;

template <int OP>
__global__ void __launch_bounds__(kProcBX *kProcBY) procedure_kernel(const ProcedureArgs a) {
    const int i = blockIdx.x * kProcBX + threadIdx.x;
    const int j = blockIdx.y * kProcBY + threadIdx.y;
    if (i >= a.nx || j >= a.ny) return;
    const int k0 = blockIdx.z * kProcKZ;
    const int k1 = min(k0 + kProcKZ, a.nz);
    const double *__restrict__ U = a.u;
    const double *__restrict__ V = a.v;
    const double *__restrict__ W = a.w;
    double *__restrict__ out = a.out;
    const long long sx = a.sx, plane = a.plane;
    long long p = (long long)(i + a.h) + sx * (long long)(j + a.h) + plane * (long long)(k0 + a.h);
#define F2C_AT(A, di, dj, dk) __ldg((A) + p + (di) + (dj)*sx + (dk)*plane)
    for (int k = k0; k < k1; ++k, p += plane) {
        if (OP == kOpSet) out[p] = a.value;
        if (OP == kOpMultiply) out[p] = out[p] * a.value;
        if (OP == kOpCduDiv) out[p] = F2C_CDU_DIV(F2C_AT, a.c);
        if (OP == kOpCduAdv) out[p] = F2C_CDU_ADV(F2C_AT, a.c, out[p]);
        if (OP == kOpCdvDiv) out[p] = F2C_CDV_DIV(F2C_AT, a.c);
        if (OP == kOpCdvAdv) out[p] = F2C_CDV_ADV(F2C_AT, a.c, out[p]);
        if (OP == kOpCdwDiv) out[p] = F2C_CDW_DIV(F2C_AT, a.c);
        if (OP == kOpCdwAdv) out[p] = F2C_CDW_ADV(F2C_AT, a.c, out[p]);
    }
#undef F2C_AT
}

inline dim3 procedure_grid(const ProcedureArgs &a) {
    return dim3((a.nx + kProcBX - 1) / kProcBX, (a.ny + kProcBY - 1) / kProcBY, (a.nz + kProcKZ - 1) / kProcKZ);
}

} // namespace f2c
