// Fused advection templates for sm_103a and their kernel-level C ABI
// (include/f2c_advection.h).
//
// One launch computes the U, V, W momentum tendencies of the reference's CDU,
// CDV and CDW procedures (benchmarks/cdu/src/cdu.f90:113-133,
// compiler/tests/fixtures/stencils/{cvd,cdw}.f90:105-125) and up to four
// passive-scalar tendencies, replacing the reference's four grid-stride
// launches per procedure (compiler/emission/cuda/kernels.py:37-69).
#include "advection_fast.cuh"
#include "advection_faces.cuh"
#include "advection_kernels.cuh"
#include "procedures.cuh"

#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <string>

#include "../../../include/f2c_advection.h"

namespace f2c {

thread_local std::string g_last_error;

int fail(int status, const std::string &message) {
    g_last_error = message;
    return status;
}

// The output mode is known, and a filled advance has room for the boundary fill's images.
int check_mode(const f2c_grid_v1 *g, int mode) {
    if (mode != F2C_TENDENCY && mode != F2C_ADVANCE && mode != F2C_ADVANCE_FILLED) return fail(1, "unknown output mode");
    if (mode == F2C_ADVANCE_FILLED && (g->nz < g->halo + 1 || g->nx < g->halo || g->ny < g->halo))
        return fail(1, "a filled advance needs nz > halo, nx >= halo and ny >= halo");
    return 0;
}

static bool aligned8(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 7u) == 0; }

int check_grid(const f2c_grid_v1 *g) {
    if (!g) return fail(1, "null grid");
    if (g->nx < 1 || g->ny < 1 || g->nz < 1 || g->halo < 1)
        return fail(1, "grid needs nx, ny, nz >= 1 and halo >= 1");
    if (g->sx < g->nx + 2 * g->halo || g->sy < g->ny + 2 * g->halo)
        return fail(1, "grid strides smaller than the padded extents");
    if (g->nx > (1 << 24) || g->ny > (1 << 24) || g->nz > (1 << 24))
        return fail(1, "grid extent beyond 2^24");
    if (!(g->dx > 0.0) || !(g->dy > 0.0) || !(g->dz > 0.0)) return fail(1, "grid spacings must be positive");
    return 0;
}

static int fill_args(const f2c_grid_v1 *g, const f2c_fields_v1 *f, AdvArgs &a) {
    if (int s = check_grid(g)) return s;
    if (!f) return fail(1, "null field record");
    if (!f->u || !f->v || !f->w) return fail(1, "U, V and W are required");
    if (f->nscalar < 0 || f->nscalar > F2C_MAX_SCALARS) return fail(1, "scalar count out of range");
    if (int s = check_mode(g, f->mode)) return s;
    if (f->mode == F2C_ADVANCE_FILLED && (!f->ut || !f->vt || !f->wt))
        return fail(1, "a filled advance needs the U, V and W outputs");
    std::memset(&a, 0, sizeof a);
    a.u = f->u; a.v = f->v; a.w = f->w;
    a.out[0] = f->ut; a.out[1] = f->vt; a.out[2] = f->wt;
    const double *ins[3] = {f->u, f->v, f->w};
    for (int n = 0; n < 3; ++n) {
        if (!aligned8(ins[n]) || !aligned8(a.out[n])) return fail(1, "field pointers must be 8-byte aligned");
        for (int m = 0; m < 3; ++m)
            if (a.out[n] && a.out[n] == ins[m]) return fail(3, "an output aliases a velocity input");
    }
    a.nscalar = f->nscalar;
    for (int n = 0; n < f->nscalar; ++n) {
        if (!f->s[n]) return fail(1, "null scalar input");
        a.s[n] = f->s[n];
        a.st[n] = f->st[n];
        for (int m = 0; m < 3; ++m)
            if (a.st[n] && (a.st[n] == ins[m] || a.st[n] == f->s[n])) return fail(3, "a scalar output aliases an input");
    }
    a.mode = f->mode;
    a.dt = f->dt;
    a.nx = (int)g->nx; a.ny = (int)g->ny; a.nz = (int)g->nz; a.h = (int)g->halo;
    a.sx = g->sx;
    a.plane = g->sx * g->sy;
    a.c = make_coefficients(g->dx, g->dy, g->dz);
    a.f = make_fast_coefficients(g->dx, g->dy, g->dz, a.mode, a.dt);
    return 0;
}

} // namespace f2c

using namespace f2c;

extern "C" uint32_t f2c_advection_abi_version(void) { return F2C_ADVECTION_ABI_VERSION; }

extern "C" const char *f2c_last_error(void) { return g_last_error.c_str(); }

namespace f2c {

// Face-sharing kernel instantiations: all three velocities with 0..4 scalars,
// one velocity alone (the per-procedure entries CDU, CDV, CDW), scalars alone.
template <int NS>
static cudaError_t faces_for_mask(const AdvArgs &a, int mask, cudaStream_t s) {
    switch (mask) {
    case 7: return launch_faces<NS, 7>(a, s);
    case 1: return launch_faces<NS, 1>(a, s);
    case 2: return launch_faces<NS, 2>(a, s);
    case 4: return launch_faces<NS, 4>(a, s);
    case 0: return NS > 0 ? launch_faces<NS, 0>(a, s) : cudaSuccess;
    default: return launch_faces<NS, 7>(a, s);  // two of three: compute all, store the requested ones
    }
}

static cudaError_t launch_faces_dispatch(const AdvArgs &a, cudaStream_t s) {
    if (a.mode == F2C_ADVANCE_FILLED) {
        switch (a.nscalar) {
        case 0: return launch_faces<0, 7 | kFillMask>(a, s);
        case 1: return launch_faces<1, 7 | kFillMask>(a, s);
        case 2: return launch_faces<2, 7 | kFillMask>(a, s);
        case 3: return launch_faces<3, 7 | kFillMask>(a, s);
        default: return launch_faces<4, 7 | kFillMask>(a, s);
        }
    }
    const int mask = (a.out[0] ? 1 : 0) | (a.out[1] ? 2 : 0) | (a.out[2] ? 4 : 0);
    switch (a.nscalar) {
    case 0: return faces_for_mask<0>(a, mask, s);
    case 1: return faces_for_mask<1>(a, mask, s);
    case 2: return faces_for_mask<2>(a, mask, s);
    case 3: return faces_for_mask<3>(a, mask, s);
    default: return faces_for_mask<4>(a, mask, s);
    }
}

// Factored (fast-fp) kernel instantiations, with the same masks.
template <int NS>
static cudaError_t fast_for_mask(const AdvArgs &a, int mask, cudaStream_t s) {
    const int sms = current_sm_count();
    switch (mask) {
    case 7: return launch_fast<NS, 7, kFastTY>(a, sms, s);
    case 1: return launch_fast<NS, 1, kFastTY>(a, sms, s);
    case 2: return launch_fast<NS, 2, kFastTY>(a, sms, s);
    case 4: return launch_fast<NS, 4, kFastTY>(a, sms, s);
    case 0: return NS > 0 ? launch_fast<NS, 0, kFastTY>(a, sms, s) : cudaSuccess;
    default: return launch_fast<NS, 7, kFastTY>(a, sms, s);
    }
}

static cudaError_t launch_fast_dispatch(const AdvArgs &a, cudaStream_t s) {
    if (a.mode == F2C_ADVANCE_FILLED) {
        const int sms = current_sm_count();
        switch (a.nscalar) {
        case 0: return launch_fast<0, 7 | kFillMask, kFastTY>(a, sms, s);
        case 1: return launch_fast<1, 7 | kFillMask, kFastTY>(a, sms, s);
        case 2: return launch_fast<2, 7 | kFillMask, kFastTY>(a, sms, s);
        case 3: return launch_fast<3, 7 | kFillMask, kFastTY>(a, sms, s);
        default: return launch_fast<4, 7 | kFillMask, kFastTY>(a, sms, s);
        }
    }
    const int mask = (a.out[0] ? 1 : 0) | (a.out[1] ? 2 : 0) | (a.out[2] ? 4 : 0);
    switch (a.nscalar) {
    case 0: return fast_for_mask<0>(a, mask, s);
    case 1: return fast_for_mask<1>(a, mask, s);
    case 2: return fast_for_mask<2>(a, mask, s);
    case 3: return fast_for_mask<3>(a, mask, s);
    default: return fast_for_mask<4>(a, mask, s);
    }
}

} // namespace f2c

extern "C" int f2c_advection_variant_v1(const f2c_grid_v1 *grid, const f2c_fields_v1 *fields, int variant,
                                        void *stream) {
    AdvArgs a;
    if (int s = fill_args(grid, fields, a)) return s;
    if (variant < F2C_KERNEL_FACES || variant > F2C_KERNEL_FAST) return fail(1, "unknown advection kernel variant");
    const cudaStream_t st = static_cast<cudaStream_t>(stream);
    const cudaError_t e = variant == F2C_KERNEL_FACES  ? launch_faces_dispatch(a, st)
                          : variant == F2C_KERNEL_FAST ? launch_fast_dispatch(a, st)
                                                       : launch_advection(a, st);
    if (e != cudaSuccess) return fail(6, std::string("advection launch: ") + cudaGetErrorString(e));
    return 0;
}

extern "C" int f2c_advection_v1(const f2c_grid_v1 *grid, const f2c_fields_v1 *fields, void *stream) {
    return f2c_advection_variant_v1(grid, fields, F2C_KERNEL_FACES, stream);
}

extern "C" int f2c_halo_fill_v1(const f2c_grid_v1 *grid, double *const *fields, const int32_t *kinds, int32_t count,
                                void *stream) {
    if (int s = check_grid(grid)) return s;
    if (count < 0 || count > kMaxHaloFields) return fail(1, "halo field count out of range");
    if (count == 0) return 0;
    if (!fields || !kinds) return fail(1, "null halo field list");
    HaloArgs h;
    std::memset(&h, 0, sizeof h);
    for (int n = 0; n < count; ++n) {
        if (!fields[n]) return fail(1, "null halo field");
        if (kinds[n] != 0 && kinds[n] != 1) return fail(1, "unknown halo kind");
        h.f[n] = fields[n];
        h.kind[n] = kinds[n];
    }
    if (grid->nz < grid->halo + 1 || grid->nx < grid->halo || grid->ny < grid->halo)
        return fail(1, "halo fill needs nz > halo, nx >= halo and ny >= halo");
    h.count = count;
    h.nx = (int)grid->nx; h.ny = (int)grid->ny; h.nz = (int)grid->nz; h.h = (int)grid->halo;
    h.sx = grid->sx;
    h.plane = grid->sx * grid->sy;
    const cudaError_t e = launch_halo(h, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(6, std::string("halo launch: ") + cudaGetErrorString(e));
    return 0;
}

extern "C" int f2c_procedure_v1(int op, const f2c_grid_v1 *grid, double *out, const double *u, const double *v,
                                const double *w, double value, void *stream) {
    if (int s = check_grid(grid)) return s;
    if (op < kOpSet || op > kOpCdwAdv) return fail(1, "unknown procedure");
    if (!out) return fail(1, "null procedure output");
    if (op >= kOpCduDiv && (!u || !v || !w)) return fail(1, "null velocity");
    if (out == u || out == v || out == w) return fail(3, "procedure output aliases a velocity");
    ProcedureArgs p{};
    p.out = out;
    p.u = u; p.v = v; p.w = w;
    p.value = value;
    p.nx = (int)grid->nx; p.ny = (int)grid->ny; p.nz = (int)grid->nz; p.h = (int)grid->halo;
    p.sx = grid->sx;
    p.plane = grid->sx * grid->sy;
    p.c = make_coefficients(grid->dx, grid->dy, grid->dz);
    const dim3 g = procedure_grid(p), b(kProcBX, kProcBY, 1);
    const cudaStream_t st = static_cast<cudaStream_t>(stream);
    switch (op) {
    case kOpSet: procedure_kernel<kOpSet><<<g, b, 0, st>>>(p); break;
    case kOpMultiply: procedure_kernel<kOpMultiply><<<g, b, 0, st>>>(p); break;
    case kOpCduDiv: procedure_kernel<kOpCduDiv><<<g, b, 0, st>>>(p); break;
    case kOpCduAdv: procedure_kernel<kOpCduAdv><<<g, b, 0, st>>>(p); break;
    case kOpCdvDiv: procedure_kernel<kOpCdvDiv><<<g, b, 0, st>>>(p); break;
    case kOpCdvAdv: procedure_kernel<kOpCdvAdv><<<g, b, 0, st>>>(p); break;
    case kOpCdwDiv: procedure_kernel<kOpCdwDiv><<<g, b, 0, st>>>(p); break;
    default: procedure_kernel<kOpCdwAdv><<<g, b, 0, st>>>(p); break;
    }
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : fail(6, std::string("procedure launch: ") + cudaGetErrorString(e));
}
