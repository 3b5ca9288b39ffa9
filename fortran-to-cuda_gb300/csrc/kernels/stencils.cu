// Kernel-level C ABI of the generality stencils (include/f2c_stencils.h).
#include "stencils.cuh"

#include <cuda_runtime.h>

#include <string>

#include "../../../include/f2c_stencils.h"

namespace f2c {
int fail(int status, const std::string &message);
int check_grid(const f2c_grid_v1 *g);
}  // namespace f2c

using namespace f2c;

extern "C" int f2c_diffusion7_v1(const f2c_grid_v1 *grid, const double *a, double *b, double dt, double nu,
                                 void *stream) {
    if (int s = check_grid(grid)) return s;
    if (!a || !b) return fail(1, "null diffusion field");
    if (a == b) return fail(3, "diffusion output aliases its input");
    DiffusionArgs p{};
    p.a = a;
    p.b = b;
    p.dtnu = dt * nu;
    p.dx2 = grid->dx * grid->dx;
    p.dx2_pow2 = power_of_two(p.dx2, &p.dx2_exp) ? 1 : 0;
    p.nx = (int)grid->nx; p.ny = (int)grid->ny; p.nz = (int)grid->nz; p.h = (int)grid->halo;
    p.sx = grid->sx;
    p.plane = grid->sx * grid->sy;
    diffusion7_kernel<<<diffusion_grid(p), dim3(kDiffBX, kDiffBY, 1), 0, static_cast<cudaStream_t>(stream)>>>(p);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : fail(6, std::string("diffusion launch: ") + cudaGetErrorString(e));
}

static int check_plane(int64_t nx, int64_t ny, int64_t halo, int64_t sx) {
    if (nx < 1 || ny < 1 || halo < 1 || nx > (1 << 28) || ny > (1 << 28)) return fail(1, "bad 2-D extents");
    if (sx < nx + 2 * halo) return fail(1, "row stride smaller than the padded extent");
    return 0;
}

extern "C" int f2c_jacobi5_v1(const double *u, double *v, int64_t nx, int64_t ny, int64_t halo, int64_t sx,
                              void *stream) {
    if (int s = check_plane(nx, ny, halo, sx)) return s;
    if (!u || !v) return fail(1, "null Jacobi field");
    if (u == v) return fail(3, "Jacobi output aliases its input");
    JacobiArgs p{u, v, (int)nx, (int)ny, (int)halo, sx};
    jacobi5_kernel<<<jacobi_grid(p), dim3(kJacBX, kJacBY, 1), 0, static_cast<cudaStream_t>(stream)>>>(p);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : fail(6, std::string("Jacobi launch: ") + cudaGetErrorString(e));
}

extern "C" int f2c_yee2d_v1(double *ez, double *hx, double *hy, int64_t nx, int64_t ny, int64_t halo, int64_t sx,
                            double ch, double ce, void *stream) {
    if (int s = check_plane(nx, ny, halo, sx)) return s;
    if (!ez || !hx || !hy) return fail(1, "null Yee field");
    if (ez == hx || ez == hy || hx == hy) return fail(3, "Yee fields alias");
    YeeArgs p{ez, hx, hy, ch, ce, (int)nx, (int)ny, (int)halo, sx};
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    yee_h_kernel<<<yee_grid(p), dim3(kYeeBX, kYeeBY, 1), 0, s>>>(p);
    yee_e_kernel<<<yee_grid(p), dim3(kYeeBX, kYeeBY, 1), 0, s>>>(p);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : fail(6, std::string("Yee launch: ") + cudaGetErrorString(e));
}
