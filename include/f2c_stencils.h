/* Kernel-level C ABI of the generality stencils (device pointers, one stream).
 *
 * Reference forms restated: the box app's explicit diffusion step
 * (compiler/tests/apps/box/stepper.f90:8-30) and the relax app's Jacobi sweep
 * (compiler/tests/apps/relax/relax.f90:28-33); the 2-D Yee leapfrog is this
 * project's form (no reference source in the mount). Column-major FP64 with
 * `halo` ghost layers; ghosts hold the Dirichlet-zero boundary and are never
 * written. Results are bit-identical to the C oracle. Statuses as
 * fort_scope_status.
 */
#ifndef F2C_STENCILS_H
#define F2C_STENCILS_H
#include <stdint.h>

#include "f2c_advection.h"
#ifdef __cplusplus
extern "C" {
#endif

/* b(interior) = a + dt*nu*laplacian(a)/(dx*dx); `b` must not alias `a`. Uses grid->dx only. */
int f2c_diffusion7_v1(const f2c_grid_v1 *grid, const double *a, double *b, double dt, double nu, void *stream);
/* v(interior) = 0.25*(u(i-1)+u(i+1)+u(j-1)+u(j+1)) on an (nx+2h) x (ny+2h) array with row stride sx. */
int f2c_jacobi5_v1(const double *u, double *v, int64_t nx, int64_t ny, int64_t halo, int64_t sx, void *stream);
/* One leapfrog step: H from E, then E from H (two launches on `stream`). */
int f2c_yee2d_v1(double *ez, double *hx, double *hy, int64_t nx, int64_t ny, int64_t halo, int64_t sx, double ch,
                 double ce, void *stream);

#ifdef __cplusplus
}
#endif
#endif
