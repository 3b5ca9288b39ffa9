/* CPU oracle for the generality stencils. TEST INFRASTRUCTURE ONLY.
 *
 * Restatements of the reference's other stencil forms so that the templates
 * of this repository that run them can be checked. Same numerical contract as
 * advection_oracle.c (-ffp-contract=off, source grouping kept).
 * Layout: column-major with h ghost layers, interior [h, h+n) per axis;
 * Dirichlet-zero boundaries are ghost values the caller keeps at zero.
 */
#include <stddef.h>
#include <stdint.h>

/* One explicit diffusion step, compiler/tests/apps/box/stepper.f90:8-30:
 *   b = a + dt*nu*laplacian,  laplacian = (a(i-1)+a(i+1)+a(j-1)+a(j+1)+a(k-1)+a(k+1) - 6*a)/(dx*dx). */
void orc_diffusion7(double *b, const double *a, double dt, double nu, double dx, int64_t nx, int64_t ny, int64_t nz,
                    int64_t h) {
    const int64_t sx = nx + 2 * h, sy = ny + 2 * h;
#define A(i, j, k) a[(size_t)(i) + sx * ((size_t)(j) + sy * (size_t)(k))]
#pragma omp parallel for collapse(2) schedule(static)
    for (int64_t k = h; k < h + nz; ++k)
        for (int64_t j = h; j < h + ny; ++j)
            for (int64_t i = h; i < h + nx; ++i) {
                const double lap = (A(i - 1, j, k) + A(i + 1, j, k) + A(i, j - 1, k) + A(i, j + 1, k) + A(i, j, k - 1) +
                                    A(i, j, k + 1) - 6.0 * A(i, j, k)) /
                                   (dx * dx);
                b[(size_t)i + sx * ((size_t)j + sy * (size_t)k)] = A(i, j, k) + dt * nu * lap;
            }
#undef A
}

/* One Jacobi sweep, compiler/tests/apps/relax/relax.f90:28-33:
 *   v = 0.25*(u(i-1,j) + u(i+1,j) + u(i,j-1) + u(i,j+1)). */
void orc_jacobi5(double *v, const double *u, int64_t nx, int64_t ny, int64_t h) {
    const int64_t sx = nx + 2 * h;
#define U(i, j) u[(size_t)(i) + sx * (size_t)(j)]
#pragma omp parallel for schedule(static)
    for (int64_t j = h; j < h + ny; ++j)
        for (int64_t i = h; i < h + nx; ++i)
            v[(size_t)i + sx * (size_t)j] = 0.25 * (U(i - 1, j) + U(i + 1, j) + U(i, j - 1) + U(i, j + 1));
#undef U
}

/* One 2-D Yee leapfrog step (TM mode). No reference source exists for it in the
 * mount (the PolyBench archive is absent), so the form is this project's:
 *   Hx(i,j) -= ch*(Ez(i,j+1) - Ez(i,j));  Hy(i,j) += ch*(Ez(i+1,j) - Ez(i,j))   over the interior,
 *   then Ez(i,j) += ce*((Hy(i,j) - Hy(i-1,j)) - (Hx(i,j) - Hx(i,j-1)))       over the interior. */
void orc_yee2d(double *ez, double *hx, double *hy, double ch, double ce, int64_t nx, int64_t ny, int64_t h) {
    const int64_t sx = nx + 2 * h;
#define AT(p, i, j) p[(size_t)(i) + sx * (size_t)(j)]
#pragma omp parallel for schedule(static)
    for (int64_t j = h; j < h + ny; ++j)
        for (int64_t i = h; i < h + nx; ++i) {
            AT(hx, i, j) = AT(hx, i, j) - ch * (AT(ez, i, j + 1) - AT(ez, i, j));
            AT(hy, i, j) = AT(hy, i, j) + ch * (AT(ez, i + 1, j) - AT(ez, i, j));
        }
#pragma omp parallel for schedule(static)
    for (int64_t j = h; j < h + ny; ++j)
        for (int64_t i = h; i < h + nx; ++i)
            AT(ez, i, j) = AT(ez, i, j) + ce * ((AT(hy, i, j) - AT(hy, i - 1, j)) - (AT(hx, i, j) - AT(hx, i, j - 1)));
#undef AT
}
