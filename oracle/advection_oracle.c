/* CPU oracle for the resident advection path. TEST INFRASTRUCTURE ONLY.
 *
 * This file restates, in plain C, the per-point arithmetic of the reference's
 * advection procedures so that the CUDA kernels of this repository can be
 * checked against it. It is the checker and the timed CPU baseline: nothing on
 * the product path links or calls it. Only tests, the smoke check and the CPU
 * baseline leg of the benchmark load it.
 *
 * Parity status: the reference stores no golden vectors for CDU/CDV/CDW and its
 * native control needs a Fortran compiler that is absent here. These
 * restatements are pinned against outputs of the reference's own source text
 * executed by a Fortran-subset interpreter (tests/golden/fortran_kernels.py,
 * fixtures tests/golden/reference_kernels.npz, bit for bit), against a second,
 * independent line-by-line Python transcription (oracle/literal.py) and against
 * hand-derived known answers.
 *
 * Numerical contract: compile with -ffp-contract=off (the reference's
 * "separate-arithmetic-v1", compiler/emission/numerical_contract.py:13-15).
 * Every expression keeps the source's left-to-right grouping; C parses
 * `a*b*c` as `(a*b)*c` and `a+b+c` as `(a+b)+c`, as Fortran does.
 *
 * Layout: Fortran column-major (i fastest), extents (nx+2h, ny+2h, nz+2h), the
 * interior is [h, h+n) on each axis. The reference driver uses h = 1
 * (benchmarks/cdu/src/main.f90:47-50); the stencil reaches +-1 only.
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define IDX(i, j, k) ((size_t)(i) + sx * ((size_t)(j) + sy * (size_t)(k)))

/* Momentum tendency of U: benchmarks/cdu/src/cdu.f90:113-133 (CDU), which calls
 * set (:12-27, dead: CDUdiv overwrites every interior point), CDUdiv (:48-76),
 * CDUadv (:79-106) and multiply by one half (:30-45). */
void orc_cdu(double *u2, const double *U, const double *V, const double *W, double dxmin, double dymin,
             double dzmin, int64_t nx, int64_t ny, int64_t nz, int64_t h) {
    const int64_t sx = nx + 2 * h, sy = ny + 2 * h;
    /* cdu.f90:57-59 */
    const double Ax = 0.25 / dxmin, Ay = 0.25 / dymin, Az = 0.25 / dzmin;
    /* cdu.f90:88-90 */
    const double Bx = 0.5 / dxmin, By = 0.125 / dymin, Bz = 0.125 / dzmin;
    const double half = 0.5;
#pragma omp parallel for collapse(2) schedule(static)
    for (int64_t k = h; k < h + nz; ++k)
        for (int64_t j = h; j < h + ny; ++j)
            for (int64_t i = h; i < h + nx; ++i) {
                /* cdu.f90:66-71 */
                double r = -((Ax * (U[IDX(i + 1, j, k)] + U[IDX(i, j, k)]) * (U[IDX(i + 1, j, k)] + U[IDX(i, j, k)]) -
                              Ax * (U[IDX(i, j, k)] + U[IDX(i - 1, j, k)]) * (U[IDX(i, j, k)] + U[IDX(i - 1, j, k)])) +
                             (Ay * (U[IDX(i, j + 1, k)] + U[IDX(i, j, k)]) * (V[IDX(i + 1, j, k)] + V[IDX(i, j, k)]) -
                              Ay * (U[IDX(i, j, k)] + U[IDX(i, j - 1, k)]) *
                                  (V[IDX(i + 1, j - 1, k)] + V[IDX(i, j - 1, k)])) +
                             (Az * (U[IDX(i, j, k + 1)] + U[IDX(i, j, k)]) * (W[IDX(i + 1, j, k)] + W[IDX(i, j, k)]) -
                              Az * (U[IDX(i, j, k)] + U[IDX(i, j, k - 1)]) *
                                  (W[IDX(i + 1, j, k - 1)] + W[IDX(i, j, k - 1)])));
                /* cdu.f90:96-101 */
                const double Vadv = (V[IDX(i, j, k)] + V[IDX(i + 1, j, k)] + V[IDX(i, j - 1, k)] + V[IDX(i + 1, j - 1, k)]);
                const double Wadv = (W[IDX(i, j, k)] + W[IDX(i + 1, j, k)] + W[IDX(i, j, k - 1)] + W[IDX(i + 1, j, k - 1)]);
                r = r - (Bx * (U[IDX(i + 1, j, k)] - U[IDX(i - 1, j, k)]) * U[IDX(i, j, k)] +
                         By * (U[IDX(i, j + 1, k)] - U[IDX(i, j - 1, k)]) * Vadv +
                         Bz * (U[IDX(i, j, k + 1)] - U[IDX(i, j, k - 1)]) * Wadv);
                /* cdu.f90:39 */
                u2[IDX(i, j, k)] = r * half;
            }
}

/* Momentum tendency of V: compiler/tests/fixtures/stencils/cvd.f90:105-125 (CDV),
 * CDVdiv formula :61-66 with coefficients :53-55, CDVadv :89-94 with :82-84. */
void orc_cdv(double *v2, const double *U, const double *V, const double *W, double dxmin, double dymin,
             double dzmin, int64_t nx, int64_t ny, int64_t nz, int64_t h) {
    const int64_t sx = nx + 2 * h, sy = ny + 2 * h;
    const double Ax = 0.25 / dxmin, Ay = 0.25 / dymin, Az = 0.25 / dzmin;
    const double Bx = 0.125 / dxmin, By = 0.5 / dymin, Bz = 0.125 / dzmin;
    const double half = 0.5;
#pragma omp parallel for collapse(2) schedule(static)
    for (int64_t k = h; k < h + nz; ++k)
        for (int64_t j = h; j < h + ny; ++j)
            for (int64_t i = h; i < h + nx; ++i) {
                double r = -((Ay * (V[IDX(i, j + 1, k)] + V[IDX(i, j, k)]) * (V[IDX(i, j + 1, k)] + V[IDX(i, j, k)]) -
                              Ay * (V[IDX(i, j, k)] + V[IDX(i, j - 1, k)]) * (V[IDX(i, j, k)] + V[IDX(i, j - 1, k)])) +
                             (Ax * (V[IDX(i + 1, j, k)] + V[IDX(i, j, k)]) * (U[IDX(i, j + 1, k)] + U[IDX(i, j, k)]) -
                              Ax * (V[IDX(i, j, k)] + V[IDX(i - 1, j, k)]) *
                                  (U[IDX(i - 1, j + 1, k)] + U[IDX(i - 1, j, k)])) +
                             (Az * (V[IDX(i, j, k + 1)] + V[IDX(i, j, k)]) * (W[IDX(i, j + 1, k)] + W[IDX(i, j, k)]) -
                              Az * (V[IDX(i, j, k)] + V[IDX(i, j, k - 1)]) *
                                  (W[IDX(i, j + 1, k - 1)] + W[IDX(i, j, k - 1)])));
                const double Uadv = (U[IDX(i, j, k)] + U[IDX(i, j + 1, k)] + U[IDX(i - 1, j, k)] + U[IDX(i - 1, j + 1, k)]);
                const double Wadv = (W[IDX(i, j, k)] + W[IDX(i, j + 1, k)] + W[IDX(i, j, k - 1)] + W[IDX(i, j + 1, k - 1)]);
                r = r - (Bx * (V[IDX(i + 1, j, k)] - V[IDX(i - 1, j, k)]) * Uadv +
                         By * (V[IDX(i, j + 1, k)] - V[IDX(i, j - 1, k)]) * V[IDX(i, j, k)] +
                         Bz * (V[IDX(i, j, k + 1)] - V[IDX(i, j, k - 1)]) * Wadv);
                v2[IDX(i, j, k)] = r * half;
            }
}

/* Momentum tendency of W: compiler/tests/fixtures/stencils/cdw.f90:105-125 (CDW),
 * CDWdiv formula :61-66 with coefficients :53-55, CDWadv :89-94 with :82-84. */
void orc_cdw(double *w2, const double *U, const double *V, const double *W, double dxmin, double dymin,
             double dzmin, int64_t nx, int64_t ny, int64_t nz, int64_t h) {
    const int64_t sx = nx + 2 * h, sy = ny + 2 * h;
    const double Ax = 0.25 / dxmin, Ay = 0.25 / dymin, Az = 0.25 / dzmin;
    const double Bx = 0.125 / dxmin, By = 0.125 / dymin, Bz = 0.5 / dzmin;
    const double half = 0.5;
#pragma omp parallel for collapse(2) schedule(static)
    for (int64_t k = h; k < h + nz; ++k)
        for (int64_t j = h; j < h + ny; ++j)
            for (int64_t i = h; i < h + nx; ++i) {
                double r = -((Az * (W[IDX(i, j, k + 1)] + W[IDX(i, j, k)]) * (W[IDX(i, j, k + 1)] + W[IDX(i, j, k)]) -
                              Az * (W[IDX(i, j, k)] + W[IDX(i, j, k - 1)]) * (W[IDX(i, j, k)] + W[IDX(i, j, k - 1)])) +
                             (Ay * (W[IDX(i, j + 1, k)] + W[IDX(i, j, k)]) * (V[IDX(i, j, k + 1)] + V[IDX(i, j, k)]) -
                              Ay * (W[IDX(i, j, k)] + W[IDX(i, j - 1, k)]) *
                                  (V[IDX(i, j - 1, k)] + V[IDX(i, j - 1, k + 1)])) +
                             (Ax * (W[IDX(i + 1, j, k)] + W[IDX(i, j, k)]) * (U[IDX(i, j, k + 1)] + U[IDX(i, j, k)]) -
                              Ax * (W[IDX(i, j, k)] + W[IDX(i - 1, j, k)]) *
                                  (U[IDX(i - 1, j, k + 1)] + U[IDX(i - 1, j, k)])));
                const double Uadv = (U[IDX(i, j, k)] + U[IDX(i, j, k + 1)] + U[IDX(i - 1, j, k)] + U[IDX(i - 1, j, k + 1)]);
                const double Vadv = (V[IDX(i, j, k)] + V[IDX(i, j, k + 1)] + V[IDX(i, j - 1, k)] + V[IDX(i, j - 1, k + 1)]);
                r = r - (Bx * (W[IDX(i + 1, j, k)] - W[IDX(i - 1, j, k)]) * Uadv +
                         By * (W[IDX(i, j + 1, k)] - W[IDX(i, j - 1, k)]) * Vadv +
                         Bz * (W[IDX(i, j, k + 1)] - W[IDX(i, j, k - 1)]) * W[IDX(i, j, k)]);
                w2[IDX(i, j, k)] = r * half;
            }
}

/* Passive scalar tendency. The reference mount has no scalar-advection source
 * (ELMM's scalar_advection.f90 is an external checkout, benchmarks/elmm/elmm.toml:46),
 * so this form is defined by this project: centred flux form on the C-grid,
 * U(i,j,k) on the east face of cell (i,j,k), V on its north face, W on its top face.
 * Face fluxes
 *   Fe = (Sx*U(i))*(s(i+1)+s(i)),  Fw = (Sx*U(i-1))*(s(i)+s(i-1)),   Sx = 0.5/dx,
 *   Fn = (Sy*V(j))*(s(j+1)+s(j)),  Fs = (Sy*V(j-1))*(s(j)+s(j-1)),   Sy = 0.5/dy,
 *   Ft = (Sz*W(k))*(s(k+1)+s(k)),  Fb = (Sz*W(k-1))*(s(k)+s(k-1)),   Sz = 0.5/dz,
 * and st = -(((Fe - Fw) + (Fn - Fs)) + (Ft - Fb)).
 * The east flux of point i is bit-identical to the west flux of point i+1 (IEEE
 * addition commutes exactly), and the products Sx*U do not depend on the
 * scalar, which lets a kernel compute each face once and share it. */
void orc_scalar(double *st, const double *s, const double *U, const double *V, const double *W, double dxmin,
                double dymin, double dzmin, int64_t nx, int64_t ny, int64_t nz, int64_t h) {
    const int64_t sx = nx + 2 * h, sy = ny + 2 * h;
    const double Sx = 0.5 / dxmin, Sy = 0.5 / dymin, Sz = 0.5 / dzmin;
#pragma omp parallel for collapse(2) schedule(static)
    for (int64_t k = h; k < h + nz; ++k)
        for (int64_t j = h; j < h + ny; ++j)
            for (int64_t i = h; i < h + nx; ++i) {
                const double c = s[IDX(i, j, k)];
                const double fe = (Sx * U[IDX(i, j, k)]) * (s[IDX(i + 1, j, k)] + c);
                const double fw = (Sx * U[IDX(i - 1, j, k)]) * (c + s[IDX(i - 1, j, k)]);
                const double fn = (Sy * V[IDX(i, j, k)]) * (s[IDX(i, j + 1, k)] + c);
                const double fs = (Sy * V[IDX(i, j - 1, k)]) * (c + s[IDX(i, j - 1, k)]);
                const double ft = (Sz * W[IDX(i, j, k)]) * (s[IDX(i, j, k + 1)] + c);
                const double fb = (Sz * W[IDX(i, j, k - 1)]) * (c + s[IDX(i, j, k - 1)]);
                st[IDX(i, j, k)] = -(((fe - fw) + (fn - fs)) + (ft - fb));
            }
}

/* Boundary fill of one field. Periodic in x, then in y over the whole x extent
 * (the order of compiler/tests/apps/box/boundaries.f90:6-41), then the vertical
 * walls over whole planes: kind 0 (U, V, scalars) mirrors the interior
 * (zero gradient); kind 1 (W, on top faces) sets the bottom wall face k=h-1 and
 * the top wall face k=h+nz-1 to zero and mirrors with a sign change beyond them.
 * Integer index work only; values are copied, never combined (bit-exact). */
void orc_halo(double *f, int kind, int64_t nx, int64_t ny, int64_t nz, int64_t h) {
    const int64_t sx = nx + 2 * h, sy = ny + 2 * h;
#pragma omp parallel for schedule(static)
    for (int64_t k = h; k < h + nz; ++k)
        for (int64_t j = h; j < h + ny; ++j)
            for (int64_t g = 0; g < h; ++g) {
                f[IDX(h + nx + g, j, k)] = f[IDX(h + g, j, k)];
                f[IDX(g, j, k)] = f[IDX(nx + g, j, k)];
            }
#pragma omp parallel for schedule(static)
    for (int64_t k = h; k < h + nz; ++k)
        for (int64_t g = 0; g < h; ++g)
            for (int64_t i = 0; i < sx; ++i) {
                f[IDX(i, h + ny + g, k)] = f[IDX(i, h + g, k)];
                f[IDX(i, g, k)] = f[IDX(i, ny + g, k)];
            }
    for (int64_t g = 0; g < h; ++g) {
#pragma omp parallel for schedule(static)
        for (int64_t j = 0; j < sy; ++j)
            for (int64_t i = 0; i < sx; ++i) {
                if (kind == 0) {
                    f[IDX(i, j, h - 1 - g)] = f[IDX(i, j, h + g)];
                    f[IDX(i, j, h + nz + g)] = f[IDX(i, j, h + nz - 1 - g)];
                } else {
                    if (g == 0) {
                        f[IDX(i, j, h - 1)] = 0.0;
                        f[IDX(i, j, h + nz - 1)] = 0.0;
                    } else {
                        f[IDX(i, j, h - 1 - g)] = -f[IDX(i, j, h - 1 + g)];
                    }
                    f[IDX(i, j, h + nz + g)] = -f[IDX(i, j, h + nz - 2 - g)];
                }
            }
    }
}

/* Forward-Euler stage of the advance mode: f(interior) = f + dt*ft. */
void orc_euler(double *f, const double *ft, double dt, int64_t nx, int64_t ny, int64_t nz, int64_t h) {
    const int64_t sx = nx + 2 * h, sy = ny + 2 * h;
#pragma omp parallel for collapse(2) schedule(static)
    for (int64_t k = h; k < h + nz; ++k)
        for (int64_t j = h; j < h + ny; ++j)
            for (int64_t i = h; i < h + nx; ++i) f[IDX(i, j, k)] = f[IDX(i, j, k)] + dt * ft[IDX(i, j, k)];
}

/* Interior checksum in the reference driver's order (main.f90:92 sums U2(2:NX+1,...)
 * in array element order); a plain left-to-right sum. */
double orc_interior_sum(const double *f, int64_t nx, int64_t ny, int64_t nz, int64_t h) {
    const int64_t sx = nx + 2 * h, sy = ny + 2 * h;
    double acc = 0.0;
    for (int64_t k = h; k < h + nz; ++k)
        for (int64_t j = h; j < h + ny; ++j)
            for (int64_t i = h; i < h + nx; ++i) acc = acc + f[IDX(i, j, k)];
    return acc;
}

int orc_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
