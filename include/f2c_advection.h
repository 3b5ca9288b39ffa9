/* Kernel-level C ABI of the GB300 resident advection templates.
 *
 * These entry points take DEVICE pointers, a geometry record and a CUDA stream
 * and enqueue the hand-written sm_103a kernels; they never allocate, copy or
 * synchronise. They are what the generated numerical entries
 * (cpp_fort_shared_*, fort_shared_entries.h) launch through the residency
 * runtime, and what batched and serving callers launch directly.
 *
 * Reference interface replaced: the per-nest kernels the reference emits for
 * the advection procedures (compiler/emission/cuda/kernels.py:37-69,118-122,
 * launched at :172-201) for benchmarks/cdu/src/cdu.f90:12-133 and
 * compiler/tests/fixtures/stencils/{cvd,cdw}.f90:44-125. One launch here does
 * the work of the reference's four launches per procedure (set, *div, *adv,
 * multiply) for all requested fields at once.
 *
 * Layout: Fortran column-major FP64, i fastest, `halo` ghost layers on every
 * side; element (i,j,k) (0-based, interior [halo, halo+n)) is at
 * i + sx*(j + sy*k). Strides may exceed the extents (pitched mirrors).
 * Status values are those of fort_scope_status (scoped_runtime.h).
 */
#ifndef F2C_ADVECTION_H
#define F2C_ADVECTION_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#define F2C_ADVECTION_ABI_VERSION 1
#define F2C_MAX_SCALARS 4

typedef struct f2c_grid_v1 {
    int64_t nx, ny, nz; /* interior cells */
    int64_t halo;       /* ghost layers per side, >= 1 */
    int64_t sx, sy;     /* elements per j row (>= nx+2*halo) and rows per k plane (>= ny+2*halo) */
    double dx, dy, dz;  /* spacings (the reference's dxmin, dymin, dzmin) */
} f2c_grid_v1;

/* Output modes. TENDENCY writes the tendency (the reference's U2, V2, W2).
 * ADVANCE writes out = in + dt*tendency (forward Euler, double-buffered: the
 * outputs must not alias any input). ADVANCE_FILLED is ADVANCE with the
 * outputs' ghost layers filled in the same launch, bit for bit as
 * f2c_halo_fill_v1 fills them afterwards (U, V and scalars periodic in x and y
 * and mirrored in z, W with zero wall faces): a complete step in one launch;
 * it needs nz > halo, nx >= halo and ny >= halo. */
enum f2c_output_mode { F2C_TENDENCY = 0, F2C_ADVANCE = 1, F2C_ADVANCE_FILLED = 2 };

typedef struct f2c_fields_v1 {
    const double *u, *v, *w;      /* velocities, required */
    double *ut, *vt, *wt;         /* outputs; a NULL output skips that field */
    int32_t nscalar;              /* 0..F2C_MAX_SCALARS passive scalars */
    int32_t mode;                 /* f2c_output_mode */
    double dt;                    /* used by F2C_ADVANCE */
    const double *s[F2C_MAX_SCALARS];
    double *st[F2C_MAX_SCALARS];
} f2c_fields_v1;

uint32_t f2c_advection_abi_version(void);
/* Last error text of this thread (never NULL). */
const char *f2c_last_error(void);

/* Tendencies (or Euler-advanced fields) of U, V, W and the scalars on the
 * interior, in one fused z-marching launch. Bit-identical to the oracle's
 * per-point expressions (built with --fmad=false). Ghost layers of outputs are
 * not written, except in F2C_ADVANCE_FILLED mode. */
int f2c_advection_v1(const f2c_grid_v1 *grid, const f2c_fields_v1 *fields, void *stream);

/* The same computation by a chosen kernel:
 *   F2C_KERNEL_FACES (0): the face-sharing kernel that f2c_advection_v1 runs;
 *   F2C_KERNEL_DIRECT (1): a direct per-point kernel kept as a cross-check;
 *   both are bit-identical to the oracle (the reference's strict contract,
 *   compiler/emission/numerical_contract.py:13-15);
 *   F2C_KERNEL_FAST (2): the fast-fp kernel, the counterpart of the
 *   reference's --fast-fp build (compiler/resident/build.py:22): FMA
 *   contraction and an algebraically regrouped form of the same tendencies
 *   (about 80 FP64 operations per point for U, V, W and three scalars, against
 *   126). Results differ from the oracle by rounding only: every field within
 *   1e-12 of its maximum magnitude (measured ~1e-15). In F2C_ADVANCE mode the
 *   time step is folded into the coefficients. */
enum f2c_kernel_variant { F2C_KERNEL_FACES = 0, F2C_KERNEL_DIRECT = 1, F2C_KERNEL_FAST = 2 };
int f2c_advection_variant_v1(const f2c_grid_v1 *grid, const f2c_fields_v1 *fields, int variant, void *stream);

/* One reference procedure as one launch (the reference resident build's
 * structure: benchmarks/cdu/src/cdu.f90:12-106, cvd.f90/cdw.f90:44-98):
 * op 0 set (out = value), 1 multiply (out *= value), 2 CDUdiv, 3 CDUadv,
 * 4 CDVdiv, 5 CDVadv, 6 CDWdiv, 7 CDWadv. The sequence set, div, adv,
 * multiply(0.5) equals the fused launch bit for bit. */
int f2c_procedure_v1(int op, const f2c_grid_v1 *grid, double *out, const double *u, const double *v, const double *w,
                     double value, void *stream);

/* Boundary fill of `count` fields: periodic in x and y; vertical walls by
 * kind: 0 mirrors the interior (U, V, scalars), 1 is a face-staggered W with
 * zero wall faces and sign-changed mirrors. Requires nz >= halo. One launch. */
int f2c_halo_fill_v1(const f2c_grid_v1 *grid, double *const *fields, const int32_t *kinds, int32_t count,
                     void *stream);

#ifdef __cplusplus
}
#endif
#endif
