/* Numerical entries of the GB300 resident advection build (generated by compiler/emission).
 *
 * Each replaces the entry the reference compiler generates for the named
 * procedure (compiler/emission/cuda/scoped.py:237-553): same argument order
 * (context, mode, array handles in declaration order, scalars by reference),
 * same statuses (scoped_runtime.h). FORT_SCOPE_NATIVE mode, device resources
 * unavailable before any work, or arrays of differing shapes return
 * FORT_SCOPE_DECLINED with nothing done: the caller runs its original statements.
 */
#ifndef FORT_SHARED_ENTRIES_H
#define FORT_SHARED_ENTRIES_H
#include "scoped_runtime.h"
#ifdef __cplusplus
extern "C" {
#endif

/* momentumadvection::set -- replaces benchmarks/cdu/src/cdu.f90:12-27 */
int cpp_fort_shared_ce4761579065(fort_scope_t fort_context, int fort_mode, fort_buffer_t arr_handle, const double *val, const int *unx, const int *uny, const int *unz);
/* momentumadvection::multiply -- replaces benchmarks/cdu/src/cdu.f90:30-45 */
int cpp_fort_shared_79b994dd0404(fort_scope_t fort_context, int fort_mode, fort_buffer_t arr_handle, const double *val, const int *unx, const int *uny, const int *unz);
/* momentumadvection::cdudiv -- replaces benchmarks/cdu/src/cdu.f90:48-76 */
int cpp_fort_shared_c332ebf80d68(fort_scope_t fort_context, int fort_mode, fort_buffer_t u2_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, const double *dxmin, const double *dymin, const double *dzmin, const int *unx, const int *uny, const int *unz);
/* momentumadvection::cduadv -- replaces benchmarks/cdu/src/cdu.f90:79-106 */
int cpp_fort_shared_ae1df5b16148(fort_scope_t fort_context, int fort_mode, fort_buffer_t u2_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, const double *dxmin, const double *dymin, const double *dzmin, const int *unx, const int *uny, const int *unz);
/* momentumadvection::cdu -- replaces benchmarks/cdu/src/cdu.f90:113-133; set, div, adv and multiply by one half fused into one face-sharing launch */
int cpp_fort_shared_42de9862e2fe(fort_scope_t fort_context, int fort_mode, fort_buffer_t u2_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, const double *dxmin, const double *dymin, const double *dzmin, const int *unx, const int *uny, const int *unz);
/* momentumadvection::cdvdiv -- replaces compiler/tests/fixtures/stencils/cvd.f90:44-70 */
int cpp_fort_shared_dc5f61a1cb0a(fort_scope_t fort_context, int fort_mode, fort_buffer_t v2_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, const double *dxmin, const double *dymin, const double *dzmin, const int *vnx, const int *vny, const int *vnz);
/* momentumadvection::cdvadv -- replaces compiler/tests/fixtures/stencils/cvd.f90:73-98 */
int cpp_fort_shared_4091fbf13dda(fort_scope_t fort_context, int fort_mode, fort_buffer_t v2_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, const double *dxmin, const double *dymin, const double *dzmin, const int *vnx, const int *vny, const int *vnz);
/* momentumadvection::cdv -- replaces compiler/tests/fixtures/stencils/cvd.f90:105-125; set, div, adv and multiply by one half fused into one face-sharing launch */
int cpp_fort_shared_a72cc49a3bc2(fort_scope_t fort_context, int fort_mode, fort_buffer_t v2_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, const double *dxmin, const double *dymin, const double *dzmin, const int *vnx, const int *vny, const int *vnz);
/* momentumadvection::cdwdiv -- replaces compiler/tests/fixtures/stencils/cdw.f90:44-70 */
int cpp_fort_shared_1664ef72e5f6(fort_scope_t fort_context, int fort_mode, fort_buffer_t w2_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, const double *dxmin, const double *dymin, const double *dzmin, const int *wnx, const int *wny, const int *wnz);
/* momentumadvection::cdwadv -- replaces compiler/tests/fixtures/stencils/cdw.f90:73-98 */
int cpp_fort_shared_93e5f62400e4(fort_scope_t fort_context, int fort_mode, fort_buffer_t w2_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, const double *dxmin, const double *dymin, const double *dzmin, const int *wnx, const int *wny, const int *wnz);
/* momentumadvection::cdw -- replaces compiler/tests/fixtures/stencils/cdw.f90:105-125; set, div, adv and multiply by one half fused into one face-sharing launch */
int cpp_fort_shared_a28440d2f301(fort_scope_t fort_context, int fort_mode, fort_buffer_t w2_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, const double *dxmin, const double *dymin, const double *dzmin, const int *wnx, const int *wny, const int *wnz);
/* advection::step0 -- replaces benchmarks/cdu/src/cdu.f90:113-133 with cvd.f90/cdw.f90:105-125 and 0 passive scalars; U, V, W tendencies (CDU, CDV, CDW) and scalar tendencies in one launch */
int cpp_fort_shared_0e71295b0ec3(fort_scope_t fort_context, int fort_mode, fort_buffer_t u2_handle, fort_buffer_t v2_handle, fort_buffer_t w2_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, const double *dx, const double *dy, const double *dz, const int *nx, const int *ny, const int *nz, const int *halo);
/* advection::advance0 -- replaces forward-Euler update of the tendencies of advection::step; out = in + dt * tendency, double-buffered */
int cpp_fort_shared_001e6a9fcfd6(fort_scope_t fort_context, int fort_mode, fort_buffer_t un_handle, fort_buffer_t vn_handle, fort_buffer_t wn_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, const double *dx, const double *dy, const double *dz, const double *dt, const int *nx, const int *ny, const int *nz, const int *halo);
/* advection::halo0 -- replaces periodic x/y boundary fill in the order of compiler/tests/apps/box/boundaries.f90:6-41; walls in z (W zero, mirrored) */
int cpp_fort_shared_4d5ee7974150(fort_scope_t fort_context, int fort_mode, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, const int *nx, const int *ny, const int *nz, const int *halo);
/* advection::step1 -- replaces benchmarks/cdu/src/cdu.f90:113-133 with cvd.f90/cdw.f90:105-125 and 1 passive scalars; U, V, W tendencies (CDU, CDV, CDW) and scalar tendencies in one launch */
int cpp_fort_shared_a5b15bb8130a(fort_scope_t fort_context, int fort_mode, fort_buffer_t u2_handle, fort_buffer_t v2_handle, fort_buffer_t w2_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, fort_buffer_t s1_handle, fort_buffer_t s1t_handle, const double *dx, const double *dy, const double *dz, const int *nx, const int *ny, const int *nz, const int *halo);
/* advection::advance1 -- replaces forward-Euler update of the tendencies of advection::step; out = in + dt * tendency, double-buffered */
int cpp_fort_shared_45d68b9decbb(fort_scope_t fort_context, int fort_mode, fort_buffer_t un_handle, fort_buffer_t vn_handle, fort_buffer_t wn_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, fort_buffer_t s1_handle, fort_buffer_t s1n_handle, const double *dx, const double *dy, const double *dz, const double *dt, const int *nx, const int *ny, const int *nz, const int *halo);
/* advection::halo1 -- replaces periodic x/y boundary fill in the order of compiler/tests/apps/box/boundaries.f90:6-41; walls in z (W zero, mirrored) */
int cpp_fort_shared_f5b3f004c0dc(fort_scope_t fort_context, int fort_mode, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, fort_buffer_t s1_handle, const int *nx, const int *ny, const int *nz, const int *halo);
/* advection::step2 -- replaces benchmarks/cdu/src/cdu.f90:113-133 with cvd.f90/cdw.f90:105-125 and 2 passive scalars; U, V, W tendencies (CDU, CDV, CDW) and scalar tendencies in one launch */
int cpp_fort_shared_cac08e022e8e(fort_scope_t fort_context, int fort_mode, fort_buffer_t u2_handle, fort_buffer_t v2_handle, fort_buffer_t w2_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, fort_buffer_t s1_handle, fort_buffer_t s2_handle, fort_buffer_t s1t_handle, fort_buffer_t s2t_handle, const double *dx, const double *dy, const double *dz, const int *nx, const int *ny, const int *nz, const int *halo);
/* advection::advance2 -- replaces forward-Euler update of the tendencies of advection::step; out = in + dt * tendency, double-buffered */
int cpp_fort_shared_405aeb9f9533(fort_scope_t fort_context, int fort_mode, fort_buffer_t un_handle, fort_buffer_t vn_handle, fort_buffer_t wn_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, fort_buffer_t s1_handle, fort_buffer_t s2_handle, fort_buffer_t s1n_handle, fort_buffer_t s2n_handle, const double *dx, const double *dy, const double *dz, const double *dt, const int *nx, const int *ny, const int *nz, const int *halo);
/* advection::halo2 -- replaces periodic x/y boundary fill in the order of compiler/tests/apps/box/boundaries.f90:6-41; walls in z (W zero, mirrored) */
int cpp_fort_shared_9f0fa829d5ff(fort_scope_t fort_context, int fort_mode, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, fort_buffer_t s1_handle, fort_buffer_t s2_handle, const int *nx, const int *ny, const int *nz, const int *halo);
/* advection::step3 -- replaces benchmarks/cdu/src/cdu.f90:113-133 with cvd.f90/cdw.f90:105-125 and 3 passive scalars; U, V, W tendencies (CDU, CDV, CDW) and scalar tendencies in one launch */
int cpp_fort_shared_c3ee1d88b7ff(fort_scope_t fort_context, int fort_mode, fort_buffer_t u2_handle, fort_buffer_t v2_handle, fort_buffer_t w2_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, fort_buffer_t s1_handle, fort_buffer_t s2_handle, fort_buffer_t s3_handle, fort_buffer_t s1t_handle, fort_buffer_t s2t_handle, fort_buffer_t s3t_handle, const double *dx, const double *dy, const double *dz, const int *nx, const int *ny, const int *nz, const int *halo);
/* advection::advance3 -- replaces forward-Euler update of the tendencies of advection::step; out = in + dt * tendency, double-buffered */
int cpp_fort_shared_f6ba06adab12(fort_scope_t fort_context, int fort_mode, fort_buffer_t un_handle, fort_buffer_t vn_handle, fort_buffer_t wn_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, fort_buffer_t s1_handle, fort_buffer_t s2_handle, fort_buffer_t s3_handle, fort_buffer_t s1n_handle, fort_buffer_t s2n_handle, fort_buffer_t s3n_handle, const double *dx, const double *dy, const double *dz, const double *dt, const int *nx, const int *ny, const int *nz, const int *halo);
/* advection::halo3 -- replaces periodic x/y boundary fill in the order of compiler/tests/apps/box/boundaries.f90:6-41; walls in z (W zero, mirrored) */
int cpp_fort_shared_4effb4648a3e(fort_scope_t fort_context, int fort_mode, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, fort_buffer_t s1_handle, fort_buffer_t s2_handle, fort_buffer_t s3_handle, const int *nx, const int *ny, const int *nz, const int *halo);
/* advection::step4 -- replaces benchmarks/cdu/src/cdu.f90:113-133 with cvd.f90/cdw.f90:105-125 and 4 passive scalars; U, V, W tendencies (CDU, CDV, CDW) and scalar tendencies in one launch */
int cpp_fort_shared_6f06b55ba3fe(fort_scope_t fort_context, int fort_mode, fort_buffer_t u2_handle, fort_buffer_t v2_handle, fort_buffer_t w2_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, fort_buffer_t s1_handle, fort_buffer_t s2_handle, fort_buffer_t s3_handle, fort_buffer_t s4_handle, fort_buffer_t s1t_handle, fort_buffer_t s2t_handle, fort_buffer_t s3t_handle, fort_buffer_t s4t_handle, const double *dx, const double *dy, const double *dz, const int *nx, const int *ny, const int *nz, const int *halo);
/* advection::advance4 -- replaces forward-Euler update of the tendencies of advection::step; out = in + dt * tendency, double-buffered */
int cpp_fort_shared_cbf2341c8e18(fort_scope_t fort_context, int fort_mode, fort_buffer_t un_handle, fort_buffer_t vn_handle, fort_buffer_t wn_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, fort_buffer_t s1_handle, fort_buffer_t s2_handle, fort_buffer_t s3_handle, fort_buffer_t s4_handle, fort_buffer_t s1n_handle, fort_buffer_t s2n_handle, fort_buffer_t s3n_handle, fort_buffer_t s4n_handle, const double *dx, const double *dy, const double *dz, const double *dt, const int *nx, const int *ny, const int *nz, const int *halo);
/* advection::halo4 -- replaces periodic x/y boundary fill in the order of compiler/tests/apps/box/boundaries.f90:6-41; walls in z (W zero, mirrored) */
int cpp_fort_shared_073d04efb82a(fort_scope_t fort_context, int fort_mode, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, fort_buffer_t s1_handle, fort_buffer_t s2_handle, fort_buffer_t s3_handle, fort_buffer_t s4_handle, const int *nx, const int *ny, const int *nz, const int *halo);
/* stencil::diffuse7 -- replaces compiler/tests/apps/box/stepper.f90:8-30 (diffuse with laplacian) */
int cpp_fort_shared_e331fbb8bf9a(fort_scope_t fort_context, int fort_mode, fort_buffer_t b_handle, fort_buffer_t a_handle, const double *dt, const double *nu, const double *dx, const int *nx, const int *ny, const int *nz, const int *halo);
/* stencil::jacobi5 -- replaces compiler/tests/apps/relax/relax.f90:28-33 (one Jacobi sweep) */
int cpp_fort_shared_03470f69376f(fort_scope_t fort_context, int fort_mode, fort_buffer_t v_handle, fort_buffer_t u_handle, const int *nx, const int *ny, const int *halo);
/* stencil::yee2d -- replaces 2-D TM Yee leapfrog (no reference source in the mount); H task then E task */
int cpp_fort_shared_82041a3f2b68(fort_scope_t fort_context, int fort_mode, fort_buffer_t ez_handle, fort_buffer_t hx_handle, fort_buffer_t hy_handle, const double *ch, const double *ce, const int *nx, const int *ny, const int *halo);

#ifdef __cplusplus
}
#endif
#endif
