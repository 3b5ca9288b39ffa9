// Generated by compiler/emission from the template registry; regenerate, do not edit.
// Each entry packs its arguments for the hand-written template runner (entry_runner.cu).
#include "entry_runner.hpp"

using f2c::entries::EntryCall;
using f2c::entries::Template;
using f2c::entries::run_entry;

// momentumadvection::set: benchmarks/cdu/src/cdu.f90:12-27
extern "C" int cpp_fort_shared_ce4761579065(fort_scope_t fort_context, int fort_mode, fort_buffer_t arr_handle, const double *val, const int *unx, const int *uny, const int *unz) {
    EntryCall call{};
    call.context = fort_context;
    call.mode = fort_mode;
    call.kind = Template::Set;
    call.code_key = 0x67ba0ab43bfa5d52ULL;
    call.nscalar = 0;
    call.narrays = 1;
    call.arrays[0] = arr_handle;
    call.nreals = 1;
    call.reals[0] = val;
    call.nints = 3;
    call.ints[0] = unx;
    call.ints[1] = uny;
    call.ints[2] = unz;
    return run_entry(call);
}

// momentumadvection::multiply: benchmarks/cdu/src/cdu.f90:30-45
extern "C" int cpp_fort_shared_79b994dd0404(fort_scope_t fort_context, int fort_mode, fort_buffer_t arr_handle, const double *val, const int *unx, const int *uny, const int *unz) {
    EntryCall call{};
    call.context = fort_context;
    call.mode = fort_mode;
    call.kind = Template::Multiply;
    call.code_key = 0x7dfbafef47878ca8ULL;
    call.nscalar = 0;
    call.narrays = 1;
    call.arrays[0] = arr_handle;
    call.nreals = 1;
    call.reals[0] = val;
    call.nints = 3;
    call.ints[0] = unx;
    call.ints[1] = uny;
    call.ints[2] = unz;
    return run_entry(call);
}

// momentumadvection::cdudiv: benchmarks/cdu/src/cdu.f90:48-76
extern "C" int cpp_fort_shared_c332ebf80d68(fort_scope_t fort_context, int fort_mode, fort_buffer_t u2_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, const double *dxmin, const double *dymin, const double *dzmin, const int *unx, const int *uny, const int *unz) {
    EntryCall call{};
    call.context = fort_context;
    call.mode = fort_mode;
    call.kind = Template::CduDiv;
    call.code_key = 0x2cb36d86612b18d3ULL;
    call.nscalar = 0;
    call.narrays = 4;
    call.arrays[0] = u2_handle;
    call.arrays[1] = u_handle;
    call.arrays[2] = v_handle;
    call.arrays[3] = w_handle;
    call.nreals = 3;
    call.reals[0] = dxmin;
    call.reals[1] = dymin;
    call.reals[2] = dzmin;
    call.nints = 3;
    call.ints[0] = unx;
    call.ints[1] = uny;
    call.ints[2] = unz;
    return run_entry(call);
}

// momentumadvection::cduadv: benchmarks/cdu/src/cdu.f90:79-106
extern "C" int cpp_fort_shared_ae1df5b16148(fort_scope_t fort_context, int fort_mode, fort_buffer_t u2_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, const double *dxmin, const double *dymin, const double *dzmin, const int *unx, const int *uny, const int *unz) {
    EntryCall call{};
    call.context = fort_context;
    call.mode = fort_mode;
    call.kind = Template::CduAdv;
    call.code_key = 0x7b94725bb007700eULL;
    call.nscalar = 0;
    call.narrays = 4;
    call.arrays[0] = u2_handle;
    call.arrays[1] = u_handle;
    call.arrays[2] = v_handle;
    call.arrays[3] = w_handle;
    call.nreals = 3;
    call.reals[0] = dxmin;
    call.reals[1] = dymin;
    call.reals[2] = dzmin;
    call.nints = 3;
    call.ints[0] = unx;
    call.ints[1] = uny;
    call.ints[2] = unz;
    return run_entry(call);
}

// momentumadvection::cdu: benchmarks/cdu/src/cdu.f90:113-133
extern "C" int cpp_fort_shared_42de9862e2fe(fort_scope_t fort_context, int fort_mode, fort_buffer_t u2_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, const double *dxmin, const double *dymin, const double *dzmin, const int *unx, const int *uny, const int *unz) {
    EntryCall call{};
    call.context = fort_context;
    call.mode = fort_mode;
    call.kind = Template::Cdu;
    call.code_key = 0x6770cb44204d3160ULL;
    call.nscalar = 0;
    call.narrays = 4;
    call.arrays[0] = u2_handle;
    call.arrays[1] = u_handle;
    call.arrays[2] = v_handle;
    call.arrays[3] = w_handle;
    call.nreals = 3;
    call.reals[0] = dxmin;
    call.reals[1] = dymin;
    call.reals[2] = dzmin;
    call.nints = 3;
    call.ints[0] = unx;
    call.ints[1] = uny;
    call.ints[2] = unz;
    return run_entry(call);
}

// momentumadvection::cdvdiv: compiler/tests/fixtures/stencils/cvd.f90:44-70
extern "C" int cpp_fort_shared_dc5f61a1cb0a(fort_scope_t fort_context, int fort_mode, fort_buffer_t v2_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, const double *dxmin, const double *dymin, const double *dzmin, const int *vnx, const int *vny, const int *vnz) {
    EntryCall call{};
    call.context = fort_context;
    call.mode = fort_mode;
    call.kind = Template::CdvDiv;
    call.code_key = 0xe73982a121a22c21ULL;
    call.nscalar = 0;
    call.narrays = 4;
    call.arrays[0] = v2_handle;
    call.arrays[1] = u_handle;
    call.arrays[2] = v_handle;
    call.arrays[3] = w_handle;
    call.nreals = 3;
    call.reals[0] = dxmin;
    call.reals[1] = dymin;
    call.reals[2] = dzmin;
    call.nints = 3;
    call.ints[0] = vnx;
    call.ints[1] = vny;
    call.ints[2] = vnz;
    return run_entry(call);
}

// momentumadvection::cdvadv: compiler/tests/fixtures/stencils/cvd.f90:73-98
extern "C" int cpp_fort_shared_4091fbf13dda(fort_scope_t fort_context, int fort_mode, fort_buffer_t v2_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, const double *dxmin, const double *dymin, const double *dzmin, const int *vnx, const int *vny, const int *vnz) {
    EntryCall call{};
    call.context = fort_context;
    call.mode = fort_mode;
    call.kind = Template::CdvAdv;
    call.code_key = 0x774b370f65435846ULL;
    call.nscalar = 0;
    call.narrays = 4;
    call.arrays[0] = v2_handle;
    call.arrays[1] = u_handle;
    call.arrays[2] = v_handle;
    call.arrays[3] = w_handle;
    call.nreals = 3;
    call.reals[0] = dxmin;
    call.reals[1] = dymin;
    call.reals[2] = dzmin;
    call.nints = 3;
    call.ints[0] = vnx;
    call.ints[1] = vny;
    call.ints[2] = vnz;
    return run_entry(call);
}

// momentumadvection::cdv: compiler/tests/fixtures/stencils/cvd.f90:105-125
extern "C" int cpp_fort_shared_a72cc49a3bc2(fort_scope_t fort_context, int fort_mode, fort_buffer_t v2_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, const double *dxmin, const double *dymin, const double *dzmin, const int *vnx, const int *vny, const int *vnz) {
    EntryCall call{};
    call.context = fort_context;
    call.mode = fort_mode;
    call.kind = Template::Cdv;
    call.code_key = 0xdda7bc2970171d65ULL;
    call.nscalar = 0;
    call.narrays = 4;
    call.arrays[0] = v2_handle;
    call.arrays[1] = u_handle;
    call.arrays[2] = v_handle;
    call.arrays[3] = w_handle;
    call.nreals = 3;
    call.reals[0] = dxmin;
    call.reals[1] = dymin;
    call.reals[2] = dzmin;
    call.nints = 3;
    call.ints[0] = vnx;
    call.ints[1] = vny;
    call.ints[2] = vnz;
    return run_entry(call);
}

// momentumadvection::cdwdiv: compiler/tests/fixtures/stencils/cdw.f90:44-70
extern "C" int cpp_fort_shared_1664ef72e5f6(fort_scope_t fort_context, int fort_mode, fort_buffer_t w2_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, const double *dxmin, const double *dymin, const double *dzmin, const int *wnx, const int *wny, const int *wnz) {
    EntryCall call{};
    call.context = fort_context;
    call.mode = fort_mode;
    call.kind = Template::CdwDiv;
    call.code_key = 0xb28e529765f39e11ULL;
    call.nscalar = 0;
    call.narrays = 4;
    call.arrays[0] = w2_handle;
    call.arrays[1] = u_handle;
    call.arrays[2] = v_handle;
    call.arrays[3] = w_handle;
    call.nreals = 3;
    call.reals[0] = dxmin;
    call.reals[1] = dymin;
    call.reals[2] = dzmin;
    call.nints = 3;
    call.ints[0] = wnx;
    call.ints[1] = wny;
    call.ints[2] = wnz;
    return run_entry(call);
}

// momentumadvection::cdwadv: compiler/tests/fixtures/stencils/cdw.f90:73-98
extern "C" int cpp_fort_shared_93e5f62400e4(fort_scope_t fort_context, int fort_mode, fort_buffer_t w2_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, const double *dxmin, const double *dymin, const double *dzmin, const int *wnx, const int *wny, const int *wnz) {
    EntryCall call{};
    call.context = fort_context;
    call.mode = fort_mode;
    call.kind = Template::CdwAdv;
    call.code_key = 0xee73731b03f368feULL;
    call.nscalar = 0;
    call.narrays = 4;
    call.arrays[0] = w2_handle;
    call.arrays[1] = u_handle;
    call.arrays[2] = v_handle;
    call.arrays[3] = w_handle;
    call.nreals = 3;
    call.reals[0] = dxmin;
    call.reals[1] = dymin;
    call.reals[2] = dzmin;
    call.nints = 3;
    call.ints[0] = wnx;
    call.ints[1] = wny;
    call.ints[2] = wnz;
    return run_entry(call);
}

// momentumadvection::cdw: compiler/tests/fixtures/stencils/cdw.f90:105-125
extern "C" int cpp_fort_shared_a28440d2f301(fort_scope_t fort_context, int fort_mode, fort_buffer_t w2_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, const double *dxmin, const double *dymin, const double *dzmin, const int *wnx, const int *wny, const int *wnz) {
    EntryCall call{};
    call.context = fort_context;
    call.mode = fort_mode;
    call.kind = Template::Cdw;
    call.code_key = 0xc4edae85039bc18bULL;
    call.nscalar = 0;
    call.narrays = 4;
    call.arrays[0] = w2_handle;
    call.arrays[1] = u_handle;
    call.arrays[2] = v_handle;
    call.arrays[3] = w_handle;
    call.nreals = 3;
    call.reals[0] = dxmin;
    call.reals[1] = dymin;
    call.reals[2] = dzmin;
    call.nints = 3;
    call.ints[0] = wnx;
    call.ints[1] = wny;
    call.ints[2] = wnz;
    return run_entry(call);
}

// advection::step0: benchmarks/cdu/src/cdu.f90:113-133 with cvd.f90/cdw.f90:105-125 and 0 passive scalars
extern "C" int cpp_fort_shared_0e71295b0ec3(fort_scope_t fort_context, int fort_mode, fort_buffer_t u2_handle, fort_buffer_t v2_handle, fort_buffer_t w2_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, const double *dx, const double *dy, const double *dz, const int *nx, const int *ny, const int *nz, const int *halo) {
    EntryCall call{};
    call.context = fort_context;
    call.mode = fort_mode;
    call.kind = Template::Step;
    call.code_key = 0xc6d87e2a783d55deULL;
    call.nscalar = 0;
    call.narrays = 6;
    call.arrays[0] = u2_handle;
    call.arrays[1] = v2_handle;
    call.arrays[2] = w2_handle;
    call.arrays[3] = u_handle;
    call.arrays[4] = v_handle;
    call.arrays[5] = w_handle;
    call.nreals = 3;
    call.reals[0] = dx;
    call.reals[1] = dy;
    call.reals[2] = dz;
    call.nints = 4;
    call.ints[0] = nx;
    call.ints[1] = ny;
    call.ints[2] = nz;
    call.ints[3] = halo;
    return run_entry(call);
}

// advection::advance0: forward-Euler update of the tendencies of advection::step
extern "C" int cpp_fort_shared_001e6a9fcfd6(fort_scope_t fort_context, int fort_mode, fort_buffer_t un_handle, fort_buffer_t vn_handle, fort_buffer_t wn_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, const double *dx, const double *dy, const double *dz, const double *dt, const int *nx, const int *ny, const int *nz, const int *halo) {
    EntryCall call{};
    call.context = fort_context;
    call.mode = fort_mode;
    call.kind = Template::StepAdvance;
    call.code_key = 0x733645de1ca3f4a0ULL;
    call.nscalar = 0;
    call.narrays = 6;
    call.arrays[0] = un_handle;
    call.arrays[1] = vn_handle;
    call.arrays[2] = wn_handle;
    call.arrays[3] = u_handle;
    call.arrays[4] = v_handle;
    call.arrays[5] = w_handle;
    call.nreals = 4;
    call.reals[0] = dx;
    call.reals[1] = dy;
    call.reals[2] = dz;
    call.reals[3] = dt;
    call.nints = 4;
    call.ints[0] = nx;
    call.ints[1] = ny;
    call.ints[2] = nz;
    call.ints[3] = halo;
    return run_entry(call);
}

// advection::halo0: periodic x/y boundary fill in the order of compiler/tests/apps/box/boundaries.f90:6-41; walls in z (W zero, mirrored)
extern "C" int cpp_fort_shared_4d5ee7974150(fort_scope_t fort_context, int fort_mode, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, const int *nx, const int *ny, const int *nz, const int *halo) {
    EntryCall call{};
    call.context = fort_context;
    call.mode = fort_mode;
    call.kind = Template::Halo;
    call.code_key = 0x98c26d96a02517a2ULL;
    call.nscalar = 0;
    call.narrays = 3;
    call.arrays[0] = u_handle;
    call.arrays[1] = v_handle;
    call.arrays[2] = w_handle;
    call.nreals = 0;
    call.nints = 4;
    call.ints[0] = nx;
    call.ints[1] = ny;
    call.ints[2] = nz;
    call.ints[3] = halo;
    return run_entry(call);
}

// advection::step1: benchmarks/cdu/src/cdu.f90:113-133 with cvd.f90/cdw.f90:105-125 and 1 passive scalars
extern "C" int cpp_fort_shared_a5b15bb8130a(fort_scope_t fort_context, int fort_mode, fort_buffer_t u2_handle, fort_buffer_t v2_handle, fort_buffer_t w2_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, fort_buffer_t s1_handle, fort_buffer_t s1t_handle, const double *dx, const double *dy, const double *dz, const int *nx, const int *ny, const int *nz, const int *halo) {
    EntryCall call{};
    call.context = fort_context;
    call.mode = fort_mode;
    call.kind = Template::Step;
    call.code_key = 0x2d994d1417c3c97aULL;
    call.nscalar = 1;
    call.narrays = 8;
    call.arrays[0] = u2_handle;
    call.arrays[1] = v2_handle;
    call.arrays[2] = w2_handle;
    call.arrays[3] = u_handle;
    call.arrays[4] = v_handle;
    call.arrays[5] = w_handle;
    call.arrays[6] = s1_handle;
    call.arrays[7] = s1t_handle;
    call.nreals = 3;
    call.reals[0] = dx;
    call.reals[1] = dy;
    call.reals[2] = dz;
    call.nints = 4;
    call.ints[0] = nx;
    call.ints[1] = ny;
    call.ints[2] = nz;
    call.ints[3] = halo;
    return run_entry(call);
}

// advection::advance1: forward-Euler update of the tendencies of advection::step
extern "C" int cpp_fort_shared_45d68b9decbb(fort_scope_t fort_context, int fort_mode, fort_buffer_t un_handle, fort_buffer_t vn_handle, fort_buffer_t wn_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, fort_buffer_t s1_handle, fort_buffer_t s1n_handle, const double *dx, const double *dy, const double *dz, const double *dt, const int *nx, const int *ny, const int *nz, const int *halo) {
    EntryCall call{};
    call.context = fort_context;
    call.mode = fort_mode;
    call.kind = Template::StepAdvance;
    call.code_key = 0x9c0a79ff58fe12b0ULL;
    call.nscalar = 1;
    call.narrays = 8;
    call.arrays[0] = un_handle;
    call.arrays[1] = vn_handle;
    call.arrays[2] = wn_handle;
    call.arrays[3] = u_handle;
    call.arrays[4] = v_handle;
    call.arrays[5] = w_handle;
    call.arrays[6] = s1_handle;
    call.arrays[7] = s1n_handle;
    call.nreals = 4;
    call.reals[0] = dx;
    call.reals[1] = dy;
    call.reals[2] = dz;
    call.reals[3] = dt;
    call.nints = 4;
    call.ints[0] = nx;
    call.ints[1] = ny;
    call.ints[2] = nz;
    call.ints[3] = halo;
    return run_entry(call);
}

// advection::halo1: periodic x/y boundary fill in the order of compiler/tests/apps/box/boundaries.f90:6-41; walls in z (W zero, mirrored)
extern "C" int cpp_fort_shared_f5b3f004c0dc(fort_scope_t fort_context, int fort_mode, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, fort_buffer_t s1_handle, const int *nx, const int *ny, const int *nz, const int *halo) {
    EntryCall call{};
    call.context = fort_context;
    call.mode = fort_mode;
    call.kind = Template::Halo;
    call.code_key = 0x6aa1bc2f2f106846ULL;
    call.nscalar = 1;
    call.narrays = 4;
    call.arrays[0] = u_handle;
    call.arrays[1] = v_handle;
    call.arrays[2] = w_handle;
    call.arrays[3] = s1_handle;
    call.nreals = 0;
    call.nints = 4;
    call.ints[0] = nx;
    call.ints[1] = ny;
    call.ints[2] = nz;
    call.ints[3] = halo;
    return run_entry(call);
}

// advection::step2: benchmarks/cdu/src/cdu.f90:113-133 with cvd.f90/cdw.f90:105-125 and 2 passive scalars
extern "C" int cpp_fort_shared_cac08e022e8e(fort_scope_t fort_context, int fort_mode, fort_buffer_t u2_handle, fort_buffer_t v2_handle, fort_buffer_t w2_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, fort_buffer_t s1_handle, fort_buffer_t s2_handle, fort_buffer_t s1t_handle, fort_buffer_t s2t_handle, const double *dx, const double *dy, const double *dz, const int *nx, const int *ny, const int *nz, const int *halo) {
    EntryCall call{};
    call.context = fort_context;
    call.mode = fort_mode;
    call.kind = Template::Step;
    call.code_key = 0x5ed2d206e57f3772ULL;
    call.nscalar = 2;
    call.narrays = 10;
    call.arrays[0] = u2_handle;
    call.arrays[1] = v2_handle;
    call.arrays[2] = w2_handle;
    call.arrays[3] = u_handle;
    call.arrays[4] = v_handle;
    call.arrays[5] = w_handle;
    call.arrays[6] = s1_handle;
    call.arrays[7] = s2_handle;
    call.arrays[8] = s1t_handle;
    call.arrays[9] = s2t_handle;
    call.nreals = 3;
    call.reals[0] = dx;
    call.reals[1] = dy;
    call.reals[2] = dz;
    call.nints = 4;
    call.ints[0] = nx;
    call.ints[1] = ny;
    call.ints[2] = nz;
    call.ints[3] = halo;
    return run_entry(call);
}

// advection::advance2: forward-Euler update of the tendencies of advection::step
extern "C" int cpp_fort_shared_405aeb9f9533(fort_scope_t fort_context, int fort_mode, fort_buffer_t un_handle, fort_buffer_t vn_handle, fort_buffer_t wn_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, fort_buffer_t s1_handle, fort_buffer_t s2_handle, fort_buffer_t s1n_handle, fort_buffer_t s2n_handle, const double *dx, const double *dy, const double *dz, const double *dt, const int *nx, const int *ny, const int *nz, const int *halo) {
    EntryCall call{};
    call.context = fort_context;
    call.mode = fort_mode;
    call.kind = Template::StepAdvance;
    call.code_key = 0x064e76a5daadffdbULL;
    call.nscalar = 2;
    call.narrays = 10;
    call.arrays[0] = un_handle;
    call.arrays[1] = vn_handle;
    call.arrays[2] = wn_handle;
    call.arrays[3] = u_handle;
    call.arrays[4] = v_handle;
    call.arrays[5] = w_handle;
    call.arrays[6] = s1_handle;
    call.arrays[7] = s2_handle;
    call.arrays[8] = s1n_handle;
    call.arrays[9] = s2n_handle;
    call.nreals = 4;
    call.reals[0] = dx;
    call.reals[1] = dy;
    call.reals[2] = dz;
    call.reals[3] = dt;
    call.nints = 4;
    call.ints[0] = nx;
    call.ints[1] = ny;
    call.ints[2] = nz;
    call.ints[3] = halo;
    return run_entry(call);
}

// advection::halo2: periodic x/y boundary fill in the order of compiler/tests/apps/box/boundaries.f90:6-41; walls in z (W zero, mirrored)
extern "C" int cpp_fort_shared_9f0fa829d5ff(fort_scope_t fort_context, int fort_mode, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, fort_buffer_t s1_handle, fort_buffer_t s2_handle, const int *nx, const int *ny, const int *nz, const int *halo) {
    EntryCall call{};
    call.context = fort_context;
    call.mode = fort_mode;
    call.kind = Template::Halo;
    call.code_key = 0x0153fb09bd998bb5ULL;
    call.nscalar = 2;
    call.narrays = 5;
    call.arrays[0] = u_handle;
    call.arrays[1] = v_handle;
    call.arrays[2] = w_handle;
    call.arrays[3] = s1_handle;
    call.arrays[4] = s2_handle;
    call.nreals = 0;
    call.nints = 4;
    call.ints[0] = nx;
    call.ints[1] = ny;
    call.ints[2] = nz;
    call.ints[3] = halo;
    return run_entry(call);
}

// advection::step3: benchmarks/cdu/src/cdu.f90:113-133 with cvd.f90/cdw.f90:105-125 and 3 passive scalars
extern "C" int cpp_fort_shared_c3ee1d88b7ff(fort_scope_t fort_context, int fort_mode, fort_buffer_t u2_handle, fort_buffer_t v2_handle, fort_buffer_t w2_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, fort_buffer_t s1_handle, fort_buffer_t s2_handle, fort_buffer_t s3_handle, fort_buffer_t s1t_handle, fort_buffer_t s2t_handle, fort_buffer_t s3t_handle, const double *dx, const double *dy, const double *dz, const int *nx, const int *ny, const int *nz, const int *halo) {
    EntryCall call{};
    call.context = fort_context;
    call.mode = fort_mode;
    call.kind = Template::Step;
    call.code_key = 0xc5776f38669a6a23ULL;
    call.nscalar = 3;
    call.narrays = 12;
    call.arrays[0] = u2_handle;
    call.arrays[1] = v2_handle;
    call.arrays[2] = w2_handle;
    call.arrays[3] = u_handle;
    call.arrays[4] = v_handle;
    call.arrays[5] = w_handle;
    call.arrays[6] = s1_handle;
    call.arrays[7] = s2_handle;
    call.arrays[8] = s3_handle;
    call.arrays[9] = s1t_handle;
    call.arrays[10] = s2t_handle;
    call.arrays[11] = s3t_handle;
    call.nreals = 3;
    call.reals[0] = dx;
    call.reals[1] = dy;
    call.reals[2] = dz;
    call.nints = 4;
    call.ints[0] = nx;
    call.ints[1] = ny;
    call.ints[2] = nz;
    call.ints[3] = halo;
    return run_entry(call);
}

// advection::advance3: forward-Euler update of the tendencies of advection::step
extern "C" int cpp_fort_shared_f6ba06adab12(fort_scope_t fort_context, int fort_mode, fort_buffer_t un_handle, fort_buffer_t vn_handle, fort_buffer_t wn_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, fort_buffer_t s1_handle, fort_buffer_t s2_handle, fort_buffer_t s3_handle, fort_buffer_t s1n_handle, fort_buffer_t s2n_handle, fort_buffer_t s3n_handle, const double *dx, const double *dy, const double *dz, const double *dt, const int *nx, const int *ny, const int *nz, const int *halo) {
    EntryCall call{};
    call.context = fort_context;
    call.mode = fort_mode;
    call.kind = Template::StepAdvance;
    call.code_key = 0xd5565f8b1e7bcda1ULL;
    call.nscalar = 3;
    call.narrays = 12;
    call.arrays[0] = un_handle;
    call.arrays[1] = vn_handle;
    call.arrays[2] = wn_handle;
    call.arrays[3] = u_handle;
    call.arrays[4] = v_handle;
    call.arrays[5] = w_handle;
    call.arrays[6] = s1_handle;
    call.arrays[7] = s2_handle;
    call.arrays[8] = s3_handle;
    call.arrays[9] = s1n_handle;
    call.arrays[10] = s2n_handle;
    call.arrays[11] = s3n_handle;
    call.nreals = 4;
    call.reals[0] = dx;
    call.reals[1] = dy;
    call.reals[2] = dz;
    call.reals[3] = dt;
    call.nints = 4;
    call.ints[0] = nx;
    call.ints[1] = ny;
    call.ints[2] = nz;
    call.ints[3] = halo;
    return run_entry(call);
}

// advection::halo3: periodic x/y boundary fill in the order of compiler/tests/apps/box/boundaries.f90:6-41; walls in z (W zero, mirrored)
extern "C" int cpp_fort_shared_4effb4648a3e(fort_scope_t fort_context, int fort_mode, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, fort_buffer_t s1_handle, fort_buffer_t s2_handle, fort_buffer_t s3_handle, const int *nx, const int *ny, const int *nz, const int *halo) {
    EntryCall call{};
    call.context = fort_context;
    call.mode = fort_mode;
    call.kind = Template::Halo;
    call.code_key = 0x32e732f5b4d223aaULL;
    call.nscalar = 3;
    call.narrays = 6;
    call.arrays[0] = u_handle;
    call.arrays[1] = v_handle;
    call.arrays[2] = w_handle;
    call.arrays[3] = s1_handle;
    call.arrays[4] = s2_handle;
    call.arrays[5] = s3_handle;
    call.nreals = 0;
    call.nints = 4;
    call.ints[0] = nx;
    call.ints[1] = ny;
    call.ints[2] = nz;
    call.ints[3] = halo;
    return run_entry(call);
}

// advection::step4: benchmarks/cdu/src/cdu.f90:113-133 with cvd.f90/cdw.f90:105-125 and 4 passive scalars
extern "C" int cpp_fort_shared_6f06b55ba3fe(fort_scope_t fort_context, int fort_mode, fort_buffer_t u2_handle, fort_buffer_t v2_handle, fort_buffer_t w2_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, fort_buffer_t s1_handle, fort_buffer_t s2_handle, fort_buffer_t s3_handle, fort_buffer_t s4_handle, fort_buffer_t s1t_handle, fort_buffer_t s2t_handle, fort_buffer_t s3t_handle, fort_buffer_t s4t_handle, const double *dx, const double *dy, const double *dz, const int *nx, const int *ny, const int *nz, const int *halo) {
    EntryCall call{};
    call.context = fort_context;
    call.mode = fort_mode;
    call.kind = Template::Step;
    call.code_key = 0x3a23f411b401be15ULL;
    call.nscalar = 4;
    call.narrays = 14;
    call.arrays[0] = u2_handle;
    call.arrays[1] = v2_handle;
    call.arrays[2] = w2_handle;
    call.arrays[3] = u_handle;
    call.arrays[4] = v_handle;
    call.arrays[5] = w_handle;
    call.arrays[6] = s1_handle;
    call.arrays[7] = s2_handle;
    call.arrays[8] = s3_handle;
    call.arrays[9] = s4_handle;
    call.arrays[10] = s1t_handle;
    call.arrays[11] = s2t_handle;
    call.arrays[12] = s3t_handle;
    call.arrays[13] = s4t_handle;
    call.nreals = 3;
    call.reals[0] = dx;
    call.reals[1] = dy;
    call.reals[2] = dz;
    call.nints = 4;
    call.ints[0] = nx;
    call.ints[1] = ny;
    call.ints[2] = nz;
    call.ints[3] = halo;
    return run_entry(call);
}

// advection::advance4: forward-Euler update of the tendencies of advection::step
extern "C" int cpp_fort_shared_cbf2341c8e18(fort_scope_t fort_context, int fort_mode, fort_buffer_t un_handle, fort_buffer_t vn_handle, fort_buffer_t wn_handle, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, fort_buffer_t s1_handle, fort_buffer_t s2_handle, fort_buffer_t s3_handle, fort_buffer_t s4_handle, fort_buffer_t s1n_handle, fort_buffer_t s2n_handle, fort_buffer_t s3n_handle, fort_buffer_t s4n_handle, const double *dx, const double *dy, const double *dz, const double *dt, const int *nx, const int *ny, const int *nz, const int *halo) {
    EntryCall call{};
    call.context = fort_context;
    call.mode = fort_mode;
    call.kind = Template::StepAdvance;
    call.code_key = 0x9c9017766840cee4ULL;
    call.nscalar = 4;
    call.narrays = 14;
    call.arrays[0] = un_handle;
    call.arrays[1] = vn_handle;
    call.arrays[2] = wn_handle;
    call.arrays[3] = u_handle;
    call.arrays[4] = v_handle;
    call.arrays[5] = w_handle;
    call.arrays[6] = s1_handle;
    call.arrays[7] = s2_handle;
    call.arrays[8] = s3_handle;
    call.arrays[9] = s4_handle;
    call.arrays[10] = s1n_handle;
    call.arrays[11] = s2n_handle;
    call.arrays[12] = s3n_handle;
    call.arrays[13] = s4n_handle;
    call.nreals = 4;
    call.reals[0] = dx;
    call.reals[1] = dy;
    call.reals[2] = dz;
    call.reals[3] = dt;
    call.nints = 4;
    call.ints[0] = nx;
    call.ints[1] = ny;
    call.ints[2] = nz;
    call.ints[3] = halo;
    return run_entry(call);
}

// advection::halo4: periodic x/y boundary fill in the order of compiler/tests/apps/box/boundaries.f90:6-41; walls in z (W zero, mirrored)
extern "C" int cpp_fort_shared_073d04efb82a(fort_scope_t fort_context, int fort_mode, fort_buffer_t u_handle, fort_buffer_t v_handle, fort_buffer_t w_handle, fort_buffer_t s1_handle, fort_buffer_t s2_handle, fort_buffer_t s3_handle, fort_buffer_t s4_handle, const int *nx, const int *ny, const int *nz, const int *halo) {
    EntryCall call{};
    call.context = fort_context;
    call.mode = fort_mode;
    call.kind = Template::Halo;
    call.code_key = 0xce1bf742cef38e4aULL;
    call.nscalar = 4;
    call.narrays = 7;
    call.arrays[0] = u_handle;
    call.arrays[1] = v_handle;
    call.arrays[2] = w_handle;
    call.arrays[3] = s1_handle;
    call.arrays[4] = s2_handle;
    call.arrays[5] = s3_handle;
    call.arrays[6] = s4_handle;
    call.nreals = 0;
    call.nints = 4;
    call.ints[0] = nx;
    call.ints[1] = ny;
    call.ints[2] = nz;
    call.ints[3] = halo;
    return run_entry(call);
}

// stencil::diffuse7: compiler/tests/apps/box/stepper.f90:8-30 (diffuse with laplacian)
extern "C" int cpp_fort_shared_e331fbb8bf9a(fort_scope_t fort_context, int fort_mode, fort_buffer_t b_handle, fort_buffer_t a_handle, const double *dt, const double *nu, const double *dx, const int *nx, const int *ny, const int *nz, const int *halo) {
    EntryCall call{};
    call.context = fort_context;
    call.mode = fort_mode;
    call.kind = Template::Diffusion;
    call.code_key = 0x297afd6e2ec2445bULL;
    call.nscalar = 0;
    call.narrays = 2;
    call.arrays[0] = b_handle;
    call.arrays[1] = a_handle;
    call.nreals = 3;
    call.reals[0] = dt;
    call.reals[1] = nu;
    call.reals[2] = dx;
    call.nints = 4;
    call.ints[0] = nx;
    call.ints[1] = ny;
    call.ints[2] = nz;
    call.ints[3] = halo;
    return run_entry(call);
}

// stencil::jacobi5: compiler/tests/apps/relax/relax.f90:28-33 (one Jacobi sweep)
extern "C" int cpp_fort_shared_03470f69376f(fort_scope_t fort_context, int fort_mode, fort_buffer_t v_handle, fort_buffer_t u_handle, const int *nx, const int *ny, const int *halo) {
    EntryCall call{};
    call.context = fort_context;
    call.mode = fort_mode;
    call.kind = Template::Jacobi;
    call.code_key = 0x6d2a628ad5006681ULL;
    call.nscalar = 0;
    call.narrays = 2;
    call.arrays[0] = v_handle;
    call.arrays[1] = u_handle;
    call.nreals = 0;
    call.nints = 3;
    call.ints[0] = nx;
    call.ints[1] = ny;
    call.ints[2] = halo;
    return run_entry(call);
}

// stencil::yee2d: 2-D TM Yee leapfrog (no reference source in the mount)
extern "C" int cpp_fort_shared_82041a3f2b68(fort_scope_t fort_context, int fort_mode, fort_buffer_t ez_handle, fort_buffer_t hx_handle, fort_buffer_t hy_handle, const double *ch, const double *ce, const int *nx, const int *ny, const int *halo) {
    EntryCall call{};
    call.context = fort_context;
    call.mode = fort_mode;
    call.kind = Template::Yee;
    call.code_key = 0x467690fb19941ed3ULL;
    call.nscalar = 0;
    call.narrays = 3;
    call.arrays[0] = ez_handle;
    call.arrays[1] = hx_handle;
    call.arrays[2] = hy_handle;
    call.nreals = 2;
    call.reals[0] = ch;
    call.reals[1] = ce;
    call.nints = 3;
    call.ints[0] = nx;
    call.ints[1] = ny;
    call.ints[2] = halo;
    return run_entry(call);
}
