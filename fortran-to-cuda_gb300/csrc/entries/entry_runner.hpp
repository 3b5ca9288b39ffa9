// Interface between the generated C-ABI entries (shared_entries.cu, written by
// compiler/emission) and the hand-written template runner (entry_runner.cu).
// A generated entry only packs its arguments into an EntryCall.
#pragma once
#include <cstdint>

#include "../../../include/scoped_runtime.h"

namespace f2c::entries {

enum class Template : int {
    Set = 0,        // momentumadvection::set
    Multiply = 1,   // momentumadvection::multiply
    CduDiv = 2,
    CduAdv = 3,
    CdvDiv = 4,
    CdvAdv = 5,
    CdwDiv = 6,
    CdwAdv = 7,
    Cdu = 8,        // momentumadvection::cdu (set, CDUdiv, CDUadv, multiply fused)
    Cdv = 9,
    Cdw = 10,
    Step = 11,      // advection::step: U, V, W and scalar tendencies in one launch
    StepAdvance = 12, // advection::advance: forward-Euler step, double-buffered
    Halo = 13,      // advection::halo: periodic x/y, walls in z
    Diffusion = 14, // stencil::diffuse7 (box app stepper)
    Jacobi = 15,    // stencil::jacobi5 (relax app sweep)
    Yee = 16,       // stencil::yee2d (H then E)
};

constexpr int kMaxEntryArrays = 16;

struct EntryCall {
    fort_scope_t context;
    int mode;
    Template kind;
    uint64_t code_key;
    int nscalar;
    int narrays;
    fort_buffer_t arrays[kMaxEntryArrays];
    int nreals;
    const double *reals[8];
    int nints;
    const int *ints[8];
};

int run_entry(const EntryCall &call);

} // namespace f2c::entries
