// Template runner behind every generated numerical entry.
//
// The protocol mirrors the reference's generated entries
// (compiler/emission/cuda/scoped.py:237-512): ABI version and mode checks,
// writable-alias check, layout check per array, loop extents, the exact
// read/write sections of the template, storage reservation, the definition
// change of intent(out) arrays, and one queued task through
// fort_scope_graph_enqueue_v1 (the runtime submits the queue as a replayed
// CUDA graph). Where the reference entry runs its generated CPU worker (native
// mode, or device resources unavailable before any work started), this entry
// returns FORT_SCOPE_DECLINED and performs nothing: the spliced call block
// then publishes the domain and runs the original Fortran statements.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <vector>

#include "../kernels/advection_fast.cuh"
#include "../kernels/advection_faces.cuh"
#include "../kernels/advection_kernels.cuh"
#include "../kernels/procedures.cuh"
#include "../kernels/stencils.cuh"
#include "entry_runner.hpp"

namespace f2c::entries {
namespace {

using Triple = std::array<size_t, 3>;

// Storage-stable list of sections for one array.
class Sections {
public:
    void add(const Triple &lo, const Triple &hi) {
        lo_.push_back(lo);
        hi_.push_back(hi);
    }
    const fort_scope_section *data() {
        list_.clear();
        for (size_t n = 0; n < lo_.size(); ++n) list_.push_back({lo_[n].data(), hi_[n].data()});
        return list_.data();
    }
    size_t size() const { return lo_.size(); }

private:
    std::deque<Triple> lo_, hi_;
    std::vector<fort_scope_section> list_;
};

struct Geometry {
    long long n[3];
    long long h;
    size_t ext[3];
    long long z0 = 0; // first interior plane of a slab (0 for the whole domain)
    // [h+a, h+n+b) on axis d, shifted by z0 along the last axis
    size_t lo(int d, int a) const { return (size_t)(h + a + (d == 2 ? z0 : 0)); }
    size_t hi(int d, int b) const { return (size_t)(h + n[d] + b + (d == 2 ? z0 : 0)); }
    Triple box_lo(int ax, int ay, int az) const { return {lo(0, ax), lo(1, ay), lo(2, az)}; }
    Triple box_hi(int bx, int by, int bz) const { return {hi(0, bx), hi(1, by), hi(2, bz)}; }
};

void add_box(Sections &s, const Geometry &g, int ax, int bx, int ay, int by, int az, int bz) {
    s.add(g.box_lo(ax, ay, az), g.box_hi(bx, by, bz));
}
void add_interior(Sections &s, const Geometry &g) { add_box(s, g, 0, 0, 0, 0, 0, 0); }
void add_cross(Sections &s, const Geometry &g) {
    add_box(s, g, -1, 1, 0, 0, 0, 0);
    add_box(s, g, 0, 0, -1, 1, 0, 0);
    add_box(s, g, 0, 0, 0, 0, -1, 1);
}
// the non-own velocity reads of each momentum procedure
void add_cdu_v(Sections &s, const Geometry &g) { add_box(s, g, 0, 1, -1, 0, 0, 0); }
void add_cdu_w(Sections &s, const Geometry &g) { add_box(s, g, 0, 1, 0, 0, -1, 0); }
void add_cdv_u(Sections &s, const Geometry &g) { add_box(s, g, -1, 0, 0, 1, 0, 0); }
void add_cdv_w(Sections &s, const Geometry &g) { add_box(s, g, 0, 0, 0, 1, -1, 0); }
void add_cdw_u(Sections &s, const Geometry &g) { add_box(s, g, -1, 0, 0, 0, 0, 1); }
void add_cdw_v(Sections &s, const Geometry &g) { add_box(s, g, 0, 0, -1, 0, 0, 1); }

struct Use {
    fort_buffer_t handle = 0;
    bool written = false;
    bool overwritten = false; // every written element is written (an exact overwrite)
    bool read = false;
    bool intent_out = false;
    Sections reads, writes;
};

int declined() { return FORT_SCOPE_DECLINED; }

// Sections of the advection step (U, V, W tendencies and ns scalars): outputs
// write the interior, each velocity is read on its own cross and on the
// staggered neighbours of the other two momentum equations, scalars on their cross.
void step_sections(std::deque<Use> &uses, const Geometry &g, int ns) {
    for (int n = 0; n < 3; ++n) add_interior(uses[n].writes, g);
    Use &U = uses[3], &V = uses[4], &W = uses[5];
    add_cross(U.reads, g);
    add_cdv_u(U.reads, g);
    add_cdw_u(U.reads, g);
    add_cross(V.reads, g);
    add_cdu_v(V.reads, g);
    add_cdw_v(V.reads, g);
    add_cross(W.reads, g);
    add_cdu_w(W.reads, g);
    add_cdv_w(W.reads, g);
    for (int n = 0; n < ns; ++n) {
        add_cross(uses[6 + n].reads, g);
        add_interior(uses[6 + ns + n].writes, g);
    }
}

// Bindings of one task: each array's reads, and its writes (exact overwrites where every written element is written).
std::vector<fort_scope_plan_binding> bindings_of(std::deque<Use> &uses) {
    std::vector<fort_scope_plan_binding> bindings;
    for (auto &u : uses) {
        fort_scope_plan_binding b{};
        b.buffer = u.handle;
        b.access.read_count = u.reads.size();
        b.access.reads = u.reads.size() ? u.reads.data() : nullptr;
        if (u.written) {
            b.access.write_count = u.writes.size();
            b.access.writes = u.writes.data();
            if (u.overwritten) {
                b.access.overwrite_count = u.writes.size();
                b.access.overwrites = b.access.writes;
            }
        }
        bindings.push_back(b);
    }
    return bindings;
}

// Launch shape of the strict face-sharing kernel (fast = false) or of the
// fast-fp kernel (fast = true) for `a`; `a.kz` is set for the chosen kernel.
template <int NS, int MASK>
int faces_spec(AdvArgs &a, bool fast, fort_scope_kernel_v1 &k) {
    int ty = kFaceTY;  // rows of a tile
    if (fast) {
        const int sms = current_sm_count();
        ty = kFastTY;
        a.kz = fast_chunk_depth(a.nx, a.ny, a.nz, kFastTY, sms);
        // the build for three CTAs per SM when the launch has enough CTAs (as launch_fast chooses)
        const long long ctas = (long long)((a.nx + kFastTX - 1) / kFastTX) * ((a.ny + kFastTY - 1) / kFastTY) *
                               ((a.nz + a.kz - 1) / a.kz);
        k.function = ctas >= (long long)kFastDeepCtas * (sms > 0 ? sms : 152)
                         ? (const void *)advection_fast_kernel<NS, MASK, kFastTY, kFastDeepCtasPerSM>
                         : (const void *)advection_fast_kernel<NS, MASK, kFastTY>;
        k.shared_bytes = 0;
    } else {
        using Smem = FaceSmem<NS, MASK>;
        static std::atomic<unsigned long long> configured{0};
        const cudaError_t e =
            configure_shared_once(configured, (const void *)advection_faces_kernel<NS, MASK>, (int)Smem::bytes);
        if (e != cudaSuccess) return fort_scope_report_error(FORT_SCOPE_RESOURCE, "cannot configure the face kernel");
        a.kz = chunk_depth(a.nx, a.ny, a.nz);
        k.function = (const void *)advection_faces_kernel<NS, MASK>;
        k.shared_bytes = Smem::bytes;
    }
    k.grid[0] = (a.nx + kFaceTX - 1) / kFaceTX;
    k.grid[1] = (a.ny + ty - 1) / ty;
    k.grid[2] = (a.nz + a.kz - 1) / a.kz;
    k.block[0] = kFaceTX;
    k.block[1] = ty + 1;
    k.block[2] = 1;
    return FORT_SCOPE_OK;
}

template <int MASK>
int faces_spec_ns(int ns, AdvArgs &a, bool fast, fort_scope_kernel_v1 &k) {
    switch (ns) {
    case 0: return faces_spec<0, MASK>(a, fast, k);
    case 1: return faces_spec<1, MASK>(a, fast, k);
    case 2: return faces_spec<2, MASK>(a, fast, k);
    case 3: return faces_spec<3, MASK>(a, fast, k);
    default: return faces_spec<4, MASK>(a, fast, k);
    }
}

// Graph-cache keys of fast-fp launches differ from the strict ones, so a
// context that changes its contract never replays a graph of the other kernel.
constexpr uint64_t kFastKeyMask = 0x6a09e667f3bcc909ULL;

// Levels per slab when a step is cut into slabs to overlap host transfers with
// the kernels: about 2.5 M points a slab (measured on GB300 over plane sizes
// from 160 x 160 to 1024 x 512: thinner slabs pay per-copy and per-launch
// costs, thicker ones a longer pipeline fill and drain), at least 4 levels.
// F2C_SLAB_PLANES fixes the depth instead (read once per process).
constexpr long long kSlabPoints = 2500000;
int slab_planes(long long nx, long long ny) {
    static const int fixed = [] {
        const char *v = std::getenv("F2C_SLAB_PLANES");
        const int p = v ? std::atoi(v) : 0;
        return p >= 2 ? p : 0;
    }();
    if (fixed) return fixed;
    const long long plane = std::max(1LL, nx * ny);
    return (int)std::max(4LL, (kSlabPoints + plane - 1) / plane);
}

// Slab boundaries along z: slabs of `planes` levels between a first and a last
// slab of half that depth (thin ends shorten the pipeline's fill, when only
// uploads run, and its drain, when only publications run); at most 62 slabs.
std::vector<int> slab_bounds(int nz, int planes) {
    planes = std::max(planes, (nz + 59) / 60);
    static const int fixed_edge = [] {
        const char *v = std::getenv("F2C_SLAB_EDGE");  // levels of the first and last slab (read once per process)
        return v ? std::atoi(v) : 0;
    }();
    const int edge = fixed_edge > 0 ? std::min(fixed_edge, planes) : std::max(1, planes / 2);
    std::vector<int> b{0};
    if (nz < 2 * edge + planes) {
        const int count = std::max(1, nz / std::max(1, planes));
        for (int s = 1; s <= count; ++s) b.push_back((int)((long long)s * nz / count));
        return b;
    }
    const int middle = nz - 2 * edge;
    const int count = (middle + planes - 1) / planes;
    b.push_back(edge);
    for (int s = 1; s <= count; ++s) b.push_back(edge + (int)((long long)s * middle / count));
    b.push_back(nz);
    return b;
}

// The step as a sequence of slab tasks along z: task s computes interior planes
// [k0, k1) with every array pointer moved to plane k0 (the kernel addresses
// planes relative to its interior start and reads one plane either side).
int enqueue_step_slabs(const EntryCall &call, const Geometry &g, const std::deque<Use> &roles, const AdvArgs &whole,
                       int ns, bool fast) {
    const std::vector<int> bounds = slab_bounds((int)g.n[2], slab_planes(g.n[0], g.n[1]));
    const int count = (int)bounds.size() - 1;
    std::vector<AdvArgs> args(count);
    std::vector<void *> argument_of(count);
    std::vector<std::deque<Use>> uses(count);
    std::vector<std::vector<fort_scope_plan_binding>> bindings(count);
    std::vector<fort_scope_graph_task_v1> tasks(count);
    std::vector<size_t> sizes(count, sizeof(AdvArgs));
    for (int s = 0; s < count; ++s) {
        const int k0 = bounds[s], k1 = bounds[s + 1];
        const long long shift = (long long)k0 * whole.plane;
        AdvArgs &a = args[s];
        a = whole;
        a.u += shift;
        a.v += shift;
        a.w += shift;
        for (int n = 0; n < 3; ++n) a.out[n] += shift;
        for (int n = 0; n < ns; ++n) {
            a.s[n] += shift;
            a.st[n] += shift;
        }
        a.nz = k1 - k0;
        Geometry slab = g;
        slab.n[2] = k1 - k0;
        slab.z0 = k0;
        for (const Use &r : roles) {
            uses[s].emplace_back();
            Use &u = uses[s].back();
            u.handle = r.handle;
            u.read = r.read;
            u.written = r.written;
            u.overwritten = r.overwritten;
            u.intent_out = r.intent_out;
        }
        step_sections(uses[s], slab, ns);
        bindings[s] = bindings_of(uses[s]);
        argument_of[s] = &args[s];
        fort_scope_kernel_v1 &k = tasks[s].kernel;
        k.version = FORT_SCOPE_GRAPH_ABI_VERSION;
        if (int st = faces_spec_ns<7>(ns, a, fast, k)) return st;
        k.arguments = &argument_of[s];
        k.argument_count = 1;
        tasks[s].bindings = bindings[s].data();
        tasks[s].binding_count = bindings[s].size();
    }
    return fort_scope_slab_enqueue_v1(call.context, fast ? call.code_key ^ kFastKeyMask : call.code_key, tasks.data(),
                                      tasks.size(), sizes.data());
}

const void *procedure_function(Template t) {
    switch (t) {
    case Template::Set: return (const void *)procedure_kernel<kOpSet>;
    case Template::Multiply: return (const void *)procedure_kernel<kOpMultiply>;
    case Template::CduDiv: return (const void *)procedure_kernel<kOpCduDiv>;
    case Template::CduAdv: return (const void *)procedure_kernel<kOpCduAdv>;
    case Template::CdvDiv: return (const void *)procedure_kernel<kOpCdvDiv>;
    case Template::CdvAdv: return (const void *)procedure_kernel<kOpCdvAdv>;
    case Template::CdwDiv: return (const void *)procedure_kernel<kOpCdwDiv>;
    case Template::CdwAdv: return (const void *)procedure_kernel<kOpCdwAdv>;
    default: return nullptr;
    }
}

int enqueue_one(const EntryCall &call, fort_scope_kernel_v1 kernel, void *argument, size_t argument_size,
                std::deque<Use> &uses, uint64_t key) {
    void *arguments[1] = {argument};
    kernel.version = FORT_SCOPE_GRAPH_ABI_VERSION;
    kernel.arguments = arguments;
    kernel.argument_count = 1;
    std::vector<fort_scope_plan_binding> bindings;
    for (auto &u : uses) {
        fort_scope_plan_binding b{};
        b.buffer = u.handle;
        b.access.read_count = u.reads.size();
        b.access.reads = u.reads.size() ? u.reads.data() : nullptr;
        if (u.written) {
            b.access.write_count = u.writes.size();
            b.access.writes = u.writes.data();
            if (u.overwritten) {
                b.access.overwrite_count = u.writes.size();
                b.access.overwrites = b.access.writes;
            }
        }
        bindings.push_back(b);
    }
    fort_scope_graph_task_v1 task{};
    task.kernel = kernel;
    task.bindings = bindings.data();
    task.binding_count = bindings.size();
    const size_t sizes[1] = {argument_size};
    return fort_scope_graph_enqueue_v1(call.context, key, &task, sizes);
}

// The Yee step is two tasks: H from E, then E from H.
int enqueue_yee(const EntryCall &call, const Geometry &g, std::deque<Use> &uses, std::vector<void *> &devices,
                long long sx) {
    YeeArgs y{static_cast<double *>(devices[0]), static_cast<double *>(devices[1]), static_cast<double *>(devices[2]),
              *call.reals[0], *call.reals[1], (int)g.n[0], (int)g.n[1], (int)g.h, sx};
    const dim3 grid = yee_grid(y);
    fort_scope_kernel_v1 k{};
    k.grid[0] = grid.x; k.grid[1] = grid.y; k.grid[2] = 1;
    k.block[0] = kYeeBX; k.block[1] = kYeeBY; k.block[2] = 1;
    // H task: Ez read at (i, j), (i+1, j), (i, j+1); Hx, Hy read and written on the interior
    std::deque<Use> h(3);
    for (int n = 0; n < 3; ++n) h[n].handle = uses[n].handle;
    add_box(h[0].reads, g, 0, 1, 0, 0, 0, 0);
    add_box(h[0].reads, g, 0, 0, 0, 1, 0, 0);
    for (int n = 1; n < 3; ++n) {
        h[n].written = h[n].overwritten = true;
        add_interior(h[n].reads, g);
        add_interior(h[n].writes, g);
    }
    k.function = (const void *)yee_h_kernel;
    if (int s = enqueue_one(call, k, &y, sizeof y, h, call.code_key)) return s;
    // E task: Hy read at (i-1, j), Hx at (i, j-1); Ez read and written on the interior
    std::deque<Use> e(3);
    for (int n = 0; n < 3; ++n) e[n].handle = uses[n].handle;
    e[0].written = e[0].overwritten = true;
    add_interior(e[0].reads, g);
    add_interior(e[0].writes, g);
    add_box(e[1].reads, g, 0, 0, -1, 0, 0, 0);
    add_box(e[2].reads, g, -1, 0, 0, 0, 0, 0);
    k.function = (const void *)yee_e_kernel;
    const int s = enqueue_one(call, k, &y, sizeof y, e, call.code_key ^ 0x9e3779b97f4a7c15ULL);
    // the H task was accepted: a failure now leaves half a step behind
    if (s && s != FORT_SCOPE_EXECUTION) return fort_scope_execution_error(call.context, "second task of a step refused");
    return s;
}

int run(const EntryCall &call) {
    if (fort_scope_abi_version() != FORT_SCOPE_ABI_VERSION)
        return fort_scope_report_error(FORT_SCOPE_ARGUMENT, "incompatible shared runtime ABI");
    if (call.mode < FORT_SCOPE_NATIVE || call.mode > FORT_SCOPE_GPU)
        return fort_scope_report_error(FORT_SCOPE_ARGUMENT, "unknown shared execution mode");
    for (int n = 0; n < call.nreals; ++n)
        if (!call.reals[n]) return fort_scope_report_error(FORT_SCOPE_ARGUMENT, "null shared scalar argument");
    for (int n = 0; n < call.nints; ++n)
        if (!call.ints[n]) return fort_scope_report_error(FORT_SCOPE_ARGUMENT, "null shared scalar argument");
    if (call.mode == FORT_SCOPE_NATIVE) return declined();
    int numerics = FORT_SCOPE_NUMERICS_STRICT;
    if (int s = fort_scope_numerics_get_v1(call.context, &numerics)) return s;
    const bool fast = numerics == FORT_SCOPE_NUMERICS_FAST;

    const Template t = call.kind;
    const int ns = call.nscalar;
    const bool step = t == Template::Step || t == Template::StepAdvance;
    const bool halo = t == Template::Halo;
    const bool procedure = static_cast<int>(t) <= static_cast<int>(Template::Cdw); // MomentumAdvection procedures

    // ---- roles of the arrays, in the declared argument order ----
    std::deque<Use> uses(call.narrays);
    for (int n = 0; n < call.narrays; ++n) uses[n].handle = call.arrays[n];
    auto role = [&](int n, bool read, bool written, bool overwritten, bool intent_out) {
        uses[n].read = read;
        uses[n].written = written;
        uses[n].overwritten = overwritten;
        uses[n].intent_out = intent_out;
    };
    switch (t) {
    case Template::Set: role(0, false, true, true, true); break;
    case Template::Multiply: role(0, true, true, false, false); break;
    case Template::CduDiv: case Template::CdvDiv: case Template::CdwDiv:
    case Template::Cdu: case Template::Cdv: case Template::Cdw:
        role(0, false, true, true, true);
        for (int n = 1; n < 4; ++n) role(n, true, false, false, false);
        break;
    case Template::CduAdv: case Template::CdvAdv: case Template::CdwAdv:
        role(0, true, true, false, false);
        for (int n = 1; n < 4; ++n) role(n, true, false, false, false);
        break;
    case Template::Step: case Template::StepAdvance:
        for (int n = 0; n < 3; ++n) role(n, false, true, true, true);
        for (int n = 3; n < 6 + ns; ++n) role(n, true, false, false, false);
        for (int n = 6 + ns; n < 6 + 2 * ns; ++n) role(n, false, true, true, true);
        break;
    case Template::Halo:
        for (int n = 0; n < call.narrays; ++n) role(n, true, true, true, false);
        break;
    case Template::Diffusion: case Template::Jacobi:
        // the output is intent(inout) in the sources (stepper.f90:17-20; relax's v keeps its boundary):
        // its interior is overwritten and its ghost values stay defined
        role(0, false, true, true, false);
        role(1, true, false, false, false);
        break;
    case Template::Yee:
        for (int n = 0; n < 3; ++n) role(n, true, true, true, false);
        break;
    }
    const bool plane2d = t == Template::Jacobi || t == Template::Yee;
    const int rank = plane2d ? 2 : 3;
    // writable arguments must not alias any other argument
    for (int a = 0; a < call.narrays; ++a)
        for (int b = 0; b < a; ++b)
            if (uses[a].handle == uses[b].handle && (uses[a].written || uses[b].written))
                return fort_scope_report_error(FORT_SCOPE_ALIAS, "writable entry arguments alias");

    // ---- layouts ----
    Geometry g{};
    for (int n = 0; n < call.narrays; ++n) {
        fort_scope_layout layout{};
        if (int s = fort_scope_layout_get(call.context, uses[n].handle, &layout)) return s;
        if ((int)layout.rank != rank || layout.type != FORT_SCOPE_REAL64 || layout.element_bytes != sizeof(double))
            return fort_scope_report_error(FORT_SCOPE_ARGUMENT, "entry layout/type mismatch");
        if (n == 0) {
            for (int d = 0; d < 3; ++d) g.ext[d] = d < rank ? layout.extents[d] : 1;
        } else {
            for (int d = 0; d < rank; ++d)
                if (layout.extents[d] != g.ext[d]) return declined(); // templates take one shape per call
        }
    }
    // ---- loop extents and the interior offset ----
    const int *ints[8];
    for (int n = 0; n < call.nints; ++n) ints[n] = call.ints[n];
    for (int d = 0; d < rank; ++d) g.n[d] = *ints[d];
    if (plane2d) g.n[2] = 1;
    g.h = procedure ? 1 : *ints[rank];
    if (g.n[0] < 1 || g.n[1] < 1 || g.n[2] < 1) return FORT_SCOPE_OK; // no iterations: nothing to do
    if (g.h < 1) return fort_scope_report_error(FORT_SCOPE_ARGUMENT, "halo width must be at least one");
    for (int d = 0; d < rank; ++d)
        if ((size_t)(g.n[d] + 2 * g.h) > g.ext[d])
            return fort_scope_report_error(FORT_SCOPE_ARGUMENT, "invalid physical entry footprint");
    if (halo) {
        for (int d = 0; d < 3; ++d)
            if ((size_t)(g.n[d] + 2 * g.h) != g.ext[d]) return declined();
        if (g.n[2] < g.h + 1 || g.n[0] < g.h || g.n[1] < g.h) return declined();
    }

    // ---- exact sections ----
    auto out_sections = [&](Use &u) {
        add_interior(u.writes, g);
        if (u.read) add_interior(u.reads, g);
    };
    switch (t) {
    case Template::Set: case Template::Multiply: out_sections(uses[0]); break;
    case Template::CduDiv: case Template::CduAdv: case Template::Cdu:
        out_sections(uses[0]);
        add_cross(uses[1].reads, g);
        add_cdu_v(uses[2].reads, g);
        add_cdu_w(uses[3].reads, g);
        break;
    case Template::CdvDiv: case Template::CdvAdv: case Template::Cdv:
        out_sections(uses[0]);
        add_cdv_u(uses[1].reads, g);
        add_cross(uses[2].reads, g);
        add_cdv_w(uses[3].reads, g);
        break;
    case Template::CdwDiv: case Template::CdwAdv: case Template::Cdw:
        out_sections(uses[0]);
        add_cdw_u(uses[1].reads, g);
        add_cdw_v(uses[2].reads, g);
        add_cross(uses[3].reads, g);
        break;
    case Template::Step: case Template::StepAdvance:
        step_sections(uses, g, ns);
        break;
    case Template::Diffusion:
        out_sections(uses[0]);
        add_cross(uses[1].reads, g);
        break;
    case Template::Jacobi:
        out_sections(uses[0]);
        add_box(uses[1].reads, g, -1, 1, 0, 0, 0, 0);
        add_box(uses[1].reads, g, 0, 0, -1, 1, 0, 0);
        break;
    case Template::Yee:
        break; // two tasks with their own sections, below
    case Template::Halo: {
        for (int n = 0; n < call.narrays; ++n) {
            Use &u = uses[n];
            add_interior(u.reads, g);
            const size_t ex = g.ext[0], ey = g.ext[1], ez = g.ext[2], h = (size_t)g.h;
            const size_t nx = (size_t)g.n[0], ny = (size_t)g.n[1], nz = (size_t)g.n[2];
            u.writes.add({0, 0, 0}, {ex, ey, h});
            u.writes.add({0, 0, h + nz}, {ex, ey, ez});
            u.writes.add({0, 0, h}, {ex, h, h + nz});
            u.writes.add({0, h + ny, h}, {ex, ey, h + nz});
            u.writes.add({0, h, h}, {h, h + ny, h + nz});
            u.writes.add({h + nx, h, h}, {ex, h + ny, h + nz});
            if (n == 2) u.writes.add({h, h, h + nz - 1}, {h + nx, h + ny, h + nz}); // W top wall faces
        }
        break;
    }
    }

    // ---- storage first, so a resource failure changes nothing ----
    std::vector<fort_buffer_t> handles;
    for (auto &u : uses) handles.push_back(u.handle);
    std::vector<void *> devices(handles.size(), nullptr);
    // a deep step may run as slabs, its host transfers overlapped with the kernels
    const bool sliceable = step && g.n[2] >= 2 * slab_planes(g.n[0], g.n[1]);
    int pipelined = 0;
    {
        const int s = sliceable ? fort_scope_device_reserve_slabs_v1(call.context, handles.data(), handles.size(),
                                                                     devices.data(), &pipelined)
                                : fort_scope_device_reserve_many_v1(call.context, handles.data(), handles.size(),
                                                                    devices.data());
        if (s == FORT_SCOPE_RESOURCE) return declined();
        if (s) return s;
    }
    for (auto &u : uses)
        if (u.intent_out)
            if (int s = fort_scope_forget_definition(call.context, u.handle)) return s;

    // ---- kernel arguments ----
    AdvArgs adv{};
    ProcedureArgs proc{};
    HaloArgs hal{};
    DiffusionArgs diff{};
    JacobiArgs jac{};
    fort_scope_kernel_v1 kernel{};
    kernel.version = FORT_SCOPE_GRAPH_ABI_VERSION;
    void *argument = nullptr;
    size_t argument_size = 0;
    const long long sx = (long long)g.ext[0], plane = (long long)(g.ext[0] * g.ext[1]);
    auto dev = [&](int n) { return static_cast<double *>(devices[n]); };
    if (procedure && (t == Template::Cdu || t == Template::Cdv || t == Template::Cdw)) {
        adv.u = dev(1); adv.v = dev(2); adv.w = dev(3);
        const int slot = t == Template::Cdu ? 0 : t == Template::Cdv ? 1 : 2;
        adv.out[slot] = dev(0);
        adv.nx = (int)g.n[0]; adv.ny = (int)g.n[1]; adv.nz = (int)g.n[2]; adv.h = (int)g.h;
        adv.sx = sx; adv.plane = plane;
        adv.c = make_coefficients(*call.reals[0], *call.reals[1], *call.reals[2]);
        adv.f = make_fast_coefficients(*call.reals[0], *call.reals[1], *call.reals[2], 0, 0.0);
        const int st = t == Template::Cdu   ? faces_spec_ns<1>(0, adv, fast, kernel)
                       : t == Template::Cdv ? faces_spec_ns<2>(0, adv, fast, kernel)
                                            : faces_spec_ns<4>(0, adv, fast, kernel);
        if (st) return st;
        argument = &adv;
        argument_size = sizeof adv;
    } else if (procedure) {
        proc.out = dev(0);
        if (t != Template::Set && t != Template::Multiply) {
            proc.u = dev(1); proc.v = dev(2); proc.w = dev(3);
            proc.c = make_coefficients(*call.reals[0], *call.reals[1], *call.reals[2]);
        } else {
            proc.value = *call.reals[0];
        }
        proc.nx = (int)g.n[0]; proc.ny = (int)g.n[1]; proc.nz = (int)g.n[2]; proc.h = 1;
        proc.sx = sx; proc.plane = plane;
        kernel.function = procedure_function(t);
        const dim3 grid = procedure_grid(proc);
        kernel.grid[0] = grid.x; kernel.grid[1] = grid.y; kernel.grid[2] = grid.z;
        kernel.block[0] = kProcBX; kernel.block[1] = kProcBY; kernel.block[2] = 1;
        argument = &proc;
        argument_size = sizeof proc;
    } else if (step) {
        adv.out[0] = dev(0); adv.out[1] = dev(1); adv.out[2] = dev(2);
        adv.u = dev(3); adv.v = dev(4); adv.w = dev(5);
        adv.nscalar = ns;
        for (int n = 0; n < ns; ++n) {
            adv.s[n] = dev(6 + n);
            adv.st[n] = dev(6 + ns + n);
        }
        adv.mode = t == Template::StepAdvance ? 1 : 0;
        adv.dt = t == Template::StepAdvance ? *call.reals[3] : 0.0;
        adv.nx = (int)g.n[0]; adv.ny = (int)g.n[1]; adv.nz = (int)g.n[2]; adv.h = (int)g.h;
        adv.sx = sx; adv.plane = plane;
        adv.c = make_coefficients(*call.reals[0], *call.reals[1], *call.reals[2]);
        adv.f = make_fast_coefficients(*call.reals[0], *call.reals[1], *call.reals[2], adv.mode, adv.dt);
        if (pipelined) return enqueue_step_slabs(call, g, uses, adv, ns, fast);
        if (int st = faces_spec_ns<7>(ns, adv, fast, kernel)) return st;
        argument = &adv;
        argument_size = sizeof adv;
    } else if (t == Template::Diffusion) {
        diff.b = dev(0);
        diff.a = dev(1);
        diff.dtnu = *call.reals[0] * *call.reals[1];
        diff.dx2 = *call.reals[2] * *call.reals[2];
        diff.dx2_pow2 = power_of_two(diff.dx2, &diff.dx2_exp) ? 1 : 0;
        diff.nx = (int)g.n[0]; diff.ny = (int)g.n[1]; diff.nz = (int)g.n[2]; diff.h = (int)g.h;
        diff.sx = sx; diff.plane = plane;
        kernel.function = (const void *)diffusion7_kernel;
        const dim3 grid = diffusion_grid(diff);
        kernel.grid[0] = grid.x; kernel.grid[1] = grid.y; kernel.grid[2] = grid.z;
        kernel.block[0] = kDiffBX; kernel.block[1] = kDiffBY; kernel.block[2] = 1;
        argument = &diff;
        argument_size = sizeof diff;
    } else if (t == Template::Jacobi) {
        jac = JacobiArgs{dev(1), dev(0), (int)g.n[0], (int)g.n[1], (int)g.h, sx};
        kernel.function = (const void *)jacobi5_kernel;
        const dim3 grid = jacobi_grid(jac);
        kernel.grid[0] = grid.x; kernel.grid[1] = grid.y; kernel.grid[2] = grid.z;
        kernel.block[0] = kJacBX; kernel.block[1] = kJacBY; kernel.block[2] = 1;
        argument = &jac;
        argument_size = sizeof jac;
    } else if (t == Template::Yee) {
        return enqueue_yee(call, g, uses, devices, sx);
    } else {
        hal.count = call.narrays;
        for (int n = 0; n < call.narrays; ++n) {
            hal.f[n] = dev(n);
            hal.kind[n] = n == 2 ? 1 : 0;
        }
        hal.nx = (int)g.n[0]; hal.ny = (int)g.n[1]; hal.nz = (int)g.n[2]; hal.h = (int)g.h;
        hal.sx = sx; hal.plane = plane;
        const long long ex = g.n[0] + 2 * g.h;
        kernel.function = (const void *)halo_fill_kernel;
        kernel.grid[0] = (unsigned)(g.ext[1] * g.ext[2]);
        kernel.grid[1] = (unsigned)call.narrays;
        kernel.grid[2] = 1;
        kernel.block[0] = ex >= 256 ? 256 : (unsigned)(((ex + 31) / 32) * 32);
        kernel.block[1] = kernel.block[2] = 1;
        argument = &hal;
        argument_size = sizeof hal;
    }
    void *arguments[1] = {argument};
    kernel.arguments = arguments;
    kernel.argument_count = 1;

    // ---- one queued task with the exact effects ----
    std::vector<fort_scope_plan_binding> bindings = bindings_of(uses);
    fort_scope_graph_task_v1 task{};
    task.kernel = kernel;
    task.bindings = bindings.data();
    task.binding_count = bindings.size();
    const size_t sizes[1] = {argument_size};
    // the fused procedures and steps ran their fast-fp kernel: keep their graphs apart from the strict ones
    const bool fast_kernel = fast && (step || t == Template::Cdu || t == Template::Cdv || t == Template::Cdw);
    const int status =
        fort_scope_graph_enqueue_v1(call.context, fast_kernel ? call.code_key ^ kFastKeyMask : call.code_key, &task, sizes);
    if (status == FORT_SCOPE_OK) return FORT_SCOPE_OK;
    if (status == FORT_SCOPE_EXECUTION) return status;
    // nothing was accepted: only definitions were forgotten, which the original statements redefine
    return status;
}

} // namespace

int run_entry(const EntryCall &call) {
    if (call.narrays < 1 || call.narrays > kMaxEntryArrays || call.nints > 8 || call.nreals > 8)
        return fort_scope_report_error(FORT_SCOPE_ARGUMENT, "malformed entry call");
    return run(call);
}

} // namespace f2c::entries
