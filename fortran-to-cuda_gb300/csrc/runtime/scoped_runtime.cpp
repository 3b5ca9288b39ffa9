// GB300 residency runtime: implementation of the fort_scope_* ABI
// (include/scoped_runtime.h), the drop-in replacement for the reference's
// compiler/runtime/scoped_runtime.cu.
//
// Design, GB300-first:
//  * A domain owns the physical state: registered arrays, their device mirrors
//    (stream-ordered allocations on the context stream), the budget with LRU
//    eviction, and the statistics. A context borrows a domain and owns the
//    execution state: one non-blocking stream, the task queue, the graph cache.
//  * Coherence is tracked per array as three rectangle sets (regions.hpp):
//    defined values, values current on the host, values current on the device.
//    A device task uploads exactly the defined sections it reads (or partially
//    writes) that the device lacks; a host access downloads exactly what the
//    host lacks; observation publishes what only the device holds.
//  * Accepted tasks join a queue that is submitted as one CUDA graph. A task
//    sequence runs with direct launches the first time it is reached, is
//    instantiated as a graph the second time, and is replayed afterwards with
//    cudaGraphExecKernelNodeSetParams for the nodes whose arguments changed
//    (the reference's policy, compiler/runtime/scoped_graphs.hpp:140-235).
//  * Host arrays of 1 MiB or more are pinned in place at registration
//    (FORT_SCOPE_PIN_HOST=0 disables it; arrays already page-locked by the
//    caller are used as they are) so uploads and downloads run as DMA
//    over NVLink-C2C without staging, and are mapped into the device address
//    space. An array the host writes or reads back between every device use
//    (two uses in a row) is then accessed IN PLACE: its tasks get the mapped
//    host address, their kernels stream it over NVLink-C2C, and no copy or
//    device mirror is involved (FORT_SCOPE_HOST_IN_PLACE=0 disables it).
//  * Failures after numerical work started poison the context and its domain;
//    nothing is replayed (scoped_runtime.h:428-438 of the reference).
#include "../../../include/scoped_runtime.h"

#include <cinttypes>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <initializer_list>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <tuple>
#include <vector>

#include "backend.hpp"
#include "regions.hpp"

namespace f2c::rt {

#ifndef F2C_RUNTIME_CPU_BACKEND
thread_local std::string Backend::error;
#endif

namespace {

thread_local std::string t_error;
std::recursive_mutex g_mutex;

int fail(int status, const std::string &message) {
    t_error = message;
    return status;
}

struct Failure {
    int status;
    std::string message;
};

[[noreturn]] void raise(int status, const std::string &message) { throw Failure{status, message}; }

bool env_flag(const char *name, bool fallback) {
    const char *v = std::getenv(name);
    if (!v || !*v) return fallback;
    return std::strcmp(v, "0") != 0;
}

bool tracing() {
    static const bool on = env_flag("FORT_RUNTIME_TRACE", false);
    return on;
}

struct Context;
struct Domain;

struct Buffer {
    uint64_t handle = 0, identity = 0, generation = 0;
    int rank = 0;
    uint32_t type = 0;
    size_t elem = 0, bytes = 0;
    void *host = nullptr;
    size_t extents[kMaxRank] = {};
    int64_t lower[kMaxRank] = {};
    void *device = nullptr;
    bool pinned_host = false;  // page-locked (and mapped) for DMA
    bool pinned_here = false;  // ... by this runtime, which unpins it
    bool pin_tried = false;      // pinning is tried once, at the array's first device use
    void *mapped = nullptr;      // device-usable address of the pinned host array
    bool host_touched = true;    // the host wrote or read it since its last device use
    int host_rounds = 0;         // consecutive device uses, each preceded by host access
    bool in_place = false;       // the pending reservation hands out `mapped`
    Region defined, host_valid, device_valid;
    // Cells whose values are real: every definition since the values were last
    // discarded. Forgetting a definition makes reads illegal but keeps these,
    // so what the device already wrote still reaches the host.
    Region physical;
    enum { NONE, HOST, DEVICE } prepared = NONE;
    Region prep_writes, prep_overwrites;
    uint64_t last_use = 0;
    int queued = 0; // accepted tasks not yet submitted that use this buffer
    // Host sections that device-side work still in flight reads (uploads, kernels
    // on the mapped array) or writes (publications, kernels on the mapped array),
    // and the completion token recorded after that work (0: none).
    Region host_reading, host_writing;
    uint64_t host_token = 0;
    bool awaits_token = false;  // queued in-place work: its token is recorded when it is submitted

    Box full() const { return whole(rank, extents); }
    CopyPlan plan() const {
        CopyPlan p;
        p.rank = rank;
        p.elem = elem;
        for (int d = 0; d < rank; ++d) p.extents[d] = extents[d];
        return p;
    }
};

// The trace state (owner, procedure, segment, operation, implementation,
// boundary) a launch is reported under.
struct Provenance {
    char fields[6][65] = {};
};

struct Task {
    uint64_t code_key = 0;
    Provenance origin;  // the trace state when the task was accepted: its launch reports it
    LaunchSpec spec;
    std::vector<std::vector<unsigned char>> values;
    std::vector<uint64_t> buffers;
    uint64_t threads = 0;
};

struct CachedGraph {
    std::vector<const void *> functions;
    std::vector<size_t> argument_counts;
    std::vector<std::vector<std::vector<unsigned char>>> values; // per node, per argument
    std::vector<LaunchSpec> specs;
    Backend::Graph *graph = nullptr;
    int reached = 0;
};

struct Domain {
    uint64_t handle = 0;
    int device = 0;
    size_t budget = 0;
    bool budget_set = false, budget_warned = false;
    bool poisoned = false, owned_by_context = false;
    Context *borrower = nullptr;
    std::map<uint64_t, std::unique_ptr<Buffer>> buffers;
    std::map<uint64_t, uint64_t> by_identity;
    size_t device_bytes = 0, scratch_bytes = 0;
    // device memory external providers allocated themselves, claimed against the same budget
    std::map<uint64_t, size_t> workspaces;
    size_t workspace_bytes = 0;
    size_t peak_total_bytes = 0;  // the most mirrors, scratch and workspace held at once
    fort_scope_stats stats{};
    fort_scope_residency_stats_v1 residency{};
    uint64_t tick = 0;
};

struct Context {
    uint64_t handle = 0;
    Domain *domain = nullptr;
    bool private_domain = false;
    bool poisoned = false;
    Stream stream = nullptr;
    bool stream_ready = false;
    // copy streams of slab pipelines: uploads ahead of the kernels, publication behind them
    Stream copy_in = nullptr, copy_out = nullptr;
    bool copies_ready = false;
    bool queue_enabled = true, graphs_enabled = true;
    int numerics = 0;  // FORT_SCOPE_NUMERICS_STRICT or FORT_SCOPE_NUMERICS_FAST, for the entries' kernels
    int pin_host = -1;  // pinning of this context's host arrays at first device use: -1 FORT_SCOPE_PIN_HOST, 0 off, 1 on
    // Timing of slab sequences (off unless asked for): per slab, events around its uploads (copy stream 1),
    // its kernel (the context stream) and its publications (copy stream 2); those of the last sequence.
    struct SlabMarks {
        Backend::Event up0{}, up1{}, k0{}, k1{}, p0{}, p1{};
        bool made = false, uploaded = false, published = false;
    };
    bool slab_timing = false;
    std::vector<SlabMarks> slab_marks;
    size_t slab_marks_used = 0;
    uint64_t queue_work_limit = uint64_t(1) << 18;
    std::vector<Task> pending;
    uint64_t pending_threads = 0;
    // Each array's coherence state before the first queued task touched it: cancelling the queue restores
    // them (queued tasks apply their effects when accepted, and a cancelled task must leave none).
    struct Before {
        Region defined, host_valid, device_valid, physical;
        bool host_touched;
        int host_rounds;
    };
    std::map<uint64_t, Before> queued_before;
    std::map<uint64_t, CachedGraph> graphs;
    std::map<uint64_t, CachedGraph> group_graphs;  // kernel groups and checked groups, by the caller's key
    fort_scope_graph_stats_v1 graph_stats{};
    fort_scope_graph_queue_stats_v1 queue_stats{};
    fort_scope_completion_stats_v1 completion{};
    // completion tokens: events recorded on the context stream, oldest first
    struct Token {
        uint64_t serial;
        Backend::Event event;
    };
    std::deque<Token> tokens;
    std::vector<Backend::Event> spare_events;
    uint64_t token_serial = 0, complete_serial = 0;
    std::vector<uint64_t> awaiting_token;  // handles of arrays with in-place work not yet submitted
    bool untracked = false;                // device work whose host accesses no token records
    char trace[6][65] = {};
    // scratch arena
    void *scratch = nullptr;
    size_t scratch_capacity = 0, scratch_active_bytes = 0;
    bool scratch_active = false;
    uint64_t scratch_token = 0;
    fort_scope_scratch_stats_v1 scratch_stats{};
};

std::map<uint64_t, std::unique_ptr<Context>> g_contexts;
std::map<uint64_t, std::unique_ptr<Domain>> g_domains;
uint64_t g_next_handle = 0x5c0de000ULL;
std::set<uint64_t> g_retired;

uint64_t new_handle() { return ++g_next_handle; }

// One trace line per runtime event, with the reference's keys: the array's
// identity and generation when the event concerns one, the bytes moved, the
// context and its domain (storage when the context owns a private domain),
// and the provenance fields, `unknown` where unset. A launch of a queued task
// reports the provenance the task was accepted under.
void trace_line(Context *c, const char *event, uint64_t buffer, uint64_t bytes, const Provenance *origin = nullptr) {
    if (!tracing()) return;
    std::string line = std::string("FORT_SCOPED ") + event;
    char text[160];
    const Buffer *b = nullptr;
    if (buffer && c && c->domain) {
        auto it = c->domain->buffers.find(buffer);
        if (it != c->domain->buffers.end()) b = it->second.get();
    }
    if (b) {
        std::snprintf(text, sizeof text, " buffer=%" PRIu64 " generation=%" PRIu64, b->identity, b->generation);
        line += text;
    }
    std::snprintf(text, sizeof text, " bytes=%" PRIu64 " provenance_version=1 context=%" PRIu64, bytes,
                  c ? c->handle : 0);
    line += text;
    if (c && c->domain) {
        std::snprintf(text, sizeof text, " domain_version=1 domain=%" PRIu64 " domain_role=%s", c->domain->handle,
                      c->private_domain ? "storage" : "execution");
        line += text;
    }
    if (b) {
        std::snprintf(text, sizeof text, " buffer_handle=%" PRIu64, b->handle);
        line += text;
    }
    static const char *const names[6] = {"owner", "procedure", "segment", "operation", "implementation", "boundary"};
    for (int n = 0; n < 6; ++n) {
        const char *value = origin ? origin->fields[n] : c ? c->trace[n] : "";
        line += std::string(" ") + names[n] + "=" + (value[0] ? value : "unknown");
    }
    line += "\n";
    std::fputs(line.c_str(), stderr);
}

Context *find_context(fort_scope_t handle) {
    auto it = g_contexts.find(handle);
    if (it == g_contexts.end()) {
        if (g_retired.count(handle)) raise(FORT_SCOPE_STALE, "stale scope context");
        raise(FORT_SCOPE_ARGUMENT, "unknown scope context");
    }
    return it->second.get();
}

Context *live_context(fort_scope_t handle) {
    Context *c = find_context(handle);
    if (c->poisoned || c->domain->poisoned)
        raise(FORT_SCOPE_EXECUTION, "context poisoned by an earlier execution failure; unsafe replay prohibited");
    return c;
}

Domain *find_domain(fort_scope_domain_t handle) {
    auto it = g_domains.find(handle);
    if (it == g_domains.end()) {
        if (g_retired.count(handle)) raise(FORT_SCOPE_STALE, "stale residency domain");
        raise(FORT_SCOPE_ARGUMENT, "unknown residency domain");
    }
    return it->second.get();
}

Buffer *find_buffer(Context *c, fort_buffer_t handle) {
    auto it = c->domain->buffers.find(handle);
    if (it == c->domain->buffers.end())
        raise(FORT_SCOPE_STALE, g_retired.count(handle) ? "stale buffer handle" : "unknown or foreign buffer handle");
    return it->second.get();
}

void poison(Context *c, const std::string &message) {
    c->poisoned = true;
    c->domain->poisoned = true;
    raise(FORT_SCOPE_EXECUTION, message + "; unsafe replay prohibited");
}

// The device is brought up the first time a context needs it: registration, host
// access, observation of host-current arrays and closing never touch it.
void ensure_stream(Context *c) {
    if (c->stream_ready) return;
    trace_line(c, "initialize", 0, 0);
    if (!Backend::select(c->domain->device)) raise(FORT_SCOPE_RESOURCE, "cannot select device: " + Backend::last_error());
    if (!Backend::make_stream(&c->stream)) raise(FORT_SCOPE_RESOURCE, "cannot create stream: " + Backend::last_error());
    c->stream_ready = true;
}

// Arrays of 1 MiB or more are pinned in place (and mapped) the first time the
// device is about to use them, so that their copies run at DMA speed; the CPU
// test backend pins only when a test asks.
void pin_for_device(Context *c, Buffer *b) {
    if (b->pin_tried) return;
    b->pin_tried = true;
    const bool pinning = c->pin_host < 0 ? env_flag("FORT_SCOPE_PIN_HOST", true) : c->pin_host != 0;
    if (b->bytes < (Backend::cpu ? size_t(0) : size_t(1) << 20) || !b->bytes || !pinning) return;
    ensure_stream(c);
    const int how = Backend::pin(b->host, b->bytes, &b->mapped);
    b->pinned_host = how != 0;
    b->pinned_here = how == 1;
}

void ensure_copy_streams(Context *c) {
    ensure_stream(c);
    if (c->copies_ready) return;
    if (!Backend::make_stream(&c->copy_in)) raise(FORT_SCOPE_RESOURCE, "cannot create stream: " + Backend::last_error());
    if (!Backend::make_stream(&c->copy_out)) {
        Backend::destroy_stream(c->copy_in);
        raise(FORT_SCOPE_RESOURCE, "cannot create stream: " + Backend::last_error());
    }
    c->copies_ready = true;
}

// ---- effects --------------------------------------------------------------------------------

struct Effects {
    Region reads, writes, overwrites; // writes include overwrites
};

Box section_box(const Buffer *b, const fort_scope_section &s) {
    if (!s.lower || !s.upper) raise(FORT_SCOPE_ARGUMENT, "null section coordinates");
    Box box;
    box.rank = b->rank;
    for (int d = 0; d < b->rank; ++d) {
        box.lo[d] = s.lower[d];
        box.hi[d] = s.upper[d];
        if (box.hi[d] < box.lo[d] || box.hi[d] > b->extents[d]) raise(FORT_SCOPE_ARGUMENT, "section outside its array");
    }
    return box;
}

Effects effects_of(const Buffer *b, const fort_scope_access &a) {
    if (a.flags & ~uint32_t(7)) raise(FORT_SCOPE_ARGUMENT, "unknown access flags");
    auto list = [&](size_t count, const fort_scope_section *s, Region &into) {
        if (count > kRegionLimit || (count && !s)) raise(FORT_SCOPE_ARGUMENT, "section list exceeds the bounded interface");
        for (size_t n = 0; n < count; ++n) into.add(section_box(b, s[n]));
    };
    Effects e;
    if (a.flags & FORT_SCOPE_READ_ALL) e.reads.add(b->full());
    else list(a.read_count, a.reads, e.reads);
    if (a.flags & FORT_SCOPE_WRITE_ALL) e.writes.add(b->full());
    else list(a.write_count, a.writes, e.writes);
    if (a.flags & FORT_SCOPE_OVERWRITE_ALL) e.overwrites.add(b->full());
    else list(a.overwrite_count, a.overwrites, e.overwrites);
    e.writes.add(e.overwrites);
    if (!e.overwrites.empty()) {
        // the definition the access would leave must stay exact: refused here, before anything changes
        Region defined = b->defined;
        defined.add(e.overwrites);
        if (!defined.fits()) raise(FORT_SCOPE_BOUNDARY, "the array's defined sections would exceed the tracked limit");
    }
    return e;
}

// Values a task needs current where it runs: what it reads, and what it may
// write without overwriting (the unwritten part keeps its old values).
Region needed(const Buffer *b, const Effects &e) {
    Region need = e.reads;
    Region partial = e.writes;
    partial.remove(e.overwrites);
    need.add(partial);
    return b->defined.clip(need);
}

void check_initialized(const Buffer *b, const Effects &e) {
    for (const auto &box : e.reads.boxes)
        if (!b->defined.covers(box))
            raise(FORT_SCOPE_UNINITIALIZED, "a task reads array values that were never defined");
}

// ---- transfers ------------------------------------------------------------------------------

Box bounding(const Region &r);

// The region actually moved for a needed transfer `r`: the whole array, the
// whole planes (every dimension but the last complete) spanning `r`, or the
// bounding box of `r`, the first of these that moves at most a quarter more
// bytes, holds only defined cells and cannot overwrite values only the
// destination holds; `r` itself otherwise. Fewer, larger (and, for whole planes, contiguous) copies keep the
// copy engines busy instead of the host.
Region widened(const Buffer *b, const Region &r, bool to_device) {
    if (r.boxes.size() <= 1) return r;
    Region only_destination = to_device ? b->device_valid : b->host_valid;
    only_destination.remove(to_device ? b->host_valid : b->device_valid);
    only_destination = b->physical.clip(only_destination);
    const size_t need = r.volume();
    Box planes = bounding(r);
    for (int d = 0; d + 1 < planes.rank; ++d) {
        planes.lo[d] = 0;
        planes.hi[d] = b->extents[d];
    }
    const Box candidates[3] = {b->full(), planes, bounding(r)};
    for (const Box &cand : candidates) {
        if ((double)cand.volume() > 1.25 * (double)need) continue;
        if (!b->defined.covers(cand)) continue;  // undefined cells are never moved
        Region clash = only_destination.clip(cand);
        clash.remove(r);
        if (!clash.empty()) continue;
        Region w;
        w.add(cand);
        return w;
    }
    return r;
}

void copy_region(Context *c, Buffer *b, const Region &r, bool to_device, Stream stream) {
    Domain *d = c->domain;
    const CopyPlan plan = b->plan();
    for (const auto &box : r.boxes) {
        const size_t bytes = box.volume() * b->elem;
        if (!bytes) continue;
        bool good = to_device ? Backend::copy(b->device, b->host, plan, box, true, stream)
                              : Backend::copy(b->host, b->device, plan, box, false, stream);
        if (!good) poison(c, std::string("transfer failed: ") + Backend::last_error());
        if (to_device) {
            d->stats.uploads++;
            d->stats.upload_bytes += bytes;
            trace_line(c, "upload", b->handle, bytes);
        } else {
            d->stats.downloads++;
            d->stats.download_bytes += bytes;
            trace_line(c, "download", b->handle, bytes);
        }
    }
}

void copy_region(Context *c, Buffer *b, const Region &r, bool to_device) { copy_region(c, b, r, to_device, c->stream); }

// The element range [lo, hi) of a region that is one run of the array's
// elements in memory order, if it is: its boxes are disjoint, so they tile the
// run from their lowest to their highest element exactly when their volumes
// add up to its length.
bool as_interval(const Buffer *b, const Region &r, size_t &lo, size_t &hi) {
    if (r.empty()) return false;
    lo = SIZE_MAX;
    hi = 0;
    size_t volume = 0;
    for (const Box &box : r.boxes) {
        size_t first = 0, last = 0, stride = 1;
        for (int e = 0; e < box.rank; ++e) {
            first += box.lo[e] * stride;
            last += (box.hi[e] - 1) * stride;
            stride *= b->extents[e];
        }
        lo = std::min(lo, first);
        hi = std::max(hi, last + 1);
        volume += box.volume();
    }
    return volume == hi - lo;
}

// Boxes tiling elements [lo, hi) of a block of dimension d (offsets relative to
// the block's start; `at` holds the indices of the dimensions above d).
void tile_interval(const Buffer *b, size_t lo, size_t hi, int d, Box &at, Region &out) {
    if (lo >= hi) return;
    size_t step = 1;
    for (int e = 0; e < d; ++e) step *= b->extents[e];
    auto whole_blocks = [&](size_t i0, size_t i1) {
        Box box = at;
        for (int e = 0; e < d; ++e) {
            box.lo[e] = 0;
            box.hi[e] = b->extents[e];
        }
        box.lo[d] = i0;
        box.hi[d] = i1;
        out.boxes.push_back(box);
    };
    if (d == 0) return whole_blocks(lo, hi);
    size_t a = lo / step;
    const size_t z = hi / step, head = lo % step, tail = hi % step;
    if (a == z) {
        at.lo[d] = a;
        at.hi[d] = a + 1;
        return tile_interval(b, head, tail, d - 1, at, out);
    }
    if (head) {
        at.lo[d] = a;
        at.hi[d] = a + 1;
        tile_interval(b, head, step, d - 1, at, out);
        ++a;
    }
    if (a < z) whole_blocks(a, z);
    if (tail) {
        at.lo[d] = z;
        at.hi[d] = z + 1;
        tile_interval(b, 0, tail, d - 1, at, out);
    }
}

Region interval_region(const Buffer *b, size_t lo, size_t hi) {
    Region out;
    Box at;
    at.rank = b->rank;
    tile_interval(b, lo, hi, b->rank - 1, at, out);
    return out;
}

// A slab upload of a pinned array (a run of 8 MiB or more) ends on a 2 MiB
// boundary of the host array, where the elements up to it are current on the
// host: the next slab's upload then starts on the boundary and goes as one copy
// at full rate (from an unaligned host start, with both directions busy, a copy
// runs at about two thirds of the rate, and splitting it at the boundary costs a
// copy). On GB300 this took the 512 x 512 x 128 end-to-end step from 12.1 to
// 11.6 ms.
Region to_host_boundary(const Buffer *b, const Region &r) {
    constexpr size_t kAlign = size_t(2) << 20;
    size_t lo, hi;
    if (!b->mapped || !as_interval(b, r, lo, hi) || (hi - lo) * b->elem < 4 * kAlign) return r;
    const uintptr_t end = reinterpret_cast<uintptr_t>(b->host) + hi * b->elem;
    const size_t pad = (kAlign - end % kAlign) % kAlign;
    if (!pad || pad % b->elem) return r;
    const size_t top = std::min(b->full().volume(), hi + pad / b->elem);
    if (top <= hi) return r;
    const Region more = interval_region(b, hi, top);
    Region stale = more;
    stale.remove(b->host_valid);
    Region undefined = more;
    undefined.remove(b->defined);
    if (!stale.empty() || !undefined.empty()) return r;
    Region out = r;
    out.boxes.insert(out.boxes.end(), more.boxes.begin(), more.boxes.end());
    return out;
}

// A region that is one run of elements goes as one copy; others box by box.
void copy_run(Context *c, Buffer *b, const Region &r, bool to_device, Stream stream) {
    size_t lo, hi;
    if (r.boxes.size() < 2 || !as_interval(b, r, lo, hi)) return copy_region(c, b, r, to_device, stream);
    char *host = static_cast<char *>(b->host) + lo * b->elem;
    char *device = static_cast<char *>(b->device) + lo * b->elem;
    const size_t bytes = (hi - lo) * b->elem;
    const bool good = to_device ? Backend::linear(device, host, bytes, true, host, stream)
                                : Backend::linear(host, device, bytes, false, host, stream);
    if (!good) poison(c, std::string("transfer failed: ") + Backend::last_error());
    Domain *d = c->domain;
    if (to_device) {
        d->stats.uploads++;
        d->stats.upload_bytes += bytes;
        trace_line(c, "upload", b->handle, bytes);
    } else {
        d->stats.downloads++;
        d->stats.download_bytes += bytes;
        trace_line(c, "download", b->handle, bytes);
    }
}

void wait_stream(Context *c) {
    if (!c->stream_ready) return;
    c->domain->stats.waits++;
    c->completion.stream_waits++;
    if (!Backend::sync(c->stream)) poison(c, std::string("device work failed: ") + Backend::last_error());
    c->complete_serial = c->token_serial;
    for (auto &t : c->tokens) c->spare_events.push_back(t.event);
    c->tokens.clear();
    c->untracked = false;
}

// ---- completion tokens ----------------------------------------------------------------------
// A token is an event recorded on the context stream after work that reads or
// writes host memory. Host accesses wait on the token of the arrays they touch,
// and only where they overlap what that work reads or writes, instead of on the
// whole stream.

uint64_t record_token(Context *c) {
    ensure_stream(c);
    Backend::Event e;
    if (!c->spare_events.empty()) {
        e = c->spare_events.back();
        c->spare_events.pop_back();
        c->completion.reused_events++;
    } else {
        if (!Backend::make_event(&e)) poison(c, std::string("event creation failed: ") + Backend::last_error());
        c->completion.created_events++;
    }
    if (!Backend::record(e, c->stream)) poison(c, std::string("event record failed: ") + Backend::last_error());
    c->completion.event_records++;
    c->tokens.push_back({++c->token_serial, e});
    return c->token_serial;
}

bool token_done(Context *c, uint64_t serial) {
    while (serial > c->complete_serial && !c->tokens.empty() && c->tokens.front().serial <= serial) {
        c->completion.event_queries++;
        if (!Backend::query(c->tokens.front().event)) return false;
        c->complete_serial = c->tokens.front().serial;
        c->spare_events.push_back(c->tokens.front().event);
        c->tokens.pop_front();
    }
    return serial <= c->complete_serial;
}

void wait_token(Context *c, uint64_t serial) {
    c->domain->stats.waits++;
    c->completion.event_waits++;
    for (auto &t : c->tokens)
        if (t.serial == serial && !Backend::wait_event(t.event))
            poison(c, std::string("device work failed: ") + Backend::last_error());
    while (!c->tokens.empty() && c->tokens.front().serial <= serial) {
        c->spare_events.push_back(c->tokens.front().event);
        c->tokens.pop_front();
    }
    if (serial > c->complete_serial) c->complete_serial = serial;
}

// Record that work up to `serial` reads / writes these host sections of `b`.
void hold_host(Buffer *b, const Region &reading, const Region &writing, uint64_t serial) {
    b->host_reading.add(reading);
    b->host_writing.add(writing);
    b->host_token = serial;
    if (!b->host_reading.fits() || !b->host_writing.fits()) {  // keep the bookkeeping small: the whole array
        b->host_reading.clear();
        b->host_reading.add(b->full());
        b->host_writing.clear();
        b->host_writing.add(b->full());
    }
}

void free_host(Buffer *b) {
    b->host_reading.clear();
    b->host_writing.clear();
    b->host_token = 0;
}

void release_events(Context *c) {
    for (auto &t : c->tokens) Backend::destroy_event(t.event);
    for (auto e : c->spare_events) Backend::destroy_event(e);
    c->tokens.clear();
    c->spare_events.clear();
}

Box bounding(const Region &r) {
    Box box = r.boxes.front();
    for (const auto &e : r.boxes)
        for (int d = 0; d < box.rank; ++d) {
            box.lo[d] = std::min(box.lo[d], e.lo[d]);
            box.hi[d] = std::max(box.hi[d], e.hi[d]);
        }
    return box;
}

void flush(Context *c);

// Install an array's new coherence sets. When one of them would exceed the
// rectangle limit, reconcile instead: bring both copies up to date everywhere
// values are defined (copying exactly what each side lacks under the new
// sets), then track each side as the whole array. A definition set that is
// still too fragmented is widened to its bounding box.
void settle(Context *c, Buffer *b, Region defined, Region host, Region device) {
    Region physical = b->physical;
    physical.add(defined);
    if (!physical.fits()) {  // only publication reads it: a hull over-approximates harmlessly
        const Box hull = bounding(physical);
        physical.clear();
        physical.add(hull);
    }
    b->physical = std::move(physical);
    if (defined.fits() && host.fits() && device.fits()) {
        b->defined = std::move(defined);
        b->host_valid = std::move(host);
        b->device_valid = std::move(device);
        return;
    }
    flush(c);
    if (b->device) {
        ensure_stream(c);
        Region down = b->physical.clip(device);
        down.remove(host);
        copy_region(c, b, down, false);
        Region up = b->physical.clip(host);
        up.remove(device);
        copy_region(c, b, up, true);
        wait_stream(c);
        b->device_valid.clear();
        b->device_valid.add(b->full());
    } else {
        b->device_valid.clear();
    }
    b->host_valid.clear();
    b->host_valid.add(b->full());
    if (!defined.fits()) {
        const Box hull = bounding(defined);
        defined.clear();
        defined.add(hull);
    }
    b->defined = std::move(defined);
    c->domain->stats.reconciliations++;
}

// ---- device storage and the budget ---------------------------------------------------------

void publish_buffer(Context *c, Buffer *b) {
    if (!b->device) return;
    Region dirty = b->physical.clip(b->device_valid);
    dirty.remove(b->host_valid);
    if (dirty.empty()) return;
    ensure_stream(c);
    const Region moved = widened(b, dirty, false);
    copy_region(c, b, moved, false);
    Region host = b->host_valid;
    host.add(dirty);
    host.add(b->device_valid.clip(moved));
    settle(c, b, b->defined, host, b->device_valid);
}

void release_mirror(Context *c, Buffer *b) {
    if (!b->device) return;
    Backend::free(b->device, c->stream);
    b->device = nullptr;
    c->domain->device_bytes -= b->bytes;
    c->domain->stats.allocated_bytes -= b->bytes;  // the bytes mirrors hold now; the peak keeps the maximum
    b->device_valid.clear();
}

size_t claimed(const Domain *d) { return d->device_bytes + d->scratch_bytes + d->workspace_bytes; }

// Values on the device that the host does not hold: evicting the mirror costs a download.
bool dirty_mirror(const Buffer *b) {
    Region dirty = b->physical.clip(b->device_valid);
    dirty.remove(b->host_valid);
    return !dirty.empty();
}

// Said once per shared domain (the resident application's), in the reference's
// words: what exceeding the device budget costs from now on.
void budget_warning(Context *c, const char *consequence) {
    Domain *d = c->domain;
    if (c->private_domain || d->budget_warned) return;
    d->budget_warned = true;
    std::fprintf(stderr, "Resident domain: the arrays in use exceed the device budget of %zu bytes; %s.\n", d->budget,
                 consequence);
}

// Make room for `bytes` more, evicting mirrors that are not in `keep`, not
// prepared and not used by queued tasks: clean ones (dropped without a
// download) before dirty ones, each kind least recently used first, ties by
// handle.
void make_room(Context *c, size_t bytes, const std::set<uint64_t> &keep);

// Refuse a footprint that cannot fit even after evicting everything evictable,
// before anything changes and before the device is brought up.
void require_fit(Context *c, size_t bytes, const std::set<uint64_t> &keep) {
    Domain *d = c->domain;
    if (!d->budget_set || claimed(d) + bytes <= d->budget) return;
    size_t evictable = 0;
    for (auto &kv : d->buffers) {
        Buffer *b = kv.second.get();
        if (b->device && !keep.count(b->handle) && b->prepared == Buffer::NONE) evictable += b->bytes;
    }
    if (claimed(d) - evictable + bytes > d->budget) {
        budget_warning(c, "loop nests whose arrays do not fit together run on the host");
        raise(FORT_SCOPE_RESOURCE, "device budget too small for the task footprint");
    }
}

void make_room(Context *c, size_t bytes, const std::set<uint64_t> &keep) {
    Domain *d = c->domain;
    if (!d->budget_set) return;
    if (claimed(d) + bytes <= d->budget) return;
    // impossible even after evicting everything evictable: fail before touching anything
    size_t evictable = 0;
    for (auto &kv : d->buffers) {
        Buffer *b = kv.second.get();
        if (b->device && !keep.count(b->handle) && b->prepared == Buffer::NONE) evictable += b->bytes;
    }
    if (claimed(d) - evictable + bytes > d->budget) {
        budget_warning(c, "loop nests whose arrays do not fit together run on the host");
        raise(FORT_SCOPE_RESOURCE, "device budget too small for the task footprint");
    }
    if (!c->pending.empty()) {
        d->residency.pressure_flushes++;
        flush(c);
    }
    while (claimed(d) + bytes > d->budget) {
        Buffer *victim = nullptr;
        bool victim_dirty = false;
        for (auto &kv : d->buffers) {
            Buffer *b = kv.second.get();
            if (!b->device || keep.count(b->handle) || b->prepared != Buffer::NONE || b->queued) continue;
            const bool dirty = dirty_mirror(b);
            if (!victim || std::make_tuple(dirty, b->last_use, b->handle) <
                               std::make_tuple(victim_dirty, victim->last_use, victim->handle)) {
                victim = b;
                victim_dirty = dirty;
            }
        }
        if (!victim) raise(FORT_SCOPE_RESOURCE, "device budget exhausted by arrays in use");
        if (victim_dirty) {
            Region dirty = victim->physical.clip(victim->device_valid);
            dirty.remove(victim->host_valid);
            d->residency.dirty_evictions++;
            d->residency.dirty_download_bytes += dirty.volume() * victim->elem;
            publish_buffer(c, victim);
            wait_stream(c);
        }
        budget_warning(c, "the least recently used ones now move back to the host");
        d->residency.evictions++;
        d->residency.evicted_bytes += victim->bytes;
        trace_line(c, "evict", victim->handle, victim->bytes);
        release_mirror(c, victim);
    }
}

bool in_place_allowed() {
    static const bool on = env_flag("FORT_SCOPE_HOST_IN_PLACE", true);
    return on;
}

void reserve(Context *c, const std::vector<Buffer *> &list, bool allow_in_place) {
    std::set<uint64_t> keep;
    size_t need = 0;
    for (Buffer *b : list) keep.insert(b->handle);
    size_t missing = 0;  // arrays without a mirror; one that goes in place later only makes this smaller
    for (Buffer *b : list)
        if (!b->device && !(b->mapped && b->host_rounds >= 1)) missing += b->bytes;
    require_fit(c, missing, keep);
    for (Buffer *b : list) {
        pin_for_device(c, b);
        b->in_place = allow_in_place && in_place_allowed() && b->mapped && b->prepared == Buffer::NONE &&
                      b->host_touched && b->host_rounds >= 1;
        if (!b->device && !b->in_place) need += b->bytes;
    }
    Domain *d = c->domain;
    if (need) {
        ensure_stream(c);
        make_room(c, need, keep);
    }
    std::set<uint64_t> seen;
    size_t reused = 0;
    for (Buffer *b : list) {
        b->last_use = ++d->tick;
        if (!seen.insert(b->handle).second) continue;  // a repeated array is one resource
        if (b->in_place || !b->bytes) continue;  // mapped host array, or an empty one: no storage
        if (b->device) {
            ++reused;
            continue;
        }
        if (!Backend::alloc(&b->device, b->bytes, c->stream)) {
            b->device = nullptr;
            raise(FORT_SCOPE_RESOURCE, "device allocation failed: " + Backend::last_error());
        }
        d->device_bytes += b->bytes;
        d->stats.allocations++;
        d->stats.allocated_bytes += b->bytes;
        if (d->device_bytes > d->stats.peak_device_bytes) d->stats.peak_device_bytes = d->device_bytes;
        if (claimed(d) > d->peak_total_bytes) d->peak_total_bytes = claimed(d);
        b->device_valid.clear();
    }
    // counted once the batch holds its storage: a refused reservation changes no counter
    d->residency.reserve_batches++;
    d->residency.requested_resources += seen.size();
    d->residency.reuse_hits += reused;
}

// ---- the task queue ------------------------------------------------------------------------

uint64_t fnv1a(uint64_t h, const void *data, size_t n) {
    const unsigned char *p = static_cast<const unsigned char *>(data);
    for (size_t i = 0; i < n; ++i) {
        h ^= p[i];
        h *= 1099511628211ULL;
    }
    return h;
}

void launch_direct(Context *c, std::vector<Task> &tasks) {
    for (auto &t : tasks) {
        trace_line(c, "launch", 0, 0, &t.origin);
        if (!Backend::launch(t.spec, c->stream)) poison(c, std::string("kernel launch failed: ") + Backend::last_error());
    }
    c->queue_stats.direct_submissions++;
    c->queue_stats.direct_kernels += tasks.size();
}

void submit(Context *c, std::vector<Task> &tasks, uint64_t key) {
    ensure_stream(c);
    Domain *d = c->domain;
    d->stats.launches += tasks.size();
    c->graph_stats.submissions++;
    c->graph_stats.logical_kernels += tasks.size();
    if (!c->graphs_enabled) {
        launch_direct(c, tasks);
        return;
    }
    CachedGraph &g = c->graphs[key];
    bool same_topology = g.functions.size() == tasks.size();
    for (size_t n = 0; same_topology && n < tasks.size(); ++n)
        same_topology = g.functions[n] == tasks[n].spec.function && g.argument_counts[n] == tasks[n].values.size();
    if (!same_topology) {
        if (g.graph) {
            Backend::graph_destroy(g.graph);
            g.graph = nullptr;
            c->graph_stats.rebuilds++;
            c->graph_stats.destructions++;
            c->graph_stats.live_graphs--;
        }
        g.functions.clear();
        g.argument_counts.clear();
        for (auto &t : tasks) {
            g.functions.push_back(t.spec.function);
            g.argument_counts.push_back(t.values.size());
        }
        g.reached = 0;
    }
    g.reached++;
    if (g.reached == 1) {
        // first reach: direct launches, as a warm-up of the sequence
        launch_direct(c, tasks);
        return;
    }
    std::vector<LaunchSpec> specs;
    for (auto &t : tasks) specs.push_back(t.spec);
    if (!g.graph) {
        Backend::Graph *built = nullptr;
        if (!Backend::graph_build(&built, specs)) {
            c->queue_stats.graph_resource_fallbacks++;
            g.reached = 0;
            launch_direct(c, tasks);
            return;
        }
        g.graph = built;
        g.specs = specs;
        g.values.clear();
        for (auto &t : tasks) g.values.push_back(t.values);
        c->graph_stats.creations++;
        c->graph_stats.instantiations++;
        c->graph_stats.live_graphs++;
    } else {
        for (size_t n = 0; n < tasks.size(); ++n) {
            const LaunchSpec &k = tasks[n].spec;
            const LaunchSpec &old = g.specs[n];
            bool changed = std::memcmp(k.grid, old.grid, sizeof k.grid) || std::memcmp(k.block, old.block, sizeof k.block) ||
                           k.shared_bytes != old.shared_bytes || g.values[n] != tasks[n].values;
            if (!changed) continue;
            if (!Backend::graph_update(g.graph, n, k)) poison(c, std::string("graph update failed: ") + Backend::last_error());
            c->graph_stats.parameter_updates++;
            g.values[n] = tasks[n].values;
            g.specs[n] = k;
        }
        c->graph_stats.replays++;
    }
    // the stored specs point into g.values; rebind before launch
    for (size_t n = 0; n < tasks.size(); ++n) {
        g.specs[n].arguments.clear();
        for (auto &v : g.values[n]) g.specs[n].arguments.push_back(v.data());
    }
    trace_line(c, "graph_submit", 0, tasks.size());
    for (size_t n = 0; n < tasks.size(); ++n) trace_line(c, "graph_kernel", 0, 0, &tasks[n].origin);
    if (!Backend::graph_launch(g.graph, g.specs, c->stream))
        poison(c, std::string("graph launch failed: ") + Backend::last_error());
}

// A group of kernels whose argument values live in the caller's storage for
// this call only (fort_scope_graph_submit_v1, fort_scope_graph_execute_v1):
// cached by the caller's key like the queue's sequences. The first reach of a
// sequence runs as direct launches, the second builds and instantiates its
// graph (the node parameters are copied then), later reaches copy every
// node's arguments into the instantiated graph again and replay it; a new
// sequence of functions under the key replaces the graph.
void submit_group(Context *c, const std::vector<LaunchSpec> &specs, uint64_t key) {
    ensure_stream(c);
    c->domain->stats.launches += specs.size();
    c->graph_stats.submissions++;
    c->graph_stats.logical_kernels += specs.size();
    std::vector<Task> direct(specs.size());
    for (size_t n = 0; n < specs.size(); ++n) direct[n].spec = specs[n];
    if (!c->graphs_enabled) {
        launch_direct(c, direct);
        return;
    }
    CachedGraph &g = c->group_graphs[key];
    bool same_topology = g.functions.size() == specs.size();
    for (size_t n = 0; same_topology && n < specs.size(); ++n)
        same_topology = g.functions[n] == specs[n].function && g.argument_counts[n] == specs[n].arguments.size();
    if (!same_topology) {
        if (g.graph) {
            Backend::graph_destroy(g.graph);
            g.graph = nullptr;
            c->graph_stats.rebuilds++;
            c->graph_stats.destructions++;
            c->graph_stats.live_graphs--;
        }
        g.functions.clear();
        g.argument_counts.clear();
        for (const auto &k : specs) {
            g.functions.push_back(k.function);
            g.argument_counts.push_back(k.arguments.size());
        }
        g.reached = 0;
    }
    if (++g.reached == 1) {
        trace_line(c, "graph_warmup_direct", 0, specs.size());
        launch_direct(c, direct);
        return;
    }
    if (!g.graph) {
        Backend::Graph *built = nullptr;
        if (!Backend::graph_build(&built, specs)) {
            c->queue_stats.graph_resource_fallbacks++;
            g.reached = 0;
            launch_direct(c, direct);
            return;
        }
        g.graph = built;
        c->graph_stats.creations++;
        c->graph_stats.instantiations++;
        c->graph_stats.live_graphs++;
    } else {
        for (size_t n = 0; n < specs.size(); ++n) {
            if (!Backend::graph_update(g.graph, n, specs[n]))
                poison(c, std::string("graph update failed: ") + Backend::last_error());
            c->graph_stats.parameter_updates++;
        }
        c->graph_stats.replays++;
    }
    trace_line(c, "graph_submit", 0, specs.size());
    for (size_t n = 0; n < specs.size(); ++n) trace_line(c, "graph_kernel", 0, 0);
    if (!Backend::graph_launch(g.graph, specs, c->stream))
        poison(c, std::string("graph launch failed: ") + Backend::last_error());
}

void flush(Context *c) {
    c->queued_before.clear();
    if (c->pending.empty()) return;
    std::vector<Task> tasks;
    tasks.swap(c->pending);
    c->pending_threads = 0;
    uint64_t key = 14695981039346656037ULL;
    for (auto &t : tasks) key = fnv1a(key, &t.code_key, sizeof t.code_key);
    for (auto &t : tasks)
        for (uint64_t h : t.buffers) {
            auto it = c->domain->buffers.find(h);
            if (it != c->domain->buffers.end()) it->second->queued--;
        }
    c->queue_stats.submissions++;
    c->queue_stats.pending_tasks = 0;
    trace_line(c, "flush", 0, tasks.size());
    submit(c, tasks, key);
    if (!c->awaiting_token.empty()) {  // kernels on mapped host arrays read and write them in place
        const uint64_t token = record_token(c);
        for (uint64_t h : c->awaiting_token) {
            auto it = c->domain->buffers.find(h);
            if (it == c->domain->buffers.end()) continue;
            Buffer *b = it->second.get();
            Region whole;
            whole.add(b->full());
            hold_host(b, whole, whole, token);
            b->awaits_token = false;
        }
        c->awaiting_token.clear();
    }
}

// Validate and apply the effects of one device task transactionally: nothing is
// changed unless every binding passes.
struct Bound {
    Buffer *buffer;
    Effects effects;
};

std::vector<Bound> bind_all(Context *c, const fort_scope_plan_binding *bindings, size_t count) {
    if (count && !bindings) raise(FORT_SCOPE_ARGUMENT, "null bindings");
    std::vector<Bound> out;
    std::set<uint64_t> seen;
    for (size_t n = 0; n < count; ++n) {
        Buffer *b = find_buffer(c, bindings[n].buffer);
        if (!seen.insert(b->handle).second) raise(FORT_SCOPE_ALIAS, "a task binds one array twice");
        if (b->prepared != Buffer::NONE) raise(FORT_SCOPE_STATE, "array already has a prepared access");
        Effects e = effects_of(b, bindings[n].access);
        check_initialized(b, e);
        out.push_back({b, std::move(e)});
    }
    return out;
}

void device_acquire(Context *c, std::vector<Bound> &bound) {
    std::vector<std::pair<Buffer *, Region>> uploads;
    for (auto &x : bound) {
        Buffer *b = x.buffer;
        Region up = needed(b, x.effects);
        up.remove(b->device_valid);
        if (!up.empty()) {
            const Region moved = widened(b, up, true);
            copy_region(c, b, moved, true);
            Region device = b->device_valid;
            device.add(up);
            device.add(b->host_valid.clip(moved));
            settle(c, b, b->defined, b->host_valid, device);
            uploads.emplace_back(b, moved);
        }
    }
    if (uploads.empty()) return;
    const uint64_t token = record_token(c);  // one token for the whole batch
    for (auto &u : uploads) hold_host(u.first, u.second, Region{}, token);
}

void device_commit(Context *c, Buffer *b, const Region &writes, const Region &overwrites) {
    Region defined = b->defined, host = b->host_valid, device = b->device_valid;
    device.add(writes);
    host.remove(writes);
    defined.add(overwrites);
    settle(c, b, std::move(defined), std::move(host), std::move(device));
    b->last_use = ++c->domain->tick;
}

// A host access orders after the work it conflicts with and nothing else:
// queued tasks on its arrays are submitted first (they may write what it
// reads); values it reads that only the device holds are downloaded and waited
// for; otherwise it waits on an array's completion token only where it writes
// what in-flight work reads from the host copy, or touches what in-flight work
// writes into it. Work without tokens (kernels launched without bindings) is
// waited for as a whole.
void host_acquire(Context *c, std::vector<Bound> &bound) {
    for (auto &x : bound)
        if (x.buffer->queued || x.buffer->awaits_token) {
            flush(c);
            break;
        }
    bool downloaded = false;
    for (auto &x : bound) {
        Region down = needed(x.buffer, x.effects);
        down.remove(x.buffer->host_valid);
        if (!down.empty()) {
            ensure_stream(c);
            const Region moved = widened(x.buffer, down, false);
            copy_region(c, x.buffer, moved, false);
            Region host = x.buffer->host_valid;
            host.add(down);
            host.add(x.buffer->device_valid.clip(moved));
            settle(c, x.buffer, x.buffer->defined, host, x.buffer->device_valid);
            downloaded = true;
        }
    }
    if (downloaded || c->untracked) {
        wait_stream(c);
        for (auto &x : bound) free_host(x.buffer);
        return;
    }
    bool waited = false;
    for (auto &x : bound) {
        Buffer *b = x.buffer;
        if (!b->host_token) continue;
        if (token_done(c, b->host_token)) {
            free_host(b);
            continue;
        }
        Region touched = needed(b, x.effects);
        touched.add(x.effects.writes);
        bool conflict = !b->host_writing.clip(touched).empty();
        for (const Box &w : x.effects.writes.boxes) conflict = conflict || b->host_reading.intersects(w);
        if (conflict) {
            wait_token(c, b->host_token);
            free_host(b);
            waited = true;
        }
    }
    if (!waited) c->completion.independent_host_tasks++;
}

void host_commit(Context *c, Buffer *b, const Region &writes, const Region &overwrites) {
    Region defined = b->defined, host = b->host_valid, device = b->device_valid;
    host.add(writes);
    device.remove(writes);
    defined.add(overwrites);
    settle(c, b, std::move(defined), std::move(host), std::move(device));
}

LaunchSpec spec_of(const fort_scope_kernel_v1 &k) {
    if (k.version != FORT_SCOPE_GRAPH_ABI_VERSION) raise(FORT_SCOPE_ARGUMENT, "unknown kernel record version");
    if (k.reserved) raise(FORT_SCOPE_ARGUMENT, "reserved kernel record field is not zero");
    if (!k.function) raise(FORT_SCOPE_ARGUMENT, "null kernel function");
    if (k.argument_count > 384) raise(FORT_SCOPE_ARGUMENT, "too many kernel arguments");
    if (k.argument_count && !k.arguments) raise(FORT_SCOPE_ARGUMENT, "null kernel arguments");
    for (int d = 0; d < 3; ++d)
        if (!k.grid[d] || !k.block[d]) raise(FORT_SCOPE_ARGUMENT, "empty launch dimension");
    if ((uint64_t)k.block[0] * k.block[1] * k.block[2] > 1024) raise(FORT_SCOPE_ARGUMENT, "block larger than 1024 threads");
    LaunchSpec s;
    s.function = k.function;
    for (int d = 0; d < 3; ++d) {
        s.grid[d] = k.grid[d];
        s.block[d] = k.block[d];
    }
    s.shared_bytes = k.shared_bytes;
    return s;
}

Task make_task(uint64_t code_key, const fort_scope_kernel_v1 &k, const size_t *sizes) {
    Task t;
    t.code_key = code_key;
    t.spec = spec_of(k);
    if (k.argument_count && !sizes) raise(FORT_SCOPE_ARGUMENT, "argument sizes are required");
    size_t total = 0;
    for (size_t n = 0; n < k.argument_count; ++n) {
        if (!sizes[n] || !k.arguments[n]) raise(FORT_SCOPE_ARGUMENT, "empty kernel argument");
        total += sizes[n];
        const unsigned char *v = static_cast<const unsigned char *>(k.arguments[n]);
        t.values.emplace_back(v, v + sizes[n]);
    }
    if (total > 32764) raise(FORT_SCOPE_ARGUMENT, "kernel arguments exceed the launch parameter space");
    for (auto &v : t.values) t.spec.arguments.push_back(v.data());
    t.threads = (uint64_t)k.grid[0] * k.grid[1] * k.grid[2] * k.block[0] * k.block[1] * k.block[2];
    return t;
}

// A device use of an array: count consecutive uses preceded by host access.
void note_device_use(Buffer *b) {
    b->host_rounds = b->host_touched ? b->host_rounds + 1 : 0;
    b->host_touched = false;
    b->in_place = false;
}

void accept(Context *c, Task &&task, std::vector<Bound> &bound) {
    for (auto &x : bound)
        if (!x.buffer->device && !x.buffer->in_place && x.buffer->bytes)
            raise(FORT_SCOPE_STATE, "task binds an array whose device storage is not reserved");
    ensure_stream(c);
    for (auto &x : bound) {
        const Buffer *b = x.buffer;
        c->queued_before.emplace(b->handle, Context::Before{b->defined, b->host_valid, b->device_valid, b->physical,
                                                             b->host_touched, b->host_rounds});
    }
    std::vector<Bound> mirrored, in_place;
    for (auto &x : bound) (x.buffer->in_place ? in_place : mirrored).push_back(x);
    device_acquire(c, mirrored);
    // arrays accessed in place: the host copy must hold what the task reads
    bool drained = false;
    for (auto &x : in_place) {
        Region down = needed(x.buffer, x.effects);
        down.remove(x.buffer->host_valid);
        if (down.empty()) continue;
        if (!drained) {
            flush(c);  // queued tasks that write the device copy run first
            drained = true;
        }
        copy_region(c, x.buffer, down, false);
        Region host = x.buffer->host_valid;
        host.add(down);
        settle(c, x.buffer, x.buffer->defined, host, x.buffer->device_valid);
    }
    for (auto &x : mirrored) device_commit(c, x.buffer, x.effects.writes, x.effects.overwrites);
    for (auto &x : in_place) {
        host_commit(c, x.buffer, x.effects.writes, x.effects.overwrites);
        trace_line(c, "in_place", x.buffer->handle, x.buffer->bytes);
        if (!x.buffer->awaits_token) {
            x.buffer->awaits_token = true;
            c->awaiting_token.push_back(x.buffer->handle);
        }
    }
    for (auto &x : bound) {
        note_device_use(x.buffer);
        x.buffer->queued++;
        task.buffers.push_back(x.buffer->handle);
    }
    size_t bytes = 0;
    for (auto &v : task.values) bytes += v.size();
    std::memcpy(task.origin.fields, c->trace, sizeof task.origin.fields);
    c->queue_stats.accepted_tasks++;
    c->queue_stats.copied_argument_bytes += bytes;
    c->pending_threads += task.threads;
    c->pending.push_back(std::move(task));
    c->queue_stats.pending_tasks = c->pending.size();
    if (c->pending.size() > c->queue_stats.peak_pending_tasks) c->queue_stats.peak_pending_tasks = c->pending.size();
    trace_line(c, "queue_enqueue", 0, bytes);
    if (!c->queue_enabled || (c->queue_work_limit && c->pending_threads >= c->queue_work_limit)) flush(c);
}

// A provider's kernels are opaque: its submission is counted, its launches are not invented.
void count_external_launch(Context *c) { c->queue_stats.direct_submissions++; }

// ---- slab pipelines -------------------------------------------------------------------------

constexpr size_t kMaxSlabs = 64;

bool streaming_allowed() {
    static const bool on = env_flag("FORT_SCOPE_HOST_STREAM", true);
    return on;
}

// An array in pinned host memory that the host read or rewrote before each of
// its recent device uses: its transfers are worth overlapping with the kernels.
bool host_round(const Buffer *b) {
    return b->mapped && b->prepared == Buffer::NONE && b->host_touched && b->host_rounds >= 1;
}

// Run tasks over successive slabs of the same arrays three streams deep:
// copy_in uploads what task n reads ahead of its kernel, the context stream
// runs the kernels in order, copy_out publishes what task n wrote into
// host-round arrays behind it. A kernel waits for its own uploads and, where
// it writes what an earlier publication still reads, for that publication.
// Uploads of an array being published move exactly what is stale on the device
// (never widened over values in flight), and publications move exactly what a
// task wrote. Finally the context stream joins both copy streams, so every
// later operation of the context, and a wait on it, orders after the sequence.
void run_slabs(Context *c, std::vector<Task> &tasks, std::vector<std::vector<Bound>> &bound) {
    std::set<Buffer *> publish, all;
    for (auto &list : bound)
        for (auto &x : list) {
            all.insert(x.buffer);
            if (host_round(x.buffer) && !x.effects.writes.empty()) publish.insert(x.buffer);
        }
    flush(c);
    ensure_copy_streams(c);
    auto join = [&](Stream waiter, Stream signaller) {
        if (!Backend::join(waiter, signaller)) poison(c, std::string("stream ordering failed: ") + Backend::last_error());
    };
    join(c->copy_in, c->stream);
    join(c->copy_out, c->stream);
    std::map<Buffer *, Region> publishing, uploading;
    // optional timing marks, one set per slab (events made once and reused)
    Context::SlabMarks *marks = nullptr;
    if (c->slab_timing) {
        if (c->slab_marks.size() < tasks.size()) c->slab_marks.resize(tasks.size());
        for (size_t n = 0; n < tasks.size(); ++n) {
            auto &m = c->slab_marks[n];
            if (!m.made) {
                bool good = true;
                for (Backend::Event *e : {&m.up0, &m.up1, &m.k0, &m.k1, &m.p0, &m.p1})
                    good = Backend::make_timing_event(e) && good;
                if (!good) raise(FORT_SCOPE_RESOURCE, "cannot create timing events: " + Backend::last_error());
                m.made = true;
            }
            m.uploaded = m.published = false;
        }
        c->slab_marks_used = tasks.size();
        marks = c->slab_marks.data();
    }
    auto mark = [&](Backend::Event e, Stream s) {
        if (!Backend::record(e, s)) poison(c, std::string("timing event failed: ") + Backend::last_error());
    };
    for (size_t n = 0; n < tasks.size(); ++n) {
        bool uploaded = false;
        for (auto &x : bound[n]) {
            Buffer *b = x.buffer;
            Region up = needed(b, x.effects);
            up.remove(b->device_valid);
            if (up.empty()) continue;
            if (marks && !uploaded) {
                mark(marks[n].up0, c->copy_in);
                marks[n].uploaded = true;
            }
            Region moved = up;
            if (!publish.count(b)) {
                // the whole planes spanning the need, less what the device holds: one run (up to a host
                // boundary) when it moves at most a quarter more than the need; else the usual widening
                Box planes = bounding(up);
                for (int d = 0; d + 1 < planes.rank; ++d) {
                    planes.lo[d] = 0;
                    planes.hi[d] = b->extents[d];
                }
                Region rest;
                rest.add(planes);
                rest.remove(b->device_valid);
                Region undefined = rest;
                undefined.remove(b->defined);
                size_t lo, hi;
                if (undefined.empty() && as_interval(b, rest, lo, hi) &&
                    (double)rest.volume() <= 1.25 * (double)up.volume())
                    moved = to_host_boundary(b, rest);
                else
                    moved = widened(b, up, true);
            }
            copy_run(c, b, moved, true, c->copy_in);
            uploading[b].add(moved);
            Region device = b->device_valid;
            Region unheld = moved;
            unheld.remove(b->host_valid);
            if (unheld.empty()) {
                device.add(moved);  // a few boxes: adding `up` first would splinter them around its pieces
            } else {
                device.add(up);
                device.add(b->host_valid.clip(moved));
            }
            settle(c, b, b->defined, b->host_valid, device);
            uploaded = true;
        }
        if (uploaded) {
            if (marks) mark(marks[n].up1, c->copy_in);
            join(c->stream, c->copy_in);
        }
        bool clash = false;
        for (auto &x : bound[n]) {
            auto it = publishing.find(x.buffer);
            if (it != publishing.end() && !it->second.clip(x.effects.writes).empty()) clash = true;
        }
        if (clash) join(c->stream, c->copy_out);
        trace_line(c, "slab_launch", 0, n);
        if (marks) mark(marks[n].k0, c->stream);
        if (!Backend::launch(tasks[n].spec, c->stream))
            poison(c, std::string("kernel launch failed: ") + Backend::last_error());
        if (marks) mark(marks[n].k1, c->stream);
        for (auto &x : bound[n]) device_commit(c, x.buffer, x.effects.writes, x.effects.overwrites);
        bool ordered = false;
        for (auto &x : bound[n]) {
            Buffer *b = x.buffer;
            if (!publish.count(b)) continue;
            Region down = b->physical.clip(x.effects.writes);
            down.remove(b->host_valid);
            if (down.empty()) continue;
            if (!ordered) {
                join(c->copy_out, c->stream);
                ordered = true;
                if (marks) {
                    mark(marks[n].p0, c->copy_out);
                    marks[n].published = true;
                }
            }
            copy_region(c, b, down, false, c->copy_out);
            publishing[b].add(down);
            Region host = b->host_valid;
            host.add(down);
            settle(c, b, b->defined, host, b->device_valid);
        }
        if (marks && marks[n].published) mark(marks[n].p1, c->copy_out);
    }
    join(c->stream, c->copy_in);
    join(c->stream, c->copy_out);
    if (!uploading.empty() || !publishing.empty()) {
        const uint64_t token = record_token(c);
        for (Buffer *b : all) {
            auto up = uploading.find(b), down = publishing.find(b);
            if (up != uploading.end() || down != publishing.end())
                hold_host(b, up != uploading.end() ? up->second : Region{},
                          down != publishing.end() ? down->second : Region{}, token);
        }
    }
    for (Buffer *b : all) note_device_use(b);
    Domain *d = c->domain;
    d->stats.launches += tasks.size();
    c->graph_stats.submissions++;
    c->graph_stats.logical_kernels += tasks.size();
    c->queue_stats.accepted_tasks += tasks.size();
    c->queue_stats.direct_submissions++;
    c->queue_stats.direct_kernels += tasks.size();
}

Context *make_context(Domain *d, bool private_domain) {
    auto c = std::make_unique<Context>();
    c->handle = new_handle();
    c->domain = d;
    c->private_domain = private_domain;
    c->queue_enabled = env_flag("FORT_SCOPE_GRAPH_QUEUE", true);
    c->graphs_enabled = env_flag("FORT_SCOPE_CUDA_GRAPHS", true);
    if (const char *w = std::getenv("FORT_SCOPE_GRAPH_QUEUE_WORK")) c->queue_work_limit = std::strtoull(w, nullptr, 10);
    c->queue_stats.version = 1;
    c->queue_stats.queue_enabled = c->queue_enabled;
    c->queue_stats.graphs_enabled = c->graphs_enabled;
    c->graph_stats.version = 1;
    c->completion.version = 1;
    c->scratch_stats.version = 1;
    d->borrower = c.get();
    Context *raw = c.get();
    g_contexts[raw->handle] = std::move(c);
    return raw;
}

Domain *make_domain(int device) {
    if (device < 0) raise(FORT_SCOPE_ARGUMENT, "negative device ordinal");
    auto d = std::make_unique<Domain>();
    d->handle = new_handle();
    d->device = device;
    d->residency.version = 1;
    Domain *raw = d.get();
    g_domains[raw->handle] = std::move(d);
    return raw;
}

void destroy_buffer(Context *c, Buffer *b) {
    release_mirror(c, b);
    if (b->pinned_here) Backend::unpin(b->host);
    c->domain->by_identity.erase(b->identity);
    g_retired.insert(b->handle);
    c->domain->buffers.erase(b->handle);
}

void release_scratch(Context *c) {
    if (c->scratch) {
        Backend::free(c->scratch, c->stream);
        c->domain->scratch_bytes -= c->scratch_capacity;
        c->scratch = nullptr;
        c->scratch_capacity = 0;
    }
}

// The statistics of a context as it closes, one `FORT_SCOPED evidence` JSON
// line per kind that saw any use (the reference's records, same keys):
// graphs, host completions, the task queue, residency.
void evidence(Context *c) {
    if (!tracing()) return;
    const bool complete = !c->poisoned && !c->domain->poisoned;
    const std::string head = "FORT_SCOPED evidence {\"schema_version\":1,\"context\":" + std::to_string(c->handle) +
                             ",\"domain_version\":1,\"domain\":" + std::to_string(c->domain->handle) +
                             ",\"domain_role\":\"" + (c->private_domain ? "storage" : "execution") + "\"";
    auto record = [&](const char *event, const std::string &extra,
                      std::initializer_list<std::pair<const char *, uint64_t>> fields) {
        std::string line = head + ",\"event\":\"" + event + "\",\"stats_version\":1,\"complete\":" +
                           (complete ? "true" : "false") + extra;
        for (const auto &f : fields) line += std::string(",\"") + f.first + "\":" + std::to_string(f.second);
        line += "}\n";
        std::fputs(line.c_str(), stderr);
    };
    const auto &g = c->graph_stats;
    const auto &q = c->queue_stats;
    const auto &k = c->completion;
    const auto &r = c->domain->residency;
    if (g.creations || q.direct_kernels)
        record("graph_statistics", "",
               {{"creations", g.creations}, {"instantiations", g.instantiations}, {"rebuilds", g.rebuilds},
                {"submissions", g.submissions}, {"replays", g.replays}, {"parameter_updates", g.parameter_updates},
                {"logical_kernels", g.logical_kernels}, {"live_graphs", g.live_graphs},
                {"destructions", g.destructions}});
    if (k.event_records || k.independent_host_tasks)
        record("completion_statistics", "",
               {{"event_records", k.event_records}, {"event_queries", k.event_queries}, {"event_waits", k.event_waits},
                {"stream_waits", k.stream_waits}, {"created_events", k.created_events},
                {"reused_events", k.reused_events}, {"independent_host_tasks", k.independent_host_tasks}});
    if (q.accepted_tasks || q.submissions || q.direct_submissions || q.direct_kernels || !q.queue_enabled ||
        !q.graphs_enabled)
        record("command_queue_statistics",
               ",\"queue_enabled\":" + std::to_string(q.queue_enabled) + ",\"graphs_enabled\":" +
                   std::to_string(q.graphs_enabled),
               {{"accepted_tasks", q.accepted_tasks}, {"submissions", q.submissions},
                {"conflict_flushes", q.conflict_flushes}, {"explicit_flushes", q.explicit_flushes},
                {"pending_tasks", q.pending_tasks}, {"peak_pending_tasks", q.peak_pending_tasks},
                {"copied_argument_bytes", q.copied_argument_bytes}, {"direct_submissions", q.direct_submissions},
                {"direct_kernels", q.direct_kernels}, {"graph_resource_fallbacks", q.graph_resource_fallbacks}});
    if (r.evictions)
        record("residency_statistics", ",\"device_budget\":" + std::to_string(c->domain->budget),
               {{"reserve_batches", r.reserve_batches}, {"requested_resources", r.requested_resources},
                {"reuse_hits", r.reuse_hits}, {"evictions", r.evictions}, {"evicted_bytes", r.evicted_bytes},
                {"dirty_evictions", r.dirty_evictions}, {"dirty_download_bytes", r.dirty_download_bytes},
                {"pressure_flushes", r.pressure_flushes}});
}

void drop_slab_marks(Context *c) {
    for (auto &m : c->slab_marks)
        if (m.made)
            for (Backend::Event e : {m.up0, m.up1, m.k0, m.k1, m.p0, m.p1}) Backend::destroy_event(e);
    c->slab_marks.clear();
    c->slab_marks_used = 0;
}

void detach(Context *c) {
    drop_slab_marks(c);
    if (c->copies_ready) {
        Backend::sync(c->copy_in);
        Backend::sync(c->copy_out);
        Backend::destroy_stream(c->copy_in);
        Backend::destroy_stream(c->copy_out);
        c->copies_ready = false;
    }
    if (c->stream_ready) {
        Backend::sync(c->stream);
        for (auto *cache : {&c->graphs, &c->group_graphs})
            for (auto &kv : *cache)
                if (kv.second.graph) {
                    Backend::graph_destroy(kv.second.graph);
                    kv.second.graph = nullptr;
                    c->graph_stats.destructions++;
                    c->graph_stats.live_graphs--;
                }
        release_events(c);
        Backend::destroy_stream(c->stream);
    }
    evidence(c);
    if (c->domain->borrower == c) c->domain->borrower = nullptr;
    g_retired.insert(c->handle);
    g_contexts.erase(c->handle);
}

// Publish and free every array of a domain through `c` (its last context).
void close_domain_through(Context *c, bool publish) {
    Domain *d = c->domain;
    if (publish) {
        flush(c);
        for (auto &kv : d->buffers) publish_buffer(c, kv.second.get());
        wait_stream(c);
    }
    std::vector<Buffer *> all;
    for (auto &kv : d->buffers) all.push_back(kv.second.get());
    for (Buffer *b : all) destroy_buffer(c, b);
    release_scratch(c);
}

template <typename F>
int guarded(F &&f) {
    std::lock_guard<std::recursive_mutex> lock(g_mutex);
    try {
        return f();
    } catch (Failure &e) {
        return fail(e.status, e.message);
    } catch (std::bad_alloc &) {
        return fail(FORT_SCOPE_RESOURCE, "host memory exhausted");
    } catch (std::exception &e) {  // nothing thrown crosses the C boundary
        return fail(FORT_SCOPE_EXECUTION, std::string("unexpected exception: ") + e.what());
    } catch (...) {
        return fail(FORT_SCOPE_EXECUTION, "unexpected exception");
    }
}

void copy_field(char *dst, const char *src) {
    if (!src) {
        dst[0] = 0;
        return;
    }
    size_t n = strnlen(src, 65);
    if (n >= 65) n = 0; // invalid identity: unknown
    std::memcpy(dst, src, n);
    dst[n] = 0;
}

// A positive count of bytes in decimal digits, optionally followed by one of
// K, M or G (either case, powers of 1024); anything else, zero or a count that
// overflows is refused.
size_t parse_bytes(const char *text, bool *ok) {
    *ok = false;
    unsigned long long v = 0;
    const char *p = text;
    for (; *p >= '0' && *p <= '9'; ++p) {
        if (v > (~0ULL - 9) / 10) return 0;
        v = v * 10 + (unsigned long long)(*p - '0');
    }
    if (p == text) return 0;
    unsigned shift = 0;
    if (*p) {
        switch (*p) {
        case 'K': case 'k': shift = 10; break;
        case 'M': case 'm': shift = 20; break;
        case 'G': case 'g': shift = 30; break;
        default: return 0;
        }
        if (p[1]) return 0;
    }
    if (!v || v > (~0ULL >> shift)) return 0;
    *ok = true;
    return (size_t)(v << shift);
}

} // namespace
} // namespace f2c::rt

using namespace f2c::rt;

extern "C" {

uint32_t fort_scope_abi_version(void) { return FORT_SCOPE_ABI_VERSION; }

const char *fort_scope_error(void) { return t_error.c_str(); }

int fort_scope_report_error(int status, const char *message) {
    t_error = message ? message : "";
    return status;
}

int fort_scope_execution_error(fort_scope_t context, const char *message) {
    std::lock_guard<std::recursive_mutex> lock(g_mutex);
    auto it = g_contexts.find(context);
    if (it != g_contexts.end()) {
        it->second->poisoned = true;
        it->second->domain->poisoned = true;
    }
    t_error = std::string(message ? message : "execution failure") + "; unsafe replay prohibited";
    return FORT_SCOPE_EXECUTION;
}

void fort_scope_trace_set_v1(fort_scope_t context, uint32_t update_mask, const char *owner, const char *procedure,
                             const char *segment, const char *operation, const char *implementation,
                             const char *boundary, fort_scope_trace_state_v1 *previous) {
    if (!tracing()) {
        if (previous) previous->version = 0;
        return;
    }
    std::lock_guard<std::recursive_mutex> lock(g_mutex);
    auto it = g_contexts.find(context);
    if (it == g_contexts.end()) {
        if (previous) previous->version = 0;
        return;
    }
    Context *c = it->second.get();
    if (previous) {
        previous->version = FORT_SCOPE_TRACE_ABI_VERSION;
        previous->reserved = 0;
        char *fields[6] = {previous->owner, previous->procedure, previous->segment, previous->operation,
                           previous->implementation, previous->boundary};
        for (int n = 0; n < 6; ++n) std::memcpy(fields[n], c->trace[n], 65);
    }
    const char *values[6] = {owner, procedure, segment, operation, implementation, boundary};
    for (int n = 0; n < 6; ++n)
        if (update_mask & (1u << n)) copy_field(c->trace[n], values[n]);
}

void fort_scope_trace_restore_v1(fort_scope_t context, const fort_scope_trace_state_v1 *previous) {
    if (!tracing() || !previous || previous->version != FORT_SCOPE_TRACE_ABI_VERSION) return;
    std::lock_guard<std::recursive_mutex> lock(g_mutex);
    auto it = g_contexts.find(context);
    if (it == g_contexts.end()) return;
    const char *fields[6] = {previous->owner, previous->procedure, previous->segment, previous->operation,
                             previous->implementation, previous->boundary};
    for (int n = 0; n < 6; ++n) std::memcpy(it->second->trace[n], fields[n], 65);
}

// ---- contexts and domains ----

int fort_scope_create(int device, fort_scope_t *context) {
    return guarded([&] {
        if (!context) raise(FORT_SCOPE_ARGUMENT, "null context output");
        Domain *d = make_domain(device);
        d->owned_by_context = true;
        *context = make_context(d, true)->handle;
        return FORT_SCOPE_OK;
    });
}

int fort_scope_domain_create_v1(int device, fort_scope_domain_t *domain) {
    return guarded([&] {
        if (!domain) raise(FORT_SCOPE_ARGUMENT, "null domain output");
        *domain = make_domain(device)->handle;
        return FORT_SCOPE_OK;
    });
}

int fort_scope_create_in_domain_v1(fort_scope_domain_t domain, fort_scope_t *context) {
    return guarded([&] {
        if (!context) raise(FORT_SCOPE_ARGUMENT, "null context output");
        Domain *d = find_domain(domain);
        if (d->poisoned) raise(FORT_SCOPE_EXECUTION, "domain poisoned by an execution failure");
        if (d->borrower) raise(FORT_SCOPE_STATE, "domain already borrowed by a context");
        *context = make_context(d, false)->handle;
        return FORT_SCOPE_OK;
    });
}

int fort_scope_domain_get_v1(fort_scope_t context, fort_scope_domain_t *domain) {
    return guarded([&] {
        if (!domain) raise(FORT_SCOPE_ARGUMENT, "null domain output");
        Context *c = find_context(context);
        *domain = c->private_domain ? 0 : c->domain->handle;
        return FORT_SCOPE_OK;
    });
}

int fort_scope_domain_device_get_v1(fort_scope_domain_t domain, int *device) {
    return guarded([&] {
        if (!device) raise(FORT_SCOPE_ARGUMENT, "null device output");
        *device = find_domain(domain)->device;
        return FORT_SCOPE_OK;
    });
}

int fort_scope_domain_stats_get_v1(fort_scope_domain_t domain, fort_scope_stats *stats) {
    return guarded([&] {
        if (!stats) raise(FORT_SCOPE_ARGUMENT, "null stats output");
        *stats = find_domain(domain)->stats;
        return FORT_SCOPE_OK;
    });
}

int fort_scope_domain_close_v1(fort_scope_domain_t domain) {
    return guarded([&] {
        Domain *d = find_domain(domain);
        if (d->poisoned) raise(FORT_SCOPE_EXECUTION, "domain poisoned; abandon it instead");
        if (d->borrower) raise(FORT_SCOPE_STATE, "domain still borrowed by a context");
        if (!d->workspaces.empty()) raise(FORT_SCOPE_STATE, "provider workspace leases are still held");
        for (auto &kv : d->buffers)
            if (kv.second->prepared != Buffer::NONE) raise(FORT_SCOPE_STATE, "domain has a prepared access");
        Context *c = make_context(d, false);
        int status = FORT_SCOPE_OK;
        try {
            close_domain_through(c, true);
        } catch (Failure &e) {
            status = fail(e.status, e.message);
        }
        detach(c);
        g_retired.insert(d->handle);
        g_domains.erase(d->handle);
        return status;
    });
}

int fort_scope_domain_abandon_v1(fort_scope_domain_t domain) {
    return guarded([&] {
        Domain *d = find_domain(domain);
        if (d->borrower) raise(FORT_SCOPE_STATE, "domain still borrowed by a context");
        // the provider destroys what it owns and releases its leases first: the runtime cannot free its bytes
        if (!d->workspaces.empty()) raise(FORT_SCOPE_STATE, "release the provider's workspace leases first");
        d->poisoned = false;
        Context *c = make_context(d, false);
        close_domain_through(c, false);
        detach(c);
        g_retired.insert(d->handle);
        g_domains.erase(d->handle);
        return FORT_SCOPE_OK;
    });
}

// Workspace claims: bytes an external provider allocated on its own, counted
// against the domain's budget like mirrors and scratch (no memory is allocated
// here). A claim that does not fit beside what the domain already holds fails
// with RESOURCE and changes nothing: mirrors are not evicted for a provider.
void fit_workspace(Domain *d, size_t after) {
    if (!d->budget_set || after <= d->workspace_bytes) return;
    const size_t growth = after - d->workspace_bytes;
    if (claimed(d) + growth > d->budget) raise(FORT_SCOPE_RESOURCE, "workspace claim exceeds the free device budget");
}

Domain *live_domain(fort_scope_domain_t handle) {
    Domain *d = find_domain(handle);
    if (d->poisoned) raise(FORT_SCOPE_EXECUTION, "residency domain has failed");
    return d;
}

int fort_scope_domain_workspace_reserve_v1(fort_scope_domain_t domain, size_t bytes, uint64_t *lease) {
    return guarded([&] {
        if (!lease) raise(FORT_SCOPE_ARGUMENT, "null workspace lease output");
        Domain *d = live_domain(domain);
        if (bytes > SIZE_MAX - d->workspace_bytes) raise(FORT_SCOPE_RESOURCE, "workspace byte overflow");
        fit_workspace(d, d->workspace_bytes + bytes);
        const uint64_t token = new_handle();
        d->workspaces[token] = bytes;
        d->workspace_bytes += bytes;
        if (claimed(d) > d->peak_total_bytes) d->peak_total_bytes = claimed(d);
        *lease = token;
        return FORT_SCOPE_OK;
    });
}

int fort_scope_domain_workspace_resize_v1(fort_scope_domain_t domain, uint64_t lease, size_t bytes) {
    return guarded([&] {
        Domain *d = live_domain(domain);
        auto it = d->workspaces.find(lease);
        if (it == d->workspaces.end()) raise(FORT_SCOPE_STALE, "foreign or stale workspace lease");
        const size_t others = d->workspace_bytes - it->second;
        if (bytes > SIZE_MAX - others) raise(FORT_SCOPE_RESOURCE, "workspace byte overflow");
        fit_workspace(d, others + bytes);
        d->workspace_bytes = others + bytes;
        if (claimed(d) > d->peak_total_bytes) d->peak_total_bytes = claimed(d);
        it->second = bytes;
        return FORT_SCOPE_OK;
    });
}

int fort_scope_domain_workspace_release_v1(fort_scope_domain_t domain, uint64_t lease) {
    return guarded([&] {
        Domain *d = find_domain(domain);
        auto it = d->workspaces.find(lease);
        if (it == d->workspaces.end()) raise(FORT_SCOPE_STALE, "foreign or stale workspace lease");
        d->workspace_bytes -= it->second;
        d->workspaces.erase(it);
        return FORT_SCOPE_OK;
    });
}

int fort_scope_set_device_budget(fort_scope_t context, size_t bytes) {
    return guarded([&] {
        Context *c = live_context(context);
        Domain *d = c->domain;
        if (c->stream_ready || d->device_bytes) {  // the device is in use: the budget is fixed
            if (!d->budget_set || bytes != d->budget) raise(FORT_SCOPE_STATE, "cannot change a live device budget");
            return FORT_SCOPE_OK;
        }
        if (bytes < d->workspace_bytes) raise(FORT_SCOPE_STATE, "the device budget must cover the workspace claims");
        c->domain->budget = bytes;
        c->domain->budget_set = true;
        return FORT_SCOPE_OK;
    });
}

int fort_scope_device_budget_default_v1(int device, size_t *bytes) {
    return guarded([&] {
        if (!bytes) raise(FORT_SCOPE_ARGUMENT, "null budget output");
        if (device < 0) raise(FORT_SCOPE_ARGUMENT, "negative device ordinal");
        // an empty value reads as unset: the budget is then derived from the device
        const char *text = std::getenv("FORT_RESIDENT_DEVICE_BUDGET");
        if (text && text[0]) {
            bool ok = false;
            const size_t v = parse_bytes(text, &ok);
            if (!ok) raise(FORT_SCOPE_ARGUMENT, "FORT_RESIDENT_DEVICE_BUDGET must be a positive count of bytes, optionally with K, M or G");
            *bytes = v;
            return FORT_SCOPE_OK;
        }
        const int previous = Backend::current();
        if (!Backend::select(device)) raise(FORT_SCOPE_RESOURCE, "cannot select device: " + Backend::last_error());
        size_t free_bytes = 0, total = 0;
        const bool ok = Backend::memory_info(&free_bytes, &total);
        Backend::select(previous);
        if (!ok) raise(FORT_SCOPE_RESOURCE, "cannot query device memory: " + Backend::last_error());
        // the driver, graphs and library plans allocate outside the budget: a sixteenth of the device, at least
        // 512 MiB, stays free
        size_t reserve = total / 16;
        if (reserve < (size_t(512) << 20)) reserve = size_t(512) << 20;
        if (free_bytes <= reserve) raise(FORT_SCOPE_RESOURCE, "the device has no free memory for a residency domain");
        *bytes = free_bytes - reserve;
        return FORT_SCOPE_OK;
    });
}

int fort_scope_domain_budget_get_v1(fort_scope_domain_t domain, size_t *budget, size_t *unclaimed) {
    return guarded([&] {
        if (!budget || !unclaimed) raise(FORT_SCOPE_ARGUMENT, "null budget output");
        Domain *d = find_domain(domain);
        *budget = d->budget_set ? d->budget : SIZE_MAX;
        const size_t used = claimed(d);
        *unclaimed = *budget > used ? *budget - used : 0;
        return FORT_SCOPE_OK;
    });
}

int fort_scope_close(fort_scope_t context) {
    return guarded([&] {
        Context *c = find_context(context);
        if (c->poisoned || c->domain->poisoned)
            raise(FORT_SCOPE_EXECUTION, "context poisoned; abandon it instead of publishing");
        if (c->scratch_active) raise(FORT_SCOPE_STATE, "context holds an active scratch lease");
        for (auto &kv : c->domain->buffers)
            if (kv.second->prepared != Buffer::NONE) raise(FORT_SCOPE_STATE, "context has a prepared access");
        Domain *d = c->domain;
        if (c->private_domain) {
            close_domain_through(c, true);
            detach(c);
            g_retired.insert(d->handle);
            g_domains.erase(d->handle);
        } else {
            flush(c);
            wait_stream(c);
            release_scratch(c);
            detach(c);
        }
        return FORT_SCOPE_OK;
    });
}

int fort_scope_abandon(fort_scope_t context) {
    return guarded([&] {
        Context *c = find_context(context);
        if (!c->poisoned && !c->domain->poisoned) raise(FORT_SCOPE_STATE, "abandon is only for failed contexts");
        c->pending.clear();
        Domain *d = c->domain;
        for (auto &kv : d->buffers) {
            kv.second->prepared = Buffer::NONE;
            kv.second->queued = 0;
        }
        c->scratch_active = false;
        release_scratch(c);
        if (c->private_domain) {
            close_domain_through(c, false);
            detach(c);
            g_retired.insert(d->handle);
            g_domains.erase(d->handle);
        } else {
            detach(c);
        }
        return FORT_SCOPE_OK;
    });
}

int fort_scope_wait(fort_scope_t context) {
    return guarded([&] {
        Context *c = live_context(context);
        flush(c);
        wait_stream(c);
        return FORT_SCOPE_OK;
    });
}

// ---- registration ----

static int register_impl(fort_scope_t context, uint64_t identity, uint64_t generation, const fort_scope_layout *layout,
                         const fort_scope_section *initialized, size_t initialized_count, bool all_defined,
                         fort_buffer_t *out) {
    return guarded([&] {
        if (!layout || !out) raise(FORT_SCOPE_ARGUMENT, "null registration argument");
        Context *c = live_context(context);
        Domain *d = c->domain;
        if (layout->rank < 1 || layout->rank > (uint32_t)kMaxRank) raise(FORT_SCOPE_ARGUMENT, "unsupported rank");
        if (layout->type > FORT_SCOPE_LOGICAL) raise(FORT_SCOPE_ARGUMENT, "unknown element type");
        if (!layout->element_bytes || !layout->extents || !layout->lower_bounds)
            raise(FORT_SCOPE_ARGUMENT, "incomplete layout");
        const size_t expect[] = {0, 4, 8, 4, 0};
        if (expect[layout->type] && layout->element_bytes != expect[layout->type])
            raise(FORT_SCOPE_ARGUMENT, "element size does not match the element type");
        size_t count = 1;
        for (uint32_t r = 0; r < layout->rank; ++r) {
            const size_t e = layout->extents[r];
            if (e && count > SIZE_MAX / e) raise(FORT_SCOPE_ARGUMENT, "array size overflows");
            count *= e;
        }
        if (count && count > SIZE_MAX / layout->element_bytes) raise(FORT_SCOPE_ARGUMENT, "array size overflows");
        const size_t bytes = count * layout->element_bytes;
        if (bytes && !layout->host) raise(FORT_SCOPE_ARGUMENT, "null host storage");
        auto existing = d->by_identity.find(identity);
        if (existing != d->by_identity.end()) {
            Buffer *b = d->buffers.at(existing->second).get();
            bool same = b->rank == (int)layout->rank && b->type == layout->type && b->elem == layout->element_bytes &&
                        b->host == layout->host;
            for (int r = 0; same && r < b->rank; ++r) same = b->extents[r] == layout->extents[r];
            if (!same) raise(FORT_SCOPE_ARGUMENT, "identity already registered with another layout or storage");
            if (b->generation != generation)
                raise(FORT_SCOPE_STALE, "allocation generation changed: unregister before changing storage");
            for (int r = 0; r < b->rank; ++r) b->lower[r] = layout->lower_bounds[r];
            *out = b->handle;
            return FORT_SCOPE_OK;
        }
        const char *lo = static_cast<const char *>(layout->host);
        for (auto &kv : d->buffers) {
            if (!bytes) break;  // an empty array occupies no host storage
            const Buffer *o = kv.second.get();
            const char *olo = static_cast<const char *>(o->host);
            if (lo < olo + o->bytes && olo < lo + bytes)
                raise(FORT_SCOPE_ALIAS, "host storage overlaps a registered array");
        }
        auto b = std::make_unique<Buffer>();
        b->handle = new_handle();
        b->identity = identity;
        b->generation = generation;
        b->rank = (int)layout->rank;
        b->type = layout->type;
        b->elem = layout->element_bytes;
        b->bytes = bytes;
        b->host = layout->host;
        for (int r = 0; r < b->rank; ++r) {
            b->extents[r] = layout->extents[r];
            b->lower[r] = layout->lower_bounds[r];
        }
        b->host_valid.add(b->full());
        if (all_defined) {
            b->defined.add(b->full());
        } else {
            if (initialized_count > kRegionLimit || (initialized_count && !initialized))
                raise(FORT_SCOPE_ARGUMENT, "initialized section list exceeds the bounded interface");
            for (size_t n = 0; n < initialized_count; ++n) b->defined.add(section_box(b.get(), initialized[n]));
        }
        b->physical = b->defined;
        *out = b->handle;
        const uint64_t handle = b->handle;
        d->by_identity[identity] = handle;
        d->buffers[handle] = std::move(b);
        trace_line(c, "register", handle, bytes);
        return FORT_SCOPE_OK;
    });
}

int fort_scope_register(fort_scope_t context, uint64_t identity, uint64_t generation, const fort_scope_layout *layout,
                        int host_initialized, fort_buffer_t *buffer) {
    return register_impl(context, identity, generation, layout, nullptr, 0, host_initialized != 0, buffer);
}

int fort_scope_register_sections(fort_scope_t context, uint64_t identity, uint64_t generation,
                                 const fort_scope_layout *layout, const fort_scope_section *initialized,
                                 size_t initialized_count, fort_buffer_t *buffer) {
    return register_impl(context, identity, generation, layout, initialized, initialized_count, false, buffer);
}

int fort_scope_admit_source_reads_v1(fort_scope_t context, fort_buffer_t buffer, const fort_scope_section *sections,
                                     size_t count) {
    return guarded([&] {
        Context *c = live_context(context);
        Buffer *b = find_buffer(c, buffer);
        if (count > kRegionLimit || (count && !sections)) raise(FORT_SCOPE_ARGUMENT, "section list exceeds the bounded interface");
        Region add;
        for (size_t n = 0; n < count; ++n) add.add(section_box(b, sections[n]));
        Region fresh = b->defined.missing(b->full()).clip(add);
        Region defined = b->defined, host = b->host_valid, device = b->device_valid;
        defined.add(fresh);
        host.add(fresh);
        device.remove(fresh);
        settle(c, b, std::move(defined), std::move(host), std::move(device));
        return FORT_SCOPE_OK;
    });
}

// Commit a descriptor exchange the program has already made (a MOVE_ALLOC
// swap): the two registered identities trade the arrays they name. Nothing
// physical moves; only the identity map changes and the caller is told which
// array each identity now names. Because the exchange already happened, every
// failed check poisons the context (EXECUTION): continuing under the old names
// could publish into the wrong array.
int fort_scope_identity_swap_v1(fort_scope_t context, fort_buffer_t first, fort_buffer_t second,
                                const fort_scope_layout *first_after, const fort_scope_layout *second_after,
                                fort_buffer_t *first_current, fort_buffer_t *second_current) {
    return guarded([&] {
        Context *c = live_context(context);
        try {
            if (first == second || !first_current || !second_current || first_current == second_current)
                raise(FORT_SCOPE_ARGUMENT, "identity exchange needs two distinct arrays and output slots");
            Buffer *a = find_buffer(c, first);
            Buffer *b = find_buffer(c, second);
            if (a->prepared != Buffer::NONE || b->prepared != Buffer::NONE)
                raise(FORT_SCOPE_STATE, "identity exchange during a prepared access");
            Domain *d = c->domain;
            auto ai = d->by_identity.find(a->identity), bi = d->by_identity.find(b->identity);
            if (a->identity == b->identity || ai == d->by_identity.end() || bi == d->by_identity.end() ||
                ai->second != first || bi->second != second)
                raise(FORT_SCOPE_STALE, "identity exchange names stale identities");
            auto describes = [](const fort_scope_layout *after, const Buffer *x) {
                if (!after || (int)after->rank != x->rank || !after->extents || !after->lower_bounds ||
                    after->host != x->host || after->type != x->type || after->element_bytes != x->elem ||
                    after->generation != x->generation)
                    return false;
                for (int r = 0; r < x->rank; ++r)
                    if (after->extents[r] != x->extents[r] || after->lower_bounds[r] != x->lower[r]) return false;
                return true;
            };
            if (!describes(first_after, b) || !describes(second_after, a))
                raise(FORT_SCOPE_STALE, "a post-exchange layout does not describe the other array");
            ai->second = second;
            bi->second = first;
            std::swap(a->identity, b->identity);
            *first_current = second;
            *second_current = first;
            trace_line(c, "identity_swap", first, second);
        } catch (Failure &f) {
            c->poisoned = true;
            c->domain->poisoned = true;
            raise(FORT_SCOPE_EXECUTION, f.message + "; unsafe replay prohibited");
        }
        return FORT_SCOPE_OK;
    });
}

int fort_scope_forget_definition(fort_scope_t context, fort_buffer_t buffer) {
    return guarded([&] {
        Context *c = live_context(context);
        Buffer *b = find_buffer(c, buffer);
        if (b->prepared != Buffer::NONE) raise(FORT_SCOPE_STATE, "cannot forget definitions under a prepared access");
        b->defined.clear();
        return FORT_SCOPE_OK;
    });
}

int fort_scope_layout_get(fort_scope_t context, fort_buffer_t buffer, fort_scope_layout *layout) {
    return guarded([&] {
        if (!layout) raise(FORT_SCOPE_ARGUMENT, "null layout output");
        Context *c = live_context(context);
        Buffer *b = find_buffer(c, buffer);
        layout->rank = (uint32_t)b->rank;
        layout->type = b->type;
        layout->element_bytes = b->elem;
        layout->host = b->host;
        layout->extents = b->extents;
        layout->lower_bounds = b->lower;
        layout->generation = b->generation;
        return FORT_SCOPE_OK;
    });
}

int fort_scope_buffer_valid_v1(fort_scope_t context, fort_buffer_t buffer, int *valid) {
    return guarded([&] {
        if (!valid) raise(FORT_SCOPE_ARGUMENT, "null output");
        Context *c = find_context(context);
        *valid = c->domain->buffers.count(buffer) ? 1 : 0;
        return FORT_SCOPE_OK;
    });
}

// ---- accesses ----

int fort_scope_access_begin_v1(fort_scope_t context, const fort_scope_plan_binding *bindings, size_t count, int device,
                               void **devices) {
    return guarded([&] {
        Context *c = live_context(context);
        if (device && count && !devices) raise(FORT_SCOPE_ARGUMENT, "null device pointer output");
        std::vector<Bound> bound = bind_all(c, bindings, count);
        if (!count) return FORT_SCOPE_OK;
        if (device) {
            // direct device work is ordered after every queued task
            flush(c);
            std::vector<Buffer *> list;
            for (auto &x : bound) list.push_back(x.buffer);
            reserve(c, list, false);
            device_acquire(c, bound);
            for (auto &x : bound) note_device_use(x.buffer);
        } else {
            host_acquire(c, bound);
        }
        for (size_t n = 0; n < bound.size(); ++n) {
            Buffer *b = bound[n].buffer;
            b->prepared = device ? Buffer::DEVICE : Buffer::HOST;
            b->prep_writes = bound[n].effects.writes;
            b->prep_overwrites = bound[n].effects.overwrites;
            if (device) devices[n] = b->device;
        }
        return FORT_SCOPE_OK;
    });
}

int fort_scope_original_host_begin_v1(fort_scope_t context, const fort_scope_plan_binding *bindings, size_t count) {
    return guarded([&] {
        Context *c = live_context(context);
        std::vector<Bound> bound;
        if (count && !bindings) raise(FORT_SCOPE_ARGUMENT, "null bindings");
        for (size_t n = 0; n < count; ++n) {
            Buffer *b = find_buffer(c, bindings[n].buffer);
            if (b->prepared != Buffer::NONE) raise(FORT_SCOPE_STATE, "array already has a prepared access");
            bound.push_back({b, effects_of(b, bindings[n].access)});
        }
        host_acquire(c, bound);
        for (auto &x : bound) {
            x.buffer->prepared = Buffer::HOST;
            x.buffer->prep_writes = x.effects.writes;
            x.buffer->prep_overwrites = x.effects.overwrites;
        }
        return FORT_SCOPE_OK;
    });
}

int fort_scope_host_begin(fort_scope_t context, fort_buffer_t buffer, const fort_scope_access *access) {
    if (!access) return fail(FORT_SCOPE_ARGUMENT, "null access");
    fort_scope_plan_binding binding{buffer, *access};
    return fort_scope_access_begin_v1(context, &binding, 1, 0, nullptr);
}

int fort_scope_device_begin(fort_scope_t context, fort_buffer_t buffer, const fort_scope_access *access, void **device) {
    if (!access || !device) return fail(FORT_SCOPE_ARGUMENT, "null access or device output");
    fort_scope_plan_binding binding{buffer, *access};
    return fort_scope_access_begin_v1(context, &binding, 1, 1, device);
}

static int end_impl(fort_scope_t context, fort_buffer_t buffer, bool device) {
    return guarded([&] {
        Context *c = live_context(context);
        Buffer *b = find_buffer(c, buffer);
        if (b->prepared != (device ? Buffer::DEVICE : Buffer::HOST))
            raise(FORT_SCOPE_STATE, device ? "no prepared device access" : "no prepared host access");
        if (device) {
            device_commit(c, b, b->prep_writes, b->prep_overwrites);
        } else {
            host_commit(c, b, b->prep_writes, b->prep_overwrites);
            b->host_touched = true;
        }
        b->prepared = Buffer::NONE;
        b->prep_writes.clear();
        b->prep_overwrites.clear();
        return FORT_SCOPE_OK;
    });
}

int fort_scope_host_end(fort_scope_t context, fort_buffer_t buffer) { return end_impl(context, buffer, false); }
int fort_scope_device_end(fort_scope_t context, fort_buffer_t buffer) { return end_impl(context, buffer, true); }

int fort_scope_cancel_access(fort_scope_t context, fort_buffer_t buffer) {
    return guarded([&] {
        Context *c = find_context(context);
        Buffer *b = find_buffer(c, buffer);
        if (b->prepared == Buffer::NONE) raise(FORT_SCOPE_STATE, "no prepared access to cancel");
        b->prepared = Buffer::NONE;
        b->prep_writes.clear();
        b->prep_overwrites.clear();
        return FORT_SCOPE_OK;
    });
}

int fort_scope_device_reserve_v1(fort_scope_t context, fort_buffer_t buffer, void **device) {
    return fort_scope_device_reserve_many_v1(context, &buffer, 1, device);
}

int fort_scope_device_reserve_many_v1(fort_scope_t context, const fort_buffer_t *buffers, size_t count,
                                      void **devices) {
    return guarded([&] {
        Context *c = live_context(context);
        if (count && (!buffers || !devices)) raise(FORT_SCOPE_ARGUMENT, "null reservation arrays");
        std::vector<Buffer *> list;
        std::set<uint64_t> seen;
        for (size_t n = 0; n < count; ++n) {
            Buffer *b = find_buffer(c, buffers[n]);
            if (b->prepared != Buffer::NONE) raise(FORT_SCOPE_STATE, "reservation of an array inside an access");
            if (seen.insert(b->handle).second) list.push_back(b);
        }
        if (list.empty()) return FORT_SCOPE_OK;
        reserve(c, list, true);
        for (size_t n = 0; n < count; ++n) {
            const Buffer *b = find_buffer(c, buffers[n]);
            devices[n] = b->in_place ? b->mapped : b->device;
        }
        return FORT_SCOPE_OK;
    });
}

// ---- publication ----

int fort_scope_observe_v1(fort_scope_t context, const fort_buffer_t *buffers, size_t count) {
    return guarded([&] {
        Context *c = live_context(context);
        if (count && !buffers) raise(FORT_SCOPE_ARGUMENT, "null buffer list");
        std::vector<Buffer *> list;
        for (size_t n = 0; n < count; ++n) {
            Buffer *b = find_buffer(c, buffers[n]);
            if (b->prepared != Buffer::NONE) raise(FORT_SCOPE_STATE, "cannot observe under a prepared access");
            list.push_back(b);
        }
        for (size_t n = 0; n < list.size(); ++n)  // all checks before any publication
            for (size_t m = 0; m < n; ++m)
                if (list[m] == list[n]) raise(FORT_SCOPE_ALIAS, "a buffer is named twice in one observation");
        if (list.empty()) return FORT_SCOPE_OK;
        flush(c);
        bool any = false;
        for (Buffer *b : list) {
            b->host_touched = true;
            if (!b->device) continue;
            Region dirty = b->physical.clip(b->device_valid);
            dirty.remove(b->host_valid);
            if (!dirty.empty()) any = true;
            publish_buffer(c, b);
        }
        if (any || c->stream_ready) wait_stream(c);
        return FORT_SCOPE_OK;
    });
}

int fort_scope_observe_all_v1(fort_scope_t context) {
    std::vector<fort_buffer_t> all;
    {
        std::lock_guard<std::recursive_mutex> lock(g_mutex);
        auto it = g_contexts.find(context);
        if (it != g_contexts.end())
            for (auto &kv : it->second->domain->buffers) all.push_back(kv.first);
    }
    return fort_scope_observe_v1(context, all.data(), all.size());
}

static int drop_values(fort_scope_t context, fort_buffer_t buffer, bool recycle) {
    return guarded([&] {
        Context *c = live_context(context);
        Buffer *b = find_buffer(c, buffer);
        if (b->prepared != Buffer::NONE) raise(FORT_SCOPE_STATE, "cannot discard under a prepared access");
        if (recycle && b->queued) return FORT_SCOPE_OK; // the new definition replaces the values
        if (b->queued) flush(c);
        b->defined.clear();
        b->physical.clear();  // dead values: nothing of them is published
        return FORT_SCOPE_OK;
    });
}

int fort_scope_discard_v1(fort_scope_t context, fort_buffer_t buffer) { return drop_values(context, buffer, false); }
int fort_scope_recycle_v1(fort_scope_t context, fort_buffer_t buffer) { return drop_values(context, buffer, true); }

int fort_scope_retire_v1(fort_scope_t context, fort_buffer_t buffer) {
    return guarded([&] {
        Context *c = live_context(context);
        Buffer *b = find_buffer(c, buffer);
        if (b->prepared != Buffer::NONE) raise(FORT_SCOPE_STATE, "cannot retire under a prepared access");
        if (b->queued) flush(c);
        wait_stream(c);
        destroy_buffer(c, b);
        return FORT_SCOPE_OK;
    });
}

int fort_scope_unregister(fort_scope_t context, fort_buffer_t buffer) {
    return guarded([&] {
        Context *c = live_context(context);
        Buffer *b = find_buffer(c, buffer);
        if (b->prepared != Buffer::NONE) raise(FORT_SCOPE_STATE, "cannot unregister under a prepared access");
        flush(c);
        publish_buffer(c, b);
        wait_stream(c);
        destroy_buffer(c, b);
        return FORT_SCOPE_OK;
    });
}

int fort_scope_stats_get(fort_scope_t context, fort_scope_stats *stats) {
    return guarded([&] {
        if (!stats) raise(FORT_SCOPE_ARGUMENT, "null stats output");
        *stats = find_context(context)->domain->stats;
        return FORT_SCOPE_OK;
    });
}

int fort_scope_residency_stats_get_v1(fort_scope_t context, fort_scope_residency_stats_v1 *stats) {
    return guarded([&] {
        if (!stats) raise(FORT_SCOPE_ARGUMENT, "null stats output");
        *stats = find_context(context)->domain->residency;
        return FORT_SCOPE_OK;
    });
}

int fort_scope_completion_stats_get_v1(fort_scope_t context, fort_scope_completion_stats_v1 *stats) {
    return guarded([&] {
        if (!stats) raise(FORT_SCOPE_ARGUMENT, "null stats output");
        *stats = find_context(context)->completion;
        return FORT_SCOPE_OK;
    });
}

// ---- scratch ----

int fort_scope_scratch_acquire_v1(fort_scope_t context, size_t bytes, fort_scope_scratch_lease_v1 *lease) {
    return guarded([&] {
        if (!lease) raise(FORT_SCOPE_ARGUMENT, "null lease output");
        *lease = fort_scope_scratch_lease_v1{};  // a refused acquisition leaves a cleared lease
        Context *c = live_context(context);
        if (c->scratch_active) raise(FORT_SCOPE_STATE, "context already holds a scratch lease");
        if (bytes) {
            if (bytes > c->scratch_capacity) {
                const size_t grow = bytes - c->scratch_capacity;
                Domain *d = c->domain;
                // the arena fits beside what the domain holds, mirrors included (it evicts none of them), or
                // the lease is refused before the device is used
                if (d->budget_set && (claimed(d) > d->budget || grow > d->budget - claimed(d)))
                    raise(FORT_SCOPE_RESOURCE, "scratch lease exceeds the free device budget");
                ensure_stream(c);
                if (c->scratch) {
                    wait_stream(c); // complete earlier uses before the old arena is retired
                    release_scratch(c);
                    c->scratch_stats.grows++;
                }
                void *p = nullptr;
                if (Backend::scratch_alloc_fails() || !Backend::alloc(&p, bytes, c->stream))
                    raise(FORT_SCOPE_RESOURCE, "scratch allocation failed");
                c->scratch = p;
                c->scratch_capacity = bytes;
                c->domain->scratch_bytes += bytes;
                c->scratch_stats.allocations++;
                if (claimed(c->domain) > c->domain->peak_total_bytes) c->domain->peak_total_bytes = claimed(c->domain);
            } else {
                c->scratch_stats.reuses++;
            }
        }
        c->scratch_active = true;
        c->scratch_active_bytes = bytes;
        c->scratch_token = new_handle();
        c->scratch_stats.acquisitions++;
        if (bytes > c->scratch_stats.peak_scratch_bytes) c->scratch_stats.peak_scratch_bytes = bytes;
        lease->version = FORT_SCOPE_SCRATCH_ABI_VERSION;
        lease->reserved = 0;
        lease->token = c->scratch_token;
        lease->device = bytes ? c->scratch : nullptr;
        lease->bytes = bytes;
        lease->capacity = c->scratch_capacity;
        return FORT_SCOPE_OK;
    });
}

int fort_scope_scratch_release_v1(fort_scope_t context, uint64_t token) {
    return guarded([&] {
        Context *c = live_context(context);
        if (!c->scratch_active || token != c->scratch_token) raise(FORT_SCOPE_STALE, "not the active scratch lease");
        c->scratch_active = false;
        c->scratch_active_bytes = 0;
        c->scratch_stats.releases++;
        return FORT_SCOPE_OK;
    });
}

int fort_scope_scratch_stats_get_v1(fort_scope_t context, fort_scope_scratch_stats_v1 *stats) {
    return guarded([&] {
        if (!stats) raise(FORT_SCOPE_ARGUMENT, "null stats output");
        Context *c = find_context(context);
        *stats = c->scratch_stats;
        stats->version = FORT_SCOPE_SCRATCH_ABI_VERSION;
        stats->active = c->scratch_active;
        stats->capacity_bytes = c->scratch_capacity;
        stats->active_bytes = c->scratch_active_bytes;
        stats->peak_total_device_bytes = c->domain->peak_total_bytes;
        return FORT_SCOPE_OK;
    });
}

// ---- launches, queue and graphs ----

int fort_scope_gpu_enter(fort_scope_t context, int *previous_device, void **stream) {
    return guarded([&] {
        if (!previous_device || !stream) raise(FORT_SCOPE_ARGUMENT, "null output");
        Context *c = live_context(context);
        *previous_device = Backend::current();
        ensure_stream(c);
        if (!Backend::select(c->domain->device)) raise(FORT_SCOPE_RESOURCE, "cannot select device");
        *stream = (void *)c->stream;
        return FORT_SCOPE_OK;
    });
}

int fort_scope_gpu_leave(fort_scope_t context, int previous_device) {
    return guarded([&] {
        find_context(context);
        Backend::select(previous_device);
        return FORT_SCOPE_OK;
    });
}

int fort_scope_note_launch(fort_scope_t context) {
    return guarded([&] {
        Context *c = live_context(context);
        c->domain->stats.launches++;
        trace_line(c, "launch", 0, 0);
        return FORT_SCOPE_OK;
    });
}

int fort_scope_graph_enqueue_v1(fort_scope_t context, uint64_t code_key, const fort_scope_graph_task_v1 *task,
                                const size_t *argument_sizes) {
    return guarded([&] {
        if (!task) raise(FORT_SCOPE_ARGUMENT, "null task");
        Context *c = live_context(context);
        Task t = make_task(code_key, task->kernel, argument_sizes);
        std::vector<Bound> bound = bind_all(c, task->bindings, task->binding_count);
        accept(c, std::move(t), bound);
        return FORT_SCOPE_OK;
    });
}

int fort_scope_device_reserve_slabs_v1(fort_scope_t context, const fort_buffer_t *buffers, size_t count,
                                       void **devices, int *pipelined) {
    return guarded([&] {
        Context *c = live_context(context);
        if (!pipelined || (count && (!buffers || !devices))) raise(FORT_SCOPE_ARGUMENT, "null reservation arrays");
        *pipelined = 0;
        std::vector<Buffer *> list;
        std::set<uint64_t> seen;
        for (size_t n = 0; n < count; ++n) {
            Buffer *b = find_buffer(c, buffers[n]);
            if (b->prepared != Buffer::NONE) raise(FORT_SCOPE_STATE, "reservation of an array inside an access");
            if (seen.insert(b->handle).second) list.push_back(b);
        }
        if (list.empty()) return FORT_SCOPE_OK;
        const bool stream = streaming_allowed();
        bool any = false;
        for (Buffer *b : list) pin_for_device(c, b);
        for (Buffer *b : list) any = any || (stream && host_round(b));
        reserve(c, list, !stream);
        for (size_t n = 0; n < count; ++n) {
            const Buffer *b = find_buffer(c, buffers[n]);
            devices[n] = b->in_place ? b->mapped : b->device;
        }
        *pipelined = any ? 1 : 0;
        return FORT_SCOPE_OK;
    });
}

int fort_scope_slab_timing_set_v1(fort_scope_t context, int enabled) {
    return guarded([&] {
        Context *c = find_context(context);
        c->slab_timing = enabled != 0;
        if (!c->slab_timing) drop_slab_marks(c);
        return FORT_SCOPE_OK;
    });
}

int fort_scope_slab_timing_get_v1(fort_scope_t context, fort_scope_slab_timing_v1 *out) {
    return guarded([&] {
        if (!out) raise(FORT_SCOPE_ARGUMENT, "null slab timing output");
        Context *c = find_context(context);
        if (!c->slab_timing || c->slab_marks_used == 0) raise(FORT_SCOPE_STATE, "no timed slab sequence");
        fort_scope_slab_timing_v1 r{};
        r.version = 1;
        r.slabs = (uint32_t)c->slab_marks_used;
        auto span = [&](Backend::Event a, Backend::Event b) {
            float ms = 0.0f;
            if (!Backend::elapsed(a, b, &ms)) raise(FORT_SCOPE_EXECUTION, "timing events failed: " + Backend::last_error());
            return (double)ms;
        };
        // the sequence starts at its first upload (or its first kernel when nothing was uploaded) and ends
        // at the later of its last kernel and its last publication
        const auto &first = c->slab_marks[0];
        const Backend::Event origin = first.uploaded ? first.up0 : first.k0;
        for (size_t n = 0; n < c->slab_marks_used; ++n) {
            const auto &m = c->slab_marks[n];
            const double k = span(m.k0, m.k1);
            r.kernel_ms += k;
            r.longest_kernel_ms = std::max(r.longest_kernel_ms, k);
            r.span_ms = std::max(r.span_ms, span(origin, m.k1));
            if (m.uploaded) {
                const double u = span(m.up0, m.up1);
                r.upload_ms += u;
                r.longest_upload_ms = std::max(r.longest_upload_ms, u);
            }
            if (m.published) {
                const double p = span(m.p0, m.p1);
                r.publish_ms += p;
                r.longest_publish_ms = std::max(r.longest_publish_ms, p);
                r.span_ms = std::max(r.span_ms, span(origin, m.p1));
            }
        }
        *out = r;
        return FORT_SCOPE_OK;
    });
}

int fort_scope_numerics_set_v1(fort_scope_t context, int numerics) {
    return guarded([&] {
        if (numerics != FORT_SCOPE_NUMERICS_STRICT && numerics != FORT_SCOPE_NUMERICS_FAST)
            raise(FORT_SCOPE_ARGUMENT, "unknown numerical contract");
        find_context(context)->numerics = numerics;
        return FORT_SCOPE_OK;
    });
}

int fort_scope_host_pinning_set_v1(fort_scope_t context, int enabled) {
    return guarded([&] {
        if (enabled < -1 || enabled > 1) raise(FORT_SCOPE_ARGUMENT, "pinning is -1 (environment), 0 or 1");
        find_context(context)->pin_host = enabled;
        return FORT_SCOPE_OK;
    });
}

int fort_scope_numerics_get_v1(fort_scope_t context, int *numerics) {
    return guarded([&] {
        if (!numerics) raise(FORT_SCOPE_ARGUMENT, "null numerical contract output");
        *numerics = find_context(context)->numerics;
        return FORT_SCOPE_OK;
    });
}

int fort_scope_slab_enqueue_v1(fort_scope_t context, uint64_t code_key, const fort_scope_graph_task_v1 *tasks,
                               size_t count, const size_t *argument_sizes) {
    return guarded([&] {
        if (!tasks || count == 0 || count > kMaxSlabs) raise(FORT_SCOPE_ARGUMENT, "a slab sequence holds 1 to 64 tasks");
        Context *c = live_context(context);
        std::vector<Task> list;
        std::vector<std::vector<Bound>> bound;
        size_t offset = 0;
        for (size_t n = 0; n < count; ++n) {
            list.push_back(make_task(code_key, tasks[n].kernel, argument_sizes ? argument_sizes + offset : nullptr));
            offset += tasks[n].kernel.argument_count;
            bound.push_back(bind_all(c, tasks[n].bindings, tasks[n].binding_count));
            for (auto &x : bound.back())
                if ((!x.buffer->device && x.buffer->bytes) || x.buffer->in_place)
                    raise(FORT_SCOPE_STATE, "a slab task binds an array without reserved device storage");
        }
        run_slabs(c, list, bound);
        return FORT_SCOPE_OK;
    });
}

int fort_scope_graph_enqueue_members_v1(fort_scope_t context, uint64_t code_key, const fort_scope_kernel_v1 *kernel,
                                        const size_t *argument_sizes, const fort_scope_graph_member_v1 *members,
                                        size_t member_count) {
    return guarded([&] {
        if (!kernel || !member_count || !members) raise(FORT_SCOPE_ARGUMENT, "a merged launch needs members");
        Context *c = live_context(context);
        Task t = make_task(code_key, *kernel, argument_sizes);
        std::vector<std::vector<Bound>> each;
        for (size_t m = 0; m < member_count; ++m) each.push_back(bind_all(c, members[m].bindings, members[m].binding_count));
        // members must be independent on their actual sections
        for (size_t a = 0; a < each.size(); ++a)
            for (size_t b = a + 1; b < each.size(); ++b)
                for (auto &x : each[a])
                    for (auto &y : each[b]) {
                        if (x.buffer != y.buffer) continue;
                        Region rw_y = y.effects.reads;
                        rw_y.add(y.effects.writes);
                        Region rw_x = x.effects.reads;
                        rw_x.add(x.effects.writes);
                        if (!x.effects.writes.clip(rw_y).empty() || !y.effects.writes.clip(rw_x).empty())
                            raise(FORT_SCOPE_BOUNDARY, "members of a merged launch touch sections another member writes");
                    }
        std::vector<Bound> merged;
        for (auto &list : each)
            for (auto &x : list) {
                Bound *into = nullptr;
                for (auto &m : merged)
                    if (m.buffer == x.buffer) into = &m;
                if (!into) {
                    merged.push_back(x);
                    continue;
                }
                into->effects.reads.add(x.effects.reads);
                into->effects.writes.add(x.effects.writes);
                into->effects.overwrites.add(x.effects.overwrites);
            }
        accept(c, std::move(t), merged);
        return FORT_SCOPE_OK;
    });
}

int fort_scope_graph_flush_v1(fort_scope_t context) {
    return guarded([&] {
        Context *c = live_context(context);
        if (!c->pending.empty()) c->queue_stats.explicit_flushes++;
        flush(c);
        return FORT_SCOPE_OK;
    });
}

int fort_scope_graph_queue_cancel_v1(fort_scope_t context) {
    return guarded([&] {
        Context *c = live_context(context);
        // the queued tasks never run: every array they touched gets back its state from before them (values
        // their uploads already moved stay on the device, no longer counted as current there)
        for (auto &kv : c->queued_before) {
            auto it = c->domain->buffers.find(kv.first);
            if (it == c->domain->buffers.end()) continue;
            Buffer *b = it->second.get();
            b->defined = kv.second.defined;
            b->host_valid = kv.second.host_valid;
            b->device_valid = kv.second.device_valid;
            b->physical = kv.second.physical;
            b->host_touched = kv.second.host_touched;
            b->host_rounds = kv.second.host_rounds;
            b->queued = 0;
            b->awaits_token = false;
        }
        c->queued_before.clear();
        c->awaiting_token.clear();
        c->pending.clear();
        c->pending_threads = 0;
        c->queue_stats.pending_tasks = 0;
        return FORT_SCOPE_OK;
    });
}

int fort_scope_graph_queue_stats_get_v1(fort_scope_t context, fort_scope_graph_queue_stats_v1 *stats) {
    return guarded([&] {
        if (!stats) raise(FORT_SCOPE_ARGUMENT, "null stats output");
        *stats = find_context(context)->queue_stats;
        return FORT_SCOPE_OK;
    });
}

int fort_scope_graph_submit_v1(fort_scope_t context, uint64_t group_key, const fort_scope_kernel_v1 *kernels,
                               size_t count) {
    return guarded([&] {
        Context *c = live_context(context);
        if (count && !kernels) raise(FORT_SCOPE_ARGUMENT, "null kernels");
        if (!count) return FORT_SCOPE_OK;
        if (!group_key) raise(FORT_SCOPE_ARGUMENT, "a kernel group needs a nonzero key");
        std::vector<Task> tasks;
        for (size_t n = 0; n < count; ++n) {
            Task t;
            t.spec = spec_of(kernels[n]);
            for (size_t a = 0; a < kernels[n].argument_count; ++a) t.spec.arguments.push_back(kernels[n].arguments[a]);
            tasks.push_back(std::move(t));
        }
        flush(c);
        c->untracked = true;  // kernels without bindings: host accesses wait for the stream
        std::vector<LaunchSpec> specs;
        for (auto &t : tasks) specs.push_back(std::move(t.spec));
        submit_group(c, specs, group_key);
        return FORT_SCOPE_OK;
    });
}

// Checked graph execution: the tasks' effects are simulated in order on
// private copies of each array's definition and device coherence, so a task
// may read what an earlier task of the group defines. Only what the group
// needs from the host (reads not defined inside the group and not current on
// the device) is uploaded, after every queued task; then the kernels launch in
// order on the context stream (their argument values are read as each launch is
// made, so the records need no argument sizes), and the final definitions and
// coherence are committed. Nothing changes unless every task validates. Every
// array needs reserved device storage; none may be under a prepared access.
int fort_scope_graph_execute_v1(fort_scope_t context, uint64_t group_key, const fort_scope_graph_task_v1 *tasks,
                                size_t count) {
    return guarded([&] {
        Context *c = live_context(context);
        if (count && !tasks) raise(FORT_SCOPE_ARGUMENT, "null tasks");
        if (!count) return FORT_SCOPE_OK;
        if (!group_key) raise(FORT_SCOPE_ARGUMENT, "a graph group needs a stable key");
        struct Sim {
            Region defined, device, upload;
        };
        std::map<Buffer *, Sim> sim;
        std::vector<LaunchSpec> list;
        std::vector<std::vector<Bound>> bound(count);
        for (size_t n = 0; n < count; ++n) {
            const fort_scope_graph_task_v1 &t = tasks[n];
            list.push_back(spec_of(t.kernel));
            for (size_t a = 0; a < t.kernel.argument_count; ++a) {
                if (!t.kernel.arguments[a]) raise(FORT_SCOPE_ARGUMENT, "empty kernel argument");
                list.back().arguments.push_back(t.kernel.arguments[a]);
            }
            if (t.binding_count && !t.bindings) raise(FORT_SCOPE_ARGUMENT, "null bindings");
            std::set<uint64_t> seen;
            for (size_t i = 0; i < t.binding_count; ++i) {
                Buffer *b = find_buffer(c, t.bindings[i].buffer);
                if (!seen.insert(b->handle).second) raise(FORT_SCOPE_ALIAS, "a task binds one array twice");
                if (b->prepared != Buffer::NONE) raise(FORT_SCOPE_STATE, "array already has a prepared access");
                if ((!b->device && b->bytes) || b->in_place)
                    raise(FORT_SCOPE_STATE, "task binds an array whose device storage is not reserved");
                Effects e = effects_of(b, t.bindings[i].access);
                auto it = sim.find(b);
                if (it == sim.end()) it = sim.emplace(b, Sim{b->defined, b->device_valid, Region{}}).first;
                Sim &st = it->second;
                for (const auto &box : e.reads.boxes)
                    if (!st.defined.covers(box))
                        raise(FORT_SCOPE_UNINITIALIZED, "a task reads array values that were never defined");
                Region need = e.reads;
                Region partial = e.writes;
                partial.remove(e.overwrites);
                need.add(partial);
                need = st.defined.clip(need);
                need.remove(st.device);
                st.upload.add(need);
                st.device.add(need);
                st.device.add(e.writes);
                st.defined.add(e.overwrites);
                bound[n].push_back({b, std::move(e)});
            }
        }
        flush(c);
        ensure_stream(c);
        for (auto &kv : sim) {
            Buffer *b = kv.first;
            Region up = kv.second.upload;
            up.remove(b->device_valid);
            if (up.empty()) continue;
            const Region moved = widened(b, up, true);
            copy_region(c, b, moved, true);
            Region device = b->device_valid;
            device.add(up);
            device.add(b->host_valid.clip(moved));
            settle(c, b, b->defined, b->host_valid, device);
        }
        c->untracked = true;  // host accesses after a checked group wait for the stream
        submit_group(c, list, group_key);
        for (auto &tb : bound)
            for (auto &x : tb) device_commit(c, x.buffer, x.effects.writes, x.effects.overwrites);
        for (auto &kv : sim) note_device_use(kv.first);
        c->queue_stats.accepted_tasks += count;
        return FORT_SCOPE_OK;
    });
}

int fort_scope_graph_stats_get_v1(fort_scope_t context, fort_scope_graph_stats_v1 *stats) {
    return guarded([&] {
        if (!stats) raise(FORT_SCOPE_ARGUMENT, "null stats output");
        *stats = find_context(context)->graph_stats;
        return FORT_SCOPE_OK;
    });
}

// A checked opaque device transaction: the bindings are validated (known,
// distinct, of the declared type, rank and element size, not under a prepared
// access, reads defined) before anything moves; storage is reserved and what
// the bindings read is uploaded after every queued task; the worker gets views
// of the device copies and the context stream. It must report started = 0 when
// it rejects the call before enqueuing anything, and started = 1 before its
// first enqueue. Success (with started = 1) commits the bindings' exact effects;
// a rejection before start changes no value; anything else after start poisons
// the context, since the device may hold half-done work.
int fort_scope_external_execute_v1(fort_scope_t context, const fort_scope_external_call_v1 *call,
                                   fort_scope_external_worker_v1 worker, void *user,
                                   fort_scope_external_report_v1 *report) {
    if (report) {
        report->version = FORT_SCOPE_EXTERNAL_ABI_VERSION;
        report->status = FORT_SCOPE_OK;
        report->started = 0;
        report->committed = 0;
    }
    const int status = guarded([&] {
        if (!call || !report || call->version != FORT_SCOPE_EXTERNAL_ABI_VERSION || call->reserved ||
            (call->binding_count && (!call->bindings || !worker)))
            raise(FORT_SCOPE_ARGUMENT, "invalid external transaction");
        Context *c = live_context(context);
        if (!call->binding_count) return FORT_SCOPE_OK;
        if (call->workspace_lease) {
            auto lease = c->domain->workspaces.find(call->workspace_lease);
            if (lease == c->domain->workspaces.end()) raise(FORT_SCOPE_STALE, "foreign or stale external workspace lease");
            if (call->workspace_bytes > lease->second) raise(FORT_SCOPE_RESOURCE, "external workspace claim is too small");
        } else if (call->workspace_bytes) {
            raise(FORT_SCOPE_ARGUMENT, "an external workspace needs a workspace lease");
        }
        const size_t n = call->binding_count;
        std::vector<fort_scope_plan_binding> plan(n);
        std::set<uint64_t> seen;
        for (size_t i = 0; i < n; ++i) {
            const fort_scope_external_binding_v1 &x = call->bindings[i];
            Buffer *b = find_buffer(c, x.buffer);
            if (!seen.insert(b->handle).second) raise(FORT_SCOPE_ALIAS, "external transaction repeats an array");
            if (x.type != b->type || (int)x.rank != b->rank || x.element_bytes != b->elem)
                raise(FORT_SCOPE_ARGUMENT, "external transaction type or rank mismatch");
            plan[i] = {x.buffer, x.access};
        }
        std::vector<Bound> bound = bind_all(c, plan.data(), n);
        std::vector<Buffer *> list;
        for (auto &x : bound) list.push_back(x.buffer);
        flush(c);
        reserve(c, list, false);
        device_acquire(c, bound);
        std::vector<fort_scope_external_view_v1> views(n);
        std::vector<std::vector<size_t>> strides(n);
        for (size_t i = 0; i < n; ++i) {
            Buffer *b = bound[i].buffer;
            strides[i].resize((size_t)b->rank);
            size_t stride = b->elem;
            for (int d = 0; d < b->rank; ++d) {
                strides[i][(size_t)d] = stride;
                stride *= b->extents[d];
            }
            views[i] = {b->handle, b->generation, b->type, (uint32_t)b->rank, b->elem, b->bytes, b->extents,
                        strides[i].data(), b->lower, b->device};
        }
        int started = -1, result = FORT_SCOPE_EXECUTION;
        try {
            result = worker(user, views.data(), n, Backend::cpu ? nullptr : (void *)c->stream, &started);
        } catch (...) {  // a provider that throws may have submitted work: contained, and never replayed
            report->started = 1;
            poison(c, "external provider threw an exception");
        }
        report->started = started == 0 ? 0u : 1u;
        const bool known = result >= FORT_SCOPE_ARGUMENT && result <= FORT_SCOPE_STATE && result != FORT_SCOPE_EXECUTION;
        if ((started != 0 && started != 1) || (result == FORT_SCOPE_OK && started != 1) ||
            (result != FORT_SCOPE_OK && (started != 0 || !known)))
            poison(c, "external execution failed or did not report its submission state");
        if (result != FORT_SCOPE_OK) raise(result, "external provider rejected the call before submission");
        if (Backend::external_commit_fails()) poison(c, "external provider effects could not be committed");
        for (auto &x : bound) {
            device_commit(c, x.buffer, x.effects.writes, x.effects.overwrites);
            note_device_use(x.buffer);
        }
        count_external_launch(c);
        report->committed = 1;
        trace_line(c, "external_commit", 0, n);
        return FORT_SCOPE_OK;
    });
    if (report) report->status = status;
    return status;
}

} // extern "C"
