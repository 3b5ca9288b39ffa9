// Continuous-batching server for advection jobs (include/f2c_serve.h).
//
// Structure, GB300-first:
//  * Residency: every admitted job registers two sets of arrays (ping-pong) in
//    the residency domain of the server's context and holds them under one
//    device access (fort_scope_access_begin_v1, whole arrays overwritten on the
//    device) from admission to retirement; its first set is defined on the
//    device by f2c_seed_fields_v1. At retirement the access ends, the final set
//    is published to host memory when the job asked for it, and every array
//    leaves the domain without a download (fort_scope_retire_v1).
//  * Admission by free device memory: the driver's free bytes plus the bytes
//    the stream-ordered pool holds unused, less a reserve, and the domain's
//    unclaimed budget must both cover the job.
//  * Ticks run on the server's own stream, ordered after the context stream
//    (where mirrors are allocated and seeded) by events. The runtime's calls
//    that wait for the context stream therefore never wait for ticks.
//  * A selection (jobs with the least remaining work, up to tick_points points)
//    is planned once: per scalar count one persistent batched plan (a filled
//    advance: the step and its boundary fill in one launch) for each of two
//    consecutive ticks, in fixed device workspace slots staged through
//    pinned host slots. The two ticks are captured as one CUDA graph, each
//    scalar group's chain on a branch of its own so that the groups' launches
//    overlap, and replayed while the selection holds; a one-tick graph serves
//    an odd remainder. The eight most recent selections stay cached.
//  * One worker thread issues bursts of ticks and keeps at most `depth` of them
//    in flight; completion is seen through one event per burst.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <exception>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../../include/f2c_batch.h"
#include "../../../include/f2c_serve.h"

namespace f2c::serve {
namespace {

constexpr int kMaxFields = 3 + F2C_MAX_SCALARS;
constexpr size_t kSlotBytes = size_t(1) << 20;  // one batched plan (descriptors + tile queue)
constexpr int kSlots = 64;
constexpr size_t kCachedSelections = 8;
using Clock = std::chrono::steady_clock;

struct Job {
    uint64_t id = 0;
    f2c_serve_job_v1 spec{};
    f2c_grid_v1 grid{};
    int fields = 0;
    size_t field_bytes = 0, bytes = 0;
    int done = 0;  // steps issued
    double admitted = -1.0, finished = -1.0;
    int status = 0;
    void *host[2][kMaxFields] = {};
    fort_buffer_t handle[2][kMaxFields] = {};
    double *dev[2][kMaxFields] = {};
    bool in_access = false;
    int result_set = -1;  // host set holding the published result (KEEP_RESULT)
    uint64_t points() const { return (uint64_t)spec.nx * spec.ny * spec.nz; }
    uint64_t remaining() const { return (uint64_t)(spec.steps - done) * points(); }
};

struct Plan {
    f2c_batch_plan_v1 plan{};
    int slot = -1;
};

// A cached selection: the jobs and the parity of each at its first tick.
struct Selection {
    std::vector<std::pair<uint64_t, int>> key;
    std::vector<Job *> jobs;
    std::vector<Plan> ticks[2];  // per scalar group, first and second tick
    cudaGraphExec_t two = nullptr, one = nullptr;
    uint64_t last_seq = 0, last_use = 0;
    uint64_t points = 0;
};

struct Burst {
    uint64_t seq;
    cudaEvent_t event;
    std::vector<Job *> finishing;
};

struct Server {
    fort_scope_t context = 0;
    fort_scope_domain_t domain = 0;
    f2c_serve_options_v1 opt{};
    Clock::time_point start;
    std::thread worker;

    std::mutex lock;  // guards the fields below up to `stats`
    std::condition_variable wake, finished_cv;
    bool stop = false;
    std::multimap<double, std::unique_ptr<Job>> submitted;  // by arrival
    uint64_t next_id = 1, outstanding = 0;
    std::deque<f2c_serve_done_v1> done;
    std::map<uint64_t, std::unique_ptr<Job>> results;
    int failure = 0;
    std::string error;
    f2c_serve_stats_v1 stats{};  // published copy of `counts`

    // worker state
    f2c_serve_stats_v1 counts{};
    cudaStream_t ctx_stream = nullptr, stream = nullptr, capture = nullptr;
    cudaStream_t branch[F2C_MAX_SCALARS] = {};  // capture branches of the scalar groups after the first
    char *slot_device = nullptr, *slot_host = nullptr;
    std::vector<uint64_t> slot_busy_until;  // burst sequence after which a free slot may be rewritten
    std::vector<bool> slot_used;
    uint64_t workspace_lease = 0;
    std::vector<std::unique_ptr<Job>> active;
    std::vector<std::unique_ptr<Selection>> cache;
    std::deque<Burst> inflight;
    std::vector<cudaEvent_t> spare_events;
    uint64_t seq = 0, completed = 0, use = 0;
    uint64_t resident_bytes = 0;
    int sms = 152;

    double now() const { return std::chrono::duration<double>(Clock::now() - start).count(); }
};

std::mutex g_servers_lock;
std::map<uint64_t, Server *> g_servers;
uint64_t g_next_server = 1;
thread_local std::string t_error;

int fail(int status, const std::string &message) {
    t_error = message;
    return status;
}

Server *find(f2c_server_t handle) {
    std::lock_guard<std::mutex> g(g_servers_lock);
    auto it = g_servers.find(handle);
    return it == g_servers.end() ? nullptr : it->second;
}

struct Failure {
    int status;
    std::string message;
};
[[noreturn]] void raise(int status, const std::string &message) { throw Failure{status, message}; }

void cuda(cudaError_t e, const char *what) {
    if (e != cudaSuccess) raise(FORT_SCOPE_EXECUTION, std::string(what) + ": " + cudaGetErrorString(e));
}
void runtime(int status, const char *what) {
    if (status != FORT_SCOPE_OK) raise(status, std::string(what) + ": " + fort_scope_error());
}
void kernel(int status, const char *what) {
    if (status != 0) raise(status, std::string(what) + ": " + f2c_last_error());
}

// z-chunk depth of a tick's batch: deep chunks (up to 32 levels) while the tick holds work for four CTAs per
// SM, shallower ones (down to 2) for small ticks, so that their tiles still reach every SM
int chunk_depth(const std::vector<Job *> &jobs, int sms) {
    uint64_t columns = 0;
    for (const Job *j : jobs)
        columns += (uint64_t)((j->spec.nx + 31) / 32) * ((j->spec.ny + 7) / 8) * j->spec.nz;
    const uint64_t per = (columns + 4 * (uint64_t)sms - 1) / (4 * (uint64_t)sms);
    return (int)std::min<uint64_t>(32, std::max<uint64_t>(2, per));
}

// ---- burst completion -------------------------------------------------------------------------

void release_job(Server *s, Job *j);

void complete_front(Server *s) {
    Burst b = std::move(s->inflight.front());
    s->inflight.pop_front();
    s->completed = b.seq;
    s->spare_events.push_back(b.event);
    for (Job *j : b.finishing) release_job(s, j);
}

// Handle every completed burst; with `block`, wait for the oldest one first.
void reap(Server *s, bool block) {
    while (!s->inflight.empty()) {
        cudaEvent_t e = s->inflight.front().event;
        if (block) {
            cuda(cudaEventSynchronize(e), "burst wait");
            block = false;
        } else {
            const cudaError_t q = cudaEventQuery(e);
            if (q == cudaErrorNotReady) {
                (void)cudaGetLastError();
                return;
            }
            cuda(q, "burst query");
        }
        complete_front(s);
    }
}

void wait_for(Server *s, uint64_t seq) {
    while (s->completed < seq && !s->inflight.empty()) reap(s, true);
}

// ---- jobs ----------------------------------------------------------------------------------------

void finish_job(Server *s, std::unique_ptr<Job> owned, int status, const std::string &message) {
    Job *j = owned.get();
    j->status = status;
    j->finished = s->now();
    std::lock_guard<std::mutex> g(s->lock);
    if (status != FORT_SCOPE_OK && !s->failure) {
        s->failure = status;
        s->error = message;
    }
    s->done.push_back({j->id, j->spec.arrival, j->admitted, j->finished, status, 0});
    s->counts.finished++;
    s->stats = s->counts;
    if (j->result_set >= 0) s->results[j->id] = std::move(owned);
    --s->outstanding;
    s->finished_cv.notify_all();
}

void free_host(Job *j, int keep_set) {
    for (int set = 0; set < 2; ++set) {
        if (set == keep_set) continue;
        for (int f = 0; f < j->fields; ++f) {
            std::free(j->host[set][f]);
            j->host[set][f] = nullptr;
        }
    }
}

// Leave the domain: end the access, publish the final set if asked, drop every array without a download.
void release_arrays(Server *s, Job *j, bool publish) {
    if (j->in_access) {
        for (int set = 0; set < 2; ++set)
            for (int f = 0; f < j->fields; ++f) runtime(fort_scope_device_end(s->context, j->handle[set][f]), "end of access");
        j->in_access = false;
    }
    const int final_set = j->spec.steps % 2;
    if (publish) {
        runtime(fort_scope_observe_v1(s->context, j->handle[final_set], (size_t)j->fields), "result publication");
        j->result_set = final_set;
    }
    for (int set = 0; set < 2; ++set)
        for (int f = 0; f < j->fields; ++f)
            if (j->handle[set][f]) {
                runtime(fort_scope_retire_v1(s->context, j->handle[set][f]), "array retirement");
                j->handle[set][f] = 0;
            }
    s->resident_bytes -= j->bytes;
}

// Selections that name a job are dropped with it (their graphs would address its freed arrays).
void drop_selections_of(Server *s, const Job *j);
void destroy_selection(Server *s, std::unique_ptr<Selection> sel);

void release_job(Server *s, Job *j) {
    drop_selections_of(s, j);
    auto it = std::find_if(s->active.begin(), s->active.end(), [&](const std::unique_ptr<Job> &p) { return p.get() == j; });
    std::unique_ptr<Job> owned = std::move(*it);
    s->active.erase(it);
    const bool keep = (j->spec.flags & F2C_SERVE_KEEP_RESULT) != 0;
    release_arrays(s, j, keep);
    free_host(j, keep ? j->result_set : -1);
    finish_job(s, std::move(owned), FORT_SCOPE_OK, "");
}

size_t job_bytes(const f2c_serve_job_v1 &spec) {
    const size_t padded = (size_t)(spec.nx + 2 * spec.halo) * (spec.ny + 2 * spec.halo) * (spec.nz + 2 * spec.halo);
    return 2 * (size_t)(3 + spec.nscalar) * padded * sizeof(double);
}

// Free device memory for a new job: the driver's free bytes, plus what the device's stream-ordered pool
// holds unused, less the reserve.
uint64_t device_room(Server *s) {
    size_t free_bytes = 0, total = 0;
    cuda(cudaMemGetInfo(&free_bytes, &total), "device memory query");
    int device = 0;
    cuda(cudaGetDevice(&device), "device query");
    cudaMemPool_t pool;
    uint64_t reserved = 0, used = 0;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved);
        cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used);
    }
    (void)cudaGetLastError();
    const uint64_t reserve = s->opt.reserve_bytes ? s->opt.reserve_bytes
                                                  : std::max<uint64_t>(total / 16, uint64_t(512) << 20);
    const uint64_t room = (uint64_t)free_bytes + (reserved > used ? reserved - used : 0);
    return room > reserve ? room - reserve : 0;
}

bool fits(Server *s, const Job &j) {
    if (s->active.size() >= s->opt.max_active) return false;
    if (s->opt.budget_bytes && s->resident_bytes + j.bytes > s->opt.budget_bytes) return false;
    size_t budget = 0, unclaimed = 0;
    runtime(fort_scope_domain_budget_get_v1(s->domain, &budget, &unclaimed), "domain budget");
    if (j.bytes > unclaimed) return false;
    return j.bytes <= device_room(s);
}

// Register both sets, open the device access, seed the first set on the context stream.
void admit(Server *s, Job *j) {
    const f2c_serve_job_v1 &p = j->spec;
    const size_t ext[3] = {(size_t)(p.nx + 2 * p.halo), (size_t)(p.ny + 2 * p.halo), (size_t)(p.nz + 2 * p.halo)};
    const int64_t lower[3] = {1, 1, 1};
    std::vector<fort_scope_plan_binding> bindings;
    for (int set = 0; set < 2; ++set)
        for (int f = 0; f < j->fields; ++f) {
            // host storage for the registration: never touched unless the result is published into it
            void *h = std::malloc(j->field_bytes);
            if (!h) raise(FORT_SCOPE_RESOURCE, "host memory for a job's arrays");
            j->host[set][f] = h;
            fort_scope_layout layout{3, FORT_SCOPE_REAL64, sizeof(double), h, ext, lower, 1};
            runtime(fort_scope_register(s->context, (uint64_t)(uintptr_t)h, 1, &layout, 0, &j->handle[set][f]),
                    "registration");
            fort_scope_plan_binding b{};
            b.buffer = j->handle[set][f];
            b.access.flags = FORT_SCOPE_WRITE_ALL | FORT_SCOPE_OVERWRITE_ALL;
            bindings.push_back(b);
        }
    std::vector<void *> devices(bindings.size());
    runtime(fort_scope_access_begin_v1(s->context, bindings.data(), bindings.size(), 1, devices.data()),
            "device access");
    j->in_access = true;
    for (int set = 0; set < 2; ++set)
        for (int f = 0; f < j->fields; ++f) j->dev[set][f] = static_cast<double *>(devices[(size_t)set * j->fields + f]);
    kernel(f2c_seed_fields_v1(&j->grid, p.seed, p.nscalar, j->dev[0], s->ctx_stream), "job seeding");
    s->resident_bytes += j->bytes;
}

void admit_arrivals(Server *s) {
    bool any = false;
    for (;;) {
        std::unique_ptr<Job> job;
        {
            std::lock_guard<std::mutex> g(s->lock);
            if (s->submitted.empty() || s->submitted.begin()->first > s->now()) break;
            Job &j = *s->submitted.begin()->second;
            if (!fits(s, j)) {
                s->counts.refused_admissions++;
                if (!s->active.empty() || !s->inflight.empty()) break;
                // nothing resident frees memory for it: it never fits
                job = std::move(s->submitted.begin()->second);
                s->submitted.erase(s->submitted.begin());
                job->admitted = s->now();
            } else {
                job = std::move(s->submitted.begin()->second);
                s->submitted.erase(s->submitted.begin());
            }
        }
        if (job->admitted >= 0) {
            finish_job(s, std::move(job), FORT_SCOPE_RESOURCE, "a job does not fit the device on its own");
            continue;
        }
        job->admitted = s->now();
        try {
            admit(s, job.get());
        } catch (const Failure &f) {
            if (job->in_access)
                for (int set = 0; set < 2; ++set)
                    for (int n = 0; n < job->fields; ++n) (void)fort_scope_cancel_access(s->context, job->handle[set][n]);
            for (int set = 0; set < 2; ++set)
                for (int n = 0; n < job->fields; ++n)
                    if (job->handle[set][n]) (void)fort_scope_retire_v1(s->context, job->handle[set][n]);
            free_host(job.get(), -1);
            finish_job(s, std::move(job), f.status, f.message);
            throw;
        }
        s->counts.admitted++;
        s->active.push_back(std::move(job));
        s->counts.peak_active = std::max<uint64_t>(s->counts.peak_active, s->active.size());
        s->counts.peak_job_bytes = std::max<uint64_t>(s->counts.peak_job_bytes, s->resident_bytes);
        any = true;
    }
    if (any) {  // ticks order after the seeding
        cudaEvent_t e;
        cuda(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
        cuda(cudaEventRecord(e, s->ctx_stream), "seed event");
        cuda(cudaStreamWaitEvent(s->stream, e, 0), "seed order");
        cudaEventDestroy(e);
    }
}

// ---- selections, plans and graphs ---------------------------------------------------------------

int take_slot(Server *s) {
    for (;;) {
        for (int n = 0; n < kSlots; ++n)
            if (!s->slot_used[(size_t)n] && s->slot_busy_until[(size_t)n] <= s->completed) {
                s->slot_used[(size_t)n] = true;
                return n;
            }
        // a free slot whose last reader is still in flight: wait for it
        uint64_t soonest = UINT64_MAX;
        for (int n = 0; n < kSlots; ++n)
            if (!s->slot_used[(size_t)n]) soonest = std::min(soonest, s->slot_busy_until[(size_t)n]);
        if (soonest != UINT64_MAX) {
            wait_for(s, soonest);
            continue;
        }
        // every slot belongs to a cached selection: drop the least recently used one (not in use now)
        if (s->cache.empty()) raise(FORT_SCOPE_RESOURCE, "no plan slot free");
        auto victim = std::min_element(s->cache.begin(), s->cache.end(),
                                       [](const std::unique_ptr<Selection> &a, const std::unique_ptr<Selection> &b) {
                                           return a->last_use < b->last_use;
                                       });
        std::unique_ptr<Selection> sel = std::move(*victim);
        s->cache.erase(victim);
        destroy_selection(s, std::move(sel));
    }
}

void destroy_selection(Server *s, std::unique_ptr<Selection> sel) {
    for (auto &tick : sel->ticks)
        for (Plan &p : tick)
            if (p.slot >= 0) {
                s->slot_used[(size_t)p.slot] = false;
                s->slot_busy_until[(size_t)p.slot] = sel->last_seq;
            }
    // an executable graph still in flight is freed by the driver when its launches complete
    if (sel->two) cudaGraphExecDestroy(sel->two);
    if (sel->one) cudaGraphExecDestroy(sel->one);
}

void drop_selections_of(Server *s, const Job *j) {
    for (size_t n = 0; n < s->cache.size();) {
        const auto &jobs = s->cache[n]->jobs;
        if (std::find(jobs.begin(), jobs.end(), j) != jobs.end()) {
            std::unique_ptr<Selection> sel = std::move(s->cache[n]);
            s->cache.erase(s->cache.begin() + (long)n);
            destroy_selection(s, std::move(sel));
        } else {
            ++n;
        }
    }
}

// One tick's batched plans of `jobs` (grouped by scalar count), each job at parity done + t.
void plan_tick(Server *s, Selection &sel, int t) {
    std::map<int, std::vector<Job *>> groups;
    for (Job *j : sel.jobs) groups[j->spec.nscalar].push_back(j);
    const bool fast = [&] {
        int numerics = 0;
        return fort_scope_numerics_get_v1(s->context, &numerics) == FORT_SCOPE_OK && numerics == FORT_SCOPE_NUMERICS_FAST;
    }();
    for (auto &kv : groups) {
        const std::vector<Job *> &jobs = kv.second;
        std::vector<f2c_grid_v1> grids;
        std::vector<f2c_fields_v1> fields;
        const int kz = chunk_depth(jobs, s->sms);
        std::vector<int32_t> depth(jobs.size(), kz);
        for (Job *j : jobs) {
            const int src = (j->done + t) % 2, dst = 1 - src;
            f2c_fields_v1 f{};
            f.u = j->dev[src][0]; f.v = j->dev[src][1]; f.w = j->dev[src][2];
            f.ut = j->dev[dst][0]; f.vt = j->dev[dst][1]; f.wt = j->dev[dst][2];
            f.nscalar = j->spec.nscalar;
            f.mode = F2C_ADVANCE_FILLED;  // the step and its boundary fill in one launch
            f.dt = j->spec.dt;
            for (int n = 0; n < j->spec.nscalar; ++n) {
                f.s[n] = j->dev[src][3 + n];
                f.st[n] = j->dev[dst][3 + n];
            }
            grids.push_back(j->grid);
            fields.push_back(f);
        }
        const size_t need = f2c_batch_workspace_bytes_v1(grids.data(), depth.data(), (int32_t)jobs.size());
        if (need > kSlotBytes) raise(FORT_SCOPE_RESOURCE, "a tick's plan exceeds its workspace slot");
        Plan p;
        p.slot = take_slot(s);
        sel.ticks[t].push_back(p);  // owned by the selection from here (its slot is returned with it)
        Plan &q = sel.ticks[t].back();
        kernel(f2c_batch_prepare_async_v1(grids.data(), fields.data(), depth.data(), (int32_t)jobs.size(),
                                          s->slot_device + (size_t)q.slot * kSlotBytes, kSlotBytes,
                                          s->slot_host + (size_t)q.slot * kSlotBytes, s->stream, &q.plan),
               "tick plan");
        if (fast) q.plan.reserved |= F2C_BATCH_FAST_FP;
        s->counts.plan_builds++;
    }
}

void launch_tick(const Selection &sel, int t, cudaStream_t stream) {
    for (const Plan &p : sel.ticks[t]) kernel(f2c_batch_step_v1(&p.plan, stream), "tick step");
}

// The selection's ticks as one graph. Each scalar group's ticks form a chain of its own (a job depends on
// nothing but itself), captured on a stream of its own: the groups' persistent launches run side by side,
// so that one group's tail overlaps another's work.
cudaGraphExec_t capture(Server *s, const Selection &sel, int ticks) {
    const size_t groups = sel.ticks[0].size();
    std::vector<cudaEvent_t> marks;
    auto mark = [&](cudaStream_t st) {
        cudaEvent_t e;
        cuda(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "capture event");
        marks.push_back(e);
        cuda(cudaEventRecord(e, st), "capture fork/join");
        return e;
    };
    cuda(cudaStreamBeginCapture(s->capture, cudaStreamCaptureModeThreadLocal), "capture begin");
    try {
        const cudaEvent_t fork = mark(s->capture);
        for (size_t g = 1; g < groups; ++g) cuda(cudaStreamWaitEvent(s->branch[g - 1], fork, 0), "capture fork");
        for (size_t g = 0; g < groups; ++g) {
            const cudaStream_t st = g ? s->branch[g - 1] : s->capture;
            for (int t = 0; t < ticks; ++t) {
                kernel(f2c_batch_step_v1(&sel.ticks[t][g].plan, st), "tick step");
            }
        }
        for (size_t g = 1; g < groups; ++g) cuda(cudaStreamWaitEvent(s->capture, mark(s->branch[g - 1]), 0), "capture join");
    } catch (...) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(s->capture, &g);
        if (g) cudaGraphDestroy(g);
        for (cudaEvent_t e : marks) cudaEventDestroy(e);
        throw;
    }
    cudaGraph_t graph = nullptr;
    const cudaError_t end = cudaStreamEndCapture(s->capture, &graph);
    for (cudaEvent_t e : marks) cudaEventDestroy(e);
    cuda(end, "capture end");
    cudaGraphExec_t exec = nullptr;
    const cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    cuda(e, "graph instantiation");
    s->counts.graph_builds++;
    return exec;
}

// Jobs whose last step is issued stay in `active` until their burst completes, but are not selected again.
std::vector<Job *> select_jobs(Server *s) {
    std::vector<Job *> ready;
    for (auto &j : s->active)
        if (j->done < j->spec.steps) ready.push_back(j.get());
    // jobs waiting longer than starve_s go first, oldest first; the others by least remaining work
    const double starving_before = s->opt.starve_s > 0 ? s->now() - s->opt.starve_s : -1e300;
    std::sort(ready.begin(), ready.end(), [&](const Job *a, const Job *b) {
        const bool sa = a->spec.arrival < starving_before, sb = b->spec.arrival < starving_before;
        if (sa != sb) return sa;
        if (sa && a->spec.arrival != b->spec.arrival) return a->spec.arrival < b->spec.arrival;
        return a->remaining() != b->remaining() ? a->remaining() < b->remaining() : a->id < b->id;
    });
    std::vector<Job *> chosen;
    uint64_t total = 0;
    for (Job *j : ready) {
        if (!chosen.empty() && total >= s->opt.tick_points) break;
        chosen.push_back(j);
        total += j->points();
    }
    return chosen;
}

Selection *selection_for(Server *s, const std::vector<Job *> &jobs) {
    std::vector<std::pair<uint64_t, int>> key;
    for (Job *j : jobs) key.emplace_back(j->id, j->done % 2);
    std::sort(key.begin(), key.end());
    for (auto &c : s->cache)
        if (c->key == key) return c.get();
    auto sel = std::make_unique<Selection>();
    sel->key = key;
    sel->jobs = jobs;
    sel->last_use = ++s->use;  // the most recent: never the one a slot shortage drops while it is planned
    for (Job *j : jobs) sel->points += j->points();
    if (s->cache.size() >= kCachedSelections) {
        auto victim = std::min_element(s->cache.begin(), s->cache.end(),
                                       [](const std::unique_ptr<Selection> &a, const std::unique_ptr<Selection> &b) {
                                           return a->last_use < b->last_use;
                                       });
        std::unique_ptr<Selection> old = std::move(*victim);
        s->cache.erase(victim);
        destroy_selection(s, std::move(old));
    }
    Selection *raw = sel.get();
    s->cache.push_back(std::move(sel));
    plan_tick(s, *raw, 0);
    plan_tick(s, *raw, 1);
    return raw;
}

void issue(Server *s) {
    const std::vector<Job *> jobs = select_jobs(s);
    Selection *sel = selection_for(s, jobs);
    int least = INT32_MAX;
    for (Job *j : jobs) least = std::min(least, j->spec.steps - j->done);
    const bool direct = (s->opt.flags & F2C_SERVE_DIRECT) != 0;
    int ticks;
    if (least >= 2) {
        const uint64_t cap = std::max<uint64_t>(1, s->opt.burst_points / std::max<uint64_t>(1, 2 * sel->points));
        const int pairs = (int)std::min<uint64_t>((uint64_t)least / 2, cap);
        if (direct) {
            for (int r = 0; r < pairs; ++r) {
                launch_tick(*sel, 0, s->stream);
                launch_tick(*sel, 1, s->stream);
            }
            s->counts.direct_launches += (uint64_t)pairs * 2 * sel->ticks[0].size();
        } else {
            if (!sel->two) sel->two = capture(s, *sel, 2);
            for (int r = 0; r < pairs; ++r) cuda(cudaGraphLaunch(sel->two, s->stream), "graph launch");
            s->counts.graph_replays += (uint64_t)pairs;
        }
        ticks = 2 * pairs;
    } else {
        if (direct) {
            launch_tick(*sel, 0, s->stream);
            s->counts.direct_launches += sel->ticks[0].size();
        } else {
            if (!sel->one) sel->one = capture(s, *sel, 1);
            cuda(cudaGraphLaunch(sel->one, s->stream), "graph launch");
            s->counts.graph_replays++;
        }
        ticks = 1;
    }
    Burst b;
    b.seq = ++s->seq;
    if (!s->spare_events.empty()) {
        b.event = s->spare_events.back();
        s->spare_events.pop_back();
    } else {
        cuda(cudaEventCreateWithFlags(&b.event, cudaEventDisableTiming), "event");
    }
    cuda(cudaEventRecord(b.event, s->stream), "burst event");
    sel->last_seq = b.seq;
    sel->last_use = ++s->use;
    for (Job *j : jobs) {
        j->done += ticks;
        if (j->done >= j->spec.steps) b.finishing.push_back(j);
    }
    s->counts.ticks += (uint64_t)ticks;
    s->counts.bursts++;
    s->inflight.push_back(std::move(b));
}

void worker_main(Server *s) {
    int previous = 0;
    void *ctx_stream = nullptr;
    try {
        runtime(fort_scope_gpu_enter(s->context, &previous, &ctx_stream), "device selection");
        s->ctx_stream = static_cast<cudaStream_t>(ctx_stream);
        int device = 0;
        cuda(cudaGetDevice(&device), "device query");
        cuda(cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, device), "SM count");
        cuda(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking), "stream");
        cuda(cudaStreamCreateWithFlags(&s->capture, cudaStreamNonBlocking), "capture stream");
        for (cudaStream_t &b : s->branch) cuda(cudaStreamCreateWithFlags(&b, cudaStreamNonBlocking), "capture stream");
        runtime(fort_scope_domain_workspace_reserve_v1(s->domain, kSlotBytes * kSlots, &s->workspace_lease),
                "plan workspace");
        cuda(cudaMalloc(&s->slot_device, kSlotBytes * kSlots), "plan workspace");
        cuda(cudaHostAlloc(&s->slot_host, kSlotBytes * kSlots, cudaHostAllocDefault), "plan staging");
        s->slot_busy_until.assign(kSlots, 0);
        s->slot_used.assign(kSlots, false);
        auto idle_since = Clock::now();
        bool idle = false;
        for (;;) {
            {
                std::unique_lock<std::mutex> g(s->lock);
                if (s->stop) break;
            }
            reap(s, false);
            admit_arrivals(s);
            std::vector<Job *> pool;
            for (auto &j : s->active)
                if (j->done < j->spec.steps) pool.push_back(j.get());
            if (pool.empty()) {
                if (!s->inflight.empty()) {
                    reap(s, true);
                    continue;
                }
                if (!idle) {
                    idle = true;
                    idle_since = Clock::now();
                }
                std::unique_lock<std::mutex> g(s->lock);
                if (s->stop) break;
                double wait_s = 0.05;
                if (!s->submitted.empty()) wait_s = std::min(wait_s, std::max(0.0, s->submitted.begin()->first - s->now()));
                if (wait_s > 0) s->wake.wait_for(g, std::chrono::duration<double>(wait_s));
                continue;
            }
            if (idle) {
                idle = false;
                s->counts.idle_s += std::chrono::duration<double>(Clock::now() - idle_since).count();
            }
            if (s->inflight.size() >= s->opt.depth) {
                reap(s, true);
                continue;
            }
            issue(s);
            std::lock_guard<std::mutex> g(s->lock);
            s->stats = s->counts;
        }
    } catch (const Failure &f) {
        std::lock_guard<std::mutex> g(s->lock);
        if (!s->failure) {
            s->failure = f.status;
            s->error = f.message;
        }
        s->finished_cv.notify_all();
    } catch (const std::exception &e) {  // host memory exhausted and the like: the server stops, it does not abort
        std::lock_guard<std::mutex> g(s->lock);
        if (!s->failure) {
            s->failure = FORT_SCOPE_RESOURCE;
            s->error = std::string("server worker: ") + e.what();
        }
        s->finished_cv.notify_all();
    }
    // shut down: wait for the device, release what is still resident
    try {
        while (!s->inflight.empty()) reap(s, true);
    } catch (const Failure &) {
        s->inflight.clear();
    }
    if (s->stream) cudaStreamSynchronize(s->stream);
    while (!s->cache.empty()) {
        std::unique_ptr<Selection> sel = std::move(s->cache.back());
        s->cache.pop_back();
        destroy_selection(s, std::move(sel));
    }
    for (auto &j : s->active) {
        try {
            release_arrays(s, j.get(), false);
        } catch (const Failure &) {
        }
        free_host(j.get(), -1);
    }
    s->active.clear();
    for (cudaEvent_t e : s->spare_events) cudaEventDestroy(e);
    s->spare_events.clear();
    if (s->slot_device) cudaFree(s->slot_device);
    if (s->slot_host) cudaFreeHost(s->slot_host);
    if (s->workspace_lease) (void)fort_scope_domain_workspace_release_v1(s->domain, s->workspace_lease);
    if (s->capture) cudaStreamDestroy(s->capture);
    for (cudaStream_t b : s->branch)
        if (b) cudaStreamDestroy(b);
    if (s->stream) cudaStreamDestroy(s->stream);
    if (ctx_stream) (void)fort_scope_gpu_leave(s->context, previous);
    std::lock_guard<std::mutex> g(s->lock);
    s->stats = s->counts;
    s->finished_cv.notify_all();
}

}  // namespace
}  // namespace f2c::serve

using namespace f2c::serve;

extern "C" int f2c_serve_create_v1(fort_scope_t context, const f2c_serve_options_v1 *options, f2c_server_t *server) {
    if (!server) return fail(FORT_SCOPE_ARGUMENT, "null server output");
    f2c_serve_options_v1 opt{};
    if (options) {
        if (options->version != F2C_SERVE_ABI_VERSION) return fail(FORT_SCOPE_ARGUMENT, "unknown server options version");
        opt = *options;
    }
    if (opt.flags & ~F2C_SERVE_DIRECT) return fail(FORT_SCOPE_ARGUMENT, "unknown server flags");
    if (!(opt.starve_s >= 0.0)) return fail(FORT_SCOPE_ARGUMENT, "starve_s must be zero or positive");
    if (!opt.max_active) opt.max_active = 256;
    if (!opt.depth) opt.depth = 4;
    if (!opt.tick_points) opt.tick_points = 8000000;
    if (!opt.burst_points) opt.burst_points = 32000000;
    fort_scope_domain_t domain = 0;
    if (int st = fort_scope_domain_get_v1(context, &domain)) return fail(st, fort_scope_error());
    auto s = std::make_unique<Server>();
    s->context = context;
    s->domain = domain;
    s->opt = opt;
    s->stats.version = s->counts.version = F2C_SERVE_ABI_VERSION;
    s->start = Clock::now();
    Server *raw = s.release();
    {
        std::lock_guard<std::mutex> g(g_servers_lock);
        *server = g_next_server++;
        g_servers[*server] = raw;
    }
    raw->worker = std::thread(worker_main, raw);
    return FORT_SCOPE_OK;
}

extern "C" int f2c_serve_submit_v1(f2c_server_t server, const f2c_serve_job_v1 *job, uint64_t *id) {
    Server *s = find(server);
    if (!s) return fail(FORT_SCOPE_STALE, "unknown server");
    if (!job || !id) return fail(FORT_SCOPE_ARGUMENT, "null job or id");
    const f2c_serve_job_v1 &p = *job;
    if (p.nx < 1 || p.ny < 1 || p.nz < 1 || p.halo < 1) return fail(FORT_SCOPE_ARGUMENT, "job grid needs positive extents");
    if (p.nz < p.halo + 1 || p.nx < p.halo || p.ny < p.halo)
        return fail(FORT_SCOPE_ARGUMENT, "job grid needs nz > halo, nx >= halo and ny >= halo (boundary fill)");
    if (p.nx > 32767 * 32 || p.ny > 32767 * 8) return fail(FORT_SCOPE_ARGUMENT, "job grid too wide for the tile queue");
    if (p.nscalar < 0 || p.nscalar > F2C_MAX_SCALARS) return fail(FORT_SCOPE_ARGUMENT, "scalar count out of range");
    if (p.steps < 1) return fail(FORT_SCOPE_ARGUMENT, "a job needs at least one step");
    if (!(p.dx > 0) || !(p.dy > 0) || !(p.dz > 0)) return fail(FORT_SCOPE_ARGUMENT, "grid spacings must be positive");
    if (p.flags & ~F2C_SERVE_KEEP_RESULT || p.reserved) return fail(FORT_SCOPE_ARGUMENT, "unknown job flags");
    auto j = std::make_unique<Job>();
    j->spec = p;
    j->fields = 3 + p.nscalar;
    j->grid = {p.nx, p.ny, p.nz, p.halo, p.nx + 2 * p.halo, p.ny + 2 * p.halo, p.dx, p.dy, p.dz};
    j->field_bytes = (size_t)(p.nx + 2 * p.halo) * (p.ny + 2 * p.halo) * (p.nz + 2 * p.halo) * sizeof(double);
    j->bytes = job_bytes(p);
    {
        std::lock_guard<std::mutex> g(s->lock);
        if (s->failure) return fail(s->failure, "server failed: " + s->error);
        j->id = s->next_id++;
        *id = j->id;
        ++s->outstanding;
        s->submitted.emplace(p.arrival, std::move(j));
    }
    s->wake.notify_all();
    return FORT_SCOPE_OK;
}

extern "C" double f2c_serve_clock_v1(f2c_server_t server) {
    Server *s = find(server);
    return s ? s->now() : -1.0;
}

extern "C" int f2c_serve_poll_v1(f2c_server_t server, f2c_serve_done_v1 *done, size_t capacity, size_t *count) {
    Server *s = find(server);
    if (!s) return fail(FORT_SCOPE_STALE, "unknown server");
    if (!count || (capacity && !done)) return fail(FORT_SCOPE_ARGUMENT, "null poll output");
    std::lock_guard<std::mutex> g(s->lock);
    size_t n = 0;
    while (n < capacity && !s->done.empty()) {
        done[n++] = s->done.front();
        s->done.pop_front();
    }
    *count = n;
    return FORT_SCOPE_OK;
}

extern "C" int f2c_serve_drain_v1(f2c_server_t server, double timeout_s) {
    Server *s = find(server);
    if (!s) return fail(FORT_SCOPE_STALE, "unknown server");
    std::unique_lock<std::mutex> g(s->lock);
    auto ready = [&] { return s->outstanding == 0 || s->failure != 0; };
    if (timeout_s < 0) {
        s->finished_cv.wait(g, ready);
    } else if (!s->finished_cv.wait_for(g, std::chrono::duration<double>(timeout_s), ready)) {
        return fail(FORT_SCOPE_STATE, "jobs still running at the timeout");
    }
    if (s->failure) return fail(s->failure, "server failed: " + s->error);
    return FORT_SCOPE_OK;
}

extern "C" int f2c_serve_result_v1(f2c_server_t server, uint64_t id, int32_t field, const double **host) {
    Server *s = find(server);
    if (!s) return fail(FORT_SCOPE_STALE, "unknown server");
    if (!host) return fail(FORT_SCOPE_ARGUMENT, "null result output");
    std::lock_guard<std::mutex> g(s->lock);
    auto it = s->results.find(id);
    if (it == s->results.end()) return fail(FORT_SCOPE_STALE, "no kept result for this job");
    Job *j = it->second.get();
    if (field < 0 || field >= j->fields) return fail(FORT_SCOPE_ARGUMENT, "field index out of range");
    *host = static_cast<const double *>(j->host[j->result_set][field]);
    return FORT_SCOPE_OK;
}

extern "C" int f2c_serve_release_v1(f2c_server_t server, uint64_t id) {
    Server *s = find(server);
    if (!s) return fail(FORT_SCOPE_STALE, "unknown server");
    std::unique_ptr<Job> j;
    {
        std::lock_guard<std::mutex> g(s->lock);
        auto it = s->results.find(id);
        if (it == s->results.end()) return fail(FORT_SCOPE_STALE, "no kept result for this job");
        j = std::move(it->second);
        s->results.erase(it);
    }
    free_host(j.get(), -1);
    return FORT_SCOPE_OK;
}

extern "C" int f2c_serve_stats_get_v1(f2c_server_t server, f2c_serve_stats_v1 *stats) {
    Server *s = find(server);
    if (!s) return fail(FORT_SCOPE_STALE, "unknown server");
    if (!stats) return fail(FORT_SCOPE_ARGUMENT, "null stats output");
    std::lock_guard<std::mutex> g(s->lock);
    *stats = s->stats;
    return FORT_SCOPE_OK;
}

extern "C" const char *f2c_serve_error_v1(f2c_server_t server) {
    Server *s = find(server);
    if (!s) return t_error.c_str();
    std::lock_guard<std::mutex> g(s->lock);
    t_error = s->error.empty() ? t_error : s->error;
    return t_error.c_str();
}

extern "C" int f2c_serve_destroy_v1(f2c_server_t server) {
    Server *s = nullptr;
    {
        std::lock_guard<std::mutex> g(g_servers_lock);
        auto it = g_servers.find(server);
        if (it == g_servers.end()) return fail(FORT_SCOPE_STALE, "unknown server");
        s = it->second;
        g_servers.erase(it);
    }
    {
        std::lock_guard<std::mutex> g(s->lock);
        s->stop = true;
    }
    s->wake.notify_all();
    if (s->worker.joinable()) s->worker.join();
    for (auto &kv : s->results) free_host(kv.second.get(), -1);
    for (auto &kv : s->submitted) free_host(kv.second.get(), -1);
    delete s;
    return FORT_SCOPE_OK;
}
