/* GB300 residency runtime: the fort_scope_* C ABI, version 1.
 *
 * Drop-in replacement for the reference runtime's public interface
 * (compiler/runtime/scoped_runtime.h:1-443, ABI version :16). The Fortran
 * residency modules (compiler/runtime/scoped_memory.f90, 63 bind(C)
 * declarations) and every generated numerical entry link against these names,
 * so the names, argument lists, enumerator values and record layouts below are
 * identical to the reference's; the implementation behind them is new
 * (fortran-to-cuda_gb300/csrc/runtime).
 *
 * Conventions (as in the reference): coordinates are zero-based physical
 * offsets with exclusive upper bounds; host arrays are borrowed and must stay
 * valid until unregister/close; one caller at a time per context, different
 * contexts may run concurrently. Every call returns a fort_scope_status.
 */
#ifndef FORT_SCOPED_RUNTIME_H
#define FORT_SCOPED_RUNTIME_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#define FORT_SCOPE_ABI_VERSION 1
typedef uint64_t fort_scope_t;
typedef uint64_t fort_buffer_t;
typedef uint64_t fort_scope_domain_t;

/* ---- statuses and enumerations (scoped_runtime.h:42-57 of the reference) ---- */
enum fort_scope_status {
    FORT_SCOPE_OK = 0,
    FORT_SCOPE_ARGUMENT = 1,
    FORT_SCOPE_STALE = 2,
    FORT_SCOPE_ALIAS = 3,
    FORT_SCOPE_RESOURCE = 4,
    FORT_SCOPE_BOUNDARY = 5,
    FORT_SCOPE_EXECUTION = 6,
    FORT_SCOPE_UNINITIALIZED = 7,
    FORT_SCOPE_STATE = 8,
    /* Not an error: the entry does nothing for these arguments; the caller runs its original statements. */
    FORT_SCOPE_DECLINED = 9
};
enum fort_scope_type {
    FORT_SCOPE_BYTES = 0, FORT_SCOPE_REAL32 = 1, FORT_SCOPE_REAL64 = 2, FORT_SCOPE_INTEGER32 = 3, FORT_SCOPE_LOGICAL = 4
};
enum fort_scope_access_flags { FORT_SCOPE_READ_ALL = 1, FORT_SCOPE_WRITE_ALL = 2, FORT_SCOPE_OVERWRITE_ALL = 4 };
enum fort_scope_execution_mode { FORT_SCOPE_NATIVE = 0, FORT_SCOPE_GPU = 1 };

/* ---- records (layouts of scoped_runtime.h:20-97,120-123 of the reference) ---- */
#define FORT_SCOPE_TRACE_ABI_VERSION 1
enum fort_scope_trace_field {
    FORT_SCOPE_TRACE_OWNER = 1, FORT_SCOPE_TRACE_PROCEDURE = 2, FORT_SCOPE_TRACE_SEGMENT = 4,
    FORT_SCOPE_TRACE_OPERATION = 8, FORT_SCOPE_TRACE_IMPLEMENTATION = 16, FORT_SCOPE_TRACE_BOUNDARY = 32,
    FORT_SCOPE_TRACE_ALL = 63
};
typedef struct fort_scope_trace_state_v1 {
    uint32_t version, reserved;
    char owner[65], procedure[65], segment[65], operation[65], implementation[65], boundary[65];
} fort_scope_trace_state_v1;

typedef struct fort_scope_section {
    const size_t *lower;
    const size_t *upper;
} fort_scope_section;

typedef struct fort_scope_access {
    uint32_t flags;
    size_t read_count;
    const fort_scope_section *reads;
    size_t write_count;
    const fort_scope_section *writes;
    size_t overwrite_count;
    const fort_scope_section *overwrites;
} fort_scope_access;

typedef struct fort_scope_layout {
    uint32_t rank, type;
    size_t element_bytes;
    void *host;
    const size_t *extents;
    const int64_t *lower_bounds;
    uint64_t generation;
} fort_scope_layout;

typedef struct fort_scope_stats {
    uint64_t uploads, downloads, upload_bytes, download_bytes;
    /* allocations: device mirrors allocated so far; allocated_bytes: the bytes mirrors hold now;
     * peak_device_bytes: the most mirrors held at once (scratch has its own statistics) */
    uint64_t allocations, allocated_bytes, peak_device_bytes;
    uint64_t launches, waits, reconciliations;
} fort_scope_stats;

#define FORT_SCOPE_COMPLETION_ABI_VERSION 1
typedef struct fort_scope_completion_stats_v1 {
    uint32_t version, reserved;
    uint64_t event_records, event_queries, event_waits, stream_waits;
    uint64_t created_events, reused_events, independent_host_tasks;
} fort_scope_completion_stats_v1;

#define FORT_SCOPE_SCRATCH_ABI_VERSION 1
typedef struct fort_scope_scratch_lease_v1 {
    uint32_t version, reserved;
    uint64_t token;
    void *device;
    size_t bytes, capacity;
} fort_scope_scratch_lease_v1;
typedef struct fort_scope_scratch_stats_v1 {
    uint32_t version, active;
    uint64_t acquisitions, allocations, reuses, releases, grows;
    uint64_t capacity_bytes, active_bytes, peak_scratch_bytes, peak_total_device_bytes;
} fort_scope_scratch_stats_v1;

typedef struct fort_scope_plan_binding {
    fort_buffer_t buffer;
    fort_scope_access access;
} fort_scope_plan_binding;

#define FORT_SCOPE_RESIDENCY_ABI_VERSION 1
typedef struct fort_scope_residency_stats_v1 {
    uint32_t version, reserved;
    uint64_t reserve_batches, requested_resources, reuse_hits;
    uint64_t evictions, evicted_bytes, dirty_evictions, dirty_download_bytes, pressure_flushes;
} fort_scope_residency_stats_v1;

#define FORT_SCOPE_GRAPH_ABI_VERSION 1
/* One kernel launch. `function` is the address of a __global__ function (on
 * the CPU test backend: a host function `void f(void **arguments)`).
 * Argument values are copied during the call. */
typedef struct fort_scope_kernel_v1 {
    uint32_t version, reserved;
    const void *function;
    uint32_t grid[3], block[3];
    size_t shared_bytes;
    void *const *arguments;
    size_t argument_count;
} fort_scope_kernel_v1;
typedef struct fort_scope_graph_stats_v1 {
    uint32_t version, reserved;
    uint64_t creations, instantiations, rebuilds, submissions, replays;
    uint64_t parameter_updates, logical_kernels, live_graphs, destructions;
} fort_scope_graph_stats_v1;
typedef struct fort_scope_graph_task_v1 {
    fort_scope_kernel_v1 kernel;
    const fort_scope_plan_binding *bindings;
    size_t binding_count;
} fort_scope_graph_task_v1;
typedef struct fort_scope_graph_queue_stats_v1 {
    uint32_t version, queue_enabled, graphs_enabled, reserved;
    uint64_t accepted_tasks, submissions, conflict_flushes, explicit_flushes;
    uint64_t pending_tasks, peak_pending_tasks, copied_argument_bytes;
    uint64_t direct_submissions, direct_kernels, graph_resource_fallbacks;
} fort_scope_graph_queue_stats_v1;
typedef struct fort_scope_graph_member_v1 {
    const fort_scope_plan_binding *bindings;
    size_t binding_count;
} fort_scope_graph_member_v1;

#define FORT_SCOPE_EXTERNAL_ABI_VERSION 1
typedef struct fort_scope_external_binding_v1 {
    fort_buffer_t buffer;
    uint32_t type, rank;
    size_t element_bytes;
    fort_scope_access access;
} fort_scope_external_binding_v1;
typedef struct fort_scope_external_view_v1 {
    fort_buffer_t buffer;
    uint64_t generation;
    uint32_t type, rank;
    size_t element_bytes, bytes;
    const size_t *extents, *strides;
    const int64_t *lower_bounds;
    void *device;
} fort_scope_external_view_v1;
typedef struct fort_scope_external_call_v1 {
    uint32_t version, reserved;
    const fort_scope_external_binding_v1 *bindings;
    size_t binding_count;
    uint64_t workspace_lease;
    size_t workspace_bytes;
} fort_scope_external_call_v1;
typedef struct fort_scope_external_report_v1 {
    uint32_t version;
    int32_t status;
    uint32_t started, committed;
} fort_scope_external_report_v1;
typedef int (*fort_scope_external_worker_v1)(void *user, const fort_scope_external_view_v1 *views, size_t count,
                                             void *stream, int *started);

/* ---- diagnostics ---- */
uint32_t fort_scope_abi_version(void);
/* Last failure text of the calling thread (never NULL). */
const char *fort_scope_error(void);
/* Keep a diagnostic and return `status`. */
int fort_scope_report_error(int status, const char *message);
/* A failure after numerical work started: poisons the context and its domain; returns EXECUTION. */
int fort_scope_execution_error(fort_scope_t context, const char *message);
void fort_scope_trace_set_v1(fort_scope_t context, uint32_t update_mask, const char *owner, const char *procedure,
                             const char *segment, const char *operation, const char *implementation,
                             const char *boundary, fort_scope_trace_state_v1 *previous);
void fort_scope_trace_restore_v1(fort_scope_t context, const fort_scope_trace_state_v1 *previous);

/* ---- contexts and domains ---- */
int fort_scope_create(int device, fort_scope_t *context);
int fort_scope_domain_create_v1(int device, fort_scope_domain_t *domain);
int fort_scope_create_in_domain_v1(fort_scope_domain_t domain, fort_scope_t *context);
int fort_scope_domain_get_v1(fort_scope_t context, fort_scope_domain_t *domain);
int fort_scope_domain_device_get_v1(fort_scope_domain_t domain, int *device);
int fort_scope_domain_stats_get_v1(fort_scope_domain_t domain, fort_scope_stats *stats);
int fort_scope_domain_close_v1(fort_scope_domain_t domain);
int fort_scope_domain_abandon_v1(fort_scope_domain_t domain);
int fort_scope_domain_workspace_reserve_v1(fort_scope_domain_t domain, size_t bytes, uint64_t *lease);
int fort_scope_domain_workspace_resize_v1(fort_scope_domain_t domain, uint64_t lease, size_t bytes);
int fort_scope_domain_workspace_release_v1(fort_scope_domain_t domain, uint64_t lease);
int fort_scope_set_device_budget(fort_scope_t context, size_t bytes);
/* FORT_RESIDENT_DEVICE_BUDGET (bytes, or a count with K, M or G) when set, else the device's free
 * memory less max(total/16, 512 MiB). */
int fort_scope_device_budget_default_v1(int device, size_t *bytes);
int fort_scope_domain_budget_get_v1(fort_scope_domain_t domain, size_t *budget, size_t *unclaimed);
int fort_scope_close(fort_scope_t context);
int fort_scope_abandon(fort_scope_t context);
int fort_scope_wait(fort_scope_t context);

/* ---- registration and coherence ---- */
int fort_scope_register(fort_scope_t context, uint64_t identity, uint64_t generation, const fort_scope_layout *layout,
                        int host_initialized, fort_buffer_t *buffer);
int fort_scope_register_sections(fort_scope_t context, uint64_t identity, uint64_t generation,
                                 const fort_scope_layout *layout, const fort_scope_section *initialized,
                                 size_t initialized_count, fort_buffer_t *buffer);
int fort_scope_admit_source_reads_v1(fort_scope_t context, fort_buffer_t buffer, const fort_scope_section *sections,
                                     size_t count);
int fort_scope_identity_swap_v1(fort_scope_t context, fort_buffer_t first, fort_buffer_t second,
                                const fort_scope_layout *first_after, const fort_scope_layout *second_after,
                                fort_buffer_t *first_current, fort_buffer_t *second_current);
int fort_scope_forget_definition(fort_scope_t context, fort_buffer_t buffer);
int fort_scope_layout_get(fort_scope_t context, fort_buffer_t buffer, fort_scope_layout *layout);
int fort_scope_buffer_valid_v1(fort_scope_t context, fort_buffer_t buffer, int *valid);
int fort_scope_access_begin_v1(fort_scope_t context, const fort_scope_plan_binding *bindings, size_t count, int device,
                               void **devices);
int fort_scope_original_host_begin_v1(fort_scope_t context, const fort_scope_plan_binding *bindings, size_t count);
int fort_scope_host_begin(fort_scope_t context, fort_buffer_t buffer, const fort_scope_access *access);
int fort_scope_host_end(fort_scope_t context, fort_buffer_t buffer);
int fort_scope_device_begin(fort_scope_t context, fort_buffer_t buffer, const fort_scope_access *access, void **device);
int fort_scope_device_end(fort_scope_t context, fort_buffer_t buffer);
int fort_scope_cancel_access(fort_scope_t context, fort_buffer_t buffer);
int fort_scope_device_reserve_v1(fort_scope_t context, fort_buffer_t buffer, void **device);
int fort_scope_device_reserve_many_v1(fort_scope_t context, const fort_buffer_t *buffers, size_t count,
                                      void **devices);
int fort_scope_observe_v1(fort_scope_t context, const fort_buffer_t *buffers, size_t count);
int fort_scope_observe_all_v1(fort_scope_t context);
int fort_scope_discard_v1(fort_scope_t context, fort_buffer_t buffer);
int fort_scope_recycle_v1(fort_scope_t context, fort_buffer_t buffer);
int fort_scope_retire_v1(fort_scope_t context, fort_buffer_t buffer);
int fort_scope_unregister(fort_scope_t context, fort_buffer_t buffer);
int fort_scope_stats_get(fort_scope_t context, fort_scope_stats *stats);
int fort_scope_residency_stats_get_v1(fort_scope_t context, fort_scope_residency_stats_v1 *stats);
int fort_scope_completion_stats_get_v1(fort_scope_t context, fort_scope_completion_stats_v1 *stats);

/* ---- scratch ---- */
int fort_scope_scratch_acquire_v1(fort_scope_t context, size_t bytes, fort_scope_scratch_lease_v1 *lease);
int fort_scope_scratch_release_v1(fort_scope_t context, uint64_t token);
int fort_scope_scratch_stats_get_v1(fort_scope_t context, fort_scope_scratch_stats_v1 *stats);

/* ---- launches, the task queue and graph replay ---- */
int fort_scope_gpu_enter(fort_scope_t context, int *previous_device, void **stream);
int fort_scope_gpu_leave(fort_scope_t context, int previous_device);
int fort_scope_note_launch(fort_scope_t context);
/* Queue one task. Its launch joins the context's pending list; the list is
 * submitted as one CUDA graph (instantiated on the second reach of the same
 * task sequence, replayed with parameter updates after that) when it holds
 * 2^18 device threads or more (FORT_SCOPE_GRAPH_QUEUE_WORK), on explicit flush,
 * or before any host access. FORT_SCOPE_GRAPH_QUEUE=0 submits every task at
 * once; FORT_SCOPE_CUDA_GRAPHS=0 uses direct launches. */
int fort_scope_graph_enqueue_v1(fort_scope_t context, uint64_t code_key, const fort_scope_graph_task_v1 *task,
                                const size_t *argument_sizes);
int fort_scope_graph_enqueue_members_v1(fort_scope_t context, uint64_t code_key, const fort_scope_kernel_v1 *kernel,
                                        const size_t *argument_sizes, const fort_scope_graph_member_v1 *members,
                                        size_t member_count);
int fort_scope_graph_flush_v1(fort_scope_t context);
int fort_scope_graph_queue_cancel_v1(fort_scope_t context);
int fort_scope_graph_queue_stats_get_v1(fort_scope_t context, fort_scope_graph_queue_stats_v1 *stats);
int fort_scope_graph_submit_v1(fort_scope_t context, uint64_t group_key, const fort_scope_kernel_v1 *kernels,
                               size_t count);
int fort_scope_graph_execute_v1(fort_scope_t context, uint64_t group_key, const fort_scope_graph_task_v1 *tasks,
                                size_t count);
int fort_scope_graph_stats_get_v1(fort_scope_t context, fort_scope_graph_stats_v1 *stats);
int fort_scope_external_execute_v1(fort_scope_t context, const fort_scope_external_call_v1 *call,
                                   fort_scope_external_worker_v1 worker, void *user,
                                   fort_scope_external_report_v1 *report);

/* ---- slab pipelines (extensions of this runtime; the reference has no counterpart) ----
 *
 * For a step whose arrays the host rewrites or reads between device uses
 * (pinned host arrays, host-round: two or more consecutive uses each preceded
 * by host access), the transfers can overlap the kernels when the step is cut
 * into slabs along its last dimension.
 *
 * fort_scope_device_reserve_slabs_v1 reserves device storage like
 * fort_scope_device_reserve_many_v1, except that no array is handed out in
 * place while pipelines are enabled (FORT_SCOPE_HOST_STREAM, default 1), and
 * sets *pipelined to 1 when at least one array is host-round: the caller then
 * submits the step as slab tasks through fort_scope_slab_enqueue_v1, otherwise
 * as one task through fort_scope_graph_enqueue_v1. With FORT_SCOPE_HOST_STREAM=0
 * it is fort_scope_device_reserve_many_v1 and *pipelined is 0.
 *
 * fort_scope_slab_enqueue_v1 runs `count` (1..64) tasks in order, after every
 * queued task: uploads of what task n reads run on a copy stream ahead of its
 * kernel, the kernels run in order on the context's stream, and what task n
 * writes into host-round arrays is published to the host on a second copy
 * stream behind it, so the host copies are current when the call's work
 * completes (a later host access or fort_scope_wait orders after all of it).
 * Every bound array needs device storage from fort_scope_device_reserve_slabs_v1
 * (FORT_SCOPE_STATE otherwise); each task's reads must be defined before the
 * sequence starts; argument_sizes holds the sizes of every task's kernel
 * arguments, task after task. Validation happens before any work; a failure
 * after work started poisons the context (FORT_SCOPE_EXECUTION). */
int fort_scope_device_reserve_slabs_v1(fort_scope_t context, const fort_buffer_t *buffers, size_t count,
                                       void **devices, int *pipelined);
int fort_scope_slab_enqueue_v1(fort_scope_t context, uint64_t code_key, const fort_scope_graph_task_v1 *tasks,
                               size_t count, const size_t *argument_sizes);

/* Timing of slab sequences (extension, off by default). While enabled, each
 * sequence records device timing events around every slab's uploads, kernel and
 * publications; fort_scope_slab_timing_get_v1 waits for the last sequence and
 * reports its span (first upload to last kernel or publication) and the summed
 * and longest durations of each kind. FORT_SCOPE_STATE when nothing was timed.
 * Disabling drops the events. */
typedef struct fort_scope_slab_timing_v1 {
    uint32_t version;
    uint32_t slabs;
    double span_ms;
    double upload_ms, kernel_ms, publish_ms;
    double longest_upload_ms, longest_kernel_ms, longest_publish_ms;
} fort_scope_slab_timing_v1;
int fort_scope_slab_timing_set_v1(fort_scope_t context, int enabled);
int fort_scope_slab_timing_get_v1(fort_scope_t context, fort_scope_slab_timing_v1 *out);

/* ---- numerical contract of a context (extension; the reference fixes it at build time) ----
 *
 * The reference compiles its generated entries either with the strict options
 * (compiler/emission/numerical_contract.py:13-15) or, under the resident
 * build's --fast-fp, with FMA contraction (compiler/resident/build.py:22,66-67).
 * This library's entries are prebuilt with both kernels; the contract is chosen
 * per context instead. FORT_SCOPE_NUMERICS_STRICT (the default) runs kernels
 * that round exactly like the strict native control; FORT_SCOPE_NUMERICS_FAST
 * lets the entries that have a fast-fp kernel (the fused momentum procedures
 * and the advection steps) use it: FMA contraction and regrouped sums, each
 * field within 1e-12 of its maximum magnitude of the strict result. A resident
 * build prepared with --fast-fp sets it when its domain opens an epoch. Tasks
 * already queued keep the contract they were accepted under. */
#define FORT_SCOPE_NUMERICS_STRICT 0
#define FORT_SCOPE_NUMERICS_FAST 1
int fort_scope_numerics_set_v1(fort_scope_t context, int numerics);
int fort_scope_numerics_get_v1(fort_scope_t context, int *numerics);

/* ---- host pinning of a context (extension; the reference has no counterpart) ----
 *
 * Host arrays of 1 MiB or more are pinned in place the first time the device
 * is about to use them, so that their copies run as DMA. A caller whose arrays
 * never move between host and device while in use (a server that defines its
 * jobs' fields on the device and reads back only some results) turns this off
 * for its context: 0 never pins, 1 always pins, -1 (the default) follows
 * FORT_SCOPE_PIN_HOST. Arrays already pinned stay pinned. */
int fort_scope_host_pinning_set_v1(fort_scope_t context, int enabled);

#ifdef __cplusplus
}
#endif
#endif
