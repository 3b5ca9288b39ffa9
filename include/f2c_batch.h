/* Batched ensembles: many independent advection instances of uneven grid
 * sizes advanced by ONE persistent launch over a flattened tile queue.
 *
 * Each instance is an f2c_grid_v1 + f2c_fields_v1 pair (include/f2c_advection.h);
 * all instances of a batch share the scalar count, the output mode and the set
 * of requested outputs. The work is cut into items of one 32 x 8 column tile
 * and a z-range of `kz` levels (per instance, chosen by the autotuner in
 * compiler/scheduling); a fixed grid of CTAs (the SM count times the resident
 * CTAs per SM) takes items from an atomic counter, largest items first. Every
 * item runs the same face-sharing arithmetic as f2c_advection_v1, so a batch
 * is bit-identical to one launch per instance.
 *
 * The caller owns the device workspace (descriptors, items, the counter):
 * f2c_batch_workspace_bytes_v1 sizes it, f2c_batch_prepare_v1 fills it (a
 * setup call: synchronous on `stream`), f2c_batch_step_v1 resets the counter
 * and launches (asynchronous; capturable in a CUDA graph). Calls that overlap
 * on the GPU with the same workspace race on its counter.
 *
 * No counterpart exists in the reference (its resident build runs one
 * procedure call at a time); statuses are fort_scope_status values.
 */
#ifndef F2C_BATCH_H
#define F2C_BATCH_H
#include <stddef.h>
#include <stdint.h>

#include "f2c_advection.h"
#ifdef __cplusplus
extern "C" {
#endif

typedef struct f2c_batch_plan_v1 {
    void *workspace;           /* device memory of at least f2c_batch_workspace_bytes_v1 bytes */
    size_t workspace_bytes;
    int32_t count, nscalar, mask, items;
    uint32_t ctas;             /* persistent grid size */
    uint32_t reserved;         /* flags: F2C_BATCH_HALO_OK (set by preparation), F2C_BATCH_FAST_FP (caller's) */
} f2c_batch_plan_v1;

/* Plan flags. F2C_BATCH_HALO_OK: every instance admits f2c_batch_halo_v1
 * (set by preparation). F2C_BATCH_FAST_FP: f2c_batch_step_v1 runs the fast-fp
 * kernel (F2C_KERNEL_FAST of f2c_advection.h: FMA contraction and regrouped
 * sums, each field within 1e-12 of its maximum of the strict result) instead of
 * the bit-exact one; the caller sets it after preparation, which clears it
 * (and sets it for tiles of 4 or 16 rows, which only the fast-fp kernel runs).
 * Bits 8-15 hold the plan's tile rows (0 reads as 8). */
#define F2C_BATCH_HALO_OK 1u
#define F2C_BATCH_FAST_FP 2u
#define F2C_BATCH_TILE_ROWS(reserved) ((((reserved) >> 8) & 0xffu) ? (((reserved) >> 8) & 0xffu) : 8u)

/* Bytes of workspace for `count` instances cut into z-chunks of kz[i] levels (kz NULL: 32). */
size_t f2c_batch_workspace_bytes_v1(const f2c_grid_v1 *grids, const int32_t *kz, int32_t count);
/* Validate the instances, build descriptors and the item queue into `workspace`. */
int f2c_batch_prepare_v1(const f2c_grid_v1 *grids, const f2c_fields_v1 *fields, const int32_t *kz, int32_t count,
                         void *workspace, size_t workspace_bytes, void *stream, f2c_batch_plan_v1 *plan);
/* One step of every instance: counter reset + one persistent launch on `stream`. */
int f2c_batch_step_v1(const f2c_batch_plan_v1 *plan, void *stream);

/* f2c_batch_prepare_v1 without waiting, for a caller that re-plans every step
 * (a server whose set of instances changes between steps): descriptors and
 * queue are written into `staging` (host memory of f2c_batch_workspace_bytes_v1
 * bytes or more; pinned memory keeps the copy asynchronous) and copied to the
 * workspace on `stream`. Neither `staging` nor the workspace may be reused
 * until the stream has passed the steps that use this plan (an event recorded
 * after them tells). */
int f2c_batch_prepare_async_v1(const f2c_grid_v1 *grids, const f2c_fields_v1 *fields, const int32_t *kz,
                               int32_t count, void *workspace, size_t workspace_bytes, void *staging, void *stream,
                               f2c_batch_plan_v1 *plan);

/* Tile shapes. The plans above cut every instance into tiles of 32 x 8
 * columns. These entries take the tile height: 4, 8 or 16 rows (one warp per
 * row plus an edge warp; 4-row tiles run four CTAs per SM, 8-row two, 16-row
 * one). Tiles of 4 or 16 rows run the fast-fp kernel only; results do not
 * depend on the tile shape or the z-chunk depths, bit for bit. `staging` NULL
 * prepares synchronously on `stream` (as f2c_batch_prepare_v1), otherwise as
 * f2c_batch_prepare_async_v1 does. */
size_t f2c_batch_workspace_bytes_rows_v1(const f2c_grid_v1 *grids, const int32_t *kz, int32_t count,
                                         int32_t tile_rows);
int f2c_batch_prepare_rows_v1(const f2c_grid_v1 *grids, const f2c_fields_v1 *fields, const int32_t *kz,
                              int32_t count, int32_t tile_rows, void *workspace, size_t workspace_bytes,
                              void *staging, void *stream, f2c_batch_plan_v1 *plan);

/* A plan's step (counter reset + persistent launch) captured once as an
 * executable CUDA graph (`*graph` receives a cudaGraphExec_t), launched on any
 * stream and destroyed by the caller. The graph reads the plan's workspace at
 * each launch; it stays valid while the workspace and the instances' arrays
 * do. The plan's flags are fixed at capture. */
int f2c_batch_graph_create_v1(const f2c_batch_plan_v1 *plan, void **graph);
int f2c_batch_graph_launch_v1(void *graph, void *stream);
int f2c_batch_graph_destroy_v1(void *graph);

/* Boundary fill of every instance's outputs in one launch on `stream` (the
 * per-instance rule of f2c_halo_fill_v1: U, V and scalars periodic in x and y
 * and mirrored in z, W with zero walls): after a forward-Euler step it
 * completes each instance's new fields. At most 4096 instances, each with
 * nz > halo, nx >= halo and ny >= halo (as f2c_halo_fill_v1 requires). */
int f2c_batch_halo_v1(const f2c_batch_plan_v1 *plan, void *stream);

/* The same batched step for callers that cannot allocate device memory. It has
 * no counterpart in the reference.
 *
 * Who needs it: a caller whose device memory is already fully handed to
 * another allocator (a caching allocator, or a residency budget sized to the
 * whole device) has no room for the workspace f2c_batch_step_v1 needs, and a
 * caller stepping an ensemble inside a time loop may not accept the
 * device-wide synchronisation that freeing device memory implies. This entry
 * allocates nothing: the work counter, instance descriptors and tile queue
 * live in one fixed array of F2C_BATCH_NO_ALLOC_SCRATCH_BYTES (1088 KiB) that
 * the library keeps in device memory; every GPU that loads the library holds it
 * until the process exits. The caller passes only its instances' grids and
 * fields (and optional z-chunk depths, as for f2c_batch_workspace_bytes_v1).
 *
 * Limits: at most F2C_BATCH_NO_ALLOC_MAX_INSTANCES instances and
 * F2C_BATCH_NO_ALLOC_MAX_ITEMS work items (32 x 8 column tiles times z-chunks);
 * larger batches are rejected with FORT_SCOPE_ARGUMENT and a message naming the
 * limit. The first call on a device looks up the array's device address with
 * that device current. Each call copies its descriptors and tile queue into the
 * array from host arrays that the library rewrites on the next call, and
 * clears the counter. Every call shares and overwrites the array, so calls that
 * overlap on the GPU, or that come from several host threads at once, race.
 * Results are bit-identical to f2c_batch_step_v1 with the strict kernel. */
#define F2C_BATCH_NO_ALLOC_MAX_INSTANCES 128
#define F2C_BATCH_NO_ALLOC_MAX_ITEMS 65536
#define F2C_BATCH_NO_ALLOC_SCRATCH_BYTES 1114112
int f2c_batch_step_static_v1(const f2c_grid_v1 *grids, const f2c_fields_v1 *fields, const int32_t *kz, int32_t count,
                             void *stream);

#ifdef __cplusplus
}
#endif
#endif
