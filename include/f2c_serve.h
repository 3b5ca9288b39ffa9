/* Serving advection jobs on one GPU with continuous batching.
 *
 * A job asks for `steps` forward-Euler steps (the boundary fill after each) of
 * one advection instance. The server keeps every admitted job's fields in the
 * residency runtime's device mirrors (scoped_runtime.h) from admission to
 * retirement: each job registers two sets of arrays (U, V, W and its scalars,
 * ping-pong) in the domain of the context the server is given, holds them
 * under one device access for its lifetime, defines the first set on the
 * device (f2c_seed_fields_v1) and never moves them to the host between steps.
 * Jobs are admitted as they arrive while the device has room for them: free
 * device memory (the driver's free bytes plus what the stream-ordered pool
 * holds unused) less a reserve, the domain's unclaimed budget and the server's
 * own budget must each cover the job.
 *
 * A worker thread advances the resident jobs in ticks: the jobs with the least
 * remaining work (steps left x points; jobs older than `starve_s` first), up
 * to `tick_points` grid points, step once, as one persistent batched launch per scalar count (f2c_batch.h) that
 * also fills the new fields' ghost layers (F2C_ADVANCE_FILLED). Two consecutive ticks of the same selection are
 * captured once as a CUDA graph (the scalar groups on parallel branches, so
 * that their launches overlap) and replayed while the selection holds; the
 * last few selections stay cached. Every job's arithmetic is the
 * single-instance kernel's, so a job's result is the same alone and in any mix,
 * bit for bit. The numerical contract is the context's
 * (fort_scope_numerics_set_v1).
 *
 * No counterpart exists in the reference: its resident build runs one
 * procedure call at a time. Statuses are fort_scope_status values; the last
 * failure text is fort_scope_error() for runtime failures and f2c_last_error()
 * otherwise, and f2c_serve_error_v1 gives the server's own.
 */
#ifndef F2C_SERVE_H
#define F2C_SERVE_H
#include <stddef.h>
#include <stdint.h>

#include "f2c_advection.h"
#include "scoped_runtime.h"
#ifdef __cplusplus
extern "C" {
#endif

#define F2C_SERVE_ABI_VERSION 1

/* Seeded synthetic fields of one instance, written on the device: U, V and W
 * are each four sine modes of amplitude 1 (integer wavenumbers 1..4 along each
 * axis, phase in [0, 2 pi), evaluated at the field's staggered position) plus
 * N(0, 0.05) noise on the interior; scalar 0 is uniform in [280, 300], scalar 1
 * uniform in [0, 0.02], scalars 2 and 3 Gaussian blobs; ghost layers are then
 * filled as f2c_halo_fill_v1 does. The values depend only on the seed and the
 * geometry (a counter-based generator), never on the launch. The modes, the
 * noise and the blobs are evaluated in single precision and stored as FP64
 * (synthetic inputs: FP64 transcendentals would cost several steps of the job);
 * the uniform scalars carry 53 random bits. `fields` holds 3 + nscalar device
 * pointers. Asynchronous on `stream`. */
int f2c_seed_fields_v1(const f2c_grid_v1 *grid, uint64_t seed, int32_t nscalar, double *const *fields,
                       void *stream);

typedef uint64_t f2c_server_t;

/* Server flags. F2C_SERVE_DIRECT: launch every tick directly instead of
 * replaying graphs. */
#define F2C_SERVE_DIRECT 1u

typedef struct f2c_serve_options_v1 {
    uint32_t version;        /* F2C_SERVE_ABI_VERSION */
    uint32_t flags;
    uint32_t max_active;     /* jobs resident at once (0: 256) */
    uint32_t depth;          /* bursts of ticks in flight on the device (0: 4) */
    uint64_t budget_bytes;   /* device bytes all resident jobs may hold (0: no limit beyond the domain's) */
    uint64_t reserve_bytes;  /* device memory left free at every admission (0: max(total/16, 512 MiB)) */
    uint64_t tick_points;    /* grid points stepped per tick (0: 8,000,000) */
    uint64_t burst_points;   /* grid points issued per scheduling decision (0: 32,000,000) */
    double starve_s;         /* a job waiting longer than this since its arrival goes first, oldest first
                                (0: least remaining work always decides) */
} f2c_serve_options_v1;

/* Job flags. F2C_SERVE_KEEP_RESULT: publish the final fields to host memory
 * the server holds until f2c_serve_release_v1. */
#define F2C_SERVE_KEEP_RESULT 1u

typedef struct f2c_serve_job_v1 {
    int64_t nx, ny, nz, halo;   /* interior cells and ghost layers */
    double dx, dy, dz, dt;
    int32_t nscalar;            /* 0..F2C_MAX_SCALARS */
    int32_t steps;              /* >= 1 */
    uint64_t seed;              /* initial fields: f2c_seed_fields_v1 */
    double arrival;             /* seconds on the server clock; not admitted earlier */
    uint32_t flags;
    uint32_t reserved;          /* 0 */
} f2c_serve_job_v1;

typedef struct f2c_serve_done_v1 {
    uint64_t id;
    double arrival, admitted, finished;  /* seconds on the server clock */
    int32_t status;                      /* FORT_SCOPE_OK, or why the job failed */
    int32_t reserved;
} f2c_serve_done_v1;

typedef struct f2c_serve_stats_v1 {
    uint32_t version, reserved;
    uint64_t admitted, finished, ticks, bursts, graph_builds, graph_replays, direct_launches, plan_builds;
    uint64_t refused_admissions;  /* admission attempts a job failed to fit (it waited) */
    uint64_t peak_active, peak_job_bytes;
    double idle_s;                /* worker time with no resident job and nothing in flight */
} f2c_serve_stats_v1;

/* Start a server on `context` (its domain, device, stream and numerical
 * contract). The worker thread becomes the context's only caller until
 * f2c_serve_destroy_v1. */
int f2c_serve_create_v1(fort_scope_t context, const f2c_serve_options_v1 *options, f2c_server_t *server);
/* Queue a job (any thread). Jobs are admitted in arrival order. */
int f2c_serve_submit_v1(f2c_server_t server, const f2c_serve_job_v1 *job, uint64_t *id);
/* Seconds since the server started (the clock of arrivals and completions). */
double f2c_serve_clock_v1(f2c_server_t server);
/* Move up to `capacity` finished jobs into `done`; *count receives how many. */
int f2c_serve_poll_v1(f2c_server_t server, f2c_serve_done_v1 *done, size_t capacity, size_t *count);
/* Wait until every submitted job has finished (timeout_s < 0: no limit).
 * FORT_SCOPE_STATE on timeout; the first failure's status if the worker failed. */
int f2c_serve_drain_v1(f2c_server_t server, double timeout_s);
/* Host copy of a finished F2C_SERVE_KEEP_RESULT job's field (0 U, 1 V, 2 W,
 * 3.. scalars), padded layout, valid until f2c_serve_release_v1. */
int f2c_serve_result_v1(f2c_server_t server, uint64_t id, int32_t field, const double **host);
int f2c_serve_release_v1(f2c_server_t server, uint64_t id);
int f2c_serve_stats_get_v1(f2c_server_t server, f2c_serve_stats_v1 *stats);
/* Last failure text of the server (never NULL). */
const char *f2c_serve_error_v1(f2c_server_t server);
/* Stop the worker (jobs not finished are dropped: their arrays are released)
 * and free the server. No other call on the same server may overlap it. */
int f2c_serve_destroy_v1(f2c_server_t server);

#ifdef __cplusplus
}
#endif
#endif
