/*
 * gbx_serve.h -- serving loop for coupled-cluster iteration requests.
 *
 * Many concurrent CC jobs (gbx_cc.h) of different sizes send iteration
 * requests.  The server keeps each admitted job's integrals, amplitudes and
 * plans resident on the GPU, admits jobs by their planned device footprint
 * (gbx_cc_footprint) against a byte budget, and batches continuously: a
 * request starts as soon as a stream slot is free and its job is resident
 * and idle, so requests that arrive while others run overlap with them on the
 * device.  A job's iterations run in order; its state is released after its
 * last request.  Every request's latency is recorded.
 *
 * The reference has no serving layer (its jobs are single MPI runs); this is
 * the request loop around the node-local contraction path.  A resident job
 * with no request waiting may be evicted to admit another: its amplitudes
 * move to pinned host memory and come back, with the job rebuilt, when its
 * next request arrives; its results do not change.
 */
#ifndef GBX_SERVE_H
#define GBX_SERVE_H
#include "gbx_cc.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    double budget_bytes; /* device bytes the resident job states may take together */
    int slots;           /* requests in flight on the GPU at once (one CUDA stream each) */
    int reserved;
} gbx_serve_config;

typedef struct {
    int job;             /* job id from gbx_server_add_job */
    int iteration;       /* 1-based iteration of that job */
    int status;          /* GBX_OK; GBX_ENOMEM when the job's footprint exceeds the budget;
                            GBX_ETIMEOUT when the run's time limit came first; other errors */
    int slot;            /* stream slot that ran it (-1 if it never ran) */
    double arrival;      /* seconds on the server clock */
    double start, end;   /* dispatch to the GPU and completion (seconds) */
    double energy;       /* correlation energy after the iteration */
} gbx_serve_result;

typedef struct {
    int requests, completed, rejected, timed_out;
    int jobs, jobs_admitted, jobs_rejected;
    double makespan_s;          /* first arrival to last completion */
    double iter_per_s;          /* completed requests / makespan */
    double latency_p50_s, latency_p99_s, latency_max_s;  /* end - arrival */
    double service_p50_s;       /* end - start */
    double peak_planned_bytes;  /* largest sum of admitted footprints */
    double peak_measured_bytes; /* largest sum of the resident jobs' measured device bytes */
    double build_s_total;       /* time spent building job states */
    int evictions;              /* idle jobs moved to host memory to admit others */
    int restores;               /* evicted jobs admitted again */
    double evict_s_total;       /* time spent saving evicted job states */
} gbx_serve_stats;

typedef struct gbx_server gbx_server;

GBX_API int gbx_server_create(const gbx_serve_config* cfg, gbx_server** out);
/* Registers a job (host planning only; nothing is allocated yet);
 * footprint_bytes receives its planned resident bytes. */
GBX_API int gbx_server_add_job(gbx_server* s, const gbx_cc_config* cfg, int* job_id, double* footprint_bytes);
/* One iteration request of job_id arriving arrival_s seconds after
 * gbx_server_run starts.  Submit every request before running. */
GBX_API int gbx_server_submit(gbx_server* s, int job_id, double arrival_s);
/* Serves until every request has finished or time_limit_s (> 0) has passed;
 * requests not started by then are marked GBX_ETIMEOUT (requests already on
 * the GPU finish).  A server runs once. */
GBX_API int gbx_server_run(gbx_server* s, double time_limit_s);
/* Results in submission order; *count in: capacity, out: number written
 * (out == NULL: *count receives the number of requests). */
GBX_API int gbx_server_results(const gbx_server* s, gbx_serve_result* out, int* count);
GBX_API int gbx_server_stats(const gbx_server* s, gbx_serve_stats* out);
GBX_API int gbx_server_destroy(gbx_server* s);

#ifdef __cplusplus
}
#endif
#endif /* GBX_SERVE_H */
