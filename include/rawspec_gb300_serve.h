/* rawspec_gb300_serve.h -- a spectrometer job server on one GPU: jobs (each a
 * stream of RAW buffers with its own channels, bits, products and Npolout)
 * are admitted under a device-memory budget, keep their integration state on
 * the device across buffers, and run concurrently: while one job's buffer is
 * being processed, the copies and kernels of the others proceed on their own
 * streams.  Jobs submitted while others run are admitted as soon as a slot and
 * the memory are free.  No counterpart in the reference library, whose CLI
 * processes one stem at a time (rawspec.c:906-1032).
 *
 * Every job is a rawspec_context of this library, driven by the server's
 * request-loop thread with the reference's per-buffer calls
 * (rawspec_copy_blocks_to_gpu_and_start_processing, rawspec_check_for_completion,
 * rawspec_wait_for_completion), so a job's results are those of the same
 * buffers streamed through a context alone. */
#ifndef RAWSPEC_GB300_SERVE_H
#define RAWSPEC_GB300_SERVE_H

#include <stddef.h>

#include "rawspec.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct rawspec_gb300_server rawspec_gb300_server;

/* Dump of one of a job's products: PRE before the job's h_pwrbuf / h_icsbuf
 * are written, POST once they hold the dump (rawspec_context.dump_callback
 * semantics), called from a CUDA callback thread. */
typedef void (*rawspec_gb300_job_dump_fn)(void *user, int job, rawspec_context *ctx, int product,
                                          int callback_type);

enum {
  RAWSPEC_GB300_JOB_PENDING = 0, /* submitted, waiting for a slot and memory */
  RAWSPEC_GB300_JOB_ACTIVE = 1,  /* initialised on the device */
  RAWSPEC_GB300_JOB_DONE = 2,    /* all buffers processed, memory released */
  RAWSPEC_GB300_JOB_FAILED = 3   /* a library call failed; memory released */
};

/* A server on GPU gpu_index that keeps at most max_active jobs initialised
 * and their device memory (rawspec_gb300_device_bytes_estimate) within
 * hbm_budget bytes; each job queues at most max_queued pushed buffers (push
 * blocks beyond that).  NULL on failure. */
rawspec_gb300_server *rawspec_gb300_server_create(int gpu_index, size_t hbm_budget, int max_active,
                                                  int max_queued);

/* Submits a job: the client fields of `job` (No, Np, Nant, Nc, Ntpb, Nbps,
 * Npolout, Nts, Nas, Nb, input_conjugated, incoherently_sum, Naws, Aws) as
 * for rawspec_initialize; Aws is copied.  fft_dir as for
 * rawspec_start_processing.  Returns the job id (>= 0), or -1 if the job is
 * invalid or needs more memory than the whole budget. */
int rawspec_gb300_server_submit(rawspec_gb300_server *s, const rawspec_context *job, int fft_dir,
                                rawspec_gb300_job_dump_fn fn, void *user);

/* Queues one input buffer of a job: Nb blocks of Nc * Ntpb * Np * 2 * Nbps / 8
 * bytes each, in block order (4-bit input: the packed bytes, half that size).
 * The data are copied into one of the job's max_queued page-locked slots,
 * which exist once the job is admitted: a push to a pending job, or to a job
 * whose slots are all queued, waits.  0, or 1 (unknown or closed job, wrong
 * size, time-out of 60 s waiting for a slot). */
int rawspec_gb300_server_push(rawspec_gb300_server *s, int job, const void *data, size_t bytes);

/* No more buffers for the job: once its queue is processed, the job waits
 * for completion, releases its memory and is DONE.  0, or 1. */
int rawspec_gb300_server_close_job(rawspec_gb300_server *s, int job);

/* Waits until the job is DONE or FAILED (timeout_s < 0: no limit).  Returns
 * the job state, or -1 on time-out or an unknown job. */
int rawspec_gb300_server_wait_job(rawspec_gb300_server *s, int job, double timeout_s);

typedef struct {
  int state;
  long long buffers;               /* buffers processed */
  long long dumps;                 /* POST_DUMP callbacks */
  double t_submit, t_admit, t_done;  /* seconds on the server's monotonic clock */
  double buffer_p50_ms, buffer_p99_ms;  /* push of a buffer -> its processing complete */
  double dump_p50_ms, dump_p99_ms;      /* push of the buffer ending a dump -> its POST_DUMP */
  size_t device_bytes;             /* device memory accounted to the job */
} rawspec_gb300_job_stats;

/* A job's statistics; those of finished jobs are kept until the server is
 * destroyed.  0, or 1 for an unknown job. */
int rawspec_gb300_server_job_stats(rawspec_gb300_server *s, int job, rawspec_gb300_job_stats *st);

typedef struct {
  int pending, active, done, failed;
  size_t budget, used, peak_used;  /* device bytes accounted to active jobs */
  int peak_active;
  long long buffers, dumps;
  double buffer_p50_ms, buffer_p99_ms, dump_p50_ms, dump_p99_ms;  /* over all jobs */
  long long group_calls;  /* times several jobs' buffers were started together, their
                             launches of one kernel configuration sharing a grid */
} rawspec_gb300_server_stats;

int rawspec_gb300_server_get_stats(rawspec_gb300_server *s, rawspec_gb300_server_stats *st);

/* Closes every job, waits for all of them and stops the request loop. */
void rawspec_gb300_server_destroy(rawspec_gb300_server *s);

#ifdef __cplusplus
}
#endif

#endif /* RAWSPEC_GB300_SERVE_H */
