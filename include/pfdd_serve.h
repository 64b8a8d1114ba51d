/*
 * pfdd_serve.h -- serving form: a queue of independent PFDD solves on one GPU.
 *
 * The reference program runs one solve per process (main, F:4087-4847).  A
 * server accepts many solves of different grid sizes, slip-system counts,
 * stress ramps and initial states and runs them concurrently:
 *
 *   - solves that share grid, slip systems, elastic and kinetic constants form
 *     a class; a class owns one batched context (pfdd_create_batched) whose
 *     replica slots hold its solves, so B(k) is built and stored once;
 *   - classes are created when the device-memory budget admits them
 *     (pfdd_required_bytes; a class gets fewer slots rather than none when
 *     memory is short) and released when idle; a solve too large for the
 *     whole budget fails with PFDD_ENOMEM;
 *   - each class has its own worker thread and CUDA stream, so the steps of
 *     different classes overlap on the GPU;
 *   - continuous batching: a worker advances its active slots in chunks of
 *     steps, retires solves that reach their step count and admits queued
 *     solves into the freed slots between chunks.  A solve's results do not
 *     depend on what else runs beside it.
 *
 * Stresses follow the ramp of the workloads: step s (0-based) of a solve
 * applies tau_max[a] * ((s + 1.0) / steps).  A converging solve (converge
 * set) ends at its loop's stop if that comes first: its slot's chunks are cut
 * to the fewest steps to that stop, so it is never run past it.
 *
 * Scheduling: free slots take the class's shortest queued solve first; class
 * streams get CUDA priorities by the size of one solve's step (grid points x
 * systems), smaller solves more urgent.  Environment switches read at
 * pfdd_server_create: PFDD_SERVER_TRACE=<file> writes one CSV line per
 * scheduling event (class creation, admission, chunk, finish, release) when
 * the server is destroyed; PFDD_SERVER_EXCLUSIVE=1 lets one class's chunk
 * run on the GPU at a time, most urgent class first (measured slower on the
 * mixed workloads; off by default).
 */
#ifndef PFDD_SERVE_H
#define PFDD_SERVE_H

#include <stddef.h>

#include "pfdd_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pfdd_server pfdd_server;

typedef struct {
  int n1, n2, n3, ns, steps;
  double C11, C12, C44;           /* cubic elastic constants (Bmatrix, F:328-412) */
  double cd2, asf, dslip, uq2;    /* CD2, Asf2, dslip2 (same for every system) and uq2 */
  double d1, d2, d3;              /* grid spacings of frec (F:2683-2754); 0 means 1 */
  const double *eps;              /* [ns][3][3] eigenstrains (seteps, F:1912-1980); copied */
  const double *tau_max;          /* [ns] resolved shear stress at the end of the ramp; copied */
  const double *xi;               /* [ns][N][2] initial order parameter */
  const double *xi_bc;            /* [ns][N][2] pinned flags, or NULL: every point evolves */
  double *xi_out;                 /* [ns][N][2] receives the final xi, or NULL */
  int converge;                   /* nonzero: the solve also ends where the reference's convergence test
                                     ends its inner loop (plasticconverge, F:3732-3785), as
                                     pfdd_step_converge does; `steps` stays the ramp's length */
  double gamma_prev;              /* with converge: the gamma its first step is compared with (F:4575) */
} pfdd_request;

/* precision: PFDD_FP64, PFDD_FFT_FP32 or PFDD_FFT_FP32_BFLY.  hbm_budget: device
 * bytes the server may hold (0: 90% of the free memory at creation).
 * max_slots: replica slots per class.  chunk_steps: steps between admissions. */
pfdd_status pfdd_server_create(pfdd_server **srv, int precision, int device, size_t hbm_budget, int max_slots,
                               int chunk_steps);

/* Queues a solve.  xi, xi_bc and xi_out are not copied: they are read when the
 * solve is admitted and written when it finishes, so they must stay valid (and
 * xi_out untouched) until pfdd_server_wait for this id returns.  *id identifies
 * the solve in pfdd_server_wait. */
pfdd_status pfdd_server_submit(pfdd_server *srv, const pfdd_request *req, long long *id);

/* Blocks until solve `id` has finished (its final xi is then in the request's
 * xi_out).  Outputs (each may be NULL): gamma [steps], gamma_a [steps][ns] and
 * the time from submit to completion in seconds.  Returns the solve's status. */
pfdd_status pfdd_server_wait(pfdd_server *srv, long long id, double *gamma, double *gamma_a, double *latency_s);

/* The same, and the number of steps the solve ran (`steps`, or fewer for a
 * converging solve that stopped; gamma and gamma_a hold zeros beyond it). */
pfdd_status pfdd_server_wait_run(pfdd_server *srv, long long id, double *gamma, double *gamma_a, double *latency_s,
                                 int *steps_run);

/* Totals since creation: solve steps executed, solves finished, classes
 * created, peak device bytes reserved. */
pfdd_status pfdd_server_stats(pfdd_server *srv, long long *steps_done, long long *solves_done,
                              long long *classes_created, size_t *peak_bytes);

/* Finishes every queued solve, then releases the server and its device memory. */
void pfdd_server_destroy(pfdd_server *srv);

#ifdef __cplusplus
}
#endif

#endif
