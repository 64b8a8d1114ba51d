/*
 * pfdd_gpu.h -- C ABI of the GB300-native PFDD TDGL hot path.
 *
 * The reference program (trungnnguyen/PFDD2, one C file PFDD_Final_GPU.c,
 * cited F:<line>) runs its TDGL loop in `main` (F:4574-4691): copy xi to a
 * float buffer, `fft_forward(data, NSV)`, contract with the interaction matrix
 * B(k), `fft_backward(data2, NS)`, then `plasticevolv` (F:3470-3501).  Its
 * swappable boundary is the FFT pair `fft_forward(float*, int batch)` /
 * `fft_backward(float*, int batch)` (F:209-273) with FOURN, FFTW or cuFFT
 * behind it.  This library replaces both levels:
 *
 *   - the whole step (pfdd_create .. pfdd_step .. pfdd_get_state), with xi,
 *     B(k) and the spectral work buffers resident on the GPU, and
 *   - the FFT boundary itself (pfdd_fft_*), a drop-in for fft_forward /
 *     fft_backward on caller-owned host or device buffers.
 *
 * Conventions (all from the reference):
 *   - grid N1 x N2 x N3, each a power of two in [1, 512]; N = N1*N2*N3;
 *   - field layout [field][i][j][k] with k fastest, complex values
 *     interleaved [re, im] (F:38-65);
 *   - forward transform exp(-2 pi i n.k / N), backward exp(+2 pi i n.k / N),
 *     neither normalised (F:209-273); the step divides by N as
 *     plasticevolv does (F:3488-3489);
 *   - the constant pi in the update is the reference's truncated
 *     3.141592654 (F:95).
 *
 * Every call returns a status; nothing calls exit() or assert().  A context
 * is used by one host thread at a time; distinct contexts may be driven from
 * distinct threads (each owns its own CUDA stream).
 */
#ifndef PFDD_GPU_H
#define PFDD_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  PFDD_OK = 0,
  PFDD_EINVAL = 1,      /* bad argument (size, pointer, replica index, state) */
  PFDD_ENOMEM = 2,      /* device or host allocation failed */
  PFDD_ECUDA = 3,       /* a CUDA runtime call failed; see pfdd_last_error */
  PFDD_ETIMEOUT = 4,    /* a bounded device-side wait ran out */
  PFDD_ENONFINITE = 5,  /* the state became NaN/Inf (divergence watchdog) */
  PFDD_ENOTREADY = 6,   /* a required input (B, parameters, state) was not set */
  PFDD_ELIMIT = 7       /* size beyond a fixed capacity (pfdd_fft_device_noalloc) */
} pfdd_status;

typedef enum {
  PFDD_FP64 = 0,          /* plain form: FFTs, contraction and update in FP64 */
  PFDD_FFT_FP32 = 1,      /* precision form: complex64 FFTs + FP32 contraction with B(k) built in
                             FP64 and stored rounded to FP32; FP64 state and sums */
  PFDD_FFT_FP32_BFLY = 2  /* as PFDD_FFT_FP32, but the x-pass evaluates B(k) in FP32 registers
                             from the same closed form instead of reading a stored table (no B
                             memory, 4 bytes x ns(ns+1)/2 less traffic per point and step); needs
                             pfdd_build_B and 32 <= N1 <= 256.  Whole-step contexts only. */
} pfdd_precision;

typedef struct pfdd_ctx pfdd_ctx;

/* ---- whole-step interface: replaces F:4574-4691 -------------------------- */

/* One solve.  Replaces the allocations of F:4137-4166 for the hot path. */
pfdd_status pfdd_create(pfdd_ctx **ctx, int n1, int n2, int n3, int ns, int precision, int device);

/* `nrep` independent solves of the same grid/system count that share one B(k)
 * (batched replicas / serving slots).  nrep >= 1. */
pfdd_status pfdd_create_batched(pfdd_ctx **ctx, int n1, int n2, int n3, int ns, int nrep, int precision,
                                int device);

void pfdd_destroy(pfdd_ctx *ctx);

/* Message of the last failed call on this context ("" if none). */
const char *pfdd_last_error(const pfdd_ctx *ctx);

/* Interaction matrix from host memory, FP64, the reference's BB layout
 * restricted to the slip block: B[kb][ka][i][j][k] for ka, kb < ns
 * (F:59 with I5, filled by Bmatrix F:328-412).  Copied; symmetric in (ka,kb). */
pfdd_status pfdd_set_B(pfdd_ctx *ctx, const double *B);

/* Builds B(k) on the device in FP64 from the cubic elastic constants and the
 * eigenstrains eps[ns][3][3] (seteps F:1912-1980), grid spacings d1,d2,d3 and
 * the frequency convention of frec (F:2683-2754).  Same formula as Bmatrix
 * (F:328-412), evaluated in closed form.  FP32 contexts round it after. */
pfdd_status pfdd_build_B(pfdd_ctx *ctx, double C11, double C12, double C44, const double *eps, double d1,
                         double d2, double d3);

/* Copies the context's B(k) back to the host as FP64 in the pfdd_set_B layout
 * B[kb][ka][N] (FP32 contexts return their rounded values).  Replaces reading
 * the reference's BB array after Bmatrix (F:4325). */
pfdd_status pfdd_get_B(pfdd_ctx *ctx, double *B);

/* Kinetic and core-energy coefficients per slip system (CD2, Asf2, dslip2 of
 * F:4277-4297, 2495-2498) and the scalar uq2 (F:4194). */
pfdd_status pfdd_set_params(pfdd_ctx *ctx, const double *cd2, const double *asf, const double *dslip, double uq2);

/* Order parameter and boundary flags of every replica:
 * xi[nrep][ns][N][2] and xi_bc[nrep][ns][N][2] (xi.dat / xi_bc.dat layout for
 * the slip fields, F:4366-4382).  A point evolves where xi_bc[...][0] == 0
 * (F:3481).  xi_bc may be NULL: every point evolves. */
pfdd_status pfdd_set_state(pfdd_ctx *ctx, const double *xi, const double *xi_bc);

/* Same for one replica r (xi[ns][N][2]); the other replicas are untouched. */
pfdd_status pfdd_set_replica_state(pfdd_ctx *ctx, int r, const double *xi, const double *xi_bc);

/* Optional spatially varying resolved shear stress tau(x) (resolSS,
 * F:1540-1637), layout tau_field[i][j][k][ns] like the reference's tau array;
 * shared by all replicas.  When set, the per-step values passed to pfdd_step
 * multiply it (the stress-ramp factor); NULL clears it. */
pfdd_status pfdd_set_tau_field(pfdd_ctx *ctx, const double *tau_field);

/* Runs `nsteps` explicit Euler TDGL steps (plasticevolv, F:3470-3501; loop
 * F:4574-4691).  tau[nsteps][nrep][ns] is the resolved shear stress of each
 * step (or the multiplier of the tau field).  Outputs, if non-NULL:
 * gamma[nsteps][nrep] (average plastic strain, F:3494) and
 * gamma_a[nsteps][nrep][ns] (per system, F:3495). */
pfdd_status pfdd_step(pfdd_ctx *ctx, int nsteps, const double *tau, double *gamma, double *gamma_a);

/* The inner loop's convergence stop (plasticconverge, F:3732-3785, applied by
 * the do-while at F:4574-4691), for a one-solve context (nrep == 1).
 *
 * pfdd_converge_reset starts an inner loop (F:4567-4572): it clears the
 * per-step pass marks and the count of full windows; gamma_prev is the gamma
 * the loop's first step is compared with (the last gamma of the previous
 * loop, 0.0 before the first, F:4192 / F:4575).
 *
 * pfdd_step_converge then runs up to max_steps steps like pfdd_step and stops
 * after the step at which the reference leaves the loop: a step passes when
 * |(gamma - gamma_last) / gamma| < 1e-8 or |gamma| < 1e-12 (for gamma == 0:
 * |gamma - gamma_last| < 1e-15 or |gamma| < 1e-14); from the loop's 30th
 * step on, a passing step adds one to a count when it and the 29 steps before
 * it all passed and resets the count otherwise (a failing step leaves it),
 * and the loop ends at the fifth count.  tau[max_steps][ns] as for pfdd_step; gamma[max_steps]
 * and gamma_a[max_steps][ns] (may be NULL) receive the steps that ran;
 * *steps_done = how many (== max_steps when the loop did not converge; on an
 * error, the steps of the chunks completed before it).  The
 * pass marks carry over between calls, so a loop may be run in pieces.  The
 * state after the call is the state after the last step that ran: steps run
 * in chunks no longer than the fewest steps to the next possible stop, so no
 * chunk runs past it. */
pfdd_status pfdd_converge_reset(pfdd_ctx *ctx, double gamma_prev);
pfdd_status pfdd_step_converge(pfdd_ctx *ctx, int max_steps, const double *tau, double *gamma, double *gamma_a,
                               int *steps_done);

/* The same for every replica of a batched context, each with its own test
 * and stop: pfdd_converge_reset_batched takes gamma_prev[nrep] (and
 * pfdd_converge_reset sets all replicas alike); pfdd_step_converge_batched
 * takes tau[max_steps][nrep][ns] and writes gamma[max_steps][nrep],
 * gamma_a[max_steps][nrep][ns] (may be NULL) and steps_done[nrep].  The
 * active replicas take part; one that stops leaves the batch (idle, its state
 * that of its stop step) and is active again when the call returns; idle
 * replicas are left alone (steps_done 0).  Chunks end at the first possible
 * stop of any running replica. */
pfdd_status pfdd_converge_reset_batched(pfdd_ctx *ctx, const double *gamma_prev);
pfdd_status pfdd_step_converge_batched(pfdd_ctx *ctx, int max_steps, const double *tau, double *gamma,
                                       double *gamma_a, int *steps_done);

/* Copies xi of every replica back: xi[nrep][ns][N][2]. */
pfdd_status pfdd_get_state(pfdd_ctx *ctx, double *xi);
pfdd_status pfdd_get_replica_state(pfdd_ctx *ctx, int r, double *xi);

/* Marks replica r active (1) or idle (0).  Idle replicas are skipped by every
 * kernel of a step and keep their state (serving slots). */
pfdd_status pfdd_set_replica_active(pfdd_ctx *ctx, int r, int active);

/* Number of kernel launches issued by the last pfdd_step call. */
long long pfdd_last_launch_count(const pfdd_ctx *ctx);

/* The context's CUDA stream (a cudaStream_t), so callers can order their own
 * work and events against the step. */
void *pfdd_get_stream(pfdd_ctx *ctx);

/* Recreates the context's stream with a CUDA stream priority (lower = more
 * urgent; clamped to the device's range, cudaDeviceGetStreamPriorityRange).
 * No counterpart in the reference (one solve per process); the server gives
 * classes of small solves more urgent streams so that their short steps are
 * not queued behind the kernels of large grids. */
pfdd_status pfdd_set_stream_priority(pfdd_ctx *ctx, int priority);

/* Measurement: with timing on, every kernel launch of the context is bracketed
 * by a CUDA event pair on the context's stream.  pfdd_kernel_stat reports, for
 * kernel kind idx (0 .. until it returns PFDD_EINVAL), its name, the number of
 * timed launches and their total device time since timing was (re)enabled. */
pfdd_status pfdd_set_kernel_timing(pfdd_ctx *ctx, int enable);
pfdd_status pfdd_kernel_stat(pfdd_ctx *ctx, int idx, const char **name, long long *launches, double *total_ms);

/* Strain and stress fields of replica r's current state, in FP64 whatever the
 * context's precision: the reference's strain (F:752-835, with the F matrix of
 * Fmatrix, F:414-598, and the microscopic strain of avestrain, F:641-749) and
 * stress (F:837-972), and their grid means (F:4063-4072, F:920).  sigma_app
 * [3][3]: the uniform applied stress in units of C44 (the reference's sigma
 * array, setstress F:3820-3918).  Outputs, each may be NULL: eps[9][N] and
 * sigma[9][N] (component 3*i + j, the real parts of DATAEPS and DATASIGMA),
 * aveps[9] and avesigma[9].  Needs the constants and eigenstrains of
 * pfdd_build_B.  Its work buffers, about (ns + 6)*N complex doubles plus 9*N
 * doubles for each field output requested, are allocated by the first call and
 * kept by the context until pfdd_destroy; the state is not changed. */
pfdd_status pfdd_strain_stress(pfdd_ctx *ctx, int r, const double *sigma_app, double *eps, double *sigma,
                               double *aveps, double *avesigma);

/* Interface-plane energy diagnostics of the reference's checkEnergy.dat and
 * checkEbarrier.dat (avestrain F:641-749, ResidualEnergy F:3920-3945, the
 * inner-loop block F:4645-4651).  They are sums over the points of the
 * interface plane: grid index i == ppoint[0] and |n . (x - ppoint)| <= 1. */
typedef struct {
  int ppoint[3];          /* the plane's penetration point (F:4196-4198: N1/2, 0, 3*N3/4) */
  double interface_n[3];  /* plane normal in the global frame (F:4215-4217) */
  double sigma[3][3];     /* the applied stress (uniform sigma of setstress, F:3820-3918) */
  double S11, S12, S44;   /* compliances (F:4261-4263) */
  double mu;              /* C44 */
  double D[4];            /* D00, D01, D10, D11 of ResidualEnergy (calculateD4int, F:3503) */
  int ns_per_material;    /* NS1 (ResidualEnergy's material of system a is a / NS1); 0 means ns */
} pfdd_diag_params;

/* Turns the per-step diagnostics on (p != NULL) or off.  While on, every step
 * of pfdd_step also gathers Re xi of every system on the interface plane and
 * on the line (ppoint[0], j, ppoint[2]); pfdd_get_diagnostics returns the
 * energies of the last pfdd_step call. */
pfdd_status pfdd_set_diagnostics(pfdd_ctx *ctx, const pfdd_diag_params *p);

/* Energies of each step of the last pfdd_step call, out[nsteps][nrep][6]:
 * energy_in (elastic energy of the virtual strain fields, Energy_calculation
 * F:3026-3467), energy_in2 (Imatrix F:2504-2616), energy_in3 (avestrain's
 * -sum over the plane of (sum_a Re xi_a eps_a) : sigma), energy_in4
 * (avestrain's -mu/2 sum over the plane of S : sigma : sigma, one call's worth:
 * the reference adds it once per call and resets it once per outer step),
 * energy_Residual, and their sum energy_intotal, each summed in the
 * reference's order.  This library carries no virtual strain fields (one
 * material), so energy_in and energy_in2 are 0 as in the reference's
 * one-material runs.  nsteps must be the last call's step count. */
pfdd_status pfdd_get_diagnostics(pfdd_ctx *ctx, int nsteps, double *out);

/* The same energies for the current state of every replica (the line the
 * reference writes for an outer step before its inner loop): out[nrep][6]. */
pfdd_status pfdd_state_diagnostics(pfdd_ctx *ctx, double *out);

/* Launch plan of the context as a JSON object: tile widths, threads and shared
 * memory of each pass, the radix plan of each axis, the steps per captured CUDA
 * graph and the autotune timings (null before the first pfdd_step, which times
 * every x-pass and y-pass tile width that fits and keeps the fastest; set
 * PFDD_NO_TUNE=1 to keep the defaults).  No counterpart in the reference. */
pfdd_status pfdd_get_plan(pfdd_ctx *ctx, char *buf, size_t len);

/* Device bytes held by a context of this shape (admission control). */
size_t pfdd_required_bytes(int n1, int n2, int n3, int ns, int nrep, int precision);

/* ---- FFT boundary: drop-in for fft_forward / fft_backward (F:209-273) ---- */

typedef struct pfdd_fft_plan pfdd_fft_plan;

/* Plan for in-place, unnormalised 3D C2C transforms of an N1 x N2 x N3 grid
 * (cufftPlan3d(N1,N2,N3,CUFFT_C2C) of F:170-173).  precision selects complex64
 * (PFDD_FFT_FP32, the reference's float buffers) or complex128 (PFDD_FP64,
 * the -Dfloat=double build).  max_batch bounds `batch` below. */
pfdd_status pfdd_fft_plan_create(pfdd_fft_plan **plan, int n1, int n2, int n3, int precision, int max_batch,
                                 int device);
void pfdd_fft_plan_destroy(pfdd_fft_plan *plan);

/* fft_forward(data, batch) / fft_backward(data, batch): `batch` contiguous
 * fields of 2*N values each, interleaved complex.  `data` is a host pointer
 * (copied to the device and back, as the reference's `acc data copy` does,
 * F:4446-4450) or a device pointer (on_device = 1).  float for FP32 plans,
 * double for FP64 plans. */
pfdd_status pfdd_fft_forward(pfdd_fft_plan *plan, void *data, int batch, int on_device);
pfdd_status pfdd_fft_backward(pfdd_fft_plan *plan, void *data, int batch, int on_device);

/* In-place 3D C2C transform (fft_forward sign = -1, fft_backward sign = +1,
 * unnormalised) of `batch` fields of 2*N values on the device, enqueued on
 * `stream` (a cudaStream_t; NULL = legacy default stream) -- without any device
 * allocation.  No counterpart in the reference: it exists for callers that
 * cannot allocate device memory themselves, such as code inside an OpenACC
 * data region whose device memory belongs to the OpenACC runtime, or a
 * process held to a fixed device-memory budget.  Its only scratch, the twiddle
 * tables, is one static device array in the library (24 KB, held by every GPU
 * that loads the library until the process exits), so N1, N2, N3 are limited
 * to powers of two <= 512: larger sizes return PFDD_ELIMIT, a batch whose
 * launch grids would exceed 2^31 - 1 blocks and other invalid arguments
 * PFDD_EINVAL.  The first call on a device looks up the array's device
 * address (again whenever the current CUDA context is not the one it was
 * looked up in); make that first call before any stream capture.  The cached
 * address does not survive cudaDeviceReset: do not reset a device between
 * calls of a process that uses this entry point.  Under CUDA's
 * default lazy module loading the first call on a device, and the first call
 * of each new line length, may load kernel code, which takes device memory:
 * make those calls once at set-up (or set CUDA_MODULE_LOADING=EAGER) if the
 * budget leaves no room for that later.  All calls share the array and each
 * rewrites it before use, so calls that overlap on the GPU (different
 * streams, or different threads) race: serialise them.  Calls queued one
 * after another on one stream are ordered.  The call returns after
 * enqueueing; synchronise `stream` before reading `data`. */
pfdd_status pfdd_fft_device_noalloc(void *data, int n1, int n2, int n3, int batch, int precision, int sign,
                                    void *stream);

const char *pfdd_status_string(int status);

#ifdef __cplusplus
}
#endif

#endif /* PFDD_GPU_H */
