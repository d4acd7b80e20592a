/*
 * actflow -- GB300-native (sm_103a) integrating-factor RK4 step of the 2-D
 * active-turbulence vorticity equation, behind a plain C ABI.
 *
 * Drop-in boundary.  The reference (DominikSuchla/2D_active_matter_simulation,
 * ActFlow_V3-2.cu) has no library API: its boundary is a process that reads
 * <dir>/specifications.txt and writes ActTurb_snap{i}.bin and energy.txt.  The
 * C++ front end `actflow` (csrc/host/cli.cpp) reproduces that process contract;
 * it, the tests and bench.py drive the solver through the entry points below.
 * Each entry point names the reference code it replaces.
 *
 * Data conventions (identical to the reference's state and snapshot files):
 *  - w_hat: the vorticity as unnormalised DFT coefficients on the Hermitian half
 *    plane, row-major [Ny][Nx/2+1] complex (re, im interleaved), rows in FFT
 *    order ky = 0, 1, ..., Ny/2, -Ny/2+1, ..., -1 (cuFFT R2C output layout,
 *    ActFlow_V3-2.cu:507, 665; snapshot layout ActFlow_V3-2.cu:1261-1262).
 *    Element type: float for AM_FP32 handles, double for AM_FP64 and AM_DF64
 *    handles.
 *  - mean[2]: the mean velocity scaled by Nx*Ny, i.e. the k = 0 entries of the
 *    unnormalised velocity spectra (ActFlow_V3-2.cu:1053-1054, 1263).
 *  - energy: E = sum(ux^2 + uy^2) / (2 (Nx Ny)^3) of the state at the start of
 *    each step (ActFlow_V3-2.cu:1118-1127), accumulated in double.
 *
 * Threading: a handle is not thread-safe; distinct handles are independent.
 * Every call returns a status and never aborts the process.
 */
#ifndef ACTFLOW_H
#define ACTFLOW_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    AM_OK = 0,
    AM_ERR_ARG = 1,          /* invalid argument / unsupported size */
    AM_ERR_CUDA = 2,         /* CUDA runtime error (no device, launch failure) */
    AM_ERR_NAN = 3,          /* Re w(0,0) became NaN (ActFlow_V3-2.cu:850-861) */
    AM_ERR_IO = 4,           /* file could not be read or written */
    AM_ERR_SPEC = 5,         /* malformed specifications.txt / unknown key */
    AM_ERR_OOM = 6,          /* device allocation failed */
    AM_ERR_UNSUPPORTED = 7,  /* request outside what the library supports */
    AM_ERR_TIMEOUT = 8       /* a wait ran out before the result was ready */
} am_status;

/* State precision.  AM_DF64 ("double-float") holds every real as the
 * unevaluated sum of two floats (about 48 significant bits against double's 53)
 * and computes with FP32 instructions only: on GB300, whose FP64 units have a
 * small fraction of the FP32 throughput, it runs an FP64-class simulation
 * several times faster than AM_FP64.  Its state is exchanged with the host as
 * double; handles only (am_step_noalloc, ensembles and ragged batches refuse
 * it); integrating factors from the double table by default. */
typedef enum { AM_FP32 = 0, AM_FP64 = 1, AM_DF64 = 2 } am_precision;

/* Dealiasing of the nonlinear term.  REFERENCE reproduces cutoff_func
 * (ActFlow_V3-2.cu:899-919) including its 32-bit overflow of the radius (every
 * mode kept up to 256^2 and at 384^2/768^2, only k = 0 at 512^2..4096^2); HALF
 * is the isotropic 1/2 rule (kx/kx_max)^2 + (ky/ky_max)^2 <= 1/4; NONE keeps
 * every mode. */
typedef enum { AM_DEALIAS_REFERENCE = 0, AM_DEALIAS_HALF = 1, AM_DEALIAS_NONE = 2 } am_dealias;

/* Linear operator L(k).  REFERENCE: -(1 - k^2)^2 - alpha (lin_func,
 * ActFlow_V3-2.cu:1030), mean-flow factor exp(-(1 + alpha) dt)
 * (ActFlow_V3-2.cu:704).  GENERAL: -alpha - gamma0 k^2 - gamma2 k^4 with
 * mean-flow factor exp(-alpha dt) -- the dimensional form of the same model. */
typedef enum { AM_FORM_REFERENCE = 0, AM_FORM_GENERAL = 1 } am_form;

/* Integrating factors exp(L(k) dt) and exp(L(k) dt / 2).  FLOAT evaluates them
 * per value in the state's precision inside the step, as lin_func does
 * (ActFlow_V3-2.cu:1020-1033, float exp); DOUBLE precomputes them once per
 * simulation in double (double wavenumbers and parameters) and rounds them to
 * the state's precision -- the precision form, where FP32 runs keep the
 * exponentials at FP64 accuracy.  AUTO: DOUBLE, except FP32 with the
 * reference's mask (the parity mode), which uses FLOAT like the reference. */
typedef enum { AM_IF_AUTO = 0, AM_IF_FLOAT = 1, AM_IF_DOUBLE = 2 } am_if_factors;

typedef struct am_params {
    int nx, ny;              /* grid; powers of two, 8..4096 (FP64: Ny <= 4096) */
    double lx, ly;           /* box lengths */
    double dt;               /* time step */
    double lambda, alpha, beta;
    double gamma0, gamma2;   /* AM_FORM_GENERAL only */
    int form;                /* am_form */
    int dealias;             /* am_dealias */
    int precision;           /* am_precision */
    int if_factors;          /* am_if_factors; 0 = AM_IF_AUTO */
    int reserved[4];         /* must be zero */
} am_params;

typedef struct am_handle am_handle;
typedef struct am_server am_server;

/* Allocate device buffers, twiddle and wavenumber tables and the integrating
 * factors for one simulation.  Replaces the reference's set-up
 * (ActFlow_V3-2.cu:409-521: derived parameters, cudaMallocManaged of every
 * array, cufftPlan2d, wavenumber_func, cutoff_func) and lin_func / lin_v
 * (ActFlow_V3-2.cu:699-705). */
am_status am_create(const am_params *p, am_handle **out);

/* Free everything (unallocate_func, ActFlow_V3-2.cu:1280-1326). */
am_status am_destroy(am_handle *h);

/* Run all work of this handle on `cuda_stream` (a cudaStream_t; NULL selects
 * the handle's own stream).  The reference runs on the default stream. */
am_status am_set_stream(am_handle *h, void *cuda_stream);

/* Load the state from host memory: w_hat [Ny][Nx/2+1] complex in the handle's
 * precision, mean[2] scaled mean velocity.  Replaces reading a snapshot into
 * w_new and the mean scalars (ActFlow_V3-2.cu:620-631). */
am_status am_set_state(am_handle *h, const void *w_hat, const double mean[2]);

/* Load the state from a real-space field w_real [Ny][Nx] (handle precision):
 * forward R2C on the device, then, when `mask_and_zero_mean` is nonzero, the
 * dealias mask and w(0,0) = 0 -- the reference's processing of a fresh initial
 * condition (ActFlow_V3-2.cu:660-679). */
am_status am_set_state_real(am_handle *h, const void *w_real, const double mean[2], int mask_and_zero_mean);

/* Copy the state to host memory (same layout as am_set_state).  Replaces the
 * device-to-host copy of save_func (ActFlow_V3-2.cu:1259-1263). */
am_status am_get_state(am_handle *h, void *w_hat, double mean[2]);

/* Advance nsteps integrating-factor RK4 steps (the time loop body,
 * ActFlow_V3-2.cu:718-862).  energy, if not NULL, receives nsteps values: the
 * energy of the state at the start of each step.  Returns AM_ERR_NAN if Re
 * w(0,0) became NaN (check_func, ActFlow_V3-2.cu:884-897); *nan_step (if not
 * NULL) then holds the 0-based index of that step within this call, otherwise -1. */
am_status am_step(am_handle *h, int nsteps, double *energy, int *nan_step);

/* Enqueue nsteps steps on the handle's stream and return without waiting.  The
 * energies stay on the device; am_sync waits and reports a NaN. */
am_status am_step_async(am_handle *h, int nsteps);
am_status am_sync(am_handle *h);

/* Advance nsteps steps as am_step does (one CUDA graph per step, the 8
 * kernels back to back), with a timing event recorded inside the graph before
 * and after each kernel, and add each kernel's duration (milliseconds) to
 * row_ms[stage-1] / col_ms[stage-1] (stage 1..4).  The host waits for every
 * step, so use it for measurement; am_step is the production path.  No
 * counterpart in the reference, which times only its whole loop
 * (ActFlow_V3-2.cu:713, 841-843). */
am_status am_step_profiled(am_handle *h, int nsteps, double row_ms[4], double col_ms[4]);

/* Enqueue reps times the four row passes of one step, as one CUDA graph, on
 * the handle's stream and return without waiting.  For measurement: a row
 * pass reads the stage input and writes only the products and row sums, which
 * the next step's row pass rewrites before any column pass reads them, so the
 * state is left as it was.  No counterpart in the reference. */
am_status am_row_passes_async(am_handle *h, int reps);

/* Advance nsteps steps without allocating anything.  No counterpart in the
 * reference: it exists for callers that may not allocate device memory -- a
 * plug-in whose host application owns the device-memory budget, or a real-time
 * loop that cannot take cudaMalloc's synchronisation and latency.  All buffers
 * are the caller's and live in device memory: w_hat [Ny][Nx/2+1] complex of the
 * precision in p (read, then overwritten with the new state), mean[2] (scaled
 * mean velocity, read and overwritten), energy[nsteps] (energy of the state
 * entering each step) or NULL.  Every intermediate buffer comes from one
 * library-owned device array of 8 MiB (held by every GPU that loads the
 * library until the process exits).  A call needs 7 fields of
 * ceil((Nx/2+1)/W)*W*Ny complex values (W = 4 in FP32, 2 in FP64; each field
 * rounded up to 256 bytes) plus at most 24*(Nx+Ny) + 56*Ny bytes of tables and
 * sums; grids that do not fit are refused with AM_ERR_UNSUPPORTED before
 * anything is touched.  In practice FP32 takes Nx*Ny <= 2^18 (512^2, 1024x256,
 * 256x1024, ...) except 64x4096, FP64 Nx*Ny <= 2^17 except 32x4096.  The same
 * parameter checks as am_create apply (AM_ERR_ARG).
 * The first call on a device looks up that array's device address (do it before
 * any stream capture); the address is kept for the process, so a device that
 * has been through cudaDeviceReset must not be used with this entry point again
 * (the reset destroyed the array).  The work is enqueued on `stream` (a
 * cudaStream_t, NULL = default stream) and the call returns without waiting; it
 * runs the full transforms, evaluates the integrating factors per value in the
 * state's precision whatever p->if_factors asks (a table would not fit the
 * array), and reports no NaN (check mean or the energies).  FP32 and FP64
 * only (AM_DF64: AM_ERR_UNSUPPORTED).
 * Calls share the array: calls that overlap on the GPU race and must be
 * serialised. */
am_status am_step_noalloc(const am_params *p, void *w_hat, double *mean, int nsteps, double *energy, void *stream);

/* ------------------------------------------------------------ ensembles --
 * A batch advances B simulations of one grid with the same launches (each pass
 * is one launch over all members, a step one CUDA graph).  The reference runs
 * one simulation per process; a batch is that loop (ActFlow_V3-2.cu:718-862)
 * for B independent states at once.  All members share nx, ny, lx, ly, dt,
 * form and dealias; lambda, alpha, beta, gamma0, gamma2 may differ.  FP32,
 * grids 128..1024 per axis.  Each member computes exactly what a handle with
 * its parameters computes. */
typedef struct am_batch am_batch;
am_status am_batch_create(const am_params *params /* [nmembers] */, int nmembers, am_batch **out);
am_status am_batch_destroy(am_batch *b);
/* Member state in and out, as am_set_state / am_get_state (host buffers). */
am_status am_batch_set_state(am_batch *b, int member, const void *w_hat, const double mean[2]);
am_status am_batch_get_state(am_batch *b, int member, void *w_hat, double mean[2]);
/* nsteps steps for every member; energy, if not NULL, receives [nsteps][B]
 * values.  AM_ERR_NAN names the first member whose w(0,0) became NaN. */
am_status am_batch_step(am_batch *b, int nsteps, double *energy, int *nan_member);
const char *am_batch_last_error(const am_batch *b);

/* ------------------------------------------------------- ragged batches --
 * A ragged batch advances R simulations of DIFFERENT grid sizes, parameters,
 * time steps and step counts together.  The reference runs one simulation per
 * process (its time loop, ActFlow_V3-2.cu:718-862); a ragged batch is that loop
 * for R independent runs.  Runs are grouped by grid size, largest first.  In
 * the default per-class mode each pass is one launch per size class (the
 * class's tuned shapes), the classes running as parallel branches of one CUDA
 * graph per step.  In work-list mode each pass of a step is ONE launch over a
 * list of (run, CTA) items of every active run, sorted by grid size, largest
 * first (8 launches per step whatever the sizes; radix-8 row and narrow
 * column passes for every size).  A run stops at its own step count.  FP32, grids
 * 128..1024 per axis.  Each run computes exactly what a handle with its
 * parameters and the same launch shapes computes. */
typedef struct am_ragged am_ragged;
am_status am_ragged_create(const am_params *params /* [nruns] */, const long long *nsteps /* [nruns] */,
                           int nruns, am_ragged **out);
am_status am_ragged_destroy(am_ragged *r);
/* Run state in and out, as am_set_state / am_get_state (host buffers). */
am_status am_ragged_set_state(am_ragged *r, int run, const void *w_hat, const double mean[2]);
am_status am_ragged_get_state(am_ragged *r, int run, void *w_hat, double mean[2]);
/* Advance every run to its step count.  energy, if not NULL, is an array of
 * nruns pointers, each NULL or receiving nsteps[run] energies.  AM_ERR_NAN
 * names the first run whose w(0,0) became NaN.  *grid_point_steps receives
 * the sum of Nx*Ny*steps advanced. */
am_status am_ragged_run(am_ragged *r, double *const *energy, int *nan_run, long long *grid_point_steps);
long long am_ragged_device_bytes(const am_ragged *r);
int am_ragged_classes(const am_ragged *r);
/* 0: one launch per size class per pass (default); 1: one launch per pass
 * over the work list.  Takes effect at the next am_ragged_run. */
am_status am_ragged_set_mode(am_ragged *r, int mode);
const char *am_ragged_last_error(const am_ragged *r);

/* ------------------------------------------------------------- serving --
 * A server takes simulation requests (grid, parameters, precision, seed or
 * initial state, step count) from any thread and runs them with continuous
 * batching on one GPU: requests are admitted while their device footprint
 * fits the HBM budget and an active slot is free, each admitted request
 * advances in chunks of steps on its own stream (so the kernels of different
 * requests overlap on the device), and a request that arrives while others run
 * is admitted as soon as memory and a slot free up.  The reference has no
 * counterpart (one simulation per process, ActFlow_V3-2.cu:214-878); each
 * request computes exactly what a lone handle computes. */
typedef enum { AM_ORDER_ARRIVAL = 0, AM_ORDER_SHORTEST_FIRST = 1 } am_order;

typedef struct am_server_config {
    long long hbm_budget_bytes;  /* device bytes the admitted requests may hold (0: 180 GiB) */
    int max_active;              /* requests on the GPU at once (0: 16) */
    int chunk_steps;             /* largest chunk of steps (0: 256; at most 4096); each request's
                                    chunks hold about 20 ms of estimated GPU time, up to this */
    int order;                   /* am_order: admission order of pending requests */
    int max_active_fp64;         /* FP64 and double-float requests on the GPU at once (0:
                                    max_active / 4, rounded up); a request waiting for this
                                    lane does not hold back the FP32 requests behind it */
    int reserved[4];             /* must be zero */
} am_server_config;

typedef struct am_job {
    am_params params;
    long long nsteps;
    const void *w_hat;           /* initial state [Ny][Nx/2+1] in the params' precision (copied at
                                    submit), or NULL: the seeded band-limited field below */
    double mean[2];              /* initial scaled mean velocity */
    unsigned long long seed;     /* am_ic_bandlimited arguments when w_hat is NULL */
    double kmin, kmax, rms;
    int want_state;              /* keep the final w_hat for am_server_wait */
    int want_energy;             /* keep the energy series for am_server_wait */
    int reserved[4];             /* must be zero */
} am_job;

typedef struct am_job_result {
    long long id;
    int status;                  /* am_status of the request */
    double t_submit, t_admit, t_done;   /* seconds since am_server_create */
    double mean[2];              /* final scaled mean velocity */
    long long steps_done;
    char error[256];
} am_job_result;

typedef struct am_server_info {
    double elapsed_s;
    long long jobs_submitted, jobs_done, jobs_pending;
    int jobs_active, peak_active;
    long long grid_point_steps;  /* completed requests' Nx*Ny*nsteps */
    long long device_bytes_reserved, peak_device_bytes;
} am_server_info;

am_status am_server_create(const am_server_config *cfg /* NULL: defaults */, am_server **out);
/* Queue a request; *id receives its id.  AM_ERR_OOM if its footprint alone
 * exceeds the budget, AM_ERR_UNSUPPORTED for a grid the solver does not take. */
am_status am_server_submit(am_server *s, const am_job *job, long long *id);
/* Wait up to timeout_s seconds (< 0: no limit) for request `id` and collect
 * its result (once): res, the final state (w_hat, if want_state) and the
 * energies (energy, nsteps values, if want_energy).  Returns the request's
 * status, or AM_ERR_TIMEOUT. */
am_status am_server_wait(am_server *s, long long id, double timeout_s, am_job_result *res, void *w_hat,
                         double *energy);
am_status am_server_stats(am_server *s, am_server_info *out);
/* Run every queued request to completion, then stop the server. */
am_status am_server_destroy(am_server *s);

/* Device bytes a handle with these parameters holds (what admission reserves). */
long long am_footprint_bytes(const am_params *p);

/* ------------------------------------------------------ launch shapes --
 * The column pass has three launch shapes: 0 "wide" (a whole tile of
 * adjacent kx columns per group of threads, whole-sector stores, 512-thread
 * CTAs, radix 16 in FP32), 1 "narrow" (one column per group, 128-thread CTAs,
 * up to four per SM) and 2 "wide8" (FP32 only: wide tiles with radix-8
 * passes, twice the threads per column, up to 1024-thread CTAs).  Which is
 * fastest depends on Ny and the precision; the process keeps one choice per
 * (precision, Ny), seeded with the rule measured on GB300 (narrow below
 * Ny = 2048, wide above), used by every handle, batch and ragged batch
 * created afterwards.  am_set_column_shape returns AM_ERR_UNSUPPORTED for a
 * shape not built for the precision.  The reference has no counterpart
 * (cuFFT picks its own plans, ActFlow_V3-2.cu:507-508). */
am_status am_set_column_shape(int precision, int ny, int shape);
int am_column_shape(int precision, int ny);   /* -1 for an unsupported size */
/* The row pass has three launch shapes: 0 "lockstep" (radix-8 passes, 128
 * threads per 2048-point row, the three inverse transforms in lockstep), 1
 * "sequence" (FP32 and double-float, Nx >= 1024: the transforms one after
 * another with two shared-memory stashes; FP32 with radix-16 passes, one
 * exchange fewer per transform and half the threads per row; double-float
 * with radix-8 passes and the transforms in a loop, a kernel small enough for
 * the instruction caches) and 2 "lockstep-tma" (FP32, Nx >= 128: shape 0
 * with each row's three input rows fetched into shared memory by tensor-map
 * copies, where the carried tiles of a row fit one exchange buffer --
 * otherwise it runs as shape 0; ensembles use this fetch in their shape-0
 * row pass).  One choice per (precision, Nx), seeded with shape 0 (FP32 from
 * Nx = 1024: shape 2; double-float from Nx = 1024: shape 1), used by every handle, batch and
 * ragged batch created afterwards; AM_ERR_UNSUPPORTED for a shape not built
 * for the precision and Nx.  No counterpart in the reference. */
am_status am_set_row_shape(int precision, int nx, int shape);
int am_row_shape(int precision, int nx);      /* -1 for an unsupported size */
/* Autotune: on the current device (a temporary handle with a seeded
 * band-limited state), time nsteps steps of a simulation with parameters p
 * under each column-pass shape built for its precision, keep the fastest for
 * p's precision and Ny, then time each row-pass shape with that column shape
 * and keep the fastest for p's precision and Nx.  The times go to ms_col[3]
 * and ms_row[3] (either may be NULL; -1 for a shape not built). */
am_status am_autotune(const am_params *p, int nsteps, double ms_col[3], double ms_row[3]);

/* Number of kernel launches one step makes (for accounting). */
int am_launches_per_step(const am_handle *h);

/* Highest kx index the stage fields carry: Nx/2 for the full transforms,
 * Nx/4 when the 1/2 rule lets the solver prune the transforms (the state
 * loaded last is zero outside the rule's ellipse).  -1 for a NULL handle. */
int am_kx_carried(const am_handle *h);

/* Device bytes held by the handle. */
long long am_device_bytes(const am_handle *h);

/* Human-readable text for a status, and the last error detail of a handle. */
const char *am_status_string(am_status s);
const char *am_last_error(const am_handle *h);

/* The reference's dealias mask value at half-plane index (ix, iy) (host-only,
 * no GPU needed).  Mirrors cutoff_func (ActFlow_V3-2.cu:899-919). */
int am_mask_value(int nx, int ny, int dealias, int ix, int iy);

/* Seeded band-limited initial field (host-only, no GPU needed): modes with
 * integer index kmin <= |(ix, iy)| <= kmax, Gaussian amplitudes and uniform
 * phases from a 64-bit Mersenne Twister seeded with `seed`, Hermitian, zero
 * mean, real-space rms `rms`.  Writes [Ny][Nx/2+1] complex doubles.  The
 * reference's own random field (ActFlow_V3-2.cu:535-559) is seeded from the
 * clock and cannot be reproduced; this generator replaces it for benchmarks. */
am_status am_ic_bandlimited(int nx, int ny, unsigned long long seed, double kmin, double kmax, double rms,
                            double *w_hat);

/* ------------------------------------------------ host-only file boundary --
 * These entry points need no GPU.  They are the reference program's file
 * contract, shared by the `actflow` front end and the tests. */

typedef struct am_spec {
    double T, dt, lx, ly;    /* parsed into float, widened to double */
    int nx, ny;
    double lambda, alpha, beta, dt_snap;
    double gamma0, gamma2;   /* extension keys Gamma0: / Gamma2: */
    int has_gamma;
    int precision;           /* extension key precision: fp32 | fp64 | df64 */
    int dealias;             /* extension key dealias: reference | half | none */
    char initial[256];
    char directory[1024];
} am_spec;

/* Read <dir>/specifications.txt (ActFlow_V3-2.cu:320-408): reference defaults
 * (ActFlow_V3-2.cu:183-204), reference keys and value parsing.  AM_ERR_IO if the
 * file is missing, AM_ERR_SPEC for an unknown key (ActFlow_V3-2.cu:392-400) or
 * an unreadable value; `err` receives the message. */
am_status am_spec_read(const char *dir, am_spec *out, char *err, int errlen);

/* Write a snapshot file in the reference's text layout (save_func,
 * ActFlow_V3-2.cu:1245-1266): Ny*(Nx/2+1) pairs "re,im," then "mx,my", each in
 * the default ostream form (%g).  w_hat is float for AM_FP32, double for AM_FP64
 * and AM_DF64. */
am_status am_write_snapshot(const char *path, int nx, int ny, int precision, const void *w_hat,
                            const double mean[2]);

/* Parse a snapshot file (the continue reader, ActFlow_V3-2.cu:614-634). */
am_status am_read_snapshot(const char *path, int nx, int ny, int precision, void *w_hat, double mean[2]);

/* Append `count` energy lines "t E" for steps m0, m0+1, ... (save_energy_func,
 * ActFlow_V3-2.cu:1268-1278); t = (float)m * dt evaluated in float. */
am_status am_append_energy(const char *path, long long m0, int count, float dt, const double *energy, int precision);

/* The whole drop-in program: `actflow <dir>` / help / spec / math
 * (main, ActFlow_V3-2.cu:214-878).  Returns the process exit code. */
int am_cli_main(int argc, char **argv);

#ifdef __cplusplus
}
#endif
#endif
