/*
 * xpfc.h -- C ABI of the GB300-native XPFC step (libxpfc.so).
 *
 * Drop-in boundary for the time loop of LC2500/XPFC_CUDA (main.cu:306-435).
 * Each entry point names the reference interface it replaces.  Plain C types
 * only: pointers, sizes, ints and doubles.  Every call returns an xpfc_status
 * and never exits the process (the reference exits inside
 * check_cufft_result, helpers_header.cuh:84-85, and read_input.cu:73,213).
 *
 * Field layout.  Host fields are double arrays in the reference's own order:
 * row-major [Mx][My][Mz], last index fastest (2-D: psi[i*My + j],
 * globals.cuh:91, initialize.cu:105).  Mz = 1 selects 2-D.
 *
 * Spectral buffers of the staged API hold the "packed real" spectrum: the
 * fastest axis (length n0 = My in 2-D, Mz in 3-D) keeps n0/2 complex bins,
 * bin 0 carrying X[0] + i X[n0/2]; the other axes are full complex transforms.
 * A packed spectrum occupies exactly the bytes of the real field, so every
 * transform is in place.  xpfc_download_spectrum unpacks to the conventional
 * half spectrum [..][n0/2+1] for callers that need it.
 */
#ifndef XPFC_H
#define XPFC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    XPFC_OK = 0,
    XPFC_EINVAL = 1,      /* bad argument or unsupported size                 */
    XPFC_ENOMEM = 2,      /* device or host allocation failed                 */
    XPFC_ECUDA = 3,       /* CUDA runtime error (message in xpfc_last_error)  */
    XPFC_ENONFINITE = 4,  /* free energy or mean became NaN/Inf               */
    XPFC_ETIMEDOUT = 5,   /* bounded device wait ran out                      */
    XPFC_EIO = 6,         /* file missing, truncated or malformed             */
    XPFC_ESTATE = 7       /* call out of order (e.g. step before initialize)  */
} xpfc_status;

typedef enum { XPFC_FP64 = 0, XPFC_MIXED = 1 } xpfc_precision;
typedef enum { XPFC_ENVELOPE_SUM = 0, XPFC_ENVELOPE_MAX = 1 } xpfc_envelope;
typedef enum { XPFC_FORWARD = -1, XPFC_INVERSE = 1 } xpfc_direction;

/* Initial-condition generators used by xpfc_initialize(ctx, NULL). */
typedef enum {
    XPFC_IC_REFERENCE = 0,   /* iconfig 0/1/2 lattices and seeds, initialize.cu:95-197 */
    XPFC_IC_NOISE = 1,       /* psi0 + ic_amp * N(0,1), Philox4x32-10 stream 0        */
    XPFC_IC_FCC_SEED = 2     /* noise liquid + sphere of 4 fcc (111) cosine modes      */
} xpfc_ic_kind;

#define XPFC_MAX_PEAKS 8

/* All model, grid and run parameters (the reference's globals,
   globals.cuh:40-52, read by read_input.cu:8-121). */
typedef struct xpfc_params {
    int Mx, My, Mz;                 /* grid points; Mz = 1 for 2-D                 */
    double Lx, Ly, Lz;              /* box lengths: k = 2 pi i / L (FFT_freq.cu)   */
    double psi0;                    /* mean density, pinned (Avg_calc.cu:21-43)   */
    double sigma;                   /* 's': Debye-Waller temperature             */
    double a, b;                    /* a = 1/a_in, b = 1/b_in (read_input.cu:28)  */
    double eps, Mo, dt;
    long long nsteps;               /* loop count, ceil(t/dt + 1) (initialize.cu:60) */
    int t_sample;                   /* diagnostics period (main.cu:326,412)        */
    int npeaks;                     /* correlation peaks (initialize.cu:10-17)    */
    double pk_k[XPFC_MAX_PEAKS], pk_alpha[XPFC_MAX_PEAKS];
    double pk_rho[XPFC_MAX_PEAKS], pk_beta[XPFC_MAX_PEAKS];
    int envelope;                   /* xpfc_envelope                              */
    int precision;                  /* xpfc_precision                             */
    int ref_compat;                 /* float powf powers, (int)Mo in the residual  */
    double ff_factor;               /* F = ff_factor * sum of density             */
    double noise_amp;               /* conserved noise per step (0 = off)         */
    unsigned long long noise_seed;
    /* initial condition */
    int ic_kind;                    /* xpfc_ic_kind                               */
    int iconfig;                    /* 0 tri, 1 square, 2 liquid, 10 VTK restart  */
    double A_10, A_11, A_tri;
    int iseed, ishape;
    double h, k, roa;
    double ic_amp;
    unsigned long long ic_seed;
    double ic_seed_amp, ic_seed_radius;
    char vtk_path[512];             /* iconfig 10 restart file                    */
    /* execution */
    int device;
    void *stream;                   /* cudaStream_t; NULL: the context's own     */
} xpfc_params;

/* Diagnostics record at one loop iteration (the values the reference prints
   with device printf at sum_reduction.cu:64 and :77). */
typedef struct xpfc_diag {
    long long iteration;
    double F;       /* free energy, valid when has & 1                  */
    double mean;    /* mean density (FP64 sum), valid when has & 1      */
    double rms;     /* residual RMS, valid when has & 2                 */
    int has;
} xpfc_diag;

typedef struct xpfc_ctx xpfc_ctx;

/* Buffers of the staged API: the reference's cudaLibXtDesc set
   (main.cu:135-141) plus its real arrays (main.cu:127). */
typedef enum {
    XPFC_BUF_PSI = 0,      /* d_psiC2C      */
    XPFC_BUF_PSI_K,        /* d_psiC2C_out  */
    XPFC_BUF_PSI_NP1,      /* d_psiC2C_np1  */
    XPFC_BUF_PSI_NP1_R,    /* d_psiC2C_np1_out */
    XPFC_BUF_PSI2,         /* d_psi2C2C     */
    XPFC_BUF_PSI3,         /* d_psi3C2C     */
    XPFC_BUF_PSI4,         /* d_psi4C2C     */
    XPFC_BUF_CONVL,        /* d_convl       */
    XPFC_BUF_RES,          /* res_k         */
    XPFC_NBUF
} xpfc_buffer;

/* ---- parameters and input deck ---------------------------------------- */
/* Defaults of the 64^3 single-peak case (kernel parameters k1=2pi, alpha=1,
   rho=1, beta=8, sigma=0.1; eta=2, chi=1; n0=0.05; dt=1). */
int xpfc_default_params(xpfc_params *p);
/* read_input.cu:8-121: positional pfc.input lines 1-18, plus optional
   "key = value" lines after line 18 (the reference stops reading there).
   Applies initialize.cu:23-33 (lattice scaling of Lx, Ly), :60 (steps) and
   :63 (ff_factor) and the reference's hard-coded two-peak sum DCF
   (initialize.cu:10-17, 215-217) unless the extension lines override it. */
int xpfc_read_input(const char *path, xpfc_params *p);

/* ---- lifecycle (replaces main.cu:106-228) ------------------------------ */
int xpfc_create(const xpfc_params *p, xpfc_ctx **out);
int xpfc_destroy(xpfc_ctx *ctx);
/* Last error message of ctx (or of the calling thread when ctx is NULL). */
const char *xpfc_last_error(const xpfc_ctx *ctx);
int xpfc_get_params(const xpfc_ctx *ctx, xpfc_params *p);
/* Host pointer to the stream the context launches on (cudaStream_t). */
void *xpfc_get_stream(const xpfc_ctx *ctx);

/* initialize.cu:6-238 + main.cu:226: builds (host_psi == NULL: the noise
   liquid and fcc seed on the device, the reference's lattices, seeds and VTK
   restart on the host) or takes the initial field, pins its mean to psi0
   (Avg_calc.cu:21-43; for XPFC_IC_REFERENCE params with the reference's own
   summation order, one running sum in index order), uploads it and prepares
   both the staged buffers (XPFC_BUF_PSI) and the fused state. */
int xpfc_initialize(xpfc_ctx *ctx, const double *host_psi);
/* The initial field of p on the host (every generator, mean pinned). */
int xpfc_build_initial_field(const xpfc_params *p, double *host_psi);
/* The same on the device: dev_psi holds Mx*My*Mz doubles; stream is a
   cudaStream_t (NULL: the legacy default stream); returns when the field is
   ready.  Every generator but the VTK restart (iconfig 10, a host file).
   No reference counterpart (the reference builds fields on the host,
   initialize.cu:95-197); agrees with xpfc_build_initial_field to rounding
   (device and host libm differ in the last bits). */
int xpfc_build_initial_field_device(const xpfc_params *p, double *dev_psi, void *stream);

/* ---- fused step: the hot path ------------------------------------------ */
/* Advances nsteps iterations of main.cu:306-435 with the fused passes.
   Diagnostics follow the reference's schedule: F and mean at the starting
   iteration 0, at every iteration divisible by t_sample and at the last
   iteration; RMS at iterations divisible by t_sample (computed from the step
   that leaves them).  Up to cap records are written to out; *count gets the
   number produced (NULL out/count allowed). */
int xpfc_step(xpfc_ctx *ctx, long long nsteps, xpfc_diag *out, int cap, int *count);
/* Enqueues nsteps fused iterations on the context stream and returns
   without waiting.  Periodic diagnostics (iterations divisible by t_sample)
   are computed on the device; the final-iteration free energy is not.
   xpfc_collect waits for the work and returns those records; they are kept
   until the next xpfc_step / xpfc_step_async call. */
int xpfc_step_async(xpfc_ctx *ctx, long long nsteps);
int xpfc_collect(xpfc_ctx *ctx, xpfc_diag *out, int cap, int *count);
/* Per-pass GPU time with CUDA events around every launch of the fused step
   (off by default).  Pass ids: 0 pencil (k-space update), 1 inverse column
   pass, 2 row pass, 3 forward column pass, 4 reductions.  xpfc_get_profile
   waits for the stream and returns the accumulated milliseconds and launch
   count of one pass since profiling was (re)enabled. */
int xpfc_set_profiling(xpfc_ctx *ctx, int enable);
int xpfc_get_profile(xpfc_ctx *ctx, int pass, double *ms, long long *launches);
/* Current iteration counter of the fused state. */
long long xpfc_iteration(const xpfc_ctx *ctx);
/* copy_to_cpu.cu:3-18: current real field of the fused state. */
int xpfc_get_field(xpfc_ctx *ctx, double *host_psi);
/* Current field of the fused state, as FP32 values on the device: the
   caller's device buffer of Mx*My*Mz floats (no host copy). */
int xpfc_get_field_device_f32(xpfc_ctx *ctx, float *dev_out);
/* copy_to_cpu.cu:3-18 without stopping the time loop (the reference copies
   synchronously after the loop, main.cu:453): _async enqueues the transform of
   the current field (the iteration after every step already enqueued) to real
   space on the context stream and its device-to-host copy on a copy stream of
   the context, and returns; steps enqueued after it run while the copy
   proceeds.  _wait blocks until that copy is done and writes the field to
   host_psi ([Mx][My][Mz] doubles) and its iteration to *iteration (may be
   NULL).  One read-back at a time: a second _async drops an uncollected one. */
int xpfc_get_field_async(xpfc_ctx *ctx);
int xpfc_get_field_wait(xpfc_ctx *ctx, double *host_psi, long long *iteration);
/* Checkpoint and resume of the fused state at full precision (the reference
   restarts only from a 6-digit VTK field, read_input.cu:124-241, and lists
   periodic checkpoints as to do, VERSIONLOG:8-10).  _save writes the spectral
   state (both fused arrays, the iteration and the grid) to path; _load reads it
   into a context of the same grid, precision and instance count, which then
   continues bit for bit as the saved solve would have.  Both wait for the
   context's stream. */
int xpfc_save_state(xpfc_ctx *ctx, const char *path);
int xpfc_load_state(xpfc_ctx *ctx, const char *path);

/* ---- staged API: the reference's per-stage wrappers ---------------------
   FP64, reference semantics, buffers named by xpfc_buffer.                 */
int xpfc_upload(xpfc_ctx *ctx, int buf, const double *host);    /* H2D (main.cu:226)       */
int xpfc_download(xpfc_ctx *ctx, int buf, double *host);        /* copy2cpu, copy_to_cpu.cu */
int xpfc_download_spectrum(xpfc_ctx *ctx, int buf, double *host_half); /* unpacked [..][n0/2+1] complex */
int xpfc_copy(xpfc_ctx *ctx, int src, int dst);                 /* cufftXtMemcpy D2D       */
int xpfc_fft(xpfc_ctx *ctx, int buf, int direction);            /* cufftXtExecDescriptor   */
int xpfc_power_functions(xpfc_ctx *ctx, int in, int out, int p);/* power_functions.cu:4-32 */
int xpfc_scaling_step(xpfc_ctx *ctx, int buf);                  /* scaling_step.cu:4-30    */
int xpfc_copy_matrix(xpfc_ctx *ctx, int in, int out);           /* copy_matrix.cu:4-31     */
int xpfc_convolve_fields(xpfc_ctx *ctx, int psi_k, int out);    /* convolve_fields.cu:3-27 */
int xpfc_euler_step(xpfc_ctx *ctx, int n, int psi_kp1, int psi_k, int psi2_k, int psi3_k); /* euler_step.cu:3-29 */
int xpfc_FE_calc(xpfc_ctx *ctx, int n, int psi, int psi2, int psi3, int psi4, int convl_r,
                 double *F);                                    /* FE_calc.cu:3-51         */
int xpfc_sse_calculation(xpfc_ctx *ctx, int n, int psi_kp1, int psi_k, int psi2_k, int psi3_k,
                         double *rms);                          /* sse_calculation.cu:3-116 */
int xpfc_Avg_calc(xpfc_ctx *ctx, int buf, double *mean);        /* Avg_calc.cu:3-18        */

/* ---- files ---------------------------------------------------------------- */
/* write_vtk.cu:4-35: legacy ASCII STRUCTURED_POINTS, x fastest; precision =
   significant digits (6 reproduces the reference's ostream default). */
int xpfc_write_vtk(const char *path, const double *host_psi, int Mx, int My, int Mz,
                   double Lx, double Ly, double Lz, int precision);
/* read_input.cu:124-241: reads DIMENSIONS/SPACING and the values (file order,
   x fastest) into host_psi in the [Mx][My][Mz] layout.  dims/L may be NULL. */
int xpfc_read_vtk(const char *path, double *host_psi, size_t cap, int dims[3], double L[3]);

/* ---- batched sweeps ---------------------------------------------------------- */
/* No counterpart in the reference, which runs one solve per process (main.cu).
   A batch advances n independent solves together.  Instances whose params
   agree on everything but psi0, sigma, the peaks (npeaks, pk_*, envelope),
   noise_seed and the initial-condition fields form one group; a group's fields
   sit back to back in HBM and every pass of a step is one launch over all of
   them (grid z = instance), so small grids fill the GPU.  Groups run
   concurrently on their own streams (ps[0].stream, when set, serialises them).
   Each instance gets the same results it would get alone in an xpfc_ctx with
   the same params.  Instances need equal box lengths on every axis
   (Lx = Ly (= Lz)): their coefficients come from per-instance shell tables. */
typedef struct xpfc_batch xpfc_batch;
int xpfc_batch_create(const xpfc_params *ps, int n, xpfc_batch **out);
int xpfc_batch_destroy(xpfc_batch *b);
const char *xpfc_batch_last_error(const xpfc_batch *b);
int xpfc_batch_size(const xpfc_batch *b);                 /* n                      */
int xpfc_batch_groups(const xpfc_batch *b);               /* groups formed          */
int xpfc_batch_group_of(const xpfc_batch *b, int i);      /* group of instance i    */
/* fields[i] (host, [Mx][My][Mz]) or NULL entries / a NULL array: the
   instance's own generator, as xpfc_initialize(ctx, NULL).  Mean pinned to
   each instance's psi0. */
int xpfc_batch_initialize(xpfc_batch *b, const double *const *fields);
/* nsteps more iterations of every instance, with the diagnostics schedule of
   xpfc_step; returns when all groups are done.  _async only enqueues. */
int xpfc_batch_step(xpfc_batch *b, long long nsteps);
int xpfc_batch_step_async(xpfc_batch *b, long long nsteps);
/* Waits for instance i's group; its diagnostics of the last step call
   (XPFC_ENONFINITE when its F or mean is not finite). */
int xpfc_batch_collect(xpfc_batch *b, int i, xpfc_diag *out, int cap, int *count);
int xpfc_batch_get_field(xpfc_batch *b, int i, double *host_psi);

/* ---- serving ------------------------------------------------------------------ */
/* No counterpart in the reference, which runs one solve per process.  A server
   runs solve requests on one GPU from a scheduler thread of its own: queued
   requests are admitted in arrival order while their device memory fits
   hbm_budget_bytes and fewer than max_running contexts are in flight; each
   running solve has a context with its own stream (reused across requests of
   the same grid and precision) and its iterations are enqueued chunk_steps at
   a time, round robin, so solves join and leave the running set at chunk
   boundaries while the GPU interleaves them.  With merge_max > 1, queued
   requests of the same grid that agree on everything but psi0, sigma, the
   peaks, the seeds and the initial field (the xpfc_batch grouping rule,
   equal box lengths), and whose step counts lie within 25 % of each other,
   are admitted together, up to merge_max at a time, as one merged group: a
   batched context whose every pass covers all of them in one launch (grid z =
   solve), counted once against max_running.  The group runs to its longest solve; a shorter solve's field is
   read back at its own last iteration and its results are handed over when
   the group finishes.  A request's diagnostics and field are those xpfc_step
   gives for the same params alone, merged or not.  Initial fields come from
   the params' generator on the device, or from the caller. */
typedef struct xpfc_server xpfc_server;
typedef struct {
    size_t hbm_budget_bytes;  /* device memory for solves (0: 80% of free memory) */
    int max_running;          /* contexts in flight, a merged group once (0: 16) */
    int chunk_steps;          /* iterations per solve per round (0: 16)          */
    int device;
    int merge_max;            /* solves per merged group (0 or 1: no merging)    */
} xpfc_server_config;
typedef enum { XPFC_REQ_QUEUED = 0, XPFC_REQ_RUNNING = 1, XPFC_REQ_DONE = 2, XPFC_REQ_FAILED = 3 } xpfc_req_state;
typedef struct {
    long long id;
    int state;                          /* xpfc_req_state                      */
    int status;                         /* xpfc_status of a finished request   */
    double t_submit, t_admit, t_done;   /* seconds since the server started    */
    size_t device_bytes;                /* device memory held while it runs    */
} xpfc_request_info;
typedef struct {
    long long submitted, queued, running, done, failed;
    long long contexts_created, contexts_reused;
    size_t bytes_in_use, peak_bytes_in_use, budget;
    long long merged_groups, merged_solves;   /* groups formed, solves they held */
} xpfc_server_stats;
int xpfc_server_create(const xpfc_server_config *cfg, xpfc_server **out);
/* Running solves finish; queued ones fail (XPFC_ESTATE). */
int xpfc_server_destroy(xpfc_server *s);
const char *xpfc_server_last_error(const xpfc_server *s);
/* host_psi: NULL (the params' generator) or a field the call copies;
   keep_field = 1 keeps the final field for xpfc_server_result. */
int xpfc_server_submit(xpfc_server *s, const xpfc_params *p, const double *host_psi, long long nsteps,
                       int keep_field, long long *id);
/* Blocks until the request finished (timeout_s < 0: no limit; XPFC_ETIMEDOUT). */
int xpfc_server_wait(xpfc_server *s, long long id, double timeout_s);
int xpfc_server_info(xpfc_server *s, long long id, xpfc_request_info *info);
/* Final field (when kept; host_psi may be NULL) and diagnostics of a
   finished request; a failed request returns its status. */
int xpfc_server_result(xpfc_server *s, long long id, double *host_psi, xpfc_diag *out, int cap, int *count);
/* Forgets a finished request. */
int xpfc_server_release(xpfc_server *s, long long id);
int xpfc_server_stats_get(xpfc_server *s, xpfc_server_stats *st);

/* ---- allocation-free reduction ---------------------------------------------- */
/* No counterpart in the reference.  The free energy of xpfc_FE_calc
   (ff_factor times the sum of the FE_calc density) from five caller-owned
   device arrays of n doubles, for callers that cannot allocate device memory
   (a host framework that owns all device memory through its own pool and
   forbids plugins to allocate, or a loop run under a fixed device-memory
   budget).  Allocates nothing: its partial sums live in a fixed 32 KB array
   in the library's device memory, which every GPU that loads the library
   keeps until exit.  n is at most XPFC_NOALLOC_MAX_POINTS (2^28; larger n
   returns XPFC_EINVAL).  stream is a cudaStream_t (NULL: the legacy default
   stream); the call waits for its own work on that stream and writes *F on
   the host.  The first call on each device looks up the array's device
   address (cudaGetSymbolAddress) and must come before any stream capture;
   the address is kept for the process, so cudaDeviceReset after that first
   call is not supported.  All calls share the array: calls that overlap on
   the GPU race, so serialise them. */
#define XPFC_NOALLOC_CHUNK 65536
#define XPFC_NOALLOC_MAX_CHUNKS 4096
#define XPFC_NOALLOC_MAX_POINTS ((long long)XPFC_NOALLOC_CHUNK * XPFC_NOALLOC_MAX_CHUNKS)
int xpfc_FE_calc_noalloc(const double *psi, const double *psi2, const double *psi3, const double *psi4,
                         const double *convl_r, long long n, double a, double b, double ff_factor,
                         double *F, void *stream);

/* ---- introspection ---------------------------------------------------------- */
/* Kernel launches issued by this context since creation (all entry points). */
long long xpfc_launch_count(const xpfc_ctx *ctx);
/* Algorithmic HBM bytes of one launch of a step pass (pass ids as in
   xpfc_get_profile: 0 pencil, 1 and 3 column passes, 2 row pass): the arrays
   the pass reads and writes once each, for the roofline of that pass.  No
   reference counterpart.  -1 for a bad pass id or context. */
long long xpfc_pass_bytes(const xpfc_ctx *ctx, int pass);
/* Library version string. */
const char *xpfc_version(void);

#ifdef __cplusplus
}
#endif
#endif /* XPFC_H */
