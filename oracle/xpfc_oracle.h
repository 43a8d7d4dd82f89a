/*
 * xpfc_oracle.h -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.
 *
 * CPU FP64 restatement of the semi-implicit spectral XPFC time step of
 * LC2500/XPFC_CUDA (2-D in the reference, dimension-generic here).  Only the
 * tests, __graft_entry__.smoke() and bench.py (cpu_baseline leg and the
 * "--impl reference" arm) may load it, and only as the checker / the timed
 * CPU implementation.  The product library never links it.
 *
 * Parity anchor: golden vectors made by tests/golden/make_golden.py from the
 * reference's own host code and kernel bodies compiled with g++ (recipe in
 * oracle/ref/Makefile).  cuFFT (closed) is replaced by the published DFT
 * definition, which the oracle's FFT implements and the tests check against
 * numpy.fft.
 *
 * Layout: real fields are C-order [nz][ny][nx], x fastest.  Complex spectra
 * are full (not half) arrays in the same order, like the reference's Z2Z
 * descriptors (main.cu:135-141).
 */
#ifndef XPFC_ORACLE_H
#define XPFC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OX_MAXPEAKS 8

typedef struct {
    int nx, ny, nz;            /* grid; nz = 1 for 2-D                          */
    double Lx, Ly, Lz;         /* box lengths (k = 2*pi*i/L, FFT_freq.cu:4-26)  */
    double a, b;               /* reference a = 1/a_in, b = 1/b_in (read_input.cu:26-28) */
    double eps, Mo, dt;
    double sigma;              /* reference 's'                                  */
    int npeaks;
    double pk_k[OX_MAXPEAKS], pk_alpha[OX_MAXPEAKS], pk_rho[OX_MAXPEAKS], pk_beta[OX_MAXPEAKS];
    int envelope;              /* 0 = sum of peaks (initialize.cu:215-217), 1 = max (:210) */
    int ref_compat;            /* 1: powers through float powf (power_functions.cu:47),
                                  residual with (int)Mo (sse_calculation.cu:120)          */
    double ff_factor;          /* F = ff_factor * sum(f) (FE_calc + initialize.cu:63)    */
    double noise_amp;          /* conserved noise amplitude per step (0 = off)           */
    uint64_t noise_seed;
} ox_params;

/* Per-iteration diagnostics; NaN where not sampled. */
typedef struct {
    double F;      /* free energy of psi at this iteration                */
    double mean;   /* mean of psi at this iteration (FP64 sum / cells)     */
    double rms;    /* residual RMS computed at this iteration (n % ts == 0) */
} ox_diag;

/* FFT ------------------------------------------------------------------- */
/* Unnormalised complex FFT of a C-order [nz][ny][nx] array, in place.
   sign = -1: forward (exp(-i...)), +1: inverse.  data is interleaved re,im. */
void ox_fft3(double *data, int nx, int ny, int nz, int sign);

/* k-space tables -------------------------------------------------------- */
void ox_fft_freq(int n, double L, double *k);                   /* FFT_freq.cu:4-26 */
double ox_c2(const ox_params *p, double kmag);                  /* initialize.cu:209-217 */
void ox_k2_c2(const ox_params *p, double *k2, double *c2);      /* full grid tables */

/* Stages (reference per-stage wrappers), full complex / real arrays ------ */
void ox_power(const ox_params *p, const double *psi, double *out, int pw, long n);
void ox_euler_step(const ox_params *p, const double *k2, const double *c2,
                   const double *psi_k, const double *psi2_k, const double *psi3_k,
                   double *psi_kp1);
void ox_convolve_fields(const ox_params *p, const double *c2, const double *psi_k, double *convl);
double ox_FE_calc(const ox_params *p, const double *psi, const double *psi2, const double *psi3,
                  const double *psi4, const double *convl_r);
double ox_sse_calculation(const ox_params *p, const double *k2, const double *c2,
                          const double *psi_kp1, const double *psi_k,
                          const double *psi2_k, const double *psi3_k);
double ox_mean(const double *psi, long n);
void ox_pin_mean(double *psi, long n, double psi0);             /* Avg_calc.cu:21-43 */

/* Conserved noise added to the update numerator (new; no reference code). */
void ox_noise_k(const ox_params *p, long step, double *noise_k);

/* Whole run mirroring main.cu:232-450.  psi: initial real field (mean already
   pinned), overwritten with the final field.  diag: nsteps+1 entries.       */
int ox_run(const ox_params *p, double *psi, long nsteps, int t_sample, ox_diag *diag);
/* The same loop without diagnostics, wall-clock timed (CPU baseline). */
int ox_bench(const ox_params *p, double *psi, long nsteps, double *seconds);
int ox_threads(void);

/* Initial conditions ------------------------------------------------------ */
/* Philox4x32-10 (Salmon et al., SC'11) and Box-Muller Gaussians. */
void ox_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
void ox_gauss_pair(uint64_t seed, uint64_t stream, uint64_t index, double *g0, double *g1);
void ox_ic_noise(double *psi, int nx, int ny, int nz, double n0, double amp, uint64_t seed);
void ox_ic_fcc_seed(double *psi, int nx, int ny, int nz, double Lx, double Ly, double Lz,
                    double n0, double amp, double radius_pts);
/* Reference 2-D initial conditions (initialize.cu:95-197). Lx, Ly already
   scaled as the reference does; returns the seed radius r actually used. */
double ox_ic_reference(double *psi, int Mx, int My, int Lx, int Ly, double psi0, int iconfig,
                       double A_10, double A_11, double A_tri, int iseed, int ishape,
                       double h, double k, double roa);

#ifdef __cplusplus
}
#endif
#endif
