/*
 * xpfc_oracle.c -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.
 *
 * CPU FP64 restatement of LC2500/XPFC_CUDA's time step (see xpfc_oracle.h).
 * Every stage cites the reference file:line it restates.  The product library
 * never links this file; only tests, smoke() and bench.py's CPU legs load it.
 *
 * Build: oracle/build_oracle.py (gcc -O2 -fopenmp -ffp-contract=off).
 */
#include "xpfc_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ======================================================================= */
/* 1-D mixed-radix Stockham FFT (textbook autosort formulation).           */
/* ======================================================================= */

typedef struct {
    int n;
    int nrad;
    int rad[32];
    double *tw;      /* exp(-2*pi*i*k/n), k in [0,n), interleaved */
} fft_plan;

static int factorise(int n, int *rad) {
    int m = 0;
    while (n % 4 == 0) { rad[m++] = 4; n /= 4; }
    while (n % 2 == 0) { rad[m++] = 2; n /= 2; }
    for (int p = 3; p <= n; p += 2)
        while (n % p == 0) { rad[m++] = p; n /= p; }
    return m;
}

static void plan_init(fft_plan *pl, int n) {
    pl->n = n;
    pl->nrad = (n == 1) ? 0 : factorise(n, pl->rad);
    pl->tw = (double *)malloc(sizeof(double) * 2 * (size_t)n);
    for (int k = 0; k < n; k++) {
        /* angle reduced in integer arithmetic before the trig call */
        double ang = -2.0 * M_PI * (double)k / (double)n;
        pl->tw[2 * k] = cos(ang);
        pl->tw[2 * k + 1] = sin(ang);
    }
}

static void plan_free(fft_plan *pl) { free(pl->tw); }

/* small DFT of radix R in place on v (interleaved), sign -1 fwd / +1 inv */
static void small_dft(double *v, int R, int sign, const fft_plan *pl) {
    double t[2 * 64];
    if (R == 2) {
        double ar = v[0], ai = v[1], br = v[2], bi = v[3];
        v[0] = ar + br; v[1] = ai + bi; v[2] = ar - br; v[3] = ai - bi;
        return;
    }
    if (R == 4) {
        double x0r = v[0], x0i = v[1], x1r = v[2], x1i = v[3];
        double x2r = v[4], x2i = v[5], x3r = v[6], x3i = v[7];
        double ar = x0r + x2r, ai = x0i + x2i, br = x0r - x2r, bi = x0i - x2i;
        double cr = x1r + x3r, ci = x1i + x3i, dr = x1r - x3r, di = x1i - x3i;
        /* forward: X1 = b - i d, X3 = b + i d ; inverse swaps */
        double sdr = (double)sign * dr, sdi = (double)sign * di;
        v[0] = ar + cr; v[1] = ai + ci;
        v[4] = ar - cr; v[5] = ai - ci;
        v[2] = br - sdi; v[3] = bi + sdr;
        v[6] = br + sdi; v[7] = bi - sdr;
        return;
    }
    /* generic O(R^2) DFT using the plan's twiddle table (R divides n) */
    int stride = pl->n / R;
    for (int k = 0; k < R; k++) {
        double sr = 0.0, si = 0.0;
        for (int j = 0; j < R; j++) {
            int idx = (int)(((long)j * k) % R) * stride;
            /* forward uses tw (exp(-i)), inverse its conjugate */
            double wr = pl->tw[2 * idx];
            double wi = (sign < 0) ? pl->tw[2 * idx + 1] : -pl->tw[2 * idx + 1];
            sr += v[2 * j] * wr - v[2 * j + 1] * wi;
            si += v[2 * j] * wi + v[2 * j + 1] * wr;
        }
        t[2 * k] = sr; t[2 * k + 1] = si;
    }
    memcpy(v, t, sizeof(double) * 2 * (size_t)R);
}

/* x: n complex (interleaved), work: n complex scratch.  Result in x. */
static void fft1d(const fft_plan *pl, double *x, double *work, int sign) {
    const int n = pl->n;
    double *a = x, *b = work;
    int ns = 1;
    for (int p = 0; p < pl->nrad; p++) {
        const int R = pl->rad[p];
        const int nb = n / R;
        const int twstep = n / (ns * R);
        for (int j = 0; j < nb; j++) {
            double v[2 * 64];
            const int k = j % ns;
            for (int r = 0; r < R; r++) {
                double xr = a[2 * (j + r * nb)], xi = a[2 * (j + r * nb) + 1];
                int idx = k * r * twstep;           /* < n */
                double wr = pl->tw[2 * idx];
                double wi = (sign < 0) ? pl->tw[2 * idx + 1] : -pl->tw[2 * idx + 1];
                v[2 * r] = xr * wr - xi * wi;
                v[2 * r + 1] = xr * wi + xi * wr;
            }
            small_dft(v, R, sign, pl);
            const int d = (j / ns) * ns * R + k;
            for (int r = 0; r < R; r++) {
                b[2 * (d + r * ns)] = v[2 * r];
                b[2 * (d + r * ns) + 1] = v[2 * r + 1];
            }
        }
        double *t = a; a = b; b = t;
        ns *= R;
    }
    if (a != x) memcpy(x, a, sizeof(double) * 2 * (size_t)n);
}

/* Apply 1-D transforms along one axis of a [nz][ny][nx] complex array. */
static void fft_axis(double *data, int nx, int ny, int nz, int axis, int sign) {
    const int len = (axis == 0) ? nx : (axis == 1) ? ny : nz;
    if (len == 1) return;
    fft_plan pl;
    plan_init(&pl, len);
    const long stride = (axis == 0) ? 1 : (axis == 1) ? nx : (long)nx * ny;
    const long nlines = (long)nx * ny * nz / len;
#pragma omp parallel
    {
        double *line = (double *)malloc(sizeof(double) * 2 * (size_t)len);
        double *work = (double *)malloc(sizeof(double) * 2 * (size_t)len);
#pragma omp for schedule(static)
        for (long l = 0; l < nlines; l++) {
            long base;
            if (axis == 0) base = l * nx;
            else if (axis == 1) base = (l / nx) * (long)nx * ny + (l % nx);
            else base = l;
            for (int i = 0; i < len; i++) {
                line[2 * i] = data[2 * (base + i * stride)];
                line[2 * i + 1] = data[2 * (base + i * stride) + 1];
            }
            fft1d(&pl, line, work, sign);
            for (int i = 0; i < len; i++) {
                data[2 * (base + i * stride)] = line[2 * i];
                data[2 * (base + i * stride) + 1] = line[2 * i + 1];
            }
        }
        free(line);
        free(work);
    }
    plan_free(&pl);
}

void ox_fft3(double *data, int nx, int ny, int nz, int sign) {
    fft_axis(data, nx, ny, nz, 0, sign);
    fft_axis(data, nx, ny, nz, 1, sign);
    fft_axis(data, nx, ny, nz, 2, sign);
}

/* ======================================================================= */
/* k-space tables                                                          */
/* ======================================================================= */

/* FFT_freq.cu:4-26: k_i = (2 pi/L) i for i < N/2+1 (even N; Nyquist positive),
   (2 pi/L)(i-N) above; odd N splits at (N+1)/2.  (The reference also writes
   k[N] out of bounds, :21; that element is never used.) */
void ox_fft_freq(int n, double L, double *k) {
    const double f = 2.0 * M_PI / L;
    const int split = (n % 2 != 0) ? (n + 1) / 2 : (n + 2) / 2;
    for (int i = 0; i < n; i++) k[i] = (i < split) ? f * (double)i : f * (double)(i - n);
}

/* initialize.cu:209-217: c2(k) = sum_i exp(-(s k_i)^2/(2 rho_i B_i)) *
   exp(-(k-k_i)^2/(2 al_i^2)); the max envelope (commented out at :210) is
   selected by envelope = 1. */
double ox_c2(const ox_params *p, double kmag) {
    double acc = 0.0;
    for (int i = 0; i < p->npeaks; i++) {
        double sk = p->sigma * p->pk_k[i];
        double dw = exp(-(sk * sk) / (2.0 * p->pk_rho[i] * p->pk_beta[i]));
        double d = kmag - p->pk_k[i];
        double g = exp(-(d * d) / (2.0 * p->pk_alpha[i] * p->pk_alpha[i]));
        double v = dw * g;
        if (p->envelope == 0) acc += v;
        else acc = (i == 0 || v > acc) ? v : acc;
    }
    return acc;
}

/* initialize.cu:77-85 (k2 = kx^2+ky^2, k_arr = sqrt(k2)) and :221-229 (c2). */
void ox_k2_c2(const ox_params *p, double *k2, double *c2) {
    double *kx = (double *)malloc(sizeof(double) * (size_t)p->nx);
    double *ky = (double *)malloc(sizeof(double) * (size_t)p->ny);
    double *kz = (double *)malloc(sizeof(double) * (size_t)p->nz);
    ox_fft_freq(p->nx, p->Lx, kx);
    ox_fft_freq(p->ny, p->Ly, ky);
    ox_fft_freq(p->nz, p->Lz, kz);
    if (p->nz == 1) kz[0] = 0.0;
#pragma omp parallel for schedule(static)
    for (int iz = 0; iz < p->nz; iz++)
        for (int iy = 0; iy < p->ny; iy++)
            for (int ix = 0; ix < p->nx; ix++) {
                long i = ((long)iz * p->ny + iy) * p->nx + ix;
                double v = kx[ix] * kx[ix] + ky[iy] * ky[iy] + kz[iz] * kz[iz];
                k2[i] = v;
                if (c2) c2[i] = ox_c2(p, sqrt(v));
            }
    free(kx); free(ky); free(kz);
}

/* ======================================================================= */
/* Stages                                                                  */
/* ======================================================================= */

/* power_functions.cu:34-53: psiN = powf(psi, p) -- a FLOAT power in the
   reference (ref_compat); exact double products otherwise. */
void ox_power(const ox_params *p, const double *psi, double *out, int pw, long n) {
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; i++) {
        double x = psi[i];
        double v;
        if (p->ref_compat) v = (double)powf((float)x, (float)pw);
        else if (pw == 2) v = x * x;
        else if (pw == 3) v = x * x * x;
        else if (pw == 4) { double s = x * x; v = s * s; }
        else v = pow(x, (double)pw);
        out[i] = v;
    }
}

/* euler_step.cu:50-59 (plus the conserved-noise term, 0 in the reference). */
void ox_euler_step(const ox_params *p, const double *k2, const double *c2,
                   const double *psi_k, const double *psi2_k, const double *psi3_k,
                   double *psi_kp1) {
    const long n = (long)p->nx * p->ny * p->nz;
    const double a = p->a, b = p->b, Mo = p->Mo, dt = p->dt, eps = p->eps;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; i++) {
        double re = psi_k[2 * i] + a * k2[i] * Mo * dt * psi2_k[2 * i] - b * k2[i] * dt * Mo * psi3_k[2 * i];
        double im = psi_k[2 * i + 1] + a * k2[i] * Mo * dt * psi2_k[2 * i + 1] - b * k2[i] * dt * Mo * psi3_k[2 * i + 1];
        double den = (1.0 + k2[i] * dt * Mo * (1.0 - eps) - k2[i] * Mo * dt * c2[i]);
        psi_kp1[2 * i] = re / den;
        psi_kp1[2 * i + 1] = im / den;
    }
}

/* convolve_fields.cu:30-51: convl = c2 * psi_k */
void ox_convolve_fields(const ox_params *p, const double *c2, const double *psi_k, double *convl) {
    const long n = (long)p->nx * p->ny * p->nz;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; i++) {
        convl[2 * i] = c2[i] * psi_k[2 * i];
        convl[2 * i + 1] = c2[i] * psi_k[2 * i + 1];
    }
}

/* Fixed-order FP64 sum: per-chunk partials in index order, then summed in
   chunk order (independent of the thread count). */
static double det_sum(const double *v, long n) {
    const long chunk = 65536;
    const long nch = (n + chunk - 1) / chunk;
    double *part = (double *)malloc(sizeof(double) * (size_t)(nch > 0 ? nch : 1));
#pragma omp parallel for schedule(static)
    for (long c = 0; c < nch; c++) {
        double s = 0.0;
        long e = (c + 1) * chunk < n ? (c + 1) * chunk : n;
        for (long i = c * chunk; i < e; i++) s += v[i];
        part[c] = s;
    }
    double s = 0.0;
    for (long c = 0; c < nch; c++) s += part[c];
    free(part);
    return s;
}

/* FE_calc.cu:54-68 (density), reduced and scaled by ff_factor as
   sum_reduction.cu:56-66 prints it. */
double ox_FE_calc(const ox_params *p, const double *psi, const double *psi2, const double *psi3,
                  const double *psi4, const double *convl_r) {
    const long n = (long)p->nx * p->ny * p->nz;
    const double a = p->a, b = p->b;
    double *ff = (double *)malloc(sizeof(double) * (size_t)n);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; i++)
        ff[i] = 0.5 * psi2[i] - (a / 3.0) * psi3[i] + (b / 4.0) * psi4[i] - 0.5 * psi[i] * convl_r[2 * i];
    double s = det_sum(ff, n);
    free(ff);
    return s * p->ff_factor;
}

/* sse_calculation.cu:120-147 (residual), :33-38 (inverse FFT, scale, square),
   sum_reduction.cu:69-80 (sqrt(sum/M2)). */
double ox_sse_calculation(const ox_params *p, const double *k2, const double *c2,
                          const double *psi_kp1, const double *psi_k,
                          const double *psi2_k, const double *psi3_k) {
    const long n = (long)p->nx * p->ny * p->nz;
    const double a = p->a, b = p->b, dt = p->dt;
    const double Mo = p->ref_compat ? (double)(int)p->Mo : p->Mo;
    double *res = (double *)malloc(sizeof(double) * 2 * (size_t)n);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; i++) {
        double d2r = -Mo * k2[i] * (psi_k[2 * i] - a * psi2_k[2 * i] + b * psi3_k[2 * i] - c2[i] * psi_k[2 * i]);
        double dtr = (psi_kp1[2 * i] - psi_k[2 * i]) / dt;
        double d2i = -Mo * k2[i] * (psi_k[2 * i + 1] - a * psi2_k[2 * i + 1] + b * psi3_k[2 * i + 1] - c2[i] * psi_k[2 * i + 1]);
        double dti = (psi_kp1[2 * i + 1] - psi_k[2 * i + 1]) / dt;
        res[2 * i] = dtr - d2r;
        res[2 * i + 1] = dti - d2i;
    }
    ox_fft3(res, p->nx, p->ny, p->nz, +1);
    double *sq = (double *)malloc(sizeof(double) * (size_t)n);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; i++) {
        double r = res[2 * i] / (double)n;
        sq[i] = p->ref_compat ? (double)powf((float)r, 2.0f) : r * r;
    }
    double s = det_sum(sq, n);
    free(sq);
    free(res);
    return sqrt(s / (double)n);
}

/* Avg_calc.cu:3-18 */
double ox_mean(const double *psi, long n) {
    double s = 0.0;
    for (long i = 0; i < n; i++) s += psi[i];
    return s / (double)n;
}

/* Avg_calc.cu:21-43: shift so the mean is psi0 */
void ox_pin_mean(double *psi, long n, double psi0) {
    double m = ox_mean(psi, n);
    double diff = 0.0;
    if (m != psi0) diff = psi0 - m;
    for (long i = 0; i < n; i++) psi[i] += diff;
}

/* ======================================================================= */
/* Philox4x32-10 and Gaussians                                             */
/* ======================================================================= */

static inline void mulhilo32(uint32_t a, uint32_t b, uint32_t *hi, uint32_t *lo) {
    uint64_t p = (uint64_t)a * (uint64_t)b;
    *hi = (uint32_t)(p >> 32);
    *lo = (uint32_t)p;
}

void ox_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; r++) {
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo32(0xD2511F53u, c0, &hi0, &lo0);
        mulhilo32(0xCD9E8D57u, c2, &hi1, &lo1);
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Counter = (index lo, index hi, stream lo, stream hi), key = seed.
   Box-Muller: u1 = (x0+1) 2^-32 in (0,1], u2 = x1 2^-32 in [0,1). */
void ox_gauss_pair(uint64_t seed, uint64_t stream, uint64_t index, double *g0, double *g1) {
    uint32_t ctr[4] = {(uint32_t)index, (uint32_t)(index >> 32), (uint32_t)stream, (uint32_t)(stream >> 32)};
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t o[4];
    ox_philox4x32(ctr, key, o);
    double u1 = ((double)o[0] + 1.0) * 2.3283064365386963e-10;
    double u2 = (double)o[1] * 2.3283064365386963e-10;
    double r = sqrt(-2.0 * log(u1));
    *g0 = r * cos(2.0 * M_PI * u2);
    *g1 = r * sin(2.0 * M_PI * u2);
}

/* Stream 0: initial-condition noise, one draw per grid point. */
void ox_ic_noise(double *psi, int nx, int ny, int nz, double n0, double amp, uint64_t seed) {
    const long n = (long)nx * ny * nz;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; i++) {
        double g0, g1;
        ox_gauss_pair(seed, 0, (uint64_t)i, &g0, &g1);
        psi[i] = n0 + amp * g0;
    }
}

/* fcc (111) seed: inside a sphere of radius_pts grid points about the box
   centre, psi = n0 + amp * sum_j cos(q_j . r), q_j = (2 pi/sqrt 3)(+-1,+-1,1). */
void ox_ic_fcc_seed(double *psi, int nx, int ny, int nz, double Lx, double Ly, double Lz,
                    double n0, double amp, double radius_pts) {
    const double q = 2.0 * M_PI / sqrt(3.0);
    const double dx = Lx / nx, dy = Ly / ny, dz = Lz / nz;
    const double cx = 0.5 * nx, cy = 0.5 * ny, cz = 0.5 * nz;
#pragma omp parallel for schedule(static)
    for (int iz = 0; iz < nz; iz++)
        for (int iy = 0; iy < ny; iy++)
            for (int ix = 0; ix < nx; ix++) {
                double rx = ix - cx, ry = iy - cy, rz = iz - cz;
                if (rx * rx + ry * ry + rz * rz > radius_pts * radius_pts) continue;
                double x = rx * dx, y = ry * dy, z = rz * dz;
                double s = cos(q * (x + y + z)) + cos(q * (x - y + z)) + cos(q * (-x + y + z)) +
                           cos(q * (-x - y + z));
                psi[((long)iz * ny + iy) * nx + ix] = n0 + amp * s;
            }
}

/* initialize.cu:95-197 (ICs + seeds).  Reference coordinates come from
   linspace.cu:5-18 (accumulated x[i+1] = x[i] + L/(M-1)).  The reference's
   memory index i*My+j has i on its x axis; this restatement keeps physical
   coordinates and stores psi[j*Mx + i] (x fastest). */
double ox_ic_reference(double *psi, int Mx, int My, int Lx, int Ly, double psi0, int iconfig,
                       double A_10, double A_11, double A_tri, int iseed, int ishape,
                       double h, double k, double roa) {
    const double a_tri = 2.0 / sqrt(3.0), a_sq = 1.0;
    const double k_sq = 2 * M_PI / a_sq, k_tri = 2 * M_PI / a_tri;
    double *x = (double *)malloc(sizeof(double) * (size_t)(Mx + 1));
    double *y = (double *)malloc(sizeof(double) * (size_t)(My + 1));
    double dux = (double)Lx / ((double)Mx - 1), duy = (double)Ly / ((double)My - 1);
    x[0] = 0.0; for (int i = 0; i < Mx; i++) x[i + 1] = x[i] + dux;
    y[0] = 0.0; for (int j = 0; j < My; j++) y[j + 1] = y[j] + duy;
    double r = 0.0;
    if (iconfig == 1) r = roa * a_sq;
    else if (iconfig == 0) r = roa * a_tri;
    for (int i = 0; i < Mx; i++)
        for (int j = 0; j < My; j++) {
            double X = x[i], Y = y[j], v;
            if (iconfig == 1)
                v = A_10 * ((3.0 * sqrt(2.0) - 2.0) * cos(k_sq * Y) - 2.0 * cos(k_sq * X)) -
                    A_11 * cos(k_sq * X) * cos(k_sq * Y);
            else if (iconfig == 0)
                v = A_tri * (cos(k_tri * X) / 2.0 + cos(k_tri * X / 2.0) * cos(sqrt(3.0) * k_tri * Y / 2.0));
            else
                v = 0.0;
            psi[(long)j * Mx + i] = v + psi0;
        }
    if (iseed == 1) {
        for (int i = 0; i < Mx; i++)
            for (int j = 0; j < My; j++) {
                double X = x[i], Y = y[j];
                long id = (long)j * Mx + i;
                if (ishape == 0) {
                    double d = sqrt((X - h) * (X - h) + (Y - k) * (Y - k));
                    if (d > r) psi[id] = psi0;
                } else if (ishape == 1) {
                    double g = exp(-((X - h) * (X - h) + (Y - k) * (Y - k)) / roa);
                    double v = psi[id] - psi0;
                    psi[id] = v * g + psi0 * (1 - g);
                }
            }
    }
    free(x); free(y);
    return r;
}

/* ======================================================================= */
/* Conserved noise in k-space                                              */
/* ======================================================================= */

/* xi_k = A |k| g_k, g the transform of unit white noise (E|g_k|^2 = cells),
   Hermitian by construction: mode k with 0 < ix < nx/2 draws its own pair;
   its partner -k takes the conjugate; on the ix = 0 and ix = nx/2 planes the
   canonical member of {k,-k} is the one with the smaller (iz*ny+iy); a
   self-conjugate mode takes a real draw.
   Draws: the slowest axis of the grid (z in 3-D, y in 2-D) is split in two
   halves; a canonical mode with slow coordinate s uses Philox4x32-10 at
   counter (index of the mode with s mod n/2, stream 1 + step), outputs 0,1 for
   the lower half and 2,3 for the upper, each pair through Box-Muller
   (u1 = (x+1) 2^-32, u2 = y 2^-32, r = sqrt(-2 ln u1), (r cos 2 pi u2,
   r sin 2 pi u2)).  One Philox call so serves two modes. */
void ox_noise_k(const ox_params *p, long step, double *noise_k) {
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    const long cells = (long)nx * ny * nz;
    const double scale = p->noise_amp * sqrt((double)cells);
    double *kx = (double *)malloc(sizeof(double) * (size_t)nx);
    double *ky = (double *)malloc(sizeof(double) * (size_t)ny);
    double *kz = (double *)malloc(sizeof(double) * (size_t)nz);
    ox_fft_freq(nx, p->Lx, kx);
    ox_fft_freq(ny, p->Ly, ky);
    ox_fft_freq(nz, p->Lz, kz);
    if (nz == 1) kz[0] = 0.0;
    const uint32_t key[2] = {(uint32_t)p->noise_seed, (uint32_t)(p->noise_seed >> 32)};
    const uint64_t stream = 1 + (uint64_t)step;
#pragma omp parallel for schedule(static)
    for (int iz = 0; iz < nz; iz++)
        for (int iy = 0; iy < ny; iy++)
            for (int ix = 0; ix < nx; ix++) {
                long i = ((long)iz * ny + iy) * nx + ix;
                int jx = (nx - ix) % nx, jy = (ny - iy) % ny, jz = (nz - iz) % nz;
                int canon, selfc = (jx == ix && jy == iy && jz == iz);
                if (ix > 0 && 2 * ix < nx) canon = 1;
                else if (2 * ix > nx) canon = 0;
                else canon = ((long)iz * ny + iy) <= ((long)jz * ny + jy);
                int cx = canon ? ix : jx, cy = canon ? iy : jy, cz = canon ? iz : jz;
                long ctr;
                int upper;
                if (nz > 1) {
                    upper = 2 * cz >= nz;
                    ctr = ((long)(cz % (nz / 2)) * ny + cy) * nx + cx;
                } else {
                    upper = 2 * cy >= ny;
                    ctr = (long)(cy % (ny / 2)) * nx + cx;
                }
                const uint32_t c[4] = {(uint32_t)ctr, (uint32_t)((uint64_t)ctr >> 32), (uint32_t)stream,
                                       (uint32_t)(stream >> 32)};
                uint32_t o[4];
                ox_philox4x32(c, key, o);
                const uint32_t a = upper ? o[2] : o[0], b = upper ? o[3] : o[1];
                const double u1 = ((double)a + 1.0) * 2.3283064365386963e-10;
                const double u2 = (double)b * 2.3283064365386963e-10;
                const double r = sqrt(-2.0 * log(u1));
                const double g0 = r * cos(2.0 * M_PI * u2), g1 = r * sin(2.0 * M_PI * u2);
                double kk = sqrt(kx[ix] * kx[ix] + ky[iy] * ky[iy] + kz[iz] * kz[iz]);
                double re, im;
                if (selfc) { re = g0; im = 0.0; }
                else { re = g0 * M_SQRT1_2; im = (canon ? 1.0 : -1.0) * g1 * M_SQRT1_2; }
                noise_k[2 * i] = scale * kk * re;
                noise_k[2 * i + 1] = scale * kk * im;
            }
    free(kx); free(ky); free(kz);
}

/* ======================================================================= */
/* The time loop, main.cu:232-450                                          */
/* ======================================================================= */

static double *cplx_from_real(const double *r, long n, double *out) {
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; i++) { out[2 * i] = r[i]; out[2 * i + 1] = 0.0; }
    return out;
}

/* FE of the real field psi with its spectrum psi_k (main.cu:268-286). */
static double fe_of(const ox_params *p, const double *c2, const double *psi, const double *psi_k,
                    double *tmpc, double *p2, double *p3, double *p4) {
    const long n = (long)p->nx * p->ny * p->nz;
    ox_convolve_fields(p, c2, psi_k, tmpc);
    ox_fft3(tmpc, p->nx, p->ny, p->nz, +1);
    for (long i = 0; i < n; i++) { tmpc[2 * i] /= (double)n; tmpc[2 * i + 1] /= (double)n; }
    ox_power(p, psi, p2, 2, n);
    ox_power(p, psi, p3, 3, n);
    ox_power(p, psi, p4, 4, n);
    return ox_FE_calc(p, psi, p2, p3, p4, tmpc);
}

/* The stepping loop alone (no diagnostics), timed by wall clock; used as the
   CPU baseline.  Returns the loop's seconds in *seconds. */
int ox_bench(const ox_params *p, double *psi, long nsteps, double *seconds) {
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    const long n = (long)nx * ny * nz;
    double *k2 = malloc(sizeof(double) * n), *c2 = malloc(sizeof(double) * n);
    double *psi_k = malloc(sizeof(double) * 2 * n), *psi2_k = malloc(sizeof(double) * 2 * n);
    double *psi3_k = malloc(sizeof(double) * 2 * n), *psi_kp1 = malloc(sizeof(double) * 2 * n);
    double *p2 = malloc(sizeof(double) * n), *p3 = malloc(sizeof(double) * n);
    double *noise = p->noise_amp != 0.0 ? malloc(sizeof(double) * 2 * n) : NULL;
    if (!k2 || !c2 || !psi_k || !psi2_k || !psi3_k || !psi_kp1 || !p2 || !p3) return -1;
    ox_k2_c2(p, k2, c2);
    ox_fft3(cplx_from_real(psi, n, psi_k), nx, ny, nz, -1);
    ox_power(p, psi, p2, 2, n);
    ox_power(p, psi, p3, 3, n);
#ifdef _OPENMP
    double t0 = omp_get_wtime();
#endif
    for (long it = 0; it < nsteps; it++) {
        ox_fft3(cplx_from_real(p2, n, psi2_k), nx, ny, nz, -1);
        ox_fft3(cplx_from_real(p3, n, psi3_k), nx, ny, nz, -1);
        ox_euler_step(p, k2, c2, psi_k, psi2_k, psi3_k, psi_kp1);
        if (noise) {
            ox_noise_k(p, it, noise);
#pragma omp parallel for schedule(static)
            for (long i = 0; i < n; i++) {
                double den = (1.0 + k2[i] * p->dt * p->Mo * (1.0 - p->eps) - k2[i] * p->Mo * p->dt * c2[i]);
                psi_kp1[2 * i] += noise[2 * i] / den;
                psi_kp1[2 * i + 1] += noise[2 * i + 1] / den;
            }
        }
        ox_fft3(psi_kp1, nx, ny, nz, +1);
#pragma omp parallel for schedule(static)
        for (long i = 0; i < n; i++) psi[i] = psi_kp1[2 * i] / (double)n;
        ox_power(p, psi, p2, 2, n);
        ox_power(p, psi, p3, 3, n);
        ox_fft3(cplx_from_real(psi, n, psi_k), nx, ny, nz, -1);
    }
#ifdef _OPENMP
    *seconds = omp_get_wtime() - t0;
#else
    *seconds = 0.0;
#endif
    free(k2); free(c2); free(psi_k); free(psi2_k); free(psi3_k); free(psi_kp1); free(p2); free(p3); free(noise);
    return 0;
}

/* Threads the oracle's OpenMP regions use. */
int ox_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int ox_run(const ox_params *p, double *psi, long nsteps, int t_sample, ox_diag *diag) {
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    const long n = (long)nx * ny * nz;
    double *k2 = malloc(sizeof(double) * n), *c2 = malloc(sizeof(double) * n);
    double *psi_k = malloc(sizeof(double) * 2 * n), *psi2_k = malloc(sizeof(double) * 2 * n);
    double *psi3_k = malloc(sizeof(double) * 2 * n), *psi_kp1 = malloc(sizeof(double) * 2 * n);
    double *tmpc = malloc(sizeof(double) * 2 * n);
    double *p2 = malloc(sizeof(double) * n), *p3 = malloc(sizeof(double) * n), *p4 = malloc(sizeof(double) * n);
    double *noise = p->noise_amp != 0.0 ? malloc(sizeof(double) * 2 * n) : NULL;
    if (!k2 || !c2 || !psi_k || !psi2_k || !psi3_k || !psi_kp1 || !tmpc || !p2 || !p3 || !p4) return -1;
    ox_k2_c2(p, k2, c2);
    for (long i = 0; i <= nsteps; i++) diag[i].F = diag[i].mean = diag[i].rms = NAN;

    /* iteration zero (main.cu:234-286) */
    ox_fft3(cplx_from_real(psi, n, psi_k), nx, ny, nz, -1);
    diag[0].F = fe_of(p, c2, psi, psi_k, tmpc, p2, p3, p4);
    diag[0].mean = ox_mean(psi, n);
    ox_power(p, psi, p2, 2, n);
    ox_power(p, psi, p3, 3, n);

    for (long it = 0; it < nsteps; it++) {
        ox_fft3(cplx_from_real(p2, n, psi2_k), nx, ny, nz, -1);           /* :309 */
        ox_fft3(cplx_from_real(p3, n, psi3_k), nx, ny, nz, -1);           /* :314 */
        ox_euler_step(p, k2, c2, psi_k, psi2_k, psi3_k, psi_kp1);          /* :323 */
        if (noise) {
            /* conserved noise enters the numerator before the implicit divide */
            ox_noise_k(p, it, noise);
            for (long i = 0; i < n; i++) {
                double den = (1.0 + k2[i] * p->dt * p->Mo * (1.0 - p->eps) - k2[i] * p->Mo * p->dt * c2[i]);
                psi_kp1[2 * i] += noise[2 * i] / den;
                psi_kp1[2 * i + 1] += noise[2 * i + 1] / den;
            }
        }
        if (t_sample > 0 && it % t_sample == 0)                            /* :326 */
            diag[it].rms = ox_sse_calculation(p, k2, c2, psi_kp1, psi_k, psi2_k, psi3_k);
        memcpy(tmpc, psi_kp1, sizeof(double) * 2 * n);
        ox_fft3(tmpc, nx, ny, nz, +1);                                     /* :343 */
        for (long i = 0; i < n; i++) psi[i] = tmpc[2 * i] / (double)n;    /* :349, :369 */
        ox_power(p, psi, p2, 2, n);                                        /* :371 */
        ox_power(p, psi, p3, 3, n);                                        /* :372 */
        ox_fft3(cplx_from_real(psi, n, psi_k), nx, ny, nz, -1);           /* :405 */
        if (t_sample > 0 && (it + 1) % t_sample == 0 && it + 1 < nsteps) { /* :412-427 */
            double *q4 = malloc(sizeof(double) * n);
            ox_convolve_fields(p, c2, psi_k, tmpc);
            ox_fft3(tmpc, nx, ny, nz, +1);
            for (long i = 0; i < n; i++) { tmpc[2 * i] /= (double)n; tmpc[2 * i + 1] /= (double)n; }
            ox_power(p, psi, q4, 4, n);
            diag[it + 1].F = ox_FE_calc(p, psi, p2, p3, q4, tmpc);
            diag[it + 1].mean = ox_mean(psi, n);
            free(q4);
        }
    }
    /* final FE after the loop (main.cu:439-450) */
    {
        double *q4 = malloc(sizeof(double) * n);
        ox_convolve_fields(p, c2, psi_k, tmpc);
        ox_fft3(tmpc, nx, ny, nz, +1);
        for (long i = 0; i < n; i++) { tmpc[2 * i] /= (double)n; tmpc[2 * i + 1] /= (double)n; }
        ox_power(p, psi, q4, 4, n);
        diag[nsteps].F = ox_FE_calc(p, psi, p2, p3, q4, tmpc);
        diag[nsteps].mean = ox_mean(psi, n);
        free(q4);
    }
    free(k2); free(c2); free(psi_k); free(psi2_k); free(psi3_k); free(psi_kp1);
    free(tmpc); free(p2); free(p3); free(p4); free(noise);
    return 0;
}
