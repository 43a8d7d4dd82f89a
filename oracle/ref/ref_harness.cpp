/*
 * ref_harness.cpp -- TEST INFRASTRUCTURE.  Runs LC2500/XPFC_CUDA's own host
 * code (read_input.cu, initialize.cu, Avg_calc.cu, FFT_freq.cu, linspace.cu,
 * write_vtk.cu) and its own kernel bodies (euler_step.cu:33-63,
 * power_functions.cu:34-53, scaling_step.cu:34-53, copy_matrix.cu:34-49,
 * convolve_fields.cu:30-51, FE_calc.cu:54-68, sse_calculation.cu:120-161),
 * compiled as host code by oracle/ref/Makefile from the reference tree, on the
 * CPU.  Each kernel is called with a 1x1 grid of 1x1 blocks, so its grid-stride
 * loops visit every point in order.
 *
 * What this harness supplies itself:
 *  - the call sequence of main.cu:232-450 (iteration 0, the time loop with its
 *    t_sample branches, the final free energy), restated here;
 *  - cuFFT-Xt's Z2Z transforms, replaced by the unnormalised DFT (the oracle's
 *    FFT, checked against numpy in the tests); at one GPU the cufftXtMemcpy
 *    re-orderings are plain copies;
 *  - the NCCL reduce + sum_reduction.cu kernels, replaced by a sequential sum.
 *
 * Run in a directory holding pfc.input (and initial_density_field.vtk for
 * iconfig = 10).  Writes ref_params.txt, ref_k2.bin, ref_c2.bin, ref_psi0.bin,
 * ref_diag.txt, ref_psi_final.bin and the reference's density_data<t>.vtk files.
 */
#define MAIN
#include "globals.cuh"

#include <vector>

extern "C" void ox_fft3(double *data, int nx, int ny, int nz, int sign);

uint3 threadIdx = {0, 0, 0}, blockIdx = {0, 0, 0};
dim3 blockDim(1, 1, 1), gridDim(1, 1, 1);

/* the reference kernels, extracted by the Makefile */
#include "kern_body.inc"

typedef std::vector<cufftDoubleComplex> cvec;

static void fft(cvec &v, int sign) { ox_fft3((double *)v.data(), My, Mx, 1, sign); }

static void scale(cvec &v) { scaling_step(v.data(), 0, Mx, M2, 1); }

static double sum(const std::vector<double> &v) {
    double s = 0.0;
    for (double x : v) s += x;
    return s;
}

static void dump(const char *name, const void *p, size_t bytes) {
    FILE *f = fopen(name, "wb");
    fwrite(p, 1, bytes, f);
    fclose(f);
}

int main() {
    num_gpus = 1;
    read_input();
    initialize();
    chunk_size_real = M2;

    FILE *pf = fopen("ref_params.txt", "w");
    fprintf(pf, "psi_0 %.17g\ns %.17g\na %.17g\nb %.17g\neps %.17g\nMo %.17g\n", psi_0, s, a, b, eps, Mo);
    fprintf(pf, "Lx %d\nLy %d\nMx %d\nMy %d\nt %d\ndt %.17g\nt_sample %d\niconfig %d\n", Lx, Ly, Mx, My, t, dt,
            t_sample, iconfig);
    fprintf(pf, "N_t_steps %.17g\nff_factor %.17g\nr %.17g\n", N_t_steps, ff_factor, r);
    fclose(pf);
    dump("ref_k2.bin", k2_host, sizeof(double) * M2);
    dump("ref_c2.bin", c2_k_host, sizeof(double) * M2);
    {
        std::vector<double> x(M2);
        for (int i = 0; i < M2; i++) x[i] = psi_host[i].x;
        dump("ref_psi0.bin", x.data(), sizeof(double) * M2);
    }

    cvec psi(M2), psi_out(M2), np1(M2), np1_out(M2), convl(M2), convl_out(M2), psi2(M2), psi2_out(M2),
        psi3(M2), psi3_out(M2), psi4(M2), res_k(M2);
    std::vector<double> ff(M2);
    for (int i = 0; i < M2; i++) psi[i] = make_double2(psi_host[i].x, psi_host[i].y);

    FILE *df = fopen("ref_diag.txt", "w");

    /* iteration zero, main.cu:234-286 */
    apply_power(psi.data(), psi2.data(), 0, Mx, M2, 1, 2);
    apply_power(psi.data(), psi3.data(), 0, Mx, M2, 1, 3);
    apply_power(psi.data(), psi4.data(), 0, Mx, M2, 1, 4);
    fft(psi, -1);
    psi_out = psi;
    convolve_fields(psi_out.data(), c2_k_host, convl.data(), 0, Mx, 1);
    fft(convl, +1);
    scale(convl);
    convl_out = convl;
    fft(psi, +1);
    scale(psi);
    FE_calc(0, a, b, psi.data(), psi2.data(), psi3.data(), psi4.data(), convl_out.data(), 0, Mx, M2, 1, ff.data());
    fprintf(df, "F 0 %.17g\n", sum(ff) * ff_factor);
    writeVTKFile(psi_host, Mx, My, Lx, Ly, 0);

    int n;
    for (n = 0; n < N_t_steps; n++) { /* main.cu:306-435 */
        fft(psi2, -1);
        fft(psi3, -1);
        psi2_out = psi2;
        psi3_out = psi3;
        euler_step(n, a, b, Mo, np1.data(), psi_out.data(), psi2_out.data(), psi3_out.data(), c2_k_host, k2_host,
                   dt, eps, 0, Mx, 1);
        if (n % t_sample == 0) { /* sse_calculation.cu:3-116 */
            residual_calc(n, res_k.data(), np1.data(), psi_out.data(), psi2_out.data(), psi3_out.data(), c2_k_host,
                          k2_host, Mo, dt, a, b, 0, Mx, 1);
            fft(res_k, +1);
            scale(res_k);
            apply_power(res_k.data(), res_k.data(), 0, Mx, M2, 1, 2);
            copy_struct(res_k.data(), ff.data(), 0, Mx, 1);
            fprintf(df, "RMS %d %.17g\n", n, sqrt(sum(ff) / M2));
        }
        fft(np1, +1);
        scale(np1);
        np1_out = np1;
        copy_matrix(np1_out.data(), psi.data(), 0, Mx, 1);
        apply_power(psi.data(), psi2.data(), 0, Mx, M2, 1, 2);
        apply_power(psi.data(), psi3.data(), 0, Mx, M2, 1, 3);
        fft(psi, -1);
        psi_out = psi;
        if ((n + 1) % t_sample == 0) {
            convolve_fields(psi_out.data(), c2_k_host, convl.data(), 0, Mx, 1);
            fft(convl, +1);
            scale(convl);
            convl_out = convl;
            apply_power(np1_out.data(), psi4.data(), 0, Mx, M2, 1, 4);
            FE_calc(n + 1, a, b, np1_out.data(), psi2.data(), psi3.data(), psi4.data(), convl_out.data(), 0, Mx, M2,
                    1, ff.data());
            fprintf(df, "F %d %.17g\n", n + 1, sum(ff) * ff_factor);
        }
    }
    /* main.cu:439-455 */
    convolve_fields(psi_out.data(), c2_k_host, convl.data(), 0, Mx, 1);
    fft(convl, +1);
    scale(convl);
    convl_out = convl;
    apply_power(np1_out.data(), psi4.data(), 0, Mx, M2, 1, 4);
    FE_calc(n, a, b, np1_out.data(), psi2.data(), psi3.data(), psi4.data(), convl_out.data(), 0, Mx, M2, 1, ff.data());
    fprintf(df, "FINAL %d %.17g\n", n, sum(ff) * ff_factor);
    fclose(df);
    {
        std::vector<double> x(M2);
        for (int i = 0; i < M2; i++) x[i] = np1_out[i].x;
        dump("ref_psi_final.bin", x.data(), sizeof(double) * M2);
        for (int i = 0; i < M2; i++) psi_host_out[i] = {np1_out[i].x, np1_out[i].y};
    }
    writeVTKFile(psi_host_out, Mx, My, Lx, Ly, n);
    return 0;
}
