// xpfc_ic.cuh -- initial fields built on the device (FP64, [Mx][My][Mz] layout),
// the same functions as the host builder (initialize.cu:95-197 for the
// reference lattices and seeds; the Philox noise liquid and the fcc (111)
// seed), followed by mean pinning (Avg_calc.cu:21-43) on the device.
#pragma once
#include "fft_core.cuh"

namespace xpfc {

enum { IC_DEV_REFERENCE = 0, IC_DEV_NOISE = 1, IC_DEV_FCC_SEED = 2 };

struct ICArgs {
    int kind;
    int Mx, My, Mz;
    double Lx, Ly, Lz, psi0;
    // noise liquid: psi0 + amp * g, g from Philox4x32-10 (key ic_seed,
    // counter = point index, stream 0) through FP64 Box-Muller
    double amp;
    unsigned long long seed;
    // fcc seed: sphere of radius R (grid points) about the box centre
    double seed_amp, seed_radius;
    // reference lattices: iconfig 0 (triangular), 1 (square), 2 (liquid);
    // the accumulated coordinates x[i], y[j] of linspace.cu:5-18 come from
    // the host, which sums them in the reference's order
    int iconfig, iseed, ishape;
    double A_10, A_11, A_tri, h, k, roa;
    const double *xs, *ys;
};

__device__ __forceinline__ double ic_gauss0(unsigned long long seed, unsigned long long index) {
    const uint4 o = philox4x32_10<false>(make_uint4((uint32_t)index, (uint32_t)(index >> 32), 0u, 0u),
                                         make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
    const double u1 = ((double)o.x + 1.0) * 2.3283064365386963e-10;
    const double u2 = (double)o.y * 2.3283064365386963e-10;
    return sqrt(-2.0 * log(u1)) * cos(2.0 * 3.14159265358979323846 * u2);
}

__device__ __forceinline__ double ic_reference_at(const ICArgs &a, int i, int j) {
    const double a_tri = 2.0 / sqrt(3.0), a_sq = 1.0;
    const double k_sq = 2 * 3.14159265358979323846 / a_sq, k_tri = 2 * 3.14159265358979323846 / a_tri;
    const double X = a.xs[i], Y = a.ys[j];
    double v;
    if (a.iconfig == 1)
        v = a.A_10 * ((3.0 * sqrt(2.0) - 2.0) * cos(k_sq * Y) - 2.0 * cos(k_sq * X)) - a.A_11 * cos(k_sq * X) * cos(k_sq * Y);
    else if (a.iconfig == 0)
        v = a.A_tri * (cos(k_tri * X) / 2.0 + cos(k_tri * X / 2.0) * cos(sqrt(3.0) * k_tri * Y / 2.0));
    else
        v = 0.0;
    double psi = v + a.psi0;
    if (a.iseed == 1) {
        const double r = a.iconfig == 1 ? a.roa * a_sq : (a.iconfig == 0 ? a.roa * a_tri : 0.0);
        if (a.ishape == 0) {
            const double d = sqrt((X - a.h) * (X - a.h) + (Y - a.k) * (Y - a.k));
            if (d > r) psi = a.psi0;
        } else {
            const double g = exp(-((X - a.h) * (X - a.h) + (Y - a.k) * (Y - a.k)) / a.roa);
            psi = (psi - a.psi0) * g + a.psi0 * (1 - g);
        }
    }
    return psi;
}

static __global__ void __launch_bounds__(256) ic_kernel(ICArgs a, double *__restrict__ psi, long long n) {
    const double q = 2.0 * 3.14159265358979323846 / sqrt(3.0);
    for (long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x; id < n; id += (long long)gridDim.x * blockDim.x) {
        const int iz = (int)(id % a.Mz);
        const int iy = (int)((id / a.Mz) % a.My);
        const int ix = (int)(id / ((long long)a.Mz * a.My));
        double v;
        if (a.kind == IC_DEV_REFERENCE) {
            v = ic_reference_at(a, ix, iy);
        } else {
            v = a.psi0 + a.amp * ic_gauss0(a.seed, (unsigned long long)id);
            if (a.kind == IC_DEV_FCC_SEED) {
                const double rx = ix - 0.5 * a.Mx, ry = iy - 0.5 * a.My, rz = iz - 0.5 * a.Mz;
                if (rx * rx + ry * ry + rz * rz <= a.seed_radius * a.seed_radius) {
                    const double X = rx * (a.Lx / a.Mx), Y = ry * (a.Ly / a.My), Z = rz * (a.Lz / a.Mz);
                    const double s = cos(q * (X + Y + Z)) + cos(q * (X - Y + Z)) + cos(q * (-X + Y + Z)) +
                                     cos(q * (-X - Y + Z));
                    v = a.psi0 + a.seed_amp * s;
                }
            }
        }
        psi[id] = v;
    }
}

// per-block partial sums of x (fixed order for a fixed grid)
static __global__ void __launch_bounds__(256) sum_partials(const double *__restrict__ x, long long n,
                                                    double *__restrict__ partials) {
    __shared__ double sred[32];
    double v[1] = {0.0};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        v[0] += x[i];
    block_reduce_store<1>(v, partials + blockIdx.x, sred);
}

// psi += psi0 - mean when the mean differs from psi0 (Avg_calc.cu:21-43)
static __global__ void __launch_bounds__(256) pin_mean_kernel(double *__restrict__ psi, long long n,
                                                       const double *__restrict__ total, double psi0) {
    const double m = *total / (double)n;
    const double diff = (m != psi0) ? psi0 - m : 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        psi[i] += diff;
}

}  // namespace xpfc
