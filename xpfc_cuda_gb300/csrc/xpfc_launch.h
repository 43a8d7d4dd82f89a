// xpfc_launch.h -- host-side launchers of the passes, one set per element
// type (float: the mixed path; double: the plain FP64 path).  Each launcher
// dispatches the runtime line length to its compile-time instance and
// returns cudaErrorInvalidValue for a length that has none.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include "xpfc_kernels.cuh"
#include "xpfc_regkernels.cuh"
#include "xpfc_tma.cuh"
#include "xpfc_ic.cuh"

namespace xpfc {

// Line lengths with compiled instances.
bool row_supported(int L);          // L = n0/2
bool col_supported(int L);          // n1 or n2 along a column pass
bool pen_supported(int L, int ng);  // pencil length, groups (2: 3-D, 1: 2-D)

template <typename T>
cudaError_t launch_row(int mode, int L, const RowArgs &a, const void *twL, const void *tw2L, cudaStream_t s,
                       int *nblocks);
template <typename T>
cudaError_t launch_col(int dir, int L, const ColArgs &a, int nouter, const void *twL, cudaStream_t s);
template <typename T>
cudaError_t launch_pencil(int L, int ng, const PenArgs &a, const KSpace &ks, int npairs, const void *twL,
                          cudaStream_t s, int *nblocks);
// The staged pencil pass of 3-D grids (xpfc_tma.cuh): a persistent kernel fed
// by TMA box loads of S and W through mapS / mapW (FP32 arrays
// [n2 * instances][n1][n0], boxes of [L][2 tx][1]).  pen_tma_tx gives the
// tile width in complex columns for a pencil length (0: no staged instance
// for that length and element size); the pass needs L0 % tx == 0.  err: a
// device word that a block which gave up waiting sets to XPFC_DEV_ETIMEDOUT.
int pen_tma_tx(int L, int esz);
// Whether a 3-D pencil length has the kept-spectrum register pencil
// (PenArgs::Shat; FP32 only).
bool pen_spec_supported(int L, int esz);
template <typename T>
cudaError_t launch_pencil_tma(int L, const PenArgs &a, const KSpace &ks, int npairs, const void *twL,
                              const CUtensorMap *mapS, const CUtensorMap *mapW, int *err, cudaStream_t s,
                              int *nblocks);
template <typename T>
cudaError_t launch_kspace(int op, const KSpace &ks, double a, double b, void *out, const void *x1, const void *x2,
                          const void *x3, const void *x4, cudaStream_t s);
template <typename T>
cudaError_t launch_power(const T *in, T *out, long long n, int p, int ref_compat, cudaStream_t s);
template <typename T>
cudaError_t launch_scale(T *f, long long n, double sc, cudaStream_t s);
template <typename T>
cudaError_t launch_density(const T *psi, const T *p2, const T *p3, const T *p4, const T *convl, long long n, double a,
                           double b, int square, int ref_compat, double *partials, cudaStream_t s, int *nblocks);
cudaError_t launch_convert_d2f(const double *in, float *out, long long n, cudaStream_t s);
cudaError_t launch_convert_f2d(const float *in, double *out, long long n, cudaStream_t s);
// ninst instances: instance z reduces part[z * nparts * nq ...] into out + z * ostride
cudaError_t launch_finalize(int nq, const double *part, long long nparts, double *out, cudaStream_t s, int ninst = 1,
                            long long ostride = 0);

// initial field on the device, then its mean pinned to a.psi0; scratch holds
// at least IC_SCRATCH doubles
constexpr int IC_BLOCKS = 1024, IC_SCRATCH = IC_BLOCKS + 8;
cudaError_t launch_initial_field(const ICArgs &a, double *psi, double *scratch, cudaStream_t s);

// grid shapes the launchers use (for sizing the partials buffer)
int row_rows(int L);
template <typename T> int col_tx(int L);
template <typename T> int pen_tx(int L, int ng);
constexpr int DENSITY_BLOCKS = 1024;

}  // namespace xpfc
