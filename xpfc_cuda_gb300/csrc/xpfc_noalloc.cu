// xpfc_noalloc.cu -- the free-energy reduction of FE_calc without any
// allocation, for callers that cannot call cudaMalloc.
//
// Who needs it: code that runs where the CUDA allocator is off limits, e.g.
// a host framework that owns all device memory through its own pool and
// forbids plugins to allocate behind its back, or a solver loop run under a
// fixed device-memory budget that counts every allocation.  xpfc_FE_calc
// reduces through a context-owned buffer that xpfc_create allocated; this
// variant takes the five density arrays from the caller and keeps its partial
// sums in a fixed array in the library's own device memory.
//
// The scratch: g_fe_scratch, a file-scope __device__ array of
// XPFC_NOALLOC_MAX_CHUNKS + 1 doubles (32 KB).  Every GPU that loads the
// library holds it until the process exits.  Each block of the first kernel
// reduces one chunk of XPFC_NOALLOC_CHUNK points into one slot, so the largest
// accepted field is XPFC_NOALLOC_MAX_POINTS = chunks x chunk = 2^28 points;
// larger fields are rejected with XPFC_EINVAL.  Every call shares the array
// and overwrites the slots it uses (the result slot is cleared first), so two
// calls whose kernels overlap on the GPU race: serialise them (one stream, or
// events).  The call waits for its own work on the given stream and returns
// F on the host.
//
// Host code must not hand the array's name to a kernel: on the host the name
// is only a stand-in for the device symbol.  The device address is looked up
// once per device with cudaGetSymbolAddress, on the first call made while
// that device is current; make that first call before any stream capture.
// The address is kept for the life of the process, so a cudaDeviceReset
// after the first call (which reloads the library's module and may move the
// array) is not supported.
#include <cuda_runtime.h>

#include <string>

#include "../../include/xpfc.h"
#include "xpfc_host.h"

namespace {

constexpr long long kChunk = XPFC_NOALLOC_CHUNK;
constexpr int kMaxChunks = XPFC_NOALLOC_MAX_CHUNKS;
constexpr int kThreads = 256;

static __device__ __align__(256) double g_fe_scratch[kMaxChunks + 1];

// one block per chunk: sum of the FE_calc.cu:64 density over the chunk
__global__ void __launch_bounds__(kThreads)
fe_chunk_sums(const double *__restrict__ psi, const double *__restrict__ p2, const double *__restrict__ p3,
              const double *__restrict__ p4, const double *__restrict__ convl, long long n, double a, double b,
              double *__restrict__ slots) {
    __shared__ double warp_sums[kThreads / 32];
    const long long lo = (long long)blockIdx.x * kChunk;
    const long long hi = (lo + kChunk < n) ? lo + kChunk : n;
    double s = 0.0;
    for (long long i = lo + threadIdx.x; i < hi; i += kThreads)
        s += 0.5 * p2[i] - (a / 3.0) * p3[i] + (b / 4.0) * p4[i] - 0.5 * psi[i] * convl[i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) warp_sums[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < kThreads / 32; w++) t += warp_sums[w];
        slots[blockIdx.x] = t;
    }
}

// one block: the chunk sums in chunk order, into the result slot
__global__ void __launch_bounds__(kThreads) fe_total(double *__restrict__ slots, int nchunks) {
    __shared__ double part[kThreads];
    double s = 0.0;
    for (int c = threadIdx.x; c < nchunks; c += kThreads) s += slots[c];
    part[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int i = 0; i < kThreads; i++) t += part[i];
        slots[kMaxChunks] = t;
    }
}

int fail(int code, const std::string &m) {
    xpfc::set_thread_error(m);
    return code;
}

}  // namespace

extern "C" int xpfc_FE_calc_noalloc(const double *psi, const double *psi2, const double *psi3, const double *psi4,
                                    const double *convl_r, long long n, double a, double b, double ff_factor,
                                    double *F, void *stream) {
    if (!psi || !psi2 || !psi3 || !psi4 || !convl_r || !F) return fail(XPFC_EINVAL, "null argument");
    if (n <= 0) return fail(XPFC_EINVAL, "n must be positive");
    if (n > XPFC_NOALLOC_MAX_POINTS)
        return fail(XPFC_EINVAL, "xpfc_FE_calc_noalloc: " + std::to_string(n) + " points exceed the maximum of " +
                                     std::to_string((long long)XPFC_NOALLOC_MAX_POINTS));
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(XPFC_ECUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    // looked up on every call (it allocates nothing): a cached address would
    // go stale if the caller reset the device and the module was reloaded
    void *sym = nullptr;
    e = cudaGetSymbolAddress(&sym, g_fe_scratch);
    if (e != cudaSuccess) return fail(XPFC_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    double *slots = static_cast<double *>(sym);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int nchunks = (int)((n + kChunk - 1) / kChunk);
    e = cudaMemsetAsync(slots + kMaxChunks, 0, sizeof(double), s);
    if (e != cudaSuccess) return fail(XPFC_ECUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
    fe_chunk_sums<<<nchunks, kThreads, 0, s>>>(psi, psi2, psi3, psi4, convl_r, n, a, b, slots);
    fe_total<<<1, kThreads, 0, s>>>(slots, nchunks);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(XPFC_ECUDA, std::string("launch: ") + cudaGetErrorString(e));
    double total = 0.0;
    e = cudaMemcpyAsync(&total, slots + kMaxChunks, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(XPFC_ECUDA, std::string("result copy: ") + cudaGetErrorString(e));
    *F = total * ff_factor;
    return XPFC_OK;
}
