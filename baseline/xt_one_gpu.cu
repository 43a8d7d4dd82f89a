// xt_one_gpu.cu -- cuFFT's multi-GPU descriptor calls for a single GPU, linked
// into the build of LC2500/XPFC_CUDA's own program (baseline/ref_gpu.py).
//
// Why: the reference plans its 2-D Z2Z transform through cufftXtSetGPUs
// (main.cu:109-110) and exits when that call fails; the cuFFT API reference
// documents CUFFT_INVALID_VALUE for fewer than two GPUs, and a GB300 machine
// here gives one process one GPU.  The reference keeps every field in
// cudaLibXtDesc descriptors (main.cu:135-180) and moves them with
// cufftXtMemcpy / cufftXtExecDescriptor.  Definitions of those five calls in
// the executable take precedence over libcufft's, so the unmodified reference
// sources run on one GPU with:
//   cufftXtSetGPUs         accepts exactly one GPU (makes it current);
//   cufftMakePlan2d        is passed through to cuFFT (a plain one-GPU plan)
//                          and the plan's size recorded for cufftXtMalloc;
//   cufftXtMalloc / Free   one device buffer of nx*ny double complex values;
//   cufftXtMemcpy          cudaMemcpy (at one GPU the natural and the
//                          transform order coincide, so the device-to-device
//                          "re-order" is a copy);
//   cufftXtExecDescriptor  cufftExecZ2Z on the descriptors' buffers.
// Everything runs on the legacy default stream, as the reference's kernels do.
#include <cuda_runtime.h>
#include <cufftXt.h>
#include <dlfcn.h>

#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>

namespace {
struct PlanSize {
    long long nx = 0, ny = 0;
};
std::mutex g_mu;
std::map<cufftHandle, PlanSize> g_plans;

size_t desc_bytes(cufftHandle plan) {
    std::lock_guard<std::mutex> g(g_mu);
    auto it = g_plans.find(plan);
    if (it == g_plans.end()) return 0;
    return (size_t)(it->second.nx * it->second.ny) * sizeof(cufftDoubleComplex);
}
}  // namespace

extern "C" {

cufftResult CUFFTAPI cufftXtSetGPUs(cufftHandle, int nGPUs, int *whichGPUs) {
    if (nGPUs != 1 || !whichGPUs) return CUFFT_INVALID_VALUE;
    return cudaSetDevice(whichGPUs[0]) == cudaSuccess ? CUFFT_SUCCESS : CUFFT_INVALID_VALUE;
}

cufftResult CUFFTAPI cufftMakePlan2d(cufftHandle plan, int nx, int ny, cufftType type, size_t *workSize) {
    typedef cufftResult (*fn_t)(cufftHandle, int, int, cufftType, size_t *);
    static fn_t real = (fn_t)dlsym(RTLD_NEXT, "cufftMakePlan2d");
    if (!real) {
        fprintf(stderr, "xt_one_gpu: cufftMakePlan2d not found in libcufft\n");
        return CUFFT_INTERNAL_ERROR;
    }
    const cufftResult r = real(plan, nx, ny, type, workSize);
    if (r == CUFFT_SUCCESS) {
        std::lock_guard<std::mutex> g(g_mu);
        g_plans[plan].nx = nx;
        g_plans[plan].ny = ny;
    }
    return r;
}

cufftResult CUFFTAPI cufftXtMalloc(cufftHandle plan, cudaLibXtDesc **descriptor, cufftXtSubFormat format) {
    const size_t bytes = desc_bytes(plan);
    if (!descriptor || bytes == 0) return CUFFT_INVALID_PLAN;
    cudaLibXtDesc *d = (cudaLibXtDesc *)calloc(1, sizeof(cudaLibXtDesc));
    cudaXtDesc *x = (cudaXtDesc *)calloc(1, sizeof(cudaXtDesc));
    if (!d || !x) {
        free(d);
        free(x);
        return CUFFT_ALLOC_FAILED;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    void *p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) {
        free(d);
        free(x);
        return CUFFT_ALLOC_FAILED;
    }
    x->version = CUDA_XT_DESCRIPTOR_VERSION;
    x->nGPUs = 1;
    x->GPUs[0] = dev;
    x->data[0] = p;
    x->size[0] = bytes;
    d->version = CUDA_XT_DESCRIPTOR_VERSION;
    d->descriptor = x;
    d->library = LIB_FORMAT_CUFFT;
    d->subFormat = format;
    d->libDescriptor = nullptr;
    *descriptor = d;
    return CUFFT_SUCCESS;
}

cufftResult CUFFTAPI cufftXtFree(cudaLibXtDesc *descriptor) {
    if (!descriptor) return CUFFT_INVALID_VALUE;
    if (descriptor->descriptor) {
        cudaFree(descriptor->descriptor->data[0]);
        free(descriptor->descriptor);
    }
    free(descriptor);
    return CUFFT_SUCCESS;
}

cufftResult CUFFTAPI cufftXtMemcpy(cufftHandle, void *dstPointer, void *srcPointer, cufftXtCopyType type) {
    cudaError_t e = cudaErrorInvalidValue;
    if (type == CUFFT_COPY_HOST_TO_DEVICE) {
        cudaLibXtDesc *dst = (cudaLibXtDesc *)dstPointer;
        e = cudaMemcpy(dst->descriptor->data[0], srcPointer, dst->descriptor->size[0], cudaMemcpyHostToDevice);
        dst->subFormat = CUFFT_XT_FORMAT_INPLACE;
    } else if (type == CUFFT_COPY_DEVICE_TO_HOST) {
        cudaLibXtDesc *src = (cudaLibXtDesc *)srcPointer;
        e = cudaMemcpy(dstPointer, src->descriptor->data[0], src->descriptor->size[0], cudaMemcpyDeviceToHost);
    } else if (type == CUFFT_COPY_DEVICE_TO_DEVICE) {
        cudaLibXtDesc *dst = (cudaLibXtDesc *)dstPointer, *src = (cudaLibXtDesc *)srcPointer;
        e = cudaMemcpy(dst->descriptor->data[0], src->descriptor->data[0], src->descriptor->size[0],
                       cudaMemcpyDeviceToDevice);
        dst->subFormat = CUFFT_XT_FORMAT_INPLACE;
    }
    return e == cudaSuccess ? CUFFT_SUCCESS : CUFFT_EXEC_FAILED;
}

cufftResult CUFFTAPI cufftXtExecDescriptor(cufftHandle plan, cudaLibXtDesc *input, cudaLibXtDesc *output,
                                           int direction) {
    if (!input || !output) return CUFFT_INVALID_VALUE;
    const cufftResult r = cufftExecZ2Z(plan, (cufftDoubleComplex *)input->descriptor->data[0],
                                       (cufftDoubleComplex *)output->descriptor->data[0], direction);
    // the multi-GPU library marks an in-place result as shuffled; the
    // reference resets the flag itself (main.cu:431-434)
    if (r == CUFFT_SUCCESS) output->subFormat = CUFFT_XT_FORMAT_INPLACE_SHUFFLED;
    return r;
}

}  // extern "C"
