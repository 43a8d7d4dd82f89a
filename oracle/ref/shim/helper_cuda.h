/* Stand-in for cuda-samples' helper_cuda.h (absent from this image): the two
   macros the reference uses, as no-ops for a host-only build. */
#pragma once
#define checkCudaErrors(x) (x)
#define getLastCudaError(msg) ((void)0)
