/* Stand-in for cuda-samples' helper_cuda.h (not shipped with the CUDA
   toolkit): the two macros LC2500/XPFC_CUDA uses, checking as the samples'
   versions do (print the error and exit). */
#pragma once
#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#define checkCudaErrors(x)                                                                     \
    do {                                                                                       \
        cudaError_t e_ = (x);                                                                  \
        if (e_ != cudaSuccess) {                                                               \
            fprintf(stderr, "CUDA error %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, __LINE__); \
            exit(EXIT_FAILURE);                                                                \
        }                                                                                      \
    } while (0)
#define getLastCudaError(msg)                                                                  \
    do {                                                                                       \
        cudaError_t e_ = cudaGetLastError();                                                   \
        if (e_ != cudaSuccess) {                                                               \
            fprintf(stderr, "%s: %s at %s:%d\n", (msg), cudaGetErrorString(e_), __FILE__, __LINE__); \
            exit(EXIT_FAILURE);                                                                \
        }                                                                                      \
    } while (0)
