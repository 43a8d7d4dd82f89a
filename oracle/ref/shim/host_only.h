/* Forced include for the host-only build of the reference: pinned host
   allocations become zeroed heap allocations (no GPU is present). */
#pragma once
#include <cuda_runtime.h>
#include <stdlib.h>
static inline cudaError_t xref_host_alloc(void **p, size_t n) { *p = calloc(1, n); return *p ? cudaSuccess : cudaErrorMemoryAllocation; }
#define cudaMallocHost(p, n) xref_host_alloc((void **)(p), (n))
#define cudaFreeHost(p) (free(p), cudaSuccess)
