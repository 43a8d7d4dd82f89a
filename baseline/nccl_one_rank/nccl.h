/* nccl.h stand-in for building LC2500/XPFC_CUDA's program on a machine
   without NCCL: the types and the three calls the reference makes
   (main.cu:75-76, FE_calc.cu:25-34, sse_calculation.cu:92-101), for one rank.
   Used by baseline/ref_gpu.py only when no NCCL header and library are found. */
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef struct ncclComm *ncclComm_t;
typedef enum { ncclSuccess = 0, ncclInvalidArgument = 4 } ncclResult_t;
typedef enum { ncclDouble = 8 } ncclDataType_t;
typedef enum { ncclSum = 0 } ncclRedOp_t;
ncclResult_t ncclCommInitAll(ncclComm_t *comms, int ndev, const int *devlist);
ncclResult_t ncclReduce(const void *sendbuff, void *recvbuff, size_t count, ncclDataType_t datatype,
                        ncclRedOp_t op, int root, ncclComm_t comm, cudaStream_t stream);
ncclResult_t ncclCommDestroy(ncclComm_t comm);
#ifdef __cplusplus
}
#endif
