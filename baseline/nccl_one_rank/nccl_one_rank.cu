// One-rank NCCL calls for the reference program (see nccl.h here): with one
// rank, a sum reduce to root 0 is a copy of the send buffer, ordered on the
// given stream as NCCL orders its kernels.
#include "nccl.h"

extern "C" {

ncclResult_t ncclCommInitAll(ncclComm_t *comms, int ndev, const int *) {
    if (ndev != 1 || !comms) return ncclInvalidArgument;
    comms[0] = nullptr;
    return ncclSuccess;
}

ncclResult_t ncclReduce(const void *sendbuff, void *recvbuff, size_t count, ncclDataType_t datatype,
                        ncclRedOp_t op, int root, ncclComm_t, cudaStream_t stream) {
    if (datatype != ncclDouble || op != ncclSum || root != 0) return ncclInvalidArgument;
    if (sendbuff == recvbuff) return ncclSuccess;
    return cudaMemcpyAsync(recvbuff, sendbuff, count * sizeof(double), cudaMemcpyDeviceToDevice, stream) ==
                   cudaSuccess
               ? ncclSuccess
               : ncclInvalidArgument;
}

ncclResult_t ncclCommDestroy(ncclComm_t) { return ncclSuccess; }

}  // extern "C"
