#pragma once
#include <cuda_runtime.h>

#include <string>

#include "props.h"

#define SG_CUDA(call)                                                                  \
    do {                                                                               \
        cudaError_t sg_err_ = (call);                                                  \
        if (sg_err_ != cudaSuccess)                                                    \
            throw ::sg::SgError(std::string("CUDA error: ") + cudaGetErrorString(sg_err_) + \
                                " (" #call ")");                                        \
    } while (0)

#define SG_LAUNCH_CHECK() SG_CUDA(cudaGetLastError())

namespace sg {
inline unsigned blocks_for(long n, int threads) { return (unsigned)((n + threads - 1) / threads); }
}  // namespace sg
