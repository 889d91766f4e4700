// bf16 slicing of FP64 arrays for the split-precision sigma path.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "kernels.cuh"

namespace bgpu {
namespace dev {

cudaError_t launch_slices(const double* x, int64_t n, int ns, __nv_bfloat16* s0, __nv_bfloat16* s1,
                          __nv_bfloat16* s2, cudaStream_t s);

}  // namespace dev
}  // namespace bgpu
