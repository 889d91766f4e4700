// Split-precision (bf16 slices, FP32 accumulation) variant of the grouped
// GEMM of kernels.cuh.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "kernels.cuh"

namespace bgpu {
namespace dev {

struct SplitBufs {
  // operand slices per buffer id (nullptr where unused)
  const __nv_bfloat16* s[kMaxBufs][3];
  // outputs: FP64 (final sigma) or bf16 slices (stage-1 intermediates)
  double* out64[kMaxBufs];
  __nv_bfloat16* out16[kMaxBufs][3];
};

// ns = number of slices (2: three products, 3: six products)
cudaError_t launch_gemm_split(int ns, const SplitBufs& bufs, const GemmUnit* units, const GemmItem* items,
                              const GemmTask* tasks, int ntasks, cudaStream_t s);
cudaError_t launch_slices(const double* x, int64_t n, int ns, __nv_bfloat16* s0, __nv_bfloat16* s1,
                          __nv_bfloat16* s2, cudaStream_t s);

}  // namespace dev
}  // namespace bgpu
