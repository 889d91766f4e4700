// Operand slicing of the split-precision path: every FP64 element x is
// carried as NS bf16 slices x = s0 + s1 (+ s2), s_i = bf16(x - s_0 - ... -
// s_{i-1}); products s_i * t_j with i + j < NS are formed on the tensor cores
// (NS = 2: three products per logical product, "BF16x3"; NS = 3: six,
// "BF16x6").  Slice arrays have exactly the layout of their FP64 arenas.
#include <cuda_bf16.h>

#include "kernels.cuh"
#include "k_split.cuh"

namespace bgpu {
namespace dev {

// x (FP64) -> NS bf16 slices, s_i = bf16(x - s_0 - ... - s_{i-1}) computed in FP64.
__global__ void slice_kernel(const double* __restrict__ x, int64_t n, int ns, __nv_bfloat16* __restrict__ s0,
                             __nv_bfloat16* __restrict__ s1, __nv_bfloat16* __restrict__ s2) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride) {
    double v = x[t];
    const __nv_bfloat16 a = __double2bfloat16(v);
    s0[t] = a;
    v -= (double)__bfloat162float(a);
    const __nv_bfloat16 b = __double2bfloat16(v);
    s1[t] = b;
    if (ns > 2) {
      v -= (double)__bfloat162float(b);
      s2[t] = __double2bfloat16(v);
    }
  }
}

cudaError_t launch_slices(const double* x, int64_t n, int ns, __nv_bfloat16* s0, __nv_bfloat16* s1,
                          __nv_bfloat16* s2, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  int64_t b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  slice_kernel<<<(int)b, 256, 0, s>>>(x, n, ns, s0, s1, s2);
  return cudaGetLastError();
}

}  // namespace dev
}  // namespace bgpu
