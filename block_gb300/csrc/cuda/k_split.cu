// Split-precision grouped GEMM: every FP64 operand element x is carried as
// NS bf16 slices x = s0 + s1 (+ s2) (s_i = bf16(x - s_0 - ... - s_{i-1})),
// products s_i * t_j with i + j < NS are formed on the tensor cores with FP32
// accumulation per product list item, and the items of an output rectangle
// are combined in FP32 registers.  NS = 2 gives 3 products per logical
// product ("BF16x3"), NS = 3 gives 6 ("BF16x6").  The work lists are the
// ones of the FP64 path (kernels.cuh); operands are read from slice arrays
// laid out exactly like their FP64 arenas.
#include <cuda_bf16.h>

#include "kernels.cuh"
#include "k_split.cuh"

namespace bgpu {
namespace dev {

namespace {
constexpr int TM = 64, TN = 64, TK = 16, NT = 128;
constexpr int SP = 24;  // smem row pitch in bf16 (48 bytes: conflict-free fragment loads)

__device__ __forceinline__ void mma_bf16(float* c, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ __nv_bfloat16 ld_op16(const __nv_bfloat16* __restrict__ p, int64_t ld, bool t, int r,
                                                 int c) {
  return t ? p[(int64_t)c * ld + r] : p[(int64_t)r * ld + c];
}
}  // namespace

template <int NS>
__global__ void __launch_bounds__(NT) gemm_split_kernel(SplitBufs bufs, const GemmUnit* __restrict__ units,
                                                        const GemmItem* __restrict__ items,
                                                        const GemmTask* __restrict__ tasks) {
  __shared__ __align__(16) __nv_bfloat16 As[NS][TM][SP];
  __shared__ __align__(16) __nv_bfloat16 Bs[NS][TN][SP];
  const GemmTask task = tasks[blockIdx.x];
  const GemmUnit u = units[task.unit];
  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int wm = warp >> 1, wn = warp & 1;  // 2x2 warps, 32x32 each
  const int g = lane >> 2, tg = lane & 3;
  const int row0 = task.tm * TM, col0 = task.tn * TN;
  float tot[2][4][4];
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b)
#pragma unroll
      for (int c = 0; c < 4; ++c) tot[a][b][c] = 0.f;
  for (int it = u.ibeg; it < u.iend; ++it) {
    const GemmItem gi = items[it];
    float acc[2][4][4];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[a][b][c] = 0.f;
    for (int k0 = 0; k0 < gi.k; k0 += TK) {
      // A tile: TM x TK of op(A), every slice; stored [m][k]
      for (int e = tid; e < TM * TK; e += NT) {
        int i, p;
        if (gi.ta) { i = e % TM; p = e / TM; }
        else { i = e / TK; p = e % TK; }
        const int gr = row0 + i, gp = k0 + p;
        const bool in = gr < u.m && gp < gi.k;
#pragma unroll
        for (int s = 0; s < NS; ++s)
          As[s][i][p] = in ? ld_op16(bufs.s[gi.a_buf][s] + gi.a_off, gi.lda, gi.ta, gr, gp) : __float2bfloat16(0.f);
      }
      // B tile: TK x TN of op(B); stored [n][k]
      for (int e = tid; e < TK * TN; e += NT) {
        int p, j;
        if (gi.tb) { p = e % TK; j = e / TK; }
        else { p = e / TN; j = e % TN; }
        const int gp = k0 + p, gc = col0 + j;
        const bool in = gp < gi.k && gc < u.n;
#pragma unroll
        for (int s = 0; s < NS; ++s)
          Bs[s][j][p] = in ? ld_op16(bufs.s[gi.b_buf][s] + gi.b_off, gi.ldb, gi.tb, gp, gc) : __float2bfloat16(0.f);
      }
      __syncthreads();
      uint32_t af[NS][2][4], bfr[NS][4][2];
#pragma unroll
      for (int s = 0; s < NS; ++s) {
#pragma unroll
        for (int mi = 0; mi < 2; ++mi) {
          const int r = wm * 32 + mi * 16 + g;
          af[s][mi][0] = *reinterpret_cast<const uint32_t*>(&As[s][r][tg * 2]);
          af[s][mi][1] = *reinterpret_cast<const uint32_t*>(&As[s][r + 8][tg * 2]);
          af[s][mi][2] = *reinterpret_cast<const uint32_t*>(&As[s][r][tg * 2 + 8]);
          af[s][mi][3] = *reinterpret_cast<const uint32_t*>(&As[s][r + 8][tg * 2 + 8]);
        }
#pragma unroll
        for (int ni = 0; ni < 4; ++ni) {
          const int c = wn * 32 + ni * 8 + g;
          bfr[s][ni][0] = *reinterpret_cast<const uint32_t*>(&Bs[s][c][tg * 2]);
          bfr[s][ni][1] = *reinterpret_cast<const uint32_t*>(&Bs[s][c][tg * 2 + 8]);
        }
      }
#pragma unroll
      for (int mi = 0; mi < 2; ++mi)
#pragma unroll
        for (int ni = 0; ni < 4; ++ni)
#pragma unroll
          for (int sa = 0; sa < NS; ++sa)
#pragma unroll
            for (int sb = 0; sb < NS; ++sb)
              if (sa + sb < NS) mma_bf16(acc[mi][ni], af[sa][mi], bfr[sb][ni]);
      __syncthreads();
    }
    const float al = (float)gi.alpha;
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b)
#pragma unroll
        for (int c = 0; c < 4; ++c) tot[a][b][c] = fmaf(al, acc[a][b][c], tot[a][b][c]);
  }
  // epilogue: FP64 output or bf16 slices of an intermediate
#pragma unroll
  for (int mi = 0; mi < 2; ++mi)
#pragma unroll
    for (int ni = 0; ni < 4; ++ni)
#pragma unroll
      for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const int r = row0 + wm * 32 + mi * 16 + g + h * 8;
          const int c = col0 + wn * 32 + ni * 8 + tg * 2 + q;
          if (r >= u.m || c >= u.n) continue;
          const float v = tot[mi][ni][h * 2 + q];
          const int64_t o = u.c_off + (int64_t)r * u.ldc + c;
          if (bufs.out64[u.c_buf]) {
            double* C = bufs.out64[u.c_buf] + o;
            *C = u.beta_one ? (*C + (double)v) : (double)v;
          } else {
            float x = v;
#pragma unroll
            for (int s = 0; s < NS; ++s) {
              const __nv_bfloat16 b = __float2bfloat16(x);
              bufs.out16[u.c_buf][s][o] = b;
              x -= __bfloat162float(b);
            }
          }
        }
}

cudaError_t launch_gemm_split(int ns, const SplitBufs& bufs, const GemmUnit* units, const GemmItem* items,
                              const GemmTask* tasks, int ntasks, cudaStream_t s) {
  if (ntasks <= 0) return cudaSuccess;
  if (ns == 2) gemm_split_kernel<2><<<ntasks, NT, 0, s>>>(bufs, units, items, tasks);
  else if (ns == 3) gemm_split_kernel<3><<<ntasks, NT, 0, s>>>(bufs, units, items, tasks);
  else return cudaErrorInvalidValue;
  return cudaGetLastError();
}

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
