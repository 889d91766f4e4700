// Fused two-stage split-precision sigma kernel.
//
// For one 64 x 64 tile of an output sector sigma(lQ, rQ) a thread block walks
// a contiguous range of its product list.  Each item is one TensorMultiply
// coupling (operatorfunctions.C:506-533):
//     S      = A(lQ, lQ') psi(lQ', rQ')         stage 1, 64 x n1 (n1 = n_rQ')
//     sigma += alpha S B(rQ, rQ')^T             stage 2
// S never leaves the registers: the FP32 accumulator fragments of the first
// tensor-core product are scaled, split into bf16 slices and fed directly as
// the A fragments of the second product (the m16n8 accumulator layout equals
// the m16n8k16 A-operand layout of two adjacent n8 tiles).  Items with an
// identity factor skip one of the stages.  Each block writes its FP32 partial
// tile once; a second kernel sums the partials of every tile in a fixed order
// (deterministic, no atomics).
#include <cuda_bf16.h>

#include "k_fused.cuh"

namespace bgpu {
namespace dev {

namespace {
constexpr int NT = 128;  // 4 warps x 16 rows
constexpr int KP = 24;   // smem pitch for 16-wide k slabs (bf16)
constexpr int BP = 72;   // smem pitch for 64-wide k slabs (bf16)

__device__ __forceinline__ void mma16816(float* c, const uint32_t* a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 a, __nv_bfloat16 b) {
  return (uint32_t)__bfloat16_as_ushort(a) | ((uint32_t)__bfloat16_as_ushort(b) << 16);
}

// split the pair (x, y) into NS bf16-pair slices
template <int NS>
__device__ __forceinline__ void split2(float x, float y, uint32_t* out) {
#pragma unroll
  for (int s = 0; s < NS; ++s) {
    const __nv_bfloat16 a = __float2bfloat16(x), b = __float2bfloat16(y);
    out[s] = pack2(a, b);
    x -= __bfloat162float(a);
    y -= __bfloat162float(b);
  }
}
}  // namespace

template <int NS>
__global__ void __launch_bounds__(NT) fused_sigma_kernel(FusedBufs fb, const FusedItem* __restrict__ items,
                                                         const FusedTask* __restrict__ tasks) {
  __shared__ __align__(16) __nv_bfloat16 As[NS][64][KP];
  __shared__ __align__(16) __nv_bfloat16 Cs[NS][64][KP];
  __shared__ __align__(16) __nv_bfloat16 Bs[NS][64][BP];
  const FusedTask task = tasks[blockIdx.x];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int g = lane >> 2, tg = lane & 3;
  const int row0 = task.tm * 64, col0 = task.tn * 64;
  const int wr = warp * 16;  // warp's first row inside the tile
  // tensor-core accumulation is chained only within one coupling item (V);
  // items are folded into a compensated pair (Vh + Vl) with IEEE FP32 adds
  float V[8][4], Vh[8][4], Vl[8][4];
#pragma unroll
  for (int j = 0; j < 8; ++j)
#pragma unroll
    for (int e = 0; e < 4; ++e) Vh[j][e] = Vl[j][e] = 0.f;
  for (int it = task.ibeg; it < task.iend; ++it) {
    const FusedItem I = items[it];
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
      for (int e = 0; e < 4; ++e) V[j][e] = 0.f;
    for (int n1c = 0; n1c < I.n1; n1c += 64) {
      if (I.kind == kFusedRIdent && n1c != col0) continue;
      float S[8][4];
#pragma unroll
      for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int e = 0; e < 4; ++e) S[j][e] = 0.f;
      if (I.kind == kFusedLIdent) {
        // S = psi(lQ, rQ') read straight from the FP64 wavefunction
        const double* P = fb.psi64 + I.a_off;
#pragma unroll
        for (int j = 0; j < 8; ++j)
#pragma unroll
          for (int h = 0; h < 2; ++h)
#pragma unroll
            for (int q = 0; q < 2; ++q) {
              const int r = row0 + wr + g + 8 * h, c = n1c + j * 8 + tg * 2 + q;
              S[j][h * 2 + q] = (r < task.m && c < I.n1) ? (float)P[(int64_t)r * I.lda + c] : 0.f;
            }
      } else {
        // stage 1: S = A(rows, :) psi(:, n1 chunk), K = k1 in slabs of 16
        for (int k0 = 0; k0 < I.k1; k0 += 16) {
          for (int e = tid; e < 64 * 16; e += NT) {
            int i, p;
            if (I.ta) { i = e & 63; p = e >> 6; }
            else { i = e >> 4; p = e & 15; }
            const int r = row0 + i, k = k0 + p;
            const bool in = r < task.m && k < I.k1;
            const int64_t o = I.ta ? (int64_t)k * I.lda + r : (int64_t)r * I.lda + k;
#pragma unroll
            for (int s = 0; s < NS; ++s) As[s][i][p] = in ? fb.L[s][I.a_off + o] : __float2bfloat16(0.f);
          }
          for (int e = tid; e < 64 * 16; e += NT) {
            const int j = e & 63, p = e >> 6;  // psi row k0+p, column n1c+j (row-major, contiguous in j)
            const int k = k0 + p, c = n1c + j;
            const bool in = k < I.k1 && c < I.n1;
            const int64_t o = (int64_t)k * I.ldc + c;
#pragma unroll
            for (int s = 0; s < NS; ++s) Cs[s][j][p] = in ? fb.psi[s][I.c_off + o] : __float2bfloat16(0.f);
          }
          __syncthreads();
          uint32_t a[NS][4];
#pragma unroll
          for (int s = 0; s < NS; ++s) {
            a[s][0] = *reinterpret_cast<const uint32_t*>(&As[s][wr + g][tg * 2]);
            a[s][1] = *reinterpret_cast<const uint32_t*>(&As[s][wr + g + 8][tg * 2]);
            a[s][2] = *reinterpret_cast<const uint32_t*>(&As[s][wr + g][tg * 2 + 8]);
            a[s][3] = *reinterpret_cast<const uint32_t*>(&As[s][wr + g + 8][tg * 2 + 8]);
          }
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            uint32_t b0[NS], b1[NS];
#pragma unroll
            for (int s = 0; s < NS; ++s) {
              b0[s] = *reinterpret_cast<const uint32_t*>(&Cs[s][j * 8 + g][tg * 2]);
              b1[s] = *reinterpret_cast<const uint32_t*>(&Cs[s][j * 8 + g][tg * 2 + 8]);
            }
#pragma unroll
            for (int sa = 0; sa < NS; ++sa)
#pragma unroll
              for (int sb = 0; sb < NS; ++sb)
                if (sa + sb < NS) mma16816(S[j], a[sa], b0[sb], b1[sb]);
          }
          __syncthreads();
        }
      }
      if (I.kind == kFusedRIdent) {
#pragma unroll
        for (int j = 0; j < 8; ++j)
#pragma unroll
          for (int e = 0; e < 4; ++e) V[j][e] = fmaf(I.alpha, S[j][e], V[j][e]);
        continue;
      }
      // S' = alpha S as bf16 slices in A-fragment layout (4 k16 steps)
      uint32_t Pf[NS][4][4];
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        uint32_t t[NS];
        split2<NS>(I.alpha * S[2 * kk][0], I.alpha * S[2 * kk][1], t);
#pragma unroll
        for (int s = 0; s < NS; ++s) Pf[s][kk][0] = t[s];
        split2<NS>(I.alpha * S[2 * kk][2], I.alpha * S[2 * kk][3], t);
#pragma unroll
        for (int s = 0; s < NS; ++s) Pf[s][kk][1] = t[s];
        split2<NS>(I.alpha * S[2 * kk + 1][0], I.alpha * S[2 * kk + 1][1], t);
#pragma unroll
        for (int s = 0; s < NS; ++s) Pf[s][kk][2] = t[s];
        split2<NS>(I.alpha * S[2 * kk + 1][2], I.alpha * S[2 * kk + 1][3], t);
#pragma unroll
        for (int s = 0; s < NS; ++s) Pf[s][kk][3] = t[s];
      }
      // stage 2 operand: Bs[j][p] = B_view(col0 + j, n1c + p)
      for (int e = tid; e < 64 * 64; e += NT) {
        int j, p;
        if (I.tb) { j = e & 63; p = e >> 6; }  // stored (rQ', rQ): contiguous in rQ
        else { p = e & 63; j = e >> 6; }       // stored (rQ, rQ'): contiguous in rQ'
        const int c = col0 + j, k = n1c + p;
        const bool in = c < task.n && k < I.n1;
        const int64_t o = I.tb ? (int64_t)k * I.ldb + c : (int64_t)c * I.ldb + k;
#pragma unroll
        for (int s = 0; s < NS; ++s) Bs[s][j][p] = in ? fb.R[s][I.b_off + o] : __float2bfloat16(0.f);
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < 4; ++kk)
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          uint32_t b0[NS], b1[NS];
#pragma unroll
          for (int s = 0; s < NS; ++s) {
            b0[s] = *reinterpret_cast<const uint32_t*>(&Bs[s][j * 8 + g][kk * 16 + tg * 2]);
            b1[s] = *reinterpret_cast<const uint32_t*>(&Bs[s][j * 8 + g][kk * 16 + tg * 2 + 8]);
          }
#pragma unroll
          for (int sa = 0; sa < NS; ++sa)
#pragma unroll
            for (int sb = 0; sb < NS; ++sb)
              if (sa + sb < NS) mma16816(V[j], Pf[sa][kk], b0[sb], b1[sb]);
        }
      __syncthreads();
    }
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        // TwoSum(Vh, V): Vh + Vl carries the running sum to ~2^-48
        const float a = Vh[j][e], b = V[j][e];
        const float t = __fadd_rn(a, b);
        const float bb = __fsub_rn(t, a);
        const float err = __fadd_rn(__fsub_rn(a, __fsub_rn(t, bb)), __fsub_rn(b, bb));
        Vh[j][e] = t;
        Vl[j][e] = __fadd_rn(Vl[j][e], err);
      }
  }
  // FP32 partial tile of this task (compensated pair folded)
  float* out = fb.partials + (int64_t)blockIdx.x * 4096;
#pragma unroll
  for (int j = 0; j < 8; ++j)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int r = wr + g + 8 * h, c = j * 8 + tg * 2;
      *reinterpret_cast<float2*>(out + r * 64 + c) =
          make_float2(Vh[j][h * 2] + Vl[j][h * 2], Vh[j][h * 2 + 1] + Vl[j][h * 2 + 1]);
    }
}

__global__ void fused_reduce_kernel(const float* __restrict__ partials, const FusedTile* __restrict__ tiles,
                                    double* __restrict__ sigma) {
  const FusedTile t = tiles[blockIdx.x];
  for (int e = threadIdx.x; e < 4096; e += blockDim.x) {
    const int r = e >> 6, c = e & 63;
    const int gr = t.tm * 64 + r, gc = t.tn * 64 + c;
    if (gr >= t.m || gc >= t.n) continue;
    double s = 0.0;
    for (int p = t.pbeg; p < t.pend; ++p) s += (double)partials[(int64_t)p * 4096 + e];
    sigma[t.s_off + (int64_t)gr * t.lds + gc] = s;
  }
}

cudaError_t launch_fused_sigma(int ns, const FusedBufs& fb, const FusedItem* items, const FusedTask* tasks,
                               int ntasks, cudaStream_t s) {
  if (ntasks > 0) {
    if (ns == 2) fused_sigma_kernel<2><<<ntasks, NT, 0, s>>>(fb, items, tasks);
    else if (ns == 3) fused_sigma_kernel<3><<<ntasks, NT, 0, s>>>(fb, items, tasks);
    else return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_fused_reduce(const FusedBufs& fb, const FusedTile* tiles, int ntiles, double* sigma,
                                cudaStream_t s) {
  if (ntiles > 0) fused_reduce_kernel<<<ntiles, 256, 0, s>>>(fb.partials, tiles, sigma);
  return cudaGetLastError();
}

}  // namespace dev
}  // namespace bgpu
