// Work-list kernels of the sweep engine (descriptors in kernels.cuh).
#include <cfloat>
#include <cmath>

#include "kernels.cuh"

namespace bgpu {
namespace dev {

// ------------------------------------------------------------------------
// Grouped FP64 sum-of-products GEMM.  64x64 output tile per 256-thread
// block, 4x4 register tile per thread, K staged through shared memory in
// slabs of 16.  Each task (unit, tile) is computed entirely by one block, so
// results are bit-reproducible and independent of scheduling.
// Restates the two MatrixMultiply calls of TensorMultiply
// (operatorfunctions.C:515,530), MultiplyProduct (operatorfunctions.C:646)
// and MatrixRotate (MatrixBLAS.C:553-572) as batched row-major DGEMM.
// ------------------------------------------------------------------------
namespace {
constexpr int TM = 64, TN = 64, TK = 16, NT = 256;

__device__ __forceinline__ double ld_op(const double* __restrict__ p, int64_t ld, bool t, int r, int c) {
  return t ? p[(int64_t)c * ld + r] : p[(int64_t)r * ld + c];
}
}  // namespace

__global__ void __launch_bounds__(NT) gemm_fp64_kernel(Bufs bufs, const GemmUnit* __restrict__ units,
                                                       const GemmItem* __restrict__ items,
                                                       const GemmTask* __restrict__ tasks) {
  __shared__ double As[TK][TM + 1];
  __shared__ double Bs[TK][TN + 1];
  const GemmTask task = tasks[blockIdx.x];
  const GemmUnit u = units[task.unit];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int row0 = task.tm * TM, col0 = task.tn * TN;
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
  for (int it = u.ibeg; it < u.iend; ++it) {
    const GemmItem g = items[it];
    const double* __restrict__ A = bufs.p[g.a_buf] + g.a_off;
    const double* __restrict__ B = bufs.p[g.b_buf] + g.b_off;
    for (int k0 = 0; k0 < g.k; k0 += TK) {
      // A tile: TM x TK of op(A)
#pragma unroll
      for (int r = 0; r < (TM * TK) / NT; ++r) {
        const int e = tid + r * NT;
        int i, p;
        if (g.ta) { i = e % TM; p = e / TM; }
        else { i = e / TK; p = e % TK; }
        const int gi = row0 + i, gp = k0 + p;
        As[p][i] = (gi < u.m && gp < g.k) ? g.alpha * ld_op(A, g.lda, g.ta, gi, gp) : 0.0;
      }
      // B tile: TK x TN of op(B)
#pragma unroll
      for (int r = 0; r < (TK * TN) / NT; ++r) {
        const int e = tid + r * NT;
        int p, j;
        if (g.tb) { p = e % TK; j = e / TK; }
        else { p = e / TN; j = e % TN; }
        const int gp = k0 + p, gj = col0 + j;
        Bs[p][j] = (gp < g.k && gj < u.n) ? ld_op(B, g.ldb, g.tb, gp, gj) : 0.0;
      }
      __syncthreads();
#pragma unroll
      for (int p = 0; p < TK; ++p) {
        double a[4], b[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) a[i] = As[p][ty * 4 + i];
#pragma unroll
        for (int j = 0; j < 4; ++j) b[j] = Bs[p][tx * 4 + j];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
      }
      __syncthreads();
    }
  }
  double* C = bufs.p[u.c_buf] + u.c_off;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gi = row0 + ty * 4 + i;
    if (gi >= u.m) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gj = col0 + tx * 4 + j;
      if (gj >= u.n) continue;
      double* c = C + (int64_t)gi * u.ldc + gj;
      *c = u.beta_one ? (*c + acc[i][j]) : acc[i][j];
    }
  }
}

cudaError_t launch_gemm(const Bufs& bufs, const GemmUnit* units, const GemmItem* items, const GemmTask* tasks,
                        int ntasks, cudaStream_t s) {
  if (ntasks <= 0) return cudaSuccess;
  gemm_fp64_kernel<<<ntasks, NT, 0, s>>>(bufs, units, items, tasks);
  return cudaGetLastError();
}

// ------------------------------------------------------------------------
// Build gather: dst rectangle = sum of scaled (possibly transposed or
// identity) source blocks.  One block per rectangle, every element written
// once.  This is TensorProductElement with the FAST_MTP single-site factor
// (operatorfunctions.C:167-254, MatrixBLAS.C:138-162) over all terms of an
// operator's build() at once.
// ------------------------------------------------------------------------
__global__ void __launch_bounds__(256) copy_kernel(Bufs bufs, double* __restrict__ dst,
                                                   const CopyUnit* __restrict__ units,
                                                   const CopyItem* __restrict__ items) {
  const CopyUnit u = units[blockIdx.x];
  const int64_t total = (int64_t)u.m * u.n;
  for (int64_t e = threadIdx.x; e < total; e += blockDim.x) {
    const int i = (int)(e / u.n), j = (int)(e % u.n);
    double s = 0.0;
    for (int it = u.ibeg; it < u.iend; ++it) {
      const CopyItem c = items[it];
      double x;
      if (c.s_buf < 0) x = (i == j) ? 1.0 : 0.0;
      else {
        const double* src = bufs.p[c.s_buf] + c.s_off;
        x = c.trans ? src[(int64_t)j * c.lds + i] : src[(int64_t)i * c.lds + j];
      }
      s = fma(c.alpha, x, s);
    }
    dst[u.c_off + (int64_t)i * u.ldc + j] = s;
  }
}

cudaError_t launch_copy(const Bufs& bufs, double* dst, const CopyUnit* units, const CopyItem* items, int nunits,
                        cudaStream_t s) {
  if (nunits <= 0) return cudaSuccess;
  copy_kernel<<<nunits, 256, 0, s>>>(bufs, dst, units, items);
  return cudaGetLastError();
}

// Diagonal of the superblock Hamiltonian (diagonal TensorProduct /
// TensorTrace, operatorfunctions.C:653-762).
// Same sums as a GEMM: over a 64 x 64 tile of a sector, d(i, j) +=
// sum_t (alpha_t a_t[i]) b_t[j] with the items t as the K dimension, 16
// items at a time gathered into shared memory (the diagonals of the
// operator blocks are strided reads), 4 x 4 outputs per thread.
__global__ void __launch_bounds__(NT) diag_tile_kernel(Bufs bufs, double* __restrict__ d,
                                                       const DiagUnit* __restrict__ units,
                                                       const DiagItem* __restrict__ items,
                                                       const GemmTask* __restrict__ tasks) {
  __shared__ double As[TK][TM + 1];
  __shared__ double Bs[TK][TN + 1];
  const GemmTask task = tasks[blockIdx.x];
  const DiagUnit u = units[task.unit];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int row0 = task.tm * TM, col0 = task.tn * TN;
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
  for (int it0 = u.ibeg; it0 < u.iend; it0 += TK) {
#pragma unroll
    for (int r = 0; r < (TM * TK) / NT; ++r) {
      const int e = tid + r * NT;
      const int p = e / TM, i = e % TM;
      const int it = it0 + p;
      double va = 0.0, vb = 0.0;
      if (it < u.iend) {
        const DiagItem c = items[it];
        if (row0 + i < u.rows)
          va = c.alpha * (c.a_off < 0 ? 1.0 : bufs.p[c.a_buf][c.a_off + (int64_t)(row0 + i) * c.a_stride]);
        if (col0 + i < u.cols) vb = c.b_off < 0 ? 1.0 : bufs.p[c.b_buf][c.b_off + (int64_t)(col0 + i) * c.b_stride];
      }
      As[p][i] = va;
      Bs[p][i] = vb;
    }
    __syncthreads();
#pragma unroll
    for (int p = 0; p < TK; ++p) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[p][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[p][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gi = row0 + ty * 4 + i;
    if (gi >= u.rows) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gj = col0 + tx * 4 + j;
      if (gj >= u.cols) continue;
      d[u.d_off + (int64_t)gi * u.cols + gj] += acc[i][j];
    }
  }
}

cudaError_t launch_diag_tiles(const Bufs& bufs, double* d, const DiagUnit* units, const DiagItem* items,
                              const GemmTask* tasks, int ntasks, cudaStream_t s) {
  if (ntasks <= 0) return cudaSuccess;
  diag_tile_kernel<<<ntasks, NT, 0, s>>>(bufs, d, units, items, tasks);
  return cudaGetLastError();
}


// ------------------------------------------------------------------------
// Deterministic reductions and BLAS-1 over the flat wavefunction arena
// (DotProduct / ScaleAdd / Scale, BaseOperator.C:240-288).
// ------------------------------------------------------------------------
constexpr int kMaxGram = 32;

__global__ void __launch_bounds__(256) gram_pass1(const double* __restrict__ X, int nx, const double* __restrict__ y,
                                                  int64_t n, int64_t ld, double* __restrict__ work) {
  __shared__ double red[256];
  double acc[kMaxGram];
#pragma unroll
  for (int i = 0; i < kMaxGram; ++i) acc[i] = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride) {
    const double yt = y[t];
#pragma unroll
    for (int i = 0; i < kMaxGram; ++i)
      if (i < nx) acc[i] = fma(X[(int64_t)i * ld + t], yt, acc[i]);
  }
  for (int i = 0; i < nx; ++i) {
    red[threadIdx.x] = acc[i];
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
      if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) work[(int64_t)blockIdx.x * nx + i] = red[0];
    __syncthreads();
  }
}

__global__ void gram_pass2(const double* __restrict__ work, int nblocks, int nx, double* __restrict__ out) {
  const int i = threadIdx.x;
  if (i >= nx) return;
  double s = 0.0;
  for (int b = 0; b < nblocks; ++b) s += work[(int64_t)b * nx + i];
  out[i] = s;
}

cudaError_t launch_gram(const double* X, int nx, const double* Y, int ny, int64_t n, int64_t ld, double* work,
                        double* out, cudaStream_t s) {
  if (nx > kMaxGram) return cudaErrorInvalidValue;
  for (int j = 0; j < ny; ++j) {
    gram_pass1<<<kGramBlocks, 256, 0, s>>>(X, nx, Y + (int64_t)j * ld, n, ld, work);
    gram_pass2<<<1, kMaxGram, 0, s>>>(work, kGramBlocks, nx, out + (int64_t)j * nx);
  }
  return cudaGetLastError();
}

__global__ void axpy_kernel(double a, const double* __restrict__ x, double* __restrict__ y, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride) y[t] = fma(a, x[t], y[t]);
}
__global__ void scale_kernel(double a, double* __restrict__ x, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride) x[t] *= a;
}
__global__ void fill_kernel(double* __restrict__ x, double v, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride) x[t] = v;
}

static int blocks_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  if (b < 1) b = 1;
  return (int)b;
}

cudaError_t launch_axpy(double a, const double* x, double* y, int64_t n, cudaStream_t s) {
  axpy_kernel<<<blocks_for(n), 256, 0, s>>>(a, x, y, n);
  return cudaGetLastError();
}
cudaError_t launch_scale(double a, double* x, int64_t n, cudaStream_t s) {
  scale_kernel<<<blocks_for(n), 256, 0, s>>>(a, x, n);
  return cudaGetLastError();
}
cudaError_t launch_fill(double* x, double v, int64_t n, cudaStream_t s) {
  fill_kernel<<<blocks_for(n), 256, 0, s>>>(x, v, n);
  return cudaGetLastError();
}

// ------------------------------------------------------------------------
// Batched parallel cyclic Jacobi (Brent-Luk style round-robin ordering):
// every round applies n/2 disjoint rotations, each annihilating one
// off-diagonal pair, as A <- J^T A J; V accumulates the rotations.  Used for
// the per-sector density-matrix eigenproblems (diagonalise_dm,
// rotationmat.C:258-279) and the Davidson subspace matrix (linear.C:273).
// ------------------------------------------------------------------------
__device__ __forceinline__ int rr_player(int pos, int round, int m) {
  return pos == 0 ? 0 : ((pos - 1 + round) % (m - 1)) + 1;
}

__global__ void __launch_bounds__(512) jacobi_kernel(double* A, const int64_t* __restrict__ a_off,
                                                     const int* __restrict__ dims, double* w,
                                                     const int64_t* __restrict__ w_off, double* V,
                                                     const int64_t* __restrict__ v_off, int* status) {
  extern __shared__ double sm[];
  const int b = blockIdx.x;
  const int n = dims[b];
  if (n <= 0) {
    if (threadIdx.x == 0) status[b] = 0;
    return;
  }
  double* a = A + a_off[b];
  double* v = V + v_off[b];
  const int m = n + (n & 1);
  const int npair = m / 2;
  double* cs = sm;               // npair
  double* sn = sm + npair;       // npair
  int* pp = (int*)(sm + 2 * npair);
  int* qq = pp + npair;
  __shared__ double red[512];
  __shared__ int done;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int64_t e = tid; e < (int64_t)n * n; e += nt) v[e] = ((e / n) == (e % n)) ? 1.0 : 0.0;
  __syncthreads();
  int sweeps = -1;
  for (int sweep = 0; sweep < 60; ++sweep) {
    // off-diagonal and total norms
    double off = 0.0, tot = 0.0;
    for (int64_t e = tid; e < (int64_t)n * n; e += nt) {
      const double x = a[e];
      tot += x * x;
      if ((e / n) != (e % n)) off += x * x;
    }
    red[tid] = off;
    __syncthreads();
    for (int s2 = nt / 2; s2 > 0; s2 >>= 1) {
      if (tid < s2) red[tid] += red[tid + s2];
      __syncthreads();
    }
    const double offsum = red[0];
    __syncthreads();
    red[tid] = tot;
    __syncthreads();
    for (int s2 = nt / 2; s2 > 0; s2 >>= 1) {
      if (tid < s2) red[tid] += red[tid + s2];
      __syncthreads();
    }
    const double totsum = red[0];
    if (tid == 0) done = (offsum <= 1e-30 * totsum) || (totsum == 0.0);
    __syncthreads();
    if (done) {
      sweeps = sweep;
      break;
    }
    for (int round = 0; round < m - 1; ++round) {
      for (int k = tid; k < npair; k += nt) {
        int p = rr_player(k, round, m), q = rr_player(m - 1 - k, round, m);
        if (p > q) { const int t = p; p = q; q = t; }
        double c = 1.0, s = 0.0;
        if (q < n) {
          const double apq = a[(int64_t)p * n + q];
          if (fabs(apq) > 1e-300) {
            const double app = a[(int64_t)p * n + p], aqq = a[(int64_t)q * n + q];
            const double theta = (aqq - app) / (2.0 * apq);
            const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
            c = 1.0 / sqrt(t * t + 1.0);
            s = t * c;
          }
        } else {
          q = p;  // dummy partner
        }
        cs[k] = c;
        sn[k] = s;
        pp[k] = p;
        qq[k] = q;
      }
      __syncthreads();
      // columns: A <- A J
      for (int64_t e = tid; e < (int64_t)n * npair; e += nt) {
        const int k = (int)(e % npair), i = (int)(e / npair);
        const int p = pp[k], q = qq[k];
        if (p == q || sn[k] == 0.0) continue;
        const double c = cs[k], s = sn[k];
        const double aip = a[(int64_t)i * n + p], aiq = a[(int64_t)i * n + q];
        a[(int64_t)i * n + p] = c * aip - s * aiq;
        a[(int64_t)i * n + q] = s * aip + c * aiq;
      }
      __syncthreads();
      // rows: A <- J^T A
      for (int64_t e = tid; e < (int64_t)n * npair; e += nt) {
        const int j = (int)(e % n), k = (int)(e / n);
        const int p = pp[k], q = qq[k];
        if (p == q || sn[k] == 0.0) continue;
        const double c = cs[k], s = sn[k];
        const double apj = a[(int64_t)p * n + j], aqj = a[(int64_t)q * n + j];
        a[(int64_t)p * n + j] = c * apj - s * aqj;
        a[(int64_t)q * n + j] = s * apj + c * aqj;
      }
      __syncthreads();
      for (int k = tid; k < npair; k += nt) {
        const int p = pp[k], q = qq[k];
        if (p != q && sn[k] != 0.0) {
          a[(int64_t)p * n + q] = 0.0;
          a[(int64_t)q * n + p] = 0.0;
        }
      }
      // V <- V J
      for (int64_t e = tid; e < (int64_t)n * npair; e += nt) {
        const int k = (int)(e % npair), i = (int)(e / npair);
        const int p = pp[k], q = qq[k];
        if (p == q || sn[k] == 0.0) continue;
        const double c = cs[k], s = sn[k];
        const double vip = v[(int64_t)i * n + p], viq = v[(int64_t)i * n + q];
        v[(int64_t)i * n + p] = c * vip - s * viq;
        v[(int64_t)i * n + q] = s * vip + c * viq;
      }
      __syncthreads();
    }
  }
  // sort ascending (rank by value, ties by index); A is reused as scratch
  double* wout = w + w_off[b];
  for (int i = tid; i < n; i += nt) wout[i] = a[(int64_t)i * n + i];
  __syncthreads();
  for (int64_t e = tid; e < (int64_t)n * n; e += nt) a[e] = v[e];
  __syncthreads();
  for (int i = tid; i < n; i += nt) {
    const double wi = wout[i];
    int r = 0;
    for (int j = 0; j < n; ++j) {
      const double wj = wout[j];
      if (wj < wi || (wj == wi && j < i)) ++r;
    }
    for (int row = 0; row < n; ++row) v[(int64_t)row * n + r] = a[(int64_t)row * n + i];
  }
  __syncthreads();
  for (int i = tid; i < n; i += nt) {
    const double wi = wout[i];
    int r = 0;
    for (int j = 0; j < n; ++j) {
      const double wj = wout[j];
      if (wj < wi || (wj == wi && j < i)) ++r;
    }
    a[r] = wi;
  }
  __syncthreads();
  for (int i = tid; i < n; i += nt) wout[i] = a[i];
  if (tid == 0) status[b] = sweeps;
}

cudaError_t launch_jacobi(double* A, const int64_t* a_off, const int* dims, double* w, const int64_t* w_off, double* V,
                          const int64_t* v_off, int* status, int nmat, int max_n, cudaStream_t s) {
  if (nmat <= 0) return cudaSuccess;
  const int m = max_n + (max_n & 1);
  const size_t smem = (size_t)(m / 2) * (2 * sizeof(double) + 2 * sizeof(int)) + 16;
  if (smem > 200 * 1024) return cudaErrorInvalidValue;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(jacobi_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  jacobi_kernel<<<nmat, 512, smem, s>>>(A, a_off, dims, w, w_off, V, v_off, status);
  return cudaGetLastError();
}

__global__ void gather_cols_kernel(const double* __restrict__ V, double* __restrict__ U,
                                   const GatherUnit* __restrict__ units, const int* __restrict__ cols) {
  const GatherUnit u = units[blockIdx.x];
  const int64_t total = (int64_t)u.n * u.m;
  for (int64_t e = threadIdx.x; e < total; e += blockDim.x) {
    const int r = (int)(e / u.m), c = (int)(e % u.m);
    const int64_t col = cols[u.c_off + c];
    U[u.u_off + e] = u.colmajor ? V[u.v_off + col * u.n + r] : V[u.v_off + (int64_t)r * u.n + col];
  }
}

cudaError_t launch_gather_cols(const double* V, double* U, const GatherUnit* units, const int* cols, int nunits,
                               cudaStream_t s) {
  if (nunits <= 0) return cudaSuccess;
  gather_cols_kernel<<<nunits, 256, 0, s>>>(V, U, units, cols);
  return cudaGetLastError();
}

}  // namespace dev
}  // namespace bgpu
