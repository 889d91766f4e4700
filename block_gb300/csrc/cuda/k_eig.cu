// Batched dense symmetric eigensolver (FP64); see k_eig.cuh for the layout.
//
// Householder step k (0 <= k <= n-3) of A = A^(0), lower triangle:
//   x = A^(k)[k+1:n, k],  beta = -sign(x_0) |x|,  tau = (beta - x_0) / beta,
//   v = (0..0, 1, x_1.. / (x_0 - beta)),  p = tau A^(k) v,
//   w = p - (tau / 2)(p . v) v,  A^(k+1) = A^(k) - v w^T - w v^T
// (Golub & Van Loan, Matrix Computations, 4th ed., sections 5.1 and 8.3.1).
// The trailing update of step k-1 and the product A^(k) v_k of step k share
// one pass over the matrix: column k of A^(k) is formed lazily from the
// stored column (still A^(k-1)) and the rank-2 correction of step k-1.
//
// The tridiagonal eigenproblem is solved by divide and conquer (k_dc.cu);
// its leaves use the implicit QL iteration with the Wilkinson shift of the
// leading 2 x 2 block (Bowdler, Martin, Reinsch and Wilkinson, "The QR and
// QL algorithms for symmetric matrices", Numer. Math. 11 (1968) 293-306).
#include <cmath>

#include "k_eig.cuh"

namespace bgpu {
namespace dev {
namespace {

constexpr int kHouseThreads = 256;
constexpr int kUpdThreads = 256;
constexpr int kBtThreads = 32 * kEigBtCols;

__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// deterministic block sum (every thread gets the result)
template <int NT>
__device__ double block_sum(double x, double* red) {
  x = warp_sum(x);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = x;
  __syncthreads();
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < NT / 32; ++i) s += red[i];
  return s;
}

struct Scal {
  double *d, *e, *tau, *eu, *wr, *prow, *pcol;
};
__device__ __forceinline__ Scal scal(const EigBufs& b, const EigJob& J) {
  Scal s;
  s.d = b.work + J.s_off;
  s.e = s.d + J.n;
  s.tau = s.e + J.n;
  s.eu = s.tau + J.n;
  s.wr = s.eu + J.n;  // two vectors of n: slot (k & 1)
  s.prow = s.wr + 2 * (int64_t)J.n;
  s.pcol = s.prow + (int64_t)J.nt * J.n;
  return s;
}

// One CTA per job: reduces the partial products of step k-1 into w_{k-1},
// forms column k of A^(k) and the reflector of step k (or, at k = n-2, the
// last 2 x 2 block of the tridiagonal matrix).
__global__ void __launch_bounds__(kHouseThreads) eig_house(EigBufs b, const EigJob* __restrict__ jobs, int k) {
  __shared__ double red[kHouseThreads / 32];
  const EigJob J = jobs[blockIdx.x];
  const int n = J.n, tid = threadIdx.x;
  const Scal S = scal(b, J);
  const double* __restrict__ A = b.a + J.a_off;
  double* __restrict__ V = b.work + J.v_off;
  if (n == 1) {
    if (k == 0 && tid == 0) {
      S.d[0] = A[0];
      S.e[0] = 0.0;
    }
    return;
  }
  if (k > n - 2) return;
  const double* vp = V + (int64_t)(k >= 1 ? k - 1 : 0) * n;  // v_{k-1} (read for k >= 1)
  double* wp = S.wr + (int64_t)((k + 1) & 1) * n;            // w_{k-1}
  double* col = S.wr + (int64_t)(k & 1) * n;
  if (k >= 1) {
    const int nt = J.nt, j0 = k / kEigTile;
    const double t = S.tau[k - 1];
    double pv = 0.0;
    for (int i = k + tid; i < n; i += kHouseThreads) {
      const int ti = i / kEigTile;
      double s = 0.0;
      for (int jt = j0; jt <= ti; ++jt) s += S.prow[(int64_t)jt * n + i];
      for (int it = ti + 1; it < nt; ++it) s += S.pcol[(int64_t)it * n + i];
      s *= t;
      wp[i] = s;
      pv += s * vp[i];
    }
    const double K = 0.5 * t * block_sum<kHouseThreads>(pv, red);
    for (int i = k + tid; i < n; i += kHouseThreads) wp[i] -= K * vp[i];
    __syncthreads();
  }
  // column k of A^(k), rows k..n-1
  const double wk = k >= 1 ? wp[k] : 0.0, vk = k >= 1 ? vp[k] : 0.0;
  double ss = 0.0;
  for (int i = k + tid; i < n; i += kHouseThreads) {
    double c = A[(int64_t)i * n + k];
    if (k >= 1) c -= vp[i] * wk + wp[i] * vk;
    col[i] = c;
    if (i >= k + 2) ss += c * c;
  }
  ss = block_sum<kHouseThreads>(ss, red);  // also orders the writes of col
  if (k == n - 2) {
    if (tid == 0) {
      S.d[k] = col[k];
      S.e[k] = col[k + 1];
      double dd = A[(int64_t)(k + 1) * n + k + 1];
      if (k >= 1) dd -= 2.0 * vp[k + 1] * wp[k + 1];
      S.d[k + 1] = dd;
      S.e[k + 1] = 0.0;
      S.tau[k] = 0.0;
    }
    return;
  }
  const double alpha = col[k + 1];
  const double xn = sqrt(ss + alpha * alpha);
  double beta = 0.0, t = 0.0, scale = 0.0, lead = 0.0;
  if (xn != 0.0) {
    beta = -copysign(xn, alpha);
    t = (beta - alpha) / beta;
    scale = 1.0 / (alpha - beta);
    lead = 1.0;
  }
  double* vk_row = V + (int64_t)k * n;
  for (int i = tid; i < n; i += kHouseThreads) vk_row[i] = i <= k ? 0.0 : (i == k + 1 ? lead : col[i] * scale);
  if (tid == 0) {
    S.d[k] = col[k];
    S.e[k] = beta;
    S.tau[k] = t;
  }
}

__device__ __forceinline__ int find_job(const EigJob* jobs, int njobs, int bid, int which) {
  int j = 0;
  for (int q = 1; q < njobs; ++q) {
    const int first = which == 0 ? jobs[q].tile0 : jobs[q].bt0;
    if (first <= bid) j = q;
  }
  return j;
}

// One CTA per 64 x 64 tile (I >= J) of a job's lower triangle: applies the
// rank-2 update of step k-1 to the tile's part of rows / columns >= k+1 and
// writes the tile's partial sums of A^(k) v_k: row sums to prow[J][rows of
// I], column sums (off-diagonal tiles) to pcol[I][columns of J]; a diagonal
// tile writes the sum of both to prow[I].
__global__ void __launch_bounds__(kUpdThreads) eig_update(EigBufs b, const EigJob* __restrict__ jobs, int njobs,
                                                          int k) {
  __shared__ double vr[kEigTile], vc[kEigTile], pvr[kEigTile], pwr[kEigTile], pvc[kEigTile], pwc[kEigTile];
  __shared__ double rows[kEigTile], colred[kUpdThreads / 32][kEigTile];
  const int bid = blockIdx.x;
  const EigJob J = jobs[find_job(jobs, njobs, bid, 0)];
  const int n = J.n;
  if (k > n - 3) return;
  const int t = bid - J.tile0;
  int I = (int)((sqrt(8.0 * t + 1.0) - 1.0) * 0.5);
  while ((I + 1) * (I + 2) / 2 <= t) ++I;
  while (I * (I + 1) / 2 > t) --I;
  const int JJ = t - I * (I + 1) / 2;
  if (I >= J.nt || JJ * kEigTile + kEigTile - 1 < k + 1) return;  // no active column
  const Scal S = scal(b, J);
  double* __restrict__ A = b.a + J.a_off;
  const double* __restrict__ V = b.work + J.v_off;
  const double* v = V + (int64_t)k * n;
  const double* vp = V + (int64_t)(k >= 1 ? k - 1 : 0) * n;
  const double* wp = S.wr + (int64_t)((k + 1) & 1) * n;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int r0 = I * kEigTile, c0 = JJ * kEigTile;
  if (tid < kEigTile) {
    const int i = r0 + tid, j = c0 + tid;
    vr[tid] = i < n ? v[i] : 0.0;
    vc[tid] = j < n ? v[j] : 0.0;
    pvr[tid] = (k >= 1 && i < n) ? vp[i] : 0.0;
    pwr[tid] = (k >= 1 && i < n) ? wp[i] : 0.0;
    pvc[tid] = (k >= 1 && j < n) ? vp[j] : 0.0;
    pwc[tid] = (k >= 1 && j < n) ? wp[j] : 0.0;
  }
  __syncthreads();
  double cacc[2] = {0.0, 0.0};
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int r = warp * 8 + q, i = r0 + r;
    double racc = 0.0;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int c = lane + 32 * h, j = c0 + c;
      if (i < n && j < n && j >= k + 1 && i >= j) {
        double* pa = A + (int64_t)i * n + j;
        double a = *pa;
        if (k >= 1) {
          a -= pvr[r] * pwc[c] + pwr[r] * pvc[c];
          *pa = a;
        }
        racc += a * vc[c];
        if (i != j) cacc[h] += a * vr[r];
      }
    }
    racc = warp_sum(racc);
    if (lane == 0) rows[r] = racc;
  }
  colred[warp][lane] = cacc[0];
  colred[warp][lane + 32] = cacc[1];
  __syncthreads();
  if (tid < kEigTile) {
    double cs = 0.0;
#pragma unroll
    for (int w = 0; w < kUpdThreads / 32; ++w) cs += colred[w][tid];
    if (I == JJ) {
      if (r0 + tid < n) S.prow[(int64_t)JJ * n + r0 + tid] = rows[tid] + cs;
    } else {
      if (r0 + tid < n) S.prow[(int64_t)JJ * n + r0 + tid] = rows[tid];
      if (c0 + tid < n) S.pcol[(int64_t)I * n + c0 + tid] = cs;
    }
  }
}

// Back-transformation V = H_0 H_1 ... H_{n-3} Z, one eigenvector per warp in
// shared memory, written at the rank of its eigenvalue (ascending; ties in
// index order).
__global__ void __launch_bounds__(kBtThreads) eig_backtransform(EigBufs b, const EigJob* __restrict__ jobs,
                                                                int njobs, int ncol) {
  extern __shared__ double sm[];
  const int bid = blockIdx.x;
  const int jidx = find_job(jobs, njobs, bid, 2);
  const EigJob J = jobs[jidx];
  const int n = J.n, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const Scal S = scal(b, J);
  const double* __restrict__ V = b.work + J.v_off;
  const double* __restrict__ Q = b.work + J.q_off;
  double* vs = sm;
  double* zc = sm + n + (int64_t)warp * n;
  const int j = (bid - J.bt0) * ncol + warp;
  const bool mine = warp < ncol && j < n;
  if (mine)
    for (int i = lane; i < n; i += 32) zc[i] = Q[(int64_t)j * n + i];
  for (int k = n - 3; k >= 0; --k) {
    __syncthreads();
    for (int i = k + 1 + tid; i < n; i += kBtThreads) vs[i] = V[(int64_t)k * n + i];
    __syncthreads();
    if (mine) {
      double dot = 0.0;
      for (int i = k + 1 + lane; i < n; i += 32) dot += vs[i] * zc[i];
      dot = warp_sum(dot) * S.tau[k];
      for (int i = k + 1 + lane; i < n; i += 32) zc[i] -= dot * vs[i];
    }
  }
  if (!mine) return;
  const double lam = S.eu[j];
  int rank = 0;
  for (int i = lane; i < n; i += 32) {
    const double x = S.eu[i];
    rank += (x < lam || (x == lam && i < j)) ? 1 : 0;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) rank += __shfl_xor_sync(0xffffffffu, rank, o);
  __syncwarp();
  double* out = b.z + J.z_off + (int64_t)rank * n;
  for (int i = lane; i < n; i += 32) out[i] = zc[i];
  if (lane == 0) b.w[J.w_off + rank] = lam;
}

}  // namespace

// One CTA per matrix, one warp per eigenvector: the vector's largest
// component (the first of equal ones) made positive.
__global__ void __launch_bounds__(256) canon_signs_kernel(double* V, const int64_t* __restrict__ off,
                                                          const int* __restrict__ dims, const int* __restrict__ colmajor) {
  const int q = blockIdx.x, n = dims[q];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double* v = V + off[q];
  const bool cm = colmajor[q] != 0;
  for (int j = warp; j < n; j += 8) {
    double best = -1.0, val = 0.0;
    int bi = n;
    for (int i = lane; i < n; i += 32) {
      const double x = cm ? v[(int64_t)j * n + i] : v[(int64_t)i * n + j];
      if (fabs(x) > best) {
        best = fabs(x);
        bi = i;
        val = x;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double b2 = __shfl_xor_sync(0xffffffffu, best, o);
      const int i2 = __shfl_xor_sync(0xffffffffu, bi, o);
      const double v2 = __shfl_xor_sync(0xffffffffu, val, o);
      if (b2 > best || (b2 == best && i2 < bi)) {
        best = b2;
        bi = i2;
        val = v2;
      }
    }
    if (val < 0.0)
      for (int i = lane; i < n; i += 32) {
        double& x = cm ? v[(int64_t)j * n + i] : v[(int64_t)i * n + j];
        x = -x;
      }
  }
}

cudaError_t launch_canon_signs(double* V, const int64_t* off, const int* dims, const int* colmajor, int nmat,
                               cudaStream_t s) {
  if (nmat > 0) canon_signs_kernel<<<nmat, 256, 0, s>>>(V, off, dims, colmajor);
  return cudaGetLastError();
}

cudaError_t launch_eig_tridiag(const EigBufs& b, const EigJob* jobs, int njobs, int max_n, int tiles,
                               cudaStream_t s) {
  if (njobs <= 0) return cudaSuccess;
  if (max_n < 1 || max_n > kEigMaxN) return cudaErrorInvalidValue;
  for (int k = 0; k <= max_n - 2 || k == 0; ++k) {
    eig_house<<<njobs, kHouseThreads, 0, s>>>(b, jobs, k);
    if (k <= max_n - 3 && tiles > 0) eig_update<<<tiles, kUpdThreads, 0, s>>>(b, jobs, njobs, k);
    if (max_n < 2) break;
  }
  return cudaGetLastError();
}

cudaError_t launch_eig_backtransform(const EigBufs& b, const EigJob* jobs, int njobs, int max_n, int bt_ctas,
                                     cudaStream_t s) {
  if (njobs <= 0) return cudaSuccess;
  if (max_n < 1 || max_n > kEigMaxN) return cudaErrorInvalidValue;
  const int bt_cols = eig_bt_cols(max_n);
  const size_t smem_bt = (size_t)(1 + bt_cols) * max_n * sizeof(double);
  cudaError_t e = cudaFuncSetAttribute(eig_backtransform, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bt);
  if (e != cudaSuccess) return e;
  eig_backtransform<<<bt_ctas, kBtThreads, smem_bt, s>>>(b, jobs, njobs, bt_cols);
  return cudaGetLastError();
}

}  // namespace dev
}  // namespace bgpu
