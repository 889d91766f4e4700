// Device-resident Davidson iteration: the O(n) passes and the scalar
// decisions of Linear::block_davidson (linear.C:179-385) as a fixed launch
// sequence steered by a DavCtl record in device memory.
//
// Reductions are deterministic: every pass-1 block writes its partial sums
// in a fixed order (warp shuffles, then warps in index order) and one pass-2
// block adds the kDavBlocks partials in block order.
#include "k_dav.cuh"
#include "kernels.cuh"

namespace bgpu {
namespace dev {
namespace {

constexpr int kNT = 256;  // threads of the streaming kernels
constexpr int kWarps = kNT / 32;

// Partial sums acc[0..NV) of this block to work[blockIdx.x * kDavMax + i].
template <int NV>
__device__ __forceinline__ void store_partials(const double (&acc)[NV], double* __restrict__ work) {
  __shared__ double part[kWarps][NV];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    double v = acc[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) part[warp][i] = v;
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    double s = 0.0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) s += part[w][threadIdx.x];
    work[(int64_t)blockIdx.x * kDavMax + threadIdx.x] = s;
  }
}

__global__ void dav_sum(const double* __restrict__ work, double* __restrict__ out, int count) {
  const int i = threadIdx.x;
  if (i >= count) return;
  double s = 0.0;
  for (int b = 0; b < kDavBlocks; ++b) s += work[(int64_t)b * kDavMax + i];
  out[i] = s;
}

__device__ __forceinline__ int64_t first_t() { return (int64_t)blockIdx.x * blockDim.x + threadIdx.x; }
__device__ __forceinline__ int64_t stride_t() { return (int64_t)gridDim.x * blockDim.x; }

// S[k-1] = y and row[j] = b_{k-1} . s_j (j < k), the products in the order of
// DotProduct(b_i, sigma_j) of the subspace matrix (linear.C:268-272)
__global__ void __launch_bounds__(kNT, 2) dav_row_p1(DavBufs b) {
  const int k = b.ctl->k;
  const int64_t n = b.n;
  const double* __restrict__ bk = b.B + (int64_t)(k - 1) * n;
  double* __restrict__ sk = b.S + (int64_t)(k - 1) * n;
  double acc[kDavMax];
#pragma unroll
  for (int j = 0; j < kDavMax; ++j) acc[j] = 0.0;
  for (int64_t t = first_t(); t < n; t += stride_t()) {
    const double bt = bk[t], yt = b.y[t];
    sk[t] = yt;
#pragma unroll
    for (int j = 0; j < kDavMax; ++j) {
      if (j < k - 1) acc[j] = fma(b.S[(int64_t)j * n + t], bt, acc[j]);
      else if (j == k - 1) acc[j] = fma(yt, bt, acc[j]);
    }
  }
  store_partials<kDavMax>(acc, b.work);
}

// Subspace matrix of this iteration (leading dimension k): after a Ritz
// rotation the basis diagonalises the projected H, so the old block is
// diag(lam) and only the row of the newest vector is new (mode 1); the first
// iteration brings the whole matrix (mode 2).
__global__ void dav_assemble(DavCtl* c) {
  const int k = c->k, mode = c->mode;
  if (mode == 2) return;
  for (int e = threadIdx.x; e < k * k; e += blockDim.x) {
    const int i = e / k, j = e % k;
    double v = (i == j) ? c->lam[i] : 0.0;
    if (mode == 1) {
      if (i == k - 1) v = c->row[j];
      else if (j == k - 1) v = c->row[i];
    }
    c->h[e] = v;
  }
}

// Ritz rotation in place: X_r <- sum_i alpha[i k + r] X_i for r < k, for the
// basis and the sigma vectors (each thread owns whole columns)
__global__ void __launch_bounds__(kNT) dav_rotate(DavBufs b) {
  __shared__ double al[kDavMax * kDavMax];
  const int k = b.ctl->k;
  for (int e = threadIdx.x; e < k * k; e += blockDim.x) al[e] = b.ctl->alpha[e];
  __syncthreads();
  const int64_t n = b.n;
  for (int64_t t = first_t(); t < n; t += stride_t()) {
    for (int which = 0; which < 2; ++which) {
      double* __restrict__ X = which ? b.S : b.B;
      double x[kDavMax];
#pragma unroll
      for (int i = 0; i < kDavMax; ++i)
        if (i < k) x[i] = X[(int64_t)i * n + t];
      for (int r = 0; r < k; ++r) {
        double s = 0.0;
#pragma unroll
        for (int i = 0; i < kDavMax; ++i)
          if (i < k) s = fma(al[i * k + r], x[i], s);
        X[(int64_t)r * n + t] = s;
      }
    }
  }
}

// squared residual norms |s_i - w_i b_i|^2 of the first roots
__global__ void __launch_bounds__(kNT, 2) dav_resnorm_p1(DavBufs b) {
  const int k = b.ctl->k;
  const int nr = min(b.nroots, k);
  const int64_t n = b.n;
  double acc[kDavMax];
#pragma unroll
  for (int i = 0; i < kDavMax; ++i) acc[i] = 0.0;
  for (int64_t t = first_t(); t < n; t += stride_t()) {
#pragma unroll
    for (int i = 0; i < kDavMax; ++i)
      if (i < nr) {
        const double rt = fma(-b.ctl->w[i], b.B[(int64_t)i * n + t], b.S[(int64_t)i * n + t]);
        acc[i] = fma(rt, rt, acc[i]);
      }
  }
  store_partials<kDavMax>(acc, b.work);
}

// Ritz values; the lowest root whose residual grew back above tol is
// reopened (linear.C:296-306)
__global__ void dav_decide_root(DavBufs b) {
  if (threadIdx.x != 0) return;
  DavCtl* c = b.ctl;
  for (int i = 0; i < c->k; ++i) c->lam[i] = c->w[i];
  if (c->eps > 0.0) {  // the rotation X_r <- sum_i alpha[i k + r] X_i of dav_rotate
    const int k = c->k;
    double nb[kDavMax];
    for (int r = 0; r < k; ++r) {
      double s = 0.0;
      for (int i = 0; i < k; ++i) s += fabs(c->alpha[i * k + r]) * c->eb[i];
      nb[r] = s;
    }
    for (int r = 0; r < k; ++r) c->eb[r] = nb[r];
  }
  int conv = c->conv;
  for (int i = 0; i < conv; ++i)
    if (c->rn[i] > b.tol) {
      conv = i;
      break;
    }
  c->conv = conv;
  c->rnorm = c->rn[conv];
}

// r = s_c - lam_c b_c, and the two Olsen products c0 . r and b_c . c0 with
// c0 = b_c / (lam_c - diag) (linear.C:27-60)
__global__ void __launch_bounds__(kNT) dav_resid_p1(DavBufs b) {
  const DavCtl* c = b.ctl;
  const int64_t n = b.n;
  double acc[2] = {0.0, 0.0};
  if (!(c->rnorm < b.tol)) {
    const int cv = c->conv;
    const double lam = c->lam[cv];
    const double* __restrict__ bc = b.B + (int64_t)cv * n;
    const double* __restrict__ sc = b.S + (int64_t)cv * n;
    for (int64_t t = first_t(); t < n; t += stride_t()) {
      const double bt = bc[t];
      const double rt = fma(-lam, bt, sc[t]);
      b.r[t] = rt;
      double c0 = bt;
      const double den = lam - b.d[t];
      if (fabs(den) > 1e-12) c0 /= den;
      acc[0] = fma(c0, rt, acc[0]);
      acc[1] = fma(bt, c0, acc[1]);
    }
  }
  store_partials<2>(acc, b.work);
}

// r <- (r - (c0.r / b.c0) b_c) / (lam_c - diag)
__global__ void __launch_bounds__(kNT) dav_olsen(DavBufs b) {
  const DavCtl* c = b.ctl;
  if (c->rnorm < b.tol) return;
  const int cv = c->conv;
  const double lam = c->lam[cv];
  const double a = -c->olsen[0] / c->olsen[1];
  const double* __restrict__ bc = b.B + (int64_t)cv * b.n;
  for (int64_t t = first_t(); t < b.n; t += stride_t()) {
    double rt = fma(a, bc[t], b.r[t]);
    const double den = lam - b.d[t];
    if (fabs(den) > 1e-12) rt /= den;
    b.r[t] = rt;
  }
}

// convergence of root conv, or expansion with deflation (linear.C:315-345)
__global__ void dav_decide_expand(DavBufs b) {
  if (threadIdx.x != 0) return;
  DavCtl* c = b.ctl;
  if (c->rnorm < b.tol) {
    ++c->conv;
    c->expand = 0;
    if (c->conv >= b.nroots) c->done = 1;
  } else {
    c->expand = 1;
    if (c->k >= b.dmax) c->k = b.dmin;
  }
  ++c->iter;
}

// Gram-Schmidt coefficients b_i . r (i < k)
__global__ void __launch_bounds__(kNT, 2) dav_gs_p1(DavBufs b) {
  const int k = b.ctl->k;
  const bool on = b.ctl->expand != 0;
  const int64_t n = b.n;
  double acc[kDavMax];
#pragma unroll
  for (int i = 0; i < kDavMax; ++i) acc[i] = 0.0;
  if (on)
    for (int64_t t = first_t(); t < n; t += stride_t()) {
      const double rt = b.r[t];
#pragma unroll
      for (int i = 0; i < kDavMax; ++i)
        if (i < k) acc[i] = fma(b.B[(int64_t)i * n + t], rt, acc[i]);
    }
  store_partials<kDavMax>(acc, b.work);
}

// r -= sum_i coef_i b_i
__global__ void __launch_bounds__(kNT) dav_project(DavBufs b) {
  __shared__ double cf[kDavMax];
  if (!b.ctl->expand) return;
  const int k = b.ctl->k;
  if (threadIdx.x < kDavMax) cf[threadIdx.x] = threadIdx.x < k ? b.ctl->coef[threadIdx.x] : 0.0;
  __syncthreads();
  const int64_t n = b.n;
  for (int64_t t = first_t(); t < n; t += stride_t()) {
    double s = 0.0;
    for (int i = 0; i < k; ++i) s = fma(cf[i], b.B[(int64_t)i * n + t], s);
    b.r[t] -= s;
  }
}

__global__ void __launch_bounds__(kNT) dav_norm_p1(DavBufs b) {
  double acc[1] = {0.0};
  if (b.ctl->expand)
    for (int64_t t = first_t(); t < b.n; t += stride_t()) acc[0] = fma(b.r[t], b.r[t], acc[0]);
  store_partials<1>(acc, b.work);
}

// r /= |r|, appended as basis vector k
__global__ void __launch_bounds__(kNT) dav_append(DavBufs b) {
  const DavCtl* c = b.ctl;
  if (!c->expand) return;
  const double a = 1.0 / sqrt(c->nrm);
  double* __restrict__ bk = b.B + (int64_t)c->k * b.n;
  for (int64_t t = first_t(); t < b.n; t += stride_t()) {
    const double v = b.r[t] * a;
    b.r[t] = v;
    bk[t] = v;
  }
}

__global__ void dav_finish(DavCtl* c) {
  if (threadIdx.x != 0) return;
  if (c->expand) {
    c->eb[c->k] = c->eps;
    ++c->k;
  }
  c->mode = c->expand ? 1 : 0;
}

}  // namespace

cudaError_t launch_dav_new_row(const DavBufs& b, cudaStream_t s) {
  dav_row_p1<<<kDavBlocks, kNT, 0, s>>>(b);
  dav_sum<<<1, kDavMax, 0, s>>>(b.work, b.ctl->row, kDavMax);
  return cudaGetLastError();
}

cudaError_t launch_dav_update(const DavBufs& b, cudaStream_t s) {
  if (b.nroots < 1 || b.nroots > kDavMax || b.dmax > kDavMax - 1 || b.dmin < b.nroots) return cudaErrorInvalidValue;
  DavCtl* c = b.ctl;
  dav_assemble<<<1, 1024, 0, s>>>(c);
  cudaError_t e = launch_jacobi(c->h, &c->zero, &c->k, c->w, &c->zero, c->alpha, &c->zero, &c->status, 1, kDavMax, s);
  if (e != cudaSuccess) return e;
  dav_rotate<<<kDavBlocks * 2, kNT, 0, s>>>(b);
  dav_resnorm_p1<<<kDavBlocks, kNT, 0, s>>>(b);
  dav_sum<<<1, kDavMax, 0, s>>>(b.work, c->rn, kDavMax);
  dav_decide_root<<<1, 32, 0, s>>>(b);
  dav_resid_p1<<<kDavBlocks, kNT, 0, s>>>(b);
  dav_sum<<<1, kDavMax, 0, s>>>(b.work, c->olsen, 2);
  dav_olsen<<<kDavBlocks * 2, kNT, 0, s>>>(b);
  dav_decide_expand<<<1, 32, 0, s>>>(b);
  // classical Gram-Schmidt twice against the whole basis
  for (int pass = 0; pass < 2; ++pass) {
    dav_gs_p1<<<kDavBlocks, kNT, 0, s>>>(b);
    dav_sum<<<1, kDavMax, 0, s>>>(b.work, c->coef, kDavMax);
    dav_project<<<kDavBlocks * 2, kNT, 0, s>>>(b);
  }
  dav_norm_p1<<<kDavBlocks, kNT, 0, s>>>(b);
  dav_sum<<<1, kDavMax, 0, s>>>(b.work, &c->nrm, 1);
  dav_append<<<kDavBlocks * 2, kNT, 0, s>>>(b);
  dav_finish<<<1, 32, 0, s>>>(c);
  return cudaGetLastError();
}

}  // namespace dev
}  // namespace bgpu
