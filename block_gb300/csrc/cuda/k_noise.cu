// Kernels of the density-matrix noise; see k_noise.cuh.
#include "../host/noise_rng.h"
#include "k_noise.cuh"

namespace bgpu {
namespace dev {
namespace {

constexpr int kNT = 256;

__device__ double block_reduce(double x) {
  __shared__ double red[kNT / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = x;
  __syncthreads();
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < kNT / 32; ++i) s += red[i];
  return s;
}

__global__ void __launch_bounds__(kNT) noise_fill_kernel(double* __restrict__ x, int64_t n, uint64_t seed, int q) {
  for (int64_t e = (int64_t)blockIdx.x * kNT + threadIdx.x; e < n; e += (int64_t)gridDim.x * kNT)
    x[e] = noise_uniform(seed, q, e);
}

__global__ void __launch_bounds__(kNT) range_norm2_kernel(const double* __restrict__ x,
                                                          const longlong2* __restrict__ ranges, double* out) {
  const longlong2 r = ranges[blockIdx.x];
  double s = 0.0;
  for (int64_t e = r.x + threadIdx.x; e < r.y; e += kNT) s += x[e] * x[e];
  s = block_reduce(s);
  if (threadIdx.x == 0) out[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kNT) range_normalise_kernel(double* __restrict__ x,
                                                              const longlong2* __restrict__ ranges,
                                                              const double* __restrict__ nrm) {
  const longlong2 r = ranges[blockIdx.x];
  const double q = nrm[blockIdx.x];
  const double a = q > 1e-15 ? 1.0 / sqrt(q) : 0.0;
  for (int64_t e = r.x + (int64_t)blockIdx.y * kNT + threadIdx.x; e < r.y; e += (int64_t)gridDim.y * kNT) x[e] *= a;
}

__global__ void __launch_bounds__(kNT) block_trace_kernel(const double* __restrict__ m,
                                                          const int64_t* __restrict__ off,
                                                          const int* __restrict__ dims, int nq, double* out) {
  double s = 0.0;
  for (int q = 0; q < nq; ++q) {
    const int n = dims[q];
    for (int i = threadIdx.x; i < n; i += kNT) s += m[off[q] + (int64_t)i * n + i];
  }
  s = block_reduce(s);
  if (threadIdx.x == 0) *out = s;
}

__global__ void __launch_bounds__(kNT) noise_update_kernel(double* __restrict__ rho, const double* __restrict__ N,
                                                           int64_t n, const double* __restrict__ tr, double amp) {
  const double t = *tr;
  if (!(t > 1.0)) return;
  const double a = amp / t;
  for (int64_t e = (int64_t)blockIdx.x * kNT + threadIdx.x; e < n; e += (int64_t)gridDim.x * kNT) rho[e] += a * N[e];
}

int grid_for(int64_t n) {
  const int64_t g = (n + kNT - 1) / kNT;
  return (int)(g < 4096 ? (g > 0 ? g : 1) : 4096);
}

}  // namespace

cudaError_t launch_noise_fill(double* x, int64_t n, uint64_t seed, int quantum, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  noise_fill_kernel<<<grid_for(n), kNT, 0, s>>>(x, n, seed, quantum);
  return cudaGetLastError();
}
cudaError_t launch_range_norm2(const double* x, const longlong2* ranges, int nranges, double* out, cudaStream_t s) {
  if (nranges <= 0) return cudaSuccess;
  range_norm2_kernel<<<nranges, kNT, 0, s>>>(x, ranges, out);
  return cudaGetLastError();
}
cudaError_t launch_range_normalise(double* x, const longlong2* ranges, int nranges, const double* nrm, cudaStream_t s) {
  if (nranges <= 0) return cudaSuccess;
  range_normalise_kernel<<<dim3(nranges, 8), kNT, 0, s>>>(x, ranges, nrm);
  return cudaGetLastError();
}
cudaError_t launch_block_trace(const double* m, const int64_t* off, const int* dims, int nq, double* out,
                               cudaStream_t s) {
  block_trace_kernel<<<1, kNT, 0, s>>>(m, off, dims, nq, out);
  return cudaGetLastError();
}
cudaError_t launch_noise_update(double* rho, const double* N, int64_t n, const double* tr, double amp, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  noise_update_kernel<<<grid_for(n), kNT, 0, s>>>(rho, N, n, tr, amp);
  return cudaGetLastError();
}

}  // namespace dev
}  // namespace bgpu
