// Device work descriptors and kernel entry points of the sweep engine.
//
// All hot-path arithmetic of the engine is expressed as a few work-list
// kernels whose lists are compiled on the host once per block step:
//   * grouped sum-of-products GEMM: every output rectangle ("unit") owns a
//     list of products alpha * op(A) * op(B) accumulated in registers and
//     written once (deterministic, no atomics).  Used for the two stages of
//     sigma = H psi, the density matrix and the U^T O U renormalisation.
//   * build gather: every rectangle of an enlarged-block operator sums
//     scaled copies of sub-block operator blocks (the Kronecker products of
//     TensorProduct with one single-site factor).
//   * batched Jacobi eigensolver, deterministic reductions, BLAS-1.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace bgpu {
namespace dev {

constexpr int kMaxBufs = 8;

struct Bufs {
  double* p[kMaxBufs];
};

// alpha * op(A) * op(B); A is m x k and B is k x n after op()
struct GemmItem {
  int64_t a_off, b_off;
  int32_t lda, ldb, k;
  uint8_t ta, tb, a_buf, b_buf;
  double alpha;
};

// C (m x n, row-major, ldc) = beta * C + sum of items [ibeg, iend)
struct GemmUnit {
  int64_t c_off;
  int32_t ldc, m, n;
  int32_t ibeg, iend;
  uint8_t c_buf;
  uint8_t beta_one;  // 1: accumulate into C, 0: overwrite
  uint16_t pad;
};

struct GemmTask {
  int32_t unit;
  int32_t tm, tn;  // tile indices
};

// dst rectangle (m x n at c_off, ldc) = sum of items [ibeg, iend)
struct CopyUnit {
  int64_t c_off;
  int32_t ldc, m, n;
  int32_t ibeg, iend;
};
// alpha * src (m x n); src_buf < 0 -> identity matrix
struct CopyItem {
  int64_t s_off;
  int32_t lds;
  int8_t trans;
  int8_t s_buf;
  int16_t pad;
  double alpha;
};

// diagonal contributions: d[off + i*cols + j] += alpha * a[i] * b[j]
struct DiagUnit {
  int64_t d_off;
  int32_t rows, cols;
  int32_t ibeg, iend;
};
struct DiagItem {
  int64_t a_off, b_off;  // <0: identity
  int32_t a_stride, b_stride;
  int8_t a_buf, b_buf;
  int16_t pad;
  double alpha;
};

// launch helpers (return cudaGetLastError())
cudaError_t launch_gemm(const Bufs& bufs, const GemmUnit* units, const GemmItem* items, const GemmTask* tasks,
                        int ntasks, cudaStream_t s);
cudaError_t launch_copy(const Bufs& bufs, double* dst, const CopyUnit* units, const CopyItem* items, int nunits,
                        cudaStream_t s);
// d[off + i*cols + j] += sum over the unit's items, by 64 x 64 tiles of the
// units (task.unit, task.tm, task.tn), the items as the K dimension of a GEMM
cudaError_t launch_diag_tiles(const Bufs& bufs, double* d, const DiagUnit* units, const DiagItem* items,
                              const GemmTask* tasks, int ntasks, cudaStream_t s);

// out[i*ny + j] = sum_t x_i[t] * y_j[t] for i < nx, j < ny, vectors stored
// row-wise with stride ld; deterministic two-pass reduction using `work`
// (at least kGramBlocks * nx * ny doubles).
constexpr int kGramBlocks = 304;
cudaError_t launch_gram(const double* X, int nx, const double* Y, int ny, int64_t n, int64_t ld, double* work,
                        double* out, cudaStream_t s);
cudaError_t launch_axpy(double a, const double* x, double* y, int64_t n, cudaStream_t s);
cudaError_t launch_scale(double a, double* x, int64_t n, cudaStream_t s);
cudaError_t launch_fill(double* x, double v, int64_t n, cudaStream_t s);

// Batched symmetric eigensolver: matrices A_b (n_b x n_b, row-major at
// a_off[b]) are overwritten; eigenvalues (ascending) to w at w_off[b],
// eigenvectors (columns) to V at v_off[b].  One thread block per matrix,
// parallel cyclic Jacobi with a round-robin pairing.  `status[b]` receives
// the number of sweeps, or -1 if the sweep limit was reached.
cudaError_t launch_jacobi(double* A, const int64_t* a_off, const int* dims, double* w, const int64_t* w_off, double* V,
                          const int64_t* v_off, int* status, int nmat, int max_n, cudaStream_t s);

// U columns gathered from eigenvector matrices: for each (sector) entry,
// U[u_off + r*m + c] = V[v_off + r*n + col[c_off + c]] (eigenvectors as
// columns of a row-major matrix), or V[v_off + col[c_off + c]*n + r] when
// colmajor is set
struct GatherUnit {
  int64_t u_off, v_off;
  int32_t n, m, c_off, colmajor;
};
cudaError_t launch_gather_cols(const double* V, double* U, const GatherUnit* units, const int* cols, int nunits,
                               cudaStream_t s);

}  // namespace dev
}  // namespace bgpu
