// Batched dense symmetric eigensolver (FP64) for the density-matrix sectors
// and the C ABI's diagonalise: the reference diagonalises every sector with
// LAPACK DSYEV (diagonalise, MatrixBLAS.C:381-414, called from
// diagonalise_dm, rotationmat.C:258-279), i.e. Householder reduction to
// tridiagonal form followed by the implicit QL/QR iteration with the
// accumulated rotations.  This is the same family of algorithm, laid out
// for the GPU:
//   1. Householder tridiagonalisation, two launches per column step for all
//      sectors at once: a per-sector "house" kernel forms the reflector of
//      column k from a lazily corrected copy of that column, and a tiled
//      "update" kernel applies the previous step's rank-2 update to the lower
//      triangle of the trailing matrix and, in the same pass, forms the
//      partial products A v_k of the next step (fixed-order reductions, no
//      atomics: results are bit-reproducible).
//   2. Divide and conquer on the tridiagonal matrix (k_dc.cuh): leaves of at
//      most 32 rows by the implicit QL iteration in one warp, merges by the
//      secular equation with one warp per root and the eigenvector update as
//      one grouped FP64 GEMM per level for all sectors.  (The QL iteration on
//      a whole sector is a chain of O(n^2) dependent rotations in one thread,
//      bound by FP64 latency; the merges are parallel across the GPU.)
//   3. Back-transformation V = Q Z by the reflectors in reverse order, one
//      warp per eigenvector held in shared memory, and the eigenpairs
//      written in ascending eigenvalue order.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace bgpu {
namespace dev {

constexpr int kEigTile = 64;     // tile edge of the tridiagonalisation update
constexpr int kEigBtCols = 8;    // eigenvectors per back-transformation CTA
constexpr int kEigMaxN = 4096;   // largest sector (shared-memory bound of the merges and back-transformation)

// One symmetric matrix of the batch.  All offsets are in doubles.
struct EigJob {
  int64_t a_off;  // input, n x n row-major (only the lower triangle is read); overwritten
  int64_t z_off;  // output eigenvectors, n x n column-major, ascending eigenvalues
  int64_t w_off;  // output eigenvalues, ascending
  int64_t v_off;  // work: reflectors, n x n (row k = v_k)
  int64_t q_off;  // work: Z, eigenvectors of the tridiagonal matrix, n x n column-major
  int64_t s_off;  // work: d, e, tau, unsorted eigenvalues, w (2 n), partial products (2 nt n)
  int32_t n, nt;  // order, tiles per edge
  int32_t tile0;  // first CTA of this job in the update launch
  int32_t bt0;    // first CTA of this job in the back-transformation launch
};
// eigenvectors per back-transformation CTA for a batch whose largest order is max_n
inline int eig_bt_cols(int max_n) { return max_n > 2048 ? kEigBtCols / 2 : kEigBtCols; }
// doubles of the per-job scalar work area
inline int64_t eig_scalar_elems(int n) {
  const int64_t nt = (n + kEigTile - 1) / kEigTile;
  return 6ll * n + 2ll * nt * n;
}

// Bufs: p[0] = A (inputs, overwritten), p[1] = Z (outputs), p[2] = w
// (outputs), p[3] = work.  status[j] < 0: the tridiagonal solver of job j
// did not converge (-1 a leaf's QL iteration, -2 a secular equation).
// Stream-ordered; `jobs` is a device array.  The host runs
// launch_eig_tridiag, the divide and conquer of k_dc.cuh on the work area's
// d, e (unsorted eigenvalues and Z out), then launch_eig_backtransform.
struct EigBufs {
  double* a;
  double* z;
  double* w;
  double* work;
  int* status;
};
cudaError_t launch_eig_tridiag(const EigBufs& b, const EigJob* jobs, int njobs, int max_n, int tiles,
                               cudaStream_t s);
// Eigenvector signs made canonical: in matrix q (order dims[q] at V +
// off[q], eigenvectors as columns, column-major when colmajor[q] else
// row-major) every eigenvector's largest component (the first of equal
// ones) positive.  Bases chosen from eigenvectors are then the same on every
// engine up to rotations inside degenerate eigenspaces.
cudaError_t launch_canon_signs(double* V, const int64_t* off, const int* dims, const int* colmajor, int nmat,
                               cudaStream_t s);
cudaError_t launch_eig_backtransform(const EigBufs& b, const EigJob* jobs, int njobs, int max_n, int bt_ctas,
                                     cudaStream_t s);

}  // namespace dev
}  // namespace bgpu
