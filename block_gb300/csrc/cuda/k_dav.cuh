// Device-resident Davidson iteration (Linear::block_davidson, linear.C:179-385).
//
// Every scalar that steers the iteration (basis size, converged roots,
// Ritz values, residual norms, Olsen and Gram-Schmidt coefficients) lives in
// one DavCtl record in device memory, and every kernel reads the basis size
// from it, so one fixed launch sequence serves all iterations of a solve and
// is captured once as a CUDA graph.  The host reads the small header of the
// record once per iteration to stop the loop.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace bgpu {
namespace dev {

constexpr int kDavMax = 32;  // largest Davidson basis

struct DavCtl {
  // header, copied to the host after every iteration
  int32_t k;       // basis size
  int32_t conv;    // converged roots
  int32_t expand;  // this iteration appended a basis vector
  int32_t done;    // all roots converged
  int32_t iter;    // iterations completed
  int32_t status;  // subspace eigensolver: sweeps used, < 0 when it did not converge
  int32_t mode;    // subspace matrix of the next iteration: 0 diag(lam), 1 diag(lam) + new row, 2 full h
  int32_t pad;
  double lam[kDavMax];  // Ritz values, ascending
  double rnorm;         // squared residual norm of root `conv` (before preconditioning)
  // device-only part
  int64_t zero;               // offset 0 for the batched eigensolver
  double row[kDavMax];        // b_{k-1} . sigma_j
  double rn[kDavMax];         // squared residual norms of the first roots
  double olsen[2];            // c0 . r and b . c0
  double nrm;                 // squared norm of the new vector
  double coef[kDavMax];       // Gram-Schmidt coefficients
  double w[kDavMax];          // eigenvalues of the subspace matrix
  double h[kDavMax * kDavMax];      // subspace matrix (leading dimension k)
  double alpha[kDavMax * kDavMax];  // its eigenvectors as columns
  // Error bounds of the sigma rows: eb[i] >= |S_i - H_64 B_i| (FP64 product),
  // carried through the Ritz rotations as sum_j |alpha_ji| eb_j; a vector
  // appended while eps > 0 gets eb = eps (the bound of one split-precision
  // product of a unit vector).  eps = 0: no bookkeeping.
  double eb[kDavMax];
  double eps;
};
constexpr size_t kDavHeaderBytes = offsetof(DavCtl, zero);

// Reduction scratch: kDavBlocks * kDavMax doubles.
constexpr int kDavBlocks = 304;

// All vectors are rows of length n: B and S hold the basis and its sigma
// vectors (row stride n), r the residual / new vector, d the diagonal of H.
struct DavBufs {
  double* B;
  double* S;
  double* r;
  const double* d;
  double* y;  // sigma of the newest basis vector (written by the sigma launches)
  double* work;
  DavCtl* ctl;
  int64_t n;
  int nroots, dmin, dmax;
  double tol;
};

// S[k-1] = y; row[j] = b_{k-1} . s_j for j < k (subspace matrix row of the
// newest vector).  Enqueued only in iterations that computed a sigma.
cudaError_t launch_dav_new_row(const DavBufs& b, cudaStream_t s);
// Subspace eigenproblem, Ritz rotation of B and S, residual of the lowest
// unconverged root with the Olsen correction, convergence and deflation
// decisions, two classical Gram-Schmidt passes and the append of the new
// normalised vector to B (also left in r, the input of the next sigma).
cudaError_t launch_dav_update(const DavBufs& b, cudaStream_t s);

}  // namespace dev
}  // namespace bgpu
