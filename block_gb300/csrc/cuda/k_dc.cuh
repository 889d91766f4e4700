// Divide and conquer for the symmetric tridiagonal eigenproblem of the
// batched eigensolver (k_eig.cuh): the reduced matrix T of every job is torn
// into leaves of at most kDcLeaf rows, each leaf is solved by the implicit QL
// iteration in one warp, and the leaves are merged pairwise, level by level
// (J. J. M. Cuppen, "A divide and conquer method for the symmetric
// tridiagonal eigenproblem", Numer. Math. 36 (1981) 177-195; deflation as in
// J. J. Dongarra and D. C. Sorensen, SIAM J. Sci. Stat. Comput. 8 (1987)
// s139-s154; eigenvectors from the recomputed weights of M. Gu and
// S. C. Eisenstat, SIAM J. Matrix Anal. Appl. 16 (1995) 172-191; secular
// equation steps with the two-pole rational model of J. R. Bunch,
// C. P. Nielsen and D. C. Sorensen, Numer. Math. 31 (1978) 31-48).
//
// A merge of the blocks T1 = T[o, o+n1) and T2 = T[o+n1, o+nm) joined by
// beta = T(o+n1-1, o+n1) works on T = diag(T1', T2') + |beta| v v^T, v =
// e_{o+n1-1} + sign(beta) e_{o+n1}, where T1' and T2' have |beta| taken off
// their touching diagonal elements (the tear, applied to d before the
// leaves are solved).  With T1' = Q1 L1 Q1^T and T2' = Q2 L2 Q2^T,
// T = Q (L + rho z z^T) Q^T with Q = diag(Q1, Q2), z = Q^T v / |Q^T v| and
// rho = |beta| |Q^T v|^2.  Each level is:
//   deflate  (one CTA per merge): sort L, deflate tiny rho |z_i| and close
//            pairs (Givens rotations of the columns of Q), leaving K poles;
//   secular  (one warp per root): lambda_j = d_o + tau_j, o the nearer pole;
//   zhat     (one warp per pole): Loewner weights from the computed roots;
//   vectors  (one warp per root): U column j = zhat / (d - lambda_j), normed;
//   gather   (one CTA per column): G = the block's columns, kept ones first;
//   GEMM     (the grouped FP64 GEMM): Q columns [0, K) = G[:, 0:K) U;
//   finish   (one CTA per column): deflated columns and eigenvalues.
// Eigenvalues land in the job's unsorted-eigenvalue vector and eigenvectors
// as the columns of its Z work matrix (column-major), in any order.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "k_eig.cuh"

namespace bgpu {
namespace dev {

constexpr int kDcLeaf = 32;  // largest leaf (one warp)

struct DcLeaf {
  int32_t job, o, len, pad;
};

// A merge of [o, o+n1) and [o+n1, o+nm) of job `job`; its nm slots start at
// x_off in the level arrays, its U (K x K column-major) at u_off and its G
// (nm x nm column-major) at g_off of the level scratch.
struct DcMerge {
  int32_t job, o, n1, nm;
  int64_t x_off, u_off, g_off;
};

struct DcLevel {
  const DcMerge* merges;
  int nmerges;
  int64_t nslots;
  int* K;          // per merge: poles left after deflation
  int* nrot;       // per merge: deflating rotations
  double* rho;     // per merge
  double* dk;      // per slot: poles (sorted) then deflated eigenvalues
  double* zk;      // per slot: z of the poles
  int* col;        // per slot: block column of the pole / deflated value
  double* tau;     // per slot: root offset from its origin pole
  int* org;        // per slot: origin pole of the root
  double* zhat;    // per slot
  int2* rot_cols;  // per slot: columns (p, q) of rotation t
  double2* rot_cs; // per slot: (c, s) of rotation t
  double* U;
  double* G;
};

// d -= |beta| on both sides of every merge's tear (all levels at once)
cudaError_t launch_dc_tear(double* work, const EigJob* jobs, const DcMerge* merges, int nmerges, cudaStream_t s);
// leaves: eigenvalues into the unsorted-eigenvalue vector, eigenvectors into
// the leaf's diagonal block of Z (the rest of Z must be zero)
cudaError_t launch_dc_leaves(double* work, const EigJob* jobs, const DcLeaf* leaves, int nleaves, int* status,
                             cudaStream_t s);
// one level, up to the GEMM (after which the host reads K)
cudaError_t launch_dc_deflate(double* work, const EigJob* jobs, const DcLevel& L, int max_nm, cudaStream_t s);
cudaError_t launch_dc_roots(double* work, const EigJob* jobs, const DcLevel& L, int* status, cudaStream_t s);
// deflated columns and eigenvalues (after the GEMM)
cudaError_t launch_dc_finish(double* work, const EigJob* jobs, const DcLevel& L, cudaStream_t s);

}  // namespace dev
}  // namespace bgpu
