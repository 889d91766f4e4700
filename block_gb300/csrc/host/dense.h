// Small dense FP64 helpers used on the host: a cyclic Jacobi symmetric
// eigensolver (Davidson subspace matrices of at most a few tens of rows, the
// Fiedler Laplacian) and modified Gram-Schmidt.
#pragma once
#include <vector>

namespace bgpu {

// Symmetric eigendecomposition of the n x n row-major matrix `a`.
// On return w holds ascending eigenvalues and v (row-major n x n) holds the
// matching eigenvectors in its columns.  Cyclic Jacobi rotations
// (Jacobi 1846; threshold strategy of Rutishauser 1971).
void jacobi_eigh(int n, const double* a, double* w, double* v);

// Orthonormalise the columns of the row-major rows x cols matrix in place
// (modified Gram-Schmidt, two passes).  Returns false if a column is
// numerically dependent.
bool orthonormalise_columns(int rows, int cols, double* m);

}  // namespace bgpu
