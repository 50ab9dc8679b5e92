// Small dense host linear algebra: complex inversion for the 6x6
// constitutive blocks and a cyclic Jacobi eigensolver for the p x p
// projected Lanczos matrices (p <= 64).
#pragma once

#include <complex>
#include <vector>

namespace fame {

// Gauss-Jordan with partial pivoting; returns false if singular.
bool invert_complex(const std::complex<double>* A, std::complex<double>* Ainv, int n);

// Eigen-decomposition of a real symmetric n x n matrix (row-major H).
// w[n] eigenvalues (unsorted), V[n*n] column-major eigenvectors: column j is
// V[j*n .. j*n+n).  Cyclic Jacobi sweeps until the off-diagonal mass is below
// round-off.
void jacobi_eig(const std::vector<double>& H, int n, std::vector<double>& w, std::vector<double>& V);

}  // namespace fame
