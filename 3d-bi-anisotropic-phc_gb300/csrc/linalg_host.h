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

// Eigen-decomposition of a complex Hermitian n x n matrix (row-major H):
// complex Jacobi rotations (a phase makes each pivot real, then a real
// rotation zeroes it).  w[n] eigenvalues, V column-major (column j at V[j*n]).
void jacobi_eig_herm(const std::vector<std::complex<double>>& H, int n, std::vector<double>& w,
                     std::vector<std::complex<double>>& V);

// Hermitian-definite pencil  L y = mu M y  (M positive definite): Cholesky of M
// and the Hermitian eigenproblem of R^-H L R^-1.  Y column-major, M-orthonormal.
// Returns false if M is not positive definite.
bool herm_pencil_eig(const std::vector<std::complex<double>>& L, const std::vector<std::complex<double>>& M, int n,
                     std::vector<double>& mu, std::vector<std::complex<double>>& Y);

}  // namespace fame
