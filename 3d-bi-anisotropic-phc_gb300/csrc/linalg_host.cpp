#include "linalg_host.h"

#include <cmath>
#include <utility>

namespace fame {

bool invert_complex(const std::complex<double>* A, std::complex<double>* Ainv, int n) {
  std::vector<std::complex<double>> M(A, A + n * n);
  for (int i = 0; i < n * n; ++i) Ainv[i] = 0.0;
  for (int i = 0; i < n; ++i) Ainv[i * n + i] = 1.0;
  for (int c = 0; c < n; ++c) {
    int piv = c;
    double best = std::abs(M[c * n + c]);
    for (int r = c + 1; r < n; ++r)
      if (std::abs(M[r * n + c]) > best) {
        best = std::abs(M[r * n + c]);
        piv = r;
      }
    if (!(best > 0.0)) return false;
    if (piv != c)
      for (int j = 0; j < n; ++j) {
        std::swap(M[c * n + j], M[piv * n + j]);
        std::swap(Ainv[c * n + j], Ainv[piv * n + j]);
      }
    const std::complex<double> inv = 1.0 / M[c * n + c];
    for (int j = 0; j < n; ++j) {
      M[c * n + j] *= inv;
      Ainv[c * n + j] *= inv;
    }
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      const std::complex<double> f = M[r * n + c];
      if (f == 0.0) continue;
      for (int j = 0; j < n; ++j) {
        M[r * n + j] -= f * M[c * n + j];
        Ainv[r * n + j] -= f * Ainv[c * n + j];
      }
    }
  }
  return true;
}

void jacobi_eig(const std::vector<double>& H, int n, std::vector<double>& w, std::vector<double>& V) {
  std::vector<double> A(H);
  V.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) V[(size_t)i * n + i] = 1.0;
  auto a = [&](int i, int j) -> double& { return A[(size_t)i * n + j]; };
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, diag = 0.0;
    for (int i = 0; i < n; ++i) {
      diag += a(i, i) * a(i, i);
      for (int j = i + 1; j < n; ++j) off += a(i, j) * a(i, j);
    }
    if (off <= 1e-34 * diag || off == 0.0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = a(p, q);
        if (apq == 0.0) continue;
        const double app = a(p, p), aqq = a(q, q);
        // rotation zeroing a(p,q): tan(2 phi) = 2 apq / (aqq - app)
        const double theta = (aqq - app) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {
          const double akp = a(k, p), akq = a(k, q);
          a(k, p) = c * akp - s * akq;
          a(k, q) = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          const double apk = a(p, k), aqk = a(q, k);
          a(p, k) = c * apk - s * aqk;
          a(q, k) = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          double& vkp = V[(size_t)p * n + k];
          double& vkq = V[(size_t)q * n + k];
          const double x = vkp, y = vkq;
          vkp = c * x - s * y;
          vkq = s * x + c * y;
        }
      }
  }
  w.resize(n);
  for (int i = 0; i < n; ++i) w[i] = a(i, i);
}

}  // namespace fame
