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

void jacobi_eig_herm(const std::vector<std::complex<double>>& H, int n, std::vector<double>& w,
                     std::vector<std::complex<double>>& V) {
  using cd = std::complex<double>;
  std::vector<cd> A(H);
  V.assign((size_t)n * n, cd(0.0));
  for (int i = 0; i < n; ++i) V[(size_t)i * n + i] = 1.0;
  auto a = [&](int i, int j) -> cd& { return A[(size_t)i * n + j]; };
  for (int i = 0; i < n; ++i) a(i, i) = cd(a(i, i).real(), 0.0);
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, diag = 0.0;
    for (int i = 0; i < n; ++i) {
      diag += std::norm(a(i, i));
      for (int j = i + 1; j < n; ++j) off += std::norm(a(i, j));
    }
    if (off <= 1e-34 * diag || off == 0.0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const cd apq = a(p, q);
        const double r = std::abs(apq);
        if (r == 0.0) continue;
        const cd eph = apq / r;  // e^{i phi}
        const cd emph = std::conj(eph);
        const double app = a(p, p).real(), aqq = a(q, q).real();
        const double theta = (aqq - app) / (2.0 * r);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        // G on (p,q): column p = (c, -s e^{-i phi}), column q = (s, c e^{-i phi});  A <- G^H A G
        for (int k = 0; k < n; ++k) {
          const cd akp = a(k, p), akq = a(k, q);
          a(k, p) = c * akp - s * emph * akq;
          a(k, q) = s * akp + c * emph * akq;
        }
        for (int k = 0; k < n; ++k) {
          const cd apk = a(p, k), aqk = a(q, k);
          a(p, k) = c * apk - s * eph * aqk;
          a(q, k) = s * apk + c * eph * aqk;
        }
        a(p, q) = 0.0;
        a(q, p) = 0.0;
        a(p, p) = cd(a(p, p).real(), 0.0);
        a(q, q) = cd(a(q, q).real(), 0.0);
        for (int k = 0; k < n; ++k) {
          cd& vkp = V[(size_t)p * n + k];
          cd& vkq = V[(size_t)q * n + k];
          const cd x = vkp, y = vkq;
          vkp = c * x - s * emph * y;
          vkq = s * x + c * emph * y;
        }
      }
  }
  w.resize(n);
  for (int i = 0; i < n; ++i) w[i] = a(i, i).real();
}

bool herm_pencil_eig(const std::vector<std::complex<double>>& L, const std::vector<std::complex<double>>& M, int n,
                     std::vector<double>& mu, std::vector<std::complex<double>>& Y) {
  using cd = std::complex<double>;
  // M = R^H R, R upper triangular (row-major)
  std::vector<cd> R((size_t)n * n, cd(0.0));
  for (int j = 0; j < n; ++j) {
    double d = M[(size_t)j * n + j].real();
    for (int k = 0; k < j; ++k) d -= std::norm(R[(size_t)k * n + j]);
    if (!(d > 0.0)) return false;
    const double rjj = std::sqrt(d);
    R[(size_t)j * n + j] = rjj;
    for (int i = j + 1; i < n; ++i) {
      cd s = M[(size_t)j * n + i];
      for (int k = 0; k < j; ++k) s -= std::conj(R[(size_t)k * n + j]) * R[(size_t)k * n + i];
      R[(size_t)j * n + i] = s / rjj;
    }
  }
  // Rinv (upper triangular)
  std::vector<cd> Ri((size_t)n * n, cd(0.0));
  for (int j = 0; j < n; ++j) {
    Ri[(size_t)j * n + j] = 1.0 / R[(size_t)j * n + j];
    for (int i = j - 1; i >= 0; --i) {
      cd s = 0.0;
      for (int k = i + 1; k <= j; ++k) s += R[(size_t)i * n + k] * Ri[(size_t)k * n + j];
      Ri[(size_t)i * n + j] = -s / R[(size_t)i * n + i];
    }
  }
  // C = Ri^H L Ri
  std::vector<cd> T((size_t)n * n, cd(0.0)), C((size_t)n * n, cd(0.0));
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      cd s = 0.0;
      for (int k = 0; k <= j; ++k) s += L[(size_t)i * n + k] * Ri[(size_t)k * n + j];
      T[(size_t)i * n + j] = s;
    }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      cd s = 0.0;
      for (int k = 0; k <= i; ++k) s += std::conj(Ri[(size_t)k * n + i]) * T[(size_t)k * n + j];
      C[(size_t)i * n + j] = s;
    }
  for (int i = 0; i < n; ++i)  // enforce Hermitian symmetry
    for (int j = i + 1; j < n; ++j) {
      cd h = 0.5 * (C[(size_t)i * n + j] + std::conj(C[(size_t)j * n + i]));
      C[(size_t)i * n + j] = h;
      C[(size_t)j * n + i] = std::conj(h);
    }
  std::vector<cd> Z;
  jacobi_eig_herm(C, n, mu, Z);
  Y.assign((size_t)n * n, cd(0.0));
  for (int c2 = 0; c2 < n; ++c2)
    for (int i = 0; i < n; ++i) {
      cd s = 0.0;
      for (int k = i; k < n; ++k) s += Ri[(size_t)i * n + k] * Z[(size_t)c2 * n + k];
      Y[(size_t)c2 * n + i] = s;
    }
  return true;
}

}  // namespace fame
