// Host-side check of the compile-time register FFT (fft_reg.cuh) against a
// direct DFT for every compiled grid size, both directions.  Prints one line
// per size with the relative max error; built and run by test_fft_host.py.
#include "fft_reg.cuh"
#include <cstdio>
#include <cmath>
using namespace fame;
template <int N, int S> double check() {
  double2 x[N], y[N];
  for (int i = 0; i < N; ++i) { x[i].x = std::sin(1.3 * i + 0.2); x[i].y = std::cos(0.7 * i * i + 0.1); y[i] = x[i]; }
  fft<double, N, S>(y);
  double err = 0, nrm = 0;
  for (int k = 0; k < N; ++k) {
    double re = 0, im = 0;
    for (int n = 0; n < N; ++n) {
      double a = S * 2 * M_PI * double((long long)n * k % N) / N;
      re += x[n].x * std::cos(a) - x[n].y * std::sin(a);
      im += x[n].x * std::sin(a) + x[n].y * std::cos(a);
    }
    err = std::fmax(err, std::hypot(re - y[k].x, im - y[k].y));
    nrm = std::fmax(nrm, std::hypot(re, im));
  }
  return err / nrm;
}
#define C(N) printf("N=%d fwd %.2e inv %.2e\n", N, check<N, -1>(), check<N, +1>());
int main() { C(4) C(6) C(8) C(10) C(12) C(16) C(18) C(20) C(24) C(30) C(32) C(36) C(40) C(48) C(50) C(60) C(64) return 0; }
