// Host-side check of the double-single (float-float) type of fame_types.cuh:
// its additions and products against long double on random operands, and
// the compile-time register FFT instantiated with it against a direct DFT in
// long double for every compiled grid size.  Prints one line per check; built
// and run by test_ds_host.py.
#include "fft_reg.cuh"
#include <cmath>
#include <cstdio>
#include <random>
using namespace fame;

static long double ld(ff a) { return (long double)a.hi + (long double)a.lo; }

// largest relative error of ff +, -, * over random operands of mixed signs
// and magnitudes (cancellation included)
static void arith() {
  std::mt19937_64 g(7);
  std::uniform_real_distribution<double> u(-1.0, 1.0), e(-20.0, 20.0);
  long double add = 0, mul = 0;
  for (int i = 0; i < 200000; ++i) {
    const double x = u(g) * std::ldexp(1.0, (int)e(g)), y = u(g) * std::ldexp(1.0, (int)e(g));
    const ff a(x), b(i % 7 == 0 ? -x * (1 + 1e-9 * u(g)) : y);  // some near-cancelling sums
    const long double la = ld(a), lb = ld(b);
    const long double s = la + lb, p = la * lb;
    if (s != 0) add = std::fmax(add, std::fabs((ld(a + b) - s) / s) / std::ldexp(1.0L, -47));
    if (p != 0) mul = std::fmax(mul, std::fabs((ld(a * b) - p) / p) / std::ldexp(1.0L, -47));
  }
  // in units of 2^-47 (about two units of the pair's last place)
  printf("arith add %.3Lf mul %.3Lf\n", add, mul);
}

template <int N, int S> double check() {
  cx<ff> y[N];
  long double xr[N], xi[N];
  for (int i = 0; i < N; ++i) {
    const double a = std::sin(1.3 * i + 0.2), b = std::cos(0.7 * i * i + 0.1);
    y[i].x = ff(a);
    y[i].y = ff(b);
    xr[i] = a;
    xi[i] = b;
  }
  fft<ff, N, S>(y);
  long double err = 0, nrm = 0;
  for (int k = 0; k < N; ++k) {
    long double re = 0, im = 0;
    for (int n = 0; n < N; ++n) {
      const long double t = S * 2 * 3.14159265358979323846264338327950288L * (long double)((long long)n * k % N) / N;
      re += xr[n] * std::cos(t) - xi[n] * std::sin(t);
      im += xr[n] * std::sin(t) + xi[n] * std::cos(t);
    }
    err = std::fmax(err, std::hypot(re - ld(y[k].x), im - ld(y[k].y)));
    nrm = std::fmax(nrm, std::hypot(re, im));
  }
  return (double)(err / nrm);
}
#define C(N) printf("N=%d fwd %.2e inv %.2e\n", N, check<N, -1>(), check<N, +1>());
int main() {
  arith();
  C(3) C(4) C(5) C(12) C(15) C(20) C(24) C(40) C(48) C(60)
  return 0;
}
