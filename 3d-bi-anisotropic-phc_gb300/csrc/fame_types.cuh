// Complex arithmetic, compile-time loops and compile-time twiddle factors
// shared by every kernel of the FAME GB300 library.
//
// Complex values are stored interleaved (re, im) as float2 / double2, the
// layout of MATLAB's interleaved-complex arrays, so one element is one 8- or
// 16-byte vector access.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <type_traits>
#include <utility>

#define FAME_HD __host__ __device__ __forceinline__

namespace fame {

template <class R> struct cx_of;
template <> struct cx_of<float> { using type = float2; };
template <> struct cx_of<double> { using type = double2; };
template <class R> using cx = typename cx_of<R>::type;

template <class R> FAME_HD cx<R> mk(R a, R b) { cx<R> z; z.x = a; z.y = b; return z; }
template <class R> FAME_HD cx<R> zero() { return mk<R>(R(0), R(0)); }
template <class V> FAME_HD V cadd(V a, V b) { a.x += b.x; a.y += b.y; return a; }
template <class V> FAME_HD V csub(V a, V b) { a.x -= b.x; a.y -= b.y; return a; }
template <class V> FAME_HD V cneg(V a) { a.x = -a.x; a.y = -a.y; return a; }
template <class V> FAME_HD V cconj(V a) { a.y = -a.y; return a; }
template <class V> FAME_HD V cmul(V a, V b) {
  V z; z.x = a.x * b.x - a.y * b.y; z.y = a.x * b.y + a.y * b.x; return z;
}
// conj(a) * b
template <class V> FAME_HD V cmulc(V a, V b) {
  V z; z.x = a.x * b.x + a.y * b.y; z.y = a.x * b.y - a.y * b.x; return z;
}
template <class V, class R> FAME_HD V cscale(V a, R s) { a.x *= s; a.y *= s; return a; }
// a + b*c
template <class V> FAME_HD V cfma(V b, V c, V a) {
  a.x += b.x * c.x - b.y * c.y; a.y += b.x * c.y + b.y * c.x; return a;
}
// a + conj(b)*c
template <class V> FAME_HD V cfmac(V b, V c, V a) {
  a.x += b.x * c.x + b.y * c.y; a.y += b.x * c.y - b.y * c.x; return a;
}
// multiply by +i (s>0) or -i (s<0)
template <int S, class V> FAME_HD V cmul_i(V a) {
  V z;
  if (S > 0) { z.x = -a.y; z.y = a.x; } else { z.x = a.y; z.y = -a.x; }
  return z;
}
template <class V> FAME_HD double cabs2d(V a) { return double(a.x) * a.x + double(a.y) * a.y; }

template <class D, class S> FAME_HD cx<D> cvt(S a) { return mk<D>(D(a.x), D(a.y)); }

// ---------------------------------------------------------------------------
// Compile-time loop: f(std::integral_constant<int, I>) for I in [B, E).
// ---------------------------------------------------------------------------
template <int B, int E, class F> FAME_HD void static_for(F&& f) {
  if constexpr (B < E) {
    f(std::integral_constant<int, B>{});
    static_for<B + 1, E>(f);
  }
}

// ---------------------------------------------------------------------------
// Compile-time cos / sin of 2*pi*m/n.
//
// Exact integer reduction to the nearest quarter turn, then Taylor series of
// sin and cos on |x| <= pi/4 (terms through x^29, far below one ulp of a
// double).  Evaluated by the compiler only: every call site binds the result
// to a constexpr variable.
// ---------------------------------------------------------------------------
constexpr double kPi = 3.141592653589793238462643383279502884;

FAME_HD constexpr double taylor_sin(double x) {
  double x2 = x * x, term = x, sum = x;
  for (int k = 1; k < 16; ++k) {
    term *= -x2 / double((2 * k) * (2 * k + 1));
    sum += term;
  }
  return sum;
}
FAME_HD constexpr double taylor_cos(double x) {
  double x2 = x * x, term = 1.0, sum = 1.0;
  for (int k = 1; k < 16; ++k) {
    term *= -x2 / double((2 * k - 1) * (2 * k));
    sum += term;
  }
  return sum;
}
// returns cos (which == 0) or sin (which == 1) of 2*pi*m/n
FAME_HD constexpr double cs2pi(long long m, long long n, int which) {
  m %= n;
  if (m < 0) m += n;
  // 4m/n = q + r/n with |r| <= n/2
  long long four_m = 4 * m;
  long long q = (four_m + n / 2) / n;
  long long r = four_m - q * n;
  double th = (kPi / 2.0) * double(r) / double(n);
  double c = taylor_cos(th), s = taylor_sin(th);
  int quad = int(q % 4);
  double cc = quad == 0 ? c : quad == 1 ? -s : quad == 2 ? -c : s;
  double ss = quad == 0 ? s : quad == 1 ? c : quad == 2 ? -s : -c;
  return which == 0 ? cc : ss;
}

}  // namespace fame
