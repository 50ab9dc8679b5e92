// Complex arithmetic, compile-time loops and compile-time twiddle factors
// shared by every kernel of the FAME GB300 library.
//
// Complex values are stored interleaved (re, im) as float2 / double2, the
// layout of MATLAB's interleaved-complex arrays, so one element is one 8- or
// 16-byte vector access.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <type_traits>
#include <utility>

#define FAME_HD __host__ __device__ __forceinline__

namespace fame {

// ---------------------------------------------------------------------------
// Double-single ("float-float") real: the unevaluated sum hi + lo of two
// floats, |lo| <= ulp(hi)/2, about 48 significant bits.  Built from the
// error-free transformations of Knuth (two-sum), Dekker (fast two-sum) and
// the FMA two-product (Hida, Li and Bailey's double-double algorithms with
// float in place of double).  On GB300 the FP32 pipes issue 64 times the
// instructions of the FP64 pipe, so an operator evaluated in this type at
// ~20 FP32 instructions per operation is faster than FP64 and as accurate to
// ~1e-14 relative.  (Needs IEEE float arithmetic without reassociation:
// these files are compiled without fast-math.)
// ---------------------------------------------------------------------------
// s + e = a + b exactly (Knuth)
FAME_HD void ff_two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bv = s - a;
  e = (a - (s - bv)) + (b - bv);
}
// s + e = a + b exactly for |a| >= |b| (Dekker)
FAME_HD void ff_fast_two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  e = b - (s - a);
}

// The operators are hidden friends: found for ff operands only, so they never
// take part in float or double expressions.
struct ff {
  float hi, lo;
  FAME_HD constexpr ff() : hi(0.0f), lo(0.0f) {}
  FAME_HD constexpr ff(double d)
      : hi(static_cast<float>(d)), lo(static_cast<float>(d - static_cast<double>(static_cast<float>(d)))) {}
  FAME_HD constexpr ff(float f) : hi(f), lo(0.0f) {}
  FAME_HD constexpr ff(int i) : ff(static_cast<double>(i)) {}
  FAME_HD constexpr ff(float h, float l, bool) : hi(h), lo(l) {}
  FAME_HD explicit operator double() const { return static_cast<double>(hi) + static_cast<double>(lo); }

  friend FAME_HD ff operator+(ff a, ff b) {
    float s1, s2, t1, t2;
    ff_two_sum(a.hi, b.hi, s1, s2);
    ff_two_sum(a.lo, b.lo, t1, t2);
    s2 += t1;
    ff_fast_two_sum(s1, s2, s1, s2);
    s2 += t2;
    ff_fast_two_sum(s1, s2, s1, s2);
    return ff(s1, s2, true);
  }
  friend FAME_HD ff operator-(ff a) { return ff(-a.hi, -a.lo, true); }
  friend FAME_HD ff operator-(ff a, ff b) { return a + (-b); }
  friend FAME_HD ff operator*(ff a, ff b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);  // the exact error of the product
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    float s, t;
    ff_fast_two_sum(p, e, s, t);
    return ff(s, t, true);
  }
  // Division and square roots through FP64: only used for per-thread scale
  // factors, never in the per-element arithmetic.
  friend FAME_HD ff operator/(ff a, ff b) { return ff(static_cast<double>(a) / static_cast<double>(b)); }
  friend FAME_HD ff& operator+=(ff& a, ff b) { return a = a + b; }
  friend FAME_HD ff& operator-=(ff& a, ff b) { return a = a - b; }
  friend FAME_HD ff& operator*=(ff& a, ff b) { return a = a * b; }
  friend FAME_HD ff sqrt(ff a) { return ff(::sqrt(static_cast<double>(a))); }
  friend FAME_HD ff rsqrt(ff a) { return ff(1.0 / ::sqrt(static_cast<double>(a))); }
};

struct cff {
  ff x, y;
};

template <class R> struct cx_of;
template <> struct cx_of<float> { using type = float2; };
template <> struct cx_of<double> { using type = double2; };
template <> struct cx_of<ff> { using type = cff; };
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
