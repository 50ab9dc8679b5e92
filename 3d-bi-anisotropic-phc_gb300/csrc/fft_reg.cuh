// In-register mixed-radix FFT of compile-time length N (N = 2^a 3^b 5^c).
//
// One thread owns one pencil of N complex values in registers.  A length
// with coprime factors N = N1*N2 (N1 the full power of its smallest prime)
// is split by the prime-factor (Good-Thomas) mapping, which needs no twiddle
// factors:
//   n = (N2*n1 + N1*n2) mod N,   k = (N2*A*k1 + N1*B*k2) mod N,
//   A = N2^{-1} mod N1, B = N1^{-1} mod N2,
//   X[k] = sum_{n2} W_N2^{n2*k2} sum_{n1} x[n] W_N1^{n1*k1}.
// A prime power is split by Cooley-Tukey with the first radix split off
// (N = R*M):
//   X[k1 + R*k2] = sum_{n2} W_N^{n2*k1} W_M^{n2*k2} sum_{n1} x[M*n1 + n2] W_R^{n1*k1}
// i.e. M radix-R butterflies on strided inputs, a twiddle, then R
// recursive length-M transforms.  All indices are compile-time constants,
// so the arrays stay in registers and every twiddle is an immediate operand.
//
// S = -1 is the forward transform (MATLAB fft: exp(-2*pi*i*n*k/N)),
// S = +1 the unnormalised inverse.  Scaling is left to the caller.
#pragma once

#include "fame_types.cuh"

namespace fame {

FAME_HD constexpr int fft_first_radix(int n) {
  return (n % 4 == 0 && n != 8) ? 4 : (n % 2 == 0) ? 2 : (n % 3 == 0) ? 3 : (n % 5 == 0) ? 5 : n;
}

// Full power of the smallest prime factor of n (n itself for a prime power).
FAME_HD constexpr int fft_pfa_part(int n) {
  int p = 2;
  while (p < n && n % p != 0) ++p;
  int q = 1;
  while (n % p == 0) {
    n /= p;
    q *= p;
  }
  return q;
}

// a^{-1} mod m for coprime a, m (m >= 1).
FAME_HD constexpr int fft_inv_mod(int a, int m) {
  if (m == 1) return 0;
  for (int x = 1; x < m; ++x)
    if ((a * x) % m == 1) return x;
  return -1;
}

FAME_HD constexpr bool fft_supported(int n) {
  while (n % 2 == 0 && n > 1) n /= 2;
  while (n % 3 == 0) n /= 3;
  while (n % 5 == 0) n /= 5;
  return n == 1;
}

// v * exp(S*2*pi*i*E/N)
template <class R, int N, int S, int E>
FAME_HD cx<R> twiddle(cx<R> v) {
  constexpr int e = ((E % N) + N) % N;
  if constexpr (e == 0) {
    return v;
  } else if constexpr ((4 * e) % N == 0) {
    constexpr int q = (4 * e) / N;  // quarter turns
    if constexpr (q == 2) return cneg(v);
    else if constexpr (q == 1) return cmul_i<S>(v);
    else return cmul_i<-S>(v);
  } else if constexpr ((8 * e) % N == 0) {
    constexpr int o = (8 * e) / N;  // odd eighth turns: (+-1 +- i)/sqrt(2)
    constexpr double h = 0.70710678118654752440084436210484903928;
    constexpr double c = (o == 1 || o == 7) ? h : -h;
    constexpr double s0 = (o == 1 || o == 3) ? h : -h;
    constexpr double s = S * s0;
    // (vx + i vy)(c + i s)
    return mk<R>(R(c) * v.x - R(s) * v.y, R(c) * v.y + R(s) * v.x);
  } else {
    constexpr double c = cs2pi(e, N, 0);
    constexpr double s = S * cs2pi(e, N, 1);
    return mk<R>(R(c) * v.x - R(s) * v.y, R(c) * v.y + R(s) * v.x);
  }
}

// Small DFTs (radix kernels).
template <class R, int P, int S>
FAME_HD void dft_small(cx<R> (&a)[P]) {
  if constexpr (P == 1) {
  } else if constexpr (P == 2) {
    cx<R> t = a[0];
    a[0] = cadd(t, a[1]);
    a[1] = csub(t, a[1]);
  } else if constexpr (P == 4) {
    cx<R> s02 = cadd(a[0], a[2]), d02 = csub(a[0], a[2]);
    cx<R> s13 = cadd(a[1], a[3]), d13 = cmul_i<S>(csub(a[1], a[3]));
    a[0] = cadd(s02, s13);
    a[2] = csub(s02, s13);
    a[1] = cadd(d02, d13);
    a[3] = csub(d02, d13);
  } else {
    // odd P: pair symmetric terms t_n = a_n + a_{P-n}, d_n = a_n - a_{P-n}
    constexpr int H = (P - 1) / 2;
    cx<R> t[H + 1], d[H + 1];
    static_for<1, H + 1>([&](auto nc) {
      constexpr int n = decltype(nc)::value;
      t[n] = cadd(a[n], a[P - n]);
      d[n] = csub(a[n], a[P - n]);
    });
    cx<R> a0 = a[0];
    cx<R> sum = a0;
    static_for<1, H + 1>([&](auto nc) { sum = cadd(sum, t[decltype(nc)::value]); });
    a[0] = sum;
    static_for<1, H + 1>([&](auto kc) {
      constexpr int k = decltype(kc)::value;
      cx<R> re = a0, im = zero<R>();
      static_for<1, H + 1>([&](auto nc) {
        constexpr int n = decltype(nc)::value;
        constexpr double c = cs2pi((long long)n * k, P, 0);
        constexpr double s = cs2pi((long long)n * k, P, 1);
        re.x += R(c) * t[n].x;
        re.y += R(c) * t[n].y;
        im.x += R(s) * d[n].x;
        im.y += R(s) * d[n].y;
      });
      // X[k] = re + S*i*im ; X[P-k] = re - S*i*im
      cx<R> iim = cmul_i<S>(im);
      a[k] = cadd(re, iim);
      a[P - k] = csub(re, iim);
    });
  }
}

template <class R, int N, int S>
FAME_HD void fft(cx<R> (&x)[N]) {
  constexpr int RD = fft_first_radix(N);
  constexpr int N1 = fft_pfa_part(N);
  if constexpr (N == 1) {
  } else if constexpr (N1 > 1 && N1 < N) {
    constexpr int N2 = N / N1;
    constexpr int A = fft_inv_mod(N2 % N1, N1);
    constexpr int B = fft_inv_mod(N1 % N2, N2);
    static_assert(A >= 0 && B >= 0, "prime-factor split needs coprime factors");
    cx<R> y[N];  // y[k1*N2 + n2]
    static_for<0, N2>([&](auto n2c) {
      constexpr int n2 = decltype(n2c)::value;
      cx<R> a[N1];
      static_for<0, N1>([&](auto n1c) {
        constexpr int n1 = decltype(n1c)::value;
        a[n1] = x[(N2 * n1 + N1 * n2) % N];
      });
      fft<R, N1, S>(a);
      static_for<0, N1>([&](auto k1c) { y[decltype(k1c)::value * N2 + n2] = a[decltype(k1c)::value]; });
    });
    static_for<0, N1>([&](auto k1c) {
      constexpr int k1 = decltype(k1c)::value;
      cx<R> z[N2];
      static_for<0, N2>([&](auto n2c) { z[decltype(n2c)::value] = y[k1 * N2 + decltype(n2c)::value]; });
      fft<R, N2, S>(z);
      static_for<0, N2>([&](auto k2c) {
        constexpr int k2 = decltype(k2c)::value;
        x[(N2 * A * k1 + N1 * B * k2) % N] = z[k2];
      });
    });
  } else if constexpr (RD == N) {
    dft_small<R, N, S>(x);
  } else {
    constexpr int M = N / RD;
    cx<R> y[N];  // y[k1*M + n2]
    static_for<0, M>([&](auto n2c) {
      constexpr int n2 = decltype(n2c)::value;
      cx<R> a[RD];
      static_for<0, RD>([&](auto n1c) { a[decltype(n1c)::value] = x[M * decltype(n1c)::value + n2]; });
      dft_small<R, RD, S>(a);
      static_for<0, RD>([&](auto k1c) {
        constexpr int k1 = decltype(k1c)::value;
        y[k1 * M + n2] = twiddle<R, N, S, n2 * k1>(a[k1]);
      });
    });
    static_for<0, RD>([&](auto k1c) {
      constexpr int k1 = decltype(k1c)::value;
      cx<R> z[M];
      static_for<0, M>([&](auto n2c) { z[decltype(n2c)::value] = y[k1 * M + decltype(n2c)::value]; });
      fft<R, M, S>(z);
      static_for<0, M>([&](auto k2c) { x[k1 + RD * decltype(k2c)::value] = z[decltype(k2c)::value]; });
    });
  }
}

// Grid sizes with a compiled transform.  FAME_FOR_EACH_N(X) expands X(n)
// for each; the dispatchers switch over this list and fncb_inst_*.cu
// instantiate exactly these sizes.
#define FAME_FOR_EACH_N(X) \
  X(4) X(6) X(8) X(10) X(12) X(16) X(18) X(20) X(24) X(30) X(32) X(36) X(40) X(48) X(50) X(60) X(64)

}  // namespace fame
