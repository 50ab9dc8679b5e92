// Vector kernels of the Krylov glue: batched complex dot products with FP64
// accumulation, the fused conjugate-gradient updates of fncinvB (pcg), and
// the block Gram-Schmidt / restart products of the Lanczos band solver.
// Every kernel works on a batch of vectors, one vector per k-point instance,
// and skips vectors whose `active` flag is 0.
#include "krylov.h"

namespace fame {
namespace {

constexpr int kRedThreads = 256;

// Block-wide sum of a (double re, double im) pair; result valid in thread 0.
__device__ __forceinline__ double2 block_sum2(double2 v) {
  __shared__ double2 sh[kRedThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v.x += __shfl_down_sync(0xffffffffu, v.x, o);
    v.y += __shfl_down_sync(0xffffffffu, v.y, o);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  if (wid == 0) {
    v = lane < (blockDim.x >> 5) ? sh[lane] : make_double2(0.0, 0.0);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      v.x += __shfl_down_sync(0xffffffffu, v.x, o);
      v.y += __shfl_down_sync(0xffffffffu, v.y, o);
    }
  }
  return v;
}

// partial[v][m][blk] = sum over the block's slice of conj(a_m) * b
// a: nvec x ma vectors (stride lda per column, cols per vector = ma), b: one vector per vec.
template <class R>
__global__ void __launch_bounds__(kRedThreads)
k_dot_partial(const cx<R>* __restrict__ a, long long a_vstride, long long a_cstride, int ma,
              const cx<R>* __restrict__ b, long long b_vstride, long long len, double2* __restrict__ partial,
              const int* __restrict__ active) {
  const int vec = blockIdx.y;
  const int m = blockIdx.z;
  const int nblk = gridDim.x;
  double2* out = partial + ((long long)vec * ma + m) * nblk + blockIdx.x;
  if (active && !active[vec]) {
    if (threadIdx.x == 0) *out = make_double2(0.0, 0.0);
    return;
  }
  const cx<R>* av = a + vec * a_vstride + m * a_cstride;
  const cx<R>* bv = b + vec * b_vstride;
  // Per-thread partial sums in the vector's own precision (a complex64 thread
  // sums a few dozen products; FP64 is rate-limited on this part), then FP64
  // across threads and blocks.
  R sx0 = 0, sy0 = 0, sx1 = 0, sy1 = 0;
  const long long step = (long long)nblk * blockDim.x;
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + step < len; i += 2 * step) {
    cx<R> x = av[i], y = bv[i], x2 = av[i + step], y2 = bv[i + step];
    sx0 += x.x * y.x + x.y * y.y;
    sy0 += x.x * y.y - x.y * y.x;
    sx1 += x2.x * y2.x + x2.y * y2.y;
    sy1 += x2.x * y2.y - x2.y * y2.x;
  }
  if (i < len) {
    cx<R> x = av[i], y = bv[i];
    sx0 += x.x * y.x + x.y * y.y;
    sy0 += x.x * y.y - x.y * y.x;
  }
  double2 s = make_double2(double(sx0) + double(sx1), double(sy0) + double(sy1));
  s = block_sum2(s);
  if (threadIdx.x == 0) *out = s;
}

// Fused CG update and residual norm: x += a p ; r -= a q ; partial |r|^2.
template <class R>
__global__ void __launch_bounds__(kRedThreads)
k_cg_xr_dot(cx<R>* __restrict__ x, cx<R>* __restrict__ r, const cx<R>* __restrict__ p, const cx<R>* __restrict__ q,
            long long len, long long stride, const double* __restrict__ alpha, const int* __restrict__ active,
            double2* __restrict__ partial) {
  const int vec = blockIdx.y;
  const int nblk = gridDim.x;
  double2* out = partial + (long long)vec * nblk + blockIdx.x;
  if (active && !active[vec]) {
    if (threadIdx.x == 0) *out = make_double2(0.0, 0.0);
    return;
  }
  const R a = R(alpha[vec]);
  const long long o = vec * stride;
  R s0 = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (long long)nblk * blockDim.x) {
    cx<R> pi = p[o + i], qi = q[o + i], xi = x[o + i], ri = r[o + i];
    xi.x += a * pi.x;
    xi.y += a * pi.y;
    ri.x -= a * qi.x;
    ri.y -= a * qi.y;
    x[o + i] = xi;
    r[o + i] = ri;
    s0 += ri.x * ri.x + ri.y * ri.y;
  }
  double2 s = block_sum2(make_double2(double(s0), double(s0)));
  if (threadIdx.x == 0) *out = s;
}

__global__ void __launch_bounds__(kRedThreads)
k_dot_final(const double2* __restrict__ partial, int nblk, double2* __restrict__ out) {
  const long long row = blockIdx.x;  // vec * ma + m
  double2 s = make_double2(0.0, 0.0);
  for (int i = threadIdx.x; i < nblk; i += blockDim.x) {
    double2 p = partial[row * nblk + i];
    s.x += p.x;
    s.y += p.y;
  }
  s = block_sum2(s);
  if (threadIdx.x == 0) out[row] = s;
}

// y_v = alpha_v * x_v + beta_v * y_v with per-vector complex scalars (FP64)
template <class R>
__global__ void k_axpby(const cx<R>* __restrict__ x, cx<R>* __restrict__ y, long long len, long long stride,
                        const double2* __restrict__ alpha, const double2* __restrict__ beta,
                        const int* __restrict__ active) {
  const int vec = blockIdx.y;
  if (active && !active[vec]) return;
  const double2 a = alpha[vec], bb = beta[vec];
  const cx<R>* xv = x + vec * stride;
  cx<R>* yv = y + vec * stride;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x) {
    cx<R> xi = xv[i], yi = yv[i];
    double rx = a.x * xi.x - a.y * xi.y + bb.x * yi.x - bb.y * yi.y;
    double ry = a.x * xi.y + a.y * xi.x + bb.x * yi.y + bb.y * yi.x;
    yv[i] = mk<R>(R(rx), R(ry));
  }
}

// CG update: x += a p ; r -= a q  with a = rho / Re(p'q) per vector.
template <class R>
__global__ void k_cg_xr(cx<R>* __restrict__ x, cx<R>* __restrict__ r, const cx<R>* __restrict__ p,
                        const cx<R>* __restrict__ q, long long len, long long stride,
                        const double* __restrict__ alpha, const int* __restrict__ active) {
  const int vec = blockIdx.y;
  if (active && !active[vec]) return;
  const R a = R(alpha[vec]);
  const long long o = vec * stride;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x) {
    cx<R> pi = p[o + i], qi = q[o + i], xi = x[o + i], ri = r[o + i];
    xi.x += a * pi.x; xi.y += a * pi.y;
    ri.x -= a * qi.x; ri.y -= a * qi.y;
    x[o + i] = xi;
    r[o + i] = ri;
  }
}

// p = r + beta p
template <class R>
__global__ void k_cg_p(cx<R>* __restrict__ p, const cx<R>* __restrict__ r, long long len, long long stride,
                       const double* __restrict__ beta, const int* __restrict__ active) {
  const int vec = blockIdx.y;
  if (active && !active[vec]) return;
  const R b = R(beta[vec]);
  const long long o = vec * stride;
  const long long step = (long long)gridDim.x * blockDim.x;
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + step < len; i += 2 * step) {  // both elements' loads before the stores
    const cx<R> pi = p[o + i], ri = r[o + i], pj = p[o + i + step], rj = r[o + i + step];
    p[o + i] = mk<R>(ri.x + b * pi.x, ri.y + b * pi.y);
    p[o + i + step] = mk<R>(rj.x + b * pj.x, rj.y + b * pj.y);
  }
  if (i < len) {
    const cx<R> pi = p[o + i], ri = r[o + i];
    p[o + i] = mk<R>(ri.x + b * pi.x, ri.y + b * pi.y);
  }
}

// Per-vector CG scalars.  stage 0: alpha = rho/Re(pq); stage 1: convergence
// test on rho_new and beta = rho_new/rho.
// iters[v] counts the completed iterations of vector v on the device (so an
// iteration needs no host-side argument and can be replayed from a graph);
// a negative count flags breakdown at that iteration.
__global__ void k_cg_scalars(int stage, int nvec, const double2* __restrict__ dot, double* __restrict__ rho,
                             double* __restrict__ alpha, double* __restrict__ beta,
                             const double* __restrict__ tol2b2, int* __restrict__ active,
                             int* __restrict__ iters, double* __restrict__ res2) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nvec || !active[v]) return;
  const int it = iters[v] + 1;
  if (stage == 0) {
    const double pq = dot[v].x;
    alpha[v] = (pq != 0.0 && isfinite(pq)) ? rho[v] / pq : 0.0;
    if (!(pq > 0.0) || !isfinite(pq)) {  // breakdown: B must be HPD
      active[v] = 0;
      iters[v] = -it;
    }
  } else {
    // dot = (Re r'z, |r|^2) with z = M r (z = r without preconditioner)
    const double rz = dot[v].x;
    const double rn = dot[v].y;
    res2[v] = rn;
    beta[v] = rho[v] != 0.0 ? rz / rho[v] : 0.0;
    rho[v] = rz;
    iters[v] = it;
    if (!isfinite(rn) || !isfinite(rz)) {  // NaN / Inf: stop and flag
      active[v] = 0;
      iters[v] = -it;
    } else if (rn <= tol2b2[v]) {
      active[v] = 0;  // converged: ||r|| <= tol ||b||
    } else if (!(rz > 0.0)) {  // indefinite preconditioned system
      active[v] = 0;
      iters[v] = -it;
    }
  }
}

// k_cg_scalars preceded by the reduction of the vector's nblk partials (one
// CTA per vector; the block sum has a fixed order, so the iterates repeat
// run to run).
__global__ void __launch_bounds__(kRedThreads)
k_cg_scalars_red(int stage, const double2* __restrict__ partial, int nblk, double2* __restrict__ dot,
                 double* __restrict__ rho, double* __restrict__ alpha, double* __restrict__ beta,
                 const double* __restrict__ tol2b2, int* __restrict__ active, int* __restrict__ iters,
                 double* __restrict__ res2) {
  const int v = blockIdx.x;
  if (!active[v]) return;
  double2 s = make_double2(0.0, 0.0);
  for (int i = threadIdx.x; i < nblk; i += blockDim.x) {
    const double2 p = partial[(long long)v * nblk + i];
    s.x += p.x;
    s.y += p.y;
  }
  s = block_sum2(s);
  if (threadIdx.x != 0) return;
  dot[v] = s;
  const int it = iters[v] + 1;
  if (stage == 0) {
    const double pq = s.x;
    alpha[v] = (pq != 0.0 && isfinite(pq)) ? rho[v] / pq : 0.0;
    if (!(pq > 0.0) || !isfinite(pq)) {  // breakdown: B must be HPD
      active[v] = 0;
      iters[v] = -it;
    }
  } else {
    const double rz = s.x, rn = s.y;  // (Re r'z, |r|^2), z = M r (z = r without preconditioner)
    res2[v] = rn;
    beta[v] = rho[v] != 0.0 ? rz / rho[v] : 0.0;
    rho[v] = rz;
    iters[v] = it;
    if (!isfinite(rn) || !isfinite(rz)) {
      active[v] = 0;
      iters[v] = -it;
    } else if (rn <= tol2b2[v]) {
      active[v] = 0;
    } else if (!(rz > 0.0)) {
      active[v] = 0;
      iters[v] = -it;
    }
  }
}

// out[:, j] = sum_i in[:, i] * U[i, j]  (U real, p x k, column-major), all columns of one vector block
template <class R>
__global__ void k_block_rot(const cx<R>* __restrict__ in, cx<R>* __restrict__ out, long long len,
                            long long ld, int p, int k, const double* __restrict__ U) {
  extern __shared__ double Us[];
  for (int i = threadIdx.x; i < p * k; i += blockDim.x) Us[i] = U[i];
  __syncthreads();
  for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < len; row += (long long)gridDim.x * blockDim.x) {
    for (int j = 0; j < k; ++j) {
      double sx = 0.0, sy = 0.0;
      for (int i = 0; i < p; ++i) {
        cx<R> q = in[(long long)i * ld + row];
        sx += double(q.x) * Us[j * p + i];
        sy += double(q.y) * Us[j * p + i];
      }
      out[(long long)j * ld + row] = mk<R>(R(sx), R(sy));
    }
  }
}

// out = a x + b y + c w (real scalars; y, w may be null)
template <class R>
__global__ void k_lincomb3(cx<R>* out, double a, const cx<R>* x, double b, const cx<R>* y, double c, const cx<R>* w,
                           long long len) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x) {
    cx<R> xi = x[i];
    double rx = a * xi.x, ry = a * xi.y;
    if (y) {
      cx<R> yi = y[i];
      rx += b * yi.x;
      ry += b * yi.y;
    }
    if (w) {
      cx<R> wi = w[i];
      rx += c * wi.x;
      ry += c * wi.y;
    }
    out[i] = mk<R>(R(rx), R(ry));
  }
}

// out[:, j] = sum_i in[:, i] * C[i, j]  (C complex m x q, column-major)
template <class R>
__global__ void k_block_comb(const cx<R>* __restrict__ in, cx<R>* __restrict__ out, long long len, long long ld,
                             int m, int q, const double2* __restrict__ C) {
  extern __shared__ double2 Cs[];
  for (int i = threadIdx.x; i < m * q; i += blockDim.x) Cs[i] = C[i];
  __syncthreads();
  for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < len; row += (long long)gridDim.x * blockDim.x) {
    for (int j = 0; j < q; ++j) {
      double sx = 0.0, sy = 0.0;
      for (int i = 0; i < m; ++i) {
        const cx<R> v = in[(long long)i * ld + row];
        const double2 c = Cs[j * m + i];
        sx += double(v.x) * c.x - double(v.y) * c.y;
        sy += double(v.x) * c.y + double(v.y) * c.x;
      }
      out[(long long)j * ld + row] = mk<R>(R(sx), R(sy));
    }
  }
}

// ---------------------------------------------------------------------------
// Gram-Schmidt over a batch of k-point instances in one launch each: vector v
// works against its own columns col0_v .. col0_v + m_v - 1 (span[v] = (col0, m),
// m = 0 skips it) of its block X + v * xs (columns len apart).
// ---------------------------------------------------------------------------
// partial[(v * maxm + i) * nblk + blk] = block's share of X_v[col0_v + i]^H r_v
__global__ void __launch_bounds__(kRedThreads)
k_gs_dot_partial(const double2* __restrict__ X, long long xs, const double2* __restrict__ r, long long rs,
                 long long len, const int2* __restrict__ span, int maxm, double2* __restrict__ partial) {
  const int v = blockIdx.y, i = blockIdx.z, nblk = gridDim.x;
  const int2 sp = span[v];
  if (i >= sp.y) return;
  const double2* a = X + v * xs + (long long)(sp.x + i) * len;
  const double2* b = r + v * rs;
  double sx = 0.0, sy = 0.0;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < len; k += (long long)nblk * blockDim.x) {
    const double2 x = a[k], y = b[k];
    sx += x.x * y.x + x.y * y.y;
    sy += x.x * y.y - x.y * y.x;
  }
  const double2 s = block_sum2(make_double2(sx, sy));
  if (threadIdx.x == 0) partial[((long long)v * maxm + i) * nblk + blockIdx.x] = s;
}

// coef[v * cstride + i] = sum over blocks (i < m_v)
__global__ void __launch_bounds__(kRedThreads)
k_gs_dot_final(const double2* __restrict__ partial, int nblk, int maxm, const int2* __restrict__ span,
               double2* __restrict__ coef, int cstride) {
  const int v = blockIdx.x / maxm, i = blockIdx.x - v * maxm;
  if (i >= span[v].y) return;
  double2 s = make_double2(0.0, 0.0);
  for (int t = threadIdx.x; t < nblk; t += blockDim.x) {
    const double2 q = partial[((long long)v * maxm + i) * nblk + t];
    s.x += q.x;
    s.y += q.y;
  }
  s = block_sum2(s);
  if (threadIdx.x == 0) coef[(long long)v * cstride + i] = s;
}

// r_v -= sum_i coef[v * cstride + i] X_v[col0_v + i]  (FP64, or from a complex64 copy when XL)
template <class XT>
__global__ void k_gs_combo(double2* __restrict__ r, long long rs, const XT* __restrict__ X, long long xs,
                           long long len, const int2* __restrict__ span, const double2* __restrict__ coef,
                           int cstride) {
  __shared__ double2 cs[128];
  const int v = blockIdx.y;
  const int2 sp = span[v];
  if (sp.y <= 0) return;
  for (int i = threadIdx.x; i < sp.y; i += blockDim.x) cs[i] = coef[(long long)v * cstride + i];
  __syncthreads();
  const XT* x = X + v * xs + (long long)sp.x * len;
  double2* rv = r + v * rs;
  for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < len;
       row += (long long)gridDim.x * blockDim.x) {
    if constexpr (sizeof(XT) == 8) {  // complex64 copy: the correction in FP32
      float ax = 0.f, ay = 0.f;
      for (int i = 0; i < sp.y; ++i) {
        const XT q = x[(long long)i * len + row];
        const float cx_ = float(cs[i].x), cy_ = float(cs[i].y);
        ax += cx_ * q.x - cy_ * q.y;
        ay += cx_ * q.y + cy_ * q.x;
      }
      double2 o = rv[row];
      o.x -= double(ax);
      o.y -= double(ay);
      rv[row] = o;
    } else {
      double ax = 0.0, ay = 0.0;
      for (int i = 0; i < sp.y; ++i) {
        const XT q = x[(long long)i * len + row];
        ax += cs[i].x * q.x - cs[i].y * q.y;
        ay += cs[i].x * q.y + cs[i].y * q.x;
      }
      double2 o = rv[row];
      o.x -= ax;
      o.y -= ay;
      rv[row] = o;
    }
  }
}

// r -= sum_i c_i X[:, i]  (complex coefficients, FP64)
template <class R>
__global__ void k_sub_combo(cx<R>* __restrict__ r, const cx<R>* __restrict__ X, long long len, long long ld, int m,
                            const double2* __restrict__ c) {
  extern __shared__ double2 cs[];
  for (int i = threadIdx.x; i < m; i += blockDim.x) cs[i] = c[i];
  __syncthreads();
  for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < len; row += (long long)gridDim.x * blockDim.x) {
    cx<R> acc = r[row];
    double ax = acc.x, ay = acc.y;
    for (int i = 0; i < m; ++i) {
      cx<R> q = X[(long long)i * ld + row];
      ax -= cs[i].x * q.x - cs[i].y * q.y;
      ay -= cs[i].x * q.y + cs[i].y * q.x;
    }
    r[row] = mk<R>(R(ax), R(ay));
  }
}

template <class D, class S>
__global__ void k_convert(const cx<S>* __restrict__ in, cx<D>* __restrict__ out, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = mk<D>(D(in[i].x), D(in[i].y));
}

// x64 += m_v * d32 (m null: m_v = 1); res = b - bx (both FP64) for active vectors
__global__ void k_refine_acc(double2* __restrict__ x, const float2* __restrict__ d, long long len,
                             const int* __restrict__ active, const double* __restrict__ mult) {
  const int vec = blockIdx.y;
  if (active && !active[vec]) return;
  const double m = mult ? mult[vec] : 1.0;
  const long long o = vec * len;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x) {
    double2 a = x[o + i];
    float2 b = d[o + i];
    a.x += m * double(b.x);
    a.y += m * double(b.y);
    x[o + i] = a;
  }
}
__global__ void k_residual(const double2* __restrict__ b, const double2* __restrict__ bx, double2* __restrict__ res,
                           float2* __restrict__ res32, long long len, const int* __restrict__ active) {
  const int vec = blockIdx.y;
  if (active && !active[vec]) return;
  const long long o = vec * len;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x) {
    double2 r = make_double2(b[o + i].x - bx[o + i].x, b[o + i].y - bx[o + i].y);
    res[o + i] = r;
    if (res32) res32[o + i] = make_float2(float(r.x), float(r.y));
  }
}
// out32 = s_v * in (FP64 -> complex64) for active vectors
__global__ void k_to32_scaled(const double2* __restrict__ in, float2* __restrict__ out, long long len,
                              const double* __restrict__ s, const int* __restrict__ active) {
  const int vec = blockIdx.y;
  if (active && !active[vec]) return;
  const double a = s[vec];
  const long long o = vec * len;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x) {
    const double2 r = in[o + i];
    out[o + i] = make_float2(float(a * r.x), float(a * r.y));
  }
}
// y = s_v * x per vector (real per-vector scalars), x and y may alias
template <class R>
__global__ void k_scale(const cx<R>* x, cx<R>* y, long long len, const double* __restrict__ s,
                        const int* __restrict__ active) {
  const int vec = blockIdx.y;
  if (active && !active[vec]) return;
  const R a = R(s[vec]);
  const long long o = vec * len;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x) {
    cx<R> v = x[o + i];
    y[o + i] = mk<R>(a * v.x, a * v.y);
  }
}

int grid_for(long long len) {
  long long b = (len + 255) / 256;
  if (b > 4096) b = 4096;
  return int(b < 1 ? 1 : b);
}

}  // namespace

template <class R>
cudaError_t dot_batched(const cx<R>* a, long long a_vstride, long long a_cstride, int ma, const cx<R>* b,
                        long long b_vstride, long long len, int nvec, double2* out, double2* partial,
                        int nblk, const int* active, cudaStream_t st) {
  if (nvec <= 0 || ma <= 0) return cudaSuccess;
  dim3 g(nblk, nvec, ma);
  FAME_LAUNCHED(1);
  k_dot_partial<R><<<g, kRedThreads, 0, st>>>(a, a_vstride, a_cstride, ma, b, b_vstride, len, partial, active);
  FAME_LAUNCHED(1);
  k_dot_final<<<nvec * ma, kRedThreads, 0, st>>>(partial, nblk, out);
  return cudaGetLastError();
}

template <class R>
cudaError_t axpby_batched(const cx<R>* x, cx<R>* y, long long len, long long stride, int nvec,
                          const double2* alpha, const double2* beta, const int* active, cudaStream_t st) {
  if (nvec <= 0) return cudaSuccess;
  int gx = grid_for(len);
  if (gx > 1024) gx = 1024;
  FAME_LAUNCHED(1);
  k_axpby<R><<<dim3(gx, nvec), 256, 0, st>>>(x, y, len, stride, alpha, beta, active);
  return cudaGetLastError();
}

template <class R>
cudaError_t cg_xr(cx<R>* x, cx<R>* r, const cx<R>* p, const cx<R>* q, long long len, long long stride, int nvec,
                  const double* alpha, const int* active, cudaStream_t st) {
  int gx = grid_for(len);
  if (gx > 1024) gx = 1024;
  FAME_LAUNCHED(1);
  k_cg_xr<R><<<dim3(gx, nvec), 256, 0, st>>>(x, r, p, q, len, stride, alpha, active);
  return cudaGetLastError();
}

cudaError_t dot_final(const double2* partial, int nblk, int nrows, double2* out, cudaStream_t st) {
  FAME_LAUNCHED(1);
  k_dot_final<<<nrows, kRedThreads, 0, st>>>(partial, nblk, out);
  return cudaGetLastError();
}

template <class R>
cudaError_t cg_xr_dot(cx<R>* x, cx<R>* r, const cx<R>* p, const cx<R>* q, long long len, long long stride, int nvec,
                      const double* alpha, const int* active, double2* out, double2* partial, int nblk,
                      cudaStream_t st) {
  FAME_LAUNCHED(1);
  k_cg_xr_dot<R><<<dim3(nblk, nvec), kRedThreads, 0, st>>>(x, r, p, q, len, stride, alpha, active, partial);
  FAME_LAUNCHED(1);
  k_dot_final<<<nvec, kRedThreads, 0, st>>>(partial, nblk, out);
  return cudaGetLastError();
}

template <class R>
cudaError_t dot_partial(const cx<R>* a, const cx<R>* b, long long len, long long stride, int nvec, double2* partial,
                        int nblk, const int* active, cudaStream_t st) {
  if (nvec <= 0) return cudaSuccess;
  FAME_LAUNCHED(1);
  k_dot_partial<R><<<dim3(nblk, nvec, 1), kRedThreads, 0, st>>>(a, stride, 0, 1, b, stride, len, partial, active);
  return cudaGetLastError();
}

template <class R>
cudaError_t cg_xr_partial(cx<R>* x, cx<R>* r, const cx<R>* p, const cx<R>* q, long long len, long long stride,
                          int nvec, const double* alpha, const int* active, double2* partial, int nblk,
                          cudaStream_t st) {
  FAME_LAUNCHED(1);
  k_cg_xr_dot<R><<<dim3(nblk, nvec), kRedThreads, 0, st>>>(x, r, p, q, len, stride, alpha, active, partial);
  return cudaGetLastError();
}

// Q_v[:, col_v] = V_v, BQ_v[:, col_v] = BV_v (and their complex64 copies when
// given) for every v with col_v >= 0.
__global__ void k_gs_store(double2* __restrict__ Q, double2* __restrict__ BQ, float2* __restrict__ Q32,
                           float2* __restrict__ BQ32, long long xs, const double2* __restrict__ V,
                           const double2* __restrict__ BV, long long len, const int* __restrict__ col) {
  const int v = blockIdx.y;
  const int c = col[v];
  if (c < 0) return;
  const long long o = v * xs + (long long)c * len;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x) {
    const double2 a = V[v * len + i], b = BV[v * len + i];
    Q[o + i] = a;
    BQ[o + i] = b;
    if (Q32) {
      Q32[o + i] = make_float2(float(a.x), float(a.y));
      BQ32[o + i] = make_float2(float(b.x), float(b.y));
    }
  }
}

cudaError_t gs_store(double2* Q, double2* BQ, float2* Q32, float2* BQ32, long long xs, const double2* V,
                     const double2* BV, long long len, int nv, const int* col, cudaStream_t st) {
  if (nv <= 0) return cudaSuccess;
  int gx = grid_for(len);
  if (gx > 1024) gx = 1024;
  FAME_LAUNCHED(1);
  k_gs_store<<<dim3(gx, nv), 256, 0, st>>>(Q, BQ, Q32, BQ32, xs, V, BV, len, col);
  return cudaGetLastError();
}

cudaError_t gs_dots(const double2* X, long long xs, const double2* r, long long rs, long long len, int nv,
                    const int2* span, int maxm, double2* coef, int cstride, double2* partial, int nblk,
                    cudaStream_t st) {
  if (nv <= 0 || maxm <= 0) return cudaSuccess;
  FAME_LAUNCHED(1);
  k_gs_dot_partial<<<dim3(nblk, nv, maxm), kRedThreads, 0, st>>>(X, xs, r, rs, len, span, maxm, partial);
  FAME_LAUNCHED(1);
  k_gs_dot_final<<<nv * maxm, kRedThreads, 0, st>>>(partial, nblk, maxm, span, coef, cstride);
  return cudaGetLastError();
}

cudaError_t gs_combo(double2* r, long long rs, const double2* X, long long xs, long long len, int nv,
                     const int2* span, const double2* coef, int cstride, cudaStream_t st) {
  if (nv <= 0) return cudaSuccess;
  int gx = grid_for(len);
  if (gx > 1024) gx = 1024;
  FAME_LAUNCHED(1);
  k_gs_combo<double2><<<dim3(gx, nv), 256, 0, st>>>(r, rs, X, xs, len, span, coef, cstride);
  return cudaGetLastError();
}

cudaError_t gs_combo_lo(double2* r, long long rs, const float2* X, long long xs, long long len, int nv,
                        const int2* span, const double2* coef, int cstride, cudaStream_t st) {
  if (nv <= 0) return cudaSuccess;
  int gx = grid_for(len);
  if (gx > 1024) gx = 1024;
  FAME_LAUNCHED(1);
  k_gs_combo<float2><<<dim3(gx, nv), 256, 0, st>>>(r, rs, X, xs, len, span, coef, cstride);
  return cudaGetLastError();
}

// The loop condition of a graph-resident iteration loop: one pass of the
// body done (*passes + 1); continue while any vector is active and fewer
// than max_passes passes have run.
__global__ void k_while_active(const int* __restrict__ active, int nvec, int* __restrict__ passes, int max_passes,
                               cudaGraphConditionalHandle h) {
  int any = 0;
  for (int v = threadIdx.x; v < nvec; v += blockDim.x) any |= active[v];
  any = __any_sync(0xffffffffu, any);
  if (threadIdx.x == 0) {
    const int b = *passes + 1;
    *passes = b;
    cudaGraphSetConditional(h, (any && b < max_passes) ? 1u : 0u);
  }
}

cudaError_t while_active(const int* active, int nvec, int* passes, int max_passes, cudaGraphConditionalHandle h,
                         cudaStream_t st) {
  FAME_LAUNCHED(1);
  k_while_active<<<1, 32, 0, st>>>(active, nvec, passes, max_passes, h);
  return cudaGetLastError();
}

cudaError_t cg_scalars_red(int stage, int nvec, const double2* partial, int nblk, double2* dot, double* rho,
                           double* alpha, double* beta, const double* tol2b2, int* active, int* iters, double* res2,
                           cudaStream_t st) {
  FAME_LAUNCHED(1);
  k_cg_scalars_red<<<nvec, kRedThreads, 0, st>>>(stage, partial, nblk, dot, rho, alpha, beta, tol2b2, active, iters,
                                                 res2);
  return cudaGetLastError();
}

template <class R>
cudaError_t cg_p(cx<R>* p, const cx<R>* r, long long len, long long stride, int nvec, const double* beta,
                 const int* active, cudaStream_t st) {
  int gx = grid_for(len);
  if (gx > 1024) gx = 1024;
  FAME_LAUNCHED(1);
  k_cg_p<R><<<dim3(gx, nvec), 256, 0, st>>>(p, r, len, stride, beta, active);
  return cudaGetLastError();
}

cudaError_t cg_scalars(int stage, int nvec, const double2* dot, double* rho, double* alpha, double* beta,
                       const double* tol2b2, int* active, int* iters, double* res2, cudaStream_t st) {
  FAME_LAUNCHED(1);
  k_cg_scalars<<<(nvec + 127) / 128, 128, 0, st>>>(stage, nvec, dot, rho, alpha, beta, tol2b2, active, iters,
                                                    res2);
  return cudaGetLastError();
}

template <class R>
cudaError_t block_rot(const cx<R>* in, cx<R>* out, long long len, long long ld, int p, int k, const double* U,
                      cudaStream_t st) {
  FAME_LAUNCHED(1);
  k_block_rot<R><<<grid_for(len), 256, sizeof(double) * p * k, st>>>(in, out, len, ld, p, k, U);
  return cudaGetLastError();
}

template <class R>
cudaError_t lincomb3(cx<R>* out, double a, const cx<R>* x, double b, const cx<R>* y, double c, const cx<R>* w,
                     long long len, cudaStream_t st) {
  FAME_LAUNCHED(1);
  k_lincomb3<R><<<grid_for(len), 256, 0, st>>>(out, a, x, b, y, c, w, len);
  return cudaGetLastError();
}
template cudaError_t lincomb3<float>(cx<float>*, double, const cx<float>*, double, const cx<float>*, double,
                                     const cx<float>*, long long, cudaStream_t);
template cudaError_t lincomb3<double>(cx<double>*, double, const cx<double>*, double, const cx<double>*, double,
                                      const cx<double>*, long long, cudaStream_t);

template <class R>
cudaError_t block_comb(const cx<R>* in, cx<R>* out, long long len, long long ld, int m, int q, const double2* C,
                       cudaStream_t st) {
  const size_t sm = sizeof(double2) * m * q;
  if (sm > 200 * 1024) return cudaErrorInvalidValue;
  if (sm > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_block_comb<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
  }
  FAME_LAUNCHED(1);
  k_block_comb<R><<<grid_for(len), 256, sm, st>>>(in, out, len, ld, m, q, C);
  return cudaGetLastError();
}
template cudaError_t block_comb<double>(const cx<double>*, cx<double>*, long long, long long, int, int, const double2*,
                                        cudaStream_t);

template <class R>
cudaError_t sub_combo(cx<R>* r, const cx<R>* X, long long len, long long ld, int m, const double2* c,
                      cudaStream_t st) {
  if (m <= 0) return cudaSuccess;
  FAME_LAUNCHED(1);
  k_sub_combo<R><<<grid_for(len), 256, sizeof(double2) * m, st>>>(r, X, len, ld, m, c);
  return cudaGetLastError();
}

template <class D, class S>
cudaError_t convert(const cx<S>* in, cx<D>* out, long long n, cudaStream_t st) {
  FAME_LAUNCHED(1);
  k_convert<D, S><<<grid_for(n), 256, 0, st>>>(in, out, n);
  return cudaGetLastError();
}

cudaError_t refine_acc(double2* x, const float2* d, long long len, int nvec, const int* active, cudaStream_t st,
                       const double* mult) {
  int gx = grid_for(len);
  if (gx > 1024) gx = 1024;
  FAME_LAUNCHED(1);
  k_refine_acc<<<dim3(gx, nvec), 256, 0, st>>>(x, d, len, active, mult);
  return cudaGetLastError();
}

cudaError_t to32_scaled(const double2* in, float2* out, long long len, int nvec, const double* s, const int* active,
                        cudaStream_t st) {
  int gx = grid_for(len);
  if (gx > 1024) gx = 1024;
  FAME_LAUNCHED(1);
  k_to32_scaled<<<dim3(gx, nvec), 256, 0, st>>>(in, out, len, s, active);
  return cudaGetLastError();
}

cudaError_t residual(const double2* b, const double2* bx, double2* res, float2* res32, long long len, int nvec,
                     const int* active, cudaStream_t st) {
  int gx = grid_for(len);
  if (gx > 1024) gx = 1024;
  FAME_LAUNCHED(1);
  k_residual<<<dim3(gx, nvec), 256, 0, st>>>(b, bx, res, res32, len, active);
  return cudaGetLastError();
}

template <class R>
cudaError_t scale_batched(const cx<R>* x, cx<R>* y, long long len, int nvec, const double* s, const int* active,
                          cudaStream_t st) {
  int gx = grid_for(len);
  if (gx > 1024) gx = 1024;
  FAME_LAUNCHED(1);
  k_scale<R><<<dim3(gx, nvec), 256, 0, st>>>(x, y, len, s, active);
  return cudaGetLastError();
}
template cudaError_t scale_batched<double>(const cx<double>*, cx<double>*, long long, int, const double*, const int*,
                                           cudaStream_t);
template cudaError_t scale_batched<float>(const cx<float>*, cx<float>*, long long, int, const double*, const int*,
                                          cudaStream_t);

#define FAME_KINST(R)                                                                                     \
  template cudaError_t dot_batched<R>(const cx<R>*, long long, long long, int, const cx<R>*, long long,  \
                                      long long, int, double2*, double2*, int, const int*, cudaStream_t); \
  template cudaError_t axpby_batched<R>(const cx<R>*, cx<R>*, long long, long long, int, const double2*, \
                                        const double2*, const int*, cudaStream_t);                       \
  template cudaError_t cg_xr<R>(cx<R>*, cx<R>*, const cx<R>*, const cx<R>*, long long, long long, int,   \
                                const double*, const int*, cudaStream_t);                                 \
  template cudaError_t cg_p<R>(cx<R>*, const cx<R>*, long long, long long, int, const double*,           \
                               const int*, cudaStream_t);                                                 \
  template cudaError_t cg_xr_dot<R>(cx<R>*, cx<R>*, const cx<R>*, const cx<R>*, long long, long long, int, \
                                    const double*, const int*, double2*, double2*, int, cudaStream_t);    \
  template cudaError_t block_rot<R>(const cx<R>*, cx<R>*, long long, long long, int, int, const double*, \
                                    cudaStream_t);                                                        \
  template cudaError_t sub_combo<R>(cx<R>*, const cx<R>*, long long, long long, int, const double2*,     \
                                    cudaStream_t);                                                        \
  template cudaError_t dot_partial<R>(const cx<R>*, const cx<R>*, long long, long long, int, double2*,   \
                                      int, const int*, cudaStream_t);                                     \
  template cudaError_t cg_xr_partial<R>(cx<R>*, cx<R>*, const cx<R>*, const cx<R>*, long long, long long, \
                                        int, const double*, const int*, double2*, int, cudaStream_t);
FAME_KINST(float)
FAME_KINST(double)
template cudaError_t convert<float, double>(const cx<double>*, cx<float>*, long long, cudaStream_t);
template cudaError_t convert<double, float>(const cx<float>*, cx<double>*, long long, cudaStream_t);

}  // namespace fame
