// Preconditioner of the conjugate-gradient solves with B (fncinvB).
//
// For a homogeneous medium every Bloch shift is diagonal in the frequency
// basis (T_d <-> t_d = exp(i(2 pi k_d + theta_d)/n) = 1 + lambda_d/n), so
// fncB reduces to one 4x4 Hermitian block per frequency voxel:
//   B0(k) = Pi(k)^H G(k) Pi(k),   Pi = blkdiag([-conj(Pi2) conj(Pi1)], [Pi1 Pi2])
// with G(k) the 6x6 material symbol of the interpolated operators
// (IntCovarForm*_vertex*.m): lumped diagonals Re Mh_ii, Re Nh_ii, and
//   M_ij: c_a c_b Mh_ij conj(c_a' c_b')/16 , N_ij: c_i Nh_ij conj(c_j)/4 ,
//   J_ij: c_i J_ij conj(c_a' c_b')/8        (c_d = 1 + t_d).
// Using the volume-averaged vertex tensors of the actual crystal, M = B0^{-1}
// is a cheap spectrally close approximation of B^{-1}; the CG iteration count
// drops by more than half on the woodpile.  The solution of B y = x does not
// depend on it.
#include "fncb_impl.cuh"
#include "krylov.h"

namespace fame {
namespace {

__device__ __forceinline__ double2 dmk(double a, double b) { return make_double2(a, b); }

// Complex slots per voxel of the stored inverse blocks (the four real
// diagonal entries packed in two).
constexpr int kPcSlots = 8;

__global__ void __launch_bounds__(128)
k_precond_build64(const double2* __restrict__ lam_all, const double2* __restrict__ avg_all, int n, double2* pc64,
                  float2* pc32) {
  const long long Nq = (long long)n * n * n;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int inst = blockIdx.y;
  if (idx >= Nq) return;
  const int i1 = int(idx % n), i2 = int((idx / n) % n), i3 = int(idx / ((long long)n * n));
  const double2* lam = lam_all + (long long)inst * 3 * n;
  const double2 L[3] = {lam[i1], lam[n + i2], lam[2 * n + i3]};
  double2 c[3];
  for (int d = 0; d < 3; ++d) c[d] = dmk(2.0 + L[d].x / n, L[d].y / n);
  const double2* T = avg_all + (long long)inst * 27;
  const double2* Nh = T;
  const double2* Mh = T + 9;
  const double2* J = T + 18;
  double2 Guu[3][3], Gvv[3][3], Gvu[3][3];
  auto ax = [](int i, int s) { return i == 0 ? (s == 0 ? 1 : 2) : i == 1 ? (s == 0 ? 0 : 2) : (s == 0 ? 0 : 1); };
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      const double2 ci = cmul(c[ax(i, 0)], c[ax(i, 1)]);
      const double2 cj = cmul(c[ax(j, 0)], c[ax(j, 1)]);
      if (i == j) {
        Guu[i][j] = dmk(Mh[i * 3 + i].x, 0.0);
        Gvv[i][j] = dmk(Nh[i * 3 + i].x, 0.0);
      } else {
        Guu[i][j] = cscale(cmul(cmul(ci, Mh[i * 3 + j]), cconj(cj)), 1.0 / 16.0);
        Gvv[i][j] = cscale(cmul(cmul(c[i], Nh[i * 3 + j]), cconj(c[j])), 0.25);
      }
      Gvu[i][j] = cscale(cmul(cmul(c[i], J[i * 3 + j]), cconj(cj)), 0.125);
    }
  detail::PiBlock<double> P = detail::pi_block<double>(L[0], L[1], L[2]);
  // columns of Pi: u-side e0 = -conj(Pi2), e1 = conj(Pi1); v-side f0 = Pi1, f1 = Pi2
  double2 col[4][3];
  for (int r = 0; r < 3; ++r) {
    col[0][r] = cneg(cconj(P.p2[r]));
    col[1][r] = cconj(P.p1[r]);
    col[2][r] = P.p1[r];
    col[3][r] = P.p2[r];
  }
  // B0[a][b] = col_a^H G col_b
  double2 B[4][4];
  for (int a = 0; a < 4; ++a)
    for (int b = 0; b < 4; ++b) {
      double2 s = dmk(0.0, 0.0);
      for (int r = 0; r < 3; ++r) {
        double2 g = dmk(0.0, 0.0);
        for (int q = 0; q < 3; ++q) {
          double2 Gr;
          if (a < 2 && b < 2) Gr = Guu[r][q];
          else if (a >= 2 && b >= 2) Gr = Gvv[r][q];
          else if (a >= 2) Gr = Gvu[r][q];   // v row, u column
          else Gr = cconj(Gvu[q][r]);        // u row, v column: Guv = Gvu^H
          g = cfma(Gr, col[b][q], g);
        }
        s = cfmac(col[a][r], g, s);
      }
      B[a][b] = s;
    }
  // Gauss-Jordan inverse of the Hermitian positive definite block
  double2 Minv[4][4];
  for (int a = 0; a < 4; ++a)
    for (int b = 0; b < 4; ++b) Minv[a][b] = dmk(a == b ? 1.0 : 0.0, 0.0);
  bool ok = true;
  for (int p = 0; p < 4; ++p) {
    const double piv = B[p][p].x;
    if (!(piv > 0.0)) {
      ok = false;
      break;
    }
    const double2 inv = dmk(1.0 / piv, 0.0);
    for (int b = 0; b < 4; ++b) {
      B[p][b] = cmul(B[p][b], inv);
      Minv[p][b] = cmul(Minv[p][b], inv);
    }
    for (int a = 0; a < 4; ++a) {
      if (a == p) continue;
      const double2 f = B[a][p];
      for (int b = 0; b < 4; ++b) {
        B[a][b] = csub(B[a][b], cmul(f, B[p][b]));
        Minv[a][b] = csub(Minv[a][b], cmul(f, Minv[p][b]));
      }
    }
  }
  if (!ok)  // not positive definite (non-physical material): identity
    for (int a = 0; a < 4; ++a)
      for (int b = 0; b < 4; ++b) Minv[a][b] = dmk(a == b ? 1.0 : 0.0, 0.0);
  // packed: (m00, m11) | (m22, m33) | m01 | m02 | m03 | m12 | m13 | m23
  double2 v[kPcSlots];
  v[0] = dmk(Minv[0][0].x, Minv[1][1].x);
  v[1] = dmk(Minv[2][2].x, Minv[3][3].x);
  const int ent[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
  for (int e = 0; e < 6; ++e) v[2 + e] = Minv[ent[e][0]][ent[e][1]];
  for (int e = 0; e < kPcSlots; ++e) {
    const long long o = ((long long)inst * kPcSlots + e) * Nq + idx;
    if (pc64) pc64[o] = v[e];
    if (pc32) pc32[o] = make_float2(float(v[e].x), float(v[e].y));
  }
}

// The inverse block of one voxel.
template <class R> struct Block4 {
  cx<R> s[kPcSlots];
};
template <class R>
__device__ __forceinline__ Block4<R> load_block(const cx<R>* __restrict__ pc, long long Nq, long long idx) {
  Block4<R> b;
#pragma unroll
  for (int e = 0; e < kPcSlots; ++e) b.s[e] = pc[e * Nq + idx];
  return b;
}
// z = M r for the 4 components of one voxel
template <class R>
__device__ __forceinline__ void mvec4(const Block4<R>& b, const cx<R> r[4], cx<R> z[4]) {
  const R m00 = b.s[0].x, m11 = b.s[0].y, m22 = b.s[1].x, m33 = b.s[1].y;
  const cx<R> m01 = b.s[2], m02 = b.s[3], m03 = b.s[4], m12 = b.s[5], m13 = b.s[6], m23 = b.s[7];
  z[0] = cfma(m03, r[3], cfma(m02, r[2], cfma(m01, r[1], cscale(r[0], m00))));
  z[1] = cfma(m13, r[3], cfma(m12, r[2], cfmac(m01, r[0], cscale(r[1], m11))));
  z[2] = cfma(m23, r[3], cfmac(m12, r[1], cfmac(m02, r[0], cscale(r[2], m22))));
  z[3] = cfmac(m23, r[2], cfmac(m13, r[1], cfmac(m03, r[0], cscale(r[3], m33))));
}

constexpr int kThreads = 256;

__device__ __forceinline__ double2 block_sum2b(double2 v) {
  __shared__ double2 sh[kThreads / 32];
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

template <class R>
__global__ void __launch_bounds__(kThreads)
k_precond_apply(const cx<R>* __restrict__ r, cx<R>* __restrict__ z, const cx<R>* __restrict__ pc_all, VecCtx ctx,
                long long Nq, double2* __restrict__ partial) {
  const int vec = blockIdx.y;
  const int nblk = gridDim.x;
  double2* out = partial + (long long)vec * nblk + blockIdx.x;
  if (ctx.active && !ctx.active[vec]) {
    if (threadIdx.x == 0) *out = make_double2(0.0, 0.0);
    return;
  }
  const cx<R>* pc = pc_all + (long long)vec_inst(ctx, vec) * kPcSlots * Nq;
  const long long o = vec * 4 * Nq;
  R srz = 0, srr = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < Nq; i += (long long)nblk * blockDim.x) {
    cx<R> rv[4], zv[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) rv[c] = r[o + c * Nq + i];
    mvec4<R>(load_block<R>(pc, Nq, i), rv, zv);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      z[o + c * Nq + i] = zv[c];
      srz += rv[c].x * zv[c].x + rv[c].y * zv[c].y;
      srr += rv[c].x * rv[c].x + rv[c].y * rv[c].y;
    }
  }
  double2 s = block_sum2b(make_double2(double(srz), double(srr)));
  if (threadIdx.x == 0) *out = s;
}

template <class R>
__global__ void __launch_bounds__(kThreads, sizeof(R) == 4 ? 2 : 1)
k_pcg_update(cx<R>* __restrict__ x, cx<R>* __restrict__ r, cx<R>* __restrict__ z, const cx<R>* __restrict__ p,
             const cx<R>* __restrict__ q, const cx<R>* __restrict__ pc_all, VecCtx ctx, long long Nq,
             const double* __restrict__ alpha, double2* __restrict__ partial, CgAlpha ca) {
  const int vec = blockIdx.y;
  const int nblk = gridDim.x;
  double2* out = partial + (long long)vec * nblk + blockIdx.x;
  if (ctx.active && !ctx.active[vec]) {
    if (threadIdx.x == 0) *out = make_double2(0.0, 0.0);
    return;
  }
  R a;
  if (ca.pq) {
    __shared__ double s_alpha;
    if (threadIdx.x < 32) {
      double sx = 0.0, sy = 0.0;
      for (int i = threadIdx.x; i < ca.nblk; i += 32) {
        const double2 t = ca.pq[(long long)vec * ca.nblk + i];
        sx += t.x;
        sy += t.y;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        sx += __shfl_down_sync(0xffffffffu, sx, o);
        sy += __shfl_down_sync(0xffffffffu, sy, o);
      }
      if (threadIdx.x == 0) {
        const bool ok = sx > 0.0 && isfinite(sx);
        const double av = ok ? ca.rho[vec] / sx : 0.0;
        s_alpha = av;
        if (blockIdx.x == 0) {
          ca.alpha[vec] = av;
          ca.dot[vec] = make_double2(sx, sy);
          if (!ok) {  // breakdown: B must be HPD
            ca.active[vec] = 0;
            ca.iters[vec] = -(ca.iters[vec] + 1);
          }
        }
      }
    }
    __syncthreads();
    a = R(s_alpha);
  } else {
    a = R(alpha[vec]);
  }
  const cx<R>* pc = pc_all + (long long)vec_inst(ctx, vec) * kPcSlots * Nq;
  const long long o = vec * 4 * Nq;
  R srz = 0, srr = 0;
  const long long stride = (long long)nblk * blockDim.x;
  // two voxels per pass, every load of both issued before any store
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < Nq; i += 2 * stride) {
    const long long i2 = i + stride;
    const bool two = i2 < Nq;
    cx<R> pk[2][4], qk[2][4], xk[2][4], rk[2][4];
    Block4<R> bk[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      if (u == 1 && !two) break;
      const long long iv = u ? i2 : i;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const long long k = o + c * Nq + iv;
        pk[u][c] = p[k];
        qk[u][c] = q[k];
        xk[u][c] = x[k];
        rk[u][c] = r[k];
      }
      bk[u] = load_block<R>(pc, Nq, iv);
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      if (u == 1 && !two) break;
      const long long iv = u ? i2 : i;
      cx<R> zv[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        xk[u][c].x += a * pk[u][c].x;
        xk[u][c].y += a * pk[u][c].y;
        rk[u][c].x -= a * qk[u][c].x;
        rk[u][c].y -= a * qk[u][c].y;
      }
      mvec4<R>(bk[u], rk[u], zv);
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const long long k = o + c * Nq + iv;
        x[k] = xk[u][c];
        r[k] = rk[u][c];
        z[k] = zv[c];
        srz += rk[u][c].x * zv[c].x + rk[u][c].y * zv[c].y;
        srr += rk[u][c].x * rk[u][c].x + rk[u][c].y * rk[u][c].y;
      }
    }
  }
  double2 s = block_sum2b(make_double2(double(srz), double(srr)));
  if (threadIdx.x == 0) *out = s;
}

}  // namespace

template <class R> PlanData<R>& pd_mut(Plan& P);
template <> PlanData<double>& pd_mut<double>(Plan& P) { return P.d64; }
template <> PlanData<float>& pd_mut<float>(Plan& P) { return P.d32; }

template <class R> cudaError_t build_precond(Plan& P, cudaStream_t st) {
  PlanData<R>& d = pd_mut<R>(P);
  if (d.pc) return cudaSuccess;
  cudaError_t e;
  if (!P.d_mat_avg) {
    e = cudaMalloc(&P.d_mat_avg, sizeof(double2) * 27 * P.nk);
    if (e != cudaSuccess) return e;
    e = cudaMemcpy(P.d_mat_avg, P.mat_avg.data(), sizeof(double2) * 27 * P.nk, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return e;
  }
  e = cudaMalloc(&d.pc, sizeof(cx<R>) * kPcSlots * (size_t)P.Nq * P.nk);
  if (e != cudaSuccess) return e;
  FAME_LAUNCHED(1);
  k_precond_build64<<<dim3((unsigned)((P.Nq + 127) / 128), P.nk), 128, 0, st>>>(
      P.d64.lam, P.d_mat_avg, P.n, sizeof(R) == 8 ? (double2*)d.pc : nullptr,
      sizeof(R) == 4 ? (float2*)d.pc : nullptr);
  return cudaGetLastError();
}

template <class R>
cudaError_t precond_apply(const Plan& P, const cx<R>* r, cx<R>* z, int nvec, const VecCtx& ctx, double2* partial,
                          int nblk, cudaStream_t st) {
  const PlanData<R>& d = detail::pdata<R>(P);
  FAME_LAUNCHED(1);
  k_precond_apply<R><<<dim3(nblk, nvec), kThreads, 0, st>>>(r, z, d.pc, ctx, P.Nq, partial);
  return cudaGetLastError();
}

template <class R>
cudaError_t pcg_update(const Plan& P, cx<R>* x, cx<R>* r, cx<R>* z, const cx<R>* p, const cx<R>* q, int nvec,
                       const VecCtx& ctx, const double* alpha, double2* partial, int nblk, cudaStream_t st,
                       const CgAlpha& ca) {
  const PlanData<R>& d = detail::pdata<R>(P);
  FAME_LAUNCHED(1);
  k_pcg_update<R><<<dim3(nblk, nvec), kThreads, 0, st>>>(x, r, z, p, q, d.pc, ctx, P.Nq, alpha, partial, ca);
  return cudaGetLastError();
}

template cudaError_t build_precond<float>(Plan&, cudaStream_t);
template cudaError_t build_precond<double>(Plan&, cudaStream_t);
template cudaError_t precond_apply<float>(const Plan&, const float2*, float2*, int, const VecCtx&, double2*, int,
                                          cudaStream_t);
template cudaError_t precond_apply<double>(const Plan&, const double2*, double2*, int, const VecCtx&, double2*, int,
                                           cudaStream_t);
template cudaError_t pcg_update<float>(const Plan&, float2*, float2*, float2*, const float2*, const float2*, int,
                                       const VecCtx&, const double*, double2*, int, cudaStream_t, const CgAlpha&);
template cudaError_t pcg_update<double>(const Plan&, double2*, double2*, double2*, const double2*, const double2*, int,
                                        const VecCtx&, const double*, double2*, int, cudaStream_t, const CgAlpha&);

}  // namespace fame
