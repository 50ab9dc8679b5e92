// Material stencil of fncB on the six spatial fields (periodic frame):
//   stage 1 (k_vertex)  : U_j, V_j gathered to every vertex, Hu, Hv = vertex
//                         tensor products  -> scratch h
//   stage 2 (k_faceedge): u'_i = m_i u_i + 1/4 (I+T_a)(I+T_b) Hu_i,
//                         v'_i = n_i v_i + 1/2 (I+T_i) Hv_i   (in place)
// One thread per vertex / voxel.  Size templated (instantiated per grid size
// with the transforms in fncb_inst_*.cu) so that the index arithmetic is
// 32-bit with compile-time divisors.
//
// A fused single-kernel form (tiles with a one-voxel halo in shared memory)
// reads and writes each field once instead of three / two times, but it
// recomputes stage 1 on the halo; at n = 60 that cost more issue slots than
// the DRAM traffic it saved, so the two-kernel form is kept.
#pragma once

#include "fame_internal.h"

namespace fame {
namespace detail {

template <class R> inline const PlanData<R>& pdata(const Plan& P);
template <> inline const PlanData<double>& pdata<double>(const Plan& P) { return P.d64; }
template <> inline const PlanData<float>& pdata<float>(const Plan& P) { return P.d32; }

template <class R, int N>
__global__ void __launch_bounds__(512)
k_vertex(const cx<R>* __restrict__ uv, cx<R>* __restrict__ h, PlanData<R> d,
         const uint8_t* __restrict__ phase, int nphase, VecCtx ctx, long long stride) {
  constexpr int NN = N * N, Nq = NN * N;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  const int vec = blockIdx.y;
  if (idx >= Nq) return;
  if (ctx.active && !ctx.active[vec]) return;
  const int inst = vec_inst(ctx, vec);
  const int i1 = idx % N, i2 = (idx / N) % N, i3 = idx / NN;
  const int dxm = i1 == 0 ? N - 1 : -1;
  const int dym = i2 == 0 ? (N - 1) * N : -N;
  const int dzm = i3 == 0 ? (N - 1) * NN : -NN;
  const cx<R>* tau = d.tau + inst * 3;
  const cx<R> tx = cconj(tau[0]), ty = cconj(tau[1]), tz = cconj(tau[2]);
  const cx<R>* f = uv + vec * stride + idx;
  // U_j = 1/4 (I + T_a^H)(I + T_b^H) u_j ; (T^H g)(r) = conj(tau) g(r - e)
  auto face2vtx = [&](const cx<R>* g, int da, int db, cx<R> ta, cx<R> tb) {
    cx<R> s = g[0];
    s = cfma(ta, g[da], s);
    s = cfma(tb, g[db], s);
    s = cfma(cmul(ta, tb), g[da + db], s);
    return cscale(s, R(0.25));
  };
  cx<R> U[3], V[3];
  U[0] = face2vtx(f, dym, dzm, ty, tz);
  U[1] = face2vtx(f + Nq, dxm, dzm, tx, tz);
  U[2] = face2vtx(f + 2 * Nq, dxm, dym, tx, ty);
  V[0] = cscale(cfma(tx, f[3 * Nq + dxm], f[3 * Nq]), R(0.5));
  V[1] = cscale(cfma(ty, f[4 * Nq + dym], f[4 * Nq]), R(0.5));
  V[2] = cscale(cfma(tz, f[5 * Nq + dzm], f[5 * Nq]), R(0.5));
  cx<R>* o = h + vec * stride + idx;
  if (d.fld) {  // field mode: Mh = b G, Nh = a G, J = -i g G
    const R a = d.fld[idx], b = d.fld[Nq + idx], g = d.fld[2 * Nq + idx];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      cx<R> su = zero<R>(), sv = zero<R>();
#pragma unroll
      for (int j = 0; j < 3; ++j)
        if (j != i) {
          su = cadd(su, cscale(U[j], d.gram[i * 3 + j]));
          sv = cadd(sv, cscale(V[j], d.gram[i * 3 + j]));
        }
      const cx<R> tu = cadd(su, cscale(U[i], d.gram[i * 4])), tv = cadd(sv, cscale(V[i], d.gram[i * 4]));
      // Hu_i = b sum_{j!=i} G_ij U_j + i g sum_j G_ij V_j ; Hv_i = a sum_{j!=i} G_ij V_j - i g sum_j G_ij U_j
      o[i * Nq] = cadd(cscale(su, b), cscale(cmul_i<+1>(tv), g));
      o[(3 + i) * Nq] = cadd(cscale(sv, a), cscale(cmul_i<-1>(tu), g));
    }
    return;
  }
  const cx<R>* T = d.mat + (inst * nphase + __ldg(phase + idx)) * 27;
  const cx<R>* Nh = T;
  const cx<R>* Mh = T + 9;
  const cx<R>* J = T + 18;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    cx<R> hu = zero<R>(), hv = zero<R>();
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      if (j != i) {
        hu = cfma(Mh[i * 3 + j], U[j], hu);
        hv = cfma(Nh[i * 3 + j], V[j], hv);
      }
      hu = cfmac(J[j * 3 + i], V[j], hu);
      hv = cfma(J[i * 3 + j], U[j], hv);
    }
    o[i * Nq] = hu;
    o[(3 + i) * Nq] = hv;
  }
}

template <class R, int N>
__global__ void __launch_bounds__(512)
k_faceedge(cx<R>* __restrict__ uv, const cx<R>* __restrict__ h, PlanData<R> d,
           const uint8_t* __restrict__ phase, int nphase, VecCtx ctx, long long stride) {
  constexpr int NN = N * N, Nq = NN * N;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  const int vec = blockIdx.y;
  if (idx >= Nq) return;
  if (ctx.active && !ctx.active[vec]) return;
  const int inst = vec_inst(ctx, vec);
  const int i1 = idx % N, i2 = (idx / N) % N, i3 = idx / NN;
  const int dxp = i1 == N - 1 ? -(N - 1) : 1;
  const int dyp = i2 == N - 1 ? -(N - 1) * N : N;
  const int dzp = i3 == N - 1 ? -(N - 1) * NN : NN;
  const cx<R>* tau = d.tau + inst * 3;
  const cx<R> tx = tau[0], ty = tau[1], tz = tau[2];
  // material diagonals at the corners r + {0,1}^3
  R m0, m1, m2, n0, n1, n2;
  if (d.fld) {  // field mode: Re Mh_ii = b G_ii, Re Nh_ii = a G_ii
    const R* fa = d.fld + idx;
    const R* fb = d.fld + Nq + idx;
    m0 = R(0.25) * d.gram[0] * (fb[0] + fb[dyp] + fb[dzp] + fb[dyp + dzp]);
    m1 = R(0.25) * d.gram[4] * (fb[0] + fb[dxp] + fb[dzp] + fb[dxp + dzp]);
    m2 = R(0.25) * d.gram[8] * (fb[0] + fb[dxp] + fb[dyp] + fb[dxp + dyp]);
    n0 = R(0.5) * d.gram[0] * (fa[0] + fa[dxp]);
    n1 = R(0.5) * d.gram[4] * (fa[0] + fa[dyp]);
    n2 = R(0.5) * d.gram[8] * (fa[0] + fa[dzp]);
  } else {
    const cx<R>* tab = d.mat + inst * nphase * 27;
    const uint8_t* ph = phase + idx;
    const int p000 = __ldg(ph), p100 = __ldg(ph + dxp), p010 = __ldg(ph + dyp), p001 = __ldg(ph + dzp);
    const int p110 = __ldg(ph + dxp + dyp), p101 = __ldg(ph + dxp + dzp), p011 = __ldg(ph + dyp + dzp);
    auto reM = [&](int p, int i) { return tab[p * 27 + 9 + i * 4].x; };
    auto reN = [&](int p, int i) { return tab[p * 27 + i * 4].x; };
    m0 = R(0.25) * (reM(p000, 0) + reM(p010, 0) + reM(p001, 0) + reM(p011, 0));
    m1 = R(0.25) * (reM(p000, 1) + reM(p100, 1) + reM(p001, 1) + reM(p101, 1));
    m2 = R(0.25) * (reM(p000, 2) + reM(p100, 2) + reM(p010, 2) + reM(p110, 2));
    n0 = R(0.5) * (reN(p000, 0) + reN(p100, 0));
    n1 = R(0.5) * (reN(p000, 1) + reN(p010, 1));
    n2 = R(0.5) * (reN(p000, 2) + reN(p001, 2));
  }
  const cx<R>* hh = h + vec * stride + idx;
  cx<R>* f = uv + vec * stride + idx;
  // u'_i = m_i u_i + 1/4 (I+T_a)(I+T_b) Hu_i ; (T g)(r) = tau g(r + e)
  auto vtx2face = [&](const cx<R>* g, int da, int db, cx<R> ta, cx<R> tb) {
    cx<R> s = g[0];
    s = cfma(ta, g[da], s);
    s = cfma(tb, g[db], s);
    s = cfma(cmul(ta, tb), g[da + db], s);
    return cscale(s, R(0.25));
  };
  cx<R> r[6];
  r[0] = cadd(cscale(f[0], m0), vtx2face(hh, dyp, dzp, ty, tz));
  r[1] = cadd(cscale(f[Nq], m1), vtx2face(hh + Nq, dxp, dzp, tx, tz));
  r[2] = cadd(cscale(f[2 * Nq], m2), vtx2face(hh + 2 * Nq, dxp, dyp, tx, ty));
  const cx<R>* hv = hh + 3 * Nq;
  r[3] = cadd(cscale(f[3 * Nq], n0), cscale(cfma(tx, hv[dxp], hv[0]), R(0.5)));
  r[4] = cadd(cscale(f[4 * Nq], n1), cscale(cfma(ty, hv[Nq + dyp], hv[Nq]), R(0.5)));
  r[5] = cadd(cscale(f[5 * Nq], n2), cscale(cfma(tz, hv[2 * Nq + dzp], hv[2 * Nq]), R(0.5)));
#pragma unroll
  for (int c = 0; c < 6; ++c) f[c * Nq] = r[c];
}

// In place on w (6-field vectors, stride 6*Nq), scratch h of the same size;
// tpb threads per block (128, 256 or 512).
template <class R, int N>
cudaError_t stencil_n(const Plan& P, cx<R>* w, cx<R>* h, int nvec, const VecCtx& ctx, cudaStream_t st,
                      int tpb = 256) {
  constexpr int Nq = N * N * N;
  if (tpb != 128 && tpb != 512) tpb = 256;
  const dim3 g((Nq + tpb - 1) / tpb, nvec);
  FAME_LAUNCHED(1);
  k_vertex<R, N><<<g, tpb, 0, st>>>(w, h, pdata<R>(P), P.d_phase, P.nphase, ctx, 6LL * Nq);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  FAME_LAUNCHED(1);
  k_faceedge<R, N><<<g, tpb, 0, st>>>(w, h, pdata<R>(P), P.d_phase, P.nphase, ctx, 6LL * Nq);
  return cudaGetLastError();
}

}  // namespace detail
}  // namespace fame
