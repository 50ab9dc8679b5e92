// Size-independent kernels of fncB (the material stencil, fncA, the Bloch
// phase) and the dispatch from a plan's grid size to the size-templated
// transforms instantiated in fncb_inst_*.cu.
#include "fncb_impl.cuh"

namespace fame {
namespace detail {


// ---------------------------------------------------------------------------
// Material stencil, stage 1: vertex values Hu, Hv from the spatial fields.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int wrapm(int i, int n) { return i == 0 ? n - 1 : i - 1; }
__device__ __forceinline__ int wrapp(int i, int n) { return i == n - 1 ? 0 : i + 1; }

template <class R>
__global__ void __launch_bounds__(256)
k_vertex(const cx<R>* __restrict__ uv, cx<R>* __restrict__ h, PlanData<R> d,
         const uint8_t* __restrict__ phase, int nphase, VecCtx ctx, int n, long long uv_stride,
         long long h_stride) {
  const long long Nq = (long long)n * n * n;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int vec = blockIdx.y;
  if (idx >= Nq) return;
  if (ctx.active && !ctx.active[vec]) return;
  const int inst = vec_inst(ctx, vec);
  const int i1 = int(idx % n), i2 = int((idx / n) % n), i3 = int(idx / ((long long)n * n));
  const long long sx = 1, sy = n, sz = (long long)n * n;
  const long long dxm = (i1 == 0 ? (n - 1) * sx : -sx);
  const long long dym = (i2 == 0 ? (n - 1) * sy : -sy);
  const long long dzm = (i3 == 0 ? (n - 1) * sz : -sz);
  const cx<R>* tau = d.tau + inst * 3;
  const cx<R> tx = cconj(tau[0]), ty = cconj(tau[1]), tz = cconj(tau[2]);
  const cx<R>* f = uv + vec * uv_stride + idx;
  // U_j = 1/4 (I + T_a^H)(I + T_b^H) u_j ; (T^H g)(r) = conj(tau) g(r - e)
  auto face2vtx = [&](const cx<R>* g, long long da, long long db, cx<R> ta, cx<R> tb) {
    cx<R> s = g[0];
    s = cfma(ta, g[da], s);
    s = cfma(tb, g[db], s);
    s = cfma(cmul(ta, tb), g[da + db], s);
    return cscale(s, R(0.25));
  };
  cx<R> U[3], V[3];
  U[0] = face2vtx(f + 0 * Nq, dym, dzm, ty, tz);
  U[1] = face2vtx(f + 1 * Nq, dxm, dzm, tx, tz);
  U[2] = face2vtx(f + 2 * Nq, dxm, dym, tx, ty);
  V[0] = cscale(cfma(tx, f[3 * Nq + dxm], f[3 * Nq]), R(0.5));
  V[1] = cscale(cfma(ty, f[4 * Nq + dym], f[4 * Nq]), R(0.5));
  V[2] = cscale(cfma(tz, f[5 * Nq + dzm], f[5 * Nq]), R(0.5));
  const cx<R>* T = d.mat + ((long long)inst * nphase + phase[idx]) * 27;
  const cx<R>* Nh = T;
  const cx<R>* Mh = T + 9;
  const cx<R>* J = T + 18;
  cx<R>* o = h + vec * h_stride + idx;
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

// ---------------------------------------------------------------------------
// Material stencil, stage 2: face/edge values, in place over u, v.
// ---------------------------------------------------------------------------
template <class R>
__global__ void __launch_bounds__(256)
k_faceedge(cx<R>* __restrict__ uv, const cx<R>* __restrict__ h, PlanData<R> d,
           const uint8_t* __restrict__ phase, int nphase, VecCtx ctx, int n, long long uv_stride,
           long long h_stride) {
  const long long Nq = (long long)n * n * n;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int vec = blockIdx.y;
  if (idx >= Nq) return;
  if (ctx.active && !ctx.active[vec]) return;
  const int inst = vec_inst(ctx, vec);
  const int i1 = int(idx % n), i2 = int((idx / n) % n), i3 = int(idx / ((long long)n * n));
  const long long sx = 1, sy = n, sz = (long long)n * n;
  const long long dxp = (i1 == n - 1 ? -(n - 1) * sx : sx);
  const long long dyp = (i2 == n - 1 ? -(n - 1) * sy : sy);
  const long long dzp = (i3 == n - 1 ? -(n - 1) * sz : sz);
  const cx<R>* tau = d.tau + inst * 3;
  const cx<R> tx = tau[0], ty = tau[1], tz = tau[2];
  // material diagonals at the 8 corners r + {0,1}^3
  const cx<R>* tab = d.mat + (long long)inst * nphase * 27;
  auto reM = [&](long long off, int i) { return tab[phase[idx + off] * 27 + 9 + i * 4].x; };
  auto reN = [&](long long off, int i) { return tab[phase[idx + off] * 27 + 0 + i * 4].x; };
  const cx<R>* hh = h + vec * h_stride + idx;
  cx<R>* f = uv + vec * uv_stride + idx;
  // u'_i = m_i u_i + 1/4 (I+T_a)(I+T_b) Hu_i ; (T g)(r) = tau g(r + e)
  auto vtx2face = [&](const cx<R>* g, long long da, long long db, cx<R> ta, cx<R> tb) {
    cx<R> s = g[0];
    s = cfma(ta, g[da], s);
    s = cfma(tb, g[db], s);
    s = cfma(cmul(ta, tb), g[da + db], s);
    return cscale(s, R(0.25));
  };
  {
    R m0 = R(0.25) * (reM(0, 0) + reM(dyp, 0) + reM(dzp, 0) + reM(dyp + dzp, 0));
    R m1 = R(0.25) * (reM(0, 1) + reM(dxp, 1) + reM(dzp, 1) + reM(dxp + dzp, 1));
    R m2 = R(0.25) * (reM(0, 2) + reM(dxp, 2) + reM(dyp, 2) + reM(dxp + dyp, 2));
    cx<R> r0 = cadd(cscale(f[0], m0), vtx2face(hh, dyp, dzp, ty, tz));
    cx<R> r1 = cadd(cscale(f[Nq], m1), vtx2face(hh + Nq, dxp, dzp, tx, tz));
    cx<R> r2 = cadd(cscale(f[2 * Nq], m2), vtx2face(hh + 2 * Nq, dxp, dyp, tx, ty));
    f[0] = r0;
    f[Nq] = r1;
    f[2 * Nq] = r2;
  }
  {
    R n0 = R(0.5) * (reN(0, 0) + reN(dxp, 0));
    R n1 = R(0.5) * (reN(0, 1) + reN(dyp, 1));
    R n2 = R(0.5) * (reN(0, 2) + reN(dzp, 2));
    const cx<R>* hv = hh + 3 * Nq;
    cx<R> r0 = cadd(cscale(f[3 * Nq], n0), cscale(cfma(tx, hv[dxp], hv[0]), R(0.5)));
    cx<R> r1 = cadd(cscale(f[4 * Nq], n1), cscale(cfma(ty, hv[Nq + dyp], hv[Nq]), R(0.5)));
    cx<R> r2 = cadd(cscale(f[5 * Nq], n2), cscale(cfma(tz, hv[2 * Nq + dzp], hv[2 * Nq]), R(0.5)));
    f[3 * Nq] = r0;
    f[4 * Nq] = r1;
    f[5 * Nq] = r2;
  }
}

// Multiply each 3Nq component block by S (conj when CONJ), in place.
template <class R, bool CONJ>
__global__ void k_phase(cx<R>* __restrict__ v, PlanData<R> d, VecCtx ctx, int n, int nfield,
                        long long stride) {
  const long long Nq = (long long)n * n * n;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int vec = blockIdx.y;
  if (idx >= Nq) return;
  if (ctx.active && !ctx.active[vec]) return;
  const int i1 = int(idx % n), i2 = int((idx / n) % n), i3 = int(idx / ((long long)n * n));
  const cx<R>* S = d.sxyz + (long long)vec_inst(ctx, vec) * 3 * n;
  cx<R> s = cmul(cmul(S[i1], S[n + i2]), S[2 * n + i3]);
  for (int c = 0; c < nfield; ++c) {
    cx<R>* p = v + vec * stride + (long long)c * Nq + idx;
    *p = CONJ ? cmulc(s, *p) : cmul(s, *p);
  }
}

// fncA.m:3-4: y = [ i/Sigma .* x2 ; -i/Sigma .* x1 ], Sigma = [sqrt(Lq); sqrt(Lq)].
template <class R>
__global__ void k_fncA(const cx<R>* __restrict__ x, cx<R>* __restrict__ y, PlanData<R> d, VecCtx ctx,
                       int n) {
  const long long Nq = (long long)n * n * n;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int vec = blockIdx.y;
  if (idx >= Nq) return;
  if (ctx.active && !ctx.active[vec]) return;
  const int i1 = int(idx % n), i2 = int((idx / n) % n), i3 = int(idx / ((long long)n * n));
  const cx<R>* lam = d.lam + (long long)vec_inst(ctx, vec) * 3 * n;
  cx<R> lx = lam[i1], ly = lam[n + i2], lz = lam[2 * n + i3];
  R lq = lx.x * lx.x + lx.y * lx.y + ly.x * ly.x + ly.y * ly.y + lz.x * lz.x + lz.y * lz.y;
  R inv = R(1) / sqrt(lq);
  const cx<R>* xv = x + vec * 4 * Nq + idx;
  cx<R>* yv = y + vec * 4 * Nq + idx;
  cx<R> a1 = xv[0], b1 = xv[Nq], a2 = xv[2 * Nq], b2 = xv[3 * Nq];
  yv[0] = cscale(cmul_i<+1>(a2), inv);
  yv[Nq] = cscale(cmul_i<+1>(b2), inv);
  yv[2 * Nq] = cscale(cmul_i<-1>(a1), inv);
  yv[3 * Nq] = cscale(cmul_i<-1>(b1), inv);
}

inline dim3 grid_pts1(long long Nq, int nvec, int tpb) {
  return dim3((unsigned)((Nq + tpb - 1) / tpb), (unsigned)nvec, 1);
}

template <class R>
cudaError_t stencil(const Plan& P, cx<R>* w0, cx<R>* w1, int nvec, const VecCtx& ctx, cudaStream_t st) {
  const PlanData<R>& d = pdata<R>(P);
  const long long s6 = 6 * P.Nq;
  FAME_LAUNCHED(1);
  k_vertex<R><<<grid_pts1(P.Nq, nvec, 256), 256, 0, st>>>(w0, w1, d, P.d_phase, P.nphase, ctx, P.n, s6, s6);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  FAME_LAUNCHED(1);
  k_faceedge<R><<<grid_pts1(P.Nq, nvec, 256), 256, 0, st>>>(w0, w1, d, P.d_phase, P.nphase, ctx, P.n, s6, s6);
  return cudaGetLastError();
}

template cudaError_t stencil<float>(const Plan&, cx<float>*, cx<float>*, int, const VecCtx&, cudaStream_t);
template cudaError_t stencil<double>(const Plan&, cx<double>*, cx<double>*, int, const VecCtx&, cudaStream_t);

}  // namespace detail

// the size-templated transforms are instantiated elsewhere
#define FAME_EXTERN(NN) extern template FAME_SIZE_SIGS(float, NN) extern template FAME_SIZE_SIGS(double, NN)
}  // namespace fame
FAME_FOR_EACH_N(FAME_EXTERN)
namespace fame {
using namespace detail;

bool n_supported(int n) {
  switch (n) {
#define FAME_CASE(NN) case NN: return NN >= 2;
    FAME_FOR_EACH_N(FAME_CASE)
#undef FAME_CASE
    default: return false;
  }
}

template <class R>
cudaError_t launch_fncB(const Plan& P, const cx<R>* x, cx<R>* y, int nvec, const VecCtx& ctx, cx<R>* w0,
                        cx<R>* w1, cudaStream_t st) {
  if (nvec <= 0) return cudaSuccess;
  switch (P.n) {
#define FAME_CASE(NN) case NN: return fncB_n<R, NN>(P, x, y, nvec, ctx, w0, w1, st);
    FAME_FOR_EACH_N(FAME_CASE)
#undef FAME_CASE
    default: return cudaErrorInvalidValue;
  }
}

template <class R>
cudaError_t launch_fncA(const Plan& P, const cx<R>* x, cx<R>* y, int nvec, const VecCtx& ctx, cudaStream_t st) {
  if (nvec <= 0) return cudaSuccess;
  FAME_LAUNCHED(1);
  k_fncA<R><<<grid_pts1(P.Nq, nvec, 256), 256, 0, st>>>(x, y, pdata<R>(P), ctx, P.n);
  return cudaGetLastError();
}

template <class R>
cudaError_t launch_transform(const Plan& P, int trans, const cx<R>* x, cx<R>* y, int nvec, const VecCtx& ctx,
                             cudaStream_t st) {
  if (nvec <= 0) return cudaSuccess;
  switch (P.n) {
#define FAME_CASE(NN) case NN: return transform_n<R, NN>(P, trans, x, y, nvec, ctx, st);
    FAME_FOR_EACH_N(FAME_CASE)
#undef FAME_CASE
    default: return cudaErrorInvalidValue;
  }
}

template <class R>
cudaError_t launch_handle(const Plan& P, int which, const cx<R>* x, cx<R>* y, int nvec, const VecCtx& ctx,
                          cx<R>* w0, cudaStream_t st) {
  if (nvec <= 0) return cudaSuccess;
  switch (P.n) {
#define FAME_CASE(NN) case NN: return handle_n<R, NN>(P, which, x, y, nvec, ctx, w0, st);
    FAME_FOR_EACH_N(FAME_CASE)
#undef FAME_CASE
    default: return cudaErrorInvalidValue;
  }
}

template <class R>
cudaError_t launch_material(const Plan& P, const cx<R>* uv, cx<R>* out, int nvec, const VecCtx& ctx, cx<R>* w1,
                            cudaStream_t st) {
  // Bloch frame in and out: strip S, apply the periodic-frame stencil, restore S.
  if (nvec <= 0) return cudaSuccess;
  const long long s6 = 6 * P.Nq;
  cudaError_t e;
  if (out != uv) {
    e = cudaMemcpyAsync(out, uv, sizeof(cx<R>) * s6 * nvec, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return e;
  }
  const PlanData<R>& d = pdata<R>(P);
  FAME_LAUNCHED(1);
  k_phase<R, true><<<grid_pts1(P.Nq, nvec, 256), 256, 0, st>>>(out, d, ctx, P.n, 6, s6);
  e = stencil<R>(P, out, w1, nvec, ctx, st);
  if (e != cudaSuccess) return e;
  FAME_LAUNCHED(1);
  k_phase<R, false><<<grid_pts1(P.Nq, nvec, 256), 256, 0, st>>>(out, d, ctx, P.n, 6, s6);
  return cudaGetLastError();
}

#define FAME_INST(R)                                                                                      \
  template cudaError_t launch_fncB<R>(const Plan&, const cx<R>*, cx<R>*, int, const VecCtx&, cx<R>*,     \
                                      cx<R>*, cudaStream_t);                                              \
  template cudaError_t launch_fncA<R>(const Plan&, const cx<R>*, cx<R>*, int, const VecCtx&,             \
                                      cudaStream_t);                                                      \
  template cudaError_t launch_transform<R>(const Plan&, int, const cx<R>*, cx<R>*, int, const VecCtx&,   \
                                           cudaStream_t);                                                 \
  template cudaError_t launch_handle<R>(const Plan&, int, const cx<R>*, cx<R>*, int, const VecCtx&,      \
                                        cx<R>*, cudaStream_t);                                            \
  template cudaError_t launch_material<R>(const Plan&, const cx<R>*, cx<R>*, int, const VecCtx&, cx<R>*, \
                                          cudaStream_t);
FAME_INST(float)
FAME_INST(double)

}  // namespace fame
