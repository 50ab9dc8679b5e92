// Eigenvector restoration, ORGSEP residual and field maxima on the GPU.
//
// Eigen_Restoration_Chiral_no_inv.m:3-25: for x = [x1; x2],
//   [e; h] = -i [N J; J^H M] [Qr x2; Pr x1].
// With u = Pr x1, v = Qr x2 this is e = -i v', h = -i u' where [u'; v'] is the
// material operator of fncB applied to [u; v] (fncB.m:4-5): the first half of
// fncB and the stencil give it, in the periodic frame (the Bloch frame is
// S .* that, S the diagonal phase of MtxVecMul_FFT).
//
// EvaluteError_Chiral_no_inv.m:19 (ORGSEP):
//   || [N J; J^H M] [C^H h; -C e] - i omega [e; h] ||
// with C the explicit curl of @DistOp/C.m (forward differences with Bloch
// wrap, mesh length 1/n).  In the periodic frame each difference is
// n (tau_d f(r + e_d) - f(r)); the material product is again the stencil, on
// [u; v] = [-C e; C^H h], giving [h-row; e-row] = [u''; v''].
//
// Fig6cd_plot_max_field.m:58-69: max over components of |e_c| and |h_c|,
// optionally only at vertices outside the inclusion (phase id 0).
#include <cmath>
#include <vector>

#include "fame_internal.h"

namespace fame {
namespace {

constexpr int kT = 256;

// EH = [e; h] = [-i v'; -i u'] from the stencil output w = [u'; v'].
__global__ void k_restore_fields(const double2* __restrict__ w, double2* __restrict__ eh, long long Nq) {
  const long long idx = (long long)blockIdx.x * kT + threadIdx.x;
  const int vec = blockIdx.y;
  if (idx >= Nq) return;
  const double2* wv = w + vec * 6 * Nq + idx;
  double2* o = eh + vec * 6 * Nq + idx;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    o[c * Nq] = cmul_i<-1>(wv[(3 + c) * Nq]);
    o[(3 + c) * Nq] = cmul_i<-1>(wv[c * Nq]);
  }
}

// Y = [-C e; C^H h] (periodic frame): D_d f = n (tau_d f(r+e_d) - f(r)),
// D_d^H g = n (conj(tau_d) g(r-e_d) - g(r)).
__global__ void k_curl_pair(const double2* __restrict__ eh, double2* __restrict__ y, PlanData<double> d, VecCtx ctx,
                            int n) {
  const long long Nq = (long long)n * n * n;
  const long long idx = (long long)blockIdx.x * kT + threadIdx.x;
  const int vec = blockIdx.y;
  if (idx >= Nq) return;
  const int inst = vec_inst(ctx, vec);
  const int i1 = int(idx % n), i2 = int((idx / n) % n), i3 = int(idx / ((long long)n * n));
  const long long sy = n, sz = (long long)n * n;
  const long long dxp = i1 == n - 1 ? -(long long)(n - 1) : 1, dxm = i1 == 0 ? (long long)(n - 1) : -1;
  const long long dyp = i2 == n - 1 ? -(n - 1) * sy : sy, dym = i2 == 0 ? (n - 1) * sy : -sy;
  const long long dzp = i3 == n - 1 ? -(n - 1) * sz : sz, dzm = i3 == 0 ? (n - 1) * sz : -sz;
  const double2* tau = d.tau + inst * 3;
  const double2 tx = tau[0], ty = tau[1], tz = tau[2];
  const double nn = double(n);
  const double2* e = eh + vec * 6 * Nq + idx;
  const double2* h = e + 3 * Nq;
  auto Df = [&](const double2* f, long long dp, double2 t) { return cscale(csub(cmul(t, f[dp]), f[0]), nn); };
  auto Db = [&](const double2* f, long long dm, double2 t) { return cscale(csub(cmulc(t, f[dm]), f[0]), nn); };
  // C e = [-Dz e1 + Dy e2; Dz e0 - Dx e2; -Dy e0 + Dx e1]
  const double2 ce0 = csub(Df(e + 2 * Nq, dyp, ty), Df(e + Nq, dzp, tz));
  const double2 ce1 = csub(Df(e, dzp, tz), Df(e + 2 * Nq, dxp, tx));
  const double2 ce2 = csub(Df(e + Nq, dxp, tx), Df(e, dyp, ty));
  // C^H h = [Dz^H h1 - Dy^H h2; -Dz^H h0 + Dx^H h2; Dy^H h0 - Dx^H h1]
  const double2 ch0 = csub(Db(h + Nq, dzm, tz), Db(h + 2 * Nq, dym, ty));
  const double2 ch1 = csub(Db(h + 2 * Nq, dxm, tx), Db(h, dzm, tz));
  const double2 ch2 = csub(Db(h, dym, ty), Db(h + Nq, dxm, tx));
  double2* o = y + vec * 6 * Nq + idx;
  o[0] = cneg(ce0);
  o[Nq] = cneg(ce1);
  o[2 * Nq] = cneg(ce2);
  o[3 * Nq] = ch0;
  o[4 * Nq] = ch1;
  o[5 * Nq] = ch2;
}

// Per block: sum |v'' - i w e|^2 + |u'' - i w h|^2, max |e_c|, max |h_c|
// (masked to phase id 0 when outside_only).
__global__ void k_orgsep(const double2* __restrict__ y, const double2* __restrict__ eh, const double* __restrict__ om,
                         const uint8_t* __restrict__ phase, int outside_only, long long Nq, double* __restrict__ part) {
  const int vec = blockIdx.y;
  const double w = om[vec];
  double s = 0.0, me = 0.0, mh = 0.0;
  for (long long idx = (long long)blockIdx.x * kT + threadIdx.x; idx < Nq; idx += (long long)gridDim.x * kT) {
    const double2* yv = y + vec * 6 * Nq + idx;
    const double2* e = eh + vec * 6 * Nq + idx;
    const bool use = !outside_only || phase[idx] == 0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const double2 ec = e[c * Nq], hc = e[(3 + c) * Nq];
      const double2 r1 = csub(yv[(3 + c) * Nq], cscale(cmul_i<+1>(ec), w));
      const double2 r2 = csub(yv[c * Nq], cscale(cmul_i<+1>(hc), w));
      s += r1.x * r1.x + r1.y * r1.y + r2.x * r2.x + r2.y * r2.y;
      if (use) {
        me = fmax(me, sqrt(ec.x * ec.x + ec.y * ec.y));
        mh = fmax(mh, sqrt(hc.x * hc.x + hc.y * hc.y));
      }
    }
  }
  __shared__ double rs[kT], re[kT], rh[kT];
  rs[threadIdx.x] = s;
  re[threadIdx.x] = me;
  rh[threadIdx.x] = mh;
  __syncthreads();
  for (int k = kT / 2; k > 0; k >>= 1) {
    if (threadIdx.x < k) {
      rs[threadIdx.x] += rs[threadIdx.x + k];
      re[threadIdx.x] = fmax(re[threadIdx.x], re[threadIdx.x + k]);
      rh[threadIdx.x] = fmax(rh[threadIdx.x], rh[threadIdx.x + k]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double* p = part + ((long long)vec * gridDim.x + blockIdx.x) * 3;
    p[0] = rs[0];
    p[1] = re[0];
    p[2] = rh[0];
  }
}

// E = S .* e, H = S .* h (Bloch frame, the reference's layout: 3Nq each).
__global__ void k_to_bloch(const double2* __restrict__ eh, double2* __restrict__ E, double2* __restrict__ H,
                           PlanData<double> d, VecCtx ctx, int n) {
  const long long Nq = (long long)n * n * n;
  const long long idx = (long long)blockIdx.x * kT + threadIdx.x;
  const int vec = blockIdx.y;
  if (idx >= Nq) return;
  const int i1 = int(idx % n), i2 = int((idx / n) % n), i3 = int(idx / ((long long)n * n));
  const double2* S = d.sxyz + (long long)vec_inst(ctx, vec) * 3 * n;
  const double2 s = cmul(cmul(S[i1], S[n + i2]), S[2 * n + i3]);
  const double2* src = eh + vec * 6 * Nq + idx;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    if (E) E[vec * 3 * Nq + c * Nq + idx] = cmul(s, src[c * Nq]);
    if (H) H[vec * 3 * Nq + c * Nq + idx] = cmul(s, src[(3 + c) * Nq]);
  }
}

}  // namespace
}  // namespace fame

using namespace fame;

extern "C" int fame_restore(fame_plan_t h, int nvec, const int* inst, const void* x, const double* omega, void* E,
                            void* H, double* res_orgsep, double* max_e, double* max_h, int outside_only) {
  if (!h) return FAME_ERR_BAD_ARG;
  Plan& P = h->P;
  if (nvec < 1 || !x || !omega) return fail(&P, FAME_ERR_BAD_ARG, "fame_restore: bad argument");
  if (inst)
    for (int v = 0; v < nvec; ++v)
      if (inst[v] < 0 || inst[v] >= P.nk) return fail(&P, FAME_ERR_BAD_ARG, "fame_restore: bad instance");
  cudaStream_t st = P.stream;
  const long long Nq = P.Nq;
  cudaError_t e = ensure_work(P, (size_t)nvec);
  if (e != cudaSuccess) return cuda_fail(&P, e, "fame_restore work");
  double2* w0 = (double2*)P.d_work;
  double2* w1 = w0 + (size_t)nvec * 6 * Nq;
  const size_t six = sizeof(double2) * 6 * (size_t)Nq * nvec;
  double2* eh = (double2*)workspace(P, 45, six, &e);
  if (e != cudaSuccess) return cuda_fail(&P, e, "fame_restore scratch");
  int* d_inst = nullptr;
  if (inst) {
    d_inst = (int*)workspace(P, 46, sizeof(int) * nvec, &e);
    if (e == cudaSuccess) e = h2d_async(P, d_inst, inst, sizeof(int) * nvec);
    if (e != cudaSuccess) return cuda_fail(&P, e, "fame_restore inst");
  }
  VecCtx ctx;
  ctx.inst = d_inst;
  ctx.nk = P.nk;
  const dim3 g((unsigned)((Nq + kT - 1) / kT), (unsigned)nvec);
#define RS_CK(expr, what)                              \
  do {                                                 \
    cudaError_t e_ = (expr);                           \
    if (e_ != cudaSuccess) return cuda_fail(&P, e_, what); \
  } while (0)
  RS_CK(launch_fields_inv<double>(P, (const double2*)x, w0, nvec, ctx, st), "fame_restore fields");
  RS_CK(launch_stencil<double>(P, w0, w1, nvec, ctx, st), "fame_restore material");
  FAME_LAUNCHED(1);
  k_restore_fields<<<g, kT, 0, st>>>(w0, eh, Nq);
  RS_CK(cudaGetLastError(), "k_restore_fields");
  const bool want_res = res_orgsep || max_e || max_h;
  if (want_res) {
    double* d_om = (double*)workspace(P, 47, sizeof(double) * nvec, &e);
    if (e == cudaSuccess) e = h2d_async(P, d_om, omega, sizeof(double) * nvec);
    RS_CK(e, "fame_restore omega");
    FAME_LAUNCHED(1);
    k_curl_pair<<<g, kT, 0, st>>>(eh, w0, P.d64, ctx, P.n);
    RS_CK(cudaGetLastError(), "k_curl_pair");
    RS_CK(launch_stencil<double>(P, w0, w1, nvec, ctx, st), "fame_restore residual material");
    const int nblk = 152;
    double* part = (double*)workspace(P, 48, sizeof(double) * 3 * nblk * nvec, &e);
    RS_CK(e, "fame_restore partials");
    FAME_LAUNCHED(1);
    k_orgsep<<<dim3(nblk, nvec), kT, 0, st>>>(w0, eh, d_om, P.d_phase, outside_only, Nq, part);
    RS_CK(cudaGetLastError(), "k_orgsep");
    std::vector<double> hp((size_t)3 * nblk * nvec);
    RS_CK(cudaMemcpyAsync(hp.data(), part, sizeof(double) * hp.size(), cudaMemcpyDeviceToHost, st), "orgsep d2h");
    RS_CK(cudaStreamSynchronize(st), "orgsep sync");
    for (int v = 0; v < nvec; ++v) {
      double s = 0.0, me = 0.0, mh = 0.0;
      for (int b = 0; b < nblk; ++b) {
        const double* p = &hp[((size_t)v * nblk + b) * 3];
        s += p[0];
        me = std::fmax(me, p[1]);
        mh = std::fmax(mh, p[2]);
      }
      if (res_orgsep) res_orgsep[v] = std::sqrt(s);
      if (max_e) max_e[v] = me;
      if (max_h) max_h[v] = mh;
    }
  }
  if (E || H) {
    FAME_LAUNCHED(1);
    k_to_bloch<<<g, kT, 0, st>>>(eh, (double2*)E, (double2*)H, P.d64, ctx, P.n);
    RS_CK(cudaGetLastError(), "k_to_bloch");
  }
#undef RS_CK
  return FAME_OK;
}
