// Per-vertex chiral media (field mode) and the adjoint gradient of
// eigenfrequencies with respect to the per-vertex fields.
//
// Field mode: eps(r) I, mu = I, xi = i gamma(r) I, zeta = -i gamma(r) I at every
// vertex.  The inverse of [eps I, i gamma I; -i gamma I, I] is
//   1/(eps - gamma^2) [I, -i gamma I; i gamma I, eps I],
// so the covariant blocks A^T X A (Physical_settings_woodpile.m:184-194) are
//   N = a G,  M = b G,  J = -i g G,   a = 1/(eps - gamma^2), b = eps a, g = gamma a,
// with G = A^T A the Gram matrix of the primitive vectors.  The stencil kernels
// evaluate these per vertex from [3][Nq] = a | b | g (fncb_material.cuh).
//
// Gradient (Hellmann-Feynman): for A x = lambda B x with omega = 1/lambda and
// only B depending on the material,
//   d omega / dp = omega * x^H (dB/dp) x / (x^H B x).
// With w = [u; v] the periodic-frame fields of x (first half of fncB) and the
// vertex gathers U_j = 1/4 (I+T_a)^H (I+T_b)^H u_j, V_j = 1/2 (I+T_j)^H v_j,
//   x^H B x = sum_vertices q,  q = b Qu + a Qv + 2 g Im(Quv),
//   Qu  = sum_i G_ii Au_i + sum_{i!=j} G_ij Re(conj(U_i) U_j),
//   Qv  = sum_i G_ii Av_i + sum_{i!=j} G_ij Re(conj(V_i) V_j),
//   Quv = sum_ij G_ij conj(V_i) U_j,
//   Au_i = 1/4 sum of |u_i|^2 over the four faces meeting at the vertex in
//          plane i, Av_i = 1/2 (|v_i(r)|^2 + |v_i(r - e_i)|^2)
// (the lumped diagonals m_i, n_i of the stencil redistribute to the vertices
// this way).  dq/d eps and dq/d gamma at each vertex follow from
//   da/deps = -a^2, db/deps = -gamma^2 a^2, dg/deps = -gamma a^2,
//   da/dgamma = 2 gamma a^2, db/dgamma = 2 eps gamma a^2, dg/dgamma = a (1 + 2 gamma^2 a).
// All of it in FP64.  No counterpart in the reference.
#include <cmath>
#include <complex>
#include <string>
#include <vector>

#include "fame_internal.h"

namespace fame {
namespace {

struct VertexQuads {
  double qu, qv;
  double2 quv;
};

__device__ __forceinline__ VertexQuads vertex_quads(const double2* __restrict__ f, long long Nq, int n,
                                                    long long idx, double2 tx, double2 ty, double2 tz,
                                                    const double* __restrict__ G) {
  const int i1 = int(idx % n), i2 = int((idx / n) % n), i3 = int(idx / ((long long)n * n));
  const long long dxm = i1 == 0 ? n - 1 : -1;
  const long long dym = i2 == 0 ? (long long)(n - 1) * n : -(long long)n;
  const long long dzm = i3 == 0 ? (long long)(n - 1) * n * n : -(long long)n * n;
  auto a2 = [](double2 z) { return z.x * z.x + z.y * z.y; };
  auto face = [&](const double2* g, long long da, long long db, double2 ta, double2 tb, double& au) {
    double2 s = g[0];
    s = cfma(ta, g[da], s);
    s = cfma(tb, g[db], s);
    s = cfma(cmul(ta, tb), g[da + db], s);
    au = 0.25 * (a2(g[0]) + a2(g[da]) + a2(g[db]) + a2(g[da + db]));
    return cscale(s, 0.25);
  };
  double2 U[3], V[3];
  double Au[3], Av[3];
  U[0] = face(f, dym, dzm, ty, tz, Au[0]);
  U[1] = face(f + Nq, dxm, dzm, tx, tz, Au[1]);
  U[2] = face(f + 2 * Nq, dxm, dym, tx, ty, Au[2]);
  const double2* v0 = f + 3 * Nq;
  const double2* v1 = f + 4 * Nq;
  const double2* v2 = f + 5 * Nq;
  V[0] = cscale(cfma(tx, v0[dxm], v0[0]), 0.5);
  V[1] = cscale(cfma(ty, v1[dym], v1[0]), 0.5);
  V[2] = cscale(cfma(tz, v2[dzm], v2[0]), 0.5);
  Av[0] = 0.5 * (a2(v0[0]) + a2(v0[dxm]));
  Av[1] = 0.5 * (a2(v1[0]) + a2(v1[dym]));
  Av[2] = 0.5 * (a2(v2[0]) + a2(v2[dzm]));
  VertexQuads r{0.0, 0.0, make_double2(0.0, 0.0)};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    r.qu += G[i * 4] * Au[i];
    r.qv += G[i * 4] * Av[i];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const double gij = G[i * 3 + j];
      if (j != i) {
        r.qu += gij * (U[i].x * U[j].x + U[i].y * U[j].y);
        r.qv += gij * (V[i].x * V[j].x + V[i].y * V[j].y);
      }
      r.quv = cadd(r.quv, cscale(cmulc(V[i], U[j]), gij));
    }
  }
  return r;
}

struct GradParams {
  double G[9];
};

constexpr int kGradThreads = 256;

// q summed per vector (x^H B x), one partial per block.
__global__ void __launch_bounds__(kGradThreads)
k_quad_sum(const double2* __restrict__ w, const double* __restrict__ fld, PlanData<double> d, VecCtx ctx, int n,
           GradParams gp, double* __restrict__ partial) {
  const long long Nq = (long long)n * n * n;
  const int vec = blockIdx.y;
  const int inst = vec_inst(ctx, vec);
  const double2 tx = cconj(d.tau[inst * 3]), ty = cconj(d.tau[inst * 3 + 1]), tz = cconj(d.tau[inst * 3 + 2]);
  double acc = 0.0;
  for (long long idx = (long long)blockIdx.x * kGradThreads + threadIdx.x; idx < Nq;
       idx += (long long)gridDim.x * kGradThreads) {
    VertexQuads q = vertex_quads(w + vec * 6 * Nq + idx, Nq, n, idx, tx, ty, tz, gp.G);
    acc += fld[Nq + idx] * q.qu + fld[idx] * q.qv + 2.0 * fld[2 * Nq + idx] * q.quv.y;
  }
  __shared__ double red[kGradThreads];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kGradThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[(long long)vec * gridDim.x + blockIdx.x] = red[0];
}

// g_eps, g_gamma (+)= sum_v scale_v dq_v/dp at every vertex.
__global__ void __launch_bounds__(kGradThreads)
k_grad(const double2* __restrict__ w, const double* __restrict__ fld, const double* __restrict__ eg,
       PlanData<double> d, VecCtx ctx, int n, int nvec, GradParams gp, const double* __restrict__ scale,
       double* __restrict__ g_eps, double* __restrict__ g_gam, int accumulate) {
  const long long Nq = (long long)n * n * n;
  const long long idx = (long long)blockIdx.x * kGradThreads + threadIdx.x;
  if (idx >= Nq) return;
  const double a = fld[idx], eps = eg[idx], gam = eg[Nq + idx];
  const double a2 = a * a;
  const double db_de = -gam * gam * a2, da_de = -a2, dg_de = -gam * a2;
  const double db_dg = 2.0 * eps * gam * a2, da_dg = 2.0 * gam * a2, dg_dg = a * (1.0 + 2.0 * gam * gam * a);
  double se = 0.0, sg = 0.0;
  for (int vec = 0; vec < nvec; ++vec) {
    const double s = scale[vec];
    if (s == 0.0) continue;
    const int inst = vec_inst(ctx, vec);
    const double2 tx = cconj(d.tau[inst * 3]), ty = cconj(d.tau[inst * 3 + 1]), tz = cconj(d.tau[inst * 3 + 2]);
    VertexQuads q = vertex_quads(w + vec * 6 * Nq + idx, Nq, n, idx, tx, ty, tz, gp.G);
    se += s * (db_de * q.qu + da_de * q.qv + 2.0 * dg_de * q.quv.y);
    sg += s * (db_dg * q.qu + da_dg * q.qv + 2.0 * dg_dg * q.quv.y);
  }
  if (accumulate) {
    g_eps[idx] += se;
    g_gam[idx] += sg;
  } else {
    g_eps[idx] = se;
    g_gam[idx] = sg;
  }
}

template <class R>
int upload_field(Plan& P, PlanData<R>& d, const std::vector<double>& abg) {
  if (!d.fld) {
    cudaError_t e = cudaMalloc(&d.fld, sizeof(R) * 3 * (size_t)P.Nq);
    if (e != cudaSuccess) return cuda_fail(&P, e, "field arrays");
  }
  std::vector<R> h(abg.size());
  for (size_t i = 0; i < abg.size(); ++i) h[i] = R(abg[i]);
  cudaError_t e = cudaMemcpy(d.fld, h.data(), sizeof(R) * h.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(&P, e, "field upload");
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double g = 0.0;  // G = A^T A, A with the primitive vectors as columns
      for (int k = 0; k < 3; ++k) g += P.lattice[k * 3 + i] * P.lattice[k * 3 + j];
      d.gram[i * 3 + j] = R(g);
    }
  return FAME_OK;
}

// Validates and installs the fields: a | b | g arrays in both precisions, the
// FP64 (eps, gamma) copy for the gradient, the volume-averaged tensors of the
// preconditioner (rebuilt lazily).
int set_field(Plan& P, const double* eps, const double* gam) {
  const long long Nq = P.Nq;
  std::vector<double> abg(3 * (size_t)Nq);
  double sa = 0.0, sb = 0.0, sg = 0.0;
  for (long long i = 0; i < Nq; ++i) {
    const double e = eps[i], g = gam[i];
    if (!std::isfinite(e) || !std::isfinite(g) || !(e > 0.0) || !(e - g * g > 0.0))
      return fail(&P, FAME_ERR_BAD_ARG,
                  "field: eps > 0 and eps - gamma^2 > 0 required at vertex " + std::to_string(i));
    const double a = 1.0 / (e - g * g);
    abg[i] = a;
    abg[Nq + i] = e * a;
    abg[2 * Nq + i] = g * a;
    sa += a;
    sb += e * a;
    sg += g * a;
  }
  P.eps_host.assign(eps, eps + Nq);
  P.gam_host.assign(gam, gam + Nq);
  int rc = upload_field<double>(P, P.d64, abg);
  if (rc == FAME_OK) rc = upload_field<float>(P, P.d32, abg);
  if (rc == FAME_OK) rc = upload_tables_ds(P);  // the double-single copies, fields included
  if (rc != FAME_OK) return rc;
  cudaError_t e = cudaSuccess;
  if (!P.d_eps_gam) e = cudaMalloc(&P.d_eps_gam, sizeof(double) * 2 * (size_t)Nq);
  if (e == cudaSuccess) e = cudaMemcpy(P.d_eps_gam, eps, sizeof(double) * Nq, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(P.d_eps_gam + Nq, gam, sizeof(double) * Nq, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(&P, e, "field upload");
  // averaged tensors: Herm(N) = <a> G, Herm(M) = <b> G, J = -i <g> G
  sa /= double(Nq);
  sb /= double(Nq);
  sg /= double(Nq);
  P.mat_avg.assign((size_t)P.nk * 54, 0.0);
  for (int k = 0; k < P.nk; ++k)
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        const double G = double(P.d64.gram[i * 3 + j]);
        double* m = &P.mat_avg[(size_t)k * 54];
        m[(0 * 9 + i * 3 + j) * 2] = sa * G;
        m[(1 * 9 + i * 3 + j) * 2] = sb * G;
        m[(2 * 9 + i * 3 + j) * 2 + 1] = -sg * G;
      }
  // the preconditioner depends on the averaged tensors: rebuild on next use
  cudaFree(P.d64.pc);
  cudaFree(P.d32.pc);
  P.d64.pc = nullptr;
  P.d32.pc = nullptr;
  cudaFree(P.d_mat_avg);
  P.d_mat_avg = nullptr;
  free_graphs(P);  // captured CG iterations hold the preconditioner's address
  return FAME_OK;
}

}  // namespace
}  // namespace fame

using namespace fame;

extern "C" {

int fame_plan_create_field(fame_plan_t* out, int n, int nk, const double* theta, const double* lattice,
                           const double* eps, const double* gamma) {
  if (!out) return FAME_ERR_BAD_ARG;
  *out = nullptr;
  if (n < 2 || nk < 1 || !theta || !lattice || !eps || !gamma) return FAME_ERR_BAD_ARG;
  const long long Nq = (long long)n * n * n;
  std::vector<uint8_t> phase((size_t)Nq, 0);
  std::vector<double> tens((size_t)nk * 54, 0.0);  // unused phase table (field mode reads the fields)
  fame_plan_t h = nullptr;
  int rc = fame_plan_create(&h, n, nk, theta, phase.data(), 1, tens.data());
  if (rc != FAME_OK) return rc;
  Plan& P = h->P;
  P.field_mode = true;
  for (int i = 0; i < 9; ++i) P.lattice[i] = lattice[i];
  rc = set_field(P, eps, gamma);
  if (rc != FAME_OK) {
    fame_plan_destroy(h);
    return rc;
  }
  *out = h;
  return FAME_OK;
}

int fame_set_field(fame_plan_t h, const double* eps, const double* gamma) {
  if (!h || !eps || !gamma) return FAME_ERR_BAD_ARG;
  Plan& P = h->P;
  if (!P.field_mode) return fail(&P, FAME_ERR_BAD_ARG, "fame_set_field: plan is not in field mode");
  cudaError_t e = cudaStreamSynchronize(P.stream);
  if (e != cudaSuccess) return cuda_fail(&P, e, "fame_set_field");
  return set_field(P, eps, gamma);
}

int fame_eig_gradient(fame_plan_t h, int nvec, const int* inst, const void* x, const double* omega,
                      const double* weight, double* g_eps, double* g_gamma, int accumulate, double* xbx) {
  if (!h) return FAME_ERR_BAD_ARG;
  Plan& P = h->P;
  if (!P.field_mode) return fail(&P, FAME_ERR_UNSUPPORTED, "fame_eig_gradient: needs a field-mode plan");
  if (nvec < 1 || !x || !omega || !weight || !g_eps || !g_gamma)
    return fail(&P, FAME_ERR_BAD_ARG, "fame_eig_gradient: bad argument");
  if (inst)
    for (int v = 0; v < nvec; ++v)
      if (inst[v] < 0 || inst[v] >= P.nk) return fail(&P, FAME_ERR_BAD_ARG, "fame_eig_gradient: bad instance");
  cudaStream_t st = P.stream;
  cudaError_t e = ensure_work(P, (size_t)nvec);
  if (e != cudaSuccess) return cuda_fail(&P, e, "fame_eig_gradient work");
  double2* w = (double2*)P.d_work;
  int* d_inst = nullptr;
  if (inst) {
    d_inst = (int*)workspace(P, 40, sizeof(int) * nvec, &e);
    if (e == cudaSuccess) e = h2d_async(P, d_inst, inst, sizeof(int) * nvec);
    if (e != cudaSuccess) return cuda_fail(&P, e, "fame_eig_gradient inst");
  }
  VecCtx ctx;
  ctx.inst = d_inst;
  ctx.nk = P.nk;
  e = launch_fields_inv<double>(P, (const double2*)x, w, nvec, ctx, st);
  if (e != cudaSuccess) return cuda_fail(&P, e, "fame_eig_gradient fields");
  GradParams gp;
  for (int i = 0; i < 9; ++i) gp.G[i] = P.d64.gram[i];
  const int nblk = 152;
  double* partial = (double*)workspace(P, 41, sizeof(double) * nblk * nvec, &e);
  if (e != cudaSuccess) return cuda_fail(&P, e, "fame_eig_gradient scratch");
  FAME_LAUNCHED(1);
  k_quad_sum<<<dim3(nblk, nvec), kGradThreads, 0, st>>>(w, P.d64.fld, P.d64, ctx, P.n, gp, partial);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(&P, e, "k_quad_sum");
  std::vector<double> hp((size_t)nblk * nvec);
  e = cudaMemcpyAsync(hp.data(), partial, sizeof(double) * hp.size(), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(&P, e, "fame_eig_gradient norm");
  std::vector<double> scale(nvec);
  for (int v = 0; v < nvec; ++v) {
    double s = 0.0;
    for (int b = 0; b < nblk; ++b) s += hp[(size_t)v * nblk + b];
    if (xbx) xbx[v] = s;
    if (!(s > 0.0) || !std::isfinite(s)) return fail(&P, FAME_ERR_NAN, "fame_eig_gradient: x^H B x is not positive");
    scale[v] = weight[v] * omega[v] / s;
  }
  double* d_scale = (double*)workspace(P, 42, sizeof(double) * nvec, &e);
  if (e == cudaSuccess) e = h2d_async(P, d_scale, scale.data(), sizeof(double) * nvec);
  if (e != cudaSuccess) return cuda_fail(&P, e, "fame_eig_gradient scale");
  FAME_LAUNCHED(1);
  k_grad<<<(unsigned)((P.Nq + kGradThreads - 1) / kGradThreads), kGradThreads, 0, st>>>(
      w, P.d64.fld, P.d_eps_gam, P.d64, ctx, P.n, nvec, gp, d_scale, g_eps, g_gamma, accumulate);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(&P, e, "k_grad");
  return FAME_OK;
}

}  // extern "C"
