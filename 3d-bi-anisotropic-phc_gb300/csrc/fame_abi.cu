// C ABI of the FAME GB300 library: plan life cycle and operator handles.
#include <cuda_runtime.h>

#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "fame_internal.h"
#include "krylov.h"
#include "linalg_host.h"


namespace fame {

// Error text of calls that have no plan to hold it (per thread: plans may be
// created from several threads at once).
static thread_local std::string g_static_error;

int fail(Plan* P, int code, const std::string& msg) {
  if (P)
    P->last_error = msg;
  else
    g_static_error = msg;
  return code;
}

int cuda_fail(Plan* P, cudaError_t e, const char* where) {
  std::string m = std::string(where) + ": " + cudaGetErrorString(e);
  return fail(P, FAME_ERR_CUDA, m);
}

template <class R> PlanData<R>& pdata_mut(Plan& P);
template <> PlanData<double>& pdata_mut<double>(Plan& P) { return P.d64; }
template <> PlanData<float>& pdata_mut<float>(Plan& P) { return P.d32; }

unsigned long long g_kernel_launches = 0;
unsigned long long g_host_launches = 0;

void* workspace(Plan& P, int id, size_t bytes, cudaError_t* err) {
  *err = cudaSuccess;
  if ((size_t)id >= P.ws_ptr.size()) {
    P.ws_ptr.resize(id + 1, nullptr);
    P.ws_size.resize(id + 1, 0);
  }
  if (bytes <= P.ws_size[id]) return P.ws_ptr[id];
  if (P.ws_ptr[id]) cudaFree(P.ws_ptr[id]);
  P.ws_ptr[id] = nullptr;
  P.ws_size[id] = 0;
  *err = cudaMalloc(&P.ws_ptr[id], bytes);
  if (*err != cudaSuccess) return nullptr;
  P.ws_size[id] = bytes;
  return P.ws_ptr[id];
}

constexpr size_t kRingBytes = 1 << 20;

cudaError_t h2d_async(Plan& P, void* dst, const void* src, size_t bytes) {
  if (bytes == 0) return cudaSuccess;
  if (!P.h_ring) {
    cudaError_t e = cudaMallocHost((void**)&P.h_ring, kRingBytes);
    if (e != cudaSuccess) return e;
    P.ring_pos = 0;
  }
  if (bytes > kRingBytes) return cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
  if (P.ring_pos + bytes > kRingBytes) {  // wrap only once earlier copies have been consumed
    cudaError_t e = cudaStreamSynchronize(P.stream);
    if (e != cudaSuccess) return e;
    P.ring_pos = 0;
  }
  char* slot = P.h_ring + P.ring_pos;
  std::memcpy(slot, src, bytes);
  P.ring_pos += (bytes + 255) & ~size_t(255);
  return cudaMemcpyAsync(dst, slot, bytes, cudaMemcpyHostToDevice, P.stream);
}

void free_workspaces(Plan& P) {
  for (void* p : P.ws_ptr) cudaFree(p);
  P.ws_ptr.clear();
  P.ws_size.clear();
}

// Grow-only device scratch of the plan.
cudaError_t ensure_work(Plan& P, size_t vecs) {
  if (vecs <= P.work_vecs) return cudaSuccess;
  if (P.d_work) cudaFree(P.d_work);
  P.d_work = nullptr;
  P.work_vecs = 0;
  size_t bytes = vecs * 2 * 6 * (size_t)P.Nq * sizeof(double2);
  cudaError_t e = cudaMalloc(&P.d_work, bytes);
  if (e == cudaSuccess) P.work_vecs = vecs;
  return e;
}

cudaError_t upload_inst(Plan& P, const int* inst_host, int nvec, const int** d_inst_out) {
  *d_inst_out = nullptr;
  if (!inst_host) return cudaSuccess;
  if ((size_t)nvec > P.inst_cap) {
    if (P.d_inst) cudaFree(P.d_inst);
    P.d_inst = nullptr;
    P.inst_cap = 0;
    cudaError_t e = cudaMalloc(&P.d_inst, sizeof(int) * nvec);
    if (e != cudaSuccess) return e;
    P.inst_cap = nvec;
  }
  cudaError_t e = cudaMemcpyAsync(P.d_inst, inst_host, sizeof(int) * nvec, cudaMemcpyHostToDevice, P.stream);
  *d_inst_out = P.d_inst;
  return e;
}

cudaError_t ensure_stage(Plan& P, size_t bytes) {
  if (bytes <= P.stage_bytes) return cudaSuccess;
  if (P.d_stage) cudaFree(P.d_stage);
  P.d_stage = nullptr;
  P.stage_bytes = 0;
  cudaError_t e = cudaMalloc(&P.d_stage, bytes);
  if (e == cudaSuccess) P.stage_bytes = bytes;
  return e;
}

template <class R>
int upload_tables(Plan& P) {
  PlanData<R>& d = pdata_mut<R>(P);
  const int n = P.n, nk = P.nk;
  std::vector<cx<R>> lam((size_t)nk * 3 * n), tau((size_t)nk * 3), sx((size_t)nk * 3 * n);
  for (int k = 0; k < nk; ++k) {
    for (int ax = 0; ax < 3; ++ax) {
      const double th = P.theta[k * 3 + ax];
      for (int j = 0; j < n; ++j) {
        // @DistOp/lambda_QuasiPeriodic.m:3 with delta = 1/n: (exp(i(2(j)pi/n + theta/n)) - 1)/delta
        const double phi = 2.0 * (double(j) * kPi / n) + th / n;
        std::complex<double> l = (std::exp(std::complex<double>(0.0, phi)) - 1.0) / (1.0 / n);
        lam[(size_t)k * 3 * n + ax * n + j] = mk<R>(R(l.real()), R(l.imag()));
        // @DistOp/S_sDFT.m:2
        std::complex<double> s = std::exp(std::complex<double>(0.0, double(j) * th / n));
        sx[(size_t)k * 3 * n + ax * n + j] = mk<R>(R(s.real()), R(s.imag()));
      }
      std::complex<double> t = std::exp(std::complex<double>(0.0, th / n));
      tau[k * 3 + ax] = mk<R>(R(t.real()), R(t.imag()));
    }
  }
  // material table: Herm(N) | Herm(M) | J per (instance, phase)
  std::vector<cx<R>> mat((size_t)nk * P.nphase * 27);
  for (size_t t = 0; t < (size_t)nk * P.nphase; ++t) {
    const double* src = &P.mat_host[t * 54];
    auto at = [&](int blk, int i, int j) {
      return std::complex<double>(src[(blk * 9 + i * 3 + j) * 2], src[(blk * 9 + i * 3 + j) * 2 + 1]);
    };
    for (int blk = 0; blk < 3; ++blk)
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          std::complex<double> v = at(blk, i, j);
          if (blk < 2) v = 0.5 * (v + std::conj(at(blk, j, i)));
          mat[t * 27 + blk * 9 + i * 3 + j] = mk<R>(R(v.real()), R(v.imag()));
        }
  }
  cudaError_t e;
  e = cudaMalloc(&d.lam, sizeof(cx<R>) * lam.size());
  if (e == cudaSuccess) e = cudaMalloc(&d.tau, sizeof(cx<R>) * tau.size());
  if (e == cudaSuccess) e = cudaMalloc(&d.sxyz, sizeof(cx<R>) * sx.size());
  if (e == cudaSuccess) e = cudaMalloc(&d.mat, sizeof(cx<R>) * mat.size());
  if (e != cudaSuccess) return cuda_fail(&P, e, "plan tables");
  e = cudaMemcpy(d.lam, lam.data(), sizeof(cx<R>) * lam.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d.tau, tau.data(), sizeof(cx<R>) * tau.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d.sxyz, sx.data(), sizeof(cx<R>) * sx.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d.mat, mat.data(), sizeof(cx<R>) * mat.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(&P, e, "plan tables upload");
  // Pi table for complex128 only: there the transform kernels are bound by
  // GB300's FP64 rate and reading Pi (96 B per voxel) beats evaluating it
  // (617 -> 496 us per n = 60 fncB vector); the complex64 kernels are
  // issue-bound with L2 traffic to spare, and the extra 48 B per voxel made
  // them slower (298 -> 314 us per 10 vectors), so they evaluate Pi.
  if (sizeof(R) == 8) {
    e = build_pi_table<R>(P);
    if (e != cudaSuccess) return cuda_fail(&P, e, "plan Pi table");
  }
  return FAME_OK;
}

template <class R> void free_tables(PlanData<R>& d) {
  cudaFree(d.lam);
  cudaFree(d.tau);
  cudaFree(d.sxyz);
  cudaFree(d.mat);
  cudaFree(d.pc);
  cudaFree(d.pi);
  cudaFree(d.fld);
  d = PlanData<R>();
}

// Sigma_r = sqrt(Lq) must be non-zero and Pi1's normaliser |conj(L) x w| too
// (SVD_Matrix_curl.m:49-53 divides by both).
int check_singular(Plan& P) {
  const int n = P.n;
  const double w[3] = {1.0 / std::sqrt(14.0), 2.0 / std::sqrt(14.0), 3.0 / std::sqrt(14.0)};
  P.sigma_min.assign(P.nk, 0.0);
  for (int k = 0; k < P.nk; ++k) {
    double lqmin = 1e300;
    std::vector<std::complex<double>> l(3 * n);
    for (int ax = 0; ax < 3; ++ax)
      for (int j = 0; j < n; ++j) {
        const double phi = 2.0 * (double(j) * kPi / n) + P.theta[k * 3 + ax] / n;
        l[ax * n + j] = (std::exp(std::complex<double>(0.0, phi)) - 1.0) * double(n);
      }
    for (int i3 = 0; i3 < n; ++i3)
      for (int i2 = 0; i2 < n; ++i2)
        for (int i1 = 0; i1 < n; ++i1) {
          std::complex<double> L[3] = {l[i1], l[n + i2], l[2 * n + i3]};
          double lq = std::norm(L[0]) + std::norm(L[1]) + std::norm(L[2]);
          lqmin = std::min(lqmin, lq);
          std::complex<double> lw = w[0] * L[0] + w[1] * L[1] + w[2] * L[2];
          double n1 = lq - std::norm(lw);
          if (!(lq > 0.0) || !(n1 > 1e-300)) {
            char buf[200];
            std::snprintf(buf, sizeof(buf),
                          "singular curl SVD at instance %d voxel (%d,%d,%d): |L|^2=%g (shift a zero wave vector, "
                          "as the reference does with +1e-4)",
                          k, i1, i2, i3, lq);
            return fail(&P, FAME_ERR_SINGULAR, buf);
          }
        }
    P.sigma_min[k] = std::sqrt(lqmin);
  }
  return FAME_OK;
}

size_t elem_size(int prec) { return prec == FAME_C64 ? sizeof(float2) : sizeof(double2); }

}  // namespace fame

using namespace fame;

extern "C" {

const char* fame_version(void) { return "fame-gb300 0.1 (sm_103a)"; }

long long fame_kernel_launches(void) { return (long long)__atomic_load_n(&g_kernel_launches, __ATOMIC_RELAXED); }
long long fame_host_launches(void) { return (long long)__atomic_load_n(&g_host_launches, __ATOMIC_RELAXED); }

int fame_plan_create(fame_plan_t* out, int n, int nk, const double* theta, const uint8_t* phase, int nphase,
                     const double* tensors) {
  if (!out) return FAME_ERR_BAD_ARG;
  *out = nullptr;
  if (n < 2 || nk < 1 || !theta || !phase || nphase < 1 || nphase > 256 || !tensors) {
    g_static_error = "fame_plan_create: bad argument";
    return FAME_ERR_BAD_ARG;
  }
  if (!n_supported(n)) {
    g_static_error = "fame_plan_create: grid size n=" + std::to_string(n) +
                     " has no compiled transform (n must be one of the FAME_FOR_EACH_N sizes)";
    return FAME_ERR_UNSUPPORTED;
  }
  fame_plan_s* h = new fame_plan_s();
  Plan& P = h->P;
  P.n = n;
  P.Nq = (long long)n * n * n;
  P.nk = nk;
  P.nphase = nphase;
  P.theta.assign(theta, theta + 3 * nk);
  P.mat_host.assign(tensors, tensors + (size_t)nk * nphase * 54);
  for (long long i = 0; i < P.Nq; ++i)
    if (phase[i] >= nphase) {
      g_static_error = "fame_plan_create: phase id out of range";
      delete h;
      return FAME_ERR_BAD_ARG;
    }
  for (double t : P.theta)
    if (!std::isfinite(t)) {
      g_static_error = "fame_plan_create: non-finite theta";
      delete h;
      return FAME_ERR_BAD_ARG;
    }
  // volume-averaged Herm(N) | Herm(M) | J per instance (CG preconditioner)
  {
    std::vector<double> frac(nphase, 0.0);
    for (long long i = 0; i < P.Nq; ++i) frac[phase[i]] += 1.0;
    for (double& f : frac) f /= double(P.Nq);
    P.mat_avg.assign((size_t)nk * 54, 0.0);
    for (int k = 0; k < nk; ++k)
      for (int ph = 0; ph < nphase; ++ph) {
        const double* src = &P.mat_host[((size_t)k * nphase + ph) * 54];
        for (int blk = 0; blk < 3; ++blk)
          for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
              const int a = (blk * 9 + i * 3 + j) * 2, t = (blk * 9 + j * 3 + i) * 2;
              double re = src[a], im = src[a + 1];
              if (blk < 2) {  // Hermitian part of N and M
                re = 0.5 * (re + src[t]);
                im = 0.5 * (im - src[t + 1]);
              }
              P.mat_avg[(size_t)k * 54 + a] += frac[ph] * re;
              P.mat_avg[(size_t)k * 54 + a + 1] += frac[ph] * im;
            }
      }
  }
  int rc = check_singular(P);
  if (rc != FAME_OK) {
    g_static_error = P.last_error;
    delete h;
    return rc;
  }
  cudaError_t e = cudaGetDevice(&P.device);
  if (e == cudaSuccess) e = cudaMalloc(&P.d_phase, P.Nq);
  if (e == cudaSuccess) e = cudaMemcpy(P.d_phase, phase, P.Nq, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    g_static_error = std::string("fame_plan_create: ") + cudaGetErrorString(e);
    delete h;
    return FAME_ERR_CUDA;
  }
  rc = upload_tables<double>(P);
  if (rc == FAME_OK) rc = upload_tables<float>(P);
  if (rc == FAME_OK) rc = upload_tables_ds(P);
  if (rc != FAME_OK) {
    g_static_error = P.last_error;
    fame_plan_destroy(h);
    return rc;
  }
  *out = h;
  return FAME_OK;
}

int fame_plan_destroy(fame_plan_t h) {
  if (!h) return FAME_OK;
  Plan& P = h->P;
  if (P.stream) cudaStreamSynchronize(P.stream);
  else cudaDeviceSynchronize();
  free_tables(P.d64);
  free_tables(P.d32);
  free_tables(P.dds);
  cudaFree(P.d_phase);
  cudaFree(P.d_work);
  cudaFree(P.d_inst);
  cudaFree(P.d_red);
  cudaFree(P.d_stage);
  cudaFree(P.d_mat_avg);
  cudaFree(P.d_eps_gam);
  free_graphs(P);
  if (P.h_ring) cudaFreeHost(P.h_ring);
  free_workspaces(P);
  delete h;
  return FAME_OK;
}

int fame_set_option(fame_plan_t h, int option, double value) {
  if (!h) return FAME_ERR_BAD_ARG;
  Plan& P = h->P;
  switch (option) {
    case FAME_OPT_PRECOND:
      P.opt_precond = value != 0.0;
      return FAME_OK;
    case FAME_OPT_GRAPH:
      P.opt_graph = value <= 0.0 ? 0 : value < 1.5 ? 1 : 2;
      return FAME_OK;
    case FAME_OPT_SIRA_NEAREST:
      P.opt_sira_nearest = value != 0.0;
      return FAME_OK;
    case FAME_OPT_PI_TABLE:
      P.opt_pi_table = value != 0.0;
      free_graphs(P);  // captured sequences hold the old kernel arguments
      return FAME_OK;
    case FAME_OPT_REFINE:
      P.opt_refine = value != 0.0;
      return FAME_OK;
    case FAME_OPT_C64_ROUND:
      P.opt_c64_round = value != 0.0;
      return FAME_OK;
    case FAME_OPT_RELAX:
      if (!(value >= 0.0 && value < 1.0)) return fail(&P, FAME_ERR_BAD_ARG, "fame_set_option: relax must be in [0, 1)");
      P.opt_relax = value;
      return FAME_OK;
    case FAME_OPT_DS_RESIDUAL:
      P.opt_ds_residual = value != 0.0;
      return FAME_OK;
    case FAME_OPT_RELAX_MAX:
      if (!(value >= 1.0 && value <= 1e8)) return fail(&P, FAME_ERR_BAD_ARG, "fame_set_option: relax_max must be in [1, 1e8]");
      P.opt_relax_max = value;
      return FAME_OK;
    case FAME_OPT_REFINE_TOL:
      if (!(value > 0.0 && value < 1.0)) return fail(&P, FAME_ERR_BAD_ARG, "fame_set_option: refine tol in (0, 1)");
      P.opt_refine_tol = value;
      return FAME_OK;
    case FAME_OPT_PLANE_SPLIT:
      P.opt_plane_split = value != 0.0;
      free_graphs(P);  // captured sequences hold the old kernels
      return FAME_OK;
    case FAME_OPT_ITOL_FLOOR:
      if (!(value > 0.0 && value < 1.0)) return fail(&P, FAME_ERR_BAD_ARG, "fame_set_option: itol floor in (0, 1)");
      P.opt_itol_floor = value;
      return FAME_OK;
    case FAME_OPT_TOL32:
      if (!(value > 0.0 && value < 1.0)) return fail(&P, FAME_ERR_BAD_ARG, "fame_set_option: tol32 in (0,1)");
      P.opt_tol32 = value;
      return FAME_OK;
    default:
      return fail(&P, FAME_ERR_BAD_ARG, "fame_set_option: unknown option");
  }
}

int fame_set_stream(fame_plan_t h, void* stream) {
  if (!h) return FAME_ERR_BAD_ARG;
  h->P.stream = reinterpret_cast<cudaStream_t>(stream);
  return FAME_OK;
}

int fame_sync(fame_plan_t h) {
  if (!h) return FAME_ERR_BAD_ARG;
  cudaError_t e = cudaStreamSynchronize(h->P.stream);
  return e == cudaSuccess ? FAME_OK : cuda_fail(&h->P, e, "fame_sync");
}

int fame_refine_residuals(fame_plan_t h, double* before, int n) {
  if (!h) return fail(nullptr, FAME_ERR_BAD_ARG, "fame_refine_residuals: null plan");
  const std::vector<double>& r = h->P.refine_res_before;
  if (before)
    for (int i = 0; i < n && i < (int)r.size(); ++i) before[i] = r[i];
  return (int)r.size();
}

const char* fame_last_error(fame_plan_t h) { return h ? h->P.last_error.c_str() : g_static_error.c_str(); }

int fame_plan_info(fame_plan_t h, int* n, int* nk, long long* nq) {
  if (!h) return FAME_ERR_BAD_ARG;
  if (n) *n = h->P.n;
  if (nk) *nk = h->P.nk;
  if (nq) *nq = h->P.Nq;
  return FAME_OK;
}

}  // extern "C"

namespace fame {

// Common wrapper: argument checks, instance upload, host staging.
// in_len / out_len: complex elements per vector.  body(x_dev, y_dev, ctx).
template <class F>
int run_op(fame_plan_t h, int prec, const void* x, void* y, int nvec, const int* inst, int flags, long long in_len,
           long long out_len, const char* name, F&& body) {
  if (!h) return FAME_ERR_BAD_ARG;
  Plan& P = h->P;
  if (prec != FAME_C128 && prec != FAME_C64 && !(prec == FAME_C128_DS && std::string(name) == "fame_apply_B"))
    return fail(&P, FAME_ERR_BAD_ARG, std::string(name) + ": bad precision");
  if (prec == FAME_C128_DS && !ds_supported(P.n))
    return fail(&P, FAME_ERR_UNSUPPORTED, std::string(name) + ": no double-single fncB for this grid size");
  if (nvec < 0 || (nvec > 0 && (!x || !y))) return fail(&P, FAME_ERR_BAD_ARG, std::string(name) + ": bad vectors");
  if (nvec == 0) return FAME_OK;
  if (inst)
    for (int v = 0; v < nvec; ++v)
      if (inst[v] < 0 || inst[v] >= P.nk) return fail(&P, FAME_ERR_BAD_ARG, std::string(name) + ": bad instance index");
  const size_t es = elem_size(prec);
  const void* xd = x;
  void* yd = y;
  cudaError_t e;
  if (flags & FAME_HOST_PTR) {
    const size_t ib = es * in_len * nvec, ob = es * out_len * nvec;
    e = ensure_stage(P, ib + ob);
    if (e != cudaSuccess) return cuda_fail(&P, e, name);
    char* base = static_cast<char*>(P.d_stage);
    e = cudaMemcpyAsync(base, x, ib, cudaMemcpyHostToDevice, P.stream);
    if (e != cudaSuccess) return cuda_fail(&P, e, name);
    xd = base;
    yd = base + ib;
  }
  VecCtx ctx;
  ctx.nk = P.nk;
  e = upload_inst(P, inst, nvec, &ctx.inst);
  if (e != cudaSuccess) return cuda_fail(&P, e, name);
  int rc = body(xd, yd, ctx);
  if (rc != FAME_OK) return rc;
  if (flags & FAME_HOST_PTR) {
    e = cudaMemcpyAsync(y, yd, es * out_len * nvec, cudaMemcpyDeviceToHost, P.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(P.stream);
    if (e != cudaSuccess) return cuda_fail(&P, e, name);
  }
  return FAME_OK;
}

}  // namespace fame

extern "C" {

int fame_apply_A(fame_plan_t h, int prec, const void* x, void* y, int nvec, const int* inst, int flags) {
  if (!h) return FAME_ERR_BAD_ARG;
  const long long L = 4 * h->P.Nq;
  return run_op(h, prec, x, y, nvec, inst, flags, L, L, "fame_apply_A", [&](const void* xd, void* yd, const VecCtx& ctx) {
    cudaError_t e = prec == FAME_C64
                        ? launch_fncA<float>(h->P, (const float2*)xd, (float2*)yd, nvec, ctx, h->P.stream)
                        : launch_fncA<double>(h->P, (const double2*)xd, (double2*)yd, nvec, ctx, h->P.stream);
    return e == cudaSuccess ? FAME_OK : cuda_fail(&h->P, e, "fame_apply_A");
  });
}

int fame_apply_B(fame_plan_t h, int prec, const void* x, void* y, int nvec, const int* inst, int flags) {
  if (!h) return FAME_ERR_BAD_ARG;
  Plan& P = h->P;
  const long long L = 4 * P.Nq;
  return run_op(h, prec, x, y, nvec, inst, flags, L, L, "fame_apply_B", [&](const void* xd, void* yd, const VecCtx& ctx) {
    cudaError_t e = ensure_work(P, nvec);
    if (e != cudaSuccess) return cuda_fail(&P, e, "fame_apply_B scratch");
    if (prec == FAME_C64) {
      float2* w0 = (float2*)P.d_work;
      float2* w1 = w0 + (size_t)nvec * 6 * P.Nq;
      e = launch_fncB<float>(P, (const float2*)xd, (float2*)yd, nvec, ctx, w0, w1, P.stream);
    } else if (prec == FAME_C128_DS) {
      e = launch_fncB_ds(P, (const double2*)xd, (double2*)yd, nvec, ctx, P.stream);
    } else {
      double2* w0 = (double2*)P.d_work;
      double2* w1 = w0 + (size_t)nvec * 6 * P.Nq;
      e = launch_fncB<double>(P, (const double2*)xd, (double2*)yd, nvec, ctx, w0, w1, P.stream);
    }
    return e == cudaSuccess ? FAME_OK : cuda_fail(&P, e, "fame_apply_B");
  });
}

int fame_curl_transform(fame_plan_t h, int prec, int trans, const void* x, void* y, int nvec, const int* inst,
                        int flags) {
  if (!h) return FAME_ERR_BAD_ARG;
  if (trans != 0 && trans != 1) return fail(&h->P, FAME_ERR_BAD_ARG, "fame_curl_transform: trans must be 0 or 1");
  const long long L = 3 * h->P.Nq;
  return run_op(h, prec, x, y, nvec, inst, flags, L, L, "fame_curl_transform",
                [&](const void* xd, void* yd, const VecCtx& ctx) {
                  cudaError_t e =
                      prec == FAME_C64
                          ? launch_transform<float>(h->P, trans, (const float2*)xd, (float2*)yd, nvec, ctx, h->P.stream)
                          : launch_transform<double>(h->P, trans, (const double2*)xd, (double2*)yd, nvec, ctx,
                                                     h->P.stream);
                  return e == cudaSuccess ? FAME_OK : cuda_fail(&h->P, e, "fame_curl_transform");
                });
}

int fame_apply_handle(fame_plan_t h, int prec, int which, const void* x, void* y, int nvec, const int* inst,
                      int flags) {
  if (!h) return FAME_ERR_BAD_ARG;
  Plan& P = h->P;
  if (which < 0 || which > 3) return fail(&P, FAME_ERR_BAD_ARG, "fame_apply_handle: bad handle");
  const long long Lin = (which < 2 ? 2 : 3) * P.Nq, Lout = (which < 2 ? 3 : 2) * P.Nq;
  return run_op(h, prec, x, y, nvec, inst, flags, Lin, Lout, "fame_apply_handle",
                [&](const void* xd, void* yd, const VecCtx& ctx) {
                  cudaError_t e = ensure_work(P, nvec);
                  if (e != cudaSuccess) return cuda_fail(&P, e, "fame_apply_handle scratch");
                  e = prec == FAME_C64 ? launch_handle<float>(P, which, (const float2*)xd, (float2*)yd, nvec, ctx,
                                                              (float2*)P.d_work, P.stream)
                                       : launch_handle<double>(P, which, (const double2*)xd, (double2*)yd, nvec,
                                                               ctx, (double2*)P.d_work, P.stream);
                  return e == cudaSuccess ? FAME_OK : cuda_fail(&P, e, "fame_apply_handle");
                });
}

int fame_apply_material(fame_plan_t h, int prec, const void* x, void* y, int nvec, const int* inst, int flags) {
  if (!h) return FAME_ERR_BAD_ARG;
  Plan& P = h->P;
  const long long L = 6 * P.Nq;
  return run_op(h, prec, x, y, nvec, inst, flags, L, L, "fame_apply_material",
                [&](const void* xd, void* yd, const VecCtx& ctx) {
                  cudaError_t e = ensure_work(P, nvec);
                  if (e != cudaSuccess) return cuda_fail(&P, e, "fame_apply_material scratch");
                  e = prec == FAME_C64 ? launch_material<float>(P, (const float2*)xd, (float2*)yd, nvec, ctx,
                                                                (float2*)P.d_work, P.stream)
                                       : launch_material<double>(P, (const double2*)xd, (double2*)yd, nvec, ctx,
                                                                 (double2*)P.d_work, P.stream);
                  return e == cudaSuccess ? FAME_OK : cuda_fail(&P, e, "fame_apply_material");
                });
}

int fame_apply_Binv(fame_plan_t h, int prec, const void* x, void* y, int nvec, const int* inst, double tol, int maxit,
                    int* iters, double* relres, int flags) {
  if (!h) return FAME_ERR_BAD_ARG;
  Plan& P = h->P;
  if (!(tol > 0.0) || maxit < 1) return fail(&P, FAME_ERR_BAD_ARG, "fame_apply_Binv: tol > 0 and maxit >= 1 required");
  const long long L = 4 * P.Nq;
  return run_op(h, prec, x, y, nvec, inst, flags, L, L, "fame_apply_Binv",
                [&](const void* xd, void* yd, const VecCtx& ctx) {
                  return prec == FAME_C64
                             ? pcg_batched<float>(P, (const float2*)xd, (float2*)yd, nvec, ctx.inst, tol, maxit, iters,
                                                  relres)
                             : pcg_batched<double>(P, (const double2*)xd, (double2*)yd, nvec, ctx.inst, tol, maxit,
                                                   iters, relres);
                });
}

int fame_material_blocks(const double* c6, const double* lattice, double* out) {
  if (!c6 || !lattice || !out) return fail(nullptr, FAME_ERR_BAD_ARG, "fame_material_blocks: null pointer");
  std::complex<double> M[36], Inv[36];
  for (int i = 0; i < 36; ++i) M[i] = std::complex<double>(c6[2 * i], c6[2 * i + 1]);
  if (!invert_complex(M, Inv, 6))
    return fail(nullptr, FAME_ERR_SINGULAR, "fame_material_blocks: singular constitutive block");
  // A: columns = primitive vectors; X_cov = A^T X A (Physical_settings_woodpile.m:184-194)
  const int off[3][2] = {{0, 0}, {3, 3}, {0, 3}};  // (1,1)=eps^-1 part -> N, (2,2) -> M, (1,2) -> J
  for (int b = 0; b < 3; ++b)
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        std::complex<double> s = 0.0;
        for (int p = 0; p < 3; ++p)
          for (int q = 0; q < 3; ++q)
            s += lattice[p * 3 + i] * Inv[(off[b][0] + p) * 6 + off[b][1] + q] * lattice[q * 3 + j];
        out[(b * 9 + i * 3 + j) * 2] = s.real();
        out[(b * 9 + i * 3 + j) * 2 + 1] = s.imag();
      }
  return FAME_OK;
}

}  // extern "C"
