// Host drivers of the Krylov glue: batched conjugate gradients on B
// (fncinvB), the mixed-precision B^{-1} used by the complex64 band solve,
// and the thick-restart Lanczos band solver of fun_Lanczos/Lanczos.m.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "graph_impl.h"
#include "krylov.h"
#include "linalg_host.h"

namespace fame {

enum WsId {
  WS_PCG_R = 0, WS_PCG_P, WS_PCG_Q, WS_PCG_SCAL, WS_PCG_PART,
  WS_MIX_B32, WS_MIX_X32, WS_MIX_RES, WS_MIX_MASK, WS_MIX_BD, WS_PCG_Z,
  WS_LZ_Q, WS_LZ_BQ, WS_LZ_VEC, WS_LZ_TMP, WS_LZ_COEF, WS_LZ_INST, WS_LZ_MASK, WS_LZ_U, WS_LZ_SCAL, WS_LZ_DOT,
  WS_LZ_PART,
  WS_LZ_Q32 = 190, WS_LZ_BQ32, WS_LZ_GSPART, WS_LZ_SPAN,
  WS_RF_X = 200, WS_RF_AX, WS_RF_BX, WS_RF_Y, WS_RF_BY, WS_RF_AY, WS_RF_R, WS_RF_Z, WS_RF_INST, WS_RF_G, WS_RF_C,
  WS_RF_PART, WS_PCG_PART2
};

#define FAME_CK(expr, where)                      \
  do {                                            \
    cudaError_t e_ = (expr);                      \
    if (e_ != cudaSuccess) return cuda_fail(&P, e_, where); \
  } while (0)

static int device_sms(int dev) {
  static std::atomic<int> cache[64];
  if (dev < 0 || dev >= 64) dev = 0;
  int v = cache[dev].load(std::memory_order_relaxed);
  if (v <= 0) {
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 152;
    cache[dev].store(v, std::memory_order_relaxed);
  }
  return v;
}

// CTAs per vector of the grid-stride reduction and update kernels: together
// at most four per SM (one wave at four resident CTAs, two at two), so that
// no CTA of a batch waits for a partial last wave.
static int dot_blocks(const Plan& P, long long len, int nvec) {
  long long target = std::max(1, 4 * device_sms(P.device) / std::max(1, nvec));
  long long maxb = (len + 2047) / 2048;
  long long b = std::min(target, maxb);
  if (b < 1) b = 1;
  if (b > 512) b = 512;
  return int(b);
}

// Device scalars of the batched CG, carved from one workspace.
struct CgScalars {
  double *rho, *alpha, *beta, *tol2b2, *res2;
  int *active, *iters;
  int* passes;  // passes of the graph-resident iteration loop
  double2* dot;
};

template <class R>
int pcg_batched(Plan& P, const cx<R>* b, cx<R>* x, int nvec, const int* d_inst, double tol, int maxit, int* iters_out,
                double* relres_out, const unsigned char* h_mask, const double* tolv) {
  if (nvec <= 0) return FAME_OK;
  cudaStream_t st = P.stream;
  const long long L = 4 * P.Nq;
  const size_t vb = sizeof(cx<R>) * L * nvec;
  cudaError_t e;
  cx<R>* r = (cx<R>*)workspace(P, WS_PCG_R + (sizeof(R) == 4 ? 100 : 0), vb, &e);
  FAME_CK(e, "pcg workspace");
  cx<R>* p = (cx<R>*)workspace(P, WS_PCG_P + (sizeof(R) == 4 ? 100 : 0), vb, &e);
  FAME_CK(e, "pcg workspace");
  cx<R>* q = (cx<R>*)workspace(P, WS_PCG_Q + (sizeof(R) == 4 ? 100 : 0), vb, &e);
  FAME_CK(e, "pcg workspace");
  const size_t sb = (5 * sizeof(double) + 2 * sizeof(int) + sizeof(double2)) * nvec + 4 * sizeof(int) + 64;
  char* s = (char*)workspace(P, WS_PCG_SCAL, sb, &e);
  FAME_CK(e, "pcg workspace");
  CgScalars S;
  S.dot = (double2*)s;
  S.rho = (double*)(S.dot + nvec);
  S.alpha = S.rho + nvec;
  S.beta = S.alpha + nvec;
  S.tol2b2 = S.beta + nvec;
  S.res2 = S.tol2b2 + nvec;
  S.active = (int*)(S.res2 + nvec);
  S.iters = S.active + nvec;
  S.passes = S.iters + nvec;
  const int nblk = dot_blocks(P, L, nvec);
  // p^H B p from the stencil pass of fncB where its tuned form provides it
  const int nblk_pq = fncB_pq_partials<R>(P, nvec);
  const int nblkv0 = dot_blocks(P, P.Nq, nvec);
  const int npart = std::max(std::max(nblk, nblk_pq), nblkv0);
  double2* part = (double2*)workspace(P, WS_PCG_PART, sizeof(double2) * npart * nvec + 64, &e);
  FAME_CK(e, "pcg workspace");
  double2* part2 = (double2*)workspace(P, WS_PCG_PART2, sizeof(double2) * nblkv0 * nvec + 64, &e);
  FAME_CK(e, "pcg workspace");
  FAME_CK(ensure_work(P, nvec), "pcg fncB scratch");
  cx<R>* w0 = (cx<R>*)P.d_work;
  cx<R>* w1 = w0 + (size_t)nvec * 6 * P.Nq;

  std::vector<int> act(nvec, 1);
  if (h_mask)
    for (int v = 0; v < nvec; ++v) act[v] = h_mask[v] ? 1 : 0;
  FAME_CK(h2d_async(P, S.active, act.data(), sizeof(int) * nvec), "pcg init");
  // ||b||^2 per vector
  FAME_CK(dot_batched<R>(b, L, 0, 1, b, L, L, nvec, S.dot, part, nblk, S.active, st), "pcg dot");
  std::vector<double2> bb(nvec);
  FAME_CK(cudaMemcpyAsync(bb.data(), S.dot, sizeof(double2) * nvec, cudaMemcpyDeviceToHost, st), "pcg init");
  FAME_CK(cudaStreamSynchronize(st), "pcg init");
  std::vector<double> rho(nvec), t2(nvec);
  for (int v = 0; v < nvec; ++v) {
    rho[v] = bb[v].x;
    const double tv = tolv ? tolv[v] : tol;
    t2[v] = tv * tv * bb[v].x;
    if (act[v] && !std::isfinite(bb[v].x)) return fail(&P, FAME_ERR_NAN, "pcg: non-finite right-hand side");
    if (act[v] && !(bb[v].x > 0.0)) {  // zero right-hand side: x = 0
      act[v] = 0;
    }
  }
  std::vector<int> it0(nvec, 0);
  const std::vector<double> zero_beta(nvec, 0.0);  // the first direction is z itself
  FAME_CK(h2d_async(P, S.beta, zero_beta.data(), sizeof(double) * nvec), "pcg init");
  FAME_CK(h2d_async(P, S.rho, rho.data(), sizeof(double) * nvec), "pcg init");
  FAME_CK(h2d_async(P, S.tol2b2, t2.data(), sizeof(double) * nvec), "pcg init");
  FAME_CK(h2d_async(P, S.res2, rho.data(), sizeof(double) * nvec), "pcg init");
  FAME_CK(h2d_async(P, S.iters, it0.data(), sizeof(int) * nvec), "pcg init");
  for (int v = 0; v < nvec; ++v) {
    const bool sel = h_mask ? h_mask[v] != 0 : true;
    if (!sel) continue;
    FAME_CK(cudaMemsetAsync(x + (size_t)v * L, 0, sizeof(cx<R>) * L, st), "pcg init");
  }
  FAME_CK(h2d_async(P, S.active, act.data(), sizeof(int) * nvec), "pcg init");
  FAME_CK(cudaMemcpyAsync(r, b, vb, cudaMemcpyDeviceToDevice, st), "pcg init");
  VecCtx ctx;
  ctx.inst = d_inst;
  ctx.active = S.active;
  ctx.nk = P.nk;
  // Preconditioned CG (M = B0^{-1}, precond.cu) or plain CG as in fncinvB.m.
  const bool pre = P.opt_precond != 0;
  cx<R>* z = nullptr;
  const int nblkv = dot_blocks(P, P.Nq, nvec);  // per-voxel fused kernels
  if (pre) {
    z = (cx<R>*)workspace(P, WS_PCG_Z + (sizeof(R) == 4 ? 100 : 0), vb, &e);
    FAME_CK(e, "pcg workspace");
    FAME_CK(build_precond<R>(P, st), "pcg preconditioner");
    FAME_CK(precond_apply<R>(P, b, z, nvec, ctx, part, nblkv, st), "pcg precond");
    FAME_CK(cudaMemcpyAsync(p, z, vb, cudaMemcpyDeviceToDevice, st), "pcg init");
    FAME_CK(dot_final(part, nblkv, nvec, S.dot, st), "pcg precond");
    std::vector<double2> rz(nvec);
    FAME_CK(cudaMemcpyAsync(rz.data(), S.dot, sizeof(double2) * nvec, cudaMemcpyDeviceToHost, st), "pcg init");
    FAME_CK(cudaStreamSynchronize(st), "pcg init");
    for (int v = 0; v < nvec; ++v) rho[v] = act[v] ? rz[v].x : 0.0;
    FAME_CK(h2d_async(P, S.rho, rho.data(), sizeof(double) * nvec), "pcg init");
    FAME_CK(cudaStreamSynchronize(st), "pcg init");
  } else {
    FAME_CK(cudaMemcpyAsync(p, b, vb, cudaMemcpyDeviceToDevice, st), "pcg init");
  }
  // One CG iteration: every kernel reads its scalars and active flags from
  // the device, so a block of iterations is a fixed launch sequence that is
  // captured once per (sizes, pointers) and replayed from a CUDA graph.
  //   p = z + beta p, q = B p         (the update done by fncB's first kernel;
  //                                     beta = 0 before the first iteration;
  //                                     with the partials of p^H q when the
  //                                     stencil pass provides them)
  //   alpha = rho / p^H q             (preconditioned: reduced by the update
  //                                     kernel itself; else one scalar launch)
  //   x += alpha p, r -= alpha q, z = M r, partials of (r^H z, |r|^2)
  //   beta, rho, convergence          (partials reduced in the same launch)
  // Preconditioned, that is two glue launches per iteration.
  CgAlpha ca;
  if (pre) {
    ca.pq = part;
    ca.nblk = nblk_pq ? nblk_pq : nblk;
    ca.rho = S.rho;
    ca.alpha = S.alpha;
    ca.dot = S.dot;
    ca.active = S.active;
    ca.iters = S.iters;
  }
  auto iteration = [&](cudaStream_t cs) -> cudaError_t {
    cudaError_t e2 = launch_fncB<R>(P, p, q, nvec, ctx, w0, w1, cs, nblk_pq ? part : nullptr, pre ? z : r, S.beta);
    if (e2 == cudaSuccess && !nblk_pq) e2 = dot_partial<R>(p, q, L, L, nvec, part, nblk, S.active, cs);
    if (pre) {
      // the update's own partial sums go to part2 (part still holds p^H q)
      if (e2 == cudaSuccess) e2 = pcg_update<R>(P, x, r, z, p, q, nvec, ctx, S.alpha, part2, nblkv, cs, ca);
    } else {
      if (e2 == cudaSuccess)
        e2 = cg_scalars_red(0, nvec, part, nblk, S.dot, S.rho, S.alpha, S.beta, S.tol2b2, S.active, S.iters,
                            S.res2, cs);
      if (e2 == cudaSuccess) e2 = cg_xr_partial<R>(x, r, p, q, L, L, nvec, S.alpha, S.active, part, nblk, cs);
    }
    if (e2 == cudaSuccess)
      e2 = cg_scalars_red(1, nvec, pre ? part2 : part, pre ? nblkv : nblk, S.dot, S.rho, S.alpha, S.beta, S.tol2b2,
                          S.active, S.iters, S.res2, cs);
    return e2;
  };
  const int chk = 4;
  const std::vector<uintptr_t> gkey = {sizeof(R), (uintptr_t)nvec, (uintptr_t)pre, (uintptr_t)chk, (uintptr_t)P.n,
                                       (uintptr_t)p, (uintptr_t)q, (uintptr_t)x, (uintptr_t)r, (uintptr_t)z,
                                       (uintptr_t)w0, (uintptr_t)w1, (uintptr_t)s, (uintptr_t)part, (uintptr_t)part2,
                                       (uintptr_t)d_inst, (uintptr_t)nblk, (uintptr_t)nblkv,
                                       sizeof(R) == 4 ? (uintptr_t)P.d32.pc : (uintptr_t)P.d64.pc,
                                       (uintptr_t)tune_for(P, tune_prec<R>(), nvec).chunk,
                                       (uintptr_t)tune_for(P, tune_prec<R>(), nvec).stencil_tpb,
                                       (uintptr_t)nblk_pq, (uintptr_t)P.opt_plane_split,
                                       (uintptr_t)P.opt_pi_table};
  bool use_graph = P.opt_graph != 0;
  bool any = std::any_of(act.begin(), act.end(), [](int a) { return a != 0; });
  int it = 1;
  if (P.opt_graph >= 2 && any && maxit >= chk) {
    // the whole loop of chk-iteration blocks in one graph launch, the
    // convergence test on the device after each block; the host waits once
    std::vector<uintptr_t> wkey = gkey;
    wkey.push_back((uintptr_t)0x5748494cu);  // distinct from the block graph
    wkey.push_back((uintptr_t)(maxit / chk));
    unsigned long long body_nodes = 0;
    cudaError_t ge = graph_replay_while(P, wkey, [&](cudaStream_t cs) -> cudaError_t {
      for (int i = 0; i < chk; ++i) {
        cudaError_t e2 = iteration(cs);
        if (e2 != cudaSuccess) return e2;
      }
      return cudaSuccess;
    }, S.active, nvec, S.passes, maxit / chk, &body_nodes);
    if (ge == cudaSuccess) {
      int passes = 0;
      FAME_CK(cudaMemcpyAsync(act.data(), S.active, sizeof(int) * nvec, cudaMemcpyDeviceToHost, st), "pcg check");
      FAME_CK(cudaMemcpyAsync(&passes, S.passes, sizeof(int), cudaMemcpyDeviceToHost, st), "pcg check");
      FAME_CK(cudaStreamSynchronize(st), "pcg check");
      FAME_KERNELS_RAN(body_nodes * (unsigned long long)passes);
      it = 1 + passes * chk;
      any = std::any_of(act.begin(), act.end(), [](int a) { return a != 0; });
    } else {
      cudaGetLastError();  // no graph loop (nothing of it ran): the blocks below take over
    }
  }
  for (; it <= maxit && any; it += chk) {
    const int nit = std::min(chk, maxit - it + 1);
    bool done = false;
    if (use_graph && nit == chk) {
      cudaError_t ge = graph_replay(P, gkey, [&](cudaStream_t cs) -> cudaError_t {
        for (int i = 0; i < chk; ++i) {
          cudaError_t e2 = iteration(cs);
          if (e2 != cudaSuccess) return e2;
        }
        return cudaSuccess;
      });
      if (ge == cudaSuccess) done = true;
      else use_graph = false;  // capture unavailable: issue directly from now on
    }
    if (!done)
      for (int i = 0; i < nit; ++i) FAME_CK(iteration(st), "pcg iteration");
    FAME_CK(cudaMemcpyAsync(act.data(), S.active, sizeof(int) * nvec, cudaMemcpyDeviceToHost, st), "pcg check");
    FAME_CK(cudaStreamSynchronize(st), "pcg check");
    any = std::any_of(act.begin(), act.end(), [](int a) { return a != 0; });
  }
  std::vector<int> its(nvec);
  std::vector<double> r2(nvec);
  FAME_CK(cudaMemcpyAsync(its.data(), S.iters, sizeof(int) * nvec, cudaMemcpyDeviceToHost, st), "pcg out");
  FAME_CK(cudaMemcpyAsync(r2.data(), S.res2, sizeof(double) * nvec, cudaMemcpyDeviceToHost, st), "pcg out");
  FAME_CK(cudaMemcpyAsync(act.data(), S.active, sizeof(int) * nvec, cudaMemcpyDeviceToHost, st), "pcg out");
  FAME_CK(cudaStreamSynchronize(st), "pcg out");
  int rc = FAME_OK;
  for (int v = 0; v < nvec; ++v) {
    const bool sel = h_mask ? h_mask[v] != 0 : true;
    if (!sel) continue;
    if (iters_out) iters_out[v] = its[v];
    if (relres_out) relres_out[v] = bb[v].x > 0.0 ? std::sqrt(std::max(r2[v], 0.0) / bb[v].x) : 0.0;
    if (its[v] < 0) rc = std::isfinite(r2[v]) ? FAME_ERR_BREAKDOWN : FAME_ERR_NAN;
    else if (act[v] && rc == FAME_OK) rc = FAME_ERR_NOT_CONVERGED;
  }
  if (rc != FAME_OK)
    fail(&P, rc, rc == FAME_ERR_NOT_CONVERGED ? "pcg: not converged within maxit" : "pcg: breakdown or NaN");
  return rc;
}

template int pcg_batched<float>(Plan&, const float2*, float2*, int, const int*, double, int, int*, double*,
                                const unsigned char*, const double*);
template int pcg_batched<double>(Plan&, const double2*, double2*, int, const int*, double, int, int*, double*,
                                 const unsigned char*, const double*);

int solve_B_mixed(Plan& P, const double2* b, double2* x, double2* Bx, int nvec, const int* d_inst, double tol,
                  int max_rounds, double inner_tol32, int maxit32, const unsigned char* h_mask, long long* cg_iters,
                  long long* b64_applies, const double* tol_per_vec, long long* cg_vec, long long* b64_vec) {
  if (nvec <= 0) return FAME_OK;
  auto tol_of = [&](int v) { return tol_per_vec ? tol_per_vec[v] : tol; };
  cudaStream_t st = P.stream;
  const long long L = 4 * P.Nq;
  cudaError_t e;
  float2* res32 = (float2*)workspace(P, WS_MIX_B32, sizeof(float2) * L * nvec, &e);
  FAME_CK(e, "mixed workspace");
  float2* d32 = (float2*)workspace(P, WS_MIX_X32, sizeof(float2) * L * nvec, &e);
  FAME_CK(e, "mixed workspace");
  double2* res = (double2*)workspace(P, WS_MIX_RES, sizeof(double2) * L * nvec, &e);
  FAME_CK(e, "mixed workspace");
  const int nblk = dot_blocks(P, L, nvec);
  char* sc = (char*)workspace(P, WS_MIX_MASK,
                              (sizeof(int) + sizeof(double2)) * nvec + sizeof(double2) * nblk * nvec +
                                  2 * sizeof(double) * nvec + 64, &e);
  FAME_CK(e, "mixed workspace");
  double2* dot = (double2*)sc;
  double2* part = dot + nvec;
  double* dscale = (double*)(part + (size_t)nblk * nvec);  // [nvec] 2^-e, [nvec] 2^e (e: exponent of ||res||)
  int* dmask = (int*)(dscale + 2 * nvec);
  FAME_CK(ensure_work(P, nvec), "mixed scratch");

  std::vector<unsigned char> m(nvec, 1);
  if (h_mask)
    for (int v = 0; v < nvec; ++v) m[v] = h_mask[v] ? 1 : 0;
  std::vector<int> mi(nvec);
  for (int v = 0; v < nvec; ++v) mi[v] = m[v];
  FAME_CK(h2d_async(P, dmask, mi.data(), sizeof(int) * nvec), "mixed init");
  FAME_CK(dot_batched<double>(b, L, 0, 1, b, L, L, nvec, dot, part, nblk, dmask, st), "mixed dot");
  std::vector<double2> bb(nvec);
  FAME_CK(cudaMemcpyAsync(bb.data(), dot, sizeof(double2) * nvec, cudaMemcpyDeviceToHost, st), "mixed init");
  FAME_CK(cudaStreamSynchronize(st), "mixed init");
  for (int v = 0; v < nvec; ++v) {
    if (!m[v]) continue;
    if (!std::isfinite(bb[v].x)) return fail(&P, FAME_ERR_NAN, "mixed solve: non-finite right-hand side");
    FAME_CK(cudaMemsetAsync(x + (size_t)v * L, 0, sizeof(double2) * L, st), "mixed init");
    FAME_CK(cudaMemsetAsync(Bx + (size_t)v * L, 0, sizeof(double2) * L, st), "mixed init");
    if (!(bb[v].x > 0.0)) m[v] = 0;
  }
  // Each complex64 round solves B d = s res with s = 2^-e, e the binary
  // exponent of ||res|| (a right-hand side of norm in [1, 2), so that no
  // product in the complex64 CG underflows however small the residual has
  // become; a power of two scales without rounding) and adds d / s to x.
  std::vector<double> scl(2 * nvec, 1.0);
  auto upload_scale = [&](const std::vector<double>& rr) -> cudaError_t {
    for (int v = 0; v < nvec; ++v) {
      const double nr = rr[v] > 0.0 && std::isfinite(rr[v]) ? std::sqrt(rr[v]) : 1.0;
      const int ex = std::ilogb(nr);
      scl[v] = std::ldexp(1.0, -ex);
      scl[nvec + v] = std::ldexp(1.0, ex);
    }
    return h2d_async(P, dscale, scl.data(), sizeof(double) * 2 * nvec);
  };
  // res = b (FP64) and its scaled complex64 copy
  FAME_CK(residual(b, Bx, res, nullptr, L, nvec, dmask, st), "mixed residual");
  for (int v = 0; v < nvec; ++v) mi[v] = m[v];
  FAME_CK(h2d_async(P, dmask, mi.data(), sizeof(int) * nvec), "mixed init");
  {
    std::vector<double> b2(nvec);
    for (int v = 0; v < nvec; ++v) b2[v] = bb[v].x;
    FAME_CK(upload_scale(b2), "mixed scale");
    FAME_CK(to32_scaled(res, res32, L, nvec, dscale, dmask, st), "mixed scale");
  }
  int rc = FAME_OK;
  std::vector<int> its(nvec);
  VecCtx ctx;
  ctx.inst = d_inst;
  ctx.active = dmask;
  ctx.nk = P.nk;
  float2* bd32 = (float2*)workspace(P, WS_MIX_BD, sizeof(float2) * L * nvec, &e);
  FAME_CK(e, "mixed workspace");
  std::vector<double> rr_prev(nvec), tolv(nvec, inner_tol32);
  for (int v = 0; v < nvec; ++v) rr_prev[v] = bb[v].x;
  for (int round = 0; round < max_rounds; ++round) {
    if (!std::any_of(m.begin(), m.end(), [](unsigned char a) { return a != 0; })) break;
    // Complex64 CG on the current residual; after the first round only as far
    // as the target needs (never below what complex64 resolves).
    // (a 5x margin below the target keeps the complex64-estimated residual of
    // the second round from missing it by a hair and costing another FP64 round)
    for (int v = 0; v < nvec; ++v)
      tolv[v] = round == 0 ? inner_tol32
                           : std::min(0.5, std::max(1e-7, 0.2 * tol_of(v) * std::sqrt(bb[v].x / std::max(rr_prev[v], 1e-300))));
    int prc = pcg_batched<float>(P, res32, d32, nvec, d_inst, inner_tol32, maxit32, its.data(), nullptr, m.data(),
                                 tolv.data());
    if (prc == FAME_ERR_NAN || prc == FAME_ERR_BREAKDOWN) return prc;
    for (int v = 0; v < nvec; ++v)
      if (m[v]) {
        if (cg_iters) *cg_iters += std::abs(its[v]);
        if (cg_vec) cg_vec[v] += std::abs(its[v]);
      }
    FAME_CK(refine_acc(x, d32, L, nvec, dmask, st, dscale + nvec), "mixed acc");
    if (round != 1 || !P.opt_c64_round) {
      // exact residual b - B x: fncB in double-single arithmetic where the
      // grid has it (~1e-14 relative, on the FP32 pipes), else FP64
      if (P.opt_ds_residual && ds_supported(P.n)) {
        FAME_CK(launch_fncB_ds(P, x, Bx, nvec, ctx, st), "mixed fncB");
      } else {
        double2* w0 = (double2*)P.d_work;
        double2* w1 = w0 + (size_t)nvec * 6 * P.Nq;
        FAME_CK(launch_fncB<double>(P, x, Bx, nvec, ctx, w0, w1, st), "mixed fncB");
      }
      for (int v = 0; v < nvec; ++v) {
        if (b64_applies) *b64_applies += m[v];
        if (b64_vec) b64_vec[v] += m[v];
      }
    } else {
      // B x = (B x_prev) + B d with B d in complex64: d is already ~1e-6 of
      // x, so the residual this estimates is good to ~1e-11 of b; a target
      // below that takes a further round, whose FP64 apply makes B x exact
      // again (B x is the B Q of the Lanczos basis).
      float2* w0 = (float2*)P.d_work;
      float2* w1 = w0 + (size_t)nvec * 6 * P.Nq;
      FAME_CK(launch_fncB<float>(P, d32, bd32, nvec, ctx, w0, w1, st), "mixed fncB32");
      FAME_CK(refine_acc(Bx, bd32, L, nvec, dmask, st, dscale + nvec), "mixed acc");
    }
    FAME_CK(residual(b, Bx, res, nullptr, L, nvec, dmask, st), "mixed residual");
    FAME_CK(dot_batched<double>(res, L, 0, 1, res, L, L, nvec, dot, part, nblk, dmask, st), "mixed dot");
    std::vector<double2> rr(nvec);
    FAME_CK(cudaMemcpyAsync(rr.data(), dot, sizeof(double2) * nvec, cudaMemcpyDeviceToHost, st), "mixed check");
    FAME_CK(cudaStreamSynchronize(st), "mixed check");
    for (int v = 0; v < nvec; ++v) {
      if (!m[v]) continue;
      if (!std::isfinite(rr[v].x)) return fail(&P, FAME_ERR_NAN, "mixed solve: non-finite residual");
      rr_prev[v] = rr[v].x;
      if (rr[v].x <= tol_of(v) * tol_of(v) * bb[v].x) m[v] = 0;
    }
    for (int v = 0; v < nvec; ++v) mi[v] = m[v];
    FAME_CK(h2d_async(P, dmask, mi.data(), sizeof(int) * nvec), "mixed mask");
    if (round + 1 < max_rounds && std::any_of(m.begin(), m.end(), [](unsigned char a) { return a != 0; })) {
      std::vector<double> r2(nvec);
      for (int v = 0; v < nvec; ++v) r2[v] = rr[v].x;
      FAME_CK(upload_scale(r2), "mixed scale");
      FAME_CK(to32_scaled(res, res32, L, nvec, dscale, dmask, st), "mixed scale");
    }
  }
  if (std::any_of(m.begin(), m.end(), [](unsigned char a) { return a != 0; })) rc = FAME_ERR_NOT_CONVERGED;
  return rc;
}

// ---------------------------------------------------------------------------
// FP64 refinement sweep of converged Ritz pairs (no reference counterpart:
// the reference's FP64 Lanczos needs none).  For the k Ritz pairs (Lambda, X)
// of every instance, batched over all instances:
//   R = A X - B X Lambda                      FP64 residuals
//   W = B^{-1} R                              mixed-precision inner solve to `tol`
//   [X W]^H A [X W] c = lambda [X W]^H B [X W] c    FP64 Rayleigh-Ritz
// W spans the same space as B^{-1} A X beside X (one step of block inverse
// iteration) without its cancellation: for converged pairs B^{-1} A X is
// X Lambda to many digits.  The pencil is reduced to the B-orthonormal basis
// of the well-conditioned part of [X W] (canonical orthogonalisation: the
// eigenvectors of [X W]^H B [X W] with eigenvalues above 1e-13 of the
// largest), and the k largest lambda are kept, as Lanczos.m:109 orders them.
// The NFSEP residual ||B x - omega A x|| (EvaluteError_Chiral_no_inv.m:20,
// x B-normalised, omega = 1/lambda) is evaluated in FP64 before and after;
// a pair keeps its old value when the sweep would not lower its residual.
// X: [na*k][4Nq] B-normalised Ritz vectors, overwritten by the refined ones;
// lam: [na][k] in and out.
// ---------------------------------------------------------------------------
int ritz_refine(Plan& P, const std::vector<int>& insts, int k, double2* X, double* lam, double* res_before,
                double* res_after, double tol, long long* b64_vec, long long* cg_vec) {
  using cd = std::complex<double>;
  const int na = (int)insts.size();
  if (na == 0 || k < 1) return FAME_OK;
  cudaStream_t st = P.stream;
  const long long L = 4 * P.Nq;
  const int nv = na * k;
  const size_t cb = sizeof(double2) * L;
  cudaError_t e;
  double2* AX = (double2*)workspace(P, WS_RF_AX, cb * nv, &e);
  FAME_CK(e, "refine workspace");
  double2* BX = (double2*)workspace(P, WS_RF_BX, cb * nv, &e);
  FAME_CK(e, "refine workspace");
  double2* W = (double2*)workspace(P, WS_RF_Y, cb * nv, &e);
  FAME_CK(e, "refine workspace");
  double2* BW = (double2*)workspace(P, WS_RF_BY, cb * nv, &e);
  FAME_CK(e, "refine workspace");
  double2* AW = (double2*)workspace(P, WS_RF_AY, cb * nv, &e);
  FAME_CK(e, "refine workspace");
  double2* Rv = (double2*)workspace(P, WS_RF_R, cb * nv, &e);
  FAME_CK(e, "refine workspace");
  double2* Z = (double2*)workspace(P, WS_RF_Z, cb * 2 * k, &e);
  FAME_CK(e, "refine workspace");
  int* dinst = (int*)workspace(P, WS_RF_INST, sizeof(int) * nv + 64, &e);
  FAME_CK(e, "refine workspace");
  const int ncall = 8 * k;  // (A, B) x (X rows, W rows) x 2k columns
  double2* G = (double2*)workspace(P, WS_RF_G, sizeof(double2) * ((size_t)ncall * na * k + 4 * nv) + 64, &e);
  FAME_CK(e, "refine workspace");
  double2* scal = G + (size_t)ncall * na * k;  // [2][nv] axpby scalars, [nv] norms
  double2* C = (double2*)workspace(P, WS_RF_C, sizeof(double2) * (size_t)na * 2 * k * k + 64, &e);
  FAME_CK(e, "refine workspace");
  const int nblk = dot_blocks(P, L, std::max(na, nv));
  double2* part = (double2*)workspace(P, WS_RF_PART, sizeof(double2) * (size_t)nblk * nv + 64, &e);
  FAME_CK(e, "refine workspace");
  FAME_CK(ensure_work(P, nv), "refine scratch");
  std::vector<int> hi(nv);
  for (int a = 0; a < na; ++a)
    for (int i = 0; i < k; ++i) hi[(size_t)a * k + i] = insts[a];
  FAME_CK(h2d_async(P, dinst, hi.data(), sizeof(int) * nv), "refine init");
  VecCtx ctx;
  ctx.inst = dinst;
  ctx.nk = P.nk;
  double2* W0 = (double2*)P.d_work;
  double2* W1 = W0 + (size_t)nv * 6 * P.Nq;
  // out = s1 * V1 + s2 * V2 per vector (s1, s2 real, per vector)
  auto combine = [&](const double2* V1, const std::vector<double>& s1, const double2* V2,
                     const std::vector<double>& s2, double2* out) -> int {
    std::vector<double2> ab(2 * (size_t)nv);
    for (int i = 0; i < nv; ++i) {
      ab[i] = make_double2(s1[i], 0.0);
      ab[nv + i] = make_double2(s2[i], 0.0);
    }
    FAME_CK(h2d_async(P, scal, ab.data(), sizeof(double2) * 2 * nv), "refine combine");
    if (out != V2) FAME_CK(cudaMemcpyAsync(out, V2, cb * nv, cudaMemcpyDeviceToDevice, st), "refine combine");
    FAME_CK(axpby_batched<double>(V1, out, L, L, nv, scal, scal + nv, nullptr, st), "refine combine");
    return FAME_OK;
  };
  auto norms = [&](const double2* V, double* out) -> int {
    FAME_CK(dot_batched<double>(V, L, 0, 1, V, L, L, nv, scal + 2 * nv, part, nblk, nullptr, st), "refine norm");
    std::vector<double2> h(nv);
    FAME_CK(cudaMemcpyAsync(h.data(), scal + 2 * nv, sizeof(double2) * nv, cudaMemcpyDeviceToHost, st), "refine norm");
    FAME_CK(cudaStreamSynchronize(st), "refine norm");
    for (int i = 0; i < nv; ++i) out[i] = std::sqrt(std::max(0.0, h[i].x));
    return FAME_OK;
  };
  std::vector<double> ones(nv, 1.0), mlam(nv), mom(nv);
  // A X, B X; NFSEP before: || B X - omega A X ||, the GEP residual A X - B X Lambda
  FAME_CK(launch_fncA<double>(P, X, AX, nv, ctx, st), "refine fncA");
  FAME_CK(launch_fncB<double>(P, X, BX, nv, ctx, W0, W1, st), "refine fncB");
  for (int i = 0; i < nv; ++i) {
    b64_vec[i]++;
    mlam[i] = -lam[i];
    mom[i] = -1.0 / lam[i];
  }
  int rc;
  std::vector<double> rb(nv);
  if ((rc = combine(AX, mom, BX, ones, Rv))) return rc;  // Rv = BX - omega AX
  if ((rc = norms(Rv, rb.data()))) return rc;
  if (res_before) std::copy(rb.begin(), rb.end(), res_before);
  if ((rc = combine(BX, mlam, AX, ones, Rv))) return rc;  // Rv = AX - lambda BX
  // W = B^{-1} R (a search direction: its accuracy does not limit the sweep,
  // whose Rayleigh-Ritz uses exact FP64 applies of A and B on W)
  long long cgi = 0, b64 = 0;
  rc = solve_B_mixed(P, Rv, W, BW, nv, dinst, tol, 8, P.opt_tol32, 4000, nullptr, &cgi, &b64, nullptr, cg_vec,
                     b64_vec);
  if (rc == FAME_ERR_NAN || rc == FAME_ERR_BREAKDOWN) {
    // no usable search direction: the pairs stay as the Lanczos run left them
    if (res_after) std::copy(rb.begin(), rb.end(), res_after);
    P.last_error.clear();
    return FAME_OK;
  }
  // W to unit B-norm (its norm is that of the residuals, ~1e-10, and would
  // otherwise vanish below the cut-off of the orthogonalisation)
  {
    FAME_CK(dot_batched<double>(W, L, 0, 1, BW, L, L, nv, scal + 2 * nv, part, nblk, nullptr, st), "refine wnorm");
    std::vector<double2> h(nv);
    FAME_CK(cudaMemcpyAsync(h.data(), scal + 2 * nv, sizeof(double2) * nv, cudaMemcpyDeviceToHost, st), "refine wnorm");
    FAME_CK(cudaStreamSynchronize(st), "refine wnorm");
    std::vector<double> sw(nv);
    for (int i = 0; i < nv; ++i) sw[i] = h[i].x > 0.0 && std::isfinite(h[i].x) ? 1.0 / std::sqrt(h[i].x) : 0.0;
    double* dsw = (double*)(scal + 3 * nv);
    FAME_CK(h2d_async(P, dsw, sw.data(), sizeof(double) * nv), "refine wnorm");
    FAME_CK(scale_batched<double>(W, W, L, nv, dsw, nullptr, st), "refine wnorm");
    FAME_CK(scale_batched<double>(BW, BW, L, nv, dsw, nullptr, st), "refine wnorm");
  }
  FAME_CK(launch_fncA<double>(P, W, AW, nv, ctx, st), "refine fncA");
  // Gram matrices on Z = [X_a W_a]: call c = ((op * 2 + rowblk) * 2k + col) fills G[c][a][0..k)
  const long long vs = (long long)k * L;  // instance stride inside X, W, AX, ...
  for (int op = 0; op < 2; ++op)
    for (int rb2 = 0; rb2 < 2; ++rb2)
      for (int col = 0; col < 2 * k; ++col) {
        const double2* rows = rb2 == 0 ? X : W;
        const double2* cv = op == 0 ? (col < k ? AX : AW) : (col < k ? BX : BW);
        cv += (size_t)(col % k) * L;
        const int c = (op * 2 + rb2) * 2 * k + col;
        FAME_CK(dot_batched<double>(rows, vs, L, k, cv, vs, L, na, G + (size_t)c * na * k, part, nblk, nullptr, st),
                "refine gram");
      }
  std::vector<double2> hG((size_t)ncall * na * k);
  FAME_CK(cudaMemcpyAsync(hG.data(), G, sizeof(double2) * hG.size(), cudaMemcpyDeviceToHost, st), "refine gram");
  FAME_CK(cudaStreamSynchronize(st), "refine gram");
  const int m = 2 * k;
  std::vector<double2> hC((size_t)na * m * k, make_double2(0.0, 0.0));
  std::vector<double> lam_new(lam, lam + nv);
  for (int a = 0; a < na; ++a) {
    std::vector<cd> GA((size_t)m * m), GB((size_t)m * m);
    for (int op = 0; op < 2; ++op)
      for (int rb2 = 0; rb2 < 2; ++rb2)
        for (int col = 0; col < m; ++col) {
          const int c = (op * 2 + rb2) * m + col;
          for (int r = 0; r < k; ++r) {
            const double2 v = hG[((size_t)c * na + a) * k + r];  // z_row^H (Op z_col)
            (op == 0 ? GA : GB)[(size_t)(rb2 * k + r) * m + col] = cd(v.x, v.y);
          }
        }
    for (int i = 0; i < m; ++i) {  // Hermitian parts
      for (int j = 0; j < i; ++j) {
        const cd ga = 0.5 * (GA[(size_t)i * m + j] + std::conj(GA[(size_t)j * m + i]));
        GA[(size_t)i * m + j] = ga;
        GA[(size_t)j * m + i] = std::conj(ga);
        const cd gb = 0.5 * (GB[(size_t)i * m + j] + std::conj(GB[(size_t)j * m + i]));
        GB[(size_t)i * m + j] = gb;
        GB[(size_t)j * m + i] = std::conj(gb);
      }
      GA[(size_t)i * m + i] = GA[(size_t)i * m + i].real();
      GB[(size_t)i * m + i] = GB[(size_t)i * m + i].real();
    }
    // canonical orthogonalisation: GB = V diag(d) V^H, T = V_keep diag(d_keep)^{-1/2}
    std::vector<double> d;
    std::vector<cd> V;
    jacobi_eig_herm(GB, m, d, V);
    const double dmax = *std::max_element(d.begin(), d.end());
    std::vector<int> keep;
    for (int j = 0; j < m; ++j)
      if (d[j] > 1e-13 * dmax) keep.push_back(j);
    const int q = (int)keep.size();
    if (q < k) continue;  // degenerate basis: keep this instance's pairs as they are
    std::vector<cd> T((size_t)m * q);  // column-major m x q
    for (int c2 = 0; c2 < q; ++c2)
      for (int i = 0; i < m; ++i) T[(size_t)c2 * m + i] = V[(size_t)keep[c2] * m + i] / std::sqrt(d[keep[c2]]);
    std::vector<cd> H((size_t)q * q, cd(0.0));  // T^H GA T, row-major
    for (int i = 0; i < q; ++i)
      for (int j = 0; j < q; ++j) {
        cd sum = 0.0;
        for (int r = 0; r < m; ++r) {
          cd t = 0.0;
          for (int c2 = 0; c2 < m; ++c2) t += GA[(size_t)r * m + c2] * T[(size_t)j * m + c2];
          sum += std::conj(T[(size_t)i * m + r]) * t;
        }
        H[(size_t)i * q + j] = sum;
      }
    for (int i = 0; i < q; ++i)
      for (int j = 0; j < i; ++j) {
        const cd h = 0.5 * (H[(size_t)i * q + j] + std::conj(H[(size_t)j * q + i]));
        H[(size_t)i * q + j] = h;
        H[(size_t)j * q + i] = std::conj(h);
      }
    std::vector<double> mu;
    std::vector<cd> Yv;
    jacobi_eig_herm(H, q, mu, Yv);
    std::vector<int> ind(q);
    std::iota(ind.begin(), ind.end(), 0);
    std::stable_sort(ind.begin(), ind.end(), [&](int x, int y) { return mu[x] > mu[y]; });
    for (int j = 0; j < k; ++j) {
      lam_new[(size_t)a * k + j] = mu[ind[j]];
      for (int i = 0; i < m; ++i) {  // c = T y
        cd v = 0.0;
        for (int c2 = 0; c2 < q; ++c2) v += T[(size_t)c2 * m + i] * Yv[(size_t)ind[j] * q + c2];
        hC[((size_t)a * k + j) * m + i] = make_double2(v.real(), v.imag());
      }
    }
  }
  FAME_CK(h2d_async(P, C, hC.data(), sizeof(double2) * hC.size()), "refine combine");
  // refined vectors Xn_a = [X_a W_a] C_a into Rv (instances whose basis was degenerate keep X_a)
  for (int a = 0; a < na; ++a) {
    bool set = false;
    for (int i = 0; i < m * k && !set; ++i) set = hC[(size_t)a * m * k + i].x != 0.0 || hC[(size_t)a * m * k + i].y != 0.0;
    if (!set) {
      FAME_CK(cudaMemcpyAsync(Rv + (size_t)a * vs, X + (size_t)a * vs, cb * k, cudaMemcpyDeviceToDevice, st),
              "refine combine");
      continue;
    }
    FAME_CK(cudaMemcpyAsync(Z, X + (size_t)a * vs, cb * k, cudaMemcpyDeviceToDevice, st), "refine combine");
    FAME_CK(cudaMemcpyAsync(Z + (size_t)k * L, W + (size_t)a * vs, cb * k, cudaMemcpyDeviceToDevice, st),
            "refine combine");
    FAME_CK(block_comb<double>(Z, Rv + (size_t)a * vs, L, L, m, k, C + (size_t)a * m * k, st), "refine combine");
  }
  // residuals after (W, AW, BW reused as the refined vectors' A / B products)
  FAME_CK(launch_fncA<double>(P, Rv, AW, nv, ctx, st), "refine fncA");
  FAME_CK(launch_fncB<double>(P, Rv, BW, nv, ctx, W0, W1, st), "refine fncB");
  for (int i = 0; i < nv; ++i) {
    b64_vec[i]++;
    mom[i] = -1.0 / lam_new[i];
  }
  std::vector<double> ra(nv);
  if ((rc = combine(AW, mom, BW, ones, W))) return rc;
  if ((rc = norms(W, ra.data()))) return rc;
  // keep the sweep's pair only where it lowered the residual
  for (int i = 0; i < nv; ++i) {
    if (ra[i] <= rb[i]) {
      FAME_CK(cudaMemcpyAsync(X + (size_t)i * L, Rv + (size_t)i * L, cb, cudaMemcpyDeviceToDevice, st), "refine out");
      lam[i] = lam_new[i];
    } else {
      ra[i] = rb[i];
    }
  }
  if (res_after) std::copy(ra.begin(), ra.end(), res_after);
  FAME_CK(cudaStreamSynchronize(st), "refine out");
  return FAME_OK;
}

// ---------------------------------------------------------------------------
// Thick-restart Lanczos (fun_Lanczos/Lanczos.m), all selected instances in
// lock step.  B*Q is cached column by column, so the reorthogonalisation of
// Lanczos.m:63,66,69,159-167 needs no extra B applies; it runs as two passes
// of classical Gram-Schmidt in the B inner product.
// ---------------------------------------------------------------------------
struct LzInst {
  int inst = 0;
  int k0 = 0, k = 0, sizeV = 1, j = 1, mm = 1;
  bool justRestarted = false, done = false;
  std::vector<double> Alpha, Beta, d, c;
  double beta = 0.0;
  std::vector<double> U;  // final Ritz combination, p x k0 column-major
  long long steps = 0, restarts = 0, bapplies = 0, cgits = 0;
  double itol = 1e-12;  // inner B^{-1} tolerance of this instance (mixed form: scaled by the spectral spread)
  bool explicit_br = false;  // mixed form: B r by an FP64 apply instead of the recurrence
  bool refresh_bq = false;   // recompute the kept B*Q columns in FP64 at this restart
};

int lanczos_run(Plan& P, int prec, const std::vector<int>& insts, int k0, double tol, int maxit, int p,
                const double* v0_host, double inner_tol, double* ew, double2* ev, double* res, long long* stats) {
  const int na = (int)insts.size();
  if (na == 0) return FAME_OK;
  if (k0 < 1 || p <= k0 || p > 64 || maxit < 1 || !(tol > 0.0))
    return fail(&P, FAME_ERR_BAD_ARG, "lanczos: need 1 <= k < p <= 64, maxit >= 1, tol > 0");
  const long long L = 4 * P.Nq;
  if (p > L) return fail(&P, FAME_ERR_BAD_ARG, "lanczos: p exceeds the vector length");
  cudaStream_t st = P.stream;
  cudaError_t e;
  const double itol = inner_tol > 0 ? inner_tol : 1e-12;
  const size_t cb = sizeof(double2) * L;
  double2* Q = (double2*)workspace(P, WS_LZ_Q, cb * p * na, &e);
  FAME_CK(e, "lanczos workspace Q");
  double2* BQ = (double2*)workspace(P, WS_LZ_BQ, cb * p * na, &e);
  FAME_CK(e, "lanczos workspace BQ");
  double2* vec = (double2*)workspace(P, WS_LZ_VEC, cb * 7 * na, &e);
  FAME_CK(e, "lanczos workspace");
  double2* V = vec;               // current Lanczos vector v
  double2* BV = V + L * na;       // B v
  double2* AQ = BV + L * na;      // A q
  double2* PR = AQ + L * na;      // B^{-1} A q   -> r
  double2* BPR = PR + L * na;     // B * pr       -> B r
  double2* T1 = BPR + L * na;     // scratch
  double2* T2 = T1 + L * na;      // scratch
  double2* TMP = (double2*)workspace(P, WS_LZ_TMP, cb * p, &e);
  FAME_CK(e, "lanczos workspace");
  int* dinst = (int*)workspace(P, WS_LZ_INST, sizeof(int) * na * 2 + 64, &e);
  FAME_CK(e, "lanczos workspace");
  int* dmask = dinst + na;
  double2* coef = (double2*)workspace(P, WS_LZ_COEF, sizeof(double2) * 128 * na, &e);
  FAME_CK(e, "lanczos workspace");
  double* dU = (double*)workspace(P, WS_LZ_U, sizeof(double) * p * p, &e);
  FAME_CK(e, "lanczos workspace");
  double* dsc = (double*)workspace(P, WS_LZ_SCAL, sizeof(double) * na * 2 + 64, &e);
  FAME_CK(e, "lanczos workspace");
  double2* ddot = (double2*)workspace(P, WS_LZ_DOT, sizeof(double2) * na * 2 * 64, &e);
  FAME_CK(e, "lanczos workspace");
  const int nblk1 = dot_blocks(P, L, 1);
  const int nblkb = dot_blocks(P, L, na);
  double2* part = (double2*)workspace(P, WS_LZ_PART, sizeof(double2) * std::max(nblk1 * 64, nblkb * na) + 64, &e);
  FAME_CK(e, "lanczos workspace");
  FAME_CK(ensure_work(P, na), "lanczos scratch");
  FAME_CK(h2d_async(P, dinst, insts.data(), sizeof(int) * na), "lanczos init");

  std::vector<LzInst> S(na);
  for (int a = 0; a < na; ++a) {
    S[a].inst = insts[a];
    S[a].k0 = S[a].k = k0;
    S[a].itol = itol;
    if (prec == FAME_C64 && P.sigma_min[insts[a]] < 1e-2) {
      // A near-zero wave vector (Gamma shifted by 1e-4) gives curl singular
      // values ~1e-4 and eigenvalues lambda ~ 1e4 among the wanted ones: run
      // this instance at the inner-tolerance floor with explicit FP64 B r
      // from the first step (see the spread rule at the restarts).  At n = 60
      // a floor of 1e-13 leaves NFSEP residuals ~3e-11 there; 1e-12 does not
      // reach 1e-8.
      S[a].itol = P.opt_itol_floor;
      S[a].explicit_br = true;
    }
  }
  std::vector<int> mask(na, 1);
  auto upload_mask = [&]() -> cudaError_t {
    return h2d_async(P, dmask, mask.data(), sizeof(int) * na);
  };
  FAME_CK(upload_mask(), "lanczos init");
  VecCtx ctx;
  ctx.inst = dinst;
  ctx.active = dmask;
  ctx.nk = P.nk;
  auto fncB64 = [&](const double2* x, double2* y) {
    double2* W0 = (double2*)P.d_work;
    return launch_fncB<double>(P, x, y, na, ctx, W0, W0 + (size_t)na * 6 * P.Nq, st);
  };
  auto batched_dot = [&](const double2* a, const double2* b, std::vector<double2>& out) -> int {
    FAME_CK(dot_batched<double>(a, L, 0, 1, b, L, L, na, ddot, part, nblkb, dmask, st), "lanczos dot");
    out.resize(na);
    FAME_CK(cudaMemcpyAsync(out.data(), ddot, sizeof(double2) * na, cudaMemcpyDeviceToHost, st), "lanczos dot");
    FAME_CK(cudaStreamSynchronize(st), "lanczos dot");
    return FAME_OK;
  };
  auto scale_vecs = [&](const double2* x, double2* y, const std::vector<double>& s) -> int {
    FAME_CK(h2d_async(P, dsc, s.data(), sizeof(double) * na), "lanczos scale");
    FAME_CK(scale_batched<double>(x, y, L, na, dsc, dmask, st), "lanczos scale");
    return FAME_OK;
  };
  const bool mixed = prec == FAME_C64;
  long long total_b = 0;
  // Mixed form: complex64 copies of Q and B*Q for the corrections of the full
  // Gram-Schmidt passes (Lanczos.m:69), whose coefficients are computed in
  // FP64 against the FP64 columns and are ~1e-10 of |r|; the correction
  // sum_i c_i q_i then needs only FP32 (section "reorthogonalisation" below).
  // GB300's FP64 rate makes those column sums the cost of the pass.
  float2* Q32 = nullptr;
  float2* BQ32 = nullptr;
  if (mixed) {
    Q32 = (float2*)workspace(P, WS_LZ_Q32, sizeof(float2) * L * p * na, &e);
    FAME_CK(e, "lanczos workspace Q32");
    BQ32 = (float2*)workspace(P, WS_LZ_BQ32, sizeof(float2) * L * p * na, &e);
    FAME_CK(e, "lanczos workspace BQ32");
  }
  auto copy_lo = [&](int a, int col0, int m) -> int {  // Q32, BQ32 columns col0 .. col0+m-1 of instance a
    if (!mixed || m <= 0) return FAME_OK;
    const size_t o = ((size_t)a * p + col0) * L;
    FAME_CK((convert<float, double>(Q + o, Q32 + o, L * m, st)), "lanczos lo copy");
    FAME_CK((convert<float, double>(BQ + o, BQ32 + o, L * m, st)), "lanczos lo copy");
    return FAME_OK;
  };
  // Batched Gram-Schmidt: every instance of the batch in one launch per
  // operation, instance a against its own columns span[a] = (col0, m)
  // (m = 0: untouched).  Spans go to one of kSpanSlots device slots in turn
  // (stream-ordered uploads, so consecutive operations may reuse a slot).
  constexpr int kSpanSlots = 8;
  int2* dspan = (int2*)workspace(P, WS_LZ_SPAN, sizeof(int2) * (size_t)na * kSpanSlots + sizeof(int) * na + 64, &e);
  FAME_CK(e, "lanczos workspace");
  int* dcol = (int*)(dspan + (size_t)na * kSpanSlots);
  const int nblkg = dot_blocks(P, L, na);
  double2* gspart = (double2*)workspace(P, WS_LZ_GSPART, sizeof(double2) * (size_t)na * 128 * nblkg + 64, &e);
  FAME_CK(e, "lanczos workspace");
  int span_slot = 0;
  auto upload_span = [&](const std::vector<int2>& sp, int* maxm) -> const int2* {
    int2* d = dspan + (size_t)na * (span_slot++ % kSpanSlots);
    *maxm = 0;
    for (const int2& q : sp) *maxm = std::max(*maxm, q.y);
    if (h2d_async(P, d, sp.data(), sizeof(int2) * na) != cudaSuccess) return nullptr;
    return d;
  };
  const long long qs = (long long)p * L;  // instance stride of Q, BQ and their copies
  // r_a -= sum (B q_i)^H r_a q_i over span (and B r likewise), FP64 or with complex64 corrections
  auto project_b = [&](const std::vector<int2>& sp, bool lo) -> int {
    int maxm = 0;
    const int2* d = upload_span(sp, &maxm);
    if (!d) return cuda_fail(&P, cudaErrorUnknown, "lanczos span upload");
    if (maxm == 0) return FAME_OK;
    FAME_CK(gs_dots(BQ, qs, PR, L, L, na, d, maxm, coef, 128, gspart, nblkg, st), "lanczos gs dot");
    if (lo) {
      FAME_CK(gs_combo_lo(PR, L, Q32, qs, L, na, d, coef, 128, st), "lanczos gs");
      if (mixed) FAME_CK(gs_combo_lo(BPR, L, BQ32, qs, L, na, d, coef, 128, st), "lanczos gs");
    } else {
      FAME_CK(gs_combo(PR, L, Q, qs, L, na, d, coef, 128, st), "lanczos gs");
      if (mixed) FAME_CK(gs_combo(BPR, L, BQ, qs, L, na, d, coef, 128, st), "lanczos gs");
    }
    return FAME_OK;
  };

  // v0 (Lanczos.m:8; band_structure...:78-80): ones, or the caller's vector
  {
    std::vector<double2> hv(L);
    for (long long i = 0; i < L; ++i) hv[i] = v0_host ? make_double2(v0_host[2 * i], v0_host[2 * i + 1]) : make_double2(1.0, 0.0);
    for (int a = 0; a < na; ++a)
      FAME_CK(h2d_async(P, V + (size_t)a * L, hv.data(), cb), "lanczos v0");
    FAME_CK(fncB64(V, BV), "lanczos v0");
    total_b += na;
    for (int a = 0; a < na; ++a) S[a].bapplies++;
    std::vector<double2> vb;
    int rc = batched_dot(V, BV, vb);
    if (rc) return rc;
    std::vector<double> s(na);
    for (int a = 0; a < na; ++a) s[a] = 1.0 / std::sqrt(std::fabs(vb[a].x));
    if ((rc = scale_vecs(V, V, s))) return rc;
    if ((rc = scale_vecs(BV, BV, s))) return rc;
  }
  const double eps = 2.2204e-16;  // Lanczos.m:23
  int rc_final = FAME_OK;
  std::vector<unsigned char> hm(na);
  // FAME_PROFILE=1 prints the wall time of each phase of the Lanczos step
  // (the stream is synchronised at every phase boundary while it is on).
  struct PhaseTimer {
    bool on = false;
    cudaStream_t st = nullptr;
    double acc[6] = {0, 0, 0, 0, 0, 0};
    std::chrono::steady_clock::time_point t0;
    void start() {
      if (!on) return;
      cudaStreamSynchronize(st);
      t0 = std::chrono::steady_clock::now();
    }
    void mark(int i) {
      if (!on) return;
      cudaStreamSynchronize(st);
      auto t1 = std::chrono::steady_clock::now();
      acc[i] += std::chrono::duration<double>(t1 - t0).count();
      t0 = t1;
    }
  } prof;
  prof.on = std::getenv("FAME_PROFILE") != nullptr;
  long long n_first = 0, n_second = 0;  // full Gram-Schmidt passes (FAME_PROFILE report)
  prof.st = st;
  prof.start();
  while (true) {
    bool any = false;
    for (int a = 0; a < na; ++a) {
      mask[a] = S[a].done ? 0 : 1;
      any |= !S[a].done;
    }
    if (!any) break;
    FAME_CK(upload_mask(), "lanczos mask");
    // Q(:, j) = v ; BQ(:, j) = B v (and the complex64 copies), all instances in one launch
    {
      std::vector<int> colv(na);
      for (int a = 0; a < na; ++a) colv[a] = S[a].done ? -1 : S[a].j - 1;
      FAME_CK(h2d_async(P, dcol, colv.data(), sizeof(int) * na), "lz");
      FAME_CK(gs_store(Q, BQ, Q32, BQ32, qs, V, BV, L, na, dcol, st), "lz");
    }
    // r = fncA(q); alpha = real(r'*q)   (Lanczos.m:50-51)
    FAME_CK(launch_fncA<double>(P, V, AQ, na, ctx, st), "lanczos fncA");
    std::vector<double2> al;
    int rc = batched_dot(AQ, V, al);
    if (rc) return rc;
    prof.mark(0);
    // pr = fncBinv(r)   (Lanczos.m:54,57,61)
    for (int a = 0; a < na; ++a) hm[a] = mask[a];
    if (mixed) {
      long long cgi = 0, b64 = 0;
      std::vector<double> tv(na);
      std::vector<long long> cgv(na, 0), bv(na, 0);
      for (int a = 0; a < na; ++a) tv[a] = S[a].itol;
      rc = solve_B_mixed(P, AQ, PR, BPR, na, dinst, itol, 8, P.opt_tol32, 2000, hm.data(), &cgi, &b64, tv.data(),
                         cgv.data(), bv.data());
      if (rc == FAME_ERR_NAN || rc == FAME_ERR_BREAKDOWN) return rc;
      total_b += b64;
      for (int a = 0; a < na; ++a) {
        S[a].cgits += cgv[a];
        S[a].bapplies += bv[a];
      }
    } else {
      std::vector<int> its(na, 0);
      rc = pcg_batched<double>(P, AQ, PR, na, dinst, itol, 10000, its.data(), nullptr, hm.data());
      if (rc == FAME_ERR_NAN || rc == FAME_ERR_BREAKDOWN) return rc;
      for (int a = 0; a < na; ++a)
        if (mask[a]) {
          S[a].cgits += std::abs(its[a]);
          S[a].bapplies += std::abs(its[a]);
          total_b += std::abs(its[a]);
        }
    }
    prof.mark(1);
    // orthogonalisation (Lanczos.m:53-69); the full Gram-Schmidt of :69 as
    // classical GS with a second pass when the first cancelled much of r
    // (||c||^2 > ||r||_B^2 / 2, the DGKS test).  The mixed form carries B r,
    // which gives ||r||_B; the FP64 form always takes the second pass.
    std::vector<int> second(na, 0);
    {
      // r -= alpha q_j (- beta q_{j-1}) (Lanczos.m:55,62), coefficients from the host
      std::vector<int2> sp(na, make_int2(0, 0)), sp63(na, make_int2(0, 0)), sp66(na, make_int2(0, 0)),
          spfull(na, make_int2(0, 0));
      std::vector<double2> hcf((size_t)na * 128, make_double2(0.0, 0.0));
      for (int a = 0; a < na; ++a) {
        if (S[a].done) continue;
        LzInst& I = S[a];
        const int j = I.j - 1;
        const double alpha = al[a].x;
        I.Alpha.push_back(alpha);
        if (I.j == 1) {
          sp[a] = make_int2(j, 1);
          hcf[(size_t)a * 128] = make_double2(alpha, 0.0);
        } else if (I.justRestarted) {
          sp63[a] = make_int2(0, I.j);  // Lanczos.m:58-59, full pass with O(1) coefficients: FP64
        } else {
          sp[a] = make_int2(j - 1, 2);
          hcf[(size_t)a * 128] = make_double2(I.beta, 0.0);
          hcf[(size_t)a * 128 + 1] = make_double2(alpha, 0.0);
          sp63[a] = make_int2(j - 1, 1);  // :63
        }
        sp66[a] = make_int2(j, 1);       // :66
        spfull[a] = make_int2(0, I.j);   // :69
        second[a] = 1;
        I.justRestarted = false;
        I.steps++;
        n_first++;
      }
      int maxm = 0;
      const int2* d = upload_span(sp, &maxm);
      if (!d) return cuda_fail(&P, cudaErrorUnknown, "lanczos span upload");
      FAME_CK(h2d_async(P, coef, hcf.data(), sizeof(double2) * hcf.size()), "lanczos gs");
      if (maxm > 0) {
        FAME_CK(gs_combo(PR, L, Q, qs, L, na, d, coef, 128, st), "lanczos gs");
        if (mixed) FAME_CK(gs_combo(BPR, L, BQ, qs, L, na, d, coef, 128, st), "lanczos gs");
      }
      if ((rc = project_b(sp63, false))) return rc;
      if ((rc = project_b(sp66, false))) return rc;
      if (mixed)  // ||r||_B^2 before the full pass (DGKS test below)
        FAME_CK(dot_batched<double>(PR, L, 0, 1, BPR, L, L, na, ddot + na, part, nblkb, dmask, st), "lanczos norm");
      if ((rc = project_b(spfull, mixed))) return rc;  // :69, first pass
    }
    if (mixed) {
      std::vector<double2> hc((size_t)na * 128), rbn(na);
      FAME_CK(cudaMemcpyAsync(hc.data(), coef, sizeof(double2) * hc.size(), cudaMemcpyDeviceToHost, st), "lanczos gs");
      FAME_CK(cudaMemcpyAsync(rbn.data(), ddot + na, sizeof(double2) * na, cudaMemcpyDeviceToHost, st), "lanczos gs");
      FAME_CK(cudaStreamSynchronize(st), "lanczos gs");
      for (int a = 0; a < na; ++a) {
        if (!second[a]) continue;
        double c2 = 0.0;
        for (int i = 0; i < S[a].j; ++i) c2 += hc[(size_t)a * 128 + i].x * hc[(size_t)a * 128 + i].x +
                                               hc[(size_t)a * 128 + i].y * hc[(size_t)a * 128 + i].y;
        second[a] = !(c2 <= 0.5 * rbn[a].x);
        n_second += second[a];
      }
    }
    {
      std::vector<int2> sp2(na, make_int2(0, 0));
      for (int a = 0; a < na; ++a)
        if (second[a] && !S[a].done) sp2[a] = make_int2(0, S[a].j);
      if ((rc = project_b(sp2, mixed))) return rc;  // :69, second pass
    }
    prof.mark(2);
    // rr = fncB(r); beta = sqrt(r'*rr); v = r/beta  (Lanczos.m:72-74)
    if (!mixed) {
      FAME_CK(fncB64(PR, BPR), "lanczos fncB");
      for (int a = 0; a < na; ++a) {
        total_b += mask[a];
        S[a].bapplies += mask[a];
      }
    } else {
      // Instances with an extreme Ritz-value spread (the shifted zero modes
      // near Gamma) take B r by an explicit FP64 apply, as Lanczos.m:72 does:
      // a 1e-13 error in the cached B*q columns would leave a component of
      // the lambda ~ 1e4 modes that the other bands' residuals amplify.
      bool anyx = false;
      std::vector<int> xm(na, 0);
      for (int a = 0; a < na; ++a) {
        xm[a] = (!S[a].done && S[a].explicit_br) ? 1 : 0;
        anyx |= xm[a] != 0;
      }
      if (anyx) {
        FAME_CK(h2d_async(P, dmask, xm.data(), sizeof(int) * na), "lanczos mask");
        FAME_CK(fncB64(PR, BPR), "lanczos fncB");
        FAME_CK(upload_mask(), "lanczos mask");
        for (int a = 0; a < na; ++a) {
          total_b += xm[a];
          S[a].bapplies += xm[a];
        }
      }
    }
    std::vector<double2> rr;
    if ((rc = batched_dot(PR, BPR, rr))) return rc;
    std::vector<double> s(na, 0.0);
    for (int a = 0; a < na; ++a) {
      if (S[a].done) continue;
      const double b2 = rr[a].x;
      if (!std::isfinite(b2)) return fail(&P, FAME_ERR_NAN, "lanczos: non-finite beta");
      S[a].beta = std::sqrt(std::fabs(b2));
      if (!(S[a].beta > 0.0)) return fail(&P, FAME_ERR_BREAKDOWN, "lanczos: zero beta (invariant subspace)");
      S[a].Beta.push_back(S[a].beta);
      s[a] = 1.0 / S[a].beta;
    }
    if ((rc = scale_vecs(PR, V, s))) return rc;
    if ((rc = scale_vecs(BPR, BV, s))) return rc;
    prof.mark(3);
    // cycle ends
    for (int a = 0; a < na; ++a) {
      if (S[a].done) continue;
      LzInst& I = S[a];
      I.j++;
      if (I.j <= p) continue;
      // H = blkdiag(diag(d), tridiag(Alpha, Beta)) with arrowhead c (Lanczos.m:93-98)
      const int kd = (int)I.d.size();
      const int m1 = (int)I.Alpha.size();
      const int np = kd + m1;
      std::vector<double> H((size_t)np * np, 0.0);
      for (int i = 0; i < kd; ++i) H[(size_t)i * np + i] = I.d[i];
      for (int i = 0; i < m1; ++i) {
        H[(size_t)(kd + i) * np + kd + i] = I.Alpha[i];
        if (i + 1 < m1) {
          H[(size_t)(kd + i) * np + kd + i + 1] = I.Beta[i];
          H[(size_t)(kd + i + 1) * np + kd + i] = I.Beta[i];
        }
      }
      for (int i = 0; i < kd; ++i) {
        H[(size_t)i * np + kd] = I.c[i];
        H[(size_t)kd * np + i] = I.c[i];
      }
      I.Alpha.clear();
      I.Beta.clear();
      std::vector<double> w, Uv;
      jacobi_eig(H, np, w, Uv);
      std::vector<int> ind(np);
      std::iota(ind.begin(), ind.end(), 0);
      std::stable_sort(ind.begin(), ind.end(), [&](int x, int y) { return w[x] > w[y]; });  // :109
      int nconv = 0;
      double rel_max = 0.0;  // largest relative Ritz residual of the wanted pairs
      for (int i = 0; i < I.k0; ++i) {
        const double resi = std::fabs(I.beta * Uv[(size_t)ind[i] * np + np - 1]);  // :106
        const double scale = std::max(std::pow(eps, 2.0 / 3.0), std::fabs(w[ind[i]]));
        if (resi < tol * scale) nconv++;  // :114
        rel_max = std::max(rel_max, resi / scale);
      }
      if (nconv >= I.k0 || I.mm == maxit) {  // :117
        if (nconv < I.k0) rc_final = FAME_ERR_NOT_CONVERGED;
        I.d.resize(I.k0);
        I.U.assign((size_t)np * I.k0, 0.0);
        for (int c2 = 0; c2 < I.k0; ++c2) {
          I.d[c2] = w[ind[c2]];
          for (int i = 0; i < np; ++i) I.U[(size_t)c2 * np + i] = Uv[(size_t)ind[c2] * np + i];
        }
        I.done = true;
        continue;
      }
      if (mixed) {
        // The error an inexact B^{-1} leaves in a Ritz pair is amplified by
        // lambda_max / lambda_j in its residual (near Gamma the shifted
        // zero modes have lambda ~ 1e4); tighten this instance's inner
        // tolerance by the spread of the wanted Ritz values.
        const double lmax = std::fabs(w[ind[0]]), lk = std::fabs(w[ind[I.k0 - 1]]);
        const double spread = lmax > 0.0 ? std::min(1.0, lk / lmax) : 1.0;
        I.itol = std::max(P.opt_itol_floor, itol * spread);
        // Relaxed inner accuracy (FAME_OPT_RELAX = c > 0): once every wanted
        // Ritz pair's relative residual is below c, the error a new Lanczos
        // vector carries enters the wanted pairs with a weight of about that
        // residual, so the inner tolerance may grow by c / residual (at most
        // FAME_OPT_RELAX_MAX); no relaxation for the Gamma-like instances at
        // the floor.
        if (P.opt_relax > 0.0 && !I.explicit_br && rel_max > 0.0)
          I.itol *= std::min(P.opt_relax_max, std::max(1.0, P.opt_relax / rel_max));
        I.refresh_bq = !I.explicit_br && spread < 1e-3;
        I.explicit_br = spread < 1e-3;
      }
      int k = I.k0 + std::min(nconv, (p - I.k0) / 2);  // :122
      if (k == 1 && p > 3) k = p / 2;
      std::vector<double> Uk((size_t)np * k);
      I.d.assign(k, 0.0);
      I.c.assign(k, 0.0);
      for (int c2 = 0; c2 < k; ++c2) {
        I.d[c2] = w[ind[c2]];
        for (int i = 0; i < np; ++i) Uk[(size_t)c2 * np + i] = Uv[(size_t)ind[c2] * np + i];
        I.c[c2] = I.beta * Uk[(size_t)c2 * np + np - 1];  // :140
      }
      // Q(:,1:k) = Q*U ; BQ likewise (Lanczos.m:135-137)
      FAME_CK(h2d_async(P, dU, Uk.data(), sizeof(double) * Uk.size()), "lz restart");
      double2* Qa = Q + (size_t)a * p * L;
      double2* BQa = BQ + (size_t)a * p * L;
      FAME_CK(block_rot<double>(Qa, TMP, L, L, np, k, dU, st), "lz restart");
      FAME_CK(cudaMemcpyAsync(Qa, TMP, cb * k, cudaMemcpyDeviceToDevice, st), "lz restart");
      FAME_CK(block_rot<double>(BQa, TMP, L, L, np, k, dU, st), "lz restart");
      FAME_CK(cudaMemcpyAsync(BQa, TMP, cb * k, cudaMemcpyDeviceToDevice, st), "lz restart");
      if (I.refresh_bq) {
        // first restart of a Gamma-like instance: exact FP64 B*Q for the kept columns
        std::vector<int> ii(k, I.inst);
        int* di = (int*)workspace(P, WS_LZ_INST + 60, sizeof(int) * k, &e);
        FAME_CK(e, "lz restart");
        FAME_CK(h2d_async(P, di, ii.data(), sizeof(int) * k), "lz restart");
        FAME_CK(ensure_work(P, std::max(k, na)), "lz restart");
        VecCtx ck;
        ck.inst = di;
        ck.nk = P.nk;
        double2* w0 = (double2*)P.d_work;
        FAME_CK(launch_fncB<double>(P, Qa, BQa, k, ck, w0, w0 + (size_t)k * 6 * P.Nq, st), "lz restart");
        total_b += k;
        I.bapplies += k;
        I.refresh_bq = false;
      }
      if (int rc2 = copy_lo(a, 0, k)) return rc2;
      FAME_CK(cudaStreamSynchronize(st), "lz restart");
      I.k = k;
      I.justRestarted = true;
      I.sizeV = k + 1;
      I.j = k + 1;
      I.mm++;
      I.restarts++;
    }
    prof.mark(4);
  }
  if (prof.on)
    std::fprintf(stderr,
                 "[fame lanczos] instances %d: fncA+alpha %.3fs  B^-1 %.3fs  reorth %.3fs  beta %.3fs  restart %.3fs"
                 "  (second GS passes %lld of %lld)\n",
                 na, prof.acc[0], prof.acc[1], prof.acc[2], prof.acc[3], prof.acc[4], n_second, n_first);
  // Ritz vectors ev = Q*U(:, ind(1:k0)) (Lanczos.m:146-152) and outputs
  double2* EV = ev;
  for (int a = 0; a < na; ++a) {
    LzInst& I = S[a];
    for (int i = 0; i < k0; ++i) ew[(size_t)a * k0 + i] = I.d[i];
  }
  P.refine_res_before.clear();
  if (mixed && P.opt_refine) {
    // FP64 refinement sweep of every Ritz pair (ritz_refine), batched over the instances
    double2* X = (double2*)workspace(P, WS_RF_X, cb * (size_t)na * k0, &e);
    FAME_CK(e, "refine workspace");
    for (int a = 0; a < na; ++a) {
      LzInst& I = S[a];
      const int np = (int)(I.U.size() / k0);
      FAME_CK(h2d_async(P, dU, I.U.data(), sizeof(double) * I.U.size()), "lz ritz");
      FAME_CK(block_rot<double>(Q + (size_t)a * p * L, X + (size_t)a * k0 * L, L, L, np, k0, dU, st), "lz ritz");
    }
    std::vector<double> rb((size_t)na * k0), ra((size_t)na * k0);
    std::vector<long long> bv((size_t)na * k0, 0), cv((size_t)na * k0, 0);
    int rrc = ritz_refine(P, insts, k0, X, ew, rb.data(), ra.data(), P.opt_refine_tol, bv.data(), cv.data());
    if (rrc != FAME_OK) return rrc;
    for (int a = 0; a < na; ++a)
      for (int i = 0; i < k0; ++i) {
        S[a].bapplies += bv[(size_t)a * k0 + i];
        S[a].cgits += cv[(size_t)a * k0 + i];
      }
    P.refine_res_before = rb;
    if (EV) FAME_CK(cudaMemcpyAsync(EV, X, cb * (size_t)na * k0, cudaMemcpyDeviceToDevice, st), "refine out");
    if (res) std::copy(ra.begin(), ra.end(), res);
    FAME_CK(cudaStreamSynchronize(st), "refine out");
  }
  if (stats)
    for (int a = 0; a < na; ++a) {
      stats[a * 4 + 0] = S[a].steps;
      stats[a * 4 + 1] = S[a].restarts;
      stats[a * 4 + 2] = S[a].bapplies;  // FP64 B applies of this instance
      stats[a * 4 + 3] = S[a].cgits;     // inner CG iterations of this instance
    }
  if ((EV || res) && !(mixed && P.opt_refine)) {
    // one instance at a time through TMP (p columns available)
    for (int a = 0; a < na; ++a) {
      LzInst& I = S[a];
      const int np = (int)(I.U.size() / k0);
      FAME_CK(h2d_async(P, dU, I.U.data(), sizeof(double) * I.U.size()), "lz ritz");
      FAME_CK(block_rot<double>(Q + (size_t)a * p * L, TMP, L, L, np, k0, dU, st), "lz ritz");
      if (EV) FAME_CK(cudaMemcpyAsync(EV + (size_t)a * k0 * L, TMP, cb * k0, cudaMemcpyDeviceToDevice, st), "lz ritz");
      if (res) {
        // ||A x - lambda B x|| / ||x|| in FP64 for each Ritz pair
        VecCtx c1;
        c1.nk = P.nk;
        std::vector<int> ii(k0, I.inst);
        int* di = (int*)workspace(P, WS_LZ_INST + 50, sizeof(int) * k0, &e);
        FAME_CK(e, "lz res");
        FAME_CK(h2d_async(P, di, ii.data(), sizeof(int) * k0), "lz res");
        c1.inst = di;
        double2* AX = (double2*)workspace(P, WS_LZ_INST + 51, cb * k0, &e);
        FAME_CK(e, "lz res");
        double2* BX = (double2*)workspace(P, WS_LZ_INST + 52, cb * k0, &e);
        FAME_CK(e, "lz res");
        FAME_CK(ensure_work(P, k0), "lz res");
        double2* w0 = (double2*)P.d_work;
        double2* w1 = w0 + (size_t)k0 * 6 * P.Nq;
        FAME_CK(launch_fncA<double>(P, TMP, AX, k0, c1, st), "lz res");
        FAME_CK(launch_fncB<double>(P, TMP, BX, k0, c1, w0, w1, st), "lz res");
        std::vector<double2> cl(k0), cb0(k0);
        for (int i = 0; i < k0; ++i) {
          cl[i] = make_double2(I.d[i], 0.0);
          cb0[i] = make_double2(-1.0, 0.0);
        }
        // NFSEP residual of EvaluteError_Chiral_no_inv.m:20 for the
        // B-normalised Ritz vector x: || B x - omega A x ||, omega = 1/lambda.
        // AX <- BX - omega AX
        double2* al2 = (double2*)workspace(P, WS_LZ_INST + 53, sizeof(double2) * 2 * k0, &e);
        FAME_CK(e, "lz res");
        std::vector<double2> ones(k0, make_double2(1.0, 0.0)), mw(k0);
        for (int i = 0; i < k0; ++i) mw[i] = make_double2(-1.0 / I.d[i], 0.0);
        FAME_CK(h2d_async(P, al2, ones.data(), sizeof(double2) * k0), "lz res");
        FAME_CK(h2d_async(P, al2 + k0, mw.data(), sizeof(double2) * k0), "lz res");
        FAME_CK(axpby_batched<double>(BX, AX, L, L, k0, al2, al2 + k0, nullptr, st), "lz res");
        const int nb = dot_blocks(P, L, k0);
        double2* pp = (double2*)workspace(P, WS_LZ_INST + 54, sizeof(double2) * (nb * k0 + 2 * k0) + 64, &e);
        FAME_CK(e, "lz res");
        double2* o1 = pp + (size_t)nb * k0;
        FAME_CK(dot_batched<double>(AX, L, 0, 1, AX, L, L, k0, o1, pp, nb, nullptr, st), "lz res");
        std::vector<double2> h2(k0);
        FAME_CK(cudaMemcpyAsync(h2.data(), o1, sizeof(double2) * k0, cudaMemcpyDeviceToHost, st), "lz res");
        FAME_CK(cudaStreamSynchronize(st), "lz res");
        for (int i = 0; i < k0; ++i) res[(size_t)a * k0 + i] = std::sqrt(std::max(0.0, h2[i].x));
      }
    }
    FAME_CK(cudaStreamSynchronize(st), "lz out");
  }
  if (rc_final != FAME_OK) fail(&P, rc_final, "lanczos: maxit restarts reached before tol");
  return rc_final;
}

}  // namespace fame

using namespace fame;


extern "C" int fame_lanczos(fame_plan_t h, int prec, int inst, int k, double tol, int maxit, int p, const double* v0,
                            double inner_tol, double* ew, void* ev, double* res, long long* stats) {
  if (!h || !ew) return FAME_ERR_BAD_ARG;
  Plan& P = h->P;
  if (inst < 0 || inst >= P.nk) return fail(&P, FAME_ERR_BAD_ARG, "fame_lanczos: bad instance");
  if (prec != FAME_C128 && prec != FAME_C64) return fail(&P, FAME_ERR_BAD_ARG, "fame_lanczos: bad precision");
  std::vector<int> insts{inst};
  return lanczos_run(P, prec, insts, k, tol, maxit, p, v0, inner_tol, ew, (double2*)ev, res, stats);
}

extern "C" int fame_band_solve(fame_plan_t h, int prec, int k, double tol, int maxit, int p, double inner_tol,
                               double* ew, void* ev, double* res, long long* stats) {
  if (!h || !ew) return FAME_ERR_BAD_ARG;
  Plan& P = h->P;
  if (prec != FAME_C128 && prec != FAME_C64) return fail(&P, FAME_ERR_BAD_ARG, "fame_band_solve: bad precision");
  std::vector<int> insts(P.nk);
  std::iota(insts.begin(), insts.end(), 0);
  return lanczos_run(P, prec, insts, k, tol, maxit, p, nullptr, inner_tol, ew, (double2*)ev, res, stats);
}
