// Interior eigenpairs by SIRA with locking, following
// light_locked_Huang/GEP_AB_Herm_JDSIRA_{Driver4,Locking4}.m.
//
// The reference calls Driver4(fncB, fncA, ...), so its pencil is
//   fncB x = theta fncA x      (theta = omega, the frequency)
// and it targets the Ritz values closest to `target` from above ('CL'; the
// option FAME_OPT_SIRA_NEAREST takes the closest on either side).  Per outer step:
//   * projected pencil  V^H B V y = theta V^H A V y  on the Euclidean-orthonormal
//     search space V, which also holds the locked eigenvectors (Locking4.m:91-103,115)
//   * the Ritz pair closest to the target among the unlocked ones (the locked
//     ones are the Ritz vectors living in the locked coordinates;
//     Choose_Ritz_Pair_Unsymm4.m matches them by value and multiplicity)
//   * residual r = B u - theta A u of the unit Ritz vector (Locking4.m:172-179)
//   * SIRA correction t = (B - shift A)^{-1} r solved loosely
//     (SIRA_solve_residual_LS_GEP.m:54); shift = 0 is the reference, whose
//     shift term (GEP_shift_mtx_prod_vec.m:29) is commented out, so the
//     correction solves with fncB alone (CG on the positive definite B);
//     shift != 0 solves the shifted indefinite system by MINRES; then MGS
//     against V and expansion (Locking4.m:306-341)
//   * restart with the current and the next Ritz vectors when V is full
//     (Locking4.m:361-381); locking of converged pairs (Locking4.m:425-505).
// B^{-1} is the batched CG of this library (complex64 or complex128, with the
// averaged-medium preconditioner when enabled) in place of MATLAB's minres on
// the same Hermitian positive definite fncB.  The projected pencil is solved
// on the host in FP64 as the Hermitian-definite pencil (V^H A V) y = mu (V^H B V) y,
// theta = 1/mu.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <complex>
#include <numeric>
#include <vector>

#include "graph_impl.h"
#include "krylov.h"
#include "linalg_host.h"

namespace fame {

using cd = std::complex<double>;

namespace {

enum JdWs { JD_V = 300, JD_BV, JD_AV, JD_VEC, JD_SMALL, JD_TMP, JD_PART, JD_R32, JD_INST };

#define JD_CK(expr, where)                                  \
  do {                                                      \
    cudaError_t e_ = (expr);                                \
    if (e_ != cudaSuccess) return cuda_fail(&P, e_, where); \
  } while (0)

}  // namespace

// MINRES (Paige & Saunders, 1975) on the Hermitian operator B - shift*A for one
// vector: the Lanczos recurrence with Givens rotations, vectors in the
// precision R, scalars in FP64.  The reference's SIRA inner solver is MATLAB
// minres (SIRA_solve_residual_LS_GEP.m:54).
//
// The scalar recurrence runs on the device (two single-thread kernels per
// iteration), every vector update reads its coefficients from device memory
// and is masked by an `active` flag cleared at convergence, and the buffer
// rotations are device copies.  An iteration is therefore a fixed launch
// sequence: blocks of kMinresBlock iterations are captured once and replayed
// from a CUDA graph, with one host check per block.
namespace {

constexpr int kMinresBlock = 8;

// Scalar state of one MINRES solve (FP64, device).
enum MrSlot {
  MR_BETA = 0, MR_OLDB, MR_DBAR, MR_EPS, MR_PHIBAR, MR_CS, MR_SN, MR_TOLB,
  MR_CV,        // 1 / beta               (v = y / beta)
  MR_CR1,       // -beta / oldb           (y -= (beta/oldb) r1; 0 in the first step)
  MR_CR2,       // -alfa / beta           (y -= (alfa/beta) r2)
  MR_PHI,       // x += phi w
  MR_W0, MR_W1, MR_W2,  // w = (v - oldeps w1 - delta w2) / gamma
  MR_ONE, MR_ZERO, MR_NSLOT
};
struct MrInt {
  int active, itn, nan;
};

__global__ void k_minres_alfa(double* S, const double2* __restrict__ dot, const MrInt* st) {
  if (!st->active) return;
  S[MR_CR2] = -dot->x / S[MR_BETA];
}

__global__ void k_minres_givens(double* S, const double2* __restrict__ alfa_dot, const double2* __restrict__ b2_dot,
                                MrInt* st) {
  if (!st->active) return;
  const double alfa = alfa_dot->x, b2n = b2_dot->x;
  st->itn += 1;
  if (!isfinite(alfa) || !isfinite(b2n)) {
    st->nan = 1;
    st->active = 0;
    return;
  }
  const double oldb = S[MR_BETA];
  const double beta = sqrt(fmax(b2n, 0.0));
  const double cs = S[MR_CS], sn = S[MR_SN], dbar = S[MR_DBAR];
  const double oldeps = S[MR_EPS];
  const double delta = cs * dbar + sn * alfa;
  const double gbar = sn * dbar - cs * alfa;
  S[MR_EPS] = sn * beta;
  S[MR_DBAR] = -cs * beta;
  const double gamma = fmax(sqrt(gbar * gbar + beta * beta), 1e-300);
  const double cs2 = gbar / gamma, sn2 = beta / gamma;
  S[MR_CS] = cs2;
  S[MR_SN] = sn2;
  S[MR_PHI] = cs2 * S[MR_PHIBAR];
  S[MR_PHIBAR] = sn2 * S[MR_PHIBAR];
  S[MR_W0] = 1.0 / gamma;
  S[MR_W1] = -oldeps / gamma;
  S[MR_W2] = -delta / gamma;
  S[MR_OLDB] = oldb;
  S[MR_BETA] = beta;
  S[MR_CV] = beta > 0.0 ? 1.0 / beta : 0.0;
  S[MR_CR1] = -beta / oldb;
  if (S[MR_PHIBAR] <= S[MR_TOLB] || beta == 0.0) st->active = 2;  // converged: finish this step's updates
}

// out = S[ia] x + S[ib] y + S[ic] w (y, w may be null), only while active.
template <class R>
__global__ void k_lincomb_dev(cx<R>* __restrict__ out, const double* __restrict__ S, int ia, const cx<R>* x, int ib,
                              const cx<R>* y, int ic, const cx<R>* w, long long len, const MrInt* __restrict__ st) {
  if (!st->active) return;
  const R a = R(S[ia]), b = R(S[ib]), c = R(S[ic]);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x) {
    cx<R> v = x[i];
    R rx = a * v.x, ry = a * v.y;
    if (y) {
      const cx<R> u = y[i];
      rx += b * u.x;
      ry += b * u.y;
    }
    if (w) {
      const cx<R> u = w[i];
      rx += c * u.x;
      ry += c * u.y;
    }
    out[i] = mk<R>(rx, ry);
  }
}

// active 2 (converged during this step) -> 0 once the step's updates are done
__global__ void k_minres_close(MrInt* st) {
  if (st->active == 2) st->active = 0;
}

int lincomb_dev_grid(long long len) {
  long long g = (len + 255) / 256;
  return (int)std::min<long long>(g, 1216);
}

}  // namespace

template <class R>
int minres_shifted(Plan& P, const cx<R>* b, cx<R>* x, const int* d_inst, double shift, double tol, int maxit,
                   int* iters, double* relres) {
  cudaStream_t st = P.stream;
  const long long L = 4 * P.Nq;
  const size_t vb = sizeof(cx<R>) * L;
  cudaError_t e;
  cx<R>* base = (cx<R>*)workspace(P, JD_R32 + 20 + (sizeof(R) == 4 ? 0 : 1), vb * 8, &e);
  JD_CK(e, "minres workspace");
  cx<R> *v = base, *y = base + L, *r1 = base + 2 * L, *r2 = base + 3 * L, *w = base + 4 * L, *w1 = base + 5 * L,
        *w2 = base + 6 * L, *ta = base + 7 * L;
  char* sm = (char*)workspace(P, JD_R32 + 30, sizeof(double2) * (3 * 256 + 8) + sizeof(double) * MR_NSLOT + 64, &e);
  static_assert(sizeof(MrInt) + sizeof(int) <= 64, "loop pass counter after the integer state");
  JD_CK(e, "minres workspace");
  double2* part = (double2*)sm;          // dot partials
  double2* dalfa = part + 256;           // v . y
  double2* db2 = dalfa + 1;              // |r2|^2
  double2* dbb = db2 + 1;                // |b|^2
  double* S = (double*)(dbb + 5);
  MrInt* SI = (MrInt*)(S + MR_NSLOT);
  JD_CK(ensure_work(P, 1), "minres scratch");
  VecCtx c1;
  c1.inst = d_inst;
  c1.nk = P.nk;
  c1.active = &SI->active;  // the operator's kernels skip once converged
  const int gl = lincomb_dev_grid(L);
  auto lc = [&](cudaStream_t cs, cx<R>* out, int ia, const cx<R>* xx, int ib, const cx<R>* yy, int ic,
                const cx<R>* ww) -> cudaError_t {
    FAME_LAUNCHED(1);
    k_lincomb_dev<R><<<gl, 256, 0, cs>>>(out, S, ia, xx, ib, yy, ic, ww, L, SI);
    return cudaGetLastError();
  };
  auto op = [&](cudaStream_t cs, const cx<R>* in, cx<R>* out) -> cudaError_t {  // out = B in - shift A in
    cx<R>* w0 = (cx<R>*)P.d_work;
    cudaError_t e2 = launch_fncB<R>(P, in, out, 1, c1, w0, w0 + 6 * P.Nq, cs);
    if (e2 != cudaSuccess || shift == 0.0) return e2;
    e2 = launch_fncA<R>(P, in, ta, 1, c1, cs);
    if (e2 != cudaSuccess) return e2;
    return lincomb3<R>(out, 1.0, out, -shift, ta, 0.0, nullptr, L, cs);
  };
  // one MINRES step (Paige-Saunders), every scalar on the device
  auto step = [&](cudaStream_t cs) -> cudaError_t {
    cudaError_t e2 = lc(cs, v, MR_CV, y, MR_ZERO, nullptr, MR_ZERO, nullptr);     // v = y / beta
    if (e2 == cudaSuccess) e2 = op(cs, v, y);                                      // y = (B - shift A) v
    if (e2 == cudaSuccess) e2 = lc(cs, y, MR_ONE, y, MR_CR1, r1, MR_ZERO, nullptr);  // y -= (beta/oldb) r1
    if (e2 == cudaSuccess) e2 = dot_batched<R>(v, 0, 0, 1, y, 0, L, 1, dalfa, part, 256, &SI->active, cs);
    if (e2 == cudaSuccess) {
      FAME_LAUNCHED(1);
      k_minres_alfa<<<1, 1, 0, cs>>>(S, dalfa, SI);
      e2 = cudaGetLastError();
    }
    if (e2 == cudaSuccess) e2 = lc(cs, y, MR_ONE, y, MR_CR2, r2, MR_ZERO, nullptr);  // y -= (alfa/beta) r2
    if (e2 == cudaSuccess) e2 = lc(cs, r1, MR_ONE, r2, MR_ZERO, nullptr, MR_ZERO, nullptr);  // r1 <- r2
    if (e2 == cudaSuccess) e2 = lc(cs, r2, MR_ONE, y, MR_ZERO, nullptr, MR_ZERO, nullptr);   // r2 <- y
    if (e2 == cudaSuccess) e2 = dot_batched<R>(r2, 0, 0, 1, r2, 0, L, 1, db2, part, 256, &SI->active, cs);
    if (e2 == cudaSuccess) {
      FAME_LAUNCHED(1);
      k_minres_givens<<<1, 1, 0, cs>>>(S, dalfa, db2, SI);
      e2 = cudaGetLastError();
    }
    if (e2 == cudaSuccess) e2 = lc(cs, w1, MR_ONE, w2, MR_ZERO, nullptr, MR_ZERO, nullptr);  // w1 <- w2
    if (e2 == cudaSuccess) e2 = lc(cs, w2, MR_ONE, w, MR_ZERO, nullptr, MR_ZERO, nullptr);   // w2 <- w
    if (e2 == cudaSuccess) e2 = lc(cs, w, MR_W0, v, MR_W1, w1, MR_W2, w2);      // w = (v - e w1 - d w2)/g
    if (e2 == cudaSuccess) e2 = lc(cs, x, MR_ONE, x, MR_PHI, w, MR_ZERO, nullptr);  // x += phi w
    if (e2 == cudaSuccess) {
      FAME_LAUNCHED(1);
      k_minres_close<<<1, 1, 0, cs>>>(SI);
      e2 = cudaGetLastError();
    }
    return e2;
  };

  JD_CK(cudaMemsetAsync(x, 0, vb, st), "minres init");
  JD_CK(cudaMemsetAsync(w, 0, vb, st), "minres init");
  JD_CK(cudaMemsetAsync(w2, 0, vb, st), "minres init");
  JD_CK(cudaMemsetAsync(r1, 0, vb, st), "minres init");
  JD_CK(cudaMemcpyAsync(r2, b, vb, cudaMemcpyDeviceToDevice, st), "minres init");
  JD_CK(cudaMemcpyAsync(y, b, vb, cudaMemcpyDeviceToDevice, st), "minres init");
  JD_CK(dot_batched<R>(b, 0, 0, 1, b, 0, L, 1, dbb, part, 256, nullptr, st), "minres dot");
  double2 hb;
  JD_CK(cudaMemcpyAsync(&hb, dbb, sizeof(double2), cudaMemcpyDeviceToHost, st), "minres dot");
  JD_CK(cudaStreamSynchronize(st), "minres dot");
  if (!std::isfinite(hb.x)) return fail(&P, FAME_ERR_NAN, "minres: non-finite right-hand side");
  const double beta1 = std::sqrt(std::max(hb.x, 0.0));
  if (beta1 == 0.0) {
    if (iters) *iters = 0;
    if (relres) *relres = 0.0;
    return FAME_OK;
  }
  double hs[MR_NSLOT] = {};
  hs[MR_BETA] = beta1;
  hs[MR_OLDB] = 0.0;
  hs[MR_PHIBAR] = beta1;
  hs[MR_CS] = -1.0;
  hs[MR_SN] = 0.0;
  hs[MR_TOLB] = tol * beta1;
  hs[MR_CV] = 1.0 / beta1;
  hs[MR_CR1] = 0.0;
  hs[MR_ONE] = 1.0;
  hs[MR_ZERO] = 0.0;
  MrInt hi{1, 0, 0};
  JD_CK(h2d_async(P, S, hs, sizeof(hs)), "minres init");
  JD_CK(h2d_async(P, SI, &hi, sizeof(hi)), "minres init");
  uint64_t shift_bits;
  std::memcpy(&shift_bits, &shift, sizeof(shift));
  const std::vector<uintptr_t> gkey = {0x4d52u, sizeof(R), (uintptr_t)P.n, (uintptr_t)base, (uintptr_t)sm,
                                       (uintptr_t)x, (uintptr_t)d_inst, (uintptr_t)P.d_work, (uintptr_t)shift_bits,
                                       (uintptr_t)kMinresBlock};
  bool use_graph = P.opt_graph != 0;
  MrInt hst = hi;
  double phibar = beta1;
  int done_steps = 0;
  if (P.opt_graph >= 2 && maxit >= kMinresBlock) {
    // all blocks of kMinresBlock steps in one graph launch, the stopping
    // test on the device after each block; the host waits once
    int* passes = (int*)(SI + 1);
    std::vector<uintptr_t> wkey = gkey;
    wkey.push_back((uintptr_t)0x5748494cu);
    wkey.push_back((uintptr_t)(maxit / kMinresBlock));
    unsigned long long body_nodes = 0;
    cudaError_t ge = graph_replay_while(P, wkey, [&](cudaStream_t cs) -> cudaError_t {
      for (int i = 0; i < kMinresBlock; ++i) {
        cudaError_t e2 = step(cs);
        if (e2 != cudaSuccess) return e2;
      }
      return cudaSuccess;
    }, &SI->active, 1, passes, maxit / kMinresBlock, &body_nodes);
    if (ge == cudaSuccess) {
      int np = 0;
      JD_CK(cudaMemcpyAsync(&hst, SI, sizeof(MrInt), cudaMemcpyDeviceToHost, st), "minres check");
      JD_CK(cudaMemcpyAsync(&phibar, S + MR_PHIBAR, sizeof(double), cudaMemcpyDeviceToHost, st), "minres check");
      JD_CK(cudaMemcpyAsync(&np, passes, sizeof(int), cudaMemcpyDeviceToHost, st), "minres check");
      JD_CK(cudaStreamSynchronize(st), "minres check");
      FAME_KERNELS_RAN(body_nodes * (unsigned long long)np);
      done_steps = np * kMinresBlock;
      if (hst.nan) return fail(&P, FAME_ERR_NAN, "minres: non-finite value");
    } else {
      cudaGetLastError();  // no graph loop (nothing of it ran): the blocks below take over
    }
  }
  while (done_steps < maxit && hst.active) {
    const int nb = std::min(kMinresBlock, maxit - done_steps);
    bool issued = false;
    if (use_graph && nb == kMinresBlock) {
      cudaError_t ge = graph_replay(P, gkey, [&](cudaStream_t cs) -> cudaError_t {
        for (int i = 0; i < kMinresBlock; ++i) {
          cudaError_t e2 = step(cs);
          if (e2 != cudaSuccess) return e2;
        }
        return cudaSuccess;
      });
      if (ge == cudaSuccess) issued = true;
      else use_graph = false;
    }
    if (!issued)
      for (int i = 0; i < nb; ++i) JD_CK(step(st), "minres step");
    done_steps += nb;
    JD_CK(cudaMemcpyAsync(&hst, SI, sizeof(MrInt), cudaMemcpyDeviceToHost, st), "minres check");
    JD_CK(cudaMemcpyAsync(&phibar, S + MR_PHIBAR, sizeof(double), cudaMemcpyDeviceToHost, st), "minres check");
    JD_CK(cudaStreamSynchronize(st), "minres check");
    if (hst.nan) return fail(&P, FAME_ERR_NAN, "minres: non-finite value");
    if (!hst.active) break;
  }
  if (iters) *iters = hst.itn;
  if (relres) *relres = phibar / beta1;
  return phibar <= tol * beta1 ? FAME_OK : FAME_ERR_NOT_CONVERGED;
}

template int minres_shifted<float>(Plan&, const float2*, float2*, const int*, double, double, int, int*, double*);
template int minres_shifted<double>(Plan&, const double2*, double2*, const int*, double, double, int, int*, double*);

int jdsira_run(Plan& P, int inst, int inner_prec, int nev, double target, double shift, double tol, int no_restart,
               int rpd, double inner_tol, int inner_maxit, double* ew_out, double2* ev_out, double* res_out,
               long long* stats) {
  if (inst < 0 || inst >= P.nk || nev < 1 || no_restart < 4 || rpd < 1 || !(tol > 0.0) || !(inner_tol > 0.0) ||
      inner_maxit < 1)
    return fail(&P, FAME_ERR_BAD_ARG, "fame_jdsira: bad argument");
  cudaStream_t st = P.stream;
  const long long L = 4 * P.Nq;
  const size_t cb = sizeof(double2) * L;
  const int mmax = no_restart + nev + rpd + 2;
  cudaError_t e;
  double2* V = (double2*)workspace(P, JD_V, cb * mmax, &e);
  JD_CK(e, "jdsira workspace");
  double2* BV = (double2*)workspace(P, JD_BV, cb * mmax, &e);
  JD_CK(e, "jdsira workspace");
  double2* AV = (double2*)workspace(P, JD_AV, cb * mmax, &e);
  JD_CK(e, "jdsira workspace");
  double2* vecs = (double2*)workspace(P, JD_VEC, cb * 4, &e);
  JD_CK(e, "jdsira workspace");
  double2* U = vecs;          // Ritz vector
  double2* R = vecs + L;      // residual
  double2* T = vecs + 2 * L;  // correction
  double2* T2 = vecs + 3 * L;
  double2* TMP = (double2*)workspace(P, JD_TMP, cb * (nev + rpd + 2), &e);
  JD_CK(e, "jdsira workspace");
  double2* small = (double2*)workspace(P, JD_SMALL, sizeof(double2) * (size_t)mmax * mmax + 4096, &e);
  JD_CK(e, "jdsira workspace");
  const int nblk = 256;
  double2* part = (double2*)workspace(P, JD_PART, sizeof(double2) * nblk * mmax + 64, &e);
  JD_CK(e, "jdsira workspace");
  int* dinst = (int*)workspace(P, JD_INST, sizeof(int) * 8, &e);
  JD_CK(e, "jdsira workspace");
  JD_CK(h2d_async(P, dinst, &inst, sizeof(int)), "jdsira init");
  JD_CK(ensure_work(P, 1), "jdsira scratch");
  VecCtx c1;
  c1.inst = dinst;
  c1.nk = P.nk;
  auto applyB = [&](const double2* x, double2* y) {
    double2* w0 = (double2*)P.d_work;
    return launch_fncB<double>(P, x, y, 1, c1, w0, w0 + 6 * P.Nq, st);
  };
  // conj(V[:,0:m])^T w  -> host
  auto vdots = [&](const double2* Vb, int m, const double2* w, std::vector<cd>& out) -> int {
    JD_CK(dot_batched<double>(Vb, 0, L, m, w, 0, L, 1, small, part, nblk, nullptr, st), "jdsira dot");
    std::vector<double2> h(m);
    JD_CK(cudaMemcpyAsync(h.data(), small, sizeof(double2) * m, cudaMemcpyDeviceToHost, st), "jdsira dot");
    JD_CK(cudaStreamSynchronize(st), "jdsira dot");
    out.resize(m);
    for (int i = 0; i < m; ++i) out[i] = cd(h[i].x, h[i].y);
    return FAME_OK;
  };
  // out[:, 0:q] = X[:, 0:m] * C  (C host, m x q column-major)
  auto comb = [&](const double2* X, int m, const std::vector<cd>& C, int q, double2* out) -> int {
    std::vector<double2> hc((size_t)m * q);
    for (size_t i = 0; i < hc.size(); ++i) hc[i] = make_double2(C[i].real(), C[i].imag());
    JD_CK(h2d_async(P, small, hc.data(), sizeof(double2) * hc.size()), "jdsira comb");
    JD_CK(block_comb<double>(X, out, L, L, m, q, small, st), "jdsira comb");
    return FAME_OK;
  };
  auto norm2 = [&](const double2* x, double* out) -> int {
    std::vector<cd> d;
    int rc = vdots(x, 1, x, d);
    *out = std::sqrt(std::max(0.0, d[0].real()));
    return rc;
  };
  auto scale = [&](double2* x, double s) -> int {
    std::vector<cd> c(1, cd(s, 0.0));
    int rc = comb(x, 1, c, 1, T2);
    if (rc) return rc;
    JD_CK(cudaMemcpyAsync(x, T2, cb, cudaMemcpyDeviceToDevice, st), "jdsira scale");
    return FAME_OK;
  };

  // projected matrices (host, row-major mmax x mmax)
  std::vector<cd> Mh((size_t)mmax * mmax), Lh((size_t)mmax * mmax);
  auto add_column = [&](int j) -> int {  // BV[j], AV[j] from V[j]; fill column/row j of M and L
    JD_CK(applyB(V + (size_t)j * L, BV + (size_t)j * L), "jdsira fncB");
    JD_CK(launch_fncA<double>(P, V + (size_t)j * L, AV + (size_t)j * L, 1, c1, st), "jdsira fncA");
    std::vector<cd> mb, la;
    int rc = vdots(V, j + 1, BV + (size_t)j * L, mb);
    if (rc) return rc;
    rc = vdots(V, j + 1, AV + (size_t)j * L, la);
    if (rc) return rc;
    for (int i = 0; i <= j; ++i) {
      Mh[(size_t)i * mmax + j] = mb[i];
      Mh[(size_t)j * mmax + i] = std::conj(mb[i]);
      Lh[(size_t)i * mmax + j] = la[i];
      Lh[(size_t)j * mmax + i] = std::conj(la[i]);
    }
    Mh[(size_t)j * mmax + j] = cd(Mh[(size_t)j * mmax + j].real(), 0.0);
    Lh[(size_t)j * mmax + j] = cd(Lh[(size_t)j * mmax + j].real(), 0.0);
    return FAME_OK;
  };
  // initial vector: deterministic pseudo-random, unit norm (Driver4 is started
  // from a random unit vector in main_EIG_np_*.m)
  {
    std::vector<double2> h(L);
    unsigned long long s = 0x9E3779B97F4A7C15ull ^ (unsigned long long)(inst + 1);
    double nn = 0.0;
    for (long long i = 0; i < L; ++i) {
      s ^= s << 13;
      s ^= s >> 7;
      s ^= s << 17;
      const double a = double(s >> 11) * (1.0 / 9007199254740992.0);
      s ^= s << 13;
      s ^= s >> 7;
      s ^= s << 17;
      const double b = double(s >> 11) * (1.0 / 9007199254740992.0);
      h[i] = make_double2(a, b);
      nn += a * a + b * b;
    }
    const double inv = 1.0 / std::sqrt(nn);
    for (auto& v : h) {
      v.x *= inv;
      v.y *= inv;
    }
    JD_CK(cudaMemcpyAsync(V, h.data(), cb, cudaMemcpyHostToDevice, st), "jdsira init");
    JD_CK(cudaStreamSynchronize(st), "jdsira init");
  }
  int m = 1, nl = 0;
  long long outer = 0, inner_its = 0, b_applies = 0;
  int rc = add_column(0);
  if (rc) return rc;
  b_applies++;
  std::vector<double> locked_ew, locked_res;
  int no_near = 0;
  const long long max_outer = 6000;  // Locking4.m:82
  int status = FAME_OK;

  // restart / lock in coefficient space: Ysel (m x q) -> orthonormal Qc, V <- V Qc
  auto restart_to = [&](std::vector<cd> Ysel, int q) -> int {
    // MGS on the columns of Ysel (V is orthonormal: coefficient and vector inner products agree)
    std::vector<cd> Q;
    int qq = 0;
    for (int c2 = 0; c2 < q; ++c2) {
      std::vector<cd> y(Ysel.begin() + (size_t)c2 * m, Ysel.begin() + (size_t)(c2 + 1) * m);
      for (int pass = 0; pass < 2; ++pass)
        for (int k = 0; k < qq; ++k) {
          cd d = 0.0;
          for (int i = 0; i < m; ++i) d += std::conj(Q[(size_t)k * m + i]) * y[i];
          for (int i = 0; i < m; ++i) y[i] -= d * Q[(size_t)k * m + i];
        }
      double nn = 0.0;
      for (int i = 0; i < m; ++i) nn += std::norm(y[i]);
      nn = std::sqrt(nn);
      if (nn > 1e-6) {  // Gram_Schmidt.m:10 drops dependent columns
        for (auto& v : y) v /= nn;
        Q.insert(Q.end(), y.begin(), y.end());
        qq++;
      }
    }
    int rc2;
    if ((rc2 = comb(V, m, Q, qq, TMP))) return rc2;
    JD_CK(cudaMemcpyAsync(V, TMP, cb * qq, cudaMemcpyDeviceToDevice, st), "jdsira restart");
    if ((rc2 = comb(BV, m, Q, qq, TMP))) return rc2;
    JD_CK(cudaMemcpyAsync(BV, TMP, cb * qq, cudaMemcpyDeviceToDevice, st), "jdsira restart");
    if ((rc2 = comb(AV, m, Q, qq, TMP))) return rc2;
    JD_CK(cudaMemcpyAsync(AV, TMP, cb * qq, cudaMemcpyDeviceToDevice, st), "jdsira restart");
    std::vector<cd> Mn((size_t)mmax * mmax, 0.0), Ln((size_t)mmax * mmax, 0.0);
    for (int a = 0; a < qq; ++a)
      for (int b = 0; b < qq; ++b) {
        cd sm = 0.0, sl = 0.0;
        for (int i = 0; i < m; ++i) {
          cd ti = 0.0, tl = 0.0;
          for (int k = 0; k < m; ++k) {
            ti += Mh[(size_t)i * mmax + k] * Q[(size_t)b * m + k];
            tl += Lh[(size_t)i * mmax + k] * Q[(size_t)b * m + k];
          }
          sm += std::conj(Q[(size_t)a * m + i]) * ti;
          sl += std::conj(Q[(size_t)a * m + i]) * tl;
        }
        Mn[(size_t)a * mmax + b] = sm;
        Ln[(size_t)a * mmax + b] = sl;
      }
    Mh.swap(Mn);
    Lh.swap(Ln);
    m = qq;
    JD_CK(cudaStreamSynchronize(st), "jdsira restart");
    return FAME_OK;
  };

  while (nl < nev && outer < max_outer) {
    outer++;
    // projected Hermitian-definite pencil  L y = mu M y,  theta = 1/mu
    std::vector<cd> Mm((size_t)m * m), Lm((size_t)m * m);
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j) {
        Mm[(size_t)i * m + j] = Mh[(size_t)i * mmax + j];
        Lm[(size_t)i * m + j] = Lh[(size_t)i * mmax + j];
      }
    std::vector<double> mu;
    std::vector<cd> Y;
    if (!herm_pencil_eig(Lm, Mm, m, mu, Y)) {
      status = FAME_ERR_BREAKDOWN;
      fail(&P, status, "fame_jdsira: projected V^H B V not positive definite");
      break;
    }
    // exclude the nl Ritz vectors that live in the locked coordinates
    std::vector<double> wlock(m, 0.0);
    for (int c2 = 0; c2 < m; ++c2) {
      double in = 0.0, all = 0.0;
      for (int i = 0; i < m; ++i) {
        const double a2 = std::norm(Y[(size_t)c2 * m + i]);
        all += a2;
        if (i < nl) in += a2;
      }
      wlock[c2] = all > 0 ? in / all : 0.0;
    }
    std::vector<int> idx(m);
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return wlock[a] > wlock[b]; });
    std::vector<int> cand(idx.begin() + std::min(nl, m), idx.end());
    auto theta_of = [&](int c2) { return mu[c2] != 0.0 ? 1.0 / mu[c2] : 1e300; };
    if (!P.opt_sira_nearest) {
      // 'CL' of Choose_Ritz_Pair_Unsymm4.m:176-186,218-224: the Ritz values
      // above the target, closest first; all of them by distance only when
      // none lies above
      std::vector<int> above;
      for (int c2 : cand)
        if (theta_of(c2) > target) above.push_back(c2);
      if (!above.empty()) cand.swap(above);
    }
    std::stable_sort(cand.begin(), cand.end(), [&](int a, int b) {
      return std::fabs(theta_of(a) - target) < std::fabs(theta_of(b) - target);
    });
    if (cand.empty()) {
      status = FAME_ERR_BREAKDOWN;
      fail(&P, status, "fame_jdsira: no unlocked Ritz pair");
      break;
    }
    const int c0 = cand[0];
    const double theta = theta_of(c0);
    std::vector<cd> y(Y.begin() + (size_t)c0 * m, Y.begin() + (size_t)(c0 + 1) * m);
    double ny = 0.0;
    for (auto& v : y) ny += std::norm(v);
    ny = std::sqrt(ny);
    for (auto& v : y) v /= ny;  // unit Ritz vector u = V y (V orthonormal)
    // u, r = B u - theta A u
    if ((rc = comb(V, m, y, 1, U))) return rc;
    std::vector<cd> y2(2 * (size_t)m);
    {
      std::vector<cd> yb(y), ya(y);
      for (auto& v : ya) v *= -theta;
      if ((rc = comb(BV, m, yb, 1, R))) return rc;
      if ((rc = comb(AV, m, ya, 1, T))) return rc;
      std::vector<cd> one(1, cd(-1.0, 0.0));  // R -= (-1) * T  -> R + T
      std::vector<double2> h1(1, make_double2(-1.0, 0.0));
      JD_CK(h2d_async(P, small, h1.data(), sizeof(double2)), "jdsira res");
      JD_CK(sub_combo<double>(R, T, L, L, 1, small, st), "jdsira res");
    }
    double rsdl;
    if ((rc = norm2(R, &rsdl))) return rc;
    if (!std::isfinite(rsdl)) {
      status = FAME_ERR_NAN;
      fail(&P, status, "fame_jdsira: non-finite residual");
      break;
    }
    if (rsdl <= 10.0 * tol && rsdl > tol) no_near++;  // Locking4.m:198-202
    else no_near = 0;
    if (rsdl <= tol || no_near >= 5) {
      // lock (Locking4.m:425-450): store the Ritz vector, restart on [locked, u, next Ritz vectors]
      if (ev_out) JD_CK(cudaMemcpyAsync(ev_out + (size_t)nl * L, U, cb, cudaMemcpyDeviceToDevice, st), "jdsira lock");
      locked_ew.push_back(theta);
      locked_res.push_back(rsdl);
      std::vector<cd> Ysel;
      for (int i = 0; i < nl; ++i) {
        std::vector<cd> ei(m, 0.0);
        ei[i] = 1.0;
        Ysel.insert(Ysel.end(), ei.begin(), ei.end());
      }
      Ysel.insert(Ysel.end(), y.begin(), y.end());
      int q = nl + 1;
      for (size_t j = 1; j < cand.size() && (int)j < rpd; ++j, ++q)
        Ysel.insert(Ysel.end(), Y.begin() + (size_t)cand[j] * m, Y.begin() + (size_t)(cand[j] + 1) * m);
      nl++;
      no_near = 0;
      if ((rc = restart_to(Ysel, q))) return rc;
      continue;
    }
    if (m >= no_restart + nl) {
      // restart (Locking4.m:361-381): locked coordinates, current and next Ritz vectors
      std::vector<cd> Ysel;
      for (int i = 0; i < nl; ++i) {
        std::vector<cd> ei(m, 0.0);
        ei[i] = 1.0;
        Ysel.insert(Ysel.end(), ei.begin(), ei.end());
      }
      Ysel.insert(Ysel.end(), y.begin(), y.end());
      int q = nl + 1;
      for (size_t j = 1; j < cand.size() && (int)j < rpd; ++j, ++q)
        Ysel.insert(Ysel.end(), Y.begin() + (size_t)cand[j] * m, Y.begin() + (size_t)(cand[j] + 1) * m);
      if ((rc = restart_to(Ysel, q))) return rc;
    }
    // SIRA correction t = B^{-1} r (loose), SIRA_solve_residual_LS_GEP.m:54
    {
      int its = 0;
      double rr = 0.0;
      int prc;
      if (inner_prec == FAME_C64) {
        float2* r32 = (float2*)workspace(P, JD_R32, sizeof(float2) * L * 2, &e);
        JD_CK(e, "jdsira workspace");
        JD_CK((convert<float, double>(R, r32, L, st)), "jdsira inner");
        prc = shift == 0.0 ? pcg_batched<float>(P, r32, r32 + L, 1, dinst, inner_tol, inner_maxit, &its, &rr)
                           : minres_shifted<float>(P, r32, r32 + L, dinst, shift, inner_tol, inner_maxit, &its, &rr);
        JD_CK((convert<double, float>(r32 + L, T, L, st)), "jdsira inner");
      } else {
        prc = shift == 0.0 ? pcg_batched<double>(P, R, T, 1, dinst, inner_tol, inner_maxit, &its, &rr)
                           : minres_shifted<double>(P, R, T, dinst, shift, inner_tol, inner_maxit, &its, &rr);
      }
      if (prc == FAME_ERR_NAN || prc == FAME_ERR_BREAKDOWN) return prc;
      inner_its += std::abs(its);
      b_applies += std::abs(its);
    }
    // MGS against V twice and normalise (Locking4.m:326-330)
    for (int pass = 0; pass < 2; ++pass) {
      std::vector<cd> d;
      if ((rc = vdots(V, m, T, d))) return rc;
      std::vector<double2> hd(m);
      for (int i = 0; i < m; ++i) hd[i] = make_double2(d[i].real(), d[i].imag());
      JD_CK(h2d_async(P, small, hd.data(), sizeof(double2) * m), "jdsira mgs");
      JD_CK(sub_combo<double>(T, V, L, L, m, small, st), "jdsira mgs");
    }
    double nt;
    if ((rc = norm2(T, &nt))) return rc;
    if (!(nt > 1e-14)) {  // stagnation: restart from the Ritz vectors only
      no_near = 5;
      continue;
    }
    if ((rc = scale(T, 1.0 / nt))) return rc;
    JD_CK(cudaMemcpyAsync(V + (size_t)m * L, T, cb, cudaMemcpyDeviceToDevice, st), "jdsira expand");
    if ((rc = add_column(m))) return rc;
    b_applies++;
    m++;
  }
  if (nl < nev && status == FAME_OK) {
    status = FAME_ERR_NOT_CONVERGED;
    fail(&P, status, "fame_jdsira: not all eigenpairs converged");
  }
  for (int i = 0; i < nl && i < nev; ++i) {
    ew_out[i] = locked_ew[i];
    if (res_out) res_out[i] = locked_res[i];
  }
  for (int i = nl; i < nev; ++i) {
    ew_out[i] = NAN;
    if (res_out) res_out[i] = NAN;
  }
  if (stats) {
    stats[0] = outer;
    stats[1] = inner_its;
    stats[2] = b_applies;
    stats[3] = nl;
  }
  JD_CK(cudaStreamSynchronize(st), "jdsira out");
  return status;
}

}  // namespace fame

using namespace fame;

extern "C" int fame_jdsira(fame_plan_t h, int inner_prec, int inst, int nev, double target, double shift,
                           double tol, int no_restart, int restart_dim, double inner_tol, int inner_maxit, double* ew,
                           void* ev, double* res, long long* stats) {
  if (!h || !ew) return FAME_ERR_BAD_ARG;
  if (inner_prec != FAME_C128 && inner_prec != FAME_C64)
    return fail(&h->P, FAME_ERR_BAD_ARG, "fame_jdsira: bad precision");
  return jdsira_run(h->P, inst, inner_prec, nev, target, shift, tol, no_restart, restart_dim, inner_tol, inner_maxit,
                    ew, (double2*)ev, res, stats);
}
