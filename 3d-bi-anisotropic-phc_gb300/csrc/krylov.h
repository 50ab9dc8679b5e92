// Krylov glue launchers (krylov_kernels.cu) and host drivers (solvers.cu).
#pragma once

#include "fame_internal.h"

namespace fame {

// out[v*ma + m] = sum_i conj(a[v][m][i]) * b[v][i]  (FP64 accumulation)
template <class R>
cudaError_t dot_batched(const cx<R>* a, long long a_vstride, long long a_cstride, int ma, const cx<R>* b,
                        long long b_vstride, long long len, int nvec, double2* out, double2* partial, int nblk,
                        const int* active, cudaStream_t st);
template <class R>
cudaError_t axpby_batched(const cx<R>* x, cx<R>* y, long long len, long long stride, int nvec,
                          const double2* alpha, const double2* beta, const int* active, cudaStream_t st);
template <class R>
cudaError_t cg_xr(cx<R>* x, cx<R>* r, const cx<R>* p, const cx<R>* q, long long len, long long stride, int nvec,
                  const double* alpha, const int* active, cudaStream_t st);
// out[row] = sum of partial[row][0..nblk)
cudaError_t dot_final(const double2* partial, int nblk, int nrows, double2* out, cudaStream_t st);
// x += alpha p ; r -= alpha q ; out[v] = (|r_v|^2, |r_v|^2) (fused)
template <class R>
cudaError_t cg_xr_dot(cx<R>* x, cx<R>* r, const cx<R>* p, const cx<R>* q, long long len, long long stride, int nvec,
                      const double* alpha, const int* active, double2* out, double2* partial, int nblk,
                      cudaStream_t st);
template <class R>
cudaError_t cg_p(cx<R>* p, const cx<R>* r, long long len, long long stride, int nvec, const double* beta,
                 const int* active, cudaStream_t st);
cudaError_t cg_scalars(int stage, int nvec, const double2* dot, double* rho, double* alpha, double* beta,
                       const double* tol2b2, int* active, int* iters, double* res2, cudaStream_t st);
// cg_scalars on the sums of nblk partials per vector (partial[v * nblk + i]),
// the sums also stored in dot[v]; one launch.
// Condition kernel of a graph-resident loop (graph_replay_while): *passes
// += 1, and the loop goes on while any active[v] and *passes < max_passes.
cudaError_t while_active(const int* active, int nvec, int* passes, int max_passes, cudaGraphConditionalHandle h,
                         cudaStream_t st);
cudaError_t cg_scalars_red(int stage, int nvec, const double2* partial, int nblk, double2* dot, double* rho,
                           double* alpha, double* beta, const double* tol2b2, int* active, int* iters, double* res2,
                           cudaStream_t st);
// Gram-Schmidt over a batch of instances, one launch each for all of them:
// vector v of r (stride rs) works against columns span[v].x ..
// span[v].x + span[v].y - 1 of its block X + v*xs (columns len apart);
// span[v].y = 0 skips it; span[v].y <= maxm <= 128.
// coef[v*cstride + i] = X_v[col0_v + i]^H r_v (FP64); partial: nv*maxm*nblk.
cudaError_t gs_dots(const double2* X, long long xs, const double2* r, long long rs, long long len, int nv,
                    const int2* span, int maxm, double2* coef, int cstride, double2* partial, int nblk,
                    cudaStream_t st);
// Q_v[:, col[v]] = V_v and BQ_v[:, col[v]] = BV_v (+ complex64 copies when Q32
// is given) for every v with col[v] >= 0; blocks xs apart, vectors len apart.
cudaError_t gs_store(double2* Q, double2* BQ, float2* Q32, float2* BQ32, long long xs, const double2* V,
                     const double2* BV, long long len, int nv, const int* col, cudaStream_t st);
// r_v -= sum_i coef[v*cstride + i] X_v[col0_v + i], FP64 or from complex64 copies
cudaError_t gs_combo(double2* r, long long rs, const double2* X, long long xs, long long len, int nv,
                     const int2* span, const double2* coef, int cstride, cudaStream_t st);
cudaError_t gs_combo_lo(double2* r, long long rs, const float2* X, long long xs, long long len, int nv,
                        const int2* span, const double2* coef, int cstride, cudaStream_t st);
// partial[v * nblk + i] = block i's share of a_v^H b_v (no final reduction)
template <class R>
cudaError_t dot_partial(const cx<R>* a, const cx<R>* b, long long len, long long stride, int nvec, double2* partial,
                        int nblk, const int* active, cudaStream_t st);
// x += alpha p ; r -= alpha q ; partial (|r|^2, |r|^2) per block (no final reduction)
template <class R>
cudaError_t cg_xr_partial(cx<R>* x, cx<R>* r, const cx<R>* p, const cx<R>* q, long long len, long long stride,
                          int nvec, const double* alpha, const int* active, double2* partial, int nblk,
                          cudaStream_t st);
template <class R>
cudaError_t block_rot(const cx<R>* in, cx<R>* out, long long len, long long ld, int p, int k, const double* U,
                      cudaStream_t st);
// out = a x + b y + c w with real scalars (y, w may be null; out may alias x)
template <class R>
cudaError_t lincomb3(cx<R>* out, double a, const cx<R>* x, double b, const cx<R>* y, double c, const cx<R>* w,
                     long long len, cudaStream_t st);
// MINRES on the Hermitian (indefinite) operator B - shift A for one vector
// of instance `inst` (d_inst: device int[1]); tol relative to ||b||.
template <class R>
int minres_shifted(Plan& P, const cx<R>* b, cx<R>* x, const int* d_inst, double shift, double tol, int maxit,
                   int* iters, double* relres);
// out[:, j] = sum_i in[:, i] * C[i, j], C complex m x q column-major (<= 12800 entries)
template <class R>
cudaError_t block_comb(const cx<R>* in, cx<R>* out, long long len, long long ld, int m, int q, const double2* C,
                       cudaStream_t st);
template <class R>
cudaError_t sub_combo(cx<R>* r, const cx<R>* X, long long len, long long ld, int m, const double2* c,
                      cudaStream_t st);
template <class D, class S>
cudaError_t convert(const cx<S>* in, cx<D>* out, long long n, cudaStream_t st);
// x += mult_v * d (mult null: 1)
cudaError_t refine_acc(double2* x, const float2* d, long long len, int nvec, const int* active, cudaStream_t st,
                       const double* mult = nullptr);
// res = b - bx; res32 (may be null) its complex64 copy
cudaError_t residual(const double2* b, const double2* bx, double2* res, float2* res32, long long len, int nvec,
                     const int* active, cudaStream_t st);
// out = s_v * in, rounded to complex64
cudaError_t to32_scaled(const double2* in, float2* out, long long len, int nvec, const double* s, const int* active,
                        cudaStream_t st);
template <class R>
cudaError_t scale_batched(const cx<R>* x, cx<R>* y, long long len, int nvec, const double* s, const int* active,
                          cudaStream_t st);

// Host drivers (solvers.cu).
// Batched CG on B (fncinvB).  h_mask (host, may be null) selects the vectors
// to solve; others are left untouched.  iters_out / relres_out (host, may be
// null) receive per-vector results; a negative iteration count marks a
// breakdown or a non-finite residual.
template <class R>
int pcg_batched(Plan& P, const cx<R>* b, cx<R>* x, int nvec, const int* d_inst, double tol, int maxit,
                int* iters_out, double* relres_out, const unsigned char* h_mask = nullptr,
                const double* tol_per_vec = nullptr);

// Mixed-precision B^{-1}: complex64 CG corrections inside FP64 residual
// refinement until ||b - B x|| <= tol ||b|| (FP64).  Bx receives B*x (FP64).
// cg_vec / b64_vec (host, may be null): per-vector complex64 CG iterations and
// FP64 B applies, added to.
int solve_B_mixed(Plan& P, const double2* b, double2* x, double2* Bx, int nvec, const int* d_inst, double tol,
                  int max_rounds, double inner_tol32, int maxit32, const unsigned char* h_mask,
                  long long* cg_iters, long long* b64_applies, const double* tol_per_vec = nullptr,
                  long long* cg_vec = nullptr, long long* b64_vec = nullptr);

}  // namespace fame
