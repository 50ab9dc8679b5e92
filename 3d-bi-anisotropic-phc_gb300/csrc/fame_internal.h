// Internal plan object and kernel launchers of the FAME GB300 library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/fame.h"
#include "fame_types.cuh"

namespace fame {

// Kernels this library has run (all plans, all threads), and the launch
// calls it made from the host for them (a graph launch counts once however
// many kernels it runs).
extern unsigned long long g_kernel_launches;
extern unsigned long long g_host_launches;
// n kernels launched directly
#define FAME_LAUNCHED(n)                                                                              \
  (__atomic_fetch_add(&::fame::g_kernel_launches, (unsigned long long)(n), __ATOMIC_RELAXED),       \
   __atomic_fetch_add(&::fame::g_host_launches, (unsigned long long)(n), __ATOMIC_RELAXED))
// one graph launch running `nodes` kernels
#define FAME_GRAPH_LAUNCHED(nodes)                                                                    \
  (__atomic_fetch_add(&::fame::g_kernel_launches, (unsigned long long)(nodes), __ATOMIC_RELAXED),   \
   __atomic_fetch_add(&::fame::g_host_launches, 1ull, __ATOMIC_RELAXED))
// kernels run by the loop body of a graph launch, counted once the loop ended
#define FAME_KERNELS_RAN(n) __atomic_fetch_add(&::fame::g_kernel_launches, (unsigned long long)(n), __ATOMIC_RELAXED)
// launches recorded by a stream capture (counted by FAME_LAUNCHED, not run)
#define FAME_UNCOUNT_CAPTURED(n)                                                                      \
  (__atomic_fetch_sub(&::fame::g_kernel_launches, (unsigned long long)(n), __ATOMIC_RELAXED),       \
   __atomic_fetch_sub(&::fame::g_host_launches, (unsigned long long)(n), __ATOMIC_RELAXED))

// Which vectors of a batch belong to which k-point instance, and which are
// still active (converged vectors of a batched solve are skipped).
struct VecCtx {
  const int* inst = nullptr;    // device [nvec] instance index, or null: (v + vofs) % nk
  const int* active = nullptr;  // device [nvec] 0/1, or null: all active
  int nk = 1;
  int vofs = 0;                 // index of vector 0 in the caller's batch (sub-batches)
};

FAME_HD int vec_inst(const VecCtx& c, int v) { return c.inst ? c.inst[v] : ((v + c.vofs) % c.nk); }

// The same context for the sub-batch of vectors [v0, ...).
inline VecCtx sub_ctx(const VecCtx& c, int v0) {
  VecCtx s = c;
  if (s.inst) s.inst += v0;
  if (s.active) s.active += v0;
  s.vofs += v0;
  return s;
}

// Threads per pencil of the split-pencil plane kernels of fncB for size n
// (0: none compiled, one thread per pencil).
FAME_HD constexpr int plane_split(int n) {
  return n == 60 ? 3 : n == 48 ? 3 : n == 40 ? 5 : n == 36 ? 4 : n == 30 ? 3 : n == 24 ? 3 : n == 20 ? 4
       : n == 12 ? 3 : 0;
}

// Lane counts compiled for size n (i = 0 the default, 0 past the last): the
// autotuner's choices of the split.  n = 60 also has 60 = 4 * 15 and 5 * 12
// (720 / 900 threads per CTA, 15 / 12 values per thread).
FAME_HD constexpr int plane_lanes_alt(int n, int i) {
  return i == 0 ? plane_split(n) : n == 60 ? (i == 1 ? 4 : i == 2 ? 5 : 0) : 0;
}
constexpr int kPlaneLanesMax = 3;

// Launch parameters of the fncB sequence picked by fame_autotune for one
// (precision, batch width): vectors per launch sequence and the material
// stencil's form (single pass, or threads per block of the two-kernel form).
struct TuneEntry {
  int prec = 0, nvec = 0;
  int chunk = 0;         // 0: whole batch
  int stencil_tpb = 0;   // 0: single-pass k_sweep; 128/256/512: two-kernel form
  int lanes = -1;        // threads per pencil of the plane kernels: -1 the size's default, 0 one
  double us = 0.0;       // measured time of one fncB on the batch
};

// Device-side data of one precision.
template <class R> struct PlanData {
  cx<R>* lam = nullptr;  // [nk][3n]  lambda_x | lambda_y | lambda_z  (QP symbols, delta = 1/n)
  cx<R>* tau = nullptr;  // [nk][3]   exp(i*theta_d/n): Bloch phase of one periodic shift
  cx<R>* sxyz = nullptr; // [nk][3n]  S_sDFT per axis (the MtxVecMul_FFT phase)
  cx<R>* mat = nullptr;  // [nk][nphase][27]: Herm(N) | Herm(M) | J, row-major 3x3 each
  cx<R>* pc = nullptr;   // [nk][8][Nq] CG preconditioner: inverse 4x4 Hermitian blocks, diagonal packed (lazy)
  cx<R>* pi = nullptr;   // [nk][Nq][6] Pi1 | Pi2 per frequency voxel (SVD_Matrix_curl.m:45-57); complex128 plans data only
  // Field mode (per-vertex isotropic chiral medium eps(r) I, mu = I,
  // xi = -zeta = i gamma(r) I): vertex tensors N = a G, M = b G, J = -i g G with
  // a = 1/(eps - gamma^2), b = eps a, g = gamma a and G = A^T A the lattice
  // Gram matrix.  fld = [3][Nq] a | b | g, or null in phase-table mode.
  R* fld = nullptr;
  R gram[9] = {};
};

// Instantiated CUDA graphs of a plan, keyed by everything a captured launch
// sequence depends on (precision, sizes, device pointers).
struct GraphEntry {
  std::vector<uintptr_t> key;
  cudaGraphExec_t exec = nullptr;
  unsigned long long nodes = 0;  // kernel nodes (launch accounting)
};

struct Plan {
  int n = 0;         // cubic grid n1 = n2 = n3 = n
  long long Nq = 0;  // n^3
  int nk = 0;        // k-point instances
  int nphase = 0;
  int device = 0;
  cudaStream_t stream = nullptr;
  // options (fame_set_option)
  int opt_precond = 1;                // CG on B preconditioned by the averaged-medium B0^{-1}
  double opt_tol32 = 1e-6;            // complex64 CG tolerance of the first refinement round
  int opt_ds_residual = 1;            // mixed B^{-1}: residuals through the double-single fncB
  double opt_relax = 0.9;             // mixed Lanczos: relax the inner tolerance once Ritz residuals < this
  double opt_relax_max = 1e6;         // largest relaxation factor
  int opt_c64_round = 1;              // mixed B^{-1}: second round's B x update in complex64 (0: exact apply)
  int opt_graph = 2;                  // CG from CUDA graphs: 1 blocks of iterations, 2 the whole loop
  double opt_itol_floor = 1e-13;      // mixed form: floor of the spread-scaled inner tolerance
  int opt_plane_split = 1;            // fncB plane kernels with several threads per pencil where compiled
  int opt_pi_table = 1;               // complex128 fncB reads Pi from the plan's table (else evaluates it)
  int opt_sira_nearest = 0;           // SIRA Ritz choice: 0 'CL' (above the target), 1 nearest either side
  int opt_refine = 1;                 // mixed form: FP64 refinement sweep of the Ritz pairs
  double opt_refine_tol = 1e-6;       // relative tolerance of its correction solve B^{-1} R
  std::vector<double> refine_res_before;  // NFSEP residuals before the last refinement sweep
  std::vector<double> theta;          // [nk][3]
  std::vector<double> sigma_min;      // [nk] smallest curl singular value sqrt(min |L|^2)
  std::vector<double> mat_avg;        // [nk][27][2] volume-averaged Herm(N) | Herm(M) | J
  double2* d_mat_avg = nullptr;       // device copy
  std::vector<double> mat_host;       // [nk][nphase][27][2] covariant N | M | J blocks
  uint8_t* d_phase = nullptr;         // [Nq] phase id per vertex
  bool field_mode = false;            // per-vertex (eps, gamma) instead of phase ids
  double lattice[9] = {};             // field mode: primitive vectors as columns (row-major)
  std::vector<double> eps_host, gam_host;  // field mode: [Nq] each
  double* d_eps_gam = nullptr;        // field mode: [2][Nq] eps | gamma (FP64, gradient)
  PlanData<double> d64;
  PlanData<float> d32;
  PlanData<ff> dds;  // double-single copies of the d64 tables (grids with ds_supported)
  // scratch: two 6-field work buffers per vector, sized for complex128
  void* d_work = nullptr;
  size_t work_vecs = 0;
  // small device buffers
  int* d_inst = nullptr;
  size_t inst_cap = 0;
  double* d_red = nullptr;            // reduction scratch
  size_t red_cap = 0;
  // host staging for FAME_HOST_PTR calls
  void* d_stage = nullptr;
  size_t stage_bytes = 0;
  std::string last_error;
  // named grow-only device workspaces of the solvers
  std::vector<void*> ws_ptr;
  std::vector<size_t> ws_size;
  // pinned ring for small host->device uploads (a copy from pageable memory
  // would synchronise the stream)
  char* h_ring = nullptr;
  size_t ring_pos = 0;
  // captured launch sequences (graph.cu)
  cudaStream_t cap_stream = nullptr;
  std::vector<GraphEntry> graphs;
  // autotuned fncB launch parameters (autotune.cu)
  std::vector<TuneEntry> tune;
};

// Tuned launch parameters for (prec, nvec), or the defaults.
TuneEntry tune_for(const Plan& P, int prec, int nvec);
// The tuning key of an arithmetic type (FAME_C64, FAME_C128, FAME_C128_DS).
template <class R> constexpr int tune_prec() {
  return std::is_same<R, float>::value ? FAME_C64 : std::is_same<R, double>::value ? FAME_C128 : FAME_C128_DS;
}

// Replay the launch sequence that `issue(stream)` enqueues, from a graph cached
// under `key` (captured on first use on a private stream), on the plan's
// stream.  Returns cudaErrorNotSupported when capture is not possible, in
// which case the caller issues the sequence directly.
template <class F>
cudaError_t graph_replay(Plan& P, const std::vector<uintptr_t>& key, F&& issue);
void free_graphs(Plan& P);

// Asynchronous small upload through the plan's pinned ring (stream-ordered).
cudaError_t h2d_async(Plan& P, void* dst, const void* src, size_t bytes);

// Workspace slot `id` of at least `bytes` bytes (contents not preserved on growth).
void* workspace(Plan& P, int id, size_t bytes, cudaError_t* err);
void free_workspaces(Plan& P);
cudaError_t ensure_work(Plan& P, size_t vecs);
int fail(Plan* P, int code, const std::string& msg);
int cuda_fail(Plan* P, cudaError_t e, const char* where);

// Pi1 | Pi2 of every frequency voxel of every instance into d.pi (allocated
// here; called once at plan creation, after the lambda tables are on the device).
template <class R> cudaError_t build_pi_table(Plan& P);

// ---- kernel launchers (fncb_kernels.cu) ----
// pq (may be null): partial sums of Re(x^H B x), fncB_pq_partials(P, nvec)
// per vector, written when that count is non-zero.  pupd_z (may be null): x
// is a CG direction that is first updated in place, x = pupd_z + pupd_beta[v] x.
template <class R>
cudaError_t launch_fncB(const Plan& P, const cx<R>* x, cx<R>* y, int nvec, const VecCtx& ctx,
                        cx<R>* w0, cx<R>* w1, cudaStream_t st, double2* pq = nullptr,
                        const cx<R>* pupd_z = nullptr, const double* pupd_beta = nullptr);
template <class R> int fncB_pq_partials(const Plan& P, int nvec);
// Grid sizes with a compiled double-single fncB (FAME_FOR_EACH_DS_N).
bool ds_supported(int n);
// y = B x for complex128 vectors, evaluated in double-single arithmetic
// (x and y may alias; scratch: the plan's work arrays for nvec vectors).
cudaError_t launch_fncB_ds(const Plan& P, const double2* x, double2* y, int nvec, const VecCtx& ctx,
                           cudaStream_t st);
// The plan's double-single tables, converted from its complex128 ones.
int upload_tables_ds(Plan& P);
template <class R>
cudaError_t launch_fncA(const Plan& P, const cx<R>* x, cx<R>* y, int nvec, const VecCtx& ctx,
                        cudaStream_t st);
// First half of fncB: w = [u; v] = periodic-frame inverse DFT of [Pi.Pr x1; Pi.Qr x2]
// (6-field vectors, stride 6*Nq).
template <class R>
cudaError_t launch_fields_inv(const Plan& P, const cx<R>* x, cx<R>* w, int nvec, const VecCtx& ctx,
                              cudaStream_t st);
// MtxVecMul_FFT on 3Nq vectors: trans = 0 'notranspose' (S .* ifftn*sqrt(N)),
// 1 'transpose' (fftn(conj(S).*x)/sqrt(N)).
template <class R>
cudaError_t launch_transform(const Plan& P, int trans, const cx<R>* x, cx<R>* y, int nvec,
                             const VecCtx& ctx, cudaStream_t st);
// Composed handles: which = 0 Pr, 1 Qr (2Nq -> 3Nq), 2 Prs, 3 Qrs (3Nq -> 2Nq)
template <class R>
cudaError_t launch_handle(const Plan& P, int which, const cx<R>* x, cx<R>* y, int nvec,
                          const VecCtx& ctx, cx<R>* w0, cudaStream_t st);
// Material stencil in place on periodic-frame 6-field vectors w (stride 6*Nq),
// scratch h of the same size: w <- [M J^H; J N] w.
template <class R>
cudaError_t launch_stencil(const Plan& P, cx<R>* w, cx<R>* h, int nvec, const VecCtx& ctx, cudaStream_t st);
// Material operator alone on spatial 6-field vectors (periodic frame, no S):
// [u'; v'] = [M J^H; J N] [u; v], the middle factor of fncB.
template <class R>
cudaError_t launch_material(const Plan& P, const cx<R>* uv, cx<R>* out, int nvec,
                            const VecCtx& ctx, cx<R>* w1, cudaStream_t st);

// CG preconditioner M = B0^{-1}: B0 is fncB of the homogeneous medium with the
// volume-averaged vertex tensors, block diagonal in the frequency basis
// (one 4x4 Hermitian block per voxel).  Built once per plan and precision.
template <class R> cudaError_t build_precond(Plan& P, cudaStream_t st);
// z = M r per vector; partial sums (Re r'z, |r|^2) per block into partial.
template <class R>
cudaError_t precond_apply(const Plan& P, const cx<R>* r, cx<R>* z, int nvec, const VecCtx& ctx, double2* partial,
                          int nblk, cudaStream_t st);
// The CG step length computed inside the update instead of by a separate
// scalar kernel: every CTA of vector v reduces v's `nblk` partial sums of
// p^H q in one fixed order, so all of them use the same alpha = rho / p^H q;
// CTA 0 records alpha and the dot, and on breakdown (p^H q <= 0 or not
// finite) clears active[v] and negates the iteration count (alpha 0).
struct CgAlpha {
  const double2* pq = nullptr;  // [nvec][nblk] partial sums, or null: alpha given
  int nblk = 0;
  const double* rho = nullptr;
  double* alpha = nullptr;
  double2* dot = nullptr;
  int* active = nullptr;
  int* iters = nullptr;
};
// x += a p ; r -= a q ; z = M r ; partial (Re r'z, |r|^2)
template <class R>
cudaError_t pcg_update(const Plan& P, cx<R>* x, cx<R>* r, cx<R>* z, const cx<R>* p, const cx<R>* q, int nvec,
                       const VecCtx& ctx, const double* alpha, double2* partial, int nblk, cudaStream_t st,
                       const CgAlpha& ca = CgAlpha());

bool n_supported(int n);

}  // namespace fame

// The opaque handle of the C ABI.
struct fame_plan_s {
  fame::Plan P;
};
