/*
 * FAME GB300: C ABI of the nullspace-free FFT eigensolver hot path for the
 * 3D bi-anisotropic Maxwell generalised eigenproblem on quasi-periodic grids.
 *
 * Every entry point replaces one MATLAB handle or function of the reference
 * (FAME-GPU/3D-Bi-Anisotropic-PhC); the replaced interface is cited beside
 * each declaration.  Conventions:
 *   - vectors are interleaved complex (double2 for FAME_C128, float2 for
 *     FAME_C64) in the reference's MATLAB order: x-fastest grids, blocks
 *     stacked as in the reference ([x1; x2] halves, components 1,2,3);
 *   - a plan holds `nk` k-point instances of one cubic n^3 grid; a call
 *     processes `nvec` vectors, vector v belonging to instance inst[v]
 *     (inst == NULL: instance v % nk);
 *   - pointers are device pointers unless `flags` has FAME_HOST_PTR, in which
 *     case the library stages them through device memory;
 *   - calls are ordered on the plan's CUDA stream (fame_set_stream); a plan is
 *     not thread-safe, distinct plans are;
 *   - every call returns a fame_status; fame_last_error() describes failures.
 */
#ifndef FAME_GB300_H
#define FAME_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fame_plan_s* fame_plan_t;

enum fame_status {
  FAME_OK = 0,
  FAME_ERR_BAD_ARG = 1,
  FAME_ERR_CUDA = 2,
  FAME_ERR_NOT_CONVERGED = 3,
  FAME_ERR_BREAKDOWN = 4,
  FAME_ERR_NAN = 5,
  FAME_ERR_UNSUPPORTED = 6,
  FAME_ERR_SINGULAR = 7,
  FAME_ERR_ALLOC = 8
};

/* FAME_C128_DS: complex128 vectors, the operator evaluated in double-single
 * (float-float) arithmetic, ~1e-14 relative (fame_apply_B only; grids with a
 * compiled double-single fncB, else FAME_ERR_UNSUPPORTED). */
enum fame_precision { FAME_C128 = 0, FAME_C64 = 1, FAME_C128_DS = 2 };

enum fame_handle { FAME_PR = 0, FAME_QR = 1, FAME_PRS = 2, FAME_QRS = 3 };

#define FAME_HOST_PTR 1

/* Library version string. */
const char* fame_version(void);

/* Kernels run by this library since it was loaded (all plans), and the
 * launch calls it made from the host for them (a kernel launched directly
 * counts once in both; a CUDA graph launch counts once here and its kernels
 * in fame_kernel_launches).  Diagnostics for benchmarks, no reference
 * counterpart. */
long long fame_kernel_launches(void);
long long fame_host_launches(void);

/*
 * Create a plan for `nk` k-points of one n^3 grid.
 *   theta   [nk*3]   Bloch angles theta_d = k . a_d per instance
 *                    (band_structure_woodpile_Lanczos_n60_gamma0p2.m:54-56).
 *   phase   [n^3]    phase id of every vertex, x fastest (host)
 *                    (the inside index set of Material_Matrix_Generate_Mult_Point.m:15).
 *   tensors [nk*nphase*27*2]  per instance and phase, the covariant N, M, J
 *                    blocks (3x3 row-major each, interleaved complex), i.e. the
 *                    A'*X*A blocks of the inverted 6x6 constitutive matrix that
 *                    DistMaterialMatrix places (Material_Matrix_Generate_Mult_Point.m:28-31,38-48).
 * Replaces the per-k setup SVD_Matrix_Generate.m:24-30,
 * Interpolation_Material_Matrix_Mult_Point_vertex.m:1-28 and
 * Funhand_Generate_Lanzcos.m:1-82 (handles closed over mtx_A / mtx_B).
 */
int fame_plan_create(fame_plan_t* plan, int n, int nk, const double* theta, const uint8_t* phase, int nphase,
                     const double* tensors);
int fame_plan_destroy(fame_plan_t plan);
/* Use `stream` (a cudaStream_t) for all later calls on this plan. */
int fame_set_stream(fame_plan_t plan, void* stream);

/* Solver options (no reference counterpart; defaults in brackets):
 *   FAME_OPT_PRECOND  CG on B preconditioned by the averaged-medium block
 *                     inverse B0^{-1} [1]; 0 gives the reference's
 *                     unpreconditioned pcg of fncinvB.m.
 *   FAME_OPT_TOL32    complex64 CG tolerance of the first refinement round of
 *                     the mixed-precision B^{-1} [1e-6].
 *   FAME_OPT_GRAPH    CG iterations from CUDA graphs captured on first use:
 *                     2 the whole iteration loop in one graph launch (blocks
 *                     of four iterations in a conditional WHILE node whose
 *                     condition, any vector still active, is set on the
 *                     device; the host waits once per solve) [2]; 1 one graph
 *                     launch per block of four iterations with a host-side
 *                     convergence check after each; 0 every kernel launched
 *                     directly.  All three give the same iterates.
 *   FAME_OPT_ITOL_FLOOR  mixed form: lower bound of the per-instance inner
 *                     tolerance, which is tightened by the spread of the
 *                     wanted Ritz values and starts there at near-zero wave
 *                     vectors [1e-13].
 *   FAME_OPT_PLANE_SPLIT  fncB plane kernels with several threads per FFT
 *                     pencil on the grid sizes that have them [1]; 0 keeps
 *                     one thread per pencil (same results to rounding).
 *   FAME_OPT_SIRA_NEAREST  fame_jdsira's Ritz choice: 0 the reference's 'CL'
 *                     (real Ritz values above the target, closest first;
 *                     Choose_Ritz_Pair_Unsymm4.m:176-186) [0]; 1 the closest
 *                     on either side of the target.
 *   FAME_OPT_REFINE   mixed form (FAME_C64) of fame_lanczos / fame_band_solve:
 *                     one FP64 refinement sweep of the converged Ritz pairs
 *                     [1]: W = B^-1 (A X - B X Lambda) by the mixed inner
 *                     solve, then FP64 Rayleigh-Ritz on [X W] per k-point; the
 *                     returned eigenvalues, vectors and residuals are the
 *                     refined ones where the sweep lowered the residual (the
 *                     residuals before: fame_refine_residuals).
 *   FAME_OPT_REFINE_TOL  relative tolerance of that correction solve [1e-6].
 *   FAME_OPT_PI_TABLE  complex128 fncB reads the per-voxel Pi blocks from the
 *                     table the plan builds at creation (96 B per voxel and
 *                     k-point) [1]; 0 evaluates them in the transform kernels
 *                     (same values to rounding).  Complex64 always evaluates.
 *   FAME_OPT_C64_ROUND  mixed B^{-1}: the second refinement round updates
 *                     B x with a complex64 apply of its correction [1]
 *                     (estimates the residual to ~1e-11 of b); 0 takes the
 *                     exact apply (double-single or FP64, see
 *                     FAME_OPT_DS_RESIDUAL) in every round.
 *   FAME_OPT_RELAX    mixed Lanczos: c in [0, 1) [0.9; 0 = off].  At a
 *                     restart where every wanted Ritz pair's relative
 *                     residual r is below c, the instance's inner tolerance is
 *                     multiplied by min(FAME_OPT_RELAX_MAX, c / max r) (relaxed inner
 *                     accuracy for the late Lanczos vectors, which enter the
 *                     wanted pairs with a weight of about r).  The
 *                     Gamma-like instances at the tolerance floor are not
 *                     relaxed.
 *   FAME_OPT_DS_RESIDUAL  mixed B^{-1}: the refinement rounds' residuals
 *                     b - B x take fncB in double-single arithmetic instead
 *                     of FP64 where the grid has it compiled [1] (FP32 pipes
 *                     instead of GB300's FP64 pipe; ~1e-14 relative).  The
 *                     reported NFSEP residuals and the refinement sweep keep
 *                     FP64.
 *   FAME_OPT_RELAX_MAX  the largest factor of that relaxation [1e6].  The error
 *                     such a solve adds to a wanted pair is bounded by about
 *                     (inner tolerance) x c whatever the factor. */
enum fame_option {
  FAME_OPT_PRECOND = 0, FAME_OPT_TOL32 = 1, FAME_OPT_GRAPH = 2, FAME_OPT_ITOL_FLOOR = 3, FAME_OPT_PLANE_SPLIT = 4,
  FAME_OPT_SIRA_NEAREST = 5, FAME_OPT_REFINE = 6, FAME_OPT_REFINE_TOL = 7, FAME_OPT_PI_TABLE = 8,
  FAME_OPT_C64_ROUND = 9, FAME_OPT_RELAX = 10, FAME_OPT_RELAX_MAX = 11, FAME_OPT_DS_RESIDUAL = 12
};
int fame_set_option(fame_plan_t plan, int option, double value);

/* NFSEP residuals ||B x - omega A x|| of the Ritz pairs before the FP64
 * refinement sweep of the last mixed-form fame_lanczos / fame_band_solve on
 * this plan ([nk][k] for a band solve); copies at most `n` of them to
 * `before` and returns their count (0 when no sweep ran).  No reference
 * counterpart. */
int fame_refine_residuals(fame_plan_t plan, double* before, int n);

/*
 * Autotuner (no reference counterpart): time the launch parameters of the
 * fncB sequence for precision `prec` and batch width `nvec` on this plan
 * (vectors per launch sequence: the whole batch, 1/2, 1/4, 1/8 of it or any
 * width up to 16; the material stencil: 0 = single pass, or 128, 256, 512
 * threads per block of the two-kernel form; the plane kernels' split of each
 * FFT pencil: threads per pencil, every count compiled for the grid size, or
 * one) and keep the fastest for later calls with that width.  Outputs (may be
 * NULL): the chosen chunk (0 = whole batch), stencil setting and the measured
 * microseconds of one fncB.  fame_set_tune installs a chunk and stencil
 * setting directly (e.g. from a cache), keeping the width's split;
 * fame_set_tune_lanes installs the split (-1 = the size's default, 0 = one
 * thread per pencil, else a compiled count; others fall back to the
 * default); fame_get_tune reads the installed setting (lanes -1 = default).
 */
int fame_autotune(fame_plan_t plan, int prec, int nvec, int* chunk, int* stencil_tpb, double* us);
int fame_set_tune(fame_plan_t plan, int prec, int nvec, int chunk, int stencil_tpb);
int fame_set_tune_lanes(fame_plan_t plan, int prec, int nvec, int lanes);
int fame_get_tune(fame_plan_t plan, int prec, int nvec, int* chunk, int* stencil_tpb, int* lanes);
int fame_sync(fame_plan_t plan);
const char* fame_last_error(fame_plan_t plan);
int fame_plan_info(fame_plan_t plan, int* n, int* nk, long long* nq);

/* y = A x on 4*Nq vectors.  Replaces fun_Lanczos/fncA.m:1-5. */
int fame_apply_A(fame_plan_t plan, int prec, const void* x, void* y, int nvec, const int* inst, int flags);

/* y = B x on 4*Nq vectors.  Replaces fun_Lanczos/fncB.m:1-7 and
 * fun_no_inv/fncB_Generate_no_inv.m:1-9. */
int fame_apply_B(fame_plan_t plan, int prec, const void* x, void* y, int nvec, const int* inst, int flags);

/* y = B x like fame_apply_B, for callers that cannot let a library allocate
 * device memory at call time (a MEX gateway under MATLAB's gpuArray memory
 * manager, an application pooling its whole device budget).  It allocates
 * nothing: its scratch is one fixed 16 MiB device array of the library,
 * whose address is looked up on the first call on each device (make that call
 * before any stream capture).  x and y are device pointers, vector v belongs
 * to instance v % nk; requests needing more than 16 MiB of scratch
 * (nvec * 12 * n^3 * element size) are rejected with FAME_ERR_BAD_ARG.  The
 * plan's device must be the current device (FAME_ERR_BAD_ARG otherwise).  All
 * calls share the array: calls whose kernels overlap on the GPU race.
 * No counterpart in the reference. */
int fame_apply_B_noalloc(fame_plan_t plan, int prec, const void* x, void* y, int nvec);

/* y = B^{-1} x by conjugate gradients to relative residual `tol` within
 * `maxit` iterations per vector; iters/relres (may be NULL) receive per-vector
 * results.  Returns FAME_ERR_NOT_CONVERGED if any vector missed `tol`.
 * Replaces fun_Lanczos/fncinvB.m:1-5 (pcg(B_op, x, tol, maxit)). */
int fame_apply_Binv(fame_plan_t plan, int prec, const void* x, void* y, int nvec, const int* inst, double tol,
                    int maxit, int* iters, double* relres, int flags);

/* Curl singular-vector transform on 3*Nq vectors: trans = 0 'notranspose'
 * (S .* ifftn(.)*sqrt(N) per component), 1 'transpose' (fftn(conj(S).*.)/sqrt(N)).
 * Replaces subroutines/MtxVecMul_FFT.m:1, gMtxVecMul_FFT.m:1 and
 * kMtxVecMul_FFT.m:1 for quasi-periodic ('DFT') types. */
int fame_curl_transform(fame_plan_t plan, int prec, int trans, const void* x, void* y, int nvec, const int* inst,
                        int flags);

/* Composed handles fnc.Pr / fnc.Qr (2Nq -> 3Nq) and fnc.Prs / fnc.Qrs
 * (3Nq -> 2Nq).  Replaces fun_Lanczos/Funhand_Generate_Lanzcos.m:79-82. */
int fame_apply_handle(fame_plan_t plan, int prec, int which, const void* x, void* y, int nvec, const int* inst,
                      int flags);

/* [u'; v'] = [M_int J_int^H; J_int N_int] [u; v] on 6*Nq vectors (the
 * material middle factor of fncB, Bloch frame).  Replaces the sparse products
 * mtx_B.M_int*u + mtx_B.J_int'*v, mtx_B.J_int*u + mtx_B.N_int*v of
 * fun_Lanczos/fncB.m:4-5. */
int fame_apply_material(fame_plan_t plan, int prec, const void* x, void* y, int nvec, const int* inst, int flags);

/*
 * Thick-restart Lanczos for the `k` largest eigenvalues of B^{-1}A of one
 * instance, in the B inner product, restart size p, Ritz tolerance `tol`,
 * at most `maxit` restarts.  v0 [4Nq] (host, complex128) or NULL for ones.
 * Inner solves: B^{-1} by CG at `inner_tol` (<= 0: 1e-12).
 * prec = FAME_C128: every matvec in complex128 (the reference's form).
 * prec = FAME_C64 : complex64 matvecs and inner CG with FP64 recurrence,
 *                   reorthogonalisation and a final FP64 refinement.
 * Outputs: ew[k] eigenvalues of B^{-1}A, descending (omega = 1/ew);
 * ev (device, complex128, 4Nq x k, may be NULL) B-normalised Ritz vectors;
 * res[k] (may be NULL) the NFSEP residual ||B x - omega A x|| of the
 * B-normalised Ritz vector with FP64 matvecs (EvaluteError_Chiral_no_inv.m:20);
 * stats[4] (may be NULL): Lanczos steps, restarts, B applies, inner CG iterations.
 * Replaces fun_Lanczos/Lanczos.m:1-167 (with op_invB of
 * band_structure_woodpile_Lanczos_n60_gamma0p2.m:74-81).
 */
int fame_lanczos(fame_plan_t plan, int prec, int inst, int k, double tol, int maxit, int p, const double* v0,
                 double inner_tol, double* ew, void* ev, double* res, long long* stats);

/*
 * Batched band solve: fame_lanczos on every instance of the plan at once
 * (vectors of all k-points advance together; converged k-points drop out).
 * ew[nk*k], ev (device complex128 [nk][k][4Nq], may be NULL) B-normalised
 * Ritz vectors, res[nk*k] (may be NULL), stats[nk*4] (may be NULL).
 */
int fame_band_solve(fame_plan_t plan, int prec, int k, double tol, int maxit, int p, double inner_tol,
                    double* ew, void* ev, double* res, long long* stats);

/*
 * Interior eigenpairs by SIRA with locking: the `nev` eigenvalues theta of
 * fncB x = theta fncA x (theta = omega) closest to `target`, residual
 * ||B u - theta A u|| <= tol for unit u.  Search space of at most
 * `no_restart` + locked vectors, restarts keep `restart_dim` Ritz vectors;
 * SIRA corrections t = (B - shift A)^{-1} r in `inner_prec` (FAME_C64 or
 * FAME_C128) to relative tolerance `inner_tol` within `inner_maxit`
 * iterations: shift = 0 is the reference's correction (its shift term is
 * commented out) solved by CG, shift != 0 the shifted correction by MINRES.
 * Outputs: ew[nev] (NaN where not converged), ev (device complex128
 * 4Nq x nev, may be NULL) unit eigenvectors, res[nev] (may be NULL),
 * stats[4] (may be NULL): outer steps, inner CG iterations, B applies,
 * pairs converged.  Replaces light_locked_Huang/GEP_AB_Herm_JDSIRA_Driver4.m:1-82
 * with GEP_AB_Herm_JDSIRA_Locking4.m and SIRA_solve_residual_LS_GEP.m
 * (called as Driver4(fncB, fncA, ...) in main_EIG_np_*.m).
 */
int fame_jdsira(fame_plan_t plan, int inner_prec, int inst, int nev, double target, double shift, double tol,
                int no_restart, int restart_dim, double inner_tol, int inner_maxit, double* ew, void* ev, double* res,
                long long* stats);

/*
 * Eigenvector restoration and checks for FP64 eigenpairs x (device complex128
 * [nvec][4Nq], vector v of instance inst[v], inst NULL: v % nk) with
 * frequencies omega[nvec] (host):
 *   E, H (device complex128 [nvec][3Nq] each, may be NULL): the fields
 *     [e; h] = -1i*[N J; J' M]*[Qr(x2); Pr(x1)]
 *     (Eigen_Restoration_Chiral_no_inv.m:3-25);
 *   res_orgsep[nvec] (host, may be NULL): the ORGSEP residual
 *     ||[N J; J' M]*[C'*h; -C*e] - 1i*omega*[e; h]|| with the explicit curl
 *     C of @DistOp/C.m (EvaluteError_Chiral_no_inv.m:19);
 *   max_e, max_h[nvec] (host, may be NULL): max over components of |e_c| and
 *     |h_c|, at every vertex or (outside_only != 0) at vertices of phase id 0
 *     only (Fig6cd_plot_max_field.m:58-69).
 */
int fame_restore(fame_plan_t plan, int nvec, const int* inst, const void* x, const double* omega, void* E, void* H,
                 double* res_orgsep, double* max_e, double* max_h, int outside_only);

/*
 * Plan in field mode: a per-vertex isotropic chiral medium eps(r) I, mu = I,
 * xi = i gamma(r) I, zeta = -i gamma(r) I (the bi-isotropic form of
 * Physical_settings_woodpile.m:76-96 with its phase constants replaced by
 * per-vertex values).  lattice: 3x3 row-major, columns are the primitive
 * vectors; eps, gamma [n^3] (host, x fastest), eps > 0 and eps - gamma^2 > 0.
 * Replaces the per-vertex material placement of
 * Material_Matrix_Generate_Mult_Point.m:38-48 for continuous fields.
 */
int fame_plan_create_field(fame_plan_t* plan, int n, int nk, const double* theta, const double* lattice,
                           const double* eps, const double* gamma);
/* Replace the fields of a field-mode plan (same constraints). */
int fame_set_field(fame_plan_t plan, const double* eps, const double* gamma);

/*
 * Backward entry: gradient of a weighted sum of eigenfrequencies,
 *   g_eps[r] = sum_v weight[v] d omega_v / d eps(r),  likewise g_gamma,
 * by the Hellmann-Feynman form d omega = omega x^H dB x / (x^H B x) evaluated
 * vertex by vertex in FP64.  x: device complex128 [nvec][4Nq] eigenvectors of
 * fncA x = (1/omega) fncB x (any normalisation), vector v of instance inst[v]
 * (inst NULL: v % nk); omega, weight [nvec] host; g_eps, g_gamma [n^3] device
 * FP64, overwritten (accumulate = 0) or added to; xbx [nvec] host (may be
 * NULL) receives x^H B x.  Field-mode plans only.  For a degenerate cluster
 * give every member the same weight (the trace is what is differentiable).
 * No counterpart in the reference.
 */
int fame_eig_gradient(fame_plan_t plan, int nvec, const int* inst, const void* x, const double* omega,
                      const double* weight, double* g_eps, double* g_gamma, int accumulate, double* xbx);

/*
 * Covariant material blocks of one phase: invert the 6x6 constitutive block
 * [eps xi; zeta mu] (row-major, interleaved complex, 36*2 doubles), split it
 * and return A'*X*A of the (1,1), (2,2) and (1,2) blocks as 27 complex
 * (N | M | J, row-major) in out[54].  lattice: 3x3 row-major, columns are the
 * primitive vectors.  Replaces Physical_settings_woodpile.m:91-96,184-194.
 */
int fame_material_blocks(const double* eps_xi_zeta_mu, const double* lattice, double* out);

/*
 * Vertex rasterisation of one inclusion on the device: every vertex of the
 * n^3 grid (lattice coefficients (i-1)/n, Public/Grid_Generate_Mult_Point.m:7-17)
 * inside the shape gets phase id `id`; the others get 0, or keep their id
 * when `flags` has FAME_RASTER_PAINT (several inclusions, the union of
 * Material_Locate_Isofunction.m:22-25).  phase [n^3], x fastest, device
 * memory unless `flags` has FAME_HOST_PTR.  lattice: 3x3 row-major, columns
 * are the primitive vectors.  Shapes and params:
 *   FAME_SHAPE_WOODPILE  {width, a}: Public/woodpile_isofun.m:1-13;
 *   FAME_SHAPE_SPHERE    {radius, cx, cy, cz}: -min_c |r - c| > -radius over
 *                        the 27 periodic images of the centre
 *                        (Physical_settings_sphere.m:18);
 *   FAME_SHAPE_TETRA     {edge, cx, cy, cz}: regular tetrahedron with
 *                        vertices along (1,1,1), (1,-1,-1), (-1,1,-1),
 *                        (-1,-1,1), inside when on the opposite vertex's side
 *                        of every face or within 1e-8 of it
 *                        (Material_Locate_Isofunction.m:135-148), 27 images.
 * Synchronous.  Replaces the host-side point location of
 * subroutines/Material_Locate_Isofunction.m:1-28.
 */
enum fame_shape { FAME_SHAPE_WOODPILE = 0, FAME_SHAPE_SPHERE = 1, FAME_SHAPE_TETRA = 2 };
#define FAME_RASTER_PAINT 2
int fame_rasterize(int n, const double* lattice, int shape, const double* params, int id, uint8_t* phase,
                   int flags);

#ifdef __cplusplus
}
#endif

#endif /* FAME_GB300_H */
