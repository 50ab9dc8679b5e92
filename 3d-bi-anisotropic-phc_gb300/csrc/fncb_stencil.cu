// fncA, the Bloch phase, and the dispatch from a plan's grid size to the
// size-templated transforms and material stencil instantiated in
// fncb_inst_*.cu.
#include "fncb_impl.cuh"

namespace fame {
namespace detail {


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

// Pi1 | Pi2 per frequency voxel of each instance (SVD_Matrix_curl.m:45-57),
// the same pi_block the transform kernels would evaluate.
template <class R>
__global__ void k_pi_table(const cx<R>* __restrict__ lam_all, int n, long long Nq, cx<R>* __restrict__ out) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int inst = blockIdx.y;
  if (idx >= Nq) return;
  const int i1 = int(idx % n), i2 = int((idx / n) % n), i3 = int(idx / ((long long)n * n));
  const cx<R>* lam = lam_all + (long long)inst * 3 * n;
  const PiBlock<R> P = pi_block<R>(lam[i1], lam[n + i2], lam[2 * n + i3]);
  cx<R>* o = out + ((long long)inst * Nq + idx) * 6;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    o[i] = P.p1[i];
    o[3 + i] = P.p2[i];
  }
}

inline dim3 grid_pts1(long long Nq, int nvec, int tpb) {
  return dim3((unsigned)((Nq + tpb - 1) / tpb), (unsigned)nvec, 1);
}

}  // namespace detail

// the size-templated transforms are instantiated elsewhere
#define FAME_EXTERN(NN) FAME_SIZE_SIGS(extern template, float, NN) FAME_SIZE_SIGS(extern template, double, NN)
#define FAME_EXTERN_DS(NN) FAME_DS_SIGS(extern template, NN)
}  // namespace fame
FAME_FOR_EACH_N(FAME_EXTERN)
FAME_FOR_EACH_DS_N(FAME_EXTERN_DS)
namespace fame {
namespace detail {

template <class R>
cudaError_t stencil(const Plan& P, cx<R>* w, cx<R>* h, int nvec, const VecCtx& ctx, cudaStream_t st) {
  switch (P.n) {
#define FAME_CASE(NN) case NN: return stencil_n<R, NN>(P, w, h, nvec, ctx, st, 256);
    FAME_FOR_EACH_N(FAME_CASE)
#undef FAME_CASE
    default: return cudaErrorInvalidValue;
  }
}

template cudaError_t stencil<float>(const Plan&, cx<float>*, cx<float>*, int, const VecCtx&, cudaStream_t);
template cudaError_t stencil<double>(const Plan&, cx<double>*, cx<double>*, int, const VecCtx&, cudaStream_t);

}  // namespace detail
using namespace detail;

template <class R>
cudaError_t build_pi_table(Plan& P) {
  PlanData<R>& d = const_cast<PlanData<R>&>(pdata<R>(P));
  if (d.pi) return cudaSuccess;
  cudaError_t e = cudaMalloc(&d.pi, sizeof(cx<R>) * 6 * (size_t)P.Nq * P.nk);
  if (e != cudaSuccess) {
    d.pi = nullptr;
    return e;
  }
  FAME_LAUNCHED(1);
  k_pi_table<R><<<dim3((unsigned)((P.Nq + 255) / 256), (unsigned)P.nk), 256, 0, P.stream>>>(d.lam, P.n, P.Nq, d.pi);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(P.stream);
  return e;
}
template cudaError_t build_pi_table<float>(Plan&);
template cudaError_t build_pi_table<double>(Plan&);

// ---------------------------------------------------------------------------
// Double-single fncB: complex128 in and out, complex float-float inside.
// ---------------------------------------------------------------------------
namespace {
// out[i] = in[i] split into hi + lo (in place allowed: same 16-byte element);
// with `active`, vector blockIdx.y of length len is skipped when inactive.
__global__ void k_to_ds(const double2* in, cff* out, long long len, const int* active) {
  if (active && !active[blockIdx.y]) return;
  const long long o = (long long)blockIdx.y * len;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x) {
    const double2 v = in[o + i];
    cff c;
    c.x = ff(v.x);
    c.y = ff(v.y);
    out[o + i] = c;
  }
}
__global__ void k_real_to_ds(const double* in, ff* out, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = ff(in[i]);
}
inline unsigned conv_grid(long long n) {
  const long long g = (n + 255) / 256;
  return (unsigned)(g < 4096 ? (g > 0 ? g : 1) : 4096);
}
// dst = double-single copy of the n complex128 values at src (allocated on
// first use)
cudaError_t copy_to_ds(const double2* src, cff** dst, long long n, cudaStream_t st) {
  if (!src) return cudaSuccess;
  if (!*dst) {
    cudaError_t e = cudaMalloc(dst, sizeof(cff) * (size_t)n);
    if (e != cudaSuccess) {
      *dst = nullptr;
      return e;
    }
  }
  FAME_LAUNCHED(1);
  k_to_ds<<<dim3(conv_grid(n), 1), 256, 0, st>>>(src, *dst, n, nullptr);
  return cudaGetLastError();
}
}  // namespace

bool ds_supported(int n) {
  switch (n) {
#define FAME_CASE(NN) case NN: return true;
    FAME_FOR_EACH_DS_N(FAME_CASE)
#undef FAME_CASE
    default: return false;
  }
}

// (Re)builds the double-single tables from the complex128 ones; called at
// plan creation and again when a field-mode plan's fields change.
int upload_tables_ds(Plan& P) {
  if (!ds_supported(P.n)) return FAME_OK;
  const PlanData<double>& s = P.d64;
  PlanData<ff>& d = P.dds;
  cudaStream_t st = P.stream;
  cudaError_t e = copy_to_ds(s.lam, &d.lam, (long long)P.nk * 3 * P.n, st);
  if (e == cudaSuccess) e = copy_to_ds(s.tau, &d.tau, (long long)P.nk * 3, st);
  if (e == cudaSuccess) e = copy_to_ds(s.sxyz, &d.sxyz, (long long)P.nk * 3 * P.n, st);
  if (e == cudaSuccess) e = copy_to_ds(s.mat, &d.mat, (long long)P.nk * P.nphase * 27, st);
  if (e == cudaSuccess) e = copy_to_ds(s.pi, &d.pi, (long long)P.nk * 6 * P.Nq, st);
  if (e == cudaSuccess && s.fld) {
    if (!d.fld) e = cudaMalloc(&d.fld, sizeof(ff) * 3 * (size_t)P.Nq);
    if (e == cudaSuccess) {
      FAME_LAUNCHED(1);
      k_real_to_ds<<<conv_grid(3 * P.Nq), 256, 0, st>>>(s.fld, d.fld, 3 * P.Nq);
      e = cudaGetLastError();
    }
  }
  for (int i = 0; i < 9; ++i) d.gram[i] = ff(s.gram[i]);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e == cudaSuccess ? FAME_OK : cuda_fail(&P, e, "double-single tables");
}

cudaError_t launch_fncB_ds(const Plan& P, const double2* x, double2* y, int nvec, const VecCtx& ctx,
                           cudaStream_t st) {
  if (nvec <= 0) return cudaSuccess;
  // the first and last kernels of the double-single fncB read and write
  // complex128 elements (load_io / store_io): the vectors are passed as they are
  const cff* xd = reinterpret_cast<const cff*>(x);
  cff* yd = reinterpret_cast<cff*>(y);
  cff* w0 = reinterpret_cast<cff*>(P.d_work);
  cff* w1 = w0 + (size_t)nvec * 6 * P.Nq;
  switch (P.n) {
#define FAME_CASE(NN) \
  case NN: return fncB_n<ff, NN>(P, xd, yd, nvec, ctx, w0, w1, st, nullptr, nullptr, nullptr);
    FAME_FOR_EACH_DS_N(FAME_CASE)
#undef FAME_CASE
    default: return cudaErrorInvalidValue;
  }
}

// Partials per vector that fncB's pq output receives for a batch of nvec, or
// 0 when the tuned form of that batch does not produce them.
template <class R>
int fncB_pq_partials(const Plan& P, int nvec) {
  if (tune_for(P, tune_prec<R>(), nvec).stencil_tpb != 0) return 0;
  switch (P.n) {
#define FAME_CASE(NN) case NN: return sweep_partials_n<R, NN>();
    FAME_FOR_EACH_N(FAME_CASE)
#undef FAME_CASE
    default: return 0;
  }
}

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
                        cx<R>* w1, cudaStream_t st, double2* pq, const cx<R>* pupd_z, const double* pupd_beta) {
  if (nvec <= 0) return cudaSuccess;
  switch (P.n) {
#define FAME_CASE(NN) case NN: return fncB_n<R, NN>(P, x, y, nvec, ctx, w0, w1, st, pq, pupd_z, pupd_beta);
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
cudaError_t launch_stencil(const Plan& P, cx<R>* w, cx<R>* h, int nvec, const VecCtx& ctx, cudaStream_t st) {
  if (nvec <= 0) return cudaSuccess;
  return stencil<R>(P, w, h, nvec, ctx, st);
}

template <class R>
cudaError_t launch_fields_inv(const Plan& P, const cx<R>* x, cx<R>* w, int nvec, const VecCtx& ctx,
                              cudaStream_t st) {
  if (nvec <= 0) return cudaSuccess;
  switch (P.n) {
#define FAME_CASE(NN) case NN: return fields_inv_n<R, NN>(P, x, w, nvec, ctx, st);
    FAME_FOR_EACH_N(FAME_CASE)
#undef FAME_CASE
    default: return cudaErrorInvalidValue;
  }
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
                                      cx<R>*, cudaStream_t, double2*, const cx<R>*, const double*);       \
  template int fncB_pq_partials<R>(const Plan&, int);                                                     \
  template cudaError_t launch_fncA<R>(const Plan&, const cx<R>*, cx<R>*, int, const VecCtx&,             \
                                      cudaStream_t);                                                      \
  template cudaError_t launch_fields_inv<R>(const Plan&, const cx<R>*, cx<R>*, int, const VecCtx&,       \
                                            cudaStream_t);                                                \
  template cudaError_t launch_stencil<R>(const Plan&, cx<R>*, cx<R>*, int, const VecCtx&, cudaStream_t); \
  template cudaError_t launch_transform<R>(const Plan&, int, const cx<R>*, cx<R>*, int, const VecCtx&,   \
                                           cudaStream_t);                                                 \
  template cudaError_t launch_handle<R>(const Plan&, int, const cx<R>*, cx<R>*, int, const VecCtx&,      \
                                        cx<R>*, cudaStream_t);                                            \
  template cudaError_t launch_material<R>(const Plan&, const cx<R>*, cx<R>*, int, const VecCtx&, cx<R>*, \
                                          cudaStream_t);
FAME_INST(float)
FAME_INST(double)

}  // namespace fame
