// Autotuner of the fncB launch sequence: times the candidate launch
// parameters on the plan's own grid, instances and batch width and keeps the
// fastest per (precision, batch width).  Knobs:
//   chunk        vectors per launch sequence (whole batch, 1/2, 1/4, 1/8,
//                any width up to 16): smaller sub-batches keep the six-field
//                intermediates in L2, and some widths fill the last wave of
//                CTAs better than others;
//   stencil_tpb  the material stencil's form: 0 the single-pass k_sweep,
//                128/256/512 threads per block of the two-kernel form;
//   lanes        the plane kernels' split of each pencil: threads per pencil
//                of the prime-factor split (every count compiled for the
//                size, plane_lanes_alt) or 0, one thread per pencil.
// chunk x stencil_tpb are timed with the size's default split, then every
// split with the best of those.  No counterpart in the reference.
#include <algorithm>
#include <vector>

#include "fame_internal.h"

namespace fame {

TuneEntry tune_for(const Plan& P, int prec, int nvec) {
  for (const TuneEntry& t : P.tune)
    if (t.prec == prec && t.nvec == nvec) return t;
  TuneEntry d;
  d.prec = prec;
  d.nvec = nvec;
  // complex64: single pass (two CTAs per SM); complex128 stages twice the
  // bytes per plane and keeps the two-kernel form unless tuned otherwise
  d.stencil_tpb = prec == FAME_C64 ? 0 : 256;
  return d;
}

// Install t; cached graphs hold the kernels of the old parameters, so a
// change drops them.
static void put_tune(Plan& P, const TuneEntry& t) {
  for (TuneEntry& u : P.tune)
    if (u.prec == t.prec && u.nvec == t.nvec) {
      if (u.chunk != t.chunk || u.stencil_tpb != t.stencil_tpb || u.lanes != t.lanes) free_graphs(P);
      u = t;
      return;
    }
  free_graphs(P);
  P.tune.push_back(t);
}

template <class R>
static int autotune_prec(Plan& P, int nvec, int reps, TuneEntry* best_out) {
  // the double-single operator takes complex128 vectors
  constexpr bool ds = std::is_same<R, ff>::value;
  using IO = typename std::conditional<ds, double, R>::type;
  cudaStream_t st = P.stream;
  const long long L = 4 * P.Nq;
  cudaError_t e;
  cx<IO>* x = (cx<IO>*)workspace(P, 60, sizeof(cx<IO>) * L * nvec, &e);
  if (e != cudaSuccess) return cuda_fail(&P, e, "autotune buffers");
  cx<IO>* y = (cx<IO>*)workspace(P, 61, sizeof(cx<IO>) * L * nvec, &e);
  if (e != cudaSuccess) return cuda_fail(&P, e, "autotune buffers");
  e = cudaMemsetAsync(x, 0x3c, sizeof(cx<IO>) * L * nvec, st);  // finite, normal values
  if (e == cudaSuccess) e = ensure_work(P, nvec);
  if (e != cudaSuccess) return cuda_fail(&P, e, "autotune setup");
  VecCtx ctx;
  ctx.nk = P.nk;
  auto launch = [&]() -> cudaError_t {
    if constexpr (ds) {
      return launch_fncB_ds(P, x, y, nvec, ctx, st);
    } else {
      cx<R>* w0 = (cx<R>*)P.d_work;
      cx<R>* w1 = w0 + (size_t)nvec * 6 * P.Nq;
      return launch_fncB<R>(P, x, y, nvec, ctx, w0, w1, st);
    }
  };
  // The whole batch, halves, quarters and eighths, and every width up to 16:
  // the plane kernels launch 2n CTAs per vector, and how well a width fills
  // the last wave of resident CTAs (2 per SM at n = 60) matters as much as
  // L2 residency.
  std::vector<int> chunks;
  auto add = [&](int c) {
    if (c >= 1 && c <= nvec && std::find(chunks.begin(), chunks.end(), c) == chunks.end()) chunks.push_back(c);
  };
  for (int div : {1, 2, 4, 8}) add((nvec + div - 1) / div);
  for (int c = 1; c <= 16; ++c) add(c);
  const int prec = tune_prec<R>();
  const TuneEntry saved = tune_for(P, prec, nvec);
  cudaEvent_t ev[2];
  cudaEventCreate(&ev[0]);
  cudaEventCreate(&ev[1]);
  TuneEntry best;
  best.us = 1e300;
  // median time of one fncB on the batch with t installed (microseconds)
  auto time_one = [&](TuneEntry& t) -> cudaError_t {
    put_tune(P, t);
    cudaError_t e2 = launch();  // warm-up
    std::vector<float> ms;
    for (int r = 0; r < reps && e2 == cudaSuccess; ++r) {
      cudaEventRecord(ev[0], st);
      e2 = launch();
      cudaEventRecord(ev[1], st);
      if (e2 == cudaSuccess) e2 = cudaEventSynchronize(ev[1]);
      float m = 0.f;
      if (e2 == cudaSuccess) e2 = cudaEventElapsedTime(&m, ev[0], ev[1]);
      ms.push_back(m);
    }
    if (e2 == cudaSuccess) {
      std::sort(ms.begin(), ms.end());
      t.us = 1e3 * double(ms[ms.size() / 2]);
    }
    return e2;
  };
  for (int c : chunks)
    for (int tpb : {0, 128, 256, 512}) {
      if (e != cudaSuccess) break;
      TuneEntry t;
      t.prec = prec;
      t.nvec = nvec;
      t.chunk = c == nvec ? 0 : c;
      t.stencil_tpb = tpb;
      e = time_one(t);
      if (e == cudaSuccess && t.us < best.us) best = t;
    }
  // the plane kernels' split, with the best chunk and stencil form
  if (e == cudaSuccess && P.opt_plane_split && plane_split(P.n) > 0) {
    std::vector<int> lanes;
    if (!ds) lanes.push_back(0);  // one thread per pencil (not compiled in double-single)
    for (int i = 1; i < kPlaneLanesMax; ++i)
      if (plane_lanes_alt(P.n, i) > 0) lanes.push_back(plane_lanes_alt(P.n, i));
    const TuneEntry base = best;
    for (int g : lanes) {
      TuneEntry t = base;
      t.lanes = g;
      e = time_one(t);
      if (e != cudaSuccess) break;
      if (t.us < best.us) best = t;
    }
  }
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  if (e != cudaSuccess) {
    put_tune(P, saved);
    return cuda_fail(&P, e, "autotune");
  }
  put_tune(P, best);
  *best_out = best;
  return FAME_OK;
}

}  // namespace fame

using namespace fame;

extern "C" {

int fame_autotune(fame_plan_t h, int prec, int nvec, int* chunk, int* stencil_tpb, double* us) {
  if (!h) return FAME_ERR_BAD_ARG;
  Plan& P = h->P;
  if (nvec < 1 || (prec != FAME_C64 && prec != FAME_C128 && prec != FAME_C128_DS))
    return fail(&P, FAME_ERR_BAD_ARG, "fame_autotune: bad argument");
  if (prec == FAME_C128_DS && !ds_supported(P.n))
    return fail(&P, FAME_ERR_UNSUPPORTED, "fame_autotune: no double-single fncB for this grid size");
  TuneEntry b;
  const int rc = prec == FAME_C64    ? autotune_prec<float>(P, nvec, 5, &b)
                 : prec == FAME_C128 ? autotune_prec<double>(P, nvec, 5, &b)
                                     : autotune_prec<ff>(P, nvec, 5, &b);
  if (rc != FAME_OK) return rc;
  if (chunk) *chunk = b.chunk;
  if (stencil_tpb) *stencil_tpb = b.stencil_tpb;
  if (us) *us = b.us;
  return FAME_OK;
}

int fame_set_tune(fame_plan_t h, int prec, int nvec, int chunk, int stencil_tpb) {
  if (!h) return FAME_ERR_BAD_ARG;
  Plan& P = h->P;
  if (nvec < 1 || chunk < 0 || (stencil_tpb != 0 && stencil_tpb != 128 && stencil_tpb != 256 && stencil_tpb != 512) ||
      (prec != FAME_C64 && prec != FAME_C128 && prec != FAME_C128_DS))
    return fail(&P, FAME_ERR_BAD_ARG, "fame_set_tune: bad argument");
  TuneEntry t = tune_for(P, prec, nvec);  // keeps the width's split
  t.chunk = chunk >= nvec ? 0 : chunk;
  t.stencil_tpb = stencil_tpb;
  put_tune(P, t);
  return FAME_OK;
}

int fame_set_tune_lanes(fame_plan_t h, int prec, int nvec, int lanes) {
  if (!h) return FAME_ERR_BAD_ARG;
  Plan& P = h->P;
  if (nvec < 1 || lanes < -1 || lanes > 64 || (prec != FAME_C64 && prec != FAME_C128 && prec != FAME_C128_DS))
    return fail(&P, FAME_ERR_BAD_ARG, "fame_set_tune_lanes: bad argument");
  TuneEntry t = tune_for(P, prec, nvec);
  t.lanes = lanes;
  put_tune(P, t);
  return FAME_OK;
}

int fame_get_tune(fame_plan_t h, int prec, int nvec, int* chunk, int* stencil_tpb, int* lanes) {
  if (!h) return FAME_ERR_BAD_ARG;
  Plan& P = h->P;
  if (nvec < 1 || (prec != FAME_C64 && prec != FAME_C128 && prec != FAME_C128_DS))
    return fail(&P, FAME_ERR_BAD_ARG, "fame_get_tune: bad argument");
  const TuneEntry t = tune_for(P, prec, nvec);
  if (chunk) *chunk = t.chunk;
  if (stencil_tpb) *stencil_tpb = t.stencil_tpb;
  if (lanes) *lanes = t.lanes;
  return FAME_OK;
}

}  // extern "C"
