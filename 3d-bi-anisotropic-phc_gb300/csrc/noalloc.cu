// fame_apply_B_noalloc: fncB for callers that cannot let the library allocate
// device memory at call time.
//
// Who needs it: a caller whose device memory belongs to another allocator --
// a MATLAB MEX gateway running under MATLAB's gpuArray memory manager, or an
// application that keeps its whole device-memory budget in its own pool
// (PyTorch's caching allocator, for one).  There a cudaMalloc inside a
// library call can fail once the pool holds the memory, and a cudaFree
// fragments the pool.  fame_apply_B grows its plan's scratch on demand; this
// variant takes its scratch from one fixed array instead.
//
// The scratch is a file-scope __device__ array of FAME_NOALLOC_SCRATCH_BYTES
// (16 MiB), so every GPU that loads the library holds 16 MiB until the process
// exits.  In host code the array's name is only a host-side stand-in, so the
// device address is looked up with cudaGetSymbolAddress once per device (with
// that device current) on the first call on that device; make that first call
// before any stream capture.  The plan's device must be the current device
// when the entry point is called (it is checked).  The call allocates nothing: no cudaMalloc, no
// cudaFree, no allocating library routine.  All calls share the one array and
// it keeps the last call's contents; the fncB pipeline overwrites both scratch
// fields before reading them, so nothing needs clearing, but calls whose
// kernels overlap on the GPU (different streams or threads without ordering)
// race on it.
#include <cuda_runtime.h>

#include <mutex>

#include "fame_internal.h"

#define FAME_NOALLOC_SCRATCH_BYTES (16u << 20)
#define FAME_NOALLOC_MAX_DEVICES 64

namespace {

__device__ __align__(256) unsigned char g_fncb_scratch[FAME_NOALLOC_SCRATCH_BYTES];

std::mutex g_scratch_mutex;
void* g_scratch_addr[FAME_NOALLOC_MAX_DEVICES] = {};

// Device address of the scratch array on the current device (set-up on first use).
cudaError_t scratch_address(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= FAME_NOALLOC_MAX_DEVICES) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_fncb_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return cudaSuccess;
}

}  // namespace

using namespace fame;

extern "C" int fame_apply_B_noalloc(fame_plan_t h, int prec, const void* x, void* y, int nvec) {
  if (!h) return fail(nullptr, FAME_ERR_BAD_ARG, "fame_apply_B_noalloc: null plan");
  Plan& P = h->P;
  // The scratch address is per device and looked up on the current one, so
  // the plan's device must be current (the library never switches devices).
  int cur = -1;
  cudaError_t de = cudaGetDevice(&cur);
  if (de != cudaSuccess) return cuda_fail(&P, de, "fame_apply_B_noalloc device");
  if (cur != P.device)
    return fail(&P, FAME_ERR_BAD_ARG,
                "fame_apply_B_noalloc: the plan's device " + std::to_string(P.device) + " is not current (device " +
                    std::to_string(cur) + " is)");
  if (prec != FAME_C128 && prec != FAME_C64) return fail(&P, FAME_ERR_BAD_ARG, "fame_apply_B_noalloc: bad precision");
  if (nvec < 0 || (nvec > 0 && (!x || !y))) return fail(&P, FAME_ERR_BAD_ARG, "fame_apply_B_noalloc: bad vectors");
  if (nvec == 0) return FAME_OK;
  const size_t elem = prec == FAME_C64 ? sizeof(float2) : sizeof(double2);
  const size_t need = (size_t)nvec * 2 * 6 * (size_t)P.Nq * elem;  // two 6-field work buffers per vector
  if (need > FAME_NOALLOC_SCRATCH_BYTES)
    return fail(&P, FAME_ERR_BAD_ARG,
                "fame_apply_B_noalloc: " + std::to_string(nvec) + " vectors of n=" + std::to_string(P.n) + " need " +
                    std::to_string(need) + " bytes of scratch, above the fixed " +
                    std::to_string(FAME_NOALLOC_SCRATCH_BYTES) + " (use fame_apply_B)");
  void* scratch = nullptr;
  cudaError_t e = scratch_address(&scratch);
  if (e != cudaSuccess) return cuda_fail(&P, e, "fame_apply_B_noalloc scratch");
  VecCtx ctx;  // vector v belongs to instance v % nk
  ctx.nk = P.nk;
  if (prec == FAME_C64) {
    float2* w0 = (float2*)scratch;
    e = launch_fncB<float>(P, (const float2*)x, (float2*)y, nvec, ctx, w0, w0 + (size_t)nvec * 6 * P.Nq, P.stream);
  } else {
    double2* w0 = (double2*)scratch;
    e = launch_fncB<double>(P, (const double2*)x, (double2*)y, nvec, ctx, w0, w0 + (size_t)nvec * 6 * P.Nq,
                            P.stream);
  }
  return e == cudaSuccess ? FAME_OK : cuda_fail(&P, e, "fame_apply_B_noalloc");
}
