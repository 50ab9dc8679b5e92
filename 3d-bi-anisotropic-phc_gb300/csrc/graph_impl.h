// Template body of graph_replay (fame_internal.h): capture once, replay after.
#pragma once

#include "fame_internal.h"

namespace fame {

cudaError_t graph_lookup(Plan& P, const std::vector<uintptr_t>& key, GraphEntry** out);
unsigned long long graph_kernel_nodes(cudaGraph_t g);
cudaError_t graph_store(Plan& P, const std::vector<uintptr_t>& key, cudaGraph_t g, unsigned long long captured,
                        GraphEntry** out);

template <class F>
cudaError_t graph_replay(Plan& P, const std::vector<uintptr_t>& key, F&& issue) {
  GraphEntry* ge = nullptr;
  cudaError_t e = graph_lookup(P, key, &ge);
  if (e != cudaSuccess) return e;
  if (!ge) {
    if (!P.cap_stream) {
      e = cudaStreamCreateWithFlags(&P.cap_stream, cudaStreamNonBlocking);
      if (e != cudaSuccess) return e;
    }
    e = cudaStreamBeginCapture(P.cap_stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    cudaError_t ie = issue(P.cap_stream);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(P.cap_stream, &g);
    // The launches above were recorded, not run (each added one to the
    // counter and one kernel node to the graph): count them when replayed.
    // The graph's own kernel nodes are counted, not the counter's change,
    // which also holds other threads' launches on other plans.
    const unsigned long long captured = g ? graph_kernel_nodes(g) : 0;
    __atomic_fetch_sub(&g_kernel_launches, captured, __ATOMIC_RELAXED);
    if (ie != cudaSuccess || e != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
      return ie != cudaSuccess ? ie : e;
    }
    e = graph_store(P, key, g, captured, &ge);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return e;
  }
  e = cudaGraphLaunch(ge->exec, P.stream);
  if (e == cudaSuccess) FAME_LAUNCHED(ge->nodes);
  return e;
}

}  // namespace fame
