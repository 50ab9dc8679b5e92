// Template body of graph_replay (fame_internal.h): capture once, replay after.
#pragma once

#include "fame_internal.h"
#include "krylov.h"

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
    FAME_UNCOUNT_CAPTURED(captured);
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
  if (e == cudaSuccess) FAME_GRAPH_LAUNCHED(ge->nodes);
  return e;
}

// Run `body(stream)` repeatedly from ONE graph launch: a conditional WHILE
// node whose body is the captured sequence followed by the loop condition
// (while_active: any active[v] and fewer than max_passes passes), so the
// host neither waits nor launches between passes.  The body always runs at
// least once.  *passes (device) counts the passes of this launch; the caller
// reads it after the stream completes and adds passes x *body_nodes to the
// kernel count (FAME_KERNELS_RAN; the graph launch itself is counted here).  Cached under
// `key` like graph_replay.  Returns cudaErrorNotSupported when conditional
// nodes or capture are unavailable (the caller falls back to graph_replay).
template <class F>
cudaError_t graph_replay_while(Plan& P, const std::vector<uintptr_t>& key, F&& body, const int* active, int nvec,
                               int* passes, int max_passes, unsigned long long* body_nodes) {
  GraphEntry* ge = nullptr;
  cudaError_t e = graph_lookup(P, key, &ge);
  if (e != cudaSuccess) return e;
  if (!ge) {
    if (!P.cap_stream) {
      e = cudaStreamCreateWithFlags(&P.cap_stream, cudaStreamNonBlocking);
      if (e != cudaSuccess) return e;
    }
    cudaGraph_t g = nullptr;
    e = cudaGraphCreate(&g, 0);
    if (e != cudaSuccess) return e;
    cudaGraphConditionalHandle h;
    e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault);
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    if (e == cudaSuccess) e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np);
    if (e != cudaSuccess) {
      cudaGraphDestroy(g);
      cudaGetLastError();
      return cudaErrorNotSupported;
    }
    cudaGraph_t bg = np.conditional.phGraph_out[0];
    e = cudaStreamBeginCaptureToGraph(P.cap_stream, bg, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
      cudaGraphDestroy(g);
      cudaGetLastError();
      return cudaErrorNotSupported;
    }
    cudaError_t ie = body(P.cap_stream);
    if (ie == cudaSuccess) ie = while_active(active, nvec, passes, max_passes, h, P.cap_stream);
    cudaGraph_t got = nullptr;
    e = cudaStreamEndCapture(P.cap_stream, &got);
    // recorded, not run: the body's kernels are counted per pass when replayed
    const unsigned long long captured = graph_kernel_nodes(bg);
    FAME_UNCOUNT_CAPTURED(captured);
    if (ie != cudaSuccess || e != cudaSuccess) {
      cudaGraphDestroy(g);
      cudaGetLastError();
      return ie != cudaSuccess ? ie : e;
    }
    e = graph_store(P, key, g, captured, &ge);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return cudaErrorNotSupported;
    }
  }
  e = cudaMemsetAsync(passes, 0, sizeof(int), P.stream);
  if (e == cudaSuccess) e = cudaGraphLaunch(ge->exec, P.stream);
  if (e == cudaSuccess) {
    FAME_GRAPH_LAUNCHED(0);  // the body's kernels: FAME_KERNELS_RAN by the caller
    *body_nodes = ge->nodes;
  }
  return e;
}

}  // namespace fame
