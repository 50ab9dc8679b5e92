// Cache of instantiated CUDA graphs per plan (see graph_replay).
#include "graph_impl.h"

namespace fame {

constexpr size_t kMaxGraphs = 8;

unsigned long long graph_kernel_nodes(cudaGraph_t g) {
  size_t n = 0;
  if (cudaGraphGetNodes(g, nullptr, &n) != cudaSuccess || n == 0) return 0;
  std::vector<cudaGraphNode_t> nodes(n);
  if (cudaGraphGetNodes(g, nodes.data(), &n) != cudaSuccess) return 0;
  unsigned long long k = 0;
  for (size_t i = 0; i < n; ++i) {
    cudaGraphNodeType t;
    if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++k;
  }
  return k;
}

cudaError_t graph_lookup(Plan& P, const std::vector<uintptr_t>& key, GraphEntry** out) {
  *out = nullptr;
  for (GraphEntry& g : P.graphs)
    if (g.key == key) {
      *out = &g;
      return cudaSuccess;
    }
  return cudaSuccess;
}

cudaError_t graph_store(Plan& P, const std::vector<uintptr_t>& key, cudaGraph_t g, unsigned long long captured,
                        GraphEntry** out) {
  if (P.graphs.size() >= kMaxGraphs) {  // evict the oldest
    cudaGraphExecDestroy(P.graphs.front().exec);
    P.graphs.erase(P.graphs.begin());
  }
  GraphEntry ge;
  ge.key = key;
  ge.nodes = captured;
  cudaError_t e = cudaGraphInstantiate(&ge.exec, g, 0);
  if (e != cudaSuccess) return e;
  P.graphs.push_back(ge);
  *out = &P.graphs.back();
  return cudaSuccess;
}

void free_graphs(Plan& P) {
  for (GraphEntry& g : P.graphs) cudaGraphExecDestroy(g.exec);
  P.graphs.clear();
  if (P.cap_stream) cudaStreamDestroy(P.cap_stream);
  P.cap_stream = nullptr;
}

}  // namespace fame
