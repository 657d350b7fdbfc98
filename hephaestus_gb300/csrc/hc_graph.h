// hc_graph.h -- building device-driven solve graphs.
//
// A solve graph is a chain of captured segments (child-graph nodes) and
// conditional WHILE and IF nodes.  A WHILE body ends with a kernel that sets the
// loop condition from device state (the solver's `done` flag and a trip
// counter with a hard bound), so a launched solve runs to completion on the
// device without host round trips and always terminates.
#pragma once
#include <cuda_runtime.h>

namespace hc {

struct GraphChain {
  cudaGraph_t graph = nullptr;      // graph the chain is appended to
  cudaGraphNode_t last = nullptr;   // last node of the chain (nullptr: empty)
};

// Capture fn(stream) and append it to the chain as one child-graph node.
template <typename F>
inline cudaError_t chain_segment(GraphChain& c, cudaStream_t cs, F&& fn) {
  cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) return e;
  const cudaError_t fe = fn(cs);
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(cs, &g);
  if (fe != cudaSuccess || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return fe != cudaSuccess ? fe : e;
  }
  cudaGraphNode_t n = nullptr;
  e = cudaGraphAddChildGraphNode(&n, c.graph, c.last ? &c.last : nullptr, c.last ? 1 : 0, g);
  cudaGraphDestroy(g);  // the node holds its own copy
  if (e == cudaSuccess) c.last = n;
  return e;
}

// Condition handle of a WHILE node that will be added to c (condition 1 at
// launch).  Created before the segments whose kernels set it are captured.
inline cudaError_t chain_handle(GraphChain& c, cudaGraphConditionalHandle* hnd) {
  return cudaGraphConditionalHandleCreate(hnd, c.graph, 1, cudaGraphCondAssignDefault);
}

// Append a WHILE node driven by hnd; body receives its (empty) chain.
inline cudaError_t chain_while(GraphChain& c, cudaGraphConditionalHandle hnd, GraphChain* body) {
  cudaGraphNodeParams p{};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = hnd;
  p.conditional.type = cudaGraphCondTypeWhile;
  p.conditional.size = 1;
  cudaGraphNode_t n = nullptr;
  const cudaError_t e = cudaGraphAddNode(&n, c.graph, c.last ? &c.last : nullptr, nullptr, c.last ? 1 : 0, &p);
  if (e != cudaSuccess) return e;
  c.last = n;
  body->graph = p.conditional.phGraph_out[0];
  body->last = nullptr;
  return cudaSuccess;
}

// Append an IF node driven by hnd (condition set by a kernel before it);
// body receives its (empty) chain.
inline cudaError_t chain_if(GraphChain& c, cudaGraphConditionalHandle hnd, GraphChain* body) {
  cudaGraphNodeParams p{};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = hnd;
  p.conditional.type = cudaGraphCondTypeIf;
  p.conditional.size = 1;
  cudaGraphNode_t n = nullptr;
  const cudaError_t e = cudaGraphAddNode(&n, c.graph, c.last ? &c.last : nullptr, nullptr, c.last ? 1 : 0, &p);
  if (e != cudaSuccess) return e;
  c.last = n;
  body->graph = p.conditional.phGraph_out[0];
  body->last = nullptr;
  return cudaSuccess;
}

}  // namespace hc
