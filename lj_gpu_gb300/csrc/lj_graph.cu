// lj_graph.cu -- the persistent step loop of the MD and batch runs: one CUDA
// graph whose single node is a conditional WHILE node.  Its body is a chunk
// of captured steps followed by k_loop_next, which counts the chunks down on
// the device and ends the loop when the count runs out or a stop word (list
// overflow) is set.  One graph launch therefore runs every chunk between two
// record points with no host involvement; the host only writes the chunk
// count before the launch.
#include <vector>

#include "lj_internal.h"

namespace ljg {
namespace {

__global__ void k_loop_next(cudaGraphConditionalHandle h, int32_t* counter, const int32_t* stop) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int32_t left = counter[0] - 1;
  counter[0] = left;
  cudaGraphSetConditional(h, (left > 0 && !(stop && *stop)) ? 1u : 0u);
}

__global__ void k_loop_set(int32_t* counter, int32_t chunks) {
  if (threadIdx.x == 0 && blockIdx.x == 0) counter[0] = chunks;
}

}  // namespace

void LoopGraph::reset() {
  if (exec) cudaGraphExecDestroy(exec);
  exec = nullptr;
  kernels_per_chunk = 0;
}

cudaError_t LoopGraph::build(cudaStream_t s, int32_t* counter_word, const int32_t* stop_word,
                             const std::function<cudaError_t(cudaStream_t)>& chunk) {
  reset();
  counter = counter_word;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaGraphCreate(&g, 0);
  if (e != cudaSuccess) return e;
  cudaGraphConditionalHandle h;
  // every launch starts with the condition set: the body runs at least once
  e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault);
  cudaGraphNodeParams np{};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  if (e == cudaSuccess) e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np);
  if (e == cudaSuccess) {
    cudaGraph_t body = np.conditional.phGraph_out[0];
    e = cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0,
                                      cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      cudaError_t ce = chunk(s);
      if (ce == cudaSuccess) {
        k_loop_next<<<1, 32, 0, s>>>(h, counter, stop_word);
        ce = cudaGetLastError();
      }
      cudaGraph_t captured = nullptr;
      const cudaError_t ee = cudaStreamEndCapture(s, &captured);
      e = ce != cudaSuccess ? ce : ee;
      if (e == cudaSuccess) {
        // kernels of one pass of the body, the loop's own kernel excluded
        size_t nn = 0;
        if (cudaGraphGetNodes(body, nullptr, &nn) == cudaSuccess && nn > 0) {
          std::vector<cudaGraphNode_t> nodes(nn);
          if (cudaGraphGetNodes(body, nodes.data(), &nn) == cudaSuccess)
            for (size_t a = 0; a < nn; a++) {
              cudaGraphNodeType t;
              if (cudaGraphNodeGetType(nodes[a], &t) == cudaSuccess &&
                  t == cudaGraphNodeTypeKernel)
                kernels_per_chunk++;
            }
        }
        kernels_per_chunk -= 1;
      }
    }
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    cudaGetLastError();  // the failed capture's error is returned here, not later
    reset();
  }
  return e;
}

cudaError_t LoopGraph::launch(int32_t chunks, cudaStream_t s) {
  if (chunks <= 0) return cudaSuccess;
  k_loop_set<<<1, 32, 0, s>>>(counter, chunks);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return cudaGraphLaunch(exec, s);
}

}  // namespace ljg
