// Explicit CUDA-graph assembly: kernel nodes in a chain, and WHILE conditional
// nodes whose bodies are chains of their own.  A step is built once per
// instance and replayed with one cudaGraphLaunch; loops whose trip count is
// decided on the device (CG iterations, refinement passes) run as conditional
// nodes, so nothing returns to the host inside a step.
#pragma once
#include <cuda_runtime.h>

#include <tuple>
#include <utility>
#include <vector>

namespace pfgb {

class GraphChain {
 public:
  explicit GraphChain(cudaGraph_t g) : g_(g) {}

  cudaGraph_t graph() const { return g_; }
  cudaError_t status() const { return err_; }

  // Append a kernel node that depends on the previous node of the chain.
  template <typename... P, typename... A>
  void kernel(void (*f)(P...), dim3 grid, dim3 block, A&&... args) {
    if (err_ != cudaSuccess) return;
    std::tuple<P...> vals(std::forward<A>(args)...);
    add_kernel(reinterpret_cast<void*>(f), grid, block, vals, std::index_sequence_for<P...>{});
  }

  // Same, with dynamic shared memory.
  template <typename... P, typename... A>
  void kernel_smem(void (*f)(P...), dim3 grid, dim3 block, size_t smem, A&&... args) {
    if (err_ != cudaSuccess) return;
    std::tuple<P...> vals(std::forward<A>(args)...);
    smem_ = smem;
    add_kernel(reinterpret_cast<void*>(f), grid, block, vals, std::index_sequence_for<P...>{});
    smem_ = 0;
  }

  // Same, as a cooperative launch (all CTAs co-resident), with dynamic shared memory.
  template <typename... P, typename... A>
  void kernel_coop(void (*f)(P...), dim3 grid, dim3 block, size_t smem, A&&... args) {
    if (err_ != cudaSuccess) return;
    std::tuple<P...> vals(std::forward<A>(args)...);
    smem_ = smem;
    add_kernel(reinterpret_cast<void*>(f), grid, block, vals, std::index_sequence_for<P...>{});
    smem_ = 0;
    if (err_ != cudaSuccess) return;
    cudaLaunchAttributeValue v = {};
    v.cooperative = 1;
    err_ = cudaGraphKernelNodeSetAttribute(last_, cudaLaunchAttributeCooperative, &v);
  }

  // Append a WHILE node on an existing conditional handle (created on this
  // graph with cudaGraphConditionalHandleCreate; kernels upstream of the node
  // or in its body set it with cudaGraphSetConditional).  The body runs while
  // the handle's value is non-zero.  Returns a chain on the body graph.
  GraphChain while_loop_with(cudaGraphConditionalHandle handle) {
    if (err_ != cudaSuccess) return GraphChain(nullptr, err_);
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = handle;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    err_ = cudaGraphAddNode(&node, g_, has_last_ ? &last_ : nullptr, nullptr, has_last_ ? 1 : 0, &p);
    if (err_ != cudaSuccess) return GraphChain(nullptr, err_);
    last_ = node;
    has_last_ = true;
    return GraphChain(p.conditional.phGraph_out[0]);
  }

 private:
  GraphChain(cudaGraph_t g, cudaError_t e) : g_(g), err_(e) {}

  template <typename T, std::size_t... I>
  void add_kernel(void* f, dim3 grid, dim3 block, T& vals, std::index_sequence<I...>) {
    void* argp[sizeof...(I) + 1] = {static_cast<void*>(&std::get<I>(vals))..., nullptr};
    cudaKernelNodeParams kp = {};
    kp.func = f;
    kp.gridDim = grid;
    kp.blockDim = block;
    kp.sharedMemBytes = (unsigned)smem_;
    kp.kernelParams = argp;
    kp.extra = nullptr;
    cudaGraphNode_t node;
    err_ = cudaGraphAddKernelNode(&node, g_, has_last_ ? &last_ : nullptr, has_last_ ? 1 : 0, &kp);
    if (err_ == cudaSuccess) {
      last_ = node;
      has_last_ = true;
    }
  }

  cudaGraph_t g_;
  cudaGraphNode_t last_ = nullptr;
  bool has_last_ = false;
  cudaError_t err_ = cudaSuccess;
  size_t smem_ = 0;
};

}  // namespace pfgb
