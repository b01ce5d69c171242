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
  // pdl: join consecutive kernel nodes by programmatic edges (the next kernel
  // is launched while the previous one runs and waits in pdl_enter)
  explicit GraphChain(cudaGraph_t g, bool pdl = false) : g_(g), pdl_(pdl) {}

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
    no_pdl_ = true;
    add_kernel(reinterpret_cast<void*>(f), grid, block, vals, std::index_sequence_for<P...>{});
    no_pdl_ = false;
    smem_ = 0;
    last_is_kernel_ = false;   // the node after a cooperative launch waits for it in the ordinary way
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
    last_is_kernel_ = false;
    return GraphChain(p.conditional.phGraph_out[0], pdl_);
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
    if (pdl_ && !no_pdl_ && has_last_ && last_is_kernel_) {
      cudaGraphNodeParams np = {};
      np.type = cudaGraphNodeTypeKernel;
      np.kernel.func = kp.func;
      np.kernel.gridDim = kp.gridDim;
      np.kernel.blockDim = kp.blockDim;
      np.kernel.sharedMemBytes = kp.sharedMemBytes;
      np.kernel.kernelParams = kp.kernelParams;
      np.kernel.extra = kp.extra;
      cudaGraphEdgeData ed = {};
      ed.from_port = cudaGraphKernelNodePortProgrammatic;
      ed.type = cudaGraphDependencyTypeProgrammatic;
      const cudaError_t pe = cudaGraphAddNode(&node, g_, &last_, &ed, 1, &np);
      if (pe == cudaSuccess) {
        last_ = node;
        ++n_prog_;
        return;
      }
      cudaGetLastError();   // not supported here: an ordinary edge
      last_prog_err_ = pe;
    }
    err_ = cudaGraphAddKernelNode(&node, g_, has_last_ ? &last_ : nullptr, has_last_ ? 1 : 0, &kp);
    if (err_ == cudaSuccess) {
      last_ = node;
      has_last_ = true;
      last_is_kernel_ = true;
    }
  }

  cudaGraph_t g_;
  cudaGraphNode_t last_ = nullptr;
  bool has_last_ = false;
  cudaError_t err_ = cudaSuccess;
  size_t smem_ = 0;
  bool pdl_ = false;
  bool no_pdl_ = false;
  bool last_is_kernel_ = false;

 public:
  int n_prog_ = 0;                              // kernel nodes joined by a programmatic edge
  cudaError_t last_prog_err_ = cudaSuccess;     // why the last programmatic edge was refused
};

}  // namespace pfgb
