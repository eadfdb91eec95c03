// Kernel nodes for the solve graphs (cudaGraphAddKernelNode with typed
// arguments).
#pragma once

#include <cuda_runtime.h>

#include <tuple>

namespace lpm {
namespace {

// A kernel node of a graph: the arguments are converted to the kernel's
// parameter types and passed by address, as cudaGraphAddKernelNode wants.
template <typename... P, typename... A>
cudaError_t add_kernel(cudaGraphNode_t* node, cudaGraph_t g, const cudaGraphNode_t* dep, void (*fn)(P...), int grid,
                       int block, A... a) {
  std::tuple<P...> vals(a...);
  void* params[sizeof...(P) > 0 ? sizeof...(P) : 1];
  std::apply([&](auto&... x) {
    int i = 0;
    ((params[i++] = (void*)&x), ...);
  }, vals);
  cudaKernelNodeParams kp = {};
  kp.func = (void*)fn;
  kp.gridDim = dim3((unsigned)grid);
  kp.blockDim = dim3((unsigned)block);
  kp.sharedMemBytes = 0;
  kp.kernelParams = params;
  return cudaGraphAddKernelNode(node, g, dep, dep ? 1 : 0, &kp);
}



}  // namespace
}  // namespace lpm
