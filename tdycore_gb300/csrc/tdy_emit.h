// tdy_emit.h -- kernel launches to a stream or into a graph.
//
// Launches go through an Emit: straight to its stream, or, while a graph is
// being built, as the next kernel node of a chain in that graph (the explicit
// graph API: the kernel's arguments are converted to its parameter types and
// copied into the node; the chain starts from `last`, which the builder may
// set).  Empty grids launch nothing in either mode.
#pragma once

#include <cuda_runtime.h>

#include <tuple>
#include <utility>

namespace tdy {

struct Emit {
  cudaStream_t st = nullptr;
  cudaGraph_t g = nullptr;
  cudaGraphNode_t last = nullptr;
  cudaError_t err = cudaSuccess;
  explicit Emit(cudaStream_t s) : st(s) {}
  template <class... P, class... A>
  void operator()(void (*k)(P...), unsigned grid, unsigned block, size_t smem, A... args) {
    static_assert(sizeof...(P) == sizeof...(A), "kernel argument count");
    if (grid == 0) return;
    if (!g) {
      k<<<grid, block, smem, st>>>(args...);
      return;
    }
    if (err != cudaSuccess) return;
    std::tuple<P...> vals(args...);
    add_node((void *)k, grid, block, smem, vals, std::index_sequence_for<P...>{});
  }

 private:
  template <class Tup, size_t... I>
  void add_node(void *fn, unsigned grid, unsigned block, size_t smem, Tup &vals, std::index_sequence<I...>) {
    void *ptrs[sizeof...(I) > 0 ? sizeof...(I) : 1] = {(void *)&std::get<I>(vals)...};
    cudaKernelNodeParams p = {};
    p.func = fn;
    p.gridDim = dim3(grid);
    p.blockDim = dim3(block);
    p.sharedMemBytes = (unsigned)smem;
    p.kernelParams = ptrs;
    p.extra = nullptr;
    cudaGraphNode_t n = nullptr;
    err = cudaGraphAddKernelNode(&n, g, last ? &last : nullptr, last ? 1 : 0, &p);
    if (err == cudaSuccess) last = n;
  }
};

}  // namespace tdy
