// tdy_arena.h -- one device allocation for many arrays.
//
// A handle (and its solver) keeps dozens of device arrays.  Allocated one by
// one, with one upload call each, their set-up takes about a hundred driver
// calls; when many threads set up handles at once (a server), every one of
// them waits on the others.  An Arena gathers the arrays first, then makes
// them 256-byte aligned ranges of a single stream-ordered allocation, and
// copies the host data of all uploaded arrays with one call from a packed
// staging buffer (per-array copies above kPackLimit bytes, to spare a second
// host copy of very large set-ups).
#pragma once

#include <cuda_runtime.h>

#include <cstring>
#include <type_traits>
#include <vector>

#include "tdy_device.h"

namespace tdy {

struct Arena {
  static constexpr size_t kPackLimit = 256u << 20;
  struct Item {
    void **dst;
    size_t bytes;
    const void *src;  // null: not uploaded
    size_t off;
  };
  std::vector<Item> items;
  std::vector<char> staging;  // must live until the stream is synchronised
  void *base = nullptr;
  size_t total = 0;

  // an array uploaded from v (v must stay alive until commit returns)
  template <class P, class T>
  void up(P **dst, const std::vector<T> &v) {
    items.push_back({slot(dst), v.size() * sizeof(T), v.empty() ? nullptr : v.data(), 0});
  }
  // an array of n elements left uninitialised
  template <class P>
  void work(P **dst, size_t n) {
    items.push_back({slot(dst), n * sizeof(P), nullptr, 0});
  }
  // the pointer variable to set (pointers to const elements included)
  template <class P>
  static void **slot(P **dst) {
    return reinterpret_cast<void **>(const_cast<typename std::remove_const<P>::type **>(dst));
  }

  // Allocates the block on `st`, sets every registered pointer and enqueues
  // the uploads; the caller synchronises `st` before other streams use the
  // arrays and releases `base` with dmem_free.
  int commit(cudaStream_t st) {
    size_t off = 0, up_end = 0;
    auto place = [&](Item &it) {
      off = (off + 255) & ~size_t(255);
      it.off = off;
      off += it.bytes ? it.bytes : 1;
    };
    for (Item &it : items)
      if (it.src) place(it);
    up_end = off;
    for (Item &it : items)
      if (!it.src) place(it);
    total = off;
    int ierr = dmem_alloc(&base, total ? total : 1, st);
    if (ierr) return ierr;
    char *b = static_cast<char *>(base);
    for (Item &it : items) *it.dst = b + it.off;
    if (up_end == 0) return 0;
    cudaError_t e = cudaSuccess;
    if (up_end <= kPackLimit) {
      staging.assign(up_end, 0);
      for (const Item &it : items)
        if (it.src) std::memcpy(staging.data() + it.off, it.src, it.bytes);
      e = cudaMemcpyAsync(base, staging.data(), up_end, cudaMemcpyHostToDevice, st);
    } else {
      for (const Item &it : items)
        if (it.src && e == cudaSuccess) e = cudaMemcpyAsync(b + it.off, it.src, it.bytes, cudaMemcpyHostToDevice, st);
    }
    if (e != cudaSuccess) return set_error(TDY_ERR_GPU, "arena upload: %s", cudaGetErrorString(e));
    return 0;
  }
};

}  // namespace tdy
