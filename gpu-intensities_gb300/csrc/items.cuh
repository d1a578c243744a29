// Work-list lookup shared by the batched kernels (one launch over the items
// of a round or of a group of final blocks).
#pragma once

#include <cuda_runtime.h>

namespace gi {

// The item of grid block b: the last one whose first block is at most b.  The
// block loads the items' first blocks into shared memory in one round of
// loads and searches there (a search in global memory is a chain of
// dependent loads, microseconds per block).
constexpr int kItemsSmem = 1024;
// first(k): the first grid block of item k (first(0) = 0, non-decreasing).
template <class F>
__device__ __forceinline__ int find_item(int nitems, long long b, F first) {
  __shared__ long long s_first[kItemsSmem];
  __shared__ int s_item;
  if (nitems <= kItemsSmem) {
    for (int k = threadIdx.x; k < nitems; k += blockDim.x) s_first[k] = first(k);
    __syncthreads();
    if (threadIdx.x == 0) {
      int lo = 0, hi = nitems - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (s_first[mid] <= b) lo = mid;
        else hi = mid - 1;
      }
      s_item = lo;
    }
  } else if (threadIdx.x == 0) {
    int lo = 0, hi = nitems - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (first(mid) <= b) lo = mid;
      else hi = mid - 1;
    }
    s_item = lo;
  }
  __syncthreads();
  return s_item;
}

}  // namespace gi
