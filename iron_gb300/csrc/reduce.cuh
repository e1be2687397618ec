// reduce.cuh -- deterministic grid-wide reductions shared by the Krylov solvers.
//
// Each block reduces its threads' values to one partial (warp shuffles, then warp totals in
// order), writes it to red[blockIdx.x], and the last block to arrive (an atomic ticket) adds the
// partials in index order.  The result therefore does not depend on block scheduling, so a solve
// repeated on the same input gives bit-identical iterates.
#pragma once

#include <cstdint>

namespace gfe_red {

constexpr int kThreads = 256;

// Sum of one double per thread of a kThreads-wide block; valid in thread 0.
__device__ __forceinline__ double block_sum(double v) {
  __shared__ double sh[kThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < kThreads / 32; ++i) s += sh[i];
  __syncthreads();
  return s;
}

// True in every thread of the last block to take a ticket; the partials written by all earlier
// blocks are visible to it.
__device__ __forceinline__ bool last_block(int* ticket) {
  __shared__ bool amlast;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    int t = atomicAdd(ticket, 1);
    amlast = (t == (int)gridDim.x - 1);
  }
  __syncthreads();
  return amlast;
}

// Sum red[0..n) in index order using the whole block; result valid in thread 0.
__device__ __forceinline__ double ordered_sum(const double* red, int n) {
  __shared__ double sh[kThreads];
  const int per = (n + kThreads - 1) / kThreads;
  double s = 0.0;
  const int i0 = threadIdx.x * per;
  for (int i = i0; i < i0 + per && i < n; ++i) s += __ldcg(red + i);
  sh[threadIdx.x] = s;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < kThreads; ++i) t += sh[i];
  __syncthreads();
  return t;
}

}  // namespace gfe_red
