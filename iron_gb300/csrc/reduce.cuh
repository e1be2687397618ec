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

// Sum of one value per thread of a kThreads-wide block, in double; valid in thread 0.  The warp
// stage runs in the threads' own type (FP32 partials of the FP32 Krylov vectors stay off the FP64
// pipe), the warp totals are added in FP64 in warp order.
template <typename T>
__device__ __forceinline__ double block_sum(T v) {
  __shared__ double sh[kThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = (double)v;
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

// Sum red[0..n) in a fixed order using the whole block: each thread adds a contiguous run of
// partials, then the runs are combined by the same fixed-shape tree as block_sum.  A serial sum of
// the 256 runs by one thread would be 256 dependent FP64 adds: at one FP64 warp instruction every
// 64 cycles per scheduler, about 8 us per reduction, several times per Krylov iteration.  Result
// valid in thread 0.
__device__ __forceinline__ double ordered_sum(const double* red, int n) {
  const int per = (n + kThreads - 1) / kThreads;
  double s = 0.0;
  const int i0 = threadIdx.x * per;
  for (int i = i0; i < i0 + per && i < n; ++i) s += __ldcg(red + i);
  return block_sum(s);
}

}  // namespace gfe_red
