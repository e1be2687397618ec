// scan.cuh -- deterministic exclusive prefix sum over int64 (three-phase block scan).
#pragma once

#include "gfe_internal.cuh"

namespace gfe {
// internal linkage: every translation unit that includes this header gets its own kernels
namespace {

constexpr int kScanBlock = 1024;
constexpr int kScanItems = 4;  // items per thread
constexpr int kScanTile = kScanBlock * kScanItems;

__device__ __forceinline__ long long warp_incl_scan(long long v) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    long long t = __shfl_up_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) >= o) v += t;
  }
  return v;
}

// Block-wide exclusive scan of one value per thread; returns the exclusive prefix and the total.
__device__ __forceinline__ long long block_excl_scan(long long v, long long* total) {
  // blockDim.x must be a multiple of 32 (all launches here use 1024).
  __shared__ long long warp_tot[32];
  __shared__ long long block_tot;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  long long inc = warp_incl_scan(v);
  if (lane == 31) warp_tot[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    long long w = lane < nw ? warp_tot[lane] : 0;
    long long wi = warp_incl_scan(w);
    if (lane < nw) warp_tot[lane] = wi - w;
    if (lane == 31) block_tot = wi;
  }
  __syncthreads();
  long long res = inc - v + warp_tot[wid];
  *total = block_tot;
  __syncthreads();
  return res;
}

template <typename TIn>
__global__ void scan_tiles_kernel(const TIn* __restrict__ in, long long n, long long* __restrict__ out,
                                  long long* __restrict__ tile_sums) {
  const long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanItems;
  long long v[kScanItems];
  long long s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    v[i] = (base + i < n) ? (long long)in[base + i] : 0;
    s += v[i];
  }
  long long tot;
  long long pre = block_excl_scan(s, &tot);
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    if (base + i < n) out[base + i] = pre;
    pre += v[i];
  }
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = tot;
}

// Single-block exclusive scan of the tile sums (sequential over chunks of the block size).
__global__ void scan_sums_kernel(long long* sums, long long n, long long* grand_total) {
  long long carry = 0;
  for (long long base = 0; base < n; base += blockDim.x) {
    long long i = base + threadIdx.x;
    long long v = i < n ? sums[i] : 0;
    long long tot;
    long long pre = block_excl_scan(v, &tot);
    if (i < n) sums[i] = pre + carry;
    carry += tot;
  }
  if (threadIdx.x == 0 && grand_total) *grand_total = carry;
}

__global__ void scan_add_kernel(long long* out, long long n, const long long* __restrict__ tile_sums) {
  const long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanItems;
  const long long add = tile_sums[blockIdx.x];
#pragma unroll
  for (int i = 0; i < kScanItems; ++i)
    if (base + i < n) out[base + i] += add;
}

// out[i] = sum_{j<i} in[j] for i < n; *total_dev = sum of all.  Scratch from the stream pool.
template <typename TIn>
int exclusive_scan(const TIn* in, long long n, long long* out, long long* total_dev, cudaStream_t s) {
  long long tiles = (n + kScanTile - 1) / kScanTile;
  if (tiles < 1) tiles = 1;
  long long* sums = nullptr;
  int rc = scratch_alloc((void**)&sums, sizeof(long long) * tiles, s, "scan tile sums");
  if (rc) return rc;
  if (n > 0) scan_tiles_kernel<TIn><<<(unsigned)tiles, kScanBlock, 0, s>>>(in, n, out, sums);
  else cudaMemsetAsync(sums, 0, sizeof(long long), s);
  scan_sums_kernel<<<1, kScanBlock, 0, s>>>(sums, tiles, total_dev);
  if (n > 0) scan_add_kernel<<<(unsigned)tiles, kScanBlock, 0, s>>>(out, n, sums);
  scratch_free(sums, s);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(GFE_ERR_CUDA, "scan launch failed: %s", cudaGetErrorString(e));
  return GFE_OK;
}

}  // namespace
}  // namespace gfe
