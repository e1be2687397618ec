// structure.cu -- K3: Iron-identical compressed-row sparsity structure on the GPU.
//
// Iron (src/equations_matrices_routines.F90:4399-4457) builds, for each local row DOF, a list of
// every DOF of every component of every element surrounding the row DOF's node, then sorts it
// ascending and removes duplicates (src/lists.F90:2652-2700), and stores rows 1-based.  Here the
// "surrounding elements" of a DOF are the elements whose DOF list contains it, which is the same
// set for node-based fields.  One warp per row gathers the candidate columns into shared memory,
// bitonic-sorts them and counts / writes the unique values; a count pass and a fill pass bracket
// one exclusive scan.  The result is independent of thread scheduling.
#include "scan.cuh"

namespace {

constexpr int kWarpsPerBlock = 4;
constexpr int kMaxCand = 2048;  // candidates per row (8 elements x 89 DOFs = 712 for Q2/Q1 u-p)

__global__ void count_dof_elements(const int32_t* __restrict__ elem_dofs, long long total, int32_t n_dofs,
                                   int32_t* __restrict__ cnt, unsigned* err) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    int d = elem_dofs[i];
    if (d < 0 || d >= n_dofs) { gfe_raise(err, GFE_DEVERR_SLOT); continue; }
    atomicAdd(&cnt[d], 1);
  }
}

__global__ void fill_dof_elements(const int32_t* __restrict__ elem_dofs, int32_t n_elem, int32_t ndpe,
                                  int32_t n_dofs, const long long* __restrict__ adj_ptr, int32_t* __restrict__ fillc,
                                  int32_t* __restrict__ adj) {
  const long long total = (long long)n_elem * ndpe;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    int d = elem_dofs[i];
    if (d < 0 || d >= n_dofs) continue;
    int e = (int)(i / ndpe);
    int pos = atomicAdd(&fillc[d], 1);
    adj[adj_ptr[d] + pos] = e;
  }
}

// Warp-cooperative bitonic sort of buf[0..P) ascending (P a power of two, P >= 32).
__device__ __forceinline__ void warp_bitonic_sort(int32_t* buf, int P) {
  const int lane = threadIdx.x & 31;
  for (int k = 2; k <= P; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = lane; i < P; i += 32) {
        int ixj = i ^ j;
        if (ixj > i) {
          int32_t a = buf[i], b = buf[ixj];
          bool up = (i & k) == 0;
          if ((a > b) == up) { buf[i] = b; buf[ixj] = a; }
        }
      }
      __syncwarp();
    }
  }
}

// mode 0: count unique columns per row into row_cnt; mode 1: write them (1-based) at row_ptr.
template <int MODE>
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
row_columns(const int32_t* __restrict__ elem_dofs, int32_t ndpe, int32_t n_dofs,
            const long long* __restrict__ adj_ptr, const int32_t* __restrict__ adj,
            int32_t* __restrict__ row_cnt, const int32_t* __restrict__ row_ptr, int32_t* __restrict__ col_idx,
            long long col_capacity, unsigned* err) {
  __shared__ int32_t sbuf[kWarpsPerBlock][kMaxCand];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int32_t* buf = sbuf[w];
  for (long long r = (long long)blockIdx.x * kWarpsPerBlock + w; r < n_dofs;
       r += (long long)gridDim.x * kWarpsPerBlock) {
    const long long a0 = adj_ptr[r], a1 = adj_ptr[r + 1];
    const long long ncand = (a1 - a0) * ndpe;
    if (ncand > kMaxCand) {
      if (lane == 0) {
        gfe_raise(err, GFE_DEVERR_SLOT);
        if (MODE == 0) row_cnt[r] = 0;
      }
      continue;
    }
    int P = 32;
    while (P < ncand) P <<= 1;
    for (int i = lane; i < P; i += 32) {
      int32_t v = 0x7fffffff;
      if (i < ncand) {
        long long ea = a0 + i / ndpe;
        v = elem_dofs[(long long)adj[ea] * ndpe + (i % ndpe)];
      }
      buf[i] = v;
    }
    __syncwarp();
    warp_bitonic_sort(buf, P);
    // unique: position i is a head if i == 0 or buf[i] != buf[i-1]
    int base = 0;
    const int out0 = MODE == 1 ? row_ptr[r] - 1 : 0;
    for (int c = 0; c < ncand; c += 32) {
      int i = c + lane;
      bool head = i < ncand && (i == 0 || buf[i] != buf[i - 1]);
      unsigned m = __ballot_sync(0xffffffffu, head);
      if (MODE == 1 && head) {
        long long pos = (long long)out0 + base + __popc(m & ((1u << lane) - 1u));
        if (pos < col_capacity) col_idx[pos] = buf[i] + 1;
        else gfe_raise(err, GFE_DEVERR_SLOT);
      }
      base += __popc(m);
    }
    if (MODE == 0 && lane == 0) row_cnt[r] = base;
    __syncwarp();
  }
}

__global__ void finish_row_ptr(const long long* __restrict__ excl, int32_t n, long long total,
                               int32_t* __restrict__ row_ptr) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i <= n; i += (long long)gridDim.x * blockDim.x)
    row_ptr[i] = (int32_t)((i < n ? excl[i] : total) + 1);
}

}  // namespace

extern "C" int gfe_csr_structure(int32_t n_elem, int32_t ndpe, const int32_t* elem_dofs, int32_t n_dofs,
                                 int32_t* row_ptr, int32_t* col_idx, int64_t col_capacity, int64_t* nnz_host,
                                 void* stream) {
  using namespace gfe;
  if (n_elem < 0 || ndpe <= 0 || n_dofs <= 0 || !row_ptr || !nnz_host || (n_elem > 0 && !elem_dofs))
    return set_error(GFE_ERR_ARG, "gfe_csr_structure: invalid arguments (n_elem=%d ndpe=%d n_dofs=%d)", n_elem,
                     ndpe, n_dofs);
  cudaStream_t s = as_stream(stream);
  unsigned* err = device_error_word();
  const long long total = (long long)n_elem * ndpe;
  if (total >= (1ll << 31)) return set_error(GFE_ERR_ARG, "gfe_csr_structure: element DOF lists exceed 2^31 entries");
  int32_t *cnt = nullptr, *fillc = nullptr, *adj = nullptr, *row_cnt = nullptr;
  long long *adj_ptr = nullptr, *excl = nullptr, *tot_dev = nullptr;
  int rc = GFE_OK;
  const int grid = 4 * sm_count();
  if ((rc = scratch_alloc((void**)&cnt, sizeof(int32_t) * n_dofs, s, "dof element counts"))) goto done;
  if ((rc = scratch_alloc((void**)&fillc, sizeof(int32_t) * n_dofs, s, "dof element fill"))) goto done;
  if ((rc = scratch_alloc((void**)&adj_ptr, sizeof(long long) * (n_dofs + 1), s, "dof element offsets"))) goto done;
  if ((rc = scratch_alloc((void**)&adj, sizeof(int32_t) * (total > 0 ? total : 1), s, "dof element lists"))) goto done;
  if ((rc = scratch_alloc((void**)&row_cnt, sizeof(int32_t) * n_dofs, s, "row counts"))) goto done;
  if ((rc = scratch_alloc((void**)&excl, sizeof(long long) * n_dofs, s, "row offsets"))) goto done;
  if ((rc = scratch_alloc((void**)&tot_dev, sizeof(long long) * 2, s, "totals"))) goto done;
  cudaMemsetAsync(cnt, 0, sizeof(int32_t) * n_dofs, s);
  cudaMemsetAsync(fillc, 0, sizeof(int32_t) * n_dofs, s);
  if (total > 0) count_dof_elements<<<grid, 256, 0, s>>>(elem_dofs, total, n_dofs, cnt, err);
  if ((rc = exclusive_scan(cnt, n_dofs, adj_ptr, tot_dev, s))) goto done;
  cudaMemcpyAsync(adj_ptr + n_dofs, tot_dev, sizeof(long long), cudaMemcpyDeviceToDevice, s);
  if (total > 0) fill_dof_elements<<<grid, 256, 0, s>>>(elem_dofs, n_elem, ndpe, n_dofs, adj_ptr, fillc, adj);
  row_columns<0><<<grid, kWarpsPerBlock * 32, 0, s>>>(elem_dofs, ndpe, n_dofs, adj_ptr, adj, row_cnt, nullptr,
                                                        nullptr, 0, err);
  if ((rc = exclusive_scan(row_cnt, n_dofs, excl, tot_dev + 1, s))) goto done;
  {
    long long nnz = 0;
    cudaError_t e = cudaMemcpyAsync(&nnz, tot_dev + 1, sizeof(long long), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { rc = set_error(GFE_ERR_CUDA, "gfe_csr_structure: %s", cudaGetErrorString(e)); goto done; }
    if (nnz >= (1ll << 31) - 1) {
      rc = set_error(GFE_ERR_ARG, "gfe_csr_structure: %lld non-zeros exceed the int32 CSR index range", nnz);
      goto done;
    }
    *nnz_host = nnz;
    finish_row_ptr<<<grid, 256, 0, s>>>(excl, n_dofs, nnz, row_ptr);
    if (col_idx) {
      if (col_capacity < nnz) {
        rc = set_error(GFE_ERR_ARG, "gfe_csr_structure: col_capacity %lld < nnz %lld", (long long)col_capacity, nnz);
        goto done;
      }
      row_columns<1><<<grid, kWarpsPerBlock * 32, 0, s>>>(elem_dofs, ndpe, n_dofs, adj_ptr, adj, nullptr, row_ptr,
                                                            col_idx, col_capacity, err);
    }
  }
  {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) rc = set_error(GFE_ERR_CUDA, "gfe_csr_structure: launch failed: %s", cudaGetErrorString(e));
  }
done:
  scratch_free(cnt, s);
  scratch_free(fillc, s);
  scratch_free(adj_ptr, s);
  scratch_free(adj, s);
  scratch_free(row_cnt, s);
  scratch_free(excl, s);
  scratch_free(tot_dev, s);
  if (rc == GFE_OK) {
    unsigned bits = 0;
    cudaError_t e = cudaMemcpyAsync(&bits, err, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return set_error(GFE_ERR_CUDA, "gfe_csr_structure: %s", cudaGetErrorString(e));
    if (bits & GFE_DEVERR_SLOT) {
      cudaMemsetAsync(err, 0, sizeof(unsigned), s);
      return set_error(GFE_ERR_STRUCTURE,
                       "gfe_csr_structure: a DOF number is out of range or a row has more than %d candidate columns",
                       kMaxCand);
    }
  }
  return rc;
}
