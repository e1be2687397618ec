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

// ------------------------------------------------------------------------------------------------
// Closed-form structure of Iron's regular generated Q2/Q1 mesh
// ------------------------------------------------------------------------------------------------
// On the regular mesh of nx x ny x nz triquadratic elements (displacement DOFs of the three
// components on the (2n+1)^3 node grid, then the pressure DOFs on the (n+1)^3 vertex grid, both
// numbered xi1 fastest) the elements around a DOF's node, and therefore the row's columns, are
// boxes: along an axis a vertex node i (even) lies in elements i/2-1 and i/2, a mid node (odd) in
// (i-1)/2 only, so the row holds the displacement nodes [i-2, i+2] resp. [i-1, i+1] and the
// pressure nodes [i/2-1, i/2+1] resp. [(i-1)/2, (i+1)/2], clipped to the mesh; a pressure row at
// vertex I holds the displacement nodes [2I-2, 2I+2] and pressure nodes [I-1, I+1].  Every row is
// three displacement boxes (one per component block) followed by one pressure box, already in
// ascending column order: the same structure that gfe_csr_structure sorts and deduplicates from
// the element DOF lists (JacobianMatrix_StructureCalculate), without the per-row sort.
namespace {

struct Box {
  int q0[3], q1[3];  // displacement node range per axis (inclusive)
  int p0[3], p1[3];  // pressure node range per axis (inclusive)
};

__device__ __forceinline__ Box mr_row_box(long long r, int nx, int ny, int nz, long long nq2) {
  const int ne[3] = {nx, ny, nz};
  Box b;
  if (r < 3 * nq2) {
    long long node = r % nq2;
    const int tq[3] = {2 * nx + 1, 2 * ny + 1, 2 * nz + 1};
    int c[3];
    c[0] = (int)(node % tq[0]);
    node /= tq[0];
    c[1] = (int)(node % tq[1]);
    c[2] = (int)(node / tq[1]);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      if ((c[a] & 1) == 0) {
        b.q0[a] = max(c[a] - 2, 0);
        b.q1[a] = min(c[a] + 2, 2 * ne[a]);
        b.p0[a] = max(c[a] / 2 - 1, 0);
        b.p1[a] = min(c[a] / 2 + 1, ne[a]);
      } else {
        b.q0[a] = c[a] - 1;
        b.q1[a] = c[a] + 1;
        b.p0[a] = (c[a] - 1) / 2;
        b.p1[a] = (c[a] + 1) / 2;
      }
    }
  } else {
    long long node = r - 3 * nq2;
    const int tl[3] = {nx + 1, ny + 1, nz + 1};
    int c[3];
    c[0] = (int)(node % tl[0]);
    node /= tl[0];
    c[1] = (int)(node % tl[1]);
    c[2] = (int)(node / tl[1]);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      b.q0[a] = max(2 * c[a] - 2, 0);
      b.q1[a] = min(2 * c[a] + 2, 2 * ne[a]);
      b.p0[a] = max(c[a] - 1, 0);
      b.p1[a] = min(c[a] + 1, ne[a]);
    }
  }
  return b;
}

__global__ void mr_regular_row_counts(int nx, int ny, int nz, long long n_rows, long long nq2,
                                      int32_t* __restrict__ cnt) {
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n_rows;
       r += (long long)gridDim.x * blockDim.x) {
    const Box b = mr_row_box(r, nx, ny, nz, nq2);
    const int nq = (b.q1[0] - b.q0[0] + 1) * (b.q1[1] - b.q0[1] + 1) * (b.q1[2] - b.q0[2] + 1);
    const int np = (b.p1[0] - b.p0[0] + 1) * (b.p1[1] - b.p0[1] + 1) * (b.p1[2] - b.p0[2] + 1);
    cnt[r] = 3 * nq + np;
  }
}

// one warp per row: column k of the row decoded from the boxes, written 1-based
__global__ void mr_regular_row_columns(int nx, int ny, int nz, long long n_rows, long long nq2,
                                       const int32_t* __restrict__ row_ptr, int32_t* __restrict__ col_idx) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (blockDim.x / 32);
  const int tq0 = 2 * nx + 1, tq1 = 2 * ny + 1, tl0 = nx + 1, tl1 = ny + 1;
  for (long long r = blockIdx.x * (long long)(blockDim.x / 32) + threadIdx.x / 32; r < n_rows; r += warps) {
    const Box b = mr_row_box(r, nx, ny, nz, nq2);
    const int qx = b.q1[0] - b.q0[0] + 1, qy = b.q1[1] - b.q0[1] + 1, qz = b.q1[2] - b.q0[2] + 1;
    const int px = b.p1[0] - b.p0[0] + 1, py = b.p1[1] - b.p0[1] + 1, pz = b.p1[2] - b.p0[2] + 1;
    const int nq = qx * qy * qz, len = 3 * nq + px * py * pz;
    const long long out = (long long)row_ptr[r] - 1;
    for (int k = lane; k < len; k += 32) {
      long long col;
      if (k < 3 * nq) {
        const int comp = k / nq, t = k % nq;
        const int i = b.q0[0] + t % qx, j = b.q0[1] + (t / qx) % qy, kk = b.q0[2] + t / (qx * qy);
        col = comp * nq2 + i + (long long)tq0 * (j + (long long)tq1 * kk);
      } else {
        const int t = k - 3 * nq;
        const int i = b.p0[0] + t % px, j = b.p0[1] + (t / px) % py, kk = b.p0[2] + t / (px * py);
        col = 3 * nq2 + i + (long long)tl0 * (j + (long long)tl1 * kk);
      }
      col_idx[out + k] = (int32_t)(col + 1);
    }
  }
}

}  // namespace

extern "C" int gfe_mr_regular_structure(int32_t nx, int32_t ny, int32_t nz, int32_t* row_ptr, int32_t* col_idx,
                                        int64_t col_capacity, int64_t* nnz_host, void* stream) {
  using namespace gfe;
  const char* fn = "gfe_mr_regular_structure";
  if (nx <= 0 || ny <= 0 || nz <= 0 || !row_ptr || !nnz_host)
    return set_error(GFE_ERR_ARG, "%s: invalid arguments", fn);
  const long long nq2 = (2ll * nx + 1) * (2ll * ny + 1) * (2ll * nz + 1);
  const long long n_rows = 3 * nq2 + (nx + 1ll) * (ny + 1ll) * (nz + 1ll);
  if (n_rows >= (1ll << 31)) return set_error(GFE_ERR_ARG, "%s: %lld rows exceed the int32 index range", fn, n_rows);
  cudaStream_t s = as_stream(stream);
  int32_t* cnt = nullptr;
  long long *excl = nullptr, *tot = nullptr;
  int rc = GFE_OK;
  long long nnz = 0;
  const int grid = 4 * sm_count();
  if ((rc = scratch_alloc((void**)&cnt, sizeof(int32_t) * n_rows, s, "row counts"))) goto done;
  if ((rc = scratch_alloc((void**)&excl, sizeof(long long) * n_rows, s, "row offsets"))) goto done;
  if ((rc = scratch_alloc((void**)&tot, sizeof(long long), s, "total"))) goto done;
  mr_regular_row_counts<<<grid, 256, 0, s>>>(nx, ny, nz, n_rows, nq2, cnt);
  if ((rc = exclusive_scan(cnt, n_rows, excl, tot, s))) goto done;
  {
    cudaError_t e = cudaMemcpyAsync(&nnz, tot, sizeof(long long), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { rc = set_error(GFE_ERR_CUDA, "%s: %s", fn, cudaGetErrorString(e)); goto done; }
  }
  if (nnz >= (1ll << 31) - 1) {
    rc = set_error(GFE_ERR_ARG, "%s: %lld non-zeros exceed the int32 CSR index range", fn, nnz);
    goto done;
  }
  *nnz_host = nnz;
  finish_row_ptr<<<grid, 256, 0, s>>>(excl, (int32_t)n_rows, nnz, row_ptr);
  if (col_idx) {
    if (col_capacity < nnz) {
      rc = set_error(GFE_ERR_ARG, "%s: col_capacity %lld < nnz %lld", fn, (long long)col_capacity, nnz);
      goto done;
    }
    mr_regular_row_columns<<<16 * sm_count(), 256, 0, s>>>(nx, ny, nz, n_rows, nq2, row_ptr, col_idx);
  }
  {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) rc = set_error(GFE_ERR_CUDA, "%s: launch failed: %s", fn, cudaGetErrorString(e));
  }
done:
  scratch_free(cnt, s);
  scratch_free(excl, s);
  scratch_free(tot, s);
  return rc;
}
