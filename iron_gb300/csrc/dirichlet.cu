// dirichlet.cu -- the solver system of a linear equations set with Dirichlet conditions.
//
// Iron hands PETSc a reduced system: the rows and columns of fixed DOFs removed, their coupling
// moved to the right-hand side (SOLVER_MATRICES_STATIC_ASSEMBLE, src/solver_routines.F90:
// 14025-15050; SOLVER_MATRIX_EQUATIONS_MATRIX_ADD, src/solver_matrices_routines.F90:806-1023;
// SOLVER_MATRIX_STRUCTURE_CALCULATE, :1612-2431; the solver mapping,
// src/solver_mapping_routines.F90:398-520).  For one equations set on one rank:
//  * solver rows and columns are the free DOFs, numbered in ascending order (one scan);
//  * each solver row holds the equations row's free columns, renumbered -- still ascending, so
//    Iron's sort + unique of the mapped columns is a stable compaction (warp ballots);
//  * each solver value is 0 + K(i, j): the zeroed solver matrix receives every free-free entry once;
//  * the solver RHS of free row i accumulates, in ascending order of the equations row r that
//    contributes, f(i) (at r = i) and -1 * K(i, r) * u(r) for each fixed column r with
//    |u(r)| >= ZERO_TOLERANCE and |K(i, r)| >= ZERO_TOLERANCE.  One warp walks row i's columns in
//    ascending order and adds the terms in exactly that order, with rounded products (no fused
//    multiply-add), so the result is bit-identical to Iron's.
#include <algorithm>

#include "gfe_internal.cuh"
#include "scan.cuh"

namespace {

constexpr double kZeroTol = 5.0 * 2.220446049250313e-16;  // ZERO_TOLERANCE_DP = 5 EPSILON(1.0_DP)
constexpr int kWarps = 8;                                  // warps per block of the row kernels
constexpr unsigned kFull = 0xffffffffu;

__global__ void free_flags(int32_t n, const uint8_t* __restrict__ fixed, int32_t* __restrict__ flag) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    flag[i] = fixed[i] ? 0 : 1;
}

__global__ void finish_dof_map(int32_t n, const uint8_t* __restrict__ fixed, const long long* __restrict__ excl,
                               int32_t* __restrict__ solver_of_dof) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    solver_of_dof[i] = fixed[i] ? -1 : (int32_t)excl[i];
}

// rows [.., n_free] of the solver CSR from the exclusive scan of the row counts (1-based)
__global__ void finish_solver_row_ptr(int32_t n_free, const long long* __restrict__ excl, long long total,
                                      int32_t* __restrict__ s_row_ptr) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i <= n_free;
       i += (long long)gridDim.x * blockDim.x)
    s_row_ptr[i] = (int32_t)((i < n_free ? excl[i] : total) + 1);
}

// One warp per equations row; free rows only.  MODE 0: count the free columns into s_cnt[solver
// row].  MODE 1: write them at s_row_ptr (1-based solver columns into s_col_idx when given, the
// values 0 + K into s_values and their FP32 roundings into s_values32 when given), in the
// equations row's (ascending) order.
template <int MODE>
__global__ void __launch_bounds__(kWarps * 32)
solver_rows(int32_t n, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
            const int32_t* __restrict__ solver_of_dof, int32_t* __restrict__ s_cnt,
            const int32_t* __restrict__ s_row_ptr, int32_t* __restrict__ s_col_idx, const double* __restrict__ values,
            double* __restrict__ s_values, float* __restrict__ s_values32, unsigned* err) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * kWarps;
  for (long long r = blockIdx.x * (long long)kWarps + threadIdx.x / 32; r < n; r += warps) {
    const int32_t sr = solver_of_dof[r];
    if (sr < 0) continue;  // uniform across the warp
    const long long lo = (long long)rp[r] - 1, hi = (long long)rp[r + 1] - 1;
    long long base = MODE == 1 ? (long long)s_row_ptr[sr] - 1 : 0;
    int count = 0;
    for (long long k0 = lo; k0 < hi; k0 += 32) {
      const long long k = k0 + lane;
      int32_t sc = -1;
      if (k < hi) {
        const int32_t c = ci[k] - 1;
        if (c < 0 || c >= n) gfe_raise(err, GFE_DEVERR_SLOT);
        else sc = solver_of_dof[c];
      }
      const unsigned m = __ballot_sync(kFull, sc >= 0);
      if (MODE == 1 && sc >= 0) {
        const long long pos = base + count + __popc(m & ((1u << lane) - 1u));
        if (s_col_idx) s_col_idx[pos] = sc + 1;
        if (s_values || s_values32) {
          const double v = __dadd_rn(0.0, values[k]);
          if (s_values) s_values[pos] = v;
          if (s_values32) s_values32[pos] = (float)v;
        }
      }
      count += __popc(m);
    }
    if (MODE == 0 && lane == 0) s_cnt[sr] = count;
  }
}

// One warp per free equations row: the solver right-hand side in Iron's accumulation order.
__global__ void __launch_bounds__(kWarps * 32)
solver_rhs_rows(int32_t n, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                const double* __restrict__ values, const double* __restrict__ f, const double* __restrict__ u,
                const uint8_t* __restrict__ fixed, const uint8_t* __restrict__ col_listed,
                const int32_t* __restrict__ solver_of_dof, double* __restrict__ s_rhs, unsigned* err) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * kWarps;
  for (long long r = blockIdx.x * (long long)kWarps + threadIdx.x / 32; r < n; r += warps) {
    const int32_t sr = solver_of_dof[r];
    if (sr < 0) continue;  // uniform across the warp
    const long long lo = (long long)rp[r] - 1, hi = (long long)rp[r + 1] - 1;
    const double fr = f ? f[r] : 0.0;
    bool f_done = f == nullptr;  // a zero equations RHS adds nothing
    double s = 0.0;              // identical in every lane
    for (long long k0 = lo; k0 < hi; k0 += 32) {
      const long long k = k0 + lane;
      bool has = false, at_f = false;
      double t = 0.0;
      if (k < hi) {
        const int32_t c = ci[k] - 1;
        if (c < 0 || c >= n) {
          gfe_raise(err, GFE_DEVERR_SLOT);
        } else {
          // f(r) enters when the contributing equations row reaches r: before the first column >= r
          at_f = !f_done && c >= r && (k == lo || ci[k - 1] - 1 < r);
          if (fixed[c] && (!col_listed || col_listed[c])) {
            const double uc = u[c], kv = values[k];
            if (fabs(uc) >= kZeroTol && fabs(kv) >= kZeroTol) {
              has = true;
              t = __dmul_rn(__dmul_rn(-1.0, kv), uc);
            }
          }
        }
      }
      const unsigned mh = __ballot_sync(kFull, has), mf = __ballot_sync(kFull, at_f);
      unsigned mm = mh | mf;
      while (mm) {  // ascending lanes = ascending columns
        const int l = __ffs(mm) - 1;
        mm &= mm - 1;
        if ((mf >> l) & 1u) {
          s = __dadd_rn(s, fr);
          f_done = true;
        }
        const double tl = __shfl_sync(kFull, t, l);
        if ((mh >> l) & 1u) s = __dadd_rn(s, tl);
      }
    }
    if (!f_done) s = __dadd_rn(s, fr);
    if (lane == 0) s_rhs[sr] = s;
  }
}

__global__ void update_dependent(int32_t n, const int32_t* __restrict__ solver_of_dof, const double* __restrict__ x,
                                 double* __restrict__ u) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int32_t sr = solver_of_dof[i];
    if (sr >= 0) u[i] = x[sr];
  }
}

int row_grid(int32_t n) {
  const long long want = ((long long)n + kWarps - 1) / kWarps;
  return (int)std::min<long long>(want > 0 ? want : 1, 16ll * gfe::sm_count());
}

int check_csr(int32_t n, const int32_t* row_ptr, const int32_t* col_idx, const char* fn) {
  if (n <= 0 || !row_ptr || !col_idx) return gfe::set_error(GFE_ERR_ARG, "%s: invalid CSR arguments (n=%d)", fn, n);
  return GFE_OK;
}

int report_device_errors(cudaStream_t s, const char* fn) {
  unsigned* err = gfe::device_error_word();
  unsigned bits = 0;
  cudaError_t e = cudaMemcpyAsync(&bits, err, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return gfe::set_error(GFE_ERR_CUDA, "%s: %s", fn, cudaGetErrorString(e));
  if (bits & GFE_DEVERR_SLOT) {
    cudaMemsetAsync(err, 0, sizeof(unsigned), s);
    return gfe::set_error(GFE_ERR_STRUCTURE, "%s: a column index lies outside [1, n]", fn);
  }
  return GFE_OK;
}

}  // namespace

extern "C" int gfe_solver_structure(int32_t n, const int32_t* row_ptr, const int32_t* col_idx, const uint8_t* fixed,
                                    int32_t* solver_of_dof, int32_t* s_row_ptr, int32_t* s_col_idx,
                                    int64_t col_capacity, int32_t* n_free_host, int64_t* nnz_host, void* stream) {
  using namespace gfe;
  const char* fn = "gfe_solver_structure";
  if (int rc = check_csr(n, row_ptr, col_idx, fn)) return rc;
  if (!fixed || !solver_of_dof || !s_row_ptr || !n_free_host || !nnz_host)
    return set_error(GFE_ERR_ARG, "%s: invalid arguments", fn);
  cudaStream_t s = as_stream(stream);
  unsigned* err = device_error_word();
  int32_t *flag = nullptr, *cnt = nullptr;
  long long *excl = nullptr, *tot = nullptr;
  int rc = GFE_OK;
  const int grid = 4 * sm_count();
  long long n_free = 0, nnz = 0;
  if ((rc = scratch_alloc((void**)&flag, sizeof(int32_t) * n, s, "free flags"))) goto done;
  if ((rc = scratch_alloc((void**)&excl, sizeof(long long) * n, s, "free DOF offsets"))) goto done;
  if ((rc = scratch_alloc((void**)&tot, sizeof(long long) * 2, s, "totals"))) goto done;
  free_flags<<<grid, 256, 0, s>>>(n, fixed, flag);
  if ((rc = exclusive_scan(flag, n, excl, tot, s))) goto done;
  finish_dof_map<<<grid, 256, 0, s>>>(n, fixed, excl, solver_of_dof);
  {
    cudaError_t e = cudaMemcpyAsync(&n_free, tot, sizeof(long long), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { rc = set_error(GFE_ERR_CUDA, "%s: %s", fn, cudaGetErrorString(e)); goto done; }
  }
  if (n_free > 0) {
    if ((rc = scratch_alloc((void**)&cnt, sizeof(int32_t) * n_free, s, "solver row counts"))) goto done;
    solver_rows<0><<<row_grid(n), kWarps * 32, 0, s>>>(n, row_ptr, col_idx, solver_of_dof, cnt, nullptr, nullptr,
                                                         nullptr, nullptr, nullptr, err);
    if ((rc = exclusive_scan(cnt, n_free, excl, tot + 1, s))) goto done;
    cudaError_t e = cudaMemcpyAsync(&nnz, tot + 1, sizeof(long long), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { rc = set_error(GFE_ERR_CUDA, "%s: %s", fn, cudaGetErrorString(e)); goto done; }
    if (nnz >= (1ll << 31) - 1) {
      rc = set_error(GFE_ERR_ARG, "%s: %lld non-zeros exceed the int32 CSR index range", fn, nnz);
      goto done;
    }
  }
  finish_solver_row_ptr<<<grid, 256, 0, s>>>((int32_t)n_free, excl, nnz, s_row_ptr);
  *n_free_host = (int32_t)n_free;
  *nnz_host = nnz;
  if (s_col_idx && n_free > 0) {
    if (col_capacity < nnz) {
      rc = set_error(GFE_ERR_ARG, "%s: col_capacity %lld < nnz %lld", fn, (long long)col_capacity, nnz);
      goto done;
    }
    solver_rows<1><<<row_grid(n), kWarps * 32, 0, s>>>(n, row_ptr, col_idx, solver_of_dof, nullptr, s_row_ptr,
                                                         s_col_idx, nullptr, nullptr, nullptr, err);
  }
  {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) rc = set_error(GFE_ERR_CUDA, "%s: launch failed: %s", fn, cudaGetErrorString(e));
  }
done:
  scratch_free(flag, s);
  scratch_free(cnt, s);
  scratch_free(excl, s);
  scratch_free(tot, s);
  if (rc == GFE_OK) rc = report_device_errors(s, fn);
  return rc;
}

extern "C" int gfe_solver_matrix(int32_t n, const int32_t* row_ptr, const int32_t* col_idx, const double* values,
                                 const int32_t* solver_of_dof, const int32_t* s_row_ptr, double* s_values,
                                 float* s_values32, void* stream) {
  const char* fn = "gfe_solver_matrix";
  if (int rc = check_csr(n, row_ptr, col_idx, fn)) return rc;
  if (!values || !solver_of_dof || !s_row_ptr || (!s_values && !s_values32))
    return gfe::set_error(GFE_ERR_ARG, "%s: invalid arguments", fn);
  cudaStream_t s = gfe::as_stream(stream);
  solver_rows<1><<<row_grid(n), kWarps * 32, 0, s>>>(n, row_ptr, col_idx, solver_of_dof, nullptr, s_row_ptr,
                                                       nullptr, values, s_values, s_values32,
                                                       gfe::device_error_word());
  GFE_LAUNCH_CHECK(fn);
  return GFE_OK;
}

extern "C" int gfe_solver_rhs(int32_t n, const int32_t* row_ptr, const int32_t* col_idx, const double* values,
                              const double* f, const double* u, const uint8_t* fixed, const uint8_t* col_listed,
                              const int32_t* solver_of_dof, double* s_rhs, void* stream) {
  const char* fn = "gfe_solver_rhs";
  if (int rc = check_csr(n, row_ptr, col_idx, fn)) return rc;
  if (!values || !u || !fixed || !solver_of_dof || !s_rhs)
    return gfe::set_error(GFE_ERR_ARG, "%s: invalid arguments", fn);
  cudaStream_t s = gfe::as_stream(stream);
  solver_rhs_rows<<<row_grid(n), kWarps * 32, 0, s>>>(n, row_ptr, col_idx, values, f, u, fixed, col_listed,
                                                        solver_of_dof, s_rhs, gfe::device_error_word());
  GFE_LAUNCH_CHECK(fn);
  return GFE_OK;
}

extern "C" int gfe_solver_update_dependent(int32_t n, const int32_t* solver_of_dof, const double* x, double* u,
                                           void* stream) {
  const char* fn = "gfe_solver_update_dependent";
  if (n <= 0 || !solver_of_dof || !x || !u) return gfe::set_error(GFE_ERR_ARG, "%s: invalid arguments", fn);
  cudaStream_t s = gfe::as_stream(stream);
  update_dependent<<<4 * gfe::sm_count(), 256, 0, s>>>(n, solver_of_dof, x, u);
  GFE_LAUNCH_CHECK(fn);
  return GFE_OK;
}
