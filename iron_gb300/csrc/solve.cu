// solve.cu -- K7: CSR SpMV and Jacobi-preconditioned CG on the Dirichlet-eliminated system.
//
// Iron assembles the solver matrix by removing fixed DOFs (SOLVER_MATRICES_STATIC_ASSEMBLE,
// src/solver_routines.F90:14025-15050) and hands it to PETSc KSP with a Jacobi preconditioner by
// default (src/solver_routines.F90:11320-11369, 11775-11991).  Here the same system is solved in
// the full DOF index space: fixed rows of A p are zeroed and fixed entries of every search
// direction are zero, which is algebraically the eliminated system.
//
// All scalars of the iteration live on the device; one iteration is three kernels (SpMV + <p,q>,
// update + <r,z>, direction update).  Reductions are deterministic: each block writes a partial
// sum and the last block to finish (detected by an atomic ticket) adds the partials in index order.
// Kernels return immediately once the device-side `done` flag is set, so the host can launch
// iterations in chunks and synchronise only between chunks.
//
// Mixed precision (precision == GFE_MIXED with an FP32 copy of the matrix): iterative refinement.
// The outer loop forms r = f - A x in FP64 with the FP64 matrix and tests ||r|| against the target;
// the correction A d = r is solved by FP32 CG (FP32 matrix and vectors, FP64 dot products) to a
// loose relative tolerance and added to x in FP64.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

#include "gfe_internal.cuh"

namespace {

constexpr int kThreads = 256;

struct Scalars {
  double rz, pq, alpha, beta, rr, rr0, tol2;
  int done, it, ticket1, ticket2, bad;
};

// Deterministic block reduction of one double per thread into red[blockIdx.x]; returns true in
// thread 0 of the last block to arrive, after which red[0..nblk) are all visible.
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
  return s;  // valid in thread 0
}

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
  // each thread sums a contiguous chunk, then thread 0 sums the chunk totals in order
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

// q = A p on free rows (0 on fixed rows), partial <p, q>.  LPR lanes per row.  The arithmetic is
// done in the vector type TV: GB300's FP64 pipe issues a warp instruction in 64 cycles, so the FP64
// solve uses one thread per row (no shuffle reduction, no idle lanes in the FMA chain) and the FP32
// inner solve of the mixed scheme stays entirely on the FP32 pipe.
template <typename TM, typename TV, int LPR>
__global__ void __launch_bounds__(kThreads)
cg_spmv(int n, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci, const TM* __restrict__ val,
        const TV* __restrict__ p, TV* __restrict__ q, const uint8_t* __restrict__ fixed, double* red,
        Scalars* sc) {
  if (sc->done) return;
  constexpr int RPB = kThreads / LPR;  // rows per block-iteration
  const int sub = threadIdx.x % LPR, grp = threadIdx.x / LPR;
  TV dot = TV(0);
  // The loop bound is block-uniform so every lane of a warp executes the same shuffles; lanes
  // whose row is past the end contribute zero.
  for (int base = blockIdx.x * RPB; base < n; base += gridDim.x * RPB) {
    const int row = base + grp;
    const bool valid = row < n;
    const int k0 = valid ? __ldg(rp + row) - 1 : 0, k1 = valid ? __ldg(rp + row + 1) - 1 : 0;
    TV s = TV(0);
#pragma unroll 4
    for (int k = k0 + sub; k < k1; k += LPR) s += (TV)__ldg(val + k) * p[__ldg(ci + k) - 1];
#pragma unroll
    for (int o = LPR / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, LPR);
    if (valid && sub == 0) {
      if (fixed && fixed[row]) s = TV(0);
      q[row] = s;
      dot += p[row] * s;
    }
  }
  double b = block_sum((double)dot);
  if (threadIdx.x == 0) red[blockIdx.x] = b;
  if (last_block(&sc->ticket1)) {
    double pq = ordered_sum(red, gridDim.x);
    if (threadIdx.x == 0) {
      sc->pq = pq;
      sc->alpha = pq != 0.0 ? sc->rz / pq : 0.0;
      if (!(pq > 0.0) || !isfinite(pq)) { sc->bad = 1; sc->done = 1; }
      sc->ticket1 = 0;
    }
  }
}

// x += alpha p; r -= alpha q; z = dinv r; partial <r,z>, <r,r>; last block: beta, convergence.
template <typename TX, typename TV>
__global__ void __launch_bounds__(kThreads)
cg_update(int n, TX* __restrict__ x, TV* __restrict__ r, TV* __restrict__ z, const TV* __restrict__ p,
          const TV* __restrict__ q, const TV* __restrict__ dinv, double* red, double* red2, Scalars* sc) {
  if (sc->done) return;
  const TV alpha = (TV)sc->alpha;
  TV rz = TV(0), rr = TV(0);
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    x[i] = x[i] + alpha * p[i];
    const TV rv = r[i] - alpha * q[i];
    r[i] = rv;
    const TV zv = dinv[i] * rv;
    z[i] = zv;
    rz += rv * zv;
    rr += rv * rv;
  }
  double b1 = block_sum((double)rz);
  double b2 = block_sum((double)rr);
  if (threadIdx.x == 0) { red[blockIdx.x] = b1; red2[blockIdx.x] = b2; }
  if (last_block(&sc->ticket2)) {
    double rzn = ordered_sum(red, gridDim.x);
    double rrn = ordered_sum(red2, gridDim.x);
    if (threadIdx.x == 0) {
      sc->beta = sc->rz != 0.0 ? rzn / sc->rz : 0.0;
      sc->rz = rzn;
      sc->rr = rrn;
      sc->it += 1;
      if (!isfinite(rrn)) { sc->bad = 1; sc->done = 1; }
      if (rrn <= sc->tol2) sc->done = 2;
      sc->ticket2 = 0;
    }
  }
}

template <typename TV>
__global__ void cg_direction(int n, TV* __restrict__ p, const TV* __restrict__ z, const Scalars* sc) {
  if (sc->done) return;
  const TV beta = (TV)sc->beta;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) p[i] = z[i] + beta * p[i];
}

__global__ void to_float(int n, const double* __restrict__ a, float* __restrict__ b) {
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) b[i] = (float)a[i];
}

// Setup: dinv (0 on fixed rows), r = f - A x0 on free rows (x0 = Dirichlet values at fixed DOFs and
// `x` elsewhere), z = dinv r, p = z, partial <r,z>, <r,r>.
template <typename TM>
__global__ void __launch_bounds__(kThreads)
cg_residual(int n, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci, const TM* __restrict__ val,
            const double* __restrict__ f, const uint8_t* __restrict__ fixed, const double* __restrict__ x,
            double* __restrict__ r) {
  const int lane = threadIdx.x & 31;
  for (int row = (blockIdx.x * kThreads + threadIdx.x) >> 5; row < n; row += (gridDim.x * kThreads) >> 5) {
    const int k0 = __ldg(rp + row) - 1, k1 = __ldg(rp + row + 1) - 1;
    double s = 0.0;
    for (int k = k0 + lane; k < k1; k += 32) s += (double)__ldg(val + k) * x[__ldg(ci + k) - 1];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) r[row] = (fixed && fixed[row]) ? 0.0 : (f ? f[row] : 0.0) - s;
  }
}

__global__ void jacobi_inverse(int n, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                               const double* __restrict__ val, const uint8_t* __restrict__ fixed,
                               double* __restrict__ dinv, unsigned* err) {
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < n; row += gridDim.x * blockDim.x) {
    double d = 0.0;
    for (int k = rp[row] - 1; k < rp[row + 1] - 1; ++k)
      if (ci[k] == row + 1) { d = val[k]; break; }
    if (fixed && fixed[row]) { dinv[row] = 0.0; continue; }
    if (!(d != 0.0) || !isfinite(d)) { gfe_raise(err, GFE_DEVERR_NONFINITE); dinv[row] = 0.0; continue; }
    dinv[row] = 1.0 / d;
  }
}

// Start an inner CG from residual r64 (FP64) into vectors of type TV: r = r64, z = p = dinv r, x = 0.
template <typename TV, typename TX>
__global__ void __launch_bounds__(kThreads)
cg_start(int n, const double* __restrict__ r64, const double* __restrict__ dinv, TV* __restrict__ r,
         TV* __restrict__ z, TV* __restrict__ p, TX* __restrict__ xz, bool zero_x, double* red, double* red2,
         Scalars* sc, double rtol2) {
  double rz = 0.0, rr = 0.0;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    TV rv = (TV)r64[i];
    TV zv = (TV)(dinv[i] * (double)rv);
    r[i] = rv; z[i] = zv; p[i] = zv;
    if (zero_x) xz[i] = (TX)0;
    rz += (double)rv * (double)zv;
    rr += (double)rv * (double)rv;
  }
  double b1 = block_sum(rz), b2 = block_sum(rr);
  if (threadIdx.x == 0) { red[blockIdx.x] = b1; red2[blockIdx.x] = b2; }
  if (last_block(&sc->ticket2)) {
    double rzn = ordered_sum(red, gridDim.x), rrn = ordered_sum(red2, gridDim.x);
    if (threadIdx.x == 0) {
      sc->rz = rzn; sc->rr = rrn; sc->rr0 = rrn; sc->tol2 = rtol2 * rrn;
      sc->done = rrn == 0.0 ? 2 : 0; sc->it = 0; sc->bad = 0; sc->ticket2 = 0; sc->ticket1 = 0;
    }
  }
}

__global__ void add_correction(int n, double* __restrict__ x, const float* __restrict__ d,
                               const uint8_t* __restrict__ fixed) {
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads)
    if (!(fixed && fixed[i])) x[i] += (double)d[i];
}

__global__ void set_dirichlet(int n, double* __restrict__ x, const uint8_t* __restrict__ fixed, bool zero_free) {
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads)
    if (zero_free && !(fixed && fixed[i])) x[i] = 0.0;
}

__global__ void norm2_kernel(int n, const double* __restrict__ v, double* red, Scalars* sc, double* out) {
  double s = 0.0;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) s += v[i] * v[i];
  double b = block_sum(s);
  if (threadIdx.x == 0) red[blockIdx.x] = b;
  if (last_block(&sc->ticket1)) {
    double t = ordered_sum(red, gridDim.x);
    if (threadIdx.x == 0) { *out = t; sc->ticket1 = 0; }
  }
}

// lanes per row: FP64 rows use one thread each (the FP64 pipe is the bound); FP32 rows use few
// lanes on short rows so several rows' loads are in flight per warp
int pick_lpr(double avg, bool fp64) {
  if (fp64) return 1;
  return avg >= 96 ? 32 : (avg >= 48 ? 16 : 8);
}

template <typename TM, typename TV>
void launch_spmv(int lpr, int grid, cudaStream_t s, int n, const int32_t* rp, const int32_t* ci, const TM* val,
                 const TV* p, TV* q, const uint8_t* fixed, double* red, Scalars* sc) {
  if (lpr == 32) cg_spmv<TM, TV, 32><<<grid, kThreads, 0, s>>>(n, rp, ci, val, p, q, fixed, red, sc);
  else if (lpr == 16) cg_spmv<TM, TV, 16><<<grid, kThreads, 0, s>>>(n, rp, ci, val, p, q, fixed, red, sc);
  else if (lpr == 8) cg_spmv<TM, TV, 8><<<grid, kThreads, 0, s>>>(n, rp, ci, val, p, q, fixed, red, sc);
  else cg_spmv<TM, TV, 1><<<grid, kThreads, 0, s>>>(n, rp, ci, val, p, q, fixed, red, sc);
}

// Runs CG iterations (chunked, device-side convergence flag) on pre-started vectors.
template <typename TM, typename TV, typename TX>
int run_cg(cudaStream_t s, int n, const int32_t* rp, const int32_t* ci, const TM* val, const uint8_t* fixed,
           const TV* dinv, TX* x, TV* r, TV* z, TV* p, TV* q, double* red, double* red2, Scalars* sc,
           Scalars* sc_host, int lpr, int grid, int max_iters, int chunk) {
  int launched = 0;
  while (launched < max_iters) {
    int k = chunk < max_iters - launched ? chunk : max_iters - launched;
    for (int i = 0; i < k; ++i) {
      void* prof = gfe::stage_begin(GFE_STAGE_SPMV, s);
      launch_spmv<TM, TV>(lpr, grid, s, n, rp, ci, val, p, q, fixed, red, sc);
      gfe::stage_end(GFE_STAGE_SPMV, prof, s, 1);
      cg_update<TX, TV><<<grid, kThreads, 0, s>>>(n, x, r, z, p, q, dinv, red, red2, sc);
      cg_direction<TV><<<grid, kThreads, 0, s>>>(n, p, z, sc);
    }
    launched += k;
    GFE_CUDA_TRY(cudaGetLastError());
    GFE_CUDA_TRY(cudaMemcpyAsync(sc_host, sc, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
    GFE_CUDA_TRY(cudaStreamSynchronize(s));
    if (sc_host->done) break;
  }
  return GFE_OK;
}

}  // namespace

extern "C" int gfe_csr_spmv(int32_t n_rows, const int32_t* row_ptr, const int32_t* col_idx, const double* values,
                            const double* x, double* y, const uint8_t* fixed, void* stream) {
  if (n_rows <= 0 || !row_ptr || !col_idx || !values || !x || !y)
    return gfe::set_error(GFE_ERR_ARG, "gfe_csr_spmv: invalid arguments");
  cudaStream_t s = gfe::as_stream(stream);
  const int grid = 8 * gfe::sm_count();
  // reuse the residual kernel with f = 0 and the sign flipped afterwards would cost a pass; use
  // the CG SpMV with a private scalar block instead.
  Scalars* sc = nullptr;
  double* red = nullptr;
  int rc = gfe::scratch_alloc((void**)&sc, sizeof(Scalars), s, "spmv scalars");
  if (rc) return rc;
  rc = gfe::scratch_alloc((void**)&red, sizeof(double) * grid, s, "spmv partials");
  if (rc) { gfe::scratch_free(sc, s); return rc; }
  cudaMemsetAsync(sc, 0, sizeof(Scalars), s);
  launch_spmv<double, double>(1, grid, s, n_rows, row_ptr, col_idx, values, x, y, fixed, red, sc);
  gfe::scratch_free(red, s);
  gfe::scratch_free(sc, s);
  GFE_LAUNCH_CHECK("gfe_csr_spmv");
  return GFE_OK;
}

extern "C" int gfe_cg_solve(int32_t n, const int32_t* row_ptr, const int32_t* col_idx, const double* values,
                            const float* values32, const double* f, const uint8_t* fixed, double* x, double rtol,
                            int32_t max_iters, int32_t precision, int32_t* iters_host, double* rel_host,
                            void* stream) {
  using namespace gfe;
  const char* fn = "gfe_cg_solve";
  if (n <= 0 || !row_ptr || !col_idx || !values || !x || !(rtol > 0.0) || max_iters <= 0)
    return set_error(GFE_ERR_ARG, "%s: invalid arguments", fn);
  if (precision != GFE_FP64 && precision != GFE_MIXED) return set_error(GFE_ERR_ARG, "%s: unknown precision", fn);
  if (precision == GFE_MIXED && !values32)
    return set_error(GFE_ERR_ARG, "%s: mixed precision needs the FP32 copy of the matrix", fn);
  cudaStream_t s = as_stream(stream);
  unsigned* err = device_error_word();
  int32_t nnz1 = 0;
  GFE_CUDA_TRY(cudaMemcpyAsync(&nnz1, row_ptr + n, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  GFE_CUDA_TRY(cudaStreamSynchronize(s));
  const int lpr = pick_lpr((double)(nnz1 - 1) / n, precision == GFE_FP64);
  const int grid = 8 * sm_count();
  const int chunk = 50;

  // scratch: dinv, r64, then vector set (FP64 or FP32) and an FP32 copy of dinv
  const size_t vbytes = precision == GFE_FP64 ? sizeof(double) : sizeof(float);
  char* buf = nullptr;
  const size_t nb = (size_t)n;
  // eleven carved pieces, each rounded up to 256 bytes
  const size_t bytes = nb * sizeof(double) * 2 + nb * vbytes * 6 + sizeof(double) * grid * 2 + sizeof(Scalars) +
                       12 * 256;
  int rc = scratch_alloc((void**)&buf, bytes, s, "CG vectors");
  if (rc) return rc;
  auto carve = [&](size_t b) {
    char* p = buf;
    buf += (b + 255) & ~size_t(255);
    return p;
  };
  char* base = buf;
  double* dinv = (double*)carve(nb * sizeof(double));
  double* r64 = (double*)carve(nb * sizeof(double));
  void* vr = carve(nb * vbytes);
  void* vz = carve(nb * vbytes);
  void* vp = carve(nb * vbytes);
  void* vq = carve(nb * vbytes);
  void* vd = carve(nb * vbytes);
  void* vdinv = carve(nb * vbytes);
  double* red = (double*)carve(sizeof(double) * grid);
  double* red2 = (double*)carve(sizeof(double) * grid);
  Scalars* sc = (Scalars*)carve(sizeof(Scalars));
  Scalars sh{};
  double b2 = 0.0, r2 = 0.0;
  int total_it = 0;
  GFE_CUDA_TRY(cudaMemsetAsync(sc, 0, sizeof(Scalars), s));
  jacobi_inverse<<<grid, kThreads, 0, s>>>(n, row_ptr, col_idx, values, fixed, dinv, err);
  // initial residual with x0 = Dirichlet values, zero elsewhere
  set_dirichlet<<<grid, kThreads, 0, s>>>(n, x, fixed, true);
  cg_residual<double><<<grid, kThreads, 0, s>>>(n, row_ptr, col_idx, values, f, fixed, x, r64);
  norm2_kernel<<<grid, kThreads, 0, s>>>(n, r64, red, sc, red2 + grid - 1);
  GFE_CUDA_TRY(cudaMemcpyAsync(&b2, red2 + grid - 1, sizeof(double), cudaMemcpyDeviceToHost, s));
  GFE_CUDA_TRY(cudaStreamSynchronize(s));
  if (b2 == 0.0) {
    if (iters_host) *iters_host = 0;
    if (rel_host) *rel_host = 0.0;
    scratch_free(base, s);
    return GFE_OK;
  }
  if (precision == GFE_FP64) {
    double* r = (double*)vr; double* z = (double*)vz; double* p = (double*)vp; double* q = (double*)vq;
    // The recurrence residual drifts from the true residual b - A x, so CG aims at half the target
    // and restarts from the true residual (residual replacement) while the latter is above it.
    double r2_start = b2;
    for (int round = 0; round < 4 && rc == GFE_OK; ++round) {
      cg_start<double, double><<<grid, kThreads, 0, s>>>(n, r64, dinv, r, z, p, x, false, red, red2, sc,
                                                         0.25 * rtol * rtol * b2 / r2_start);
      rc = run_cg<double, double, double>(s, n, row_ptr, col_idx, values, fixed, dinv, x, r, z, p, q, red, red2, sc,
                                          &sh, lpr, grid, max_iters - total_it, chunk);
      total_it += sh.it;
      if (rc || sh.bad || total_it >= max_iters) break;
      cg_residual<double><<<grid, kThreads, 0, s>>>(n, row_ptr, col_idx, values, f, fixed, x, r64);
      norm2_kernel<<<grid, kThreads, 0, s>>>(n, r64, red, sc, red2 + grid - 1);
      GFE_CUDA_TRY(cudaMemcpyAsync(&r2_start, red2 + grid - 1, sizeof(double), cudaMemcpyDeviceToHost, s));
      GFE_CUDA_TRY(cudaStreamSynchronize(s));
      if (r2_start <= rtol * rtol * b2 || r2_start == 0.0) break;
    }
  } else {
    float* r = (float*)vr; float* z = (float*)vz; float* p = (float*)vp; float* q = (float*)vq; float* d = (float*)vd;
    float* dinv32 = (float*)vdinv;
    to_float<<<grid, kThreads, 0, s>>>(n, dinv, dinv32);
    const double inner_rtol = 1e-4;
    for (int outer = 0; outer < 64 && rc == GFE_OK; ++outer) {
      if (outer > 0) {
        cg_residual<double><<<grid, kThreads, 0, s>>>(n, row_ptr, col_idx, values, f, fixed, x, r64);
        norm2_kernel<<<grid, kThreads, 0, s>>>(n, r64, red, sc, red2 + grid - 1);
        GFE_CUDA_TRY(cudaMemcpyAsync(&r2, red2 + grid - 1, sizeof(double), cudaMemcpyDeviceToHost, s));
        GFE_CUDA_TRY(cudaStreamSynchronize(s));
        if (r2 <= rtol * rtol * b2) break;
        if (total_it >= max_iters) break;
      }
      cg_start<float, float><<<grid, kThreads, 0, s>>>(n, r64, dinv, r, z, p, d, true, red, red2, sc,
                                                       inner_rtol * inner_rtol);
      rc = run_cg<float, float, float>(s, n, row_ptr, col_idx, values32, fixed, dinv32, d, r, z, p, q, red, red2, sc,
                                       &sh, lpr, grid, max_iters - total_it, chunk);
      total_it += sh.it;
      if (sh.bad) break;
      add_correction<<<grid, kThreads, 0, s>>>(n, x, d, fixed);
    }
  }
  // final FP64 residual
  cg_residual<double><<<grid, kThreads, 0, s>>>(n, row_ptr, col_idx, values, f, fixed, x, r64);
  norm2_kernel<<<grid, kThreads, 0, s>>>(n, r64, red, sc, red2 + grid - 1);
  cudaMemcpyAsync(&r2, red2 + grid - 1, sizeof(double), cudaMemcpyDeviceToHost, s);
  cudaError_t e = cudaStreamSynchronize(s);
  scratch_free(base, s);
  if (rc) return rc;
  if (e != cudaSuccess) return set_error(GFE_ERR_CUDA, "%s: %s", fn, cudaGetErrorString(e));
  const double rel = std::sqrt(r2 / b2);
  if (iters_host) *iters_host = total_it;
  if (rel_host) *rel_host = rel;
  if (sh.bad) return set_error(GFE_ERR_NUMERIC, "%s: CG breakdown (non-positive curvature or non-finite value)", fn);
  if (!(rel <= rtol)) return set_error(GFE_ERR_NOCONV, "%s: relative residual %.3e above %.3e after %d iterations",
                                       fn, rel, rtol, total_it);
  return GFE_OK;
}

// ---------------------------------------------------------------------------------------------
// Allocation-free variant of the FP64 solve
// ---------------------------------------------------------------------------------------------
// Some callers of this library may not allocate device memory at all: host codes that run the
// solve from inside a memory pool they do not own (a framework's caching allocator, a
// statically partitioned serving process) or from places where a cudaMalloc would synchronise the
// device or be forbidden.  gfe_cg_solve_noalloc serves them: its working vectors live in one
// fixed array in the library's own device memory, sized for GFE_NOALLOC_MAX_ROWS rows, which every
// GPU that loads the library keeps for the lifetime of the process.
namespace {

constexpr long long kNoAllocGrid = 8 * 256;  // partial-sum slots: grid capped at 8 blocks x 256 SMs
constexpr long long kNoAllocScalars = 32;    // doubles reserved for the Scalars block and the error word
constexpr long long kNoAllocDoubles = 6ll * GFE_NOALLOC_MAX_ROWS + 2 * kNoAllocGrid + kNoAllocScalars;

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocDoubles];

std::mutex g_noalloc_mu;
double* g_noalloc_ptr[64] = {nullptr};

// Device address of g_noalloc_scratch on the current device, looked up once per device.  The
// symbol name is only a host-side handle; kernels must be given this address.
int noalloc_scratch(double** out) {
  int dev = 0;
  GFE_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return gfe::set_error(GFE_ERR_ARG, "gfe_cg_solve_noalloc: device %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return gfe::set_error(GFE_ERR_CUDA, "gfe_cg_solve_noalloc: cudaGetSymbolAddress failed: %s",
                            cudaGetErrorString(e));
    g_noalloc_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_noalloc_ptr[dev];
  return GFE_OK;
}

}  // namespace

extern "C" int gfe_cg_solve_noalloc(int32_t n, const int32_t* row_ptr, const int32_t* col_idx, const double* values,
                                    const double* f, const uint8_t* fixed, double* x, double rtol, int32_t max_iters,
                                    int32_t* iters_host, double* rel_host, void* stream) {
  using namespace gfe;
  const char* fn = "gfe_cg_solve_noalloc";
  if (n <= 0 || !row_ptr || !col_idx || !values || !x || !(rtol > 0.0) || max_iters <= 0)
    return set_error(GFE_ERR_ARG, "%s: invalid arguments", fn);
  if (n > GFE_NOALLOC_MAX_ROWS)
    return set_error(GFE_ERR_ARG, "%s: %d rows exceed the fixed scratch capacity of %d rows (use gfe_cg_solve)", fn,
                     n, GFE_NOALLOC_MAX_ROWS);
  double* base = nullptr;
  int rc = noalloc_scratch(&base);
  if (rc) return rc;
  cudaStream_t s = as_stream(stream);
  int32_t nnz1 = 0;
  GFE_CUDA_TRY(cudaMemcpyAsync(&nnz1, row_ptr + n, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  GFE_CUDA_TRY(cudaStreamSynchronize(s));
  const int lpr = pick_lpr((double)(nnz1 - 1) / n, true);
  const int grid = std::min<int>(8 * sm_count(), (int)kNoAllocGrid);
  const int chunk = 25;
  const size_t nb = (size_t)n;
  double* dinv = base;
  double* r64 = dinv + GFE_NOALLOC_MAX_ROWS;
  double* r = r64 + GFE_NOALLOC_MAX_ROWS;
  double* z = r + GFE_NOALLOC_MAX_ROWS;
  double* p = z + GFE_NOALLOC_MAX_ROWS;
  double* q = p + GFE_NOALLOC_MAX_ROWS;
  double* red = q + GFE_NOALLOC_MAX_ROWS;
  double* red2 = red + kNoAllocGrid;
  Scalars* sc = reinterpret_cast<Scalars*>(red2 + kNoAllocGrid);
  unsigned* err = reinterpret_cast<unsigned*>(red2 + kNoAllocGrid + kNoAllocScalars - 1);
  static_assert(sizeof(Scalars) <= (kNoAllocScalars - 1) * sizeof(double), "scalar block too small");
  (void)nb;
  // the array keeps the previous call's contents: the scalars (tickets, flags) and the error word
  // must start at zero; every vector is written before it is read
  GFE_CUDA_TRY(cudaMemsetAsync(sc, 0, sizeof(double) * kNoAllocScalars, s));
  Scalars sh{};
  double b2 = 0.0, r2 = 0.0;
  jacobi_inverse<<<grid, kThreads, 0, s>>>(n, row_ptr, col_idx, values, fixed, dinv, err);
  set_dirichlet<<<grid, kThreads, 0, s>>>(n, x, fixed, true);
  cg_residual<double><<<grid, kThreads, 0, s>>>(n, row_ptr, col_idx, values, f, fixed, x, r64);
  norm2_kernel<<<grid, kThreads, 0, s>>>(n, r64, red, sc, red2 + grid - 1);
  GFE_CUDA_TRY(cudaMemcpyAsync(&b2, red2 + grid - 1, sizeof(double), cudaMemcpyDeviceToHost, s));
  GFE_CUDA_TRY(cudaStreamSynchronize(s));
  if (b2 == 0.0) {
    if (iters_host) *iters_host = 0;
    if (rel_host) *rel_host = 0.0;
    return GFE_OK;
  }
  // same residual-replacement rounds as gfe_cg_solve
  int total_it = 0;
  r2 = b2;
  for (int round = 0; round < 4; ++round) {
    cg_start<double, double><<<grid, kThreads, 0, s>>>(n, r64, dinv, r, z, p, x, false, red, red2, sc,
                                                       0.25 * rtol * rtol * b2 / r2);
    rc = run_cg<double, double, double>(s, n, row_ptr, col_idx, values, fixed, dinv, x, r, z, p, q, red, red2, sc,
                                        &sh, lpr, grid, max_iters - total_it, chunk);
    if (rc) return rc;
    total_it += sh.it;
    cg_residual<double><<<grid, kThreads, 0, s>>>(n, row_ptr, col_idx, values, f, fixed, x, r64);
    norm2_kernel<<<grid, kThreads, 0, s>>>(n, r64, red, sc, red2 + grid - 1);
    GFE_CUDA_TRY(cudaMemcpyAsync(&r2, red2 + grid - 1, sizeof(double), cudaMemcpyDeviceToHost, s));
    GFE_CUDA_TRY(cudaStreamSynchronize(s));
    if (sh.bad || total_it >= max_iters || r2 <= rtol * rtol * b2 || r2 == 0.0) break;
  }
  sh.it = total_it;
  const double rel = std::sqrt(r2 / b2);
  if (iters_host) *iters_host = sh.it;
  if (rel_host) *rel_host = rel;
  if (sh.bad) return set_error(GFE_ERR_NUMERIC, "%s: CG breakdown (non-positive curvature or non-finite value)", fn);
  if (!(rel <= rtol))
    return set_error(GFE_ERR_NOCONV, "%s: relative residual %.3e above %.3e after %d iterations", fn, rel, rtol, sh.it);
  return GFE_OK;
}
