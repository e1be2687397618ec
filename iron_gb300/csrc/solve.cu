// solve.cu -- K7: CSR SpMV and Jacobi-preconditioned CG on the Dirichlet-eliminated system.
//
// Iron assembles the solver matrix by removing fixed DOFs (SOLVER_MATRICES_STATIC_ASSEMBLE,
// src/solver_routines.F90:14025-15050) and hands it to PETSc KSP with a Jacobi preconditioner by
// default (src/solver_routines.F90:11320-11369, 11775-11991).  Here the same system is solved in
// the full DOF index space: fixed rows of A p are zeroed and fixed entries of every search
// direction are zero, which is algebraically the eliminated system.
//
// All scalars of the iteration live on the device; one iteration is three kernels (SpMV + <p,q>,
// update + <r,z>, direction update).  The product takes the form that suits the rows: short rows
// (the trilinear hexahedron's 27) a batched-load CSR form in FP64 and a sliced-ELL copy in FP32,
// long rows (the Q2/Q1 tangent's ~390) several lanes a row.  Reductions are deterministic: each block writes a partial
// sum and the last block to finish (detected by an atomic ticket) adds the partials in index order.
// Kernels return immediately once the device-side `done` flag is set, so the host can launch
// iterations in chunks and synchronise only between chunks.
//
// Mixed precision (precision == GFE_MIXED with an FP32 copy of the matrix): FP32 CG (FP32 matrix
// and vectors, FP64 dot products) with reliable updates.  Each time its recurrence residual has
// dropped 1e3-fold, the FP32 correction is added to x in FP64, the true residual f - A x is formed
// in FP64 with the FP64 matrix and tested against the target, and it replaces the FP32 residual
// while the FP32 CG keeps its search direction.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <type_traits>
#include <vector>

#include "gfe_internal.cuh"
#include "reduce.cuh"
#include "scan.cuh"

namespace {

constexpr int kThreads = gfe_red::kThreads;

struct Scalars {
  double rz, pq, alpha, beta, rr, rr0, tol2;
  int done, it, ticket1, ticket2, bad;
};

using gfe_red::block_sum;
using gfe_red::last_block;
using gfe_red::ordered_sum;

// q = A p on free rows (0 on fixed rows), partial <p, q>.  LPR lanes per row.  The arithmetic is
// done in the vector type TV: GB300's FP64 pipe issues a warp instruction in 64 cycles, so the FP64
// solve uses one thread per row (no shuffle reduction, no idle lanes in the FMA chain) and the FP32
// inner solve of the mixed scheme stays entirely on the FP32 pipe.
// CSR value / column loads of the sparse matrix-vector products.  With several lanes per row the
// lanes read consecutive entries (each line once), so the loads stream with evict-first priority
// (__ldcs) and L1 keeps the gathered vector entries that neighbouring rows reuse: 17 % per MINRES
// iteration on the 1.4 G-entry Q2/Q1 Jacobian.  With one thread per row each thread walks its own
// row and relies on L1 keeping the line between its iterations, so the loads stay cached (__ldg).
template <int LPR, typename T>
__device__ __forceinline__ T ld_csr(const T* p) {
  if constexpr (LPR >= 8) return __ldcs(p);
  else return __ldg(p);
}

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
    for (int k = k0 + sub; k < k1; k += LPR) s += (TV)ld_csr<LPR>(val + k) * p[ld_csr<LPR>(ci + k) - 1];
#pragma unroll
    for (int o = LPR / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, LPR);
    if (valid && sub == 0) {
      if (fixed && fixed[row]) s = TV(0);
      q[row] = s;
      dot += p[row] * s;
    }
  }
  double b = block_sum(dot);
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

// q = A p as cg_spmv, with each lane's first E entries of its row loaded before any is used (the
// per-row loop keeps about four loads in flight a lane, and each row waits on its bounds, then on
// its entries, then on the gathers), R rows per lane group at a time, and the next rows' bounds
// loaded ahead.  Same summation order as cg_spmv with the same LPR.
template <typename TM, typename TV, int LPR, int E, int R, int MINB>
__global__ void __launch_bounds__(kThreads, MINB)
cg_spmv_batched(int n, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci, const TM* __restrict__ val,
                const TV* __restrict__ p, TV* __restrict__ q, const uint8_t* __restrict__ fixed, double* red,
                Scalars* sc) {
  if (sc->done) return;
  constexpr int RPB = kThreads / LPR;  // rows per block for each of the R row slots
  const int sub = threadIdx.x % LPR, grp = threadIdx.x / LPR;
  const int stride = gridDim.x * RPB * R;
  TV dot = TV(0);
  int k0[R], k1[R];
#pragma unroll
  for (int j = 0; j < R; ++j) {
    const int row = blockIdx.x * RPB * R + j * RPB + grp;
    k0[j] = row < n ? __ldg(rp + row) - 1 : 0;
    k1[j] = row < n ? __ldg(rp + row + 1) - 1 : 0;
  }
  for (int base = blockIdx.x * RPB * R; base < n; base += stride) {
    int nk0[R], nk1[R];
    TM v[R][E];
    int c[R][E];
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const int nrow = base + stride + j * RPB + grp;
      nk0[j] = nrow < n ? __ldg(rp + nrow) - 1 : 0;
      nk1[j] = nrow < n ? __ldg(rp + nrow + 1) - 1 : 0;
#pragma unroll
      for (int u = 0; u < E; ++u) {
        const int k = k0[j] + sub + u * LPR;
        v[j][u] = k < k1[j] ? ld_csr<LPR>(val + k) : TM(0);
        c[j][u] = k < k1[j] ? ld_csr<LPR>(ci + k) : 0;
      }
    }
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const int row = base + j * RPB + grp;
      TV s = TV(0);
#pragma unroll
      for (int u = 0; u < E; ++u)
        if (c[j][u] > 0) s += (TV)v[j][u] * p[c[j][u] - 1];
#pragma unroll 1
      for (int k = k0[j] + sub + E * LPR; k < k1[j]; k += LPR) s += (TV)ld_csr<LPR>(val + k) * p[ld_csr<LPR>(ci + k) - 1];
#pragma unroll
      for (int o = LPR / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, LPR);
      if (row < n && sub == 0) {
        if (fixed && fixed[row]) s = TV(0);
        q[row] = s;
        dot += p[row] * s;
      }
      k0[j] = nk0[j];
      k1[j] = nk1[j];
    }
  }
  double b = block_sum(dot);
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
  double b1 = block_sum(rz);
  double b2 = block_sum(rr);
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

// cg_residual for short rows (up to about 32 entries): 2 lanes a row, 14 entries a lane loaded
// before the first gather, the next row's bounds loaded ahead (the loads of cg_spmv_batched).  The warp-per-row form spends 5 levels of FP64 shuffle additions on every row,
// more FP64 work than the row's own products.
__global__ void __launch_bounds__(kThreads, 4)
cg_residual_short(int n, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                  const double* __restrict__ val, const double* __restrict__ f, const uint8_t* __restrict__ fixed,
                  const double* __restrict__ x, double* __restrict__ r) {
  constexpr int LPR = 2, E = 14, R = 1, RPB = kThreads / LPR;
  const int sub = threadIdx.x % LPR, grp = threadIdx.x / LPR;
  const int stride = gridDim.x * RPB * R;
  int k0[R], k1[R];
#pragma unroll
  for (int j = 0; j < R; ++j) {
    const int row = blockIdx.x * RPB * R + j * RPB + grp;
    k0[j] = row < n ? __ldg(rp + row) - 1 : 0;
    k1[j] = row < n ? __ldg(rp + row + 1) - 1 : 0;
  }
  for (int base = blockIdx.x * RPB * R; base < n; base += stride) {
    int nk0[R], nk1[R];
    double v[R][E];
    int c[R][E];
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const int nrow = base + stride + j * RPB + grp;
      nk0[j] = nrow < n ? __ldg(rp + nrow) - 1 : 0;
      nk1[j] = nrow < n ? __ldg(rp + nrow + 1) - 1 : 0;
#pragma unroll
      for (int u = 0; u < E; ++u) {
        const int k = k0[j] + sub + u * LPR;
        v[j][u] = k < k1[j] ? __ldg(val + k) : 0.0;
        c[j][u] = k < k1[j] ? __ldg(ci + k) : 0;
      }
    }
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const int row = base + j * RPB + grp;
      double acc = 0.0;
#pragma unroll
      for (int u = 0; u < E; ++u)
        if (c[j][u] > 0) acc += v[j][u] * x[c[j][u] - 1];
#pragma unroll 1
      for (int k = k0[j] + sub + E * LPR; k < k1[j]; k += LPR) acc += __ldg(val + k) * x[__ldg(ci + k) - 1];
      acc += __shfl_down_sync(0xffffffffu, acc, 1, LPR);
      if (row < n && sub == 0) r[row] = (fixed && fixed[row]) ? 0.0 : (f ? f[row] : 0.0) - acc;
      k0[j] = nk0[j];
      k1[j] = nk1[j];
    }
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

// Start an inner CG from residual r64 (FP64) into vectors of type TV: r = r64, z = dinv r, x = 0
// when zero_x.  keep_p false: a fresh start, p = z.  keep_p true: a reliable update after a CG that
// stopped on convergence (so its last direction update was skipped): the true residual replaces
// the recurrence residual r_k+1 and the search direction p_k is kept; beta = <r,z> / rho_k, where
// rho_k = rho_k+1 / beta_k+1 from the stopped CG's scalars, for a following cg_direction, which
// forms p = z + beta p.
template <typename TV, typename TX>
__global__ void __launch_bounds__(kThreads)
cg_start(int n, const double* __restrict__ r64, const double* __restrict__ dinv, TV* __restrict__ r,
         TV* __restrict__ z, TV* __restrict__ p, TX* __restrict__ xz, bool zero_x, bool keep_p, double* red,
         double* red2, Scalars* sc, double rtol2) {
  double rz = 0.0, rr = 0.0;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    TV rv = (TV)r64[i];
    TV zv = (TV)(dinv[i] * (double)rv);
    r[i] = rv; z[i] = zv;
    if (!keep_p) p[i] = zv;
    if (zero_x) xz[i] = (TX)0;
    rz += (double)rv * (double)zv;
    rr += (double)rv * (double)rv;
  }
  double b1 = block_sum(rz), b2 = block_sum(rr);
  if (threadIdx.x == 0) { red[blockIdx.x] = b1; red2[blockIdx.x] = b2; }
  if (last_block(&sc->ticket2)) {
    double rzn = ordered_sum(red, gridDim.x), rrn = ordered_sum(red2, gridDim.x);
    if (threadIdx.x == 0) {
      sc->beta = keep_p && sc->rz != 0.0 ? sc->beta * (rzn / sc->rz) : 0.0;
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

// sum_i v_i^2, or sum_i w_i v_i^2 when w is given (the M^-1-norm for w = minv)
__global__ void norm2_kernel(int n, const double* __restrict__ v, double* red, Scalars* sc, double* out,
                             const double* __restrict__ w = nullptr) {
  double s = 0.0;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) s += (w ? w[i] : 1.0) * v[i] * v[i];
  double b = block_sum(s);
  if (threadIdx.x == 0) red[blockIdx.x] = b;
  if (last_block(&sc->ticket1)) {
    double t = ordered_sum(red, gridDim.x);
    if (threadIdx.x == 0) { *out = t; sc->ticket1 = 0; }
  }
}

// Sliced-ELL copy of a CSR matrix with short rows, for the CG products: slices of 32 consecutive
// rows, each stored column-major and padded to its longest row (column 0 marks padding), so entry
// k of row r sits at sptr[r / 32] + 32 k + r % 32.  A lane per row then reads one contiguous
// 128-byte line per warp and entry, and no row waits on its bounds; the per-row CSR forms wait on
// the row bounds, then on the entries, then on the gathers.  Built inside each solve call from the
// caller's CSR (the values change with every assembly).
constexpr int kSell = 32;

template <typename TM>
struct SellMatrix {
  const long long* sptr;  // [n_slices] first entry of each slice
  const int32_t* slen;    // [n_slices] entries of each slice (32 x its longest row)
  const int32_t* col;     // 1-based column, 0 = padding
  const TM* val;
};

__global__ void sell_slice_len(int n, const int32_t* __restrict__ rp, int32_t* __restrict__ slen) {
  const int n_pad = (n + kSell - 1) / kSell * kSell;
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < n_pad; row += gridDim.x * blockDim.x) {
    const int len = row < n ? __ldg(rp + row + 1) - __ldg(rp + row) : 0;
    const int mx = __reduce_max_sync(0xffffffffu, len);
    if ((row & (kSell - 1)) == 0) slen[row / kSell] = mx * kSell;
  }
}

template <typename TM>
__global__ void sell_fill(int n, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                          const TM* __restrict__ val, const long long* __restrict__ sptr,
                          const int32_t* __restrict__ slen, int32_t* __restrict__ col, TM* __restrict__ sval) {
  const int n_pad = (n + kSell - 1) / kSell * kSell;
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < n_pad; row += gridDim.x * blockDim.x) {
    const int sl = row / kSell, lane = row & (kSell - 1);
    const long long base = sptr[sl] + lane;
    const int L = slen[sl] / kSell;
    const int k0 = row < n ? __ldg(rp + row) - 1 : 0, len = row < n ? __ldg(rp + row + 1) - 1 - k0 : 0;
    for (int k = 0; k < L; ++k) {
      const bool in = k < len;
      col[base + (long long)k * kSell] = in ? __ldg(ci + k0 + k) : 0;
      sval[base + (long long)k * kSell] = in ? __ldg(val + k0 + k) : TM(0);
    }
  }
}

// q = A p on free rows (0 on fixed rows) from the sliced-ELL copy, partial <p, q> and alpha as
// cg_spmv; each row's entries in column order, kSellUnroll loads in flight a lane.
constexpr int kSellUnroll = 8;

template <typename TM, typename TV>
__global__ void __launch_bounds__(kThreads)
cg_spmv_sell(int n, SellMatrix<TM> A, const TV* __restrict__ p, TV* __restrict__ q,
             const uint8_t* __restrict__ fixed, double* red, Scalars* sc) {
  if (sc->done) return;
  const int n_pad = (n + kSell - 1) / kSell * kSell;
  TV dot = TV(0);
  // the loop bound is warp-uniform (whole slices)
  for (int row = blockIdx.x * kThreads + threadIdx.x; row < n_pad; row += gridDim.x * kThreads) {
    const int sl = row / kSell, lane = row & (kSell - 1);
    const long long base = __ldg(A.sptr + sl) + lane;
    const int L = __ldg(A.slen + sl) / kSell;
    TV acc = TV(0);
    for (int k0 = 0; k0 < L; k0 += kSellUnroll) {
      TM v[kSellUnroll];
      int c[kSellUnroll];
#pragma unroll
      for (int u = 0; u < kSellUnroll; ++u) {
        const bool in = k0 + u < L;
        const long long at = base + (long long)(k0 + u) * kSell;
        v[u] = in ? __ldcs(A.val + at) : TM(0);
        c[u] = in ? __ldcs(A.col + at) : 0;
      }
#pragma unroll
      for (int u = 0; u < kSellUnroll; ++u)
        if (c[u] > 0) acc += (TV)v[u] * p[c[u] - 1];
    }
    if (row < n) {
      if (fixed && fixed[row]) acc = TV(0);
      q[row] = acc;
      dot += p[row] * acc;
    }
  }
  double b = block_sum(dot);
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

// Builds the sliced-ELL copy of (rp, ci, val) in two scratch allocations bufs[0], bufs[1] (the
// caller frees both with scratch_free).  Synchronises the stream once (the copy's size).
template <typename TM>
int build_sell(int n, const int32_t* rp, const int32_t* ci, const TM* val, cudaStream_t s, void* bufs[2],
               SellMatrix<TM>* out) {
  using namespace gfe;
  bufs[0] = bufs[1] = nullptr;
  const long long n_slices = (n + kSell - 1) / kSell;
  char* head = nullptr;
  const size_t head_bytes = ((sizeof(long long) * (n_slices + 1) + 255) & ~size_t(255)) +
                            ((sizeof(int32_t) * n_slices + 255) & ~size_t(255));
  int rc = scratch_alloc((void**)&head, head_bytes, s, "sliced-ELL offsets");
  if (rc) return rc;
  long long* sptr = (long long*)head;
  int32_t* slen = (int32_t*)(head + ((sizeof(long long) * (n_slices + 1) + 255) & ~size_t(255)));
  const int grid = 8 * sm_count();
  sell_slice_len<<<grid, kThreads, 0, s>>>(n, rp, slen);
  if ((rc = exclusive_scan(slen, n_slices, sptr, sptr + n_slices, s))) { scratch_free(head, s); return rc; }
  long long total = 0;
  cudaError_t e = cudaMemcpyAsync(&total, sptr + n_slices, sizeof(long long), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) { scratch_free(head, s); return set_error(GFE_ERR_CUDA, "sliced-ELL size: %s", cudaGetErrorString(e)); }
  char* body = nullptr;
  const size_t col_bytes = ((sizeof(int32_t) * (size_t)total + 255) & ~size_t(255));
  if ((rc = scratch_alloc((void**)&body, col_bytes + sizeof(TM) * (size_t)total + 256, s, "sliced-ELL copy"))) {
    scratch_free(head, s);
    return rc;
  }
  int32_t* col = (int32_t*)body;
  TM* sval = (TM*)(body + col_bytes);
  sell_fill<TM><<<grid, kThreads, 0, s>>>(n, rp, ci, val, sptr, slen, col, sval);
  out->sptr = sptr;
  out->slen = slen;
  out->col = col;
  out->val = sval;
  bufs[0] = head;
  bufs[1] = body;
  return GFE_OK;
}

// SpMV form of the CG iterations.  Short rows (the trilinear hexahedron's 27-entry rows, tetrahedra)
// take cg_spmv_batched: FP32 with 8 lanes a row and 4 entries a lane loaded at once (128^3 Laplace:
// 105 us a product, 126 us for the per-row loop, 4-28 lanes a row and two rows a group measured
// slower); FP64 with 2 lanes a row, 14 entries a lane and two rows a group (152 us, 216 us for one
// thread a row with the per-row loop; the shuffle of the 2-lane sum is one FP64 add a row).
// Longer FP32 rows keep the per-row loop with 16 or 32 lanes; longer FP64 rows one thread a row.
constexpr int kSpmvShort32 = -1;
constexpr int kSpmvShort64 = -2;

int pick_lpr(double avg, bool fp64) {
  if (fp64) return avg <= 32 ? kSpmvShort64 : 1;
  return avg < 48 ? kSpmvShort32 : (avg >= 96 ? 32 : 16);
}

template <typename TM, typename TV>
void launch_spmv(int lpr, int grid, cudaStream_t s, int n, const int32_t* rp, const int32_t* ci, const TM* val,
                 const TV* p, TV* q, const uint8_t* fixed, double* red, Scalars* sc) {
  // the batched kernels' register bounds guarantee MINB resident blocks an SM: their grids are
  // whole waves
  if constexpr (std::is_same<TM, float>::value && std::is_same<TV, float>::value) {
    if (lpr == kSpmvShort32) {
      const int g = std::min(grid, 8 * gfe::sm_count());
      cg_spmv_batched<TM, TV, 8, 4, 1, 8><<<g, kThreads, 0, s>>>(n, rp, ci, val, p, q, fixed, red, sc);
      return;
    }
  }
  if constexpr (std::is_same<TM, double>::value && std::is_same<TV, double>::value) {
    if (lpr == kSpmvShort64) {
      const int g = std::min(grid, 4 * gfe::sm_count());
      cg_spmv_batched<TM, TV, 2, 14, 2, 4><<<g, kThreads, 0, s>>>(n, rp, ci, val, p, q, fixed, red, sc);
      return;
    }
  }
  if (lpr == 32) cg_spmv<TM, TV, 32><<<grid, kThreads, 0, s>>>(n, rp, ci, val, p, q, fixed, red, sc);
  else if (lpr == 16) cg_spmv<TM, TV, 16><<<grid, kThreads, 0, s>>>(n, rp, ci, val, p, q, fixed, red, sc);
  else if (lpr == 8) cg_spmv<TM, TV, 8><<<grid, kThreads, 0, s>>>(n, rp, ci, val, p, q, fixed, red, sc);
  else cg_spmv<TM, TV, 1><<<grid, kThreads, 0, s>>>(n, rp, ci, val, p, q, fixed, red, sc);
}

// r = f - A x (FP64) on free rows: the batched 2-lane form for short rows, a warp a row otherwise.
void residual64(bool short_rows, int grid, cudaStream_t s, int n, const int32_t* rp, const int32_t* ci,
                const double* val, const double* f, const uint8_t* fixed, const double* x, double* r) {
  if (short_rows)
    cg_residual_short<<<std::min(grid, 4 * gfe::sm_count()), kThreads, 0, s>>>(n, rp, ci, val, f, fixed, x, r);
  else
    cg_residual<double><<<grid, kThreads, 0, s>>>(n, rp, ci, val, f, fixed, x, r);
}

// Runs CG iterations (chunked, device-side convergence flag) on pre-started vectors.
template <typename TM, typename TV, typename TX>
int run_cg(cudaStream_t s, int n, const int32_t* rp, const int32_t* ci, const TM* val, const uint8_t* fixed,
           const TV* dinv, TX* x, TV* r, TV* z, TV* p, TV* q, double* red, double* red2, Scalars* sc,
           Scalars* sc_host, int lpr, int grid, int max_iters, int chunk, const SellMatrix<TM>* sell = nullptr) {
  int launched = 0;
  while (launched < max_iters) {
    int k = chunk < max_iters - launched ? chunk : max_iters - launched;
    for (int i = 0; i < k; ++i) {
      void* prof = gfe::stage_begin(GFE_STAGE_SPMV, s);
      if (sell) cg_spmv_sell<TM, TV><<<grid, kThreads, 0, s>>>(n, *sell, p, q, fixed, red, sc);
      else launch_spmv<TM, TV>(lpr, grid, s, n, rp, ci, val, p, q, fixed, red, sc);
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
  launch_spmv<double, double>(kSpmvShort64, grid, s, n_rows, row_ptr, col_idx, values, x, y, fixed, red, sc);
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
  const bool short_rows = (double)(nnz1 - 1) / n <= 32.0;
  // short rows: the FP32 iterations of the mixed solve run on a sliced-ELL copy of values32 (128^3
  // Laplace: 104 -> 91 us a product, 103 -> 93 ms a solve); the FP64 product, bound by FP64 work
  // as much as by its loads, gained nothing from it and keeps the batched CSR form
  const bool use_sell = precision == GFE_MIXED && (double)(nnz1 - 1) / n <= 32.0 && n >= 4 * kSell;
  void* sell_bufs[2] = {nullptr, nullptr};

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
  residual64(short_rows, grid, s, n, row_ptr, col_idx, values, f, fixed, x, r64);
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
    // and, while the true residual is above it, replaces the recurrence residual by the true one
    // and continues along the same search direction (a reliable update).
    double r2_start = b2;
    for (int round = 0; round < 4 && rc == GFE_OK; ++round) {
      cg_start<double, double><<<grid, kThreads, 0, s>>>(n, r64, dinv, r, z, p, x, false, round > 0, red, red2, sc,
                                                         0.25 * rtol * rtol * b2 / r2_start);
      if (round > 0) cg_direction<double><<<grid, kThreads, 0, s>>>(n, p, z, sc);
      rc = run_cg<double, double, double>(s, n, row_ptr, col_idx, values, fixed, dinv, x, r, z, p, q, red, red2, sc,
                                          &sh, lpr, grid, max_iters - total_it, chunk);
      total_it += sh.it;
      if (rc || sh.bad || total_it >= max_iters) break;
      residual64(short_rows, grid, s, n, row_ptr, col_idx, values, f, fixed, x, r64);
      norm2_kernel<<<grid, kThreads, 0, s>>>(n, r64, red, sc, red2 + grid - 1);
      GFE_CUDA_TRY(cudaMemcpyAsync(&r2_start, red2 + grid - 1, sizeof(double), cudaMemcpyDeviceToHost, s));
      GFE_CUDA_TRY(cudaStreamSynchronize(s));
      if (r2_start <= rtol * rtol * b2 || r2_start == 0.0) break;
    }
  } else {
    float* r = (float*)vr; float* z = (float*)vz; float* p = (float*)vp; float* q = (float*)vq; float* d = (float*)vd;
    float* dinv32 = (float*)vdinv;
    to_float<<<grid, kThreads, 0, s>>>(n, dinv, dinv32);
    // Reliable updates: the FP32 CG runs until its recurrence residual has dropped by inner_rtol
    // since the last update; then its correction d is added to x in FP64, the true residual
    // f - A x is formed with the FP64 matrix, replaces the FP32 residual, and the FP32 CG continues
    // along its current search direction.  At 128^3 to 1e-12: 727 iterations (FP64 CG: 670);
    // restarting the FP32 CG from the true residual instead discards its Krylov space (928
    // iterations with the best restart tolerance, 1e-5).  Reductions of 1e-1 to 1e-3 per update
    // all take 727-742 iterations; 1e-3 needs the fewest updates.
    const double inner_rtol = 1e-3;
    SellMatrix<float> sell{};
    if (use_sell) rc = build_sell<float>(n, row_ptr, col_idx, values32, s, sell_bufs, &sell);
    for (int outer = 0; outer < 200 && rc == GFE_OK; ++outer) {
      if (outer > 0) {
        residual64(short_rows, grid, s, n, row_ptr, col_idx, values, f, fixed, x, r64);
        norm2_kernel<<<grid, kThreads, 0, s>>>(n, r64, red, sc, red2 + grid - 1);
        GFE_CUDA_TRY(cudaMemcpyAsync(&r2, red2 + grid - 1, sizeof(double), cudaMemcpyDeviceToHost, s));
        GFE_CUDA_TRY(cudaStreamSynchronize(s));
        if (r2 <= rtol * rtol * b2) break;
        if (total_it >= max_iters) break;
      }
      cg_start<float, float><<<grid, kThreads, 0, s>>>(n, r64, dinv, r, z, p, d, true, outer > 0, red, red2, sc,
                                                       inner_rtol * inner_rtol);
      if (outer > 0) cg_direction<float><<<grid, kThreads, 0, s>>>(n, p, z, sc);
      rc = run_cg<float, float, float>(s, n, row_ptr, col_idx, values32, fixed, dinv32, d, r, z, p, q, red, red2, sc,
                                       &sh, lpr, grid, max_iters - total_it, chunk, use_sell ? &sell : nullptr);
      total_it += sh.it;
      if (sh.bad) break;
      add_correction<<<grid, kThreads, 0, s>>>(n, x, d, fixed);
    }
  }
  // final FP64 residual
  residual64(short_rows, grid, s, n, row_ptr, col_idx, values, f, fixed, x, r64);
  norm2_kernel<<<grid, kThreads, 0, s>>>(n, r64, red, sc, red2 + grid - 1);
  cudaMemcpyAsync(&r2, red2 + grid - 1, sizeof(double), cudaMemcpyDeviceToHost, s);
  cudaError_t e = cudaStreamSynchronize(s);
  scratch_free(base, s);
  scratch_free(sell_bufs[0], s);
  scratch_free(sell_bufs[1], s);
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
// Graph-capturable FP64 CG with a caller-owned workspace
// ---------------------------------------------------------------------------------------------
// gfe_cg_begin / gfe_cg_steps / gfe_cg_status only enqueue kernels and copies on the stream: no
// allocation and no synchronisation, so a host loop can capture "begin" and "k steps + status"
// once into CUDA graphs and replay them, checking the pinned status between replays.  Steps after
// convergence are no-ops (the device-side done flag), so a replay may overrun safely.  The
// convergence test is the recurrence residual ||r_k||^2 <= rtol^2 ||r_0||^2 (no residual
// replacement: use gfe_cg_solve for targets near FP64 round-off).
namespace {

struct CgWork {
  double *dinv, *r, *z, *p, *q, *red, *red2;
  Scalars* sc;
  gfe_cg_state* state;
  int grid;
};

int cg_work_layout(int32_t n, void* ws, CgWork* w) {
  if (!ws || (reinterpret_cast<uintptr_t>(ws) & 255))
    return gfe::set_error(GFE_ERR_ARG, "CG workspace must be a 256-byte aligned device pointer");
  const size_t nb = ((size_t)n * sizeof(double) + 255) & ~size_t(255);
  w->grid = 8 * gfe::sm_count();
  const size_t gb = ((size_t)w->grid * sizeof(double) + 255) & ~size_t(255);
  char* b = static_cast<char*>(ws);
  w->dinv = (double*)b; b += nb;
  w->r = (double*)b; b += nb;
  w->z = (double*)b; b += nb;
  w->p = (double*)b; b += nb;
  w->q = (double*)b; b += nb;
  w->red = (double*)b; b += gb;
  w->red2 = (double*)b; b += gb;
  w->sc = (Scalars*)b; b += 256;
  w->state = (gfe_cg_state*)b;
  return GFE_OK;
}

__global__ void cg_export_state(const Scalars* sc, gfe_cg_state* st) {
  st->rr = sc->rr;
  st->rr0 = sc->rr0;
  st->done = sc->done;
  st->iterations = sc->it;
  st->breakdown = sc->bad;
  st->reserved = 0;
}

}  // namespace

extern "C" int64_t gfe_cg_workspace_bytes(int32_t n) {
  if (n <= 0) return 0;
  const size_t nb = ((size_t)n * sizeof(double) + 255) & ~size_t(255);
  const size_t gb = ((size_t)8 * gfe::sm_count() * sizeof(double) + 255) & ~size_t(255);
  static_assert(sizeof(Scalars) <= 256, "scalar block");
  return (int64_t)(5 * nb + 2 * gb + 256 + 256);
}

extern "C" int gfe_cg_begin(int32_t n, const int32_t* row_ptr, const int32_t* col_idx, const double* values,
                            const double* f, const uint8_t* fixed, double* x, double rtol, void* workspace,
                            void* stream) {
  using namespace gfe;
  if (n <= 0 || !row_ptr || !col_idx || !values || !x || !(rtol > 0.0))
    return set_error(GFE_ERR_ARG, "gfe_cg_begin: invalid arguments");
  CgWork w;
  if (int rc = cg_work_layout(n, workspace, &w)) return rc;
  cudaStream_t s = as_stream(stream);
  unsigned* err = device_error_word();
  GFE_CUDA_TRY(cudaMemsetAsync(w.sc, 0, sizeof(Scalars), s));
  jacobi_inverse<<<w.grid, kThreads, 0, s>>>(n, row_ptr, col_idx, values, fixed, w.dinv, err);
  set_dirichlet<<<w.grid, kThreads, 0, s>>>(n, x, fixed, true);
  cg_residual<double><<<w.grid, kThreads, 0, s>>>(n, row_ptr, col_idx, values, f, fixed, x, w.q);
  cg_start<double, double><<<w.grid, kThreads, 0, s>>>(n, w.q, w.dinv, w.r, w.z, w.p, x, false, false, w.red, w.red2, w.sc,
                                                       rtol * rtol);
  GFE_LAUNCH_CHECK("gfe_cg_begin");
  return GFE_OK;
}

extern "C" int gfe_cg_steps(int32_t n, const int32_t* row_ptr, const int32_t* col_idx, const double* values,
                            const uint8_t* fixed, double* x, int32_t steps, void* workspace, void* stream) {
  using namespace gfe;
  if (n <= 0 || !row_ptr || !col_idx || !values || !x || steps < 0)
    return set_error(GFE_ERR_ARG, "gfe_cg_steps: invalid arguments");
  CgWork w;
  if (int rc = cg_work_layout(n, workspace, &w)) return rc;
  cudaStream_t s = as_stream(stream);
  for (int i = 0; i < steps; ++i) {
    launch_spmv<double, double>(kSpmvShort64, w.grid, s, n, row_ptr, col_idx, values, w.p, w.q, fixed, w.red, w.sc);
    cg_update<double, double><<<w.grid, kThreads, 0, s>>>(n, x, w.r, w.z, w.p, w.q, w.dinv, w.red, w.red2, w.sc);
    cg_direction<double><<<w.grid, kThreads, 0, s>>>(n, w.p, w.z, w.sc);
  }
  GFE_LAUNCH_CHECK("gfe_cg_steps");
  return GFE_OK;
}

extern "C" int gfe_cg_status(int32_t n, void* workspace, gfe_cg_state* state_host, void* stream) {
  using namespace gfe;
  if (n <= 0 || !state_host) return set_error(GFE_ERR_ARG, "gfe_cg_status: invalid arguments");
  CgWork w;
  if (int rc = cg_work_layout(n, workspace, &w)) return rc;
  cudaStream_t s = as_stream(stream);
  cg_export_state<<<1, 1, 0, s>>>(w.sc, w.state);
  GFE_CUDA_TRY(cudaMemcpyAsync(state_host, w.state, sizeof(gfe_cg_state), cudaMemcpyDeviceToHost, s));
  return GFE_OK;
}

// ---------------------------------------------------------------------------------------------
// Preconditioned MINRES for symmetric indefinite systems
// ---------------------------------------------------------------------------------------------
// The consistent tangent of the mixed u-p Mooney-Rivlin residual is symmetric with a zero p-p
// block, so CG does not apply.  Iron hands such systems to PETSc (GMRES + Jacobi by default,
// src/solver_routines.F90:11320-11369, or a direct solver); here they are solved by MINRES with a
// symmetric positive definite diagonal preconditioner M, in the Lanczos form of Elman, Silvester
// and Wathen (Finite Elements and Fast Iterative Solvers, Algorithm 2.4):
//   v_{j+1} = A z_j - (delta_j / gamma_j) v_j - (gamma_j / gamma_{j-1}) v_{j-1},  z = M^-1 v / gamma
// with Givens rotations giving the update direction w and the M^-1-norm of the residual |eta|.
// One iteration is two kernels: (A) the deferred w / x update of the previous iteration fused with
// the SpMV q = A z_j and delta_j = <q, z_j>; (B) the Lanczos update, z_{j+1} = M^-1 v_{j+1},
// gamma_{j+1} and, in the last block, the rotation scalars and the convergence flag.  Vector
// buffers rotate between two copies on the host side; the kernels return at once after `done`, so
// iterations are launched in chunks exactly like the CG.
namespace {

struct MinresScalars {
  double gamma, gamma_old, delta, c, c_old, s, s_old, eta, tol;
  double zs_prev, a1, a2, a3, ceta;
  int done, pending, it, ticket1, ticket2, bad;
};

constexpr int kNodalBatch = 8;  // entries a lane loads at once in the MINRES products

// (A): pending w / x update of the previous iteration, then q = A z / gamma (0 on fixed rows) and
// delta = <q, z / gamma>.
template <typename TM, typename TV, typename TX, int LPR>
__global__ void __launch_bounds__(kThreads)
minres_spmv(int n, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci, const TM* __restrict__ val,
            const TV* __restrict__ z, TV* __restrict__ q, const uint8_t* __restrict__ fixed,
            const TV* __restrict__ zprev, TV* __restrict__ wold, const TV* __restrict__ wnew, TX* __restrict__ x,
            double* red, MinresScalars* sc) {
  const int pending = sc->pending, done = sc->done;
  if (done && !pending) return;
  if (pending) {
    const TV zs = (TV)sc->zs_prev, a1i = (TV)(1.0 / sc->a1), a2 = (TV)sc->a2, a3 = (TV)sc->a3, ce = (TV)sc->ceta;
    for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
      const TV w = (zprev[i] * zs - a3 * wold[i] - a2 * wnew[i]) * a1i;
      wold[i] = w;
      x[i] = x[i] + (TX)(ce * w);
    }
  }
  TV dot = TV(0);
  if (!done) {
    const TV g = (TV)(1.0 / sc->gamma);
    constexpr int RPB = kThreads / LPR;
    const int sub = threadIdx.x % LPR, grp = threadIdx.x / LPR;
    for (int base = blockIdx.x * RPB; base < n; base += gridDim.x * RPB) {
      const int row = base + grp;
      const bool valid = row < n;
      const int k0 = valid ? __ldg(rp + row) - 1 : 0, k1 = valid ? __ldg(rp + row + 1) - 1 : 0;
      TV acc = TV(0);
      if constexpr (std::is_same<TV, double>::value) {
        // FP64: bound by the FP64 pipe; the batched loads below cost it 3 % (32^3 Newton)
#pragma unroll 4
        for (int k = k0 + sub; k < k1; k += LPR) acc += (TV)ld_csr<LPR>(val + k) * z[ld_csr<LPR>(ci + k) - 1];
      } else {
        // batches of kNodalBatch entries a lane, all loaded before the first gather
        for (int t0 = k0 + sub; t0 < k1; t0 += kNodalBatch * LPR) {
          TM v[kNodalBatch];
          int c[kNodalBatch];
#pragma unroll
          for (int u = 0; u < kNodalBatch; ++u) {
            const int k = t0 + u * LPR;
            v[u] = k < k1 ? ld_csr<LPR>(val + k) : TM(0);
            c[u] = k < k1 ? ld_csr<LPR>(ci + k) : 0;
          }
#pragma unroll
          for (int u = 0; u < kNodalBatch; ++u)
            if (c[u] > 0) acc += (TV)v[u] * z[c[u] - 1];
        }
      }
#pragma unroll
      for (int o = LPR / 2; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o, LPR);
      if (valid && sub == 0) {
        const TV qv = (fixed && fixed[row]) ? TV(0) : acc * g;
        q[row] = qv;
        dot += z[row] * g * qv;
      }
    }
  }
  const double b = block_sum(dot);
  if (threadIdx.x == 0) red[blockIdx.x] = b;
  if (last_block(&sc->ticket1)) {
    const double d = ordered_sum(red, gridDim.x);
    if (threadIdx.x == 0) {
      if (!done) {
        sc->delta = d;
        if (!isfinite(d)) { sc->bad = 1; sc->done = 1; }
      }
      sc->pending = 0;
      sc->ticket1 = 0;
    }
  }
}

// (A) for a matrix whose first NC * n_node rows are the NC components of n_node nodes, numbered
// component-major (Iron's separated component DOF order of a vector field whose components share
// one basis), so the rows node, node + n_node, ... hold one column list.  A group of LPR lanes
// takes one node: each column index and gathered z entry is loaded once for the NC rows, which
// cuts the matrix traffic from 8 to 4 + 4 / NC bytes an entry in FP32.  Groups past n_node are the
// remaining rows (the pressure rows of a u-p system), one each.
constexpr int kNodalBlocks = 4;  // resident blocks an SM the register bound guarantees

template <typename TM, typename TV, typename TX, int LPR, int NC>
__global__ void __launch_bounds__(kThreads, kNodalBlocks)
minres_spmv_nodal(int n, int n_node, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                  const TM* __restrict__ val, const TV* __restrict__ z, TV* __restrict__ q,
                  const uint8_t* __restrict__ fixed, const TV* __restrict__ zprev, TV* __restrict__ wold,
                  const TV* __restrict__ wnew, TX* __restrict__ x, double* red, MinresScalars* sc) {
  const int pending = sc->pending, done = sc->done;
  if (done && !pending) return;
  if (pending) {
    const TV zs = (TV)sc->zs_prev, a1i = (TV)(1.0 / sc->a1), a2 = (TV)sc->a2, a3 = (TV)sc->a3, ce = (TV)sc->ceta;
    for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
      const TV w = (zprev[i] * zs - a3 * wold[i] - a2 * wnew[i]) * a1i;
      wold[i] = w;
      x[i] = x[i] + (TX)(ce * w);
    }
  }
  TV dot = TV(0);
  if (!done) {
    const TV g = (TV)(1.0 / sc->gamma);
    constexpr int RPB = kThreads / LPR;
    const int sub = threadIdx.x % LPR, grp = threadIdx.x / LPR;
    const int n_groups = n - (NC - 1) * n_node;
    for (int base = blockIdx.x * RPB; base < n_groups; base += gridDim.x * RPB) {
      const int grp_id = base + grp;
      const bool valid = grp_id < n_groups, multi = grp_id < n_node;
      const int row0 = multi ? grp_id : grp_id + (NC - 1) * n_node;
      int k0[NC];
      int len = 0;
      if (valid) {
#pragma unroll
        for (int j = 0; j < NC; ++j) k0[j] = (j == 0 || multi) ? __ldg(rp + row0 + j * n_node) - 1 : 0;
        len = __ldg(rp + row0 + 1) - 1 - k0[0];
      }
      TV acc[NC];
#pragma unroll
      for (int j = 0; j < NC; ++j) acc[j] = TV(0);
      if (multi) {
        // batches of kNodalBatch columns a lane: all their column indices and NC values are loaded
        // before the first gather, so a lane keeps (1 + NC) kNodalBatch loads in flight
        for (int t0 = sub; t0 < len; t0 += kNodalBatch * LPR) {
          int c[kNodalBatch];
          TM v[NC][kNodalBatch];
#pragma unroll
          for (int u = 0; u < kNodalBatch; ++u) {
            const int t = t0 + u * LPR;
            c[u] = t < len ? ld_csr<LPR>(ci + k0[0] + t) : 0;
#pragma unroll
            for (int j = 0; j < NC; ++j) v[j][u] = t < len ? ld_csr<LPR>(val + k0[j] + t) : TM(0);
          }
#pragma unroll
          for (int u = 0; u < kNodalBatch; ++u) {
            if (c[u] > 0) {
              const TV zc = z[c[u] - 1];
#pragma unroll
              for (int j = 0; j < NC; ++j) acc[j] += (TV)v[j][u] * zc;
            }
          }
        }
      } else {
#pragma unroll 4
        for (int t = sub; t < len; t += LPR) acc[0] += (TV)ld_csr<LPR>(val + k0[0] + t) * z[ld_csr<LPR>(ci + k0[0] + t) - 1];
      }
#pragma unroll
      for (int j = 0; j < NC; ++j) {
#pragma unroll
        for (int o = LPR / 2; o > 0; o >>= 1) acc[j] += __shfl_down_sync(0xffffffffu, acc[j], o, LPR);
      }
      if (valid && sub == 0) {
#pragma unroll
        for (int j = 0; j < NC; ++j) {
          if (j == 0 || multi) {
            const int row = row0 + j * n_node;
            const TV qv = (fixed && fixed[row]) ? TV(0) : acc[j] * g;
            q[row] = qv;
            dot += z[row] * g * qv;
          }
        }
      }
    }
  }
  const double b = block_sum(dot);
  if (threadIdx.x == 0) red[blockIdx.x] = b;
  if (last_block(&sc->ticket1)) {
    const double d = ordered_sum(red, gridDim.x);
    if (threadIdx.x == 0) {
      if (!done) {
        sc->delta = d;
        if (!isfinite(d)) { sc->bad = 1; sc->done = 1; }
      }
      sc->pending = 0;
      sc->ticket1 = 0;
    }
  }
}

// Clears *ok unless the rows node, node + n_node, ..., node + (nc - 1) n_node of every node hold
// the same column list (one warp a node).
__global__ void nodal_rows_check(int n_node, int nc, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                 int* ok) {
  const int lane = threadIdx.x & 31, warps = gridDim.x * (blockDim.x / 32);
  for (int node = (blockIdx.x * blockDim.x + threadIdx.x) / 32; node < n_node; node += warps) {
    const int k0 = rp[node] - 1, len = rp[node + 1] - 1 - k0;
    bool same = true;
    for (int j = 1; j < nc; ++j) {
      const int r = node + j * n_node, kj = rp[r] - 1;
      if (rp[r + 1] - 1 - kj != len) { same = false; break; }
      for (int t = lane; t < len; t += 32) same &= ci[k0 + t] == ci[kj + t];
    }
    if (!__all_sync(0xffffffffu, same) && lane == 0) *ok = 0;
  }
}

// (B): v_{j+1} (into vold), z_{j+1} = minv v_{j+1}, gamma_{j+1}; last block: rotation.
template <typename TV>
__global__ void __launch_bounds__(kThreads)
minres_lanczos(int n, const TV* __restrict__ q, const TV* __restrict__ vcur, TV* __restrict__ vold,
               const TV* __restrict__ minv, TV* __restrict__ znew, double* red, MinresScalars* sc) {
  if (sc->done) return;
  const TV a = (TV)(sc->delta / sc->gamma), b = (TV)(sc->gamma / sc->gamma_old);
  // partials in the vector type (FP32 for the inner solves: no FP64 conversions per entry), warp
  // totals and the grid sum in FP64
  TV acc = TV(0);
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const TV vn = q[i] - a * vcur[i] - b * vold[i];
    vold[i] = vn;
    const TV zn = minv[i] * vn;
    znew[i] = zn;
    acc += zn * vn;
  }
  const double bs = block_sum(acc);
  if (threadIdx.x == 0) red[blockIdx.x] = bs;
  if (last_block(&sc->ticket2)) {
    const double g2 = ordered_sum(red, gridDim.x);
    if (threadIdx.x == 0) {
      const double gn = sqrt(fmax(g2, 0.0)), g = sc->gamma, d = sc->delta;
      const double a0 = sc->c * d - sc->c_old * sc->s * g;
      const double a1 = hypot(a0, gn);
      if (!(g2 >= 0.0) || !isfinite(g2) || !(a1 > 0.0)) {
        sc->bad = 1;
        sc->done = 1;
      } else {
        const double cn = a0 / a1, sn = gn / a1;
        sc->a1 = a1;
        sc->a2 = sc->s * d + sc->c_old * sc->c * g;
        sc->a3 = sc->s_old * g;
        sc->ceta = cn * sc->eta;
        sc->zs_prev = 1.0 / g;
        sc->eta = -sn * sc->eta;
        sc->gamma_old = g;
        sc->gamma = gn;
        sc->c_old = sc->c;
        sc->c = cn;
        sc->s_old = sc->s;
        sc->s = sn;
        sc->pending = 1;
        sc->it += 1;
        if (fabs(sc->eta) <= sc->tol || gn == 0.0) sc->done = 2;
      }
      sc->ticket2 = 0;
    }
  }
}

// Start from the FP64 residual r64 (0 on fixed rows): v_1 = r64, v_0 = 0, z_1 = minv v_1,
// w = 0, gamma_1 = sqrt(<z_1, v_1>), eta = gamma_1, tol = rtol_m gamma_1; optionally x = 0.
template <typename TV, typename TX>
__global__ void __launch_bounds__(kThreads)
minres_start(int n, const double* __restrict__ r64, const TV* __restrict__ minv, TV* __restrict__ v1,
             TV* __restrict__ v0, TV* __restrict__ z1, TV* __restrict__ w0, TV* __restrict__ w1, TX* __restrict__ x,
             bool zero_x, double* red, MinresScalars* sc, double rtol_m) {
  double acc = 0.0;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const TV v = (TV)r64[i];
    const TV z = minv[i] * v;
    v1[i] = v; v0[i] = TV(0); z1[i] = z; w0[i] = TV(0); w1[i] = TV(0);
    if (zero_x) x[i] = TX(0);
    acc += (double)z * (double)v;
  }
  const double bs = block_sum(acc);
  if (threadIdx.x == 0) red[blockIdx.x] = bs;
  if (last_block(&sc->ticket2)) {
    const double g2 = ordered_sum(red, gridDim.x);
    if (threadIdx.x == 0) {
      const double g = sqrt(fmax(g2, 0.0));
      sc->gamma = g; sc->gamma_old = 1.0; sc->delta = 0.0;
      sc->c = sc->c_old = 1.0; sc->s = sc->s_old = 0.0;
      sc->eta = g; sc->tol = rtol_m * g;
      sc->pending = 0; sc->it = 0; sc->ticket1 = 0; sc->ticket2 = 0;
      sc->bad = (!(g2 >= 0.0) || !isfinite(g2)) ? 1 : 0;
      sc->done = sc->bad ? 1 : (g == 0.0 ? 2 : 0);
    }
  }
}

// Effective preconditioner: the caller's minv (must be > 0 on free rows) or, when NULL,
// 1/|a_ii| with 1 for a zero diagonal (PETSc's Jacobi convention); 0 on fixed rows.
__global__ void minres_minv(int n, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                            const double* __restrict__ val, const double* __restrict__ user,
                            const uint8_t* __restrict__ fixed, double* __restrict__ m64, float* __restrict__ m32,
                            unsigned* err) {
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < n; row += gridDim.x * blockDim.x) {
    double m = 0.0;
    if (!(fixed && fixed[row])) {
      if (user) {
        m = user[row];
        if (!(m > 0.0) || !isfinite(m)) { gfe_raise(err, GFE_DEVERR_NONFINITE); m = 0.0; }
      } else {
        double d = 0.0;
        for (int k = rp[row] - 1; k < rp[row + 1] - 1; ++k)
          if (ci[k] == row + 1) { d = val[k]; break; }
        m = (d != 0.0 && isfinite(d)) ? 1.0 / fabs(d) : 1.0;
      }
    }
    m64[row] = m;
    if (m32) m32[row] = (float)m;
  }
}

// Node grouping of the MINRES product: n_node > 0 takes minres_spmv_nodal with nc components.
struct NodalRows {
  int n_node = 0, nc = 1;
};

template <typename TM, typename TV, typename TX>
void launch_minres_spmv(int lpr, int grid, cudaStream_t s, int n, const int32_t* rp, const int32_t* ci,
                        const TM* val, const TV* z, TV* q, const uint8_t* fixed, const TV* zprev, TV* wold,
                        const TV* wnew, TX* x, double* red, MinresScalars* sc, NodalRows nodal) {
#define GFE_MINRES_NODAL(L, C)                                                                                 \
  minres_spmv_nodal<TM, TV, TX, L, C><<<std::min(grid, kNodalBlocks * gfe::sm_count()), kThreads, 0, s>>>(         \
      n, nodal.n_node, rp, ci, val, z, q, fixed, zprev, wold, wnew, x, red, sc)
  if constexpr (std::is_same<TV, float>::value) {
   if (nodal.n_node > 0) {
    if (nodal.nc == 3) {
      if (lpr == 32) GFE_MINRES_NODAL(32, 3);
      else if (lpr == 16) GFE_MINRES_NODAL(16, 3);
      else GFE_MINRES_NODAL(8, 3);
    } else {
      if (lpr == 32) GFE_MINRES_NODAL(32, 2);
      else if (lpr == 16) GFE_MINRES_NODAL(16, 2);
      else GFE_MINRES_NODAL(8, 2);
    }
    return;
   }
  }
#undef GFE_MINRES_NODAL
#define GFE_MINRES_SPMV(L) \
  minres_spmv<TM, TV, TX, L><<<grid, kThreads, 0, s>>>(n, rp, ci, val, z, q, fixed, zprev, wold, wnew, x, red, sc)
  if (lpr == 32) GFE_MINRES_SPMV(32);
  else if (lpr == 16) GFE_MINRES_SPMV(16);
  else if (lpr == 8) GFE_MINRES_SPMV(8);
  else GFE_MINRES_SPMV(1);
#undef GFE_MINRES_SPMV
}

// Runs MINRES iterations on started vectors (V[1] = v_1, V[0] = 0, Z[1] = z_1, W = 0).
template <typename TM, typename TV, typename TX>
int run_minres(cudaStream_t s, int n, const int32_t* rp, const int32_t* ci, const TM* val, const uint8_t* fixed,
               const TV* minv, TX* x, TV* const V[2], TV* const Z[2], TV* const W[2], TV* q, double* red,
               MinresScalars* sc, MinresScalars* sc_host, int lpr, int grid, int max_iters, int chunk,
               NodalRows nodal) {
  int j = 1;
  while (j <= max_iters) {
    const int k = std::min(chunk, max_iters - j + 1);
    for (int t = 0; t < k; ++t, ++j) {
      void* prof = gfe::stage_begin(GFE_STAGE_SPMV, s);
      launch_minres_spmv<TM, TV, TX>(lpr, grid, s, n, rp, ci, val, Z[j & 1], q, fixed, Z[(j + 1) & 1], W[j & 1],
                                     W[(j + 1) & 1], x, red, sc, nodal);
      gfe::stage_end(GFE_STAGE_SPMV, prof, s, 1);
      minres_lanczos<TV><<<grid, kThreads, 0, s>>>(n, q, V[j & 1], V[(j + 1) & 1], minv, Z[(j + 1) & 1], red, sc);
    }
    GFE_CUDA_TRY(cudaGetLastError());
    GFE_CUDA_TRY(cudaMemcpyAsync(sc_host, sc, sizeof(MinresScalars), cudaMemcpyDeviceToHost, s));
    GFE_CUDA_TRY(cudaStreamSynchronize(s));
    if (sc_host->done) break;
  }
  // the update of the last completed iteration is deferred to the next (A) launch: flush it
  launch_minres_spmv<TM, TV, TX>(lpr, grid, s, n, rp, ci, val, Z[j & 1], q, fixed, Z[(j + 1) & 1], W[j & 1],
                                 W[(j + 1) & 1], x, red, sc, nodal);
  GFE_CUDA_TRY(cudaGetLastError());
  return GFE_OK;
}

// lanes per row of the MINRES SpMV: long rows (the u-p tangent has ~200 entries a row) use 8 lanes
// in FP64, so the shuffle reduction adds little to the FP64-pipe work, and a full warp in FP32
int minres_lpr(double avg, bool fp64) {
  if (fp64) return avg >= 64 ? 8 : 1;
  return avg >= 96 ? 32 : (avg >= 48 ? 16 : 8);
}

int minres_solve(const char* fn, int32_t n, int32_t n_node, int32_t n_comp, const int32_t* row_ptr,
                 const int32_t* col_idx, const double* values, const float* values32, const double* minv,
                 const double* f, const uint8_t* fixed, double* x, double rtol, int32_t max_iters, int32_t precision,
                 int32_t* iters_host, double* rel_host, int32_t* nodal_used, void* stream);

}  // namespace

extern "C" int gfe_minres_solve(int32_t n, const int32_t* row_ptr, const int32_t* col_idx, const double* values,
                                const float* values32, const double* minv, const double* f, const uint8_t* fixed,
                                double* x, double rtol, int32_t max_iters, int32_t precision, int32_t* iters_host,
                                double* rel_host, void* stream) {
  return minres_solve("gfe_minres_solve", n, 0, 1, row_ptr, col_idx, values, values32, minv, f, fixed, x, rtol,
                      max_iters, precision, iters_host, rel_host, nullptr, stream);
}

extern "C" int gfe_minres_solve_nodal(int32_t n, int32_t n_node, int32_t n_comp, const int32_t* row_ptr,
                                      const int32_t* col_idx, const double* values, const float* values32,
                                      const double* minv, const double* f, const uint8_t* fixed, double* x,
                                      double rtol, int32_t max_iters, int32_t precision, int32_t* iters_host,
                                      double* rel_host, int32_t* nodal_used, void* stream) {
  return minres_solve("gfe_minres_solve_nodal", n, n_node, n_comp, row_ptr, col_idx, values, values32, minv, f,
                      fixed, x, rtol, max_iters, precision, iters_host, rel_host, nodal_used, stream);
}

namespace {

int minres_solve(const char* fn, int32_t n, int32_t n_node, int32_t n_comp, const int32_t* row_ptr,
                 const int32_t* col_idx, const double* values, const float* values32, const double* minv,
                 const double* f, const uint8_t* fixed, double* x, double rtol, int32_t max_iters, int32_t precision,
                 int32_t* iters_host, double* rel_host, int32_t* nodal_used, void* stream) {
  using namespace gfe;
  if (nodal_used) *nodal_used = 0;
  if (n <= 0 || !row_ptr || !col_idx || !values || !x || !(rtol > 0.0) || max_iters <= 0)
    return set_error(GFE_ERR_ARG, "%s: invalid arguments", fn);
  if (n_node < 0 || n_comp < 1 || n_comp > 3 || (int64_t)n_node * n_comp > n)
    return set_error(GFE_ERR_ARG, "%s: need 0 <= n_node, 1 <= n_comp <= 3, n_node * n_comp <= n", fn);
  if (precision != GFE_FP64 && precision != GFE_MIXED) return set_error(GFE_ERR_ARG, "%s: unknown precision", fn);
  if (precision == GFE_MIXED && !values32)
    return set_error(GFE_ERR_ARG, "%s: mixed precision needs the FP32 copy of the matrix", fn);
  cudaStream_t s = as_stream(stream);
  unsigned* err = device_error_word();
  int32_t nnz1 = 0;
  GFE_CUDA_TRY(cudaMemcpyAsync(&nnz1, row_ptr + n, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  GFE_CUDA_TRY(cudaStreamSynchronize(s));
  const bool fp64 = precision == GFE_FP64;
  const int lpr = minres_lpr((double)(nnz1 - 1) / n, fp64);
  const int grid = 8 * sm_count();
  const int chunk = 50;
  const size_t nb = (size_t)n, vbytes = fp64 ? sizeof(double) : sizeof(float);
  // pieces: m64, m32, r64, eight vectors of the working type (V0 V1 Z0 Z1 W0 W1 q d), the block
  // partials, the MINRES scalars, a Scalars block for the norm kernel and the norm result
  const int pieces = 15;
  const size_t bytes = nb * sizeof(double) * 2 + nb * sizeof(float) + nb * vbytes * 8 + sizeof(double) * grid +
                       sizeof(MinresScalars) + sizeof(Scalars) + sizeof(double) + sizeof(int) + (pieces + 2) * 256;
  char* buf = nullptr;
  int rc = scratch_alloc((void**)&buf, bytes, s, "MINRES vectors");
  if (rc) return rc;
  char* base = buf;
  auto carve = [&](size_t b) {
    char* p = buf;
    buf += (b + 255) & ~size_t(255);
    return p;
  };
  double* m64 = (double*)carve(nb * sizeof(double));
  float* m32 = (float*)carve(nb * sizeof(float));
  double* r64 = (double*)carve(nb * sizeof(double));
  void* vec[8];
  for (int i = 0; i < 8; ++i) vec[i] = carve(nb * vbytes);
  double* red = (double*)carve(sizeof(double) * grid);
  MinresScalars* sc = (MinresScalars*)carve(sizeof(MinresScalars));
  Scalars* nsc = (Scalars*)carve(sizeof(Scalars));
  double* r2dev = (double*)carve(sizeof(double));
  int* nodal_ok = (int*)carve(sizeof(int));
  MinresScalars sh{};
  double b2 = 0.0, r2 = 0.0;
  int total_it = 0;
  // r64 = f - A x on free rows and r2 = ||r64||^2 in the preconditioner's norm, sum minv_i r_i^2
  // (the norm MINRES minimises; PETSc's default norm for KSPMINRES)
  auto true_residual = [&]() -> int {
    cg_residual<double><<<grid, kThreads, 0, s>>>(n, row_ptr, col_idx, values, f, fixed, x, r64);
    norm2_kernel<<<grid, kThreads, 0, s>>>(n, r64, red, nsc, r2dev, m64);
    GFE_CUDA_TRY(cudaMemcpyAsync(&r2, r2dev, sizeof(double), cudaMemcpyDeviceToHost, s));
    GFE_CUDA_TRY(cudaStreamSynchronize(s));
    return GFE_OK;
  };
  GFE_CUDA_TRY(cudaMemsetAsync(sc, 0, sizeof(MinresScalars), s));
  GFE_CUDA_TRY(cudaMemsetAsync(nsc, 0, sizeof(Scalars), s));
  minres_minv<<<grid, kThreads, 0, s>>>(n, row_ptr, col_idx, values, minv, fixed, m64, fp64 ? nullptr : m32, err);
  set_dirichlet<<<grid, kThreads, 0, s>>>(n, x, fixed, true);
  // node-grouped product only where the rows of each node share their column list (and there are
  // at least two components to group), and only in the FP32 Krylov iterations of GFE_MIXED: the
  // FP64 product is bound by the FP64 pipe, and grouped it was 19 % slower (64^3 u-p tangent)
  NodalRows nodal;
  int nodal_host = 0;
  if (n_node > 0 && n_comp > 1 && !fp64) {
    const int one = 1;
    GFE_CUDA_TRY(cudaMemcpyAsync(nodal_ok, &one, sizeof(int), cudaMemcpyHostToDevice, s));
    nodal_rows_check<<<grid, kThreads, 0, s>>>(n_node, n_comp, row_ptr, col_idx, nodal_ok);
    GFE_CUDA_TRY(cudaMemcpyAsync(&nodal_host, nodal_ok, sizeof(int), cudaMemcpyDeviceToHost, s));
  }
  rc = true_residual();
  if (rc) { scratch_free(base, s); return rc; }
  if (nodal_host) {
    nodal.n_node = n_node;
    nodal.nc = n_comp;
    if (nodal_used) *nodal_used = 1;
  }
  b2 = r2;
  if (b2 == 0.0) {
    if (iters_host) *iters_host = 0;
    if (rel_host) *rel_host = 0.0;
    scratch_free(base, s);
    return GFE_OK;
  }
  if (fp64) {
    double* V[2] = {(double*)vec[0], (double*)vec[1]};
    double* Z[2] = {(double*)vec[2], (double*)vec[3]};
    double* W[2] = {(double*)vec[4], (double*)vec[5]};
    double* q = (double*)vec[6];
    // the recurrence tracks the M^-1-norm of the residual; a round aims a little below the target
    // and restarts from the true residual in the rare case that rounding left it above
    for (int round = 0; round < 6 && rc == GFE_OK; ++round) {
      minres_start<double, double><<<grid, kThreads, 0, s>>>(n, r64, m64, V[1], V[0], Z[1], W[0], W[1], x, false, red,
                                                             sc, 0.7 * rtol * std::sqrt(b2 / r2));
      rc = run_minres<double, double, double>(s, n, row_ptr, col_idx, values, fixed, m64, x, V, Z, W, q, red, sc, &sh,
                                              lpr, grid, max_iters - total_it, chunk, nodal);
      total_it += sh.it;
      if (rc) break;
      rc = true_residual();
      if (rc || sh.bad || r2 <= rtol * rtol * b2 || r2 == 0.0 || total_it >= max_iters) break;
    }
  } else {
    // iterative refinement: FP64 residual outside, FP32 MINRES on the FP32 matrix for the correction
    float* V[2] = {(float*)vec[0], (float*)vec[1]};
    float* Z[2] = {(float*)vec[2], (float*)vec[3]};
    float* W[2] = {(float*)vec[4], (float*)vec[5]};
    float* q = (float*)vec[6];
    float* d = (float*)vec[7];
    for (int outer = 0; outer < 64 && rc == GFE_OK; ++outer) {
      // the reduction still needed, halved, but no tighter than FP32 MINRES usefully reaches: a
      // floor of 5e-6 (rather than 2e-5) saves refinement restarts, 12 % of the 24^3 mixed
      // Newton solve at the same iteration counts and error
      const double inner_rtol = std::max(0.7 * rtol * std::sqrt(b2 / r2), 5e-6);
      minres_start<float, float><<<grid, kThreads, 0, s>>>(n, r64, m32, V[1], V[0], Z[1], W[0], W[1], d, true, red, sc,
                                                           inner_rtol);
      rc = run_minres<float, float, float>(s, n, row_ptr, col_idx, values32, fixed, m32, d, V, Z, W, q, red, sc, &sh,
                                           lpr, grid, max_iters - total_it, chunk, nodal);
      total_it += sh.it;
      if (rc) break;
      add_correction<<<grid, kThreads, 0, s>>>(n, x, d, fixed);
      rc = true_residual();
      if (rc || sh.bad || r2 <= rtol * rtol * b2 || total_it >= max_iters) break;
    }
  }
  cudaError_t e = cudaStreamSynchronize(s);
  scratch_free(base, s);
  if (rc) return rc;
  if (e != cudaSuccess) return set_error(GFE_ERR_CUDA, "%s: %s", fn, cudaGetErrorString(e));
  const double rel = std::sqrt(r2 / b2);
  if (iters_host) *iters_host = total_it;
  if (rel_host) *rel_host = rel;
  if (sh.bad)
    return set_error(GFE_ERR_NUMERIC, "%s: breakdown (indefinite preconditioner, singular system or non-finite value)",
                     fn);
  if (!(rel <= rtol))
    return set_error(GFE_ERR_NOCONV, "%s: relative residual %.3e above %.3e after %d iterations", fn, rel, rtol,
                     total_it);
  return GFE_OK;
}

}  // namespace

// ---------------------------------------------------------------------------------------------
// Restarted GMRES for non-symmetric systems
// ---------------------------------------------------------------------------------------------
// Iron's default linear solver inside Newton is PETSc GMRES with restart 30 and classical
// Gram-Schmidt without refinement (src/solver_routines.F90:11320-11369); Iron's analytic Jacobian
// of the mixed u-p Mooney-Rivlin element is not symmetric (its u-p and p-u blocks differ), so it
// needs a non-symmetric Krylov method.  GMRES(m) with right preconditioning by a diagonal M^-1:
// the Hessenberg residual estimate |g_{j+1}| is the true residual norm, every cycle starts from
// the FP64 residual b - A x formed with the FP64 matrix, and the correction M^-1 V y is added to x
// in FP64.  With precision GFE_MIXED the Krylov basis and the matrix of the cycle are FP32, which
// makes each restart an FP64 iterative-refinement step.
//
// One iteration is three kernels, all reading the column index j from device memory so the host
// launches whole cycles without synchronising: (1) w = s A M^-1 v_j (s = 1 / ||v_j|| pending);
// (2) normalise v_j in place and h_kj = <w, v_k>, k <= j (a 2-D grid, one column k per blockIdx.y);
// (3) w -= sum_k h_kj v_k into v_{j+1}, ||w|| and, in the last block, the Givens rotations and the
// convergence / end-of-cycle flags.  At the end of a cycle one thread solves H y = g and a kernel
// adds M^-1 V y to x.
namespace {

constexpr int kGmresMaxRestart = 64;

struct GmresScalars {
  double H[(kGmresMaxRestart + 1) * kGmresMaxRestart];  // column-major, leading dimension m + 1
  double cs[kGmresMaxRestart], sn[kGmresMaxRestart], g[kGmresMaxRestart + 1], y[kGmresMaxRestart];
  double vscale, tol;
  int j, cols, done, bad, it, ticket1, ticket2;
};

template <typename TM, typename TV, int LPR>
__global__ void __launch_bounds__(kThreads)
gmres_spmv(int n, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci, const TM* __restrict__ val,
           const TV* __restrict__ minv, const TV* __restrict__ V, size_t ldv, TV* __restrict__ w,
           const uint8_t* __restrict__ fixed, GmresScalars* sc) {
  if (sc->done) return;
  const TV* __restrict__ v = V + (size_t)sc->j * ldv;
  const TV s = (TV)sc->vscale;
  constexpr int RPB = kThreads / LPR;
  const int sub = threadIdx.x % LPR, grp = threadIdx.x / LPR;
  for (int base = blockIdx.x * RPB; base < n; base += gridDim.x * RPB) {
    const int row = base + grp;
    const bool valid = row < n;
    const int k0 = valid ? __ldg(rp + row) - 1 : 0, k1 = valid ? __ldg(rp + row + 1) - 1 : 0;
    TV acc = TV(0);
#pragma unroll 4
    for (int k = k0 + sub; k < k1; k += LPR) {
      const int c = ld_csr<LPR>(ci + k) - 1;
      acc += (TV)ld_csr<LPR>(val + k) * (minv[c] * v[c]);
    }
#pragma unroll
    for (int o = LPR / 2; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o, LPR);
    if (valid && sub == 0) w[row] = (fixed && fixed[row]) ? TV(0) : acc * s;
  }
}

// blockIdx.y = k: partial <w, v_k> for k <= j; the k == j blocks normalise v_j first.
template <typename TV>
__global__ void __launch_bounds__(kThreads)
gmres_dots(int n, TV* __restrict__ V, size_t ldv, const TV* __restrict__ w, double* red, GmresScalars* sc) {
  if (sc->done) return;
  const int j = sc->j, k = blockIdx.y;
  if (k > j) return;
  TV* __restrict__ v = V + (size_t)k * ldv;
  double acc = 0.0;
  if (k == j) {
    const TV s = (TV)sc->vscale;
    for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
      const TV vi = v[i] * s;
      v[i] = vi;
      acc += (double)vi * (double)w[i];
    }
  } else {
    for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads)
      acc += (double)v[i] * (double)w[i];
  }
  const double b = block_sum(acc);
  if (threadIdx.x == 0) red[(size_t)k * gridDim.x + blockIdx.x] = b;
  // ticket over the (j + 1) * gridDim.x active blocks
  __shared__ bool amlast;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const int t = atomicAdd(&sc->ticket1, 1);
    amlast = (t == (j + 1) * (int)gridDim.x - 1);
  }
  __syncthreads();
  if (!amlast) return;
  const int ldh = kGmresMaxRestart + 1;
  for (int kk = 0; kk <= j; ++kk) {
    const double h = ordered_sum(red + (size_t)kk * gridDim.x, gridDim.x);
    if (threadIdx.x == 0) sc->H[(size_t)j * ldh + kk] = h;
  }
  if (threadIdx.x == 0) sc->ticket1 = 0;
}

// w -= sum_{k<=j} h_kj v_k, stored into v_{j+1}; ||w||^2; last block: rotations and flags.
template <typename TV>
__global__ void __launch_bounds__(kThreads)
gmres_orth(int n, TV* __restrict__ V, size_t ldv, const TV* __restrict__ w, double* red, GmresScalars* sc, int m) {
  if (sc->done) return;
  const int j = sc->j;
  const int ldh = kGmresMaxRestart + 1;
  __shared__ TV hs[kGmresMaxRestart + 1];
  for (int k = threadIdx.x; k <= j; k += kThreads) hs[k] = (TV)sc->H[(size_t)j * ldh + k];
  __syncthreads();
  TV* __restrict__ vn = V + (size_t)(j + 1) * ldv;
  double acc = 0.0;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    TV wi = w[i];
    for (int k = 0; k <= j; ++k) wi -= hs[k] * V[(size_t)k * ldv + i];
    vn[i] = wi;
    acc += (double)wi * (double)wi;
  }
  const double b = block_sum(acc);
  if (threadIdx.x == 0) red[blockIdx.x] = b;
  if (last_block(&sc->ticket2)) {
    const double hn2 = ordered_sum(red, gridDim.x);
    if (threadIdx.x == 0) {
      double* h = sc->H + (size_t)j * ldh;
      const double hn = sqrt(fmax(hn2, 0.0));
      h[j + 1] = hn;
      for (int k = 0; k < j; ++k) {
        const double t = sc->cs[k] * h[k] + sc->sn[k] * h[k + 1];
        h[k + 1] = -sc->sn[k] * h[k] + sc->cs[k] * h[k + 1];
        h[k] = t;
      }
      const double den = hypot(h[j], h[j + 1]);
      if (!isfinite(hn2) || !(den > 0.0)) {
        sc->bad = 1;
        sc->done = 1;
      } else {
        sc->cs[j] = h[j] / den;
        sc->sn[j] = h[j + 1] / den;
        h[j] = den;
        h[j + 1] = 0.0;
        sc->g[j + 1] = -sc->sn[j] * sc->g[j];
        sc->g[j] = sc->cs[j] * sc->g[j];
        sc->cols = j + 1;
        sc->it += 1;
        sc->vscale = hn > 0.0 ? 1.0 / hn : 0.0;
        if (fabs(sc->g[j + 1]) <= sc->tol || hn == 0.0) sc->done = 2;
        else if (j + 1 == m) sc->done = 3;
        sc->j = j + 1;
      }
      sc->ticket2 = 0;
    }
  }
}

// back substitution H y = g on the cols x cols upper triangle (one thread)
__global__ void gmres_solve_y(GmresScalars* sc) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int c = sc->cols, ldh = kGmresMaxRestart + 1;
  for (int r = c - 1; r >= 0; --r) {
    double s = sc->g[r];
    for (int k = r + 1; k < c; ++k) s -= sc->H[(size_t)k * ldh + r] * sc->y[k];
    sc->y[r] = s / sc->H[(size_t)r * ldh + r];
  }
}

template <typename TV>
__global__ void __launch_bounds__(kThreads)
gmres_update_x(int n, const TV* __restrict__ V, size_t ldv, const TV* __restrict__ minv, double* __restrict__ x,
               const GmresScalars* sc) {
  __shared__ double ys[kGmresMaxRestart];
  const int c = sc->cols;
  for (int k = threadIdx.x; k < c; k += kThreads) ys[k] = sc->y[k];
  __syncthreads();
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    double s = 0.0;
    for (int k = 0; k < c; ++k) s += ys[k] * (double)V[(size_t)k * ldv + i];
    x[i] += (double)minv[i] * s;
  }
}

// cycle start: v_0 = r64 (raw; its norm is applied by the first dots kernel), g = beta e_1
template <typename TV>
__global__ void gmres_start(int n, const double* __restrict__ r64, TV* __restrict__ v0, GmresScalars* sc,
                            double beta, double tol) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v0[i] = (TV)r64[i];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    for (int k = 0; k <= kGmresMaxRestart; ++k) sc->g[k] = 0.0;
    sc->g[0] = beta;
    sc->vscale = 1.0 / beta;
    sc->tol = tol;
    sc->j = 0; sc->cols = 0; sc->done = 0; sc->bad = 0; sc->it = 0; sc->ticket1 = 0; sc->ticket2 = 0;
  }
}

template <typename TM, typename TV>
void launch_gmres_spmv(int lpr, int grid, cudaStream_t s, int n, const int32_t* rp, const int32_t* ci, const TM* val,
                       const TV* minv, const TV* V, size_t ldv, TV* w, const uint8_t* fixed, GmresScalars* sc) {
#define GFE_GMRES_SPMV(L) gmres_spmv<TM, TV, L><<<grid, kThreads, 0, s>>>(n, rp, ci, val, minv, V, ldv, w, fixed, sc)
  if (lpr == 32) GFE_GMRES_SPMV(32);
  else if (lpr == 16) GFE_GMRES_SPMV(16);
  else if (lpr == 8) GFE_GMRES_SPMV(8);
  else GFE_GMRES_SPMV(1);
#undef GFE_GMRES_SPMV
}

// one GMRES cycle of at most m iterations from r64 (||r64|| = beta); adds the correction to x
template <typename TM, typename TV>
int gmres_cycle(cudaStream_t s, int n, const int32_t* rp, const int32_t* ci, const TM* val, const uint8_t* fixed,
                const TV* minv, double* x, const double* r64, double beta, double tol_abs, TV* V, size_t ldv, TV* w,
                double* red, GmresScalars* sc, int* it_host, int* flag_host, int lpr, int grid, int m) {
  gmres_start<TV><<<grid, kThreads, 0, s>>>(n, r64, V, sc, beta, tol_abs);
  for (int t = 0; t < m; ++t) {
    void* prof = gfe::stage_begin(GFE_STAGE_SPMV, s);
    launch_gmres_spmv<TM, TV>(lpr, grid, s, n, rp, ci, val, minv, V, ldv, w, fixed, sc);
    gfe::stage_end(GFE_STAGE_SPMV, prof, s, 1);
    gmres_dots<TV><<<dim3(grid, t + 1), kThreads, 0, s>>>(n, V, ldv, w, red, sc);
    gmres_orth<TV><<<grid, kThreads, 0, s>>>(n, V, ldv, w, red, sc, m);
  }
  gmres_solve_y<<<1, 32, 0, s>>>(sc);
  gmres_update_x<TV><<<grid, kThreads, 0, s>>>(n, V, ldv, minv, x, sc);
  GFE_CUDA_TRY(cudaGetLastError());
  int hv[2];
  GFE_CUDA_TRY(cudaMemcpyAsync(hv, &sc->done, sizeof(int) * 2, cudaMemcpyDeviceToHost, s));
  int itv = 0;
  GFE_CUDA_TRY(cudaMemcpyAsync(&itv, &sc->it, sizeof(int), cudaMemcpyDeviceToHost, s));
  GFE_CUDA_TRY(cudaStreamSynchronize(s));
  *flag_host = hv[1] ? -1 : hv[0];
  *it_host = itv;
  return GFE_OK;
}

}  // namespace

extern "C" int gfe_gmres_solve(int32_t n, const int32_t* row_ptr, const int32_t* col_idx, const double* values,
                               const float* values32, const double* minv, const double* f, const uint8_t* fixed,
                               double* x, double rtol, int32_t max_iters, int32_t restart, int32_t precision,
                               int32_t* iters_host, double* rel_host, void* stream) {
  using namespace gfe;
  const char* fn = "gfe_gmres_solve";
  if (n <= 0 || !row_ptr || !col_idx || !values || !x || !(rtol > 0.0) || max_iters <= 0)
    return set_error(GFE_ERR_ARG, "%s: invalid arguments", fn);
  if (restart < 1 || restart > kGmresMaxRestart)
    return set_error(GFE_ERR_ARG, "%s: restart %d outside 1..%d", fn, restart, kGmresMaxRestart);
  if (precision != GFE_FP64 && precision != GFE_MIXED) return set_error(GFE_ERR_ARG, "%s: unknown precision", fn);
  if (precision == GFE_MIXED && !values32)
    return set_error(GFE_ERR_ARG, "%s: mixed precision needs the FP32 copy of the matrix", fn);
  cudaStream_t s = as_stream(stream);
  unsigned* err = device_error_word();
  int32_t nnz1 = 0;
  GFE_CUDA_TRY(cudaMemcpyAsync(&nnz1, row_ptr + n, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  GFE_CUDA_TRY(cudaStreamSynchronize(s));
  const bool fp64 = precision == GFE_FP64;
  const int lpr = minres_lpr((double)(nnz1 - 1) / n, fp64);
  const int grid = 2 * sm_count();
  const int m = restart;
  const size_t nb = (size_t)n, vbytes = fp64 ? sizeof(double) : sizeof(float);
  const size_t ldv = (nb + 63) & ~size_t(63);
  // pieces: m64, m32, r64, basis (m + 1 columns), w, partials (m + 1 columns of grid), scalars,
  // norm-kernel scalars, norm result
  const int pieces = 9;
  const size_t bytes = nb * sizeof(double) * 2 + nb * sizeof(float) + ldv * vbytes * (m + 1) + nb * vbytes +
                       sizeof(double) * grid * (m + 1) + sizeof(GmresScalars) + sizeof(Scalars) + sizeof(double) +
                       (pieces + 1) * 256;
  char* buf = nullptr;
  int rc = scratch_alloc((void**)&buf, bytes, s, "GMRES vectors");
  if (rc) return rc;
  char* base = buf;
  auto carve = [&](size_t b) {
    char* p = buf;
    buf += (b + 255) & ~size_t(255);
    return p;
  };
  double* m64 = (double*)carve(nb * sizeof(double));
  float* m32 = (float*)carve(nb * sizeof(float));
  double* r64 = (double*)carve(nb * sizeof(double));
  void* Vb = carve(ldv * vbytes * (m + 1));
  void* wb = carve(nb * vbytes);
  double* red = (double*)carve(sizeof(double) * grid * (m + 1));
  GmresScalars* sc = (GmresScalars*)carve(sizeof(GmresScalars));
  Scalars* nsc = (Scalars*)carve(sizeof(Scalars));
  double* r2dev = (double*)carve(sizeof(double));
  double b2 = 0.0, r2 = 0.0;
  int total_it = 0, flag = 0, bad = 0;
  auto true_residual = [&]() -> int {
    cg_residual<double><<<grid, kThreads, 0, s>>>(n, row_ptr, col_idx, values, f, fixed, x, r64);
    norm2_kernel<<<grid, kThreads, 0, s>>>(n, r64, red, nsc, r2dev);
    GFE_CUDA_TRY(cudaMemcpyAsync(&r2, r2dev, sizeof(double), cudaMemcpyDeviceToHost, s));
    GFE_CUDA_TRY(cudaStreamSynchronize(s));
    return GFE_OK;
  };
  GFE_CUDA_TRY(cudaMemsetAsync(sc, 0, sizeof(GmresScalars), s));
  GFE_CUDA_TRY(cudaMemsetAsync(nsc, 0, sizeof(Scalars), s));
  minres_minv<<<grid, kThreads, 0, s>>>(n, row_ptr, col_idx, values, minv, fixed, m64, fp64 ? nullptr : m32, err);
  set_dirichlet<<<grid, kThreads, 0, s>>>(n, x, fixed, true);
  rc = true_residual();
  if (rc) { scratch_free(base, s); return rc; }
  b2 = r2;
  if (b2 == 0.0) {
    if (iters_host) *iters_host = 0;
    if (rel_host) *rel_host = 0.0;
    scratch_free(base, s);
    return GFE_OK;
  }
  const double target2 = rtol * rtol * b2;
  while (total_it < max_iters && rc == GFE_OK) {
    const double beta = std::sqrt(r2);
    // aim each cycle at half the target so the true residual (which the FP64 check below
    // measures) lands under it despite rounding in the recurrence
    const double tol_abs = 0.5 * rtol * std::sqrt(b2);
    const int mm = std::min(m, max_iters - total_it);
    int it = 0;
    if (fp64)
      rc = gmres_cycle<double, double>(s, n, row_ptr, col_idx, values, fixed, m64, x, r64, beta, tol_abs, (double*)Vb,
                                       ldv, (double*)wb, red, sc, &it, &flag, lpr, grid, mm);
    else
      rc = gmres_cycle<float, float>(s, n, row_ptr, col_idx, values32, fixed, m32, x, r64, beta, tol_abs, (float*)Vb,
                                     ldv, (float*)wb, red, sc, &it, &flag, lpr, grid, mm);
    total_it += it;
    if (rc) break;
    if (flag < 0) { bad = 1; break; }
    rc = true_residual();
    if (rc || r2 <= target2) break;
    if (!isfinite(r2)) { bad = 1; break; }
  }
  cudaError_t e = cudaStreamSynchronize(s);
  scratch_free(base, s);
  if (rc) return rc;
  if (e != cudaSuccess) return set_error(GFE_ERR_CUDA, "%s: %s", fn, cudaGetErrorString(e));
  const double rel = std::sqrt(r2 / b2);
  if (iters_host) *iters_host = total_it;
  if (rel_host) *rel_host = rel;
  if (bad) return set_error(GFE_ERR_NUMERIC, "%s: breakdown (zero Hessenberg diagonal or non-finite value)", fn);
  if (!(rel <= rtol))
    return set_error(GFE_ERR_NOCONV, "%s: relative residual %.3e above %.3e after %d iterations", fn, rel, rtol,
                     total_it);
  return GFE_OK;
}

// ---------------------------------------------------------------------------------------------
// Diagonal preconditioner for the u-p saddle-point matrix [K_uu B^T; B 0]
// ---------------------------------------------------------------------------------------------
namespace {

// u rows (row < n_u): 1/|K_ii| (1 when K_ii = 0); fixed rows 0
__global__ void saddle_minv_u(int n_u, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                              const double* __restrict__ val, const uint8_t* __restrict__ fixed,
                              double* __restrict__ minv) {
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < n_u; row += gridDim.x * blockDim.x) {
    double d = 0.0;
    for (int k = rp[row] - 1; k < rp[row + 1] - 1; ++k)
      if (ci[k] == row + 1) { d = val[k]; break; }
    minv[row] = (fixed && fixed[row]) ? 0.0 : ((d != 0.0 && isfinite(d)) ? 1.0 / fabs(d) : 1.0);
  }
}

// p rows (row >= n_u), one warp each: 1 / sum_{free j < n_u} B_pj^2 / |K_jj| (the diagonal of the
// Schur complement B diag(K_uu)^-1 B^T); 1 when that sum is 0; fixed rows 0.  minv of the u rows
// must already be set (it is |K_jj|^-1 there, 0 on fixed u rows).
__global__ void saddle_minv_p(int n, int n_u, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                              const double* __restrict__ val, const uint8_t* __restrict__ fixed,
                              double* __restrict__ minv) {
  const int lane = threadIdx.x & 31;
  for (int row = n_u + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5); row < n;
       row += (gridDim.x * blockDim.x) >> 5) {
    const int k0 = rp[row] - 1, k1 = rp[row + 1] - 1;
    double s = 0.0;
    for (int k = k0 + lane; k < k1; k += 32) {
      const int j = ci[k] - 1;
      if (j < n_u) s += val[k] * val[k] * minv[j];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) minv[row] = (fixed && fixed[row]) ? 0.0 : ((s > 0.0 && isfinite(s)) ? 1.0 / s : 1.0);
  }
}

}  // namespace

extern "C" int gfe_saddle_preconditioner(int32_t n, int32_t n_u, const int32_t* row_ptr, const int32_t* col_idx,
                                         const double* values, const uint8_t* fixed, double* minv, void* stream) {
  using namespace gfe;
  if (n <= 0 || n_u < 0 || n_u > n || !row_ptr || !col_idx || !values || !minv)
    return set_error(GFE_ERR_ARG, "gfe_saddle_preconditioner: invalid arguments");
  cudaStream_t s = as_stream(stream);
  const int grid = 4 * sm_count();
  if (n_u > 0) saddle_minv_u<<<grid, kThreads, 0, s>>>(n_u, row_ptr, col_idx, values, fixed, minv);
  if (n > n_u) saddle_minv_p<<<grid, kThreads, 0, s>>>(n, n_u, row_ptr, col_idx, values, fixed, minv);
  GFE_LAUNCH_CHECK("gfe_saddle_preconditioner");
  return GFE_OK;
}

// ---------------------------------------------------------------------------------------------
// Allocation-free variant of the FP64 solve
// ---------------------------------------------------------------------------------------------
// Some callers of this library may not allocate device memory at all: host codes that run the
// solve from inside a memory pool they do not own (a framework's caching allocator, a
// statically partitioned serving process), where a cudaMalloc is forbidden.  gfe_cg_solve_noalloc serves them: its working vectors live in one
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
  unsigned dev_err = 0;
  GFE_CUDA_TRY(cudaMemcpyAsync(&b2, red2 + grid - 1, sizeof(double), cudaMemcpyDeviceToHost, s));
  GFE_CUDA_TRY(cudaMemcpyAsync(&dev_err, err, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  GFE_CUDA_TRY(cudaStreamSynchronize(s));
  // this entry point holds no library error word (that word is allocated on first use), so a
  // zero or non-finite diagonal on a free row, which gfe_cg_solve raises as GFE_DEVERR_NONFINITE on
  // the device error word, is returned here as the call's status
  if (dev_err)
    return set_error(GFE_ERR_NUMERIC, "%s: zero or non-finite diagonal entry on a free row (device error bits 0x%x)",
                     fn, dev_err);
  if (b2 == 0.0) {
    if (iters_host) *iters_host = 0;
    if (rel_host) *rel_host = 0.0;
    return GFE_OK;
  }
  // same residual-replacement rounds as gfe_cg_solve
  int total_it = 0;
  r2 = b2;
  for (int round = 0; round < 4; ++round) {
    cg_start<double, double><<<grid, kThreads, 0, s>>>(n, r64, dinv, r, z, p, x, false, round > 0, red, red2, sc,
                                                       0.25 * rtol * rtol * b2 / r2);
    if (round > 0) cg_direction<double><<<grid, kThreads, 0, s>>>(n, p, z, sc);
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
