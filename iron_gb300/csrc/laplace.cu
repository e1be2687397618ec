// laplace.cu -- K1 + K2: trilinear-hex Laplace stiffness, fused with the deterministic CSR scatter.
//
// Element routine: LaplaceEquation_FiniteElementCalculate (src/Laplace_equations_routines.F90:482-552
// standard, :585-707 generalised).  Per Gauss point Iron forms DX_DXI from the interpolated
// geometry, GL = DX_DXI^T DX_DXI, GU = GL^-1, Jacobian = sqrt|det GL|
// (src/coordinate_routines.F90:703-822) and adds
//     K(m,n) += sum_{a,b} dphi_m/dxi_a * GU(a,b) * dphi_n/dxi_b * Jacobian * w_g.
// The same integrand is evaluated here by sum factorisation over the tensor-product 2x2x2 rule:
//  * for a trilinear map dx/dxi_a does not depend on xi_a, so the 9 Jacobian columns are bilinear
//    interpolants of 4 nodal edge differences each;
//  * M_g = GU * Jacobian * w_g = adj(GL) * w_g / sqrt(det GL) (6 numbers per Gauss point);
//  * the contraction over Gauss points is done one xi direction at a time, using that the 1D
//    basis at the 1D Gauss points takes only the values p = (1+1/sqrt3)/2 and q = (1-1/sqrt3)/2,
//    and is symmetrised over (a,b) because GU is symmetric.
// The result equals Iron's element matrix up to floating-point rounding (checked against the
// oracle's literal restatement of Iron's loops).
//
// Scatter: EquationsMatrices_ElementAdd -> MATRIX_VALUES_ADD_DP2 (src/matrix_vector.F90:3202-3240)
// adds each element matrix into fixed CSR storage.  Elements are processed colour by colour (no
// two elements of a colour share a node), so every CSR entry receives at most one read-modify-write
// per colour launch: no atomics, and a summation order fixed by the colouring.
#include <cmath>

#include "gfe_internal.cuh"

namespace {

constexpr int kBlock = 128;

__host__ __device__ constexpr int tri(int m, int n) {  // packed upper-triangular index, m <= n < 8
  return m * 8 - (m * (m - 1)) / 2 + (n - m);
}

template <typename T>
struct Lin1D {
  T p, q;  // 1D linear basis values at the two Gauss points: L_m(t_g) = (m == g) ? p : q
};

template <typename T>
__device__ __forceinline__ T wv(int m, int g, T p, T q) {
  return m == g ? p : q;
}
// w(m,g) * w(n,g) keyed by k = m + n in {0,1,2}
template <typename T>
__device__ __forceinline__ T wwv(int k, int g, T p, T q) {
  if (k == 1) return p * q;
  return (k == 0) == (g == 0) ? p * p : q * q;
}

// Element stiffness of one trilinear hexahedron.  x[c][m]: coordinates of local node m
// (m = m1 + 2 m2 + 4 m3, Iron's local node order).  Returns the 36 unique entries of the
// symmetric 8x8 matrix (packed upper triangle, tri(m,n)).  Returns false if det(GL) <= 0.
template <typename T>
__device__ __forceinline__ bool laplace_hex8(const T (&x)[3][8], T kappa, T p, T q, T (&K)[36]) {
  // Jacobian columns: Jt[c][a][gd1][gd2]
  T Jt[3][3][2][2];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const int d1 = a == 0 ? 1 : 0, d2 = a == 2 ? 1 : 2;
      T D[2][2];
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          const int m0 = (i << d1) | (j << d2);
          D[i][j] = x[c][m0 | (1 << a)] - x[c][m0];
        }
#pragma unroll
      for (int g2 = 0; g2 < 2; ++g2) {
        T E0 = D[0][0] * wv(0, g2, p, q) + D[0][1] * wv(1, g2, p, q);
        T E1 = D[1][0] * wv(0, g2, p, q) + D[1][1] * wv(1, g2, p, q);
#pragma unroll
        for (int g1 = 0; g1 < 2; ++g1) Jt[c][a][g1][g2] = E0 * wv(0, g1, p, q) + E1 * wv(1, g1, p, q);
      }
    }
  }
  // M_g[ab] for the 8 Gauss points, symmetric: 00 11 22 01 02 12
  T M[8][6];
  bool ok = true;
#pragma unroll
  for (int g = 0; g < 8; ++g) {
    const int gb[3] = {g & 1, (g >> 1) & 1, (g >> 2) & 1};
    T J[3][3];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const int d1 = a == 0 ? 1 : 0, d2 = a == 2 ? 1 : 2;
        J[c][a] = Jt[c][a][gb[d1]][gb[d2]];
      }
    T G00 = J[0][0] * J[0][0] + J[1][0] * J[1][0] + J[2][0] * J[2][0];
    T G11 = J[0][1] * J[0][1] + J[1][1] * J[1][1] + J[2][1] * J[2][1];
    T G22 = J[0][2] * J[0][2] + J[1][2] * J[1][2] + J[2][2] * J[2][2];
    T G01 = J[0][0] * J[0][1] + J[1][0] * J[1][1] + J[2][0] * J[2][1];
    T G02 = J[0][0] * J[0][2] + J[1][0] * J[1][2] + J[2][0] * J[2][2];
    T G12 = J[0][1] * J[0][2] + J[1][1] * J[1][2] + J[2][1] * J[2][2];
    T A00 = G11 * G22 - G12 * G12;
    T A11 = G00 * G22 - G02 * G02;
    T A22 = G00 * G11 - G01 * G01;
    T A01 = G02 * G12 - G01 * G22;
    T A02 = G01 * G12 - G02 * G11;
    T A12 = G01 * G02 - G00 * G12;
    T det = G00 * A00 + G01 * A01 + G02 * A02;
    ok = ok && (det > T(0));
    // GU * sqrt(det) * w = adj / det * sqrt(det) * w = adj * w * rsqrt(det); w = 1/8
    T sc = kappa * T(0.125) * rsqrt(det);
    M[g][0] = A00 * sc; M[g][1] = A11 * sc; M[g][2] = A22 * sc;
    M[g][3] = A01 * sc; M[g][4] = A02 * sc; M[g][5] = A12 * sc;
  }
#pragma unroll
  for (int k = 0; k < 36; ++k) K[k] = T(0);

  // diagonal pairs (a,a)
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int d1 = a == 0 ? 1 : 0, d2 = a == 2 ? 1 : 2;
    T S[2][2];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int g0 = (i << d1) | (j << d2);
        S[i][j] = M[g0][a] + M[g0 | (1 << a)][a];
      }
    T Tt[3][2];
#pragma unroll
    for (int k1 = 0; k1 < 3; ++k1)
#pragma unroll
      for (int j = 0; j < 2; ++j) Tt[k1][j] = S[0][j] * wwv(k1, 0, p, q) + S[1][j] * wwv(k1, 1, p, q);
    T V[3][3];
#pragma unroll
    for (int k1 = 0; k1 < 3; ++k1)
#pragma unroll
      for (int k2 = 0; k2 < 3; ++k2) V[k1][k2] = Tt[k1][0] * wwv(k2, 0, p, q) + Tt[k1][1] * wwv(k2, 1, p, q);
#pragma unroll
    for (int m = 0; m < 8; ++m)
#pragma unroll
      for (int n = m; n < 8; ++n) {
        const int ma = (m >> a) & 1, na = (n >> a) & 1;
        const int k1 = ((m >> d1) & 1) + ((n >> d1) & 1), k2 = ((m >> d2) & 1) + ((n >> d2) & 1);
        if (ma == na) K[tri(m, n)] += V[k1][k2];
        else K[tri(m, n)] -= V[k1][k2];
      }
  }
  // off-diagonal pairs (a,b), a < b, c the third direction; M index 3:(0,1) 4:(0,2) 5:(1,2)
#pragma unroll
  for (int pr = 0; pr < 3; ++pr) {
    const int a = pr == 2 ? 1 : 0, b = pr == 0 ? 1 : 2, c = 3 - a - b, mi = 3 + pr;
    T U[2][2][2];  // [i = n_a][gb][gc]
#pragma unroll
    for (int gbb = 0; gbb < 2; ++gbb)
#pragma unroll
      for (int gcc = 0; gcc < 2; ++gcc) {
        const int g0 = (gbb << b) | (gcc << c);
        const T m0 = M[g0][mi], m1 = M[g0 | (1 << a)][mi];
#pragma unroll
        for (int i = 0; i < 2; ++i) U[i][gbb][gcc] = m0 * wv(i, 0, p, q) + m1 * wv(i, 1, p, q);
      }
    T U2[2][2][2];  // [i][j = m_b][gc]
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < 2; ++j)
#pragma unroll
        for (int gcc = 0; gcc < 2; ++gcc)
          U2[i][j][gcc] = U[i][0][gcc] * wv(j, 0, p, q) + U[i][1][gcc] * wv(j, 1, p, q);
    T W[2][2][3];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < 2; ++j)
#pragma unroll
        for (int k = 0; k < 3; ++k) W[i][j][k] = U2[i][j][0] * wwv(k, 0, p, q) + U2[i][j][1] * wwv(k, 1, p, q);
#pragma unroll
    for (int m = 0; m < 8; ++m)
#pragma unroll
      for (int n = m; n < 8; ++n) {
        const int k = ((m >> c) & 1) + ((n >> c) & 1);
        // C_ab(m,n) = s(m_a) s(n_b) W[n_a][m_b][k];  C_ab(n,m) = s(n_a) s(m_b) W[m_a][n_b][k]
        const int sa = ((m >> a) & 1) == ((n >> b) & 1) ? 1 : -1;
        const int sb = ((n >> a) & 1) == ((m >> b) & 1) ? 1 : -1;
        const T t1 = W[(n >> a) & 1][(m >> b) & 1][k];
        const T t2 = W[(m >> a) & 1][(n >> b) & 1][k];
        K[tri(m, n)] += (sa > 0 ? t1 : -t1) + (sb > 0 ? t2 : -t2);
      }
  }
  return ok;
}

template <typename T>
__device__ __forceinline__ void load_element(int e, const int32_t* __restrict__ elem_nodes,
                                             const double* __restrict__ coords, int32_t n_nodes, int (&nd)[8],
                                             T (&x)[3][8]) {
  const int4* en = reinterpret_cast<const int4*>(elem_nodes + (size_t)e * 8);
  int4 a = __ldg(en), b = __ldg(en + 1);
  nd[0] = a.x; nd[1] = a.y; nd[2] = a.z; nd[3] = a.w;
  nd[4] = b.x; nd[5] = b.y; nd[6] = b.z; nd[7] = b.w;
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int m = 0; m < 8; ++m) x[c][m] = (T)__ldg(coords + (size_t)c * n_nodes + nd[m]);
}

template <typename T>
__global__ void __launch_bounds__(kBlock)
laplace_assemble_color(const int32_t* __restrict__ elems, int32_t count, int32_t n_nodes,
                       const int32_t* __restrict__ elem_nodes, const double* __restrict__ coords,
                       const double* __restrict__ kappa, const int32_t* __restrict__ rp,
                       const int32_t* __restrict__ ci, double* __restrict__ values, unsigned* err) {
  const int t = blockIdx.x * kBlock + threadIdx.x;
  if (t >= count) return;
  const int e = __ldg(elems + t);
  int nd[8];
  T x[3][8];
  load_element<T>(e, elem_nodes, coords, n_nodes, nd, x);
  const T kap = kappa ? (T)__ldg(kappa + e) : T(1);
  const T s3 = T(1) / sqrt(T(3));
  const T p = (s3 + T(1)) / T(2), q = (-s3 + T(1)) / T(2);
  T K[36];
  if (!laplace_hex8<T>(x, kap, p, q, K)) gfe_raise(err, GFE_DEVERR_JACOBIAN);
  bool missing = false;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int row = nd[i];
    const int lo0 = __ldg(rp + row) - 1, hi0 = __ldg(rp + row + 1) - 1;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int col = nd[j] + 1;
      int lo = lo0, hi = hi0;  // lower_bound of col in ci[lo0, hi0)
      while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (__ldg(ci + mid) < col) lo = mid + 1; else hi = mid;
      }
      if (lo < hi0 && __ldg(ci + lo) == col) {
        values[lo] += (double)K[i <= j ? tri(i, j) : tri(j, i)];
      } else {
        missing = true;
      }
    }
  }
  if (missing) gfe_raise(err, GFE_DEVERR_SLOT);
}

template <typename T>
__global__ void __launch_bounds__(kBlock)
laplace_element_kernel(int32_t n_elem, int32_t n_nodes, const int32_t* __restrict__ elem_nodes,
                       const double* __restrict__ coords, const double* __restrict__ kappa,
                       double* __restrict__ Kout, unsigned* err) {
  const int e = blockIdx.x * kBlock + threadIdx.x;
  if (e >= n_elem) return;
  int nd[8];
  T x[3][8];
  load_element<T>(e, elem_nodes, coords, n_nodes, nd, x);
  const T kap = kappa ? (T)kappa[e] : T(1);
  const T s3 = T(1) / sqrt(T(3));
  const T p = (s3 + T(1)) / T(2), q = (-s3 + T(1)) / T(2);
  T K[36];
  if (!laplace_hex8<T>(x, kap, p, q, K)) gfe_raise(err, GFE_DEVERR_JACOBIAN);
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) Kout[(size_t)e * 64 + i * 8 + j] = (double)K[i <= j ? tri(i, j) : tri(j, i)];
}

__global__ void to_fp32(const double* __restrict__ v, float* __restrict__ v32, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    v32[i] = (float)v[i];
}

int check_common(int32_t n_elem, int32_t n_nodes, const int32_t* elem_nodes, const double* coords, int precision,
                 const char* fn) {
  if (n_elem < 0 || n_nodes <= 0 || (n_elem > 0 && (!elem_nodes || !coords)))
    return gfe::set_error(GFE_ERR_ARG, "%s: invalid mesh arguments (n_elem=%d n_nodes=%d)", fn, n_elem, n_nodes);
  if (precision != GFE_FP64 && precision != GFE_MIXED)
    return gfe::set_error(GFE_ERR_ARG, "%s: unknown precision %d", fn, precision);
  if (reinterpret_cast<uintptr_t>(elem_nodes) % 16 != 0)
    return gfe::set_error(GFE_ERR_ARG, "%s: elem_nodes must be 16-byte aligned", fn);
  return GFE_OK;
}

int check_device_errors(cudaStream_t s, const char* fn, bool sync) {
  if (!sync) return GFE_OK;
  unsigned* err = gfe::device_error_word();
  unsigned bits = 0;
  GFE_CUDA_TRY(cudaMemcpyAsync(&bits, err, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  GFE_CUDA_TRY(cudaStreamSynchronize(s));
  if (bits) {
    cudaMemsetAsync(err, 0, sizeof(unsigned), s);
    if (bits & GFE_DEVERR_SLOT)
      return gfe::set_error(GFE_ERR_STRUCTURE, "%s: an element entry has no slot in the CSR structure", fn);
    if (bits & GFE_DEVERR_JACOBIAN)
      return gfe::set_error(GFE_ERR_NUMERIC, "%s: zero or negative metric determinant at a Gauss point", fn);
    return gfe::set_error(GFE_ERR_NUMERIC, "%s: device error bits 0x%x", fn, bits);
  }
  return GFE_OK;
}

}  // namespace

extern "C" int gfe_laplace_assemble(int32_t n_elem, int32_t n_nodes, const int32_t* elem_nodes, const double* coords,
                                    const double* kappa, const int32_t* color_elems, const int32_t* color_ptr_host,
                                    int32_t n_colors, const int32_t* row_ptr, const int32_t* col_idx, int64_t nnz,
                                    double* values, float* values32, double* rhs, int32_t precision,
                                    void* stream) {
  const char* fn = "gfe_laplace_assemble";
  int rc = check_common(n_elem, n_nodes, elem_nodes, coords, precision, fn);
  if (rc) return rc;
  if (!row_ptr || !col_idx || !values || (n_elem > 0 && (!color_elems || !color_ptr_host || n_colors <= 0)))
    return gfe::set_error(GFE_ERR_ARG, "%s: missing CSR or colouring arguments", fn);
  if (color_ptr_host && n_colors > 0 && (color_ptr_host[0] != 0 || color_ptr_host[n_colors] != n_elem))
    return gfe::set_error(GFE_ERR_ARG, "%s: colour offsets must run from 0 to n_elem", fn);
  cudaStream_t s = gfe::as_stream(stream);
  unsigned* err = gfe::device_error_word();
  if (nnz < 0) return gfe::set_error(GFE_ERR_ARG, "%s: invalid nnz", fn);
  // EquationsMatrices_VectorValuesInitialise: zero the matrix and RHS before the element loop
  GFE_CUDA_TRY(cudaMemsetAsync(values, 0, sizeof(double) * (size_t)nnz, s));
  if (rhs) GFE_CUDA_TRY(cudaMemsetAsync(rhs, 0, sizeof(double) * (size_t)n_nodes, s));
  void* prof = gfe::stage_begin(GFE_STAGE_LAPLACE_ELEMENTS, s);
  int launches = 0;
  for (int c = 0; c < n_colors; ++c) {
    const int c0 = color_ptr_host[c], cnt = color_ptr_host[c + 1] - c0;
    if (cnt <= 0) continue;
    const int grid = (cnt + kBlock - 1) / kBlock;
    if (precision == GFE_FP64)
      laplace_assemble_color<double><<<grid, kBlock, 0, s>>>(color_elems + c0, cnt, n_nodes, elem_nodes, coords,
                                                             kappa, row_ptr, col_idx, values, err);
    else
      laplace_assemble_color<float><<<grid, kBlock, 0, s>>>(color_elems + c0, cnt, n_nodes, elem_nodes, coords,
                                                            kappa, row_ptr, col_idx, values, err);
    ++launches;
  }
  gfe::stage_end(GFE_STAGE_LAPLACE_ELEMENTS, prof, s, launches);
  if (values32) to_fp32<<<4 * gfe::sm_count(), 256, 0, s>>>(values, values32, nnz);
  GFE_LAUNCH_CHECK(fn);
  return GFE_OK;
}

extern "C" int gfe_laplace_element_matrices(int32_t n_elem, int32_t n_nodes, const int32_t* elem_nodes,
                                            const double* coords, const double* kappa, double* K_out,
                                            int32_t precision, void* stream) {
  const char* fn = "gfe_laplace_element_matrices";
  int rc = check_common(n_elem, n_nodes, elem_nodes, coords, precision, fn);
  if (rc) return rc;
  if (!K_out) return gfe::set_error(GFE_ERR_ARG, "%s: K_out is NULL", fn);
  cudaStream_t s = gfe::as_stream(stream);
  unsigned* err = gfe::device_error_word();
  if (n_elem == 0) return GFE_OK;
  const int grid = (n_elem + kBlock - 1) / kBlock;
  if (precision == GFE_FP64)
    laplace_element_kernel<double><<<grid, kBlock, 0, s>>>(n_elem, n_nodes, elem_nodes, coords, kappa, K_out, err);
  else
    laplace_element_kernel<float><<<grid, kBlock, 0, s>>>(n_elem, n_nodes, elem_nodes, coords, kappa, K_out, err);
  GFE_LAUNCH_CHECK(fn);
  return check_device_errors(s, fn, true);
}
