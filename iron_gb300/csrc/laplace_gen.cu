// laplace_gen.cu -- generalised Laplace on trilinear hexahedra: a full conductivity tensor in a
// material frame, assembled into Iron's CSR matrix by the deterministic colour scatter.
//
// Element routine: LaplaceEquation_FiniteElementCalculate, EQUATIONS_SET_GENERALISED_LAPLACE_SUBTYPE
// (src/Laplace_equations_routines.F90:585-707).  Per Gauss point:
//  * metrics of the geometric field: DX_DXI, GL = DX_DXI^T DX_DXI, GU = GL^-1,
//    RWG = sqrt|det GL| * w (src/coordinate_routines.F90:703-822);
//  * the conductivity in material coordinates from the element's materials field components
//    K11 K22 K33 K12 K23 K13 (:640-656; element-constant here);
//  * the material frame dX/dNu (Coordinates_MaterialSystemCalculate,
//    src/coordinate_routines.F90:3841-3947): with a fibre field, the reference frame
//    f = DX_DXI(:,1), h = f x DX_DXI(:,2), g = h x f, normalised, rotated by the fibre angle about
//    axis 3, the imbrication angle about the new axis 2 and the sheet angle about the new axis 1
//    (:4020-4127), the angles interpolated from the nodal fibre field with the element basis;
//    without one, the normalised columns of DX_DXI (:3879-3884);
//  * dNu/dXi = (dX/dNu)^T DX_DXI, dXi/dNu = (dNu/dXi)^-1 and the conductivity in xi space
//    C = dNu/dXi K dXi/dNu (:660-670);
//  * K(ms,ns) += RWG * sum_{i,k,h} C(i,k) dphi_ns/dxi_k dphi_ms/dxi_h GU(i,h) (:680-693),
//    here as RWG * dphi_ms^T (GU C) dphi_ns.  The RHS is zero.
// One thread per element: the Gauss-point matrices RWG * GU C (8 x 9 numbers) go to shared memory,
// then the element rows are formed and scattered one at a time.  Elements of one colour share no
// node, so each CSR entry is written by one thread per launch; colours run in order, so the
// summation order is fixed.  FP64 throughout.
#include <cmath>

#include "gfe_internal.cuh"

namespace {

constexpr int kGenBlock = 64;

__device__ __forceinline__ void normalise3(double v[3]) {
  const double l = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  v[0] /= l;
  v[1] /= l;
  v[2] /= l;
}

__device__ __forceinline__ void cross3(const double a[3], const double b[3], double c[3]) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

__device__ __forceinline__ void mm3(const double A[3][3], const double B[3][3], double C[3][3]) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) C[i][j] = A[i][0] * B[0][j] + A[i][1] * B[1][j] + A[i][2] * B[2][j];
}

// Inverse by cofactors over the determinant (Iron's Invert, src/maths.F90:2807-2868); returns det.
__device__ __forceinline__ double inv3(const double A[3][3], double B[3][3]) {
  const double det = A[0][0] * A[1][1] * A[2][2] + A[0][1] * A[1][2] * A[2][0] + A[0][2] * A[1][0] * A[2][1] -
                     A[0][0] * A[2][1] * A[1][2] - A[1][0] * A[0][1] * A[2][2] - A[2][0] * A[1][1] * A[0][2];
  B[0][0] = (A[1][1] * A[2][2] - A[2][1] * A[1][2]) / det;
  B[1][0] = (A[1][2] * A[2][0] - A[2][2] * A[1][0]) / det;
  B[2][0] = (A[1][0] * A[2][1] - A[2][0] * A[1][1]) / det;
  B[0][1] = (A[2][1] * A[0][2] - A[0][1] * A[2][2]) / det;
  B[1][1] = (A[2][2] * A[0][0] - A[0][2] * A[2][0]) / det;
  B[2][1] = (A[2][0] * A[0][1] - A[0][0] * A[2][1]) / det;
  B[0][2] = (A[0][1] * A[1][2] - A[1][1] * A[0][2]) / det;
  B[1][2] = (A[0][2] * A[1][0] - A[1][2] * A[0][0]) / det;
  B[2][2] = (A[0][0] * A[1][1] - A[1][0] * A[0][1]) / det;
  return det;
}

// 1D linear Lagrange basis on [0,1] at the 2-point Gauss-Legendre abscissae: value and slope of
// local node a (0: 1 - xi, 1: xi) at Gauss point gi.
__device__ __forceinline__ double l1(int a, int gi) {
  const double x = gi == 0 ? 0.21132486540518711775 : 0.78867513459481288225;  // (1 -+ 1/sqrt 3) / 2
  return a == 0 ? 1.0 - x : x;
}
__device__ __forceinline__ double dl1(int a) { return a == 0 ? -1.0 : 1.0; }

// dphi_m / dxi_k at Gauss point (g1, g2, g3); m = m1 + 2 m2 + 4 m3 (Iron's local node order).
__device__ __forceinline__ double dphi(int m, int k, int g1, int g2, int g3) {
  const int m1 = m & 1, m2 = (m >> 1) & 1, m3 = m >> 2;
  const double a = k == 0 ? dl1(m1) : l1(m1, g1);
  const double b = k == 1 ? dl1(m2) : l1(m2, g2);
  const double c = k == 2 ? dl1(m3) : l1(m3, g3);
  return a * b * c;
}

__global__ void __launch_bounds__(kGenBlock)
laplace_generalised_color(const int32_t* __restrict__ elems, int32_t count, int32_t n_elem, int32_t n_nodes,
                          const int32_t* __restrict__ elem_nodes, const double* __restrict__ coords,
                          const double* __restrict__ cond, const double* __restrict__ fibre, int32_t n_angles,
                          const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                          double* __restrict__ values, unsigned* err) {
  __shared__ double sM[8 * 9][kGenBlock];  // RWG * GU C per Gauss point, one column per thread
  const int t = blockIdx.x * kGenBlock + threadIdx.x;
  if (t >= count) return;
  const int e = __ldg(elems + t);
  int nd[8];
  double x[3][8];
#pragma unroll
  for (int m = 0; m < 8; ++m) {
    nd[m] = __ldg(elem_nodes + (size_t)e * 8 + m);
#pragma unroll
    for (int c = 0; c < 3; ++c) x[c][m] = __ldg(coords + (size_t)c * n_nodes + nd[m]);
  }
  double Km[3][3];
  {
    double k[6];
    bool finite = true;
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      k[c] = __ldg(cond + (size_t)c * n_elem + e);
      finite = finite && isfinite(k[c]);
    }
    if (!finite) gfe_raise(err, GFE_DEVERR_NONFINITE);
    Km[0][0] = k[0]; Km[1][1] = k[1]; Km[2][2] = k[2];
    Km[0][1] = Km[1][0] = k[3];
    Km[1][2] = Km[2][1] = k[4];
    Km[0][2] = Km[2][0] = k[5];
  }
  bool bad = false;
#pragma unroll 1
  for (int g = 0; g < 8; ++g) {
    const int g1 = g & 1, g2 = (g >> 1) & 1, g3 = g >> 2;
    double J[3][3];  // DX_DXI
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        double s = 0.0;
#pragma unroll
        for (int m = 0; m < 8; ++m) s += x[c][m] * dphi(m, k, g1, g2, g3);
        J[c][k] = s;
      }
    double GL[3][3], GU[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) GL[a][b] = J[0][a] * J[0][b] + J[1][a] * J[1][b] + J[2][a] * J[2][b];
    const double detgl = inv3(GL, GU);
    if (!(detgl > 0.0)) bad = true;
    const double rwg = sqrt(fabs(detgl)) * 0.125;
    // material frame dX/dNu
    double F[3][3];
    if (fibre) {
      double ang[3] = {0.0, 0.0, 0.0};
      for (int a = 0; a < n_angles; ++a) {
        double s = 0.0;
#pragma unroll
        for (int m = 0; m < 8; ++m)
          s += l1(m & 1, g1) * l1((m >> 1) & 1, g2) * l1(m >> 2, g3) * __ldg(fibre + (size_t)a * n_nodes + nd[m]);
        ang[a] = s;
      }
      double f[3] = {J[0][0], J[1][0], J[2][0]}, d2[3] = {J[0][1], J[1][1], J[2][1]}, h[3], gg[3];
      cross3(f, d2, h);
      cross3(h, f, gg);
      normalise3(f);
      normalise3(gg);
      normalise3(h);
      const double R0[3][3] = {{f[0], gg[0], h[0]}, {f[1], gg[1], h[1]}, {f[2], gg[2], h[2]}};
      double sa, ca, sb, cb, sg, cg;
      sincos(ang[0], &sa, &ca);
      sincos(ang[1], &sb, &cb);
      sincos(ang[2], &sg, &cg);
      const double Rz[3][3] = {{ca, -sa, 0.0}, {sa, ca, 0.0}, {0.0, 0.0, 1.0}};
      const double Ry[3][3] = {{cb, 0.0, sb}, {0.0, 1.0, 0.0}, {-sb, 0.0, cb}};
      const double Rx[3][3] = {{1.0, 0.0, 0.0}, {0.0, cg, -sg}, {0.0, sg, cg}};
      double T1[3][3], T2[3][3];
      mm3(R0, Rz, T1);
      mm3(T1, Ry, T2);
      mm3(T2, Rx, F);
    } else {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        double col[3] = {J[0][k], J[1][k], J[2][k]};
        normalise3(col);
#pragma unroll
        for (int c = 0; c < 3; ++c) F[c][k] = col[c];
      }
    }
    // dNu/dXi = F^T J, dXi/dNu its inverse, C = dNu/dXi Km dXi/dNu
    double P[3][3], Pi[3][3], T[3][3], C[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) P[i][j] = F[0][i] * J[0][j] + F[1][i] * J[1][j] + F[2][i] * J[2][j];
    inv3(P, Pi);
    mm3(P, Km, T);
    mm3(T, Pi, C);
    // M = RWG * GU C (GU symmetric: sum_i GU(i,h) C(i,k) = (GU C)(h,k))
#pragma unroll
    for (int h = 0; h < 3; ++h)
#pragma unroll
      for (int k = 0; k < 3; ++k)
        sM[g * 9 + h * 3 + k][threadIdx.x] = rwg * (GU[h][0] * C[0][k] + GU[h][1] * C[1][k] + GU[h][2] * C[2][k]);
  }
  if (bad) gfe_raise(err, GFE_DEVERR_JACOBIAN);
  bool missing = false;
#pragma unroll 1
  for (int ms = 0; ms < 8; ++ms) {
    double row[8];
#pragma unroll
    for (int ns = 0; ns < 8; ++ns) row[ns] = 0.0;
#pragma unroll 1
    for (int g = 0; g < 8; ++g) {
      const int g1 = g & 1, g2 = (g >> 1) & 1, g3 = g >> 2;
      double v[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        double s = 0.0;
#pragma unroll
        for (int h = 0; h < 3; ++h) s += dphi(ms, h, g1, g2, g3) * sM[g * 9 + h * 3 + k][threadIdx.x];
        v[k] = s;
      }
#pragma unroll
      for (int ns = 0; ns < 8; ++ns)
        row[ns] += v[0] * dphi(ns, 0, g1, g2, g3) + v[1] * dphi(ns, 1, g1, g2, g3) + v[2] * dphi(ns, 2, g1, g2, g3);
    }
    const int r = nd[ms];
    const int lo0 = __ldg(rp + r) - 1, hi0 = __ldg(rp + r + 1) - 1;
#pragma unroll
    for (int ns = 0; ns < 8; ++ns) {
      const int col = nd[ns] + 1;
      int lo = lo0, hi = hi0;  // lower_bound of col in ci[lo0, hi0)
      while (lo < hi) {
        const int mid = lo + ((hi - lo) >> 1);
        if (__ldg(ci + mid) < col) lo = mid + 1; else hi = mid;
      }
      if (lo < hi0 && __ldg(ci + lo) == col) values[lo] += row[ns];
      else missing = true;
    }
  }
  if (missing) gfe_raise(err, GFE_DEVERR_SLOT);
}

}  // namespace

extern "C" int gfe_laplace_assemble_generalised(int32_t n_elem, int32_t n_nodes, const int32_t* elem_nodes,
                                                const double* coords, const double* conductivity,
                                                const double* fibre, int32_t n_angles, const int32_t* color_elems,
                                                const int32_t* color_ptr_host, int32_t n_colors,
                                                const int32_t* row_ptr, const int32_t* col_idx, int64_t nnz,
                                                double* values, double* rhs, void* stream) {
  const char* fn = "gfe_laplace_assemble_generalised";
  if (n_elem < 0 || n_nodes <= 0 || (n_elem > 0 && (!elem_nodes || !coords || !conductivity)))
    return gfe::set_error(GFE_ERR_ARG, "%s: invalid mesh arguments (n_elem=%d n_nodes=%d)", fn, n_elem, n_nodes);
  if (!row_ptr || !col_idx || !values || nnz < 0 || (n_elem > 0 && (!color_elems || !color_ptr_host || n_colors <= 0)))
    return gfe::set_error(GFE_ERR_ARG, "%s: missing CSR or colouring arguments", fn);
  if (color_ptr_host && n_colors > 0 && (color_ptr_host[0] != 0 || color_ptr_host[n_colors] != n_elem))
    return gfe::set_error(GFE_ERR_ARG, "%s: colour offsets must run from 0 to n_elem", fn);
  if (fibre ? (n_angles < 1 || n_angles > 3) : n_angles != 0)
    return gfe::set_error(GFE_ERR_ARG, "%s: a fibre field has 1 to 3 angles (none without one), got %d", fn,
                          n_angles);
  cudaStream_t s = gfe::as_stream(stream);
  unsigned* err = gfe::device_error_word();
  // EquationsMatrices_VectorValuesInitialise: zero the matrix and RHS before the element loop
  GFE_CUDA_TRY(cudaMemsetAsync(values, 0, sizeof(double) * (size_t)nnz, s));
  if (rhs) GFE_CUDA_TRY(cudaMemsetAsync(rhs, 0, sizeof(double) * (size_t)n_nodes, s));
  void* prof = gfe::stage_begin(GFE_STAGE_LAPLACE_ELEMENTS, s);
  int launches = 0;
  for (int c = 0; c < n_colors; ++c) {
    const int c0 = color_ptr_host[c], cnt = color_ptr_host[c + 1] - c0;
    if (cnt <= 0) continue;
    laplace_generalised_color<<<(cnt + kGenBlock - 1) / kGenBlock, kGenBlock, 0, s>>>(
        color_elems + c0, cnt, n_elem, n_nodes, elem_nodes, coords, conductivity, fibre, n_angles, row_ptr, col_idx,
        values, err);
    ++launches;
  }
  gfe::stage_end(GFE_STAGE_LAPLACE_ELEMENTS, prof, s, launches);
  GFE_LAUNCH_CHECK(fn);
  return GFE_OK;
}
