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
// oracle's literal restatement of Iron's loops).  The element arithmetic is templated on
// double (GFE_FP64), float (GFE_MIXED) or float-float (GFE_MIXED_DF, df.cuh).
//
// Two scatter strategies, both deterministic (fixed summation order, no atomics), both replacing
// EquationsMatrices_ElementAdd -> MATRIX_VALUES_ADD_DP2 (src/matrix_vector.F90:3202-3240):
//  * general meshes: elements colour by colour (no two elements of a colour share a node), one
//    thread per element searches each of its 64 entries in the CSR row and adds it;
//  * Iron's regular generated mesh (GENERATED_MESH_REGULAR_TYPE, implicit topology): a CTA owns a
//    tile of nodes in the x-y plane and marches up the z layers; it computes the element matrices
//    of the two element layers touching the current node layer into shared memory once, then each
//    thread sums its node's 27-entry row from the 8 surrounding elements in a fixed order and
//    writes the row exactly once.  CSR slot positions follow from the 27-point stencil
//    (verified once against the structure by gfe_laplace_regular_check), so the kernel reads no
//    column indices.
#include <atomic>
#include <cmath>
#include <type_traits>
#include <vector>

#include "df.cuh"
#include "gfe_internal.cuh"

namespace {

constexpr int kBlock = 128;

__host__ __device__ constexpr int tri(int m, int n) {  // packed upper-triangular index, m <= n < 8
  return m * 8 - (m * (m - 1)) / 2 + (n - m);
}

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

// Metrics of one trilinear hexahedron at its 8 Gauss points: M[g] = GU Jacobian w kappa as the six
// entries 00 11 22 01 02 12 of the symmetric 3x3 matrix.  x[c][m]: coordinates of local node m
// (m = m1 + 2 m2 + 4 m3, Iron's local node order).  Returns false if det(GL) <= 0.
template <typename T>
__device__ __forceinline__ bool hex8_metrics(const T (&x)[3][8], T kappa, T p, T q, T (&M)[8][6]) {
  const T zero = from_double<T>(0.0);
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
  bool ok = true;
  const T eighth = kappa * from_double<T>(0.125);
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
    ok = ok && (det > zero);
    // GU * sqrt(det) * w = adj / det * sqrt(det) * w = adj * w * rsqrt(det); w = 1/8
    T sc = eighth * rsqrt(det);
    M[g][0] = A00 * sc; M[g][1] = A11 * sc; M[g][2] = A22 * sc;
    M[g][3] = A01 * sc; M[g][4] = A02 * sc; M[g][5] = A12 * sc;
  }
  return ok;
}

// The element matrix from the Gauss-point metrics: the 36 unique entries of the symmetric 8x8
// matrix (packed upper triangle, tri(m,n)), contracted one xi direction at a time.
// Mg(g, k): entry k (00 11 22 01 02 12) of the metric at Gauss point g, read where it is needed.
template <typename T, typename MetricAt>
__device__ __forceinline__ void hex8_contract_at(MetricAt Mg, T p, T q, T (&K)[36]) {
  const T zero = from_double<T>(0.0);
#pragma unroll
  for (int k = 0; k < 36; ++k) K[k] = zero;

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
        S[i][j] = Mg(g0, a) + Mg(g0 | (1 << a), a);
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
        if (ma == na) accum(K[tri(m, n)], V[k1][k2]);
        else accum_sub(K[tri(m, n)], V[k1][k2]);
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
        const T m0 = Mg(g0, mi), m1 = Mg(g0 | (1 << a), mi);
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
        const bool sa = ((m >> a) & 1) == ((n >> b) & 1);
        const bool sb = ((n >> a) & 1) == ((m >> b) & 1);
        const T t1 = W[(n >> a) & 1][(m >> b) & 1][k];
        const T t2 = W[(m >> a) & 1][(n >> b) & 1][k];
        if (sa) accum(K[tri(m, n)], t1); else accum_sub(K[tri(m, n)], t1);
        if (sb) accum(K[tri(m, n)], t2); else accum_sub(K[tri(m, n)], t2);
      }
  }
#pragma unroll
  for (int k = 0; k < 36; ++k) finish(K[k]);
}

template <typename T>
__device__ __forceinline__ void hex8_contract(const T (&M)[8][6], T p, T q, T (&K)[36]) {
  hex8_contract_at<T>([&](int g, int k) { return M[g][k]; }, p, q, K);
}

// Element stiffness of one trilinear hexahedron (metrics, then contraction).  Returns the 36
// unique entries of the symmetric 8x8 matrix; false if det(GL) <= 0.
template <typename T>
__device__ __forceinline__ bool laplace_hex8(const T (&x)[3][8], T kappa, T p, T q, T (&K)[36]) {
  T M[8][6];
  const bool ok = hex8_metrics<T>(x, kappa, p, q, M);
  hex8_contract<T>(M, p, q, K);
  return ok;
}

// Gauss-point constants of the 2-point rule on [0,1] (src/basis_routines.F90:6804-6890):
// p = L_0(t_0) = 1 - (1 - 1/sqrt3)/2, q = L_1(t_0).
template <typename T>
__device__ __forceinline__ void gauss_pq(T& p, T& q) {
  const double s3 = 1.0 / sqrt(3.0);
  p = from_double<T>((s3 + 1.0) / 2.0);
  q = from_double<T>((-s3 + 1.0) / 2.0);
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
    for (int m = 0; m < 8; ++m) x[c][m] = from_double<T>(__ldg(coords + (size_t)c * n_nodes + nd[m]));
}

// ---------------------------------------------------------------------------------------------
// general meshes: colour by colour
// ---------------------------------------------------------------------------------------------
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
  const double kd = kappa ? __ldg(kappa + e) : 1.0;
  if (!isfinite(kd)) gfe_raise(err, GFE_DEVERR_NONFINITE);
  const T kap = from_double<T>(kd);
  T p, q;
  gauss_pq(p, q);
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
        int mid = lo + ((hi - lo) >> 1);  // no int32 overflow past 2^30 entries
        if (__ldg(ci + mid) < col) lo = mid + 1; else hi = mid;
      }
      if (lo < hi0 && __ldg(ci + lo) == col) {
        values[lo] += to_double(K[i <= j ? tri(i, j) : tri(j, i)]);
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
  const double kd = kappa ? kappa[e] : 1.0;
  if (!isfinite(kd)) gfe_raise(err, GFE_DEVERR_NONFINITE);
  const T kap = from_double<T>(kd);
  T p, q;
  gauss_pq(p, q);
  T K[36];
  if (!laplace_hex8<T>(x, kap, p, q, K)) gfe_raise(err, GFE_DEVERR_JACOBIAN);
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) Kout[(size_t)e * 64 + i * 8 + j] = to_double(K[i <= j ? tri(i, j) : tri(j, i)]);
}

__global__ void to_fp32(const double* __restrict__ v, float* __restrict__ v32, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    v32[i] = (float)v[i];
}

// ---------------------------------------------------------------------------------------------
// Iron's regular generated mesh: tiled, row-owning assembly
// ---------------------------------------------------------------------------------------------
// Node tile TX x TY in x-y; the element tile is (TX+1) x (TY+1) = 16 x 12 = 192 elements, one per
// thread.  Element matrices are kept in shared memory in the element arithmetic type; the row sums
// are accumulated in FP64 (GFE_FP64) or float-float (the FP32-pipe precisions), so the FP32 paths
// issue FP64 instructions only for the final conversion of each written entry.
// The kernel is persistent: the work, (tile column) x (node layer), is linearised column by
// column and cut into one contiguous, equal share per CTA; a CTA walks its share as runs of
// consecutive node layers, recomputing only the element layer below each run.  So the grid is
// sized to the resident CTAs (no tail wave) and runs are long (little recomputation in z).
constexpr int kRTX = 15, kRTY = 11;
constexpr int kREX = kRTX + 1, kREY = kRTY + 1;  // 16 x 12 elements
constexpr int kRThreads = kREX * kREY;           // 192
constexpr int kRZ = 8;                           // alignment of the layer ranges of the slab API
constexpr int kRMinRun = 8;                      // node layers per CTA at least, when work is scarce
// Resident CTAs per SM the register allocation must allow: two 192-thread CTAs fill the shared
// memory with float-float or FP64 element matrices; FP32 matrices take half of it.
template <typename T>
struct RMinBlocks {
  static constexpr int value = 2;
};
template <>
struct RMinBlocks<float> {
  static constexpr int value = 3;
};

template <typename T>
struct StoreOf {
  using type = T;
};
template <typename T>
struct AccOf {
  using type = f2;
};
template <>
struct AccOf<double> {
  using type = double;
};

// Output of one assembled entry.  FP64: as accumulated.  Float-float: hi + lo in FP64 (one add,
// the conversions done with integer operations) and hi + lo rounded to FP32 for the copy.  FP32
// element arithmetic: the sum rounded to FP32, widened exactly to FP64.
__device__ __forceinline__ void entry_out(double a, bool, double& v, float& v32) {
  v = a;
  v32 = (float)a;
}
__device__ __forceinline__ void entry_out(f2 a, bool full, double& v, float& v32) {
  v32 = __fadd_rn(a.hi, a.lo);
  v = full ? f32_to_f64_exact(a.hi) + f32_to_f64_exact(a.lo) : f32_to_f64_exact(v32);
}

// row-sum accumulation (the final FP64 conversion hi + lo needs no normalised form)
__device__ __forceinline__ double acc_add(double a, double b) { return a + b; }
__device__ __forceinline__ f2 acc_add(f2 a, float b) {
  const f2 s = two_sum(a.hi, b);
  return {s.hi, __fadd_rn(a.lo, s.lo)};
}
__device__ __forceinline__ f2 acc_add(f2 a, f2 b) {
  accum(a, b);
  return a;
}

// Coordinates are read in the element arithmetic type: the FP32-pipe precisions take them from a
// copy split once per node (float or float-float), so no element converts FP64 values itself.
template <typename T>
__global__ void split_coords(long long n, const double* __restrict__ in, T* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = from_double<T>(in[i]);
}

template <typename P>
__device__ __forceinline__ void prefetch_l1(const P* p) {
  asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

__device__ __forceinline__ double load_coord(const double* p) { return __ldg(p); }
__device__ __forceinline__ float load_coord(const float* p) { return __ldg(p); }
__device__ __forceinline__ f2 load_coord(const f2* p) {
  const float2 v = __ldg(reinterpret_cast<const float2*>(p));
  return {v.x, v.y};
}

template <typename T>
__global__ void __launch_bounds__(kRThreads, RMinBlocks<T>::value)
laplace_regular_kernel(int32_t nx, int32_t ny, int32_t nz, const T* __restrict__ coords,
                       const double* __restrict__ kappa, const int32_t* __restrict__ rp, double* __restrict__ values,
                       float* __restrict__ values32, double* __restrict__ rhs, unsigned* err, int32_t layer0,
                       int32_t layer_end) {
  using S = typename StoreOf<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  S(*sK)[36][kRThreads] = reinterpret_cast<S(*)[36][kRThreads]>(smem_raw);  // [layer buffer][entry][element]
  const int tid = threadIdx.x;
  const int NX = nx + 1, NY = ny + 1, NZ = nz + 1;
  const long long NXY = (long long)NX * NY;
  // node layers [layer0, layer_end) of every tile column; this CTA's share [s, e) of the
  // linearised (column, layer) work
  const int tiles_x = (NX + kRTX - 1) / kRTX, tiles_y = (NY + kRTY - 1) / kRTY;
  const long long nl = layer_end - layer0;
  const long long W = (long long)tiles_x * tiles_y * nl;
  long long s = W * blockIdx.x / gridDim.x;
  const long long e_share = W * (blockIdx.x + 1) / gridDim.x;
  T p, q;
  gauss_pq(p, q);
  bool bad = false, nonfinite = false;
  while (s < e_share) {  // uniform across the CTA
    const long long col = s / nl;
    const int off = (int)(s - col * nl);
    const int run = (int)min(nl - off, e_share - s);
    s += run;
    const int k0 = layer0 + off, k1 = k0 + run;
    const int x0 = (int)(col % tiles_x) * kRTX, y0 = (int)(col / tiles_x) * kRTY;
    // element owned by this thread in each element layer
    const int ex = x0 - 1 + (tid % kREX), ey = y0 - 1 + (tid / kREX);
    const bool e_in_xy = ex >= 0 && ex < nx && ey >= 0 && ey < ny;
    // node owned by this thread (threads 0 .. TX*TY-1)
    const int ni = x0 + tid % kRTX, nj = y0 + tid / kRTX;
    const bool owns_node = tid < kRTX * kRTY && ni < NX && nj < NY;

    auto compute_layer = [&](int ez, int buf) {
      if (e_in_xy && ez >= 0 && ez < nz) {
        T x[3][8];
#pragma unroll
        for (int m = 0; m < 8; ++m) {
          const long long n = (long long)(ex + (m & 1)) + (long long)(ey + ((m >> 1) & 1)) * NX + (ez + (m >> 2)) * NXY;
#pragma unroll
          for (int c = 0; c < 3; ++c) x[c][m] = load_coord(coords + c * NXY * NZ + n);
        }
        const long long e = (long long)ex + (long long)ey * nx + (long long)ez * nx * ny;
        const double kd = kappa ? __ldg(kappa + e) : 1.0;
        if (!isfinite(kd)) nonfinite = true;
        const T kap = from_double<T>(kd);
        T K[36];
        if (!laplace_hex8<T>(x, kap, p, q, K)) bad = true;
#pragma unroll
        for (int k = 0; k < 36; ++k) sK[buf][k][tid] = K[k];
      }
    };
    // The next element layer's new node plane (z = ez + 1) and conductivities are prefetched into
    // L1 before the node phase of the current layer, so that phase hides their latency; the lower
    // plane is the one the current layer has just read.
    auto prefetch_layer = [&](int ez) {
      if (e_in_xy && ez >= 0 && ez < nz) {
#pragma unroll
        for (int m = 4; m < 8; ++m) {
          const long long n = (long long)(ex + (m & 1)) + (long long)(ey + ((m >> 1) & 1)) * NX + (ez + 1) * NXY;
#pragma unroll
          for (int c = 0; c < 3; ++c) prefetch_l1(coords + c * NXY * NZ + n);
        }
        if (kappa) prefetch_l1(kappa + (long long)ex + (long long)ey * nx + (long long)ez * nx * ny);
      }
    };
    using A = typename AccOf<T>::type;

    // element layer k0 - 1 (below the first node layer) is computed in the first pass; the element
    // routine has a single call site, so its code is not duplicated
#pragma unroll 1
    for (int k = k0 - 1; k < k1; ++k) {
      compute_layer(k, k & 1);
      if (k + 1 < k1) prefetch_layer(k + 1);
      if (k < k0) continue;  // uniform across the CTA
      __syncthreads();
      if (owns_node) {
        A acc[27];
#pragma unroll
        for (int s = 0; s < 27; ++s) acc[s] = from_double<A>(0.0);
        // surrounding elements (i-1+a, j-1+b, k-1+c) in the fixed order c, b, a
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          const int ez = k - 1 + c;
          if (ez < 0 || ez >= nz) continue;
          const int buf = ez & 1;
#pragma unroll
          for (int b = 0; b < 2; ++b) {
            const int ey2 = nj - 1 + b;
            if (ey2 < 0 || ey2 >= ny) continue;
#pragma unroll
            for (int a = 0; a < 2; ++a) {
              const int ex2 = ni - 1 + a;
              if (ex2 < 0 || ex2 >= nx) continue;
              const int slot = (ex2 - (x0 - 1)) + (ey2 - (y0 - 1)) * kREX;
              const int li = (1 - a) + 2 * (1 - b) + 4 * (1 - c);
#pragma unroll
              for (int lj = 0; lj < 8; ++lj) {
                const int di = a - 1 + (lj & 1), dj = b - 1 + ((lj >> 1) & 1), dk = c - 1 + (lj >> 2);
                const int m = li < lj ? li : lj, n = li < lj ? lj : li;
                const int q = (dk + 1) * 9 + (dj + 1) * 3 + (di + 1);
                acc[q] = acc_add(acc[q], sK[buf][tri(m, n)][slot]);
              }
            }
          }
        }
        // write the row: the 27-point stencil clipped to the mesh, in ascending column order
        const long long r = (long long)ni + (long long)nj * NX + (long long)k * NXY;
        long long pos = (long long)__ldg(rp + r) - 1;
#pragma unroll
        for (int dk = -1; dk <= 1; ++dk) {
          if (k + dk < 0 || k + dk >= NZ) continue;
#pragma unroll
          for (int dj = -1; dj <= 1; ++dj) {
            if (nj + dj < 0 || nj + dj >= NY) continue;
#pragma unroll
            for (int di = -1; di <= 1; ++di) {
              if (ni + di < 0 || ni + di >= NX) continue;
              double v;
              float v32;
              entry_out(acc[(dk + 1) * 9 + (dj + 1) * 3 + (di + 1)], !std::is_same<T, float>::value, v, v32);
              values[pos] = v;
              if (values32) values32[pos] = v32;
              ++pos;
            }
          }
        }
        if (rhs) rhs[r] = 0.0;
      }
      __syncthreads();
    }
  }
  if (bad) gfe_raise(err, GFE_DEVERR_JACOBIAN);
  if (nonfinite) gfe_raise(err, GFE_DEVERR_NONFINITE);
}

// ---------------------------------------------------------------------------------------------
// Float-float on Iron's regular mesh: element work in two kernels, then a row gather
// ---------------------------------------------------------------------------------------------
// The float-float element routine is ~13.6 k instructions of straight-line code per element; inside
// the row-owning kernel its instruction stream does not fit the SM's instruction cache and warps
// stall on instruction fetch.  Split, each kernel's code fits: the metric kernel forms the 8
// Gauss-point metrics of every element once, the contraction kernel turns them into the 36 element
// matrix entries, and the gather kernel sums each CSR row from the matrices of the elements around
// its node, in the fixed order of the row-owning kernel (the values are bit-identical to it).

// Gauss-point metrics of element layers [ez0, ez1) into metrics, tiled by 32 elements (entry k of
// Gauss point g of element e at (48 (e / 32) + 8 k + g) 32 + e % 32).
template <typename T>
__global__ void __launch_bounds__(128)
laplace_metric_kernel(int32_t nx, int32_t ny, int32_t nz, const T* __restrict__ coords,
                      const double* __restrict__ kappa, T* __restrict__ metrics, int32_t ez0, int32_t ez1,
                      unsigned* err) {
  const long long EXY = (long long)nx * ny;
  const long long NX = nx + 1, NXY = NX * (ny + 1), N = NXY * (nz + 1);
  T p, q;
  gauss_pq(p, q);
  bool bad = false, nonfinite = false;
  for (long long e = ez0 * EXY + blockIdx.x * (long long)blockDim.x + threadIdx.x; e < ez1 * EXY;
       e += (long long)gridDim.x * blockDim.x) {
    const long long ex = e % nx, ey = (e / nx) % ny, ez = e / EXY;
    T x[3][8];
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      const long long n = (ex + (m & 1)) + (ey + ((m >> 1) & 1)) * NX + (ez + (m >> 2)) * NXY;
#pragma unroll
      for (int c = 0; c < 3; ++c) x[c][m] = load_coord(coords + c * N + n);
    }
    const double kd = kappa ? __ldg(kappa + e) : 1.0;
    if (!isfinite(kd)) nonfinite = true;
    T M[8][6];
    if (!hex8_metrics<T>(x, from_double<T>(kd), p, q, M)) bad = true;
    // tiles of 32 elements: entry j = 8 k + g of element e at (48 (e / 32) + j) 32 + e % 32, so a
    // warp's 32 consecutive elements write (and the contraction reads) each entry as 256
    // contiguous bytes, and a thread's 48 entries sit at immediate offsets from one address
    T* dst = metrics + (e >> 5) * (48 * 32) + (e & 31);
#pragma unroll
    for (int k = 0; k < 6; ++k)
#pragma unroll
      for (int g = 0; g < 8; ++g) dst[(k * 8 + g) * 32] = M[g][k];
  }
  if (bad) gfe_raise(err, GFE_DEVERR_JACOBIAN);
  if (nonfinite) gfe_raise(err, GFE_DEVERR_NONFINITE);
}

// Element matrices of element layers [ez0, ez1) from their metrics into Kel[36][E] (entry
// tri(m, n) of element e at tri(m, n) E + e).
template <typename T>
__global__ void __launch_bounds__(128)
laplace_contract_kernel(int32_t nx, int32_t ny, int32_t nz, const T* __restrict__ metrics, T* __restrict__ Kel,
                        int32_t ez0, int32_t ez1) {
  const long long EXY = (long long)nx * ny, E = EXY * nz;
  T p, q;
  gauss_pq(p, q);
  for (long long e = ez0 * EXY + blockIdx.x * (long long)blockDim.x + threadIdx.x; e < ez1 * EXY;
       e += (long long)gridDim.x * blockDim.x) {
    // a direction's component is loaded where the contraction uses it, not all 48 entries up front
    const T* src = metrics + (e >> 5) * (48 * 32) + (e & 31);
    T K[36];
    hex8_contract_at<T>([&](int g, int k) { return load_coord(src + (k * 8 + g) * 32); }, p, q, K);
#pragma unroll
    for (int k = 0; k < 36; ++k) Kel[k * E + e] = K[k];
  }
}

// Rows of node layers [l0, l1) gathered from the element matrices Kel of the (up to 8) elements
// around each node: a lane per row sums its 27-entry row in the order of the row-owning kernel
// (surrounding elements c, b, a; local column lj).  A warp takes 32 consecutive rows, whose entries
// are one contiguous range of the CSR values: the lanes stage their rows in shared memory and the
// warp writes the range with coalesced stores.  No CTA barrier; each element matrix is read by its 8
// nodes, mostly from L1/L2.
constexpr int kGatherWarps = 8;
constexpr int kGatherStage = 32 * 27;  // entries of 32 rows at most

template <typename T>
__global__ void __launch_bounds__(kGatherWarps * 32, 4)
laplace_gather_kernel(int32_t nx, int32_t ny, int32_t nz, const T* __restrict__ Kel, const int32_t* __restrict__ rp,
                      double* __restrict__ values, float* __restrict__ values32, double* __restrict__ rhs,
                      int32_t l0, int32_t l1) {
  using A = typename AccOf<T>::type;
  extern __shared__ __align__(16) unsigned char gsm[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  A* stage = reinterpret_cast<A*>(gsm) + w * kGatherStage;  // the rows' sums, converted on the way out
  const long long NX = nx + 1, NY = ny + 1, NZ = nz + 1, NXY = NX * NY;
  const long long EXY = (long long)nx * ny, E = EXY * nz;
  const long long r_end = l1 * NXY;
  for (long long base = l0 * NXY + ((long long)blockIdx.x * kGatherWarps + w) * 32; base < r_end;
       base += (long long)gridDim.x * kGatherWarps * 32) {
    const long long r = base + lane;
    const bool active = r < r_end;
    const long long pos0 = (long long)__ldg(rp + base) - 1;
    const long long pos_end = (long long)__ldg(rp + (base + 32 < r_end ? base + 32 : r_end)) - 1;
    if (active) {
      const int ni = (int)(r % NX), nj = (int)((r / NX) % NY), k = (int)(r / NXY);
      int o = (int)((long long)__ldg(rp + r) - 1 - pos0);
      // one column layer dk of the row at a time (9 accumulators live instead of 27): the element
      // layer ez = k - 1 + c adds its local columns lj < 4 to layer dk = c - 1 and lj >= 4 to
      // dk = c, so every entry is loaded once and each sum keeps the order c, b, a
#pragma unroll
      for (int dk = -1; dk <= 1; ++dk) {
        if (k + dk < 0 || k + dk >= NZ) continue;
        A acc[9];
#pragma unroll
        for (int t = 0; t < 9; ++t) acc[t] = from_double<A>(0.0);
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          const int hi = dk - c + 1;  // which half of the element's local columns
          if (hi < 0 || hi > 1) continue;
          const int ez = k - 1 + c;
          if (ez < 0 || ez >= nz) continue;
#pragma unroll
          for (int b = 0; b < 2; ++b) {
            const int ey2 = nj - 1 + b;
            if (ey2 < 0 || ey2 >= ny) continue;
#pragma unroll
            for (int a = 0; a < 2; ++a) {
              const int ex2 = ni - 1 + a;
              if (ex2 < 0 || ex2 >= nx) continue;
              const long long e = ex2 + ey2 * (long long)nx + ez * EXY;
              const int li = (1 - a) + 2 * (1 - b) + 4 * (1 - c);
#pragma unroll
              for (int l4 = 0; l4 < 4; ++l4) {
                const int lj = hi * 4 + l4;
                const int di = a - 1 + (lj & 1), dj = b - 1 + ((lj >> 1) & 1);
                const int m = li < lj ? li : lj, n = li < lj ? lj : li;
                const int t = (dj + 1) * 3 + (di + 1);
                acc[t] = acc_add(acc[t], load_coord(Kel + tri(m, n) * E + e));
              }
            }
          }
        }
        // this layer of the row, clipped to the mesh, in ascending column order, staged at its
        // offset in the range
#pragma unroll
        for (int dj = -1; dj <= 1; ++dj) {
          if (nj + dj < 0 || nj + dj >= NY) continue;
#pragma unroll
          for (int di = -1; di <= 1; ++di) {
            if (ni + di < 0 || ni + di >= NX) continue;
            stage[o++] = acc[(dj + 1) * 3 + (di + 1)];
          }
        }
      }
      if (rhs) rhs[r] = 0.0;
    }
    __syncwarp();
    const int total = (int)(pos_end - pos0);  // <= 32 x 27: the rows of a regular mesh
    for (int i = lane; i < total; i += 32) {
      double v;
      float v32;
      entry_out(stage[i], !std::is_same<T, float>::value, v, v32);
      values[pos0 + i] = v;
      if (values32) values32[pos0 + i] = v32;
    }
    __syncwarp();
  }
}

// Persistent grid of the regular-mesh kernel: the resident CTAs, but no more than one CTA per
// kRMinRun layers of one tile column.
template <typename T>
int regular_grid(int32_t nx, int32_t ny, int32_t l0, int32_t l1, size_t smem, int* grid) {
  static std::atomic<int> cached[64];  // resident CTAs per SM, per device (0: not yet queried)
  int dev = 0;
  GFE_CUDA_TRY(cudaGetDevice(&dev));
  int per_sm = dev < 64 ? cached[dev].load(std::memory_order_relaxed) : 0;
  if (per_sm == 0) {
    GFE_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, laplace_regular_kernel<T>, kRThreads, smem));
    if (dev < 64) cached[dev].store(per_sm, std::memory_order_relaxed);
  }
  const long long cols = (long long)((nx + 1 + kRTX - 1) / kRTX) * ((ny + 1 + kRTY - 1) / kRTY);
  const long long W = cols * (l1 - l0);
  const long long g = std::min<long long>((long long)std::max(per_sm, 1) * gfe::sm_count(),
                                          std::max<long long>(1, (W + kRMinRun - 1) / kRMinRun));
  *grid = (int)g;
  return GFE_OK;
}

// Structure check: every row of the CSR is the clipped 27-point stencil of a regular mesh.
__global__ void laplace_regular_check_kernel(int32_t nx, int32_t ny, int32_t nz, const int32_t* __restrict__ rp,
                                             const int32_t* __restrict__ ci, unsigned long long* bad) {
  const int NX = nx + 1, NY = ny + 1, NZ = nz + 1;
  const long long N = (long long)NX * NY * NZ;
  unsigned long long mism = 0;
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < N; r += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(r % NX), j = (int)((r / NX) % NY), k = (int)(r / ((long long)NX * NY));
    long long pos = rp[r] - 1;
    const long long end = rp[r + 1] - 1;
    for (int dk = -1; dk <= 1; ++dk)
      for (int dj = -1; dj <= 1; ++dj)
        for (int di = -1; di <= 1; ++di) {
          if (i + di < 0 || i + di >= NX || j + dj < 0 || j + dj >= NY || k + dk < 0 || k + dk >= NZ) continue;
          const long long col = r + di + (long long)dj * NX + (long long)dk * NX * NY;
          if (pos >= end || ci[pos] != col + 1) ++mism;
          ++pos;
        }
    if (pos != end) ++mism;
  }
  if (mism) atomicAdd(bad, mism);
}

int check_precision(int precision, const char* fn) {
  if (precision != GFE_FP64 && precision != GFE_MIXED && precision != GFE_MIXED_DF)
    return gfe::set_error(GFE_ERR_ARG, "%s: unknown precision %d", fn, precision);
  return GFE_OK;
}

int check_common(int32_t n_elem, int32_t n_nodes, const int32_t* elem_nodes, const double* coords, int precision,
                 const char* fn) {
  if (n_elem < 0 || n_nodes <= 0 || (n_elem > 0 && (!elem_nodes || !coords)))
    return gfe::set_error(GFE_ERR_ARG, "%s: invalid mesh arguments (n_elem=%d n_nodes=%d)", fn, n_elem, n_nodes);
  if (int rc = check_precision(precision, fn)) return rc;
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

// Workspace of the FP32-pipe precisions: the converted coordinates and, for float-float, behind
// them at a 256-byte boundary the Gauss-point metrics (48 float-float numbers an element) and the
// element matrices (36) of every element.  0 for FP64.
size_t regular_coords_bytes(int32_t nx, int32_t ny, int32_t nz, int precision) {
  const size_t n3 = 3ull * (nx + 1) * (ny + 1) * (nz + 1);
  if (precision == GFE_FP64) return 0;
  return (n3 * (precision == GFE_MIXED ? sizeof(float) : sizeof(f2)) + 255) & ~size_t(255);
}
size_t regular_metric_entries(int32_t nx, int32_t ny, int32_t nz) {  // 48 per element, tiles of 32
  return 48ull * (((size_t)nx * ny * nz + 31) & ~size_t(31));
}
size_t regular_workspace_bytes(int32_t nx, int32_t ny, int32_t nz, int precision) {
  const size_t cb = regular_coords_bytes(nx, ny, nz, precision);
  if (precision != GFE_MIXED_DF) return cb;
  return cb + (regular_metric_entries(nx, ny, nz) + 36ull * nx * ny * nz) * sizeof(f2);
}

constexpr int kSplitThreads = 128;
constexpr int kContractThreads = 128;

// Float-float element work of element layers [ez0, ez1): metric kernel, then contraction kernel,
// each element once, into the workspace's element-matrix array.
void launch_elements_f2(cudaStream_t s, int32_t nx, int32_t ny, int32_t nz, const f2* ct, const double* kappa,
                        void* ws, int32_t ez0, int32_t ez1, unsigned* err) {
  if (ez1 <= ez0) return;
  const long long cnt = (long long)(ez1 - ez0) * nx * ny;
  const int grid = (int)std::min<long long>((cnt + kSplitThreads - 1) / kSplitThreads, 40ll * gfe::sm_count());
  // 128-thread blocks: with ~170 (metric) and ~130 (contraction) registers a thread, three and four
  // blocks share an SM (12 and 16 warps), where 256-thread blocks left room for one
  const int cgrid = (int)std::min<long long>((cnt + kContractThreads - 1) / kContractThreads, 60ll * gfe::sm_count());
  f2* metrics = reinterpret_cast<f2*>(static_cast<char*>(ws) + regular_coords_bytes(nx, ny, nz, GFE_MIXED_DF));
  f2* Kel = metrics + regular_metric_entries(nx, ny, nz);
  laplace_metric_kernel<f2><<<grid, kSplitThreads, 0, s>>>(nx, ny, nz, ct, kappa, metrics, ez0, ez1, err);
  laplace_contract_kernel<f2><<<cgrid, kContractThreads, 0, s>>>(nx, ny, nz, metrics, Kel, ez0, ez1);
}

void launch_gather_f2(cudaStream_t s, int32_t nx, int32_t ny, int32_t nz, const void* ws, const int32_t* rp,
                      double* values, float* values32, double* rhs, int32_t l0, int32_t l1) {
  if (l1 <= l0) return;
  const long long rows = (long long)(l1 - l0) * (nx + 1) * (ny + 1);
  const int grid = (int)std::min<long long>((rows + kGatherWarps * 32 - 1) / (kGatherWarps * 32),
                                            8ll * gfe::sm_count());
  const f2* Kel = reinterpret_cast<const f2*>(static_cast<const char*>(ws) +
                                              regular_coords_bytes(nx, ny, nz, GFE_MIXED_DF)) +
                  regular_metric_entries(nx, ny, nz);
  const size_t smem = (size_t)kGatherWarps * kGatherStage * sizeof(f2);
  cudaFuncSetAttribute((const void*)laplace_gather_kernel<f2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  laplace_gather_kernel<f2><<<grid, kGatherWarps * 32, smem, s>>>(nx, ny, nz, Kel, rp, values, values32, rhs, l0, l1);
}

// Node layers [l0, l1) (l0 a multiple of kRZ).  ws: caller workspace of regular_workspace_bytes(),
// or NULL to allocate it on the stream; split: convert the coordinates into it first (the later
// layer calls of one assembly reuse the converted array).  FP32: the row-owning tiled kernel.
// Float-float: the element work of the element layers the rows read ([l0 - 1, l1) within the mesh;
// a neighbouring slab on another stream may write the matrices of the layer between them at the
// same time, with identical values), then the row gather.
template <typename T>
int launch_regular(cudaStream_t s, int32_t nx, int32_t ny, int32_t nz, const double* coords,
                   const double* kappa, const int32_t* rp, double* values, float* values32, double* rhs,
                   unsigned* err, void* ws, int32_t l0, int32_t l1, bool split) {
  constexpr bool DF = std::is_same<T, f2>::value;
  const int prec = DF ? GFE_MIXED_DF : GFE_MIXED;
  const long long n3 = 3ll * (nx + 1) * (ny + 1) * (nz + 1);
  char* base = static_cast<char*>(ws);
  if (!base)
    if (int rc = gfe::scratch_alloc((void**)&base, regular_workspace_bytes(nx, ny, nz, prec), s, "split coordinates"))
      return rc;
  T* ct = reinterpret_cast<T*>(base);
  if (split || !ws) split_coords<T><<<4 * gfe::sm_count(), 256, 0, s>>>(n3, coords, ct);
  if constexpr (DF) {
    launch_elements_f2(s, nx, ny, nz, ct, kappa, base, std::max(l0 - 1, 0), std::min(l1, nz), err);
    launch_gather_f2(s, nx, ny, nz, base, rp, values, values32, rhs, l0, l1);
  } else {
    const size_t smem = 2 * 36 * kRThreads * sizeof(typename StoreOf<T>::type);
    GFE_CUDA_TRY(cudaFuncSetAttribute((const void*)laplace_regular_kernel<T>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int grid = 0;
    if (int rc = regular_grid<T>(nx, ny, l0, l1, smem, &grid)) return rc;
    laplace_regular_kernel<T><<<grid, kRThreads, smem, s>>>(nx, ny, nz, ct, kappa, rp, values, values32, rhs, err,
                                                             l0, l1);
  }
  if (!ws) gfe::scratch_free(base, s);
  return GFE_OK;
}

template <>
int launch_regular<double>(cudaStream_t s, int32_t nx, int32_t ny, int32_t nz, const double* coords,
                           const double* kappa, const int32_t* rp, double* values, float* values32, double* rhs,
                           unsigned* err, void*, int32_t l0, int32_t l1, bool) {
  const size_t smem = 2 * 36 * kRThreads * sizeof(double);
  GFE_CUDA_TRY(cudaFuncSetAttribute((const void*)laplace_regular_kernel<double>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int grid = 0;
  if (int rc = regular_grid<double>(nx, ny, l0, l1, smem, &grid)) return rc;
  laplace_regular_kernel<double><<<grid, kRThreads, smem, s>>>(nx, ny, nz, coords, kappa, rp, values, values32, rhs,
                                                               err, l0, l1);
  return GFE_OK;
}

template <typename T>
void launch_color(int grid, cudaStream_t s, const int32_t* ce, int cnt, int32_t n_nodes, const int32_t* en,
                  const double* xyz, const double* kappa, const int32_t* rp, const int32_t* ci, double* values,
                  unsigned* err) {
  laplace_assemble_color<T><<<grid, kBlock, 0, s>>>(ce, cnt, n_nodes, en, xyz, kappa, rp, ci, values, err);
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
      launch_color<double>(grid, s, color_elems + c0, cnt, n_nodes, elem_nodes, coords, kappa, row_ptr, col_idx,
                           values, err);
    else if (precision == GFE_MIXED)
      launch_color<float>(grid, s, color_elems + c0, cnt, n_nodes, elem_nodes, coords, kappa, row_ptr, col_idx,
                          values, err);
    else
      launch_color<f2>(grid, s, color_elems + c0, cnt, n_nodes, elem_nodes, coords, kappa, row_ptr, col_idx, values,
                       err);
    ++launches;
  }
  gfe::stage_end(GFE_STAGE_LAPLACE_ELEMENTS, prof, s, launches);
  if (values32) to_fp32<<<4 * gfe::sm_count(), 256, 0, s>>>(values, values32, nnz);
  GFE_LAUNCH_CHECK(fn);
  return GFE_OK;
}

extern "C" int64_t gfe_laplace_regular_workspace_bytes(int32_t nx, int32_t ny, int32_t nz, int32_t precision) {
  if (nx <= 0 || ny <= 0 || nz <= 0) return 0;
  return (int64_t)regular_workspace_bytes(nx, ny, nz, precision);
}

extern "C" int gfe_laplace_assemble_regular(int32_t nx, int32_t ny, int32_t nz, const double* coords,
                                            const double* kappa, const int32_t* row_ptr, double* values,
                                            float* values32, double* rhs, int32_t precision, void* stream) {
  return gfe_laplace_assemble_regular_ws(nx, ny, nz, coords, kappa, row_ptr, values, values32, rhs, precision,
                                         nullptr, stream);
}

extern "C" int gfe_laplace_assemble_regular_ws(int32_t nx, int32_t ny, int32_t nz, const double* coords,
                                               const double* kappa, const int32_t* row_ptr, double* values,
                                               float* values32, double* rhs, int32_t precision, void* workspace,
                                               void* stream) {
  return gfe_laplace_assemble_regular_layers(nx, ny, nz, coords, kappa, row_ptr, values, values32, rhs, precision,
                                             workspace, 0, nz + 1, 1, stream);
}

extern "C" int gfe_laplace_assemble_regular_layers(int32_t nx, int32_t ny, int32_t nz, const double* coords,
                                                   const double* kappa, const int32_t* row_ptr, double* values,
                                                   float* values32, double* rhs, int32_t precision, void* workspace,
                                                   int32_t layer_begin, int32_t layer_end, int32_t convert_coords,
                                                   void* stream) {
  const char* fn = "gfe_laplace_assemble_regular";
  if (nx <= 0 || ny <= 0 || nz <= 0 || !coords || !row_ptr || !values)
    return gfe::set_error(GFE_ERR_ARG, "%s: invalid arguments", fn);
  if (int rc = check_precision(precision, fn)) return rc;
  if (workspace && (reinterpret_cast<uintptr_t>(workspace) & 15))
    return gfe::set_error(GFE_ERR_ARG, "%s: workspace must be 16-byte aligned", fn);
  if (layer_begin < 0 || layer_end > nz + 1 || layer_begin > layer_end || layer_begin % kRZ != 0)
    return gfe::set_error(GFE_ERR_ARG, "%s: node layers [%d, %d) must lie in [0, %d) and start at a multiple of %d",
                          fn, layer_begin, layer_end, nz + 1, kRZ);
  if (!workspace && !convert_coords)
    return gfe::set_error(GFE_ERR_ARG, "%s: without a workspace the coordinates are converted every call", fn);
  cudaStream_t s = gfe::as_stream(stream);
  if (layer_begin == layer_end) {
    // an empty range only converts the coordinates into the workspace
    if (!workspace || !convert_coords)
      return gfe::set_error(GFE_ERR_ARG, "%s: an empty layer range needs a workspace and convert_coords", fn);
    const long long n3 = 3ll * (nx + 1) * (ny + 1) * (nz + 1);
    if (precision == GFE_MIXED) split_coords<float><<<4 * gfe::sm_count(), 256, 0, s>>>(n3, coords, (float*)workspace);
    else if (precision == GFE_MIXED_DF) split_coords<f2><<<4 * gfe::sm_count(), 256, 0, s>>>(n3, coords, (f2*)workspace);
    GFE_LAUNCH_CHECK(fn);
    return GFE_OK;
  }
  unsigned* err = gfe::device_error_word();
  void* prof = gfe::stage_begin(GFE_STAGE_LAPLACE_ELEMENTS, s);
  int rc;
  const int32_t l0 = layer_begin, l1 = layer_end;
  const bool cv = convert_coords != 0;
  if (precision == GFE_FP64)
    rc = launch_regular<double>(s, nx, ny, nz, coords, kappa, row_ptr, values, values32, rhs, err, workspace,
                                l0, l1, cv);
  else if (precision == GFE_MIXED)
    rc = launch_regular<float>(s, nx, ny, nz, coords, kappa, row_ptr, values, values32, rhs, err, workspace,
                               l0, l1, cv);
  else
    rc = launch_regular<f2>(s, nx, ny, nz, coords, kappa, row_ptr, values, values32, rhs, err, workspace, l0,
                            l1, cv);
  gfe::stage_end(GFE_STAGE_LAPLACE_ELEMENTS, prof, s, precision == GFE_MIXED_DF ? 3 : 1);
  if (rc) return rc;
  GFE_LAUNCH_CHECK(fn);
  return GFE_OK;
}

namespace {

// Node layers [a, a + n) of each coordinate component (component-major [3][NXY * NZ], layers
// contiguous) converted into the workspace: the slab-wise form of split_coords.
template <typename T>
__global__ void split_coords_layers(long long per_comp, long long a, long long n, const double* __restrict__ in,
                                    T* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < 3 * n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long j = (i / n) * per_comp + a + i % n;
    out[j] = from_double<T>(in[j]);
  }
}

// CSR entries in the rows of node layers [0, L) of the regular mesh: every row holds its clipped
// 27-point stencil, so the count factorises into (3 NX - 2)(3 NY - 2) times the clipped widths
// along xi3.  Equals row_ptr[L * NX * NY] - 1 for the structure gfe_laplace_regular_check accepts.
long long regular_entries_before(int32_t nx, int32_t ny, int32_t nz, int32_t L) {
  const long long NX = nx + 1, NY = ny + 1, NZ = nz + 1;
  long long w = 0;
  for (long long l = 0; l < L; ++l) w += 3 - (l == 0) - (l == NZ - 1);
  return (3 * NX - 2) * (3 * NY - 2) * w;
}

// Streams and events of the host-buffer pipeline, one set per host thread and device, created on
// first use and kept for the thread's lifetime (the driver releases them at process exit).
struct HostPipe {
  int dev = -1;
  cudaStream_t in = nullptr, comp[2] = {nullptr, nullptr}, out = nullptr;
  std::vector<cudaEvent_t> ev;
};
thread_local std::vector<HostPipe> t_pipes;

int host_pipe(HostPipe** out, size_t n_events) {
  int dev = 0;
  GFE_CUDA_TRY(cudaGetDevice(&dev));
  HostPipe* hp = nullptr;
  for (auto& p : t_pipes)
    if (p.dev == dev) hp = &p;
  if (!hp) {
    HostPipe p;
    p.dev = dev;
    GFE_CUDA_TRY(cudaStreamCreateWithFlags(&p.in, cudaStreamNonBlocking));
    GFE_CUDA_TRY(cudaStreamCreateWithFlags(&p.comp[0], cudaStreamNonBlocking));
    GFE_CUDA_TRY(cudaStreamCreateWithFlags(&p.comp[1], cudaStreamNonBlocking));
    GFE_CUDA_TRY(cudaStreamCreateWithFlags(&p.out, cudaStreamNonBlocking));
    t_pipes.push_back(p);
    hp = &t_pipes.back();
  }
  while (hp->ev.size() < n_events) {
    cudaEvent_t e;
    GFE_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    hp->ev.push_back(e);
  }
  *out = hp;
  return GFE_OK;
}

}  // namespace

extern "C" int gfe_laplace_assemble_regular_host(int32_t nx, int32_t ny, int32_t nz, const double* coords_host,
                                                 const double* kappa_host, double* coords, double* kappa,
                                                 const int32_t* row_ptr, double* values, double* values_host,
                                                 double* rhs, int32_t precision, void* workspace,
                                                 int32_t slab_layers, void* stream) {
  const char* fn = "gfe_laplace_assemble_regular_host";
  if (nx <= 0 || ny <= 0 || nz <= 0 || !coords || !row_ptr || !values || !values_host)
    return gfe::set_error(GFE_ERR_ARG, "%s: invalid arguments", fn);
  if (int rc = check_precision(precision, fn)) return rc;
  if (kappa_host && !kappa) return gfe::set_error(GFE_ERR_ARG, "%s: kappa_host needs a device kappa array", fn);
  if (precision != GFE_FP64 && (!workspace || (reinterpret_cast<uintptr_t>(workspace) & 15)))
    return gfe::set_error(GFE_ERR_ARG, "%s: the FP32-pipe precisions need a 16-byte aligned workspace", fn);
  if (slab_layers == 0) slab_layers = 2 * kRZ;
  if (slab_layers < 0 || slab_layers % kRZ != 0)
    return gfe::set_error(GFE_ERR_ARG, "%s: slab_layers must be a positive multiple of %d", fn, kRZ);
  const long long NX = nx + 1, NY = ny + 1, NZ = nz + 1, NXY = NX * NY, N = NXY * NZ, EXY = (long long)nx * ny;
  // slabs of node layers: [0, kRZ) first, so the first copy-out starts early, then slab_layers each
  std::vector<int32_t> cut{0};
  for (long long l = std::min<long long>(kRZ, NZ); cut.back() < NZ; l = std::min<long long>(l + slab_layers, NZ))
    cut.push_back((int32_t)l);
  const int n_slabs = (int)cut.size() - 1;
  HostPipe* hp = nullptr;
  if (int rc = host_pipe(&hp, 2 * (size_t)n_slabs + 4)) return rc;
  cudaStream_t s = gfe::as_stream(stream);
  cudaEvent_t* ev = hp->ev.data();
  unsigned* err = gfe::device_error_word();
  void* prof = gfe::stage_begin(GFE_STAGE_LAPLACE_ELEMENTS, s);
  // every pipeline stream starts after the work already on `stream`
  GFE_CUDA_TRY(cudaEventRecord(ev[0], s));
  for (cudaStream_t t : {hp->in, hp->comp[0], hp->comp[1], hp->out}) GFE_CUDA_TRY(cudaStreamWaitEvent(t, ev[0], 0));
  long long node_hi = 0, elem_hi = 0;  // node / element layers uploaded so far
  const int cvt_grid = 2 * gfe::sm_count();
  for (int i = 0; i < n_slabs; ++i) {
    const int32_t l0 = cut[i], l1 = cut[i + 1];
    cudaEvent_t ev_in = ev[1 + 2 * i], ev_c = ev[2 + 2 * i];
    // inputs: the node layers [l0 - 1, l1] and element layers [l0 - 1, l1 - 1] this slab reads
    const long long nh = std::min<long long>(l1 + 1, NZ), eh = std::min<long long>(l1, nz);
    if (nh > node_hi) {
      if (coords_host)
        for (int c = 0; c < 3; ++c) {
          const long long o = c * N + node_hi * NXY;
          GFE_CUDA_TRY(cudaMemcpyAsync(coords + o, coords_host + o, sizeof(double) * (nh - node_hi) * NXY,
                                       cudaMemcpyHostToDevice, hp->in));
        }
      if (precision == GFE_MIXED)
        split_coords_layers<float><<<cvt_grid, 256, 0, hp->in>>>(N, node_hi * NXY, (nh - node_hi) * NXY, coords,
                                                                 static_cast<float*>(workspace));
      else if (precision == GFE_MIXED_DF)
        split_coords_layers<f2><<<cvt_grid, 256, 0, hp->in>>>(N, node_hi * NXY, (nh - node_hi) * NXY, coords,
                                                              static_cast<f2*>(workspace));
      node_hi = nh;
    }
    if (kappa_host && eh > elem_hi) {
      GFE_CUDA_TRY(cudaMemcpyAsync(kappa + elem_hi * EXY, kappa_host + elem_hi * EXY,
                                   sizeof(double) * (eh - elem_hi) * EXY, cudaMemcpyHostToDevice, hp->in));
      elem_hi = eh;
    }
    // float-float: the element work of the slab's own element layers on the input stream, in slab
    // order, so the next slab's rows find the matrices of the element layer below them written
    if (precision == GFE_MIXED_DF)
      launch_elements_f2(hp->in, nx, ny, nz, static_cast<const f2*>(workspace), kappa, workspace, l0,
                         std::min<int32_t>(l1, nz), err);
    GFE_CUDA_TRY(cudaEventRecord(ev_in, hp->in));
    // the slab on alternating compute streams: one slab's last wave overlaps the next one's first
    cudaStream_t cs = hp->comp[i & 1];
    GFE_CUDA_TRY(cudaStreamWaitEvent(cs, ev_in, 0));
    int rc;
    if (precision == GFE_FP64)
      rc = launch_regular<double>(cs, nx, ny, nz, coords, kappa, row_ptr, values, nullptr, rhs, err, nullptr,
                                  l0, l1, false);
    else if (precision == GFE_MIXED)
      rc = launch_regular<float>(cs, nx, ny, nz, coords, kappa, row_ptr, values, nullptr, rhs, err, workspace,
                                 l0, l1, false);
    else {
      launch_gather_f2(cs, nx, ny, nz, workspace, row_ptr, values, nullptr, rhs, l0, l1);
      rc = GFE_OK;
    }
    if (rc) return rc;
    GFE_CUDA_TRY(cudaEventRecord(ev_c, cs));
    // the slab's rows are one contiguous range of the CSR values
    GFE_CUDA_TRY(cudaStreamWaitEvent(hp->out, ev_c, 0));
    const long long a = regular_entries_before(nx, ny, nz, l0), b = regular_entries_before(nx, ny, nz, l1);
    GFE_CUDA_TRY(cudaMemcpyAsync(values_host + a, values + a, sizeof(double) * (b - a), cudaMemcpyDeviceToHost,
                                 hp->out));
  }
  // `stream` resumes after the copies (which follow every slab) and the input stream
  cudaEvent_t ev_out = ev[1 + 2 * n_slabs], ev_in_end = ev[2 + 2 * n_slabs];
  GFE_CUDA_TRY(cudaEventRecord(ev_out, hp->out));
  GFE_CUDA_TRY(cudaEventRecord(ev_in_end, hp->in));
  GFE_CUDA_TRY(cudaStreamWaitEvent(s, ev_out, 0));
  GFE_CUDA_TRY(cudaStreamWaitEvent(s, ev_in_end, 0));
  gfe::stage_end(GFE_STAGE_LAPLACE_ELEMENTS, prof, s, n_slabs);
  GFE_LAUNCH_CHECK(fn);
  return GFE_OK;
}

extern "C" int gfe_laplace_regular_check(int32_t nx, int32_t ny, int32_t nz, const int32_t* row_ptr,
                                         const int32_t* col_idx, int64_t* mismatches_host, void* stream) {
  const char* fn = "gfe_laplace_regular_check";
  if (nx <= 0 || ny <= 0 || nz <= 0 || !row_ptr || !col_idx || !mismatches_host)
    return gfe::set_error(GFE_ERR_ARG, "%s: invalid arguments", fn);
  cudaStream_t s = gfe::as_stream(stream);
  unsigned long long* bad = nullptr;
  int rc = gfe::scratch_alloc((void**)&bad, sizeof(unsigned long long), s, "check counter");
  if (rc) return rc;
  cudaMemsetAsync(bad, 0, sizeof(unsigned long long), s);
  laplace_regular_check_kernel<<<8 * gfe::sm_count(), 256, 0, s>>>(nx, ny, nz, row_ptr, col_idx, bad);
  unsigned long long h = 0;
  cudaMemcpyAsync(&h, bad, sizeof(h), cudaMemcpyDeviceToHost, s);
  gfe::scratch_free(bad, s);
  GFE_CUDA_TRY(cudaStreamSynchronize(s));
  GFE_LAUNCH_CHECK(fn);
  *mismatches_host = (int64_t)h;
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
  else if (precision == GFE_MIXED)
    laplace_element_kernel<float><<<grid, kBlock, 0, s>>>(n_elem, n_nodes, elem_nodes, coords, kappa, K_out, err);
  else
    laplace_element_kernel<f2><<<grid, kBlock, 0, s>>>(n_elem, n_nodes, elem_nodes, coords, kappa, K_out, err);
  GFE_LAUNCH_CHECK(fn);
  return check_device_errors(s, fn, true);
}
