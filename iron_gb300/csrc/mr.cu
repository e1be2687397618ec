// mr.cu -- K4 / K5: Mooney-Rivlin (mixed u-p, triquadratic u + trilinear p) residual and Iron's
// analytic Jacobian, batched over elements (and over parameter sets for the residual).
//
// Reference: FiniteElasticity_FiniteElementResidualEvaluate, MOONEY_RIVLIN_SUBTYPE branch
// (src/finite_elasticity_routines.F90:1669-1756), FINITE_ELASTICITY_GAUSS_STRESS_TENSOR (:6985-7061),
// FiniteElasticity_GaussDeformationGradientTensor (:5148-5215) with the material frame of
// Coordinates_MaterialSystemCalculate (src/coordinate_routines.F90:3841-3947),
// FiniteElasticity_FiniteElementJacobianEvaluate (:1016-1274) and
// FINITE_ELASTICITY_GAUSS_ELASTICITY_TENSOR (:649-795).
//
// Field layout (Iron's separated component order): the dependent vector holds the deformed
// positions z1, z2, z3 over the n_q2 quadratic nodes followed by the pressure over the n_lin
// linear (corner) nodes; the geometric field x is [3][n_q2].  Element DOF order: 27 z1, 27 z2,
// 27 z3, 8 p (Iron's element parameter order, local nodes xi1 fastest).
//
// Residual: one warp per (element, parameter set).  Lane g < 27 evaluates Gauss point g (metrics,
// deformation gradient, stress) and leaves P_g = J_z w_g Z^-1 sigma (3x3) and
// J_x w_g (J_z/J_x - 1) in shared memory; the lanes then form the 89 entries as sums over Gauss
// points in a fixed order (deterministic) and scatter them into the global residual.  Elements
// are processed colour by colour, so no two elements of a launch share a DOF.
//
// Jacobian: one CTA per element.  Threads 0..26 build, per Gauss point, the spatial basis
// gradients dphi/dz and the 3x3 blocks J_z w (c + sigma) of Iron's analytic tangent; all threads
// then form the lower u-u triangle and the u-p / p-u blocks and add them into the CSR values
// through a precomputed per-element slot map (u-u upper triangle mirrored, p-p structurally zero).
#include <mutex>
#include <type_traits>

#include "df.cuh"
#include "gfe_internal.cuh"
#include "tcgen05.cuh"

namespace {

constexpr int NQ = 27;   // quadratic element nodes
constexpr int NL = 8;    // linear (pressure) element nodes
constexpr int NG = 27;   // Gauss points (3x3x3)
constexpr int ND = 89;   // element DOFs

// 16-byte multiple in size, so that a TMA bulk copy can stage the whole table
template <typename S>
struct alignas(16) TablesT {
  S dphi[NG][3][NQ];  // d phi_ns / d xi_k at Gauss point g (quadratic basis)
  S w[NG];
  S psi[NG][NL];      // linear basis values at the Gauss points
};
using Tables = TablesT<double>;
using TablesF = TablesT<float>;  // FP32 copy read by the FP32 Gauss-point kernel

// Host construction of the tables (Gauss-Legendre 3-point rule on [0,1], Lagrange bases),
// src/basis_routines.F90:3720-4090, 6804-6890, 7969-8090.
void build_tables(Tables& t) {
  const double s = std::sqrt(0.6);
  const double gx[3] = {(-s + 1.0) / 2.0, 0.5, (s + 1.0) / 2.0};
  const double gw[3] = {2.5 / 9.0, 4.0 / 9.0, 2.5 / 9.0};
  auto q = [](int a, int d, double x) {
    if (d == 0) return a == 0 ? 1.0 - 3.0 * x + 2.0 * x * x : (a == 1 ? 4.0 * x * (1.0 - x) : x * (x + x - 1.0));
    return a == 0 ? 4.0 * x - 3.0 : (a == 1 ? 4.0 - 8.0 * x : 4.0 * x - 1.0);
  };
  auto l = [](int a, double x) { return a == 0 ? 1.0 - x : x; };
  for (int g3 = 0; g3 < 3; ++g3)
    for (int g2 = 0; g2 < 3; ++g2)
      for (int g1 = 0; g1 < 3; ++g1) {
        const int g = g1 + 3 * (g2 + 3 * g3);
        const double xg[3] = {gx[g1], gx[g2], gx[g3]};
        t.w[g] = gw[g1] * gw[g2] * gw[g3];
        for (int a3 = 0; a3 < 3; ++a3)
          for (int a2 = 0; a2 < 3; ++a2)
            for (int a1 = 0; a1 < 3; ++a1) {
              const int ns = a1 + 3 * (a2 + 3 * a3);
              const int ai[3] = {a1, a2, a3};
              for (int k = 0; k < 3; ++k) {
                double v = 1.0;
                for (int d = 0; d < 3; ++d) v *= q(ai[d], d == k ? 1 : 0, xg[d]);
                t.dphi[g][k][ns] = v;
              }
            }
        for (int b3 = 0; b3 < 2; ++b3)
          for (int b2 = 0; b2 < 2; ++b2)
            for (int b1 = 0; b1 < 2; ++b1) t.psi[g][b1 + 2 * (b2 + 2 * b3)] = l(b1, xg[0]) * l(b2, xg[1]) * l(b3, xg[2]);
      }
}

std::mutex g_tab_mu;
Tables* g_tables[64] = {nullptr};

int device_tables(const Tables** out) {
  int dev = 0;
  GFE_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_tab_mu);
  if (!g_tables[dev]) {
    Tables h;
    build_tables(h);
    void* p = nullptr;
    GFE_CUDA_TRY(cudaMalloc(&p, sizeof(Tables)));
    GFE_CUDA_TRY(cudaMemcpy(p, &h, sizeof(Tables), cudaMemcpyHostToDevice));
    g_tables[dev] = static_cast<Tables*>(p);
  }
  *out = g_tables[dev];
  return GFE_OK;
}

TablesF* g_tables_f[64] = {nullptr};

int device_tables_f(const TablesF** out) {
  int dev = 0;
  GFE_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_tab_mu);
  if (!g_tables_f[dev]) {
    Tables h;
    build_tables(h);
    TablesF f;
    for (int g = 0; g < NG; ++g) {
      f.w[g] = (float)h.w[g];
      for (int k = 0; k < 3; ++k)
        for (int n = 0; n < NQ; ++n) f.dphi[g][k][n] = (float)h.dphi[g][k][n];
      for (int m = 0; m < NL; ++m) f.psi[g][m] = (float)h.psi[g][m];
    }
    void* p = nullptr;
    GFE_CUDA_TRY(cudaMalloc(&p, sizeof(TablesF)));
    GFE_CUDA_TRY(cudaMemcpy(p, &f, sizeof(TablesF), cudaMemcpyHostToDevice));
    g_tables_f[dev] = static_cast<TablesF*>(p);
  }
  *out = g_tables_f[dev];
  return GFE_OK;
}

// Voigt index of tensor entry (i, j) and the tensor entries of Voigt index v, as arithmetic so that
// unrolled loops index register arrays with constants: 11 22 33 12 13 23.
__host__ __device__ constexpr int t2v(int i, int j) { return i == j ? i : i + j + 2; }
__host__ __device__ constexpr int v2t_a(int v) { return v < 3 ? v : (v == 5 ? 1 : 0); }
__host__ __device__ constexpr int v2t_b(int v) { return v < 3 ? v : (v == 3 ? 1 : 2); }

// Inverse and determinant with Iron's cofactor formulas (src/maths.F90:2807-2868).
template <typename S>
__device__ __forceinline__ S inv3(const S A[3][3], S B[3][3]) {
  const S det = A[0][0] * A[1][1] * A[2][2] + A[0][1] * A[1][2] * A[2][0] + A[0][2] * A[1][0] * A[2][1] -
                A[0][0] * A[2][1] * A[1][2] - A[1][0] * A[0][1] * A[2][2] - A[2][0] * A[1][1] * A[0][2];
  const S r = S(1) / det;
  B[0][0] = (A[1][1] * A[2][2] - A[2][1] * A[1][2]) * r;
  B[1][0] = (A[1][2] * A[2][0] - A[2][2] * A[1][0]) * r;
  B[2][0] = (A[1][0] * A[2][1] - A[2][0] * A[1][1]) * r;
  B[0][1] = (A[2][1] * A[0][2] - A[0][1] * A[2][2]) * r;
  B[1][1] = (A[2][2] * A[0][0] - A[0][2] * A[2][0]) * r;
  B[2][1] = (A[2][0] * A[0][1] - A[0][0] * A[2][1]) * r;
  B[0][2] = (A[0][1] * A[1][2] - A[1][1] * A[0][2]) * r;
  B[1][2] = (A[0][2] * A[1][0] - A[1][2] * A[0][0]) * r;
  B[2][2] = (A[0][0] * A[1][1] - A[1][0] * A[0][1]) * r;
  return det;
}

template <typename S>
__device__ __forceinline__ S det3(const S A[3][3]) {
  return A[0][0] * A[1][1] * A[2][2] + A[0][1] * A[1][2] * A[2][0] + A[0][2] * A[1][0] * A[2][1] -
         A[0][0] * A[2][1] * A[1][2] - A[1][0] * A[0][1] * A[2][2] - A[2][0] * A[1][1] * A[0][2];
}

// Volume Jacobian sqrt|det(M^T M)| (src/coordinate_routines.F90:818-822).
__device__ __forceinline__ double vol_jacobian(const double M[3][3]) {
  double G[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) G[i][j] = M[0][i] * M[0][j] + M[1][i] * M[1][j] + M[2][i] * M[2][j];
  return sqrt(fabs(det3(G)));
}
// The FP32 path keeps the volume Jacobian in FP64: the gradient matrix is widened exactly (integer
// re-packing, no FP64-pipe conversion) and |det M| (= sqrt(det(M^T M)) for a square M) is taken
// directly, which also avoids the Gram product and the square root.
__device__ __forceinline__ float vol_jacobian(const float M[3][3]) {
  double D[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) D[i][j] = f32_to_f64_exact(M[i][j]);
  return (float)fabs(det3(D));
}

// Per-Gauss-point kinematics shared by residual and Jacobian.
template <typename S>
struct GPT {
  S Zi[3][3];  // dxi/dz
  S F[3][3];   // dz/dnu
  S Jz, Jx, p, w;
};
using GP = GPT<double>;

template <typename S>
__device__ __forceinline__ bool gauss_point(const TablesT<S>& T, int g, const S* sz, const S* sx, const S* sp,
                                            GPT<S>& o) {
  S Z[3][3], X[3][3];
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      S a = S(0), b = S(0);
#pragma unroll 9
      for (int ns = 0; ns < NQ; ++ns) {
        const S d = T.dphi[g][k][ns];
        a += d * sz[c * NQ + ns];
        b += d * sx[c * NQ + ns];
      }
      Z[c][k] = a;
      X[c][k] = b;
    }
  o.Jz = vol_jacobian(Z);
  o.Jx = vol_jacobian(X);
  const S dz = inv3(Z, o.Zi);
  // material frame without fibres: dX/dNu columns = normalised DX_DXI columns
  S N[3][3], NX[3][3], A[3][3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const S n = sqrt(X[0][k] * X[0][k] + X[1][k] * X[1][k] + X[2][k] * X[2][k]);
#pragma unroll
    for (int c = 0; c < 3; ++c) N[c][k] = X[c][k] / n;
  }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) NX[i][j] = N[0][i] * X[0][j] + N[1][i] * X[1][j] + N[2][i] * X[2][j];
  inv3(NX, A);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) o.F[i][j] = Z[i][0] * A[0][j] + Z[i][1] * A[1][j] + Z[i][2] * A[2][j];
  S p = S(0);
#pragma unroll
  for (int m = 0; m < NL; ++m) p += T.psi[g][m] * sp[m];
  o.p = p;
  o.w = T.w[g];
  return dz > S(0) && o.Jx > S(0) && isfinite(dz);
}

// push-forward matrix t (src/finite_elasticity_routines.F90:1343-1375)
template <typename S>
__device__ __forceinline__ void push_t(const S F[3][3], S t[6][6]) {
#pragma unroll
  for (int j = 0; j < 6; ++j)
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      const int ai = v2t_a(i), bi = v2t_b(i), aj = v2t_a(j), bj = v2t_b(j);
      S v = F[ai][aj] * F[bi][bj];
      if (j >= 3) v += F[ai][bj] * F[bi][aj];
      t[i][j] = v;
    }
}

template <typename R>
__device__ __forceinline__ void push_vec(const R t[6][6], R S[6], R J) {
  R o[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    R s = R(0);
#pragma unroll
    for (int j = 0; j < 6; ++j) s += t[i][j] * S[j];
    o[i] = s / J;
  }
#pragma unroll
  for (int i = 0; i < 6; ++i) S[i] = o[i];
}

// Cauchy stress of the residual (deviatoric MR + p), src/finite_elasticity_routines.F90:6985-7061.
__device__ __forceinline__ void residual_stress(const GP& q, double c1, double c2, double sig[6]) {
  const double J = q.Jz / q.Jx;
  const double s = pow(J, -1.0 / 3.0);
  double Fb[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) Fb[i][j] = q.F[i][j] * s;
  double C[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) C[i][j] = Fb[0][i] * Fb[0][j] + Fb[1][i] * Fb[1][j] + Fb[2][i] * Fb[2][j];
  const double I1 = C[0][0] + C[1][1] + C[2][2];
  const double t1 = -2.0 * c2, t2 = 2.0 * (c1 + I1 * c2);
  sig[0] = t1 * C[0][0] + t2; sig[1] = t1 * C[1][1] + t2; sig[2] = t1 * C[2][2] + t2;
  sig[3] = t1 * C[1][0]; sig[4] = t1 * C[2][0]; sig[5] = t1 * C[2][1];
  double t[6][6];
  push_t(Fb, t);
  push_vec(t, sig, J);
  const double tr3 = (sig[0] + sig[1] + sig[2]) / 3.0;
  sig[0] = sig[0] - tr3 + q.p; sig[1] = sig[1] - tr3 + q.p; sig[2] = sig[2] - tr3 + q.p;
}

// ----------------------------------------------------------------------------------------------
// residual
// ----------------------------------------------------------------------------------------------
constexpr int kResWarps = 4;

// One warp: the 89 residual entries of one element from its staged geometry sx[81], deformed
// positions sz[81] and pressures sp[8] (shared memory), with Gauss-point scratch sP[27*9] and
// stp[27].  Lane g < 27 evaluates Gauss point g (metrics, deformation gradient, stress) and leaves
// P_g = J_z w_g Z^-1 sigma (3x3) and J_x w_g (J_z/J_x - 1); then lane i forms entries i, i + 32,
// i + 64 as sums over the Gauss points in a fixed order and hands each to emit(i, value).
template <typename Emit>
__device__ __forceinline__ void warp_element_residual(const Tables& T, int lane, const double* sx, const double* sz,
                                                      const double* sp, double c1, double c2, double* sP, double* stp,
                                                      unsigned* err, Emit emit) {
  if (lane < NG) {
    GP q;
    if (!gauss_point(T, lane, sz, sx, sp, q)) gfe_raise(err, GFE_DEVERR_JACOBIAN);
    double sig[6];
    residual_stress(q, c1, c2, sig);
    const double jgw = q.Jz * q.w;
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int mh = 0; mh < 3; ++mh)
        sP[lane * 9 + k * 3 + mh] = jgw * (q.Zi[k][0] * sig[t2v(0, mh)] + q.Zi[k][1] * sig[t2v(1, mh)] +
                                           q.Zi[k][2] * sig[t2v(2, mh)]);
    stp[lane] = q.Jx * q.w * (q.Jz / q.Jx - 1.0);
  }
  __syncwarp();
  for (int i = lane; i < ND; i += 32) {
    double s = 0.0;
    if (i < 81) {
      const int ms = i % NQ, mh = i / NQ;
      for (int g = 0; g < NG; ++g)
        s += T.dphi[g][0][ms] * sP[g * 9 + 0 + mh] + T.dphi[g][1][ms] * sP[g * 9 + 3 + mh] +
             T.dphi[g][2][ms] * sP[g * 9 + 6 + mh];
    } else {
      const int ms = i - 81;
      for (int g = 0; g < NG; ++g) s += stp[g] * T.psi[g][ms];
    }
    emit(i, s);
  }
  __syncwarp();
}

__global__ void __launch_bounds__(kResWarps * 32)
mr_residual_kernel(const int32_t* __restrict__ elems, int32_t count, int32_t batch, const int32_t* __restrict__ eq2,
                   const int32_t* __restrict__ elin, int32_t nq2, int32_t nlin, const double* __restrict__ xg,
                   const double* __restrict__ dep, const double* __restrict__ cpar, const Tables* __restrict__ Tg,
                   double* __restrict__ R, int64_t dep_stride, unsigned* err) {
  extern __shared__ double smem[];
  Tables& T = *reinterpret_cast<Tables*>(smem);
  double* wbase = smem + sizeof(Tables) / sizeof(double);
  // stage the tables
  {
    const double* src = reinterpret_cast<const double*>(Tg);
    double* dst = smem;
    for (int i = threadIdx.x; i < (int)(sizeof(Tables) / sizeof(double)); i += blockDim.x) dst[i] = src[i];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  // per-warp scratch: x[81], z[81], p[8], P[27][9], tp[27], dofs (int) [89]
  double* sx = wbase + w * (81 + 81 + 8 + NG * 9 + NG + 48);
  double* sz = sx + 81;
  double* sp = sz + 81;
  double* sP = sp + 8;
  double* stp = sP + NG * 9;
  int* sd = reinterpret_cast<int*>(stp + NG);
  const long long total = (long long)count * batch;
  for (long long item = (long long)blockIdx.x * kResWarps + w; item < total; item += (long long)gridDim.x * kResWarps) {
    const int b = (int)(item / count);
    const int e = __ldg(elems + (item % count));
    const double* d = dep + b * dep_stride;
    for (int i = lane; i < NQ; i += 32) {
      const int n = __ldg(eq2 + (size_t)e * NQ + i);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        sx[c * NQ + i] = __ldg(xg + (size_t)c * nq2 + n);
        sz[c * NQ + i] = d[(size_t)c * nq2 + n];
        sd[c * NQ + i] = c * nq2 + n;
      }
    }
    if (lane < NL) {
      const int n = __ldg(elin + (size_t)e * NL + lane);
      sp[lane] = d[(size_t)3 * nq2 + n];
      sd[81 + lane] = 3 * nq2 + n;
    }
    const double c1 = cpar[2 * b], c2 = cpar[2 * b + 1];
    __syncwarp();
    double* Rb = R + b * dep_stride;
    warp_element_residual(T, lane, sx, sz, sp, c1, c2, sP, stp, err, [&](int i, double s) {
      if (!isfinite(s)) gfe_raise(err, GFE_DEVERR_NONFINITE);
      Rb[sd[i]] += s;
    });
  }
}

// ----------------------------------------------------------------------------------------------
// Finite-difference Jacobian (Iron's default for finite elasticity)
// ----------------------------------------------------------------------------------------------
// EquationsSet_FiniteElementJacobianEvaluateFD (src/equations_set_routines.F90:2839-2962): the
// element residual R0 at the current parameters, then for every element parameter j (27 nodes of
// each displacement component, then the 8 pressure nodes) the residual with that parameter raised
// by delta = (1 + ||dep||_2) * step, and column j = (R_j - R0) / delta.  ||dep||_2 is the L2 norm
// of the whole dependent parameter vector (DistributedVector_L2Norm).  One CTA per element of a
// colour: warp 0 forms R0, then the warps take the 89 perturbed residuals in turn, each on its
// own copy of the element parameters, and add their column into the CSR values through the slot
// map (elements of one colour share no DOF).
constexpr int kFDWarps = 4;
constexpr int kNormParts = 512;

struct FDShared {
  double x[81], z0[81], p0[8], R0[ND];
  double z[kFDWarps][81], p[kFDWarps][8], P[kFDWarps][NG * 9], tp[kFDWarps][NG], col[kFDWarps][ND];
  double delta;
};

// partial sums of squares of the dependent vector in a fixed order (kNormParts contiguous chunks)
__global__ void sumsq_parts(const double* __restrict__ v, int64_t n, double* __restrict__ parts) {
  __shared__ double red[256];
  const int64_t chunk = (n + kNormParts - 1) / kNormParts;
  const int64_t a = blockIdx.x * chunk, b = a + chunk < n ? a + chunk : n;
  double s = 0.0;
  for (int64_t i = a + threadIdx.x; i < b; i += blockDim.x) s += v[i] * v[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) parts[blockIdx.x] = red[0];
}

__global__ void __launch_bounds__(kFDWarps * 32)
mr_jacobian_fd_kernel(const int32_t* __restrict__ elems, int32_t count, const int32_t* __restrict__ eq2,
                      const int32_t* __restrict__ elin, int32_t nq2, const double* __restrict__ xg,
                      const double* __restrict__ dep, const double* __restrict__ cpar, const Tables* __restrict__ Tg,
                      const double* __restrict__ norm_parts, double step, const int32_t* __restrict__ slots,
                      double* __restrict__ values, double* __restrict__ Kout, unsigned* err) {
  extern __shared__ double smem[];
  Tables& T = *reinterpret_cast<Tables*>(smem);
  FDShared& S = *reinterpret_cast<FDShared*>(smem + sizeof(Tables) / sizeof(double));
  {
    const double* src = reinterpret_cast<const double*>(Tg);
    for (int i = threadIdx.x; i < (int)(sizeof(Tables) / sizeof(double)); i += blockDim.x) smem[i] = src[i];
  }
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < kNormParts; ++i) s += norm_parts[i];
    S.delta = (1.0 + sqrt(s)) * step;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const double c1 = cpar[0], c2 = cpar[1];
  const double delta = S.delta;
  for (int item = blockIdx.x; item < count; item += gridDim.x) {
    const int e = __ldg(elems + item);
    for (int i = threadIdx.x; i < NQ; i += blockDim.x) {
      const int n = __ldg(eq2 + (size_t)e * NQ + i);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        S.x[c * NQ + i] = __ldg(xg + (size_t)c * nq2 + n);
        S.z0[c * NQ + i] = dep[(size_t)c * nq2 + n];
      }
    }
    if (threadIdx.x < NL) S.p0[threadIdx.x] = dep[(size_t)3 * nq2 + __ldg(elin + (size_t)e * NL + threadIdx.x)];
    __syncthreads();
    if (w == 0)
      warp_element_residual(T, lane, S.x, S.z0, S.p0, c1, c2, S.P[0], S.tp[0], err,
                            [&](int i, double s) { S.R0[i] = s; });
    __syncthreads();
    const int32_t* sl = slots ? slots + (size_t)e * ND * ND : nullptr;
    double* Ke = Kout ? Kout + (size_t)e * ND * ND : nullptr;
    for (int j = w; j < ND; j += kFDWarps) {
      for (int i = lane; i < 81; i += 32) S.z[w][i] = S.z0[i];
      if (lane < NL) S.p[w][lane] = S.p0[lane];
      __syncwarp();
      if (lane == 0) {
        if (j < 81) S.z[w][j] = S.z0[j] + delta;
        else S.p[w][j - 81] = S.p0[j - 81] + delta;
      }
      __syncwarp();
      warp_element_residual(T, lane, S.x, S.z[w], S.p[w], c1, c2, S.P[w], S.tp[w], err,
                            [&](int i, double s) { S.col[w][i] = (s - S.R0[i]) / delta; });
      // column j: rows r = lane, lane + 32, lane + 64
      for (int r = lane; r < ND; r += 32) {
        const double v = S.col[w][r];
        if (!isfinite(v)) gfe_raise(err, GFE_DEVERR_NONFINITE);
        if (Ke) Ke[(size_t)r * ND + j] = v;
        if (sl && !(r >= 81 && j >= 81)) {
          const int pos = __ldg(sl + (size_t)r * ND + j);
          if (pos >= 0) values[pos] += v;
          else gfe_raise(err, GFE_DEVERR_SLOT);
        }
      }
      __syncwarp();
    }
    __syncthreads();
  }
}

// slot map: for each element and each (r, c), the 0-based CSR position of (dof_r, dof_c); -1 when
// absent, at slots[(e * 89 + r) * 89 + c] (element number e).  One warp per (element, row).
__global__ void mr_slot_kernel(const int32_t* __restrict__ elems, int32_t count, const int32_t* __restrict__ eq2,
                               const int32_t* __restrict__ elin, int32_t nq2, const int32_t* __restrict__ rp,
                               const int32_t* __restrict__ ci, int32_t* __restrict__ slots) {
  const int lane = threadIdx.x & 31;
  const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; wid < (long long)count * ND;
       wid += nw) {
    const int item = (int)(wid / ND), r = (int)(wid % ND);
    const int e = elems[item];
    auto dof = [&](int i) {
      return i < 81 ? (i / NQ) * nq2 + eq2[(size_t)e * NQ + i % NQ] : 3 * nq2 + elin[(size_t)e * NL + i - 81];
    };
    const int row = dof(r);
    const int lo0 = rp[row] - 1, hi0 = rp[row + 1] - 1;
    for (int c = lane; c < ND; c += 32) {
      const int col = dof(c) + 1;
      int lo = lo0, hi = hi0;
      while (lo < hi) {
        const int mid = lo + ((hi - lo) >> 1);  // no int32 overflow past 2^30 entries
        if (ci[mid] < col) lo = mid + 1; else hi = mid;
      }
      slots[((size_t)e * ND + r) * ND + c] = (lo < hi0 && ci[lo] == col) ? lo : -1;
    }
  }
}

// ----------------------------------------------------------------------------------------------
// Row-owning assembly of element matrices (replaces EquationsMatrices_JacobianElementAdd,
// src/equations_matrices_routines.F90:2866-2909, for a whole mesh at once)
// ----------------------------------------------------------------------------------------------
// The element matrices of all elements are first written to Kel[e][89][89]; then each CSR row is
// summed once from the element rows of the elements around its node, in ascending element order,
// in shared memory, and written out exactly once with coalesced stores.  Each element row and its
// slot-map row are read once, contiguously.  Node incidence: for node k (quadratic nodes 0..nq2-1,
// then linear nodes nq2 + l) up to kMaxInc entries (e * 64 + local index; local 0..26 quadratic,
// 27..34 linear), sorted by element.
constexpr int kMaxInc = 16;       // elements around one node (8 on a hexahedral grid)
constexpr int kRowWarps = 8;      // warps (rows in flight) per CTA of mr_row_gather_kernel
constexpr int kMaxRowLen = 512;   // entries of one Jacobian row (at most 402 on a regular Q2/Q1 grid)
constexpr int kGatherGroup = 4;   // element rows whose loads are in flight together

__global__ void mr_incidence_fill(const int32_t* __restrict__ elems, int32_t count, const int32_t* __restrict__ eq2,
                                  const int32_t* __restrict__ elin, int32_t nq2, int32_t* __restrict__ cnt,
                                  int32_t* __restrict__ list, unsigned* err) {
  const long long n = (long long)count * (NQ + NL);
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int item = (int)(t / (NQ + NL)), loc = (int)(t % (NQ + NL));
    const int e = __ldg(elems + item);
    const int node = loc < NQ ? __ldg(eq2 + (size_t)e * NQ + loc) : nq2 + __ldg(elin + (size_t)e * NL + loc - NQ);
    const int k = atomicAdd(cnt + node, 1);
    if (k < kMaxInc) list[(size_t)node * kMaxInc + k] = e * 64 + loc;
    else gfe_raise(err, GFE_DEVERR_SLOT);
  }
}

// sort each node's incidence list by element (insertion sort of at most kMaxInc entries)
__global__ void mr_incidence_sort(int32_t n_nodes, const int32_t* __restrict__ cnt, int32_t* __restrict__ list) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n_nodes; k += gridDim.x * blockDim.x) {
    int32_t* L = list + (size_t)k * kMaxInc;
    const int m = min(cnt[k], kMaxInc);
    for (int i = 1; i < m; ++i) {
      const int32_t v = L[i];
      int j = i - 1;
      while (j >= 0 && L[j] > v) {
        L[j + 1] = L[j];
        --j;
      }
      L[j + 1] = v;
    }
  }
}

// One warp per CSR row: values[row] = sum over the elements around the row's node of their element
// rows, through the slot map (element number order).  Rows of displacement component mh take local
// row mh * 27 + node index; pressure rows local row 81 + corner index.  The pressure-pressure block
// is not assembled (zero in Iron's matrix).  Every entry of every row is written, so the values
// need no zeroing first.  FP32 element matrices are summed in FP32 (at most 8 terms an entry,
// against the 5e-6 of their own contraction) and widened exactly with integer operations
// (f32_to_f64_exact): the FP64 additions and conversions kept the FP64 pipe 77 % busy and bounded
// the kernel.
template <typename TS>
__global__ void __launch_bounds__(kRowWarps * 32)
mr_row_gather_kernel(int32_t nq2, int32_t nlin, const int32_t* __restrict__ cnt, const int32_t* __restrict__ list,
                     const TS* __restrict__ Kel, const int32_t* __restrict__ slots, const int32_t* __restrict__ rp,
                     double* __restrict__ values, float* __restrict__ values32, unsigned* err) {
  __shared__ TS buf[kRowWarps][kMaxRowLen];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  TS* B = buf[w];
  const long long n_rows = 3ll * nq2 + nlin;
  for (long long row = (long long)blockIdx.x * kRowWarps + w; row < n_rows; row += (long long)gridDim.x * kRowWarps) {
    int node, mh;
    if (row < 3ll * nq2) {
      mh = (int)(row / nq2);
      node = (int)(row - (long long)mh * nq2);
    } else {
      mh = 0;
      node = nq2 + (int)(row - 3ll * nq2);
    }
    const long long r0 = __ldg(rp + row) - 1;
    const int len = (int)(__ldg(rp + row + 1) - 1 - r0);
    if (len > kMaxRowLen) {
      if (lane == 0) gfe_raise(err, GFE_DEVERR_SLOT);
      continue;
    }
    for (int j = lane; j < len; j += 32) B[j] = TS(0);
    __syncwarp();
    const int m = min(__ldg(cnt + node), kMaxInc);
    const int32_t* L = list + (size_t)node * kMaxInc;
    // groups of kGatherGroup element rows: every slot and value load of a group is issued before
    // the group's additions, which then run in ascending element order
    for (int i0 = 0; i0 < m; i0 += kGatherGroup) {
      int pos[kGatherGroup][3];
      TS val[kGatherGroup][3];
#pragma unroll
      for (int u = 0; u < kGatherGroup; ++u) {
        const int i = i0 + u;
        const int32_t packed = i < m ? __ldg(L + i) : -1;
        const int e = packed >> 6, loc = packed & 63;
        const int lr = loc < NQ ? mh * NQ + loc : 81 + loc - NQ;
        const size_t base = ((size_t)(packed < 0 ? 0 : e) * ND + lr) * ND;
        const int cmax = packed < 0 ? 0 : (lr >= 81 ? 81 : ND);
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const int c = lane + 32 * j;
          pos[u][j] = -2;  // nothing to add
          val[u][j] = TS(0);
          if (c < cmax) {
            pos[u][j] = __ldg(slots + base + c);
            val[u][j] = __ldg(Kel + base + c);
          }
        }
      }
#pragma unroll
      for (int u = 0; u < kGatherGroup; ++u) {
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const long long o = (long long)pos[u][j] - r0;
          if (pos[u][j] >= 0 && o >= 0 && o < len) B[o] += val[u][j];
          else if (pos[u][j] != -2) gfe_raise(err, GFE_DEVERR_SLOT);
        }
        __syncwarp();  // the next element may add to the same entries
      }
    }
    for (int j = lane; j < len; j += 32) {
      const TS v = B[j];
      if constexpr (std::is_same<TS, float>::value) values[r0 + j] = f32_to_f64_exact(v);
      else values[r0 + j] = v;
      if (values32) values32[r0 + j] = (float)v;
    }
    __syncwarp();
  }
}

template <typename TS>
__global__ void widen_element_matrices(const TS* __restrict__ src, size_t n, double* __restrict__ dst) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = (double)src[i];
}

// ----------------------------------------------------------------------------------------------
// Consistent tangent and adjoint of Iron's residual (forward-mode dual numbers per Gauss point)
// ----------------------------------------------------------------------------------------------
// Per Gauss point the u-rows of the residual are R(ms,mh) += sum_xi g_ms[xi] P[xi][mh] with
// P = w J_z Z^-1 sigma(Z, p) (Z = dz/dxi, g = reference basis gradients) and the p-rows
// R(ms) += w (J_z - J_x) psi_ms.  The exact derivatives dP/dZ (81 numbers) and dP/dp (9) are
// obtained by 10 forward-mode passes through the same formulas with dual numbers; dJ_z/dZ =
// J_z Z^-T.  The element tangent / vector-Jacobian products are then contractions with the
// constant basis tables.  This is the derivative that Iron's finite-difference Jacobian
// (src/equations_set_routines.F90:2839-2962) approximates.
struct Dual {
  double v, d;
};
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ Dual operator-(Dual a) { return {-a.v, -a.d}; }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return {a.v * b.v, a.v * b.d + a.d * b.v}; }
__device__ __forceinline__ Dual operator*(double a, Dual b) { return {a * b.v, a * b.d}; }
__device__ __forceinline__ Dual operator*(Dual a, double b) { return {a.v * b, a.d * b}; }
__device__ __forceinline__ Dual operator/(Dual a, Dual b) {
  const double r = 1.0 / b.v;
  return {a.v * r, (a.d - a.v * r * b.d) * r};
}
__device__ __forceinline__ Dual operator/(Dual a, double b) { return {a.v / b, a.d / b}; }
__device__ __forceinline__ Dual operator+(Dual a, double b) { return {a.v + b, a.d}; }
__device__ __forceinline__ Dual dsqrt(Dual a) {
  const double s = sqrt(a.v);
  return {s, a.d / (2.0 * s)};
}
__device__ __forceinline__ Dual dabs(Dual a) { return a.v < 0.0 ? -a : a; }
// x^(-1/3)
__device__ __forceinline__ Dual dpowm13(Dual a) {
  const double v = pow(a.v, -1.0 / 3.0);
  return {v, -v / (3.0 * a.v) * a.d};
}

template <typename T>
__device__ __forceinline__ T tdet3(const T A[3][3]) {
  return A[0][0] * A[1][1] * A[2][2] + A[0][1] * A[1][2] * A[2][0] + A[0][2] * A[1][0] * A[2][1] -
         A[0][0] * A[2][1] * A[1][2] - A[1][0] * A[0][1] * A[2][2] - A[2][0] * A[1][1] * A[0][2];
}

template <typename T>
__device__ __forceinline__ void tinv3(const T A[3][3], T B[3][3]) {
  const T det = tdet3(A);
  B[0][0] = (A[1][1] * A[2][2] - A[2][1] * A[1][2]) / det;
  B[1][0] = (A[1][2] * A[2][0] - A[2][2] * A[1][0]) / det;
  B[2][0] = (A[1][0] * A[2][1] - A[2][0] * A[1][1]) / det;
  B[0][1] = (A[2][1] * A[0][2] - A[0][1] * A[2][2]) / det;
  B[1][1] = (A[2][2] * A[0][0] - A[0][2] * A[2][0]) / det;
  B[2][1] = (A[2][0] * A[0][1] - A[0][0] * A[2][1]) / det;
  B[0][2] = (A[0][1] * A[1][2] - A[1][1] * A[0][2]) / det;
  B[1][2] = (A[0][2] * A[1][0] - A[1][2] * A[0][0]) / det;
  B[2][2] = (A[0][0] * A[1][1] - A[1][0] * A[0][1]) / det;
}

// The same forward-mode arithmetic in FP32 for the FP32 paths of the consistent tangent.
struct DualF {
  float v, d;
};
__device__ __forceinline__ DualF operator+(DualF a, DualF b) { return {a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ DualF operator-(DualF a, DualF b) { return {a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ DualF operator*(DualF a, DualF b) { return {a.v * b.v, a.v * b.d + a.d * b.v}; }
__device__ __forceinline__ DualF operator*(float a, DualF b) { return {a * b.v, a * b.d}; }
__device__ __forceinline__ DualF operator*(DualF a, float b) { return {a.v * b, a.d * b}; }
__device__ __forceinline__ DualF operator/(DualF a, DualF b) {
  const float r = 1.0f / b.v;
  return {a.v * r, (a.d - a.v * r * b.d) * r};
}
__device__ __forceinline__ DualF operator/(DualF a, float b) { return {a.v / b, a.d / b}; }
__device__ __forceinline__ DualF operator+(DualF a, float b) { return {a.v + b, a.d}; }
__device__ __forceinline__ DualF dpowm13(DualF a) {
  const float v = 1.0f / cbrtf(a.v);
  return {v, -v / (3.0f * a.v) * a.d};
}

template <typename S>
struct DualOf {
  using type = Dual;
};
template <>
struct DualOf<float> {
  using type = DualF;
};

// J_z = sqrt|det(Z^T Z)| as Iron forms it (COORDINATE_METRICS_CALCULATE); the FP32 dual path takes
// |det Z| (the same value for a square Z) in FP64 dual arithmetic on the exactly widened entries.
template <typename T>
__device__ __forceinline__ T point_jz(const T (&)[3][3], const T (&G)[3][3]) {
  return dsqrt(dabs(tdet3(G)));
}
__device__ __forceinline__ DualF point_jz(const DualF (&Z)[3][3], const DualF (&)[3][3]) {
  Dual D[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) D[i][j] = {f32_to_f64_exact(Z[i][j].v), f32_to_f64_exact(Z[i][j].d)};
  const Dual j = dabs(tdet3(D));
  return {(float)j.v, (float)j.d};
}

// P = w Jz Z^-1 sigma(Z, p) of the residual; also returns Jz.  R: type of the constants.  jz_given:
// J_z (with its derivative) when the caller has formed it already.
template <typename T, typename R = double>
__device__ __forceinline__ void point_P(const T (&Z)[3][3], const R A[3][3], R Jx, R w, T p, R c1, R c2, T P[3][3],
                                        T& Jz, const T* jz_given = nullptr) {
  if (jz_given) {
    Jz = *jz_given;
  } else {
    T G[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) G[i][j] = Z[0][i] * Z[0][j] + Z[1][i] * Z[1][j] + Z[2][i] * Z[2][j];
    Jz = point_jz(Z, G);
  }
  T Zi[3][3];
  tinv3(Z, Zi);
  const T J = Jz / Jx;
  const T s = dpowm13(J);
  T Fb[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) Fb[i][j] = (Z[i][0] * A[0][j] + Z[i][1] * A[1][j] + Z[i][2] * A[2][j]) * s;
  T C[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) C[i][j] = Fb[0][i] * Fb[0][j] + Fb[1][i] * Fb[1][j] + Fb[2][i] * Fb[2][j];
  const T I1 = C[0][0] + C[1][1] + C[2][2];
  const R t1 = R(-2.0) * c2;
  const T t2 = R(2.0) * (I1 * c2 + c1);
  T Sv[6] = {t1 * C[0][0] + t2, t1 * C[1][1] + t2, t1 * C[2][2] + t2, t1 * C[1][0], t1 * C[2][0], t1 * C[2][1]};
  // sigma_bar = Fb S Fb^T / J (full tensor form of the Voigt push-forward)
  T Sm[3][3] = {{Sv[0], Sv[3], Sv[4]}, {Sv[3], Sv[1], Sv[5]}, {Sv[4], Sv[5], Sv[2]}};
  T FS[3][3], sg[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) FS[i][j] = Fb[i][0] * Sm[0][j] + Fb[i][1] * Sm[1][j] + Fb[i][2] * Sm[2][j];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) sg[i][j] = (FS[i][0] * Fb[j][0] + FS[i][1] * Fb[j][1] + FS[i][2] * Fb[j][2]) / J;
  const T tr3 = (sg[0][0] + sg[1][1] + sg[2][2]) / R(3.0);
#pragma unroll
  for (int i = 0; i < 3; ++i) sg[i][i] = sg[i][i] - tr3 + p;
  const T wj = Jz * w;
#pragma unroll
  for (int k = 0; k < 3; ++k)
#pragma unroll
    for (int mh = 0; mh < 3; ++mh) P[k][mh] = wj * (Zi[k][0] * sg[0][mh] + Zi[k][1] * sg[1][mh] + Zi[k][2] * sg[2][mh]);
}

// Gauss-point inputs of the tangent: Z (3x3), the material-frame matrix A, J_x, w, p
template <typename S>
struct GPInT {
  S Z[3][3], A[3][3], Jx, w, p;
};
using GPIn = GPInT<double>;

template <typename S>
__device__ __forceinline__ void gauss_inputs(const TablesT<S>& T, int g, const S* sz, const S* sx, const S* sp,
                                             GPInT<S>& o) {
  S X[3][3];
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      S a = S(0), b = S(0);
      for (int ns = 0; ns < NQ; ++ns) {
        const S d = T.dphi[g][k][ns];
        a += d * sz[c * NQ + ns];
        b += d * sx[c * NQ + ns];
      }
      o.Z[c][k] = a;
      X[c][k] = b;
    }
  o.Jx = vol_jacobian(X);
  S N[3][3], NX[3][3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const S n = sqrt(X[0][k] * X[0][k] + X[1][k] * X[1][k] + X[2][k] * X[2][k]);
#pragma unroll
    for (int c = 0; c < 3; ++c) N[c][k] = X[c][k] / n;
  }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) NX[i][j] = N[0][i] * X[0][j] + N[1][i] * X[1][j] + N[2][i] * X[2][j];
  inv3(NX, o.A);
  S p = S(0);
  for (int m = 0; m < NL; ++m) p += T.psi[g][m] * sp[m];
  o.p = p;
  o.w = T.w[g];
}

// J_z = |det Z| and its derivatives for the FP32 dual path, once per Gauss point: the value and the
// signed cofactors (d|det Z| / dZ_ij) in FP64 on the exactly widened entries, rounded to FP32.
// jz[0] = J_z, jz[1 + 3 i + j] = dJ_z/dZ_ij.  The seeds are unit directions, so each seed's
// derivative is one cofactor: forming |det Z| in FP64 dual arithmetic per seed cost about 460 FP64
// operations a Gauss point on GB300's narrow FP64 pipe, this about 30.
__device__ __forceinline__ void jz_seeds(const float (&Zf)[3][3], float jz[10]) {
  double Z[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) Z[i][j] = f32_to_f64_exact(Zf[i][j]);
  double cof[3][3];
  cof[0][0] = Z[1][1] * Z[2][2] - Z[1][2] * Z[2][1];
  cof[0][1] = Z[1][2] * Z[2][0] - Z[1][0] * Z[2][2];
  cof[0][2] = Z[1][0] * Z[2][1] - Z[1][1] * Z[2][0];
  cof[1][0] = Z[0][2] * Z[2][1] - Z[0][1] * Z[2][2];
  cof[1][1] = Z[0][0] * Z[2][2] - Z[0][2] * Z[2][0];
  cof[1][2] = Z[0][1] * Z[2][0] - Z[0][0] * Z[2][1];
  cof[2][0] = Z[0][1] * Z[1][2] - Z[0][2] * Z[1][1];
  cof[2][1] = Z[0][2] * Z[1][0] - Z[0][0] * Z[1][2];
  cof[2][2] = Z[0][0] * Z[1][1] - Z[0][1] * Z[1][0];
  const double det = tdet3(Z);
  const double sg = det < 0.0 ? -1.0 : 1.0;
  jz[0] = (float)(sg * det);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) jz[1 + 3 * i + j] = (float)(sg * cof[i][j]);
}

// dP/d(seed) for seed 0..8 = Z[seed/3][seed%3], seed 9 = p.  out[9] = dP[xi][mh] row-major.
// jz: J_z and its seed derivatives from jz_seeds (FP32 path), or NULL.
template <typename S>
__device__ __forceinline__ void point_dP(const GPInT<S>& in, int seed, S c1, S c2, S out[9], S* Jz_v,
                                         const float* jz = nullptr) {
  using D = typename DualOf<S>::type;
  D Z[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) Z[i][j] = {in.Z[i][j], (i * 3 + j == seed) ? S(1) : S(0)};
  const D p = {in.p, seed == 9 ? S(1) : S(0)};
  D P[3][3], Jz;
  if constexpr (std::is_same<S, float>::value) {
    if (jz) {
      const D jg = {jz[0], seed < 9 ? jz[1 + seed] : 0.0f};
      point_P<D, S>(Z, in.A, in.Jx, in.w, p, c1, c2, P, Jz, &jg);
    } else {
      point_P<D, S>(Z, in.A, in.Jx, in.w, p, c1, c2, P, Jz);
    }
  } else {
    point_P<D, S>(Z, in.A, in.Jx, in.w, p, c1, c2, P, Jz);
  }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) out[i * 3 + j] = P[i][j].d;
  if (Jz_v) *Jz_v = Jz.v;
}

// ----------------------------------------------------------------------------------------------
// Reverse-mode adjoint of the residual (one reverse sweep per Gauss point)
// ----------------------------------------------------------------------------------------------
// For a cotangent v of the element residual, the u-rows give the cotangent of P_g,
// V_g[xi][mh] = sum_ms v(mh, ms) g_ms[xi], and the p-rows that of w (J_z - J_x), Vp_g = sum_ms
// v_p(ms) psi_ms.  One reverse sweep through the formulas of point_P, in the opposite order,
// yields Zbar = dL/dZ (3x3), pbar = dL/dp and the material cotangents (c1bar, c2bar) at the cost
// of a few forward evaluations, instead of the 10 forward-mode passes of the tangent.  The
// element's du is then sum_g Zbar_g[c][k] g_ms[k] (u) and sum_g pbar_g psi_ms (p).
//   Q = Z^-1 sgd,  P = w J_z Q                      Qbar = w J_z V,  Jzbar += w V:Q
//   sgd = sg - tr(sg)/3 I + p I                    sgbar = dev(sgdbar), pbar = tr(sgdbar)
//   sg = Fb S Fb^T / J                             Hbar = sgbar / J, FSbar = Hbar Fb, Fbbar = Hbar^T FS
//   S = t1 C + t2 I, C = Fb^T Fb, t1 = -2 c2, t2 = 2 (I1 c2 + c1), I1 = tr C
//   Fb = s Z A, s = J^(-1/3), J = J_z / J_x, J_z = |det Z| (dJ_z/dZ = J_z Z^-T)
__device__ __forceinline__ void mm3(const double A[3][3], const double B[3][3], double C[3][3]) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) C[i][j] = A[i][0] * B[0][j] + A[i][1] * B[1][j] + A[i][2] * B[2][j];
}
// C = A^T B
__device__ __forceinline__ void mtm3(const double A[3][3], const double B[3][3], double C[3][3]) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) C[i][j] = A[0][i] * B[0][j] + A[1][i] * B[1][j] + A[2][i] * B[2][j];
}
// C = A B^T
__device__ __forceinline__ void mmt3(const double A[3][3], const double B[3][3], double C[3][3]) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) C[i][j] = A[i][0] * B[j][0] + A[i][1] * B[j][1] + A[i][2] * B[j][2];
}
__device__ __forceinline__ double dot9(const double A[3][3], const double B[3][3]) {
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) s += A[i][j] * B[i][j];
  return s;
}

__device__ __forceinline__ void point_P_vjp(const GPIn& in, double c1, double c2, const double V[3][3], double Vp,
                                            double Zb[3][3], double& pb, double& c1b, double& c2b) {
  // forward
  double G[3][3];
  mtm3(in.Z, in.Z, G);
  const double Jz = sqrt(fabs(det3(G)));
  double Zi[3][3];
  inv3(in.Z, Zi);
  const double J = Jz / in.Jx;
  const double s = pow(J, -1.0 / 3.0);
  double M[3][3], Fb[3][3];
  mm3(in.Z, in.A, M);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) Fb[i][j] = M[i][j] * s;
  double C[3][3];
  mtm3(Fb, Fb, C);
  const double I1 = C[0][0] + C[1][1] + C[2][2];
  const double t1 = -2.0 * c2, t2 = 2.0 * (I1 * c2 + c1);
  double S[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) S[i][j] = t1 * C[i][j] + (i == j ? t2 : 0.0);
  double FS[3][3], sg[3][3];
  mm3(Fb, S, FS);
  mmt3(FS, Fb, sg);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) sg[i][j] /= J;
  const double tr3 = (sg[0][0] + sg[1][1] + sg[2][2]) / 3.0;
  double sgd[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) sgd[i][j] = sg[i][j] - (i == j ? tr3 - in.p : 0.0);
  double Q[3][3];
  mm3(Zi, sgd, Q);
  const double wj = Jz * in.w;
  // reverse
  double Jzb = in.w * (dot9(V, Q) + Vp);  // P = wj Q and the p-row term w (J_z - J_x)
  double Qb[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) Qb[i][j] = wj * V[i][j];
  double Zib[3][3], sgdb[3][3];
  mmt3(Qb, sgd, Zib);  // Q = Zi sgd: Zibar = Qbar sgd^T, sgdbar = Zi^T Qbar
  mtm3(Zi, Qb, sgdb);
  const double trb = sgdb[0][0] + sgdb[1][1] + sgdb[2][2];
  pb = trb;
  double sgb[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) sgb[i][j] = sgdb[i][j] - (i == j ? trb / 3.0 : 0.0);
  // sg = H / J with H = FS Fb^T
  double Jb = -dot9(sgb, sg) / J;
  double Hb[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) Hb[i][j] = sgb[i][j] / J;
  double FSb[3][3], Fbb[3][3], T1[3][3];
  mm3(Hb, Fb, FSb);   // H = FS Fb^T: FSbar = Hbar Fb
  mtm3(Hb, FS, Fbb);  // Fbbar += Hbar^T FS
  // FS = Fb S: Fbbar += FSbar S^T (S symmetric), Sbar = Fb^T FSbar
  mm3(FSb, S, T1);
  double Sb[3][3];
  mtm3(Fb, FSb, Sb);
  const double t2b = Sb[0][0] + Sb[1][1] + Sb[2][2];
  const double t1b = dot9(Sb, C);
  const double I1b = 2.0 * c2 * t2b;
  c1b = 2.0 * t2b;
  c2b = 2.0 * I1 * t2b - 2.0 * t1b;
  double Cb[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) Cb[i][j] = t1 * Sb[i][j] + (i == j ? I1b : 0.0);
  // C = Fb^T Fb: Fbbar += Fb (Cbar + Cbar^T)
  double Cs[3][3], T2[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) Cs[i][j] = Cb[i][j] + Cb[j][i];
  mm3(Fb, Cs, T2);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) Fbb[i][j] += T1[i][j] + T2[i][j];
  // Fb = s M: sbar = Fbbar : M, Mbar = s Fbbar; M = Z A: Zbar += Mbar A^T
  const double sb = dot9(Fbb, M);
  double Mb[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) Mb[i][j] = s * Fbb[i][j];
  mmt3(Mb, in.A, Zb);
  // s = J^(-1/3), J = J_z / J_x
  Jb += sb * (-s / (3.0 * J));
  Jzb += Jb / in.Jx;
  // Zi = Z^-1: Zbar -= Zi^T Zibar Zi^T;  J_z = |det Z|: Zbar += Jzbar J_z Zi^T
  double T3[3][3], T4[3][3];
  mtm3(Zi, Zib, T3);   // Zi^T Zibar
  mmt3(T3, Zi, T4);    // (Zi^T Zibar) Zi^T
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) Zb[i][j] += -T4[i][j] + Jzb * Jz * Zi[j][i];
}

constexpr int kAdjWarps = 4;

struct AdjWarpShared {
  double x[81], z[81], p[8], v[ND];
  double Zb[NG][9], pb[NG], cb[NG][2];
  int dofs[ND];
};

// Reverse-mode vector-Jacobian products: one warp per (element, parameter set) of a colour.
__global__ void __launch_bounds__(kAdjWarps * 32)
mr_vjp_reverse_kernel(const int32_t* __restrict__ elems, int32_t count, int32_t batch,
                      const int32_t* __restrict__ eq2, const int32_t* __restrict__ elin, int32_t nq2, int32_t nlin,
                      const double* __restrict__ xg, const double* __restrict__ dep, const double* __restrict__ cpar,
                      const double* __restrict__ v, const Tables* __restrict__ Tg, double* __restrict__ du,
                      double* __restrict__ dc_elem, int32_t n_elem, unsigned* err) {
  extern __shared__ double smem[];
  Tables& T = *reinterpret_cast<Tables*>(smem);
  AdjWarpShared* W = reinterpret_cast<AdjWarpShared*>(smem + sizeof(Tables) / sizeof(double));
  for (int i = threadIdx.x; i < (int)(sizeof(Tables) / sizeof(double)); i += blockDim.x)
    smem[i] = reinterpret_cast<const double*>(Tg)[i];
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  AdjWarpShared& S = W[w];
  const int64_t ndof = 3ll * nq2 + nlin;
  const long long total = (long long)count * batch;
  for (long long item = (long long)blockIdx.x * kAdjWarps + w; item < total; item += (long long)gridDim.x * kAdjWarps) {
    const int b = (int)(item / count);
    const int e = __ldg(elems + (item % count));
    const double* d = dep + b * ndof;
    const double* vb = v + b * ndof;
    for (int i = lane; i < NQ; i += 32) {
      const int n = __ldg(eq2 + (size_t)e * NQ + i);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        S.x[c * NQ + i] = __ldg(xg + (size_t)c * nq2 + n);
        S.z[c * NQ + i] = d[(size_t)c * nq2 + n];
        S.dofs[c * NQ + i] = c * nq2 + n;
        S.v[c * NQ + i] = vb[(size_t)c * nq2 + n];
      }
    }
    if (lane < NL) {
      const int n = __ldg(elin + (size_t)e * NL + lane);
      S.p[lane] = d[(size_t)3 * nq2 + n];
      S.dofs[81 + lane] = 3 * nq2 + n;
      S.v[81 + lane] = vb[(size_t)3 * nq2 + n];
    }
    const double c1 = cpar[2 * b], c2 = cpar[2 * b + 1];
    __syncwarp();
    if (lane < NG) {
      const int g = lane;
      GPIn in;
      gauss_inputs(T, g, S.z, S.x, S.p, in);
      double V[3][3];
#pragma unroll
      for (int xi = 0; xi < 3; ++xi)
#pragma unroll
        for (int mh = 0; mh < 3; ++mh) {
          double t = 0.0;
          for (int ms = 0; ms < NQ; ++ms) t += S.v[mh * NQ + ms] * T.dphi[g][xi][ms];
          V[xi][mh] = t;
        }
      double Vp = 0.0;
#pragma unroll
      for (int ms = 0; ms < NL; ++ms) Vp += S.v[81 + ms] * T.psi[g][ms];
      double Zb[3][3], pb, c1b, c2b;
      point_P_vjp(in, c1, c2, V, Vp, Zb, pb, c1b, c2b);
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k) S.Zb[g][i * 3 + k] = Zb[i][k];
      S.pb[g] = pb;
      S.cb[g][0] = c1b;
      S.cb[g][1] = c2b;
    }
    __syncwarp();
    if (lane < 2) {
      double t = 0.0;
      for (int g = 0; g < NG; ++g) t += S.cb[g][lane];
      dc_elem[((size_t)b * n_elem + e) * 2 + lane] = t;
    }
    double* dub = du + b * ndof;
    for (int i = lane; i < ND; i += 32) {
      double t = 0.0;
      if (i < 81) {
        const int c = i / NQ, ns = i % NQ;
        for (int g = 0; g < NG; ++g)
          t += S.Zb[g][c * 3 + 0] * T.dphi[g][0][ns] + S.Zb[g][c * 3 + 1] * T.dphi[g][1][ns] +
               S.Zb[g][c * 3 + 2] * T.dphi[g][2][ns];
      } else {
        const int ns = i - 81;
        for (int g = 0; g < NG; ++g) t += S.pb[g] * T.psi[g][ns];
      }
      if (!isfinite(t)) gfe_raise(err, GFE_DEVERR_NONFINITE);
      dub[S.dofs[i]] += t;
    }
    __syncwarp();
  }
}

__global__ void sum_dc(const double* __restrict__ dc_elem, int32_t n_elem, int32_t batch, double* __restrict__ dc) {
  const int b = blockIdx.x, q = threadIdx.x & 1;
  if (threadIdx.x >= 2) return;
  double s = 0.0;
  for (int e = 0; e < n_elem; ++e) s += dc_elem[((size_t)b * n_elem + e) * 2 + q];
  dc[b * 2 + q] = s;
}

// ----------------------------------------------------------------------------------------------
// Element Jacobians: Iron's analytic tangent and the consistent tangent
// ----------------------------------------------------------------------------------------------
// Both are sums over Gauss points of  K(ms mh, ns nh) = g_ms^T D_g^(mh,nh) g_ns  (u-u block) with
// the reference basis gradients g (constant tables) and 3x3 blocks D_g expressed in xi space, plus
// the u-p / p-u blocks.  The work is split in two kernels:
//  * mr_gp_kernel, one thread per (element, Gauss point): kinematics and material tangent in FP64,
//    written as D_g (9 blocks x 9), Hv_g (u-p coefficients) and Pv_g (p-u coefficients);
//  * mr_contract_kernel, one CTA per element: H_g = D_g G_g (per Gauss point, 3 x 81 x 81 values
//    in shared memory), then the contraction K_mh^T = H_mh^T G^T against the constant table
//    G[(g,xi)][ms] (a 81 x 27 x 81 product per displacement component), the u-p / p-u blocks, and
//    the scatter into CSR through the per-element slot map.
// The contraction runs in FP64 (GFE_FP64) or FP32 (GFE_MIXED; the kinematics and det(F) stay FP64,
// the assembled values are accumulated in FP64).
//
// Iron's analytic tangent (src/finite_elasticity_routines.F90:1016-1274): the spatial blocks
// J_z w (c + sigma) / J_z w c of FINITE_ELASTICITY_GAUSS_ELASTICITY_TENSOR (:649-795) mapped to xi
// space with Z^-1 = dxi/dz (dphi/dz = Z^-T g), only the lower u-u triangle evaluated and mirrored
// to the upper (:1269-1274), p-u = J_z w dphi_ns/dz_nh psi_ms, u-p = J_z w (push(C^-1) dphi_ms)_mh
// psi_ns.  Consistent tangent: D_g^(mh,nh)[xi][zeta] = dP[xi][mh]/dZ[nh][zeta] from the forward-mode
// passes of point_dP, Hv = dP/dp, Pv = w J_z Z^-1.

// Iron's per-Gauss-point tangent blocks in spatial coordinates (src/finite_elasticity_routines.F90:
// 649-795 and 1072-1192): sub[0..2] = J_z w (c_sub + sigma) for the diagonal component blocks,
// sub[3..5] = J_z w c_sub for the off-diagonal blocks (mh, nh) = (1,0), (2,0), (2,1);
// hyd = J_z w push(C^-1).
template <typename S>
__device__ void iron_point_tensors(const GPT<S>& q, S c1, S c2, S sub[6][9], S hyd[9], S& jgw) {
  const S J = q.Jz / q.Jx;
  // unmodified right Cauchy-Green tensor and its inverse
  S C[3][3], Ci[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) C[i][j] = q.F[0][i] * q.F[0][j] + q.F[1][i] * q.F[1][j] + q.F[2][i] * q.F[2][j];
  const S I3 = inv3(C, Ci);
  const S L[6] = {C[0][0], C[1][1], C[2][2], C[0][1], C[0][2], C[1][2]};
  const S U[6] = {Ci[0][0], Ci[1][1], Ci[2][2], Ci[0][1], Ci[0][2], Ci[1][2]};
  // I3EE as filled by Fortran RESHAPE (column j listed): I3EE[i][j] = col[j][i]
  const S z0 = S(0), f4 = S(4), f2 = S(2);
  const S col[6][6] = {{z0, f4 * L[2], f4 * L[1], z0, z0, -f4 * L[5]},
                       {f4 * L[2], z0, f4 * L[0], z0, -f4 * L[4], z0},
                       {f4 * L[1], f4 * L[0], z0, -f2 * L[3], z0, z0},
                       {z0, z0, -f4 * L[3], -f2 * L[2], f2 * L[5], f2 * L[4]},
                       {z0, -f4 * L[4], z0, f2 * L[5], -f2 * L[1], f2 * L[3]},
                       {-f4 * L[5], z0, z0, f2 * L[4], f2 * L[3], -f2 * L[0]}};
  S D[6][6];
#pragma unroll
  for (int i = 0; i < 6; ++i)
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      S v = S(0);
      if (i < 3 && j < 3 && i != j) v = f4 * c2;
      if (i >= 3 && i == j) v = -f2 * c2;
      D[i][j] = v + q.p * (-f2 * U[i] * U[j] + S(0.5) * col[j][i] / I3);
    }
  const S I1 = C[0][0] + C[1][1] + C[2][2];
  const S t2 = f2 * (c1 + I1 * c2);
  S Sv[6] = {-f2 * c2 * C[0][0] + t2, -f2 * c2 * C[1][1] + t2, -f2 * c2 * C[2][2] + t2,
             -f2 * c2 * C[1][0], -f2 * c2 * C[2][0], -f2 * c2 * C[2][1]};
  S H[6] = {U[0], U[1], U[2], U[3], U[4], U[5]};
  S t[6][6];
  push_t(q.F, t);
  push_vec(t, Sv, J);
  push_vec(t, H, J);
  S tD[6][6];
#pragma unroll
  for (int i = 0; i < 6; ++i)
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      S s = S(0);
#pragma unroll
      for (int k = 0; k < 6; ++k) s += t[i][k] * D[k][j];
      tD[i][j] = s;
    }
#pragma unroll
  for (int i = 0; i < 6; ++i)
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      S s = S(0);
#pragma unroll
      for (int k = 0; k < 6; ++k) s += tD[i][k] * t[j][k];
      D[i][j] = s / J;
    }
  Sv[0] += q.p; Sv[1] += q.p; Sv[2] += q.p;
  jgw = q.Jz * q.w;
#pragma unroll
  for (int nh = 0; nh < 3; ++nh)
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) sub[nh][i * 3 + j] = jgw * (D[t2v(i, nh)][t2v(j, nh)] + Sv[t2v(i, j)]);
  const int om[3] = {1, 2, 2}, on[3] = {0, 0, 1};
#pragma unroll
  for (int o = 0; o < 3; ++o)
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) sub[3 + o][i * 3 + j] = jgw * D[t2v(i, om[o])][t2v(j, on[o])];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) hyd[i * 3 + j] = jgw * H[t2v(i, j)];
}

constexpr int kGPElems = 4;                // elements per CTA of mr_gp_kernel
constexpr uint32_t kTableWaitPolls = 1u << 24;  // bounded wait for the TMA copy of the tables
constexpr int kGPThreads = kGPElems * NG;  // 108
constexpr int kGPOut = 81 + 9 + 9;         // D (9 blocks x 9), Hv, Pv per Gauss point
constexpr int kGPItem = (NG * kGPOut + 3) / 4 * 4;  // per-element stride: a 16-byte multiple (TMA)

template <typename KS>
struct GPShared {
  KS x[kGPElems][81], z[kGPElems][81], p[kGPElems][8];
};

// One thread per (element, Gauss point).  out[item * kGPItem + g * kGPOut + j] in the contraction type TO:
// D[(mh*3+nh)*9 + xi*3+zeta], Hv[81 + xi*3+mh], Pv[90 + xi*3+nh].  KS is the kinematics type:
// double, or float on the FP32 paths (element data rounded once per node when staged, the volume
// Jacobians det(Z), det(X) still evaluated in FP64 from the exactly widened gradients; for the
// consistent tangent (EXACT) the forward-mode passes run in FP32 dual numbers, with J_z and its
// derivative in FP64 dual arithmetic).
template <typename TO, bool EXACT, typename KS = double>
__global__ void __launch_bounds__(kGPThreads)
mr_gp_kernel(const int32_t* __restrict__ elems, int32_t count, const int32_t* __restrict__ eq2,
             const int32_t* __restrict__ elin, int32_t nq2, const double* __restrict__ xg,
             const double* __restrict__ dep, const double* __restrict__ cpar, const TablesT<KS>* __restrict__ Tg,
             TO* __restrict__ out, unsigned* err) {
  extern __shared__ __align__(16) double smem_d[];
  unsigned char* sbase = reinterpret_cast<unsigned char*>(smem_d);
  TablesT<KS>& T = *reinterpret_cast<TablesT<KS>*>(sbase);
  GPShared<KS>& S = *reinterpret_cast<GPShared<KS>*>(sbase + sizeof(TablesT<KS>));
  uint64_t* tbar = reinterpret_cast<uint64_t*>(sbase + sizeof(TablesT<KS>) + sizeof(GPShared<KS>));
  // the basis tables arrive by one TMA bulk copy while the threads gather the element data
  if (threadIdx.x == 0) {
    tc::mbar_init(tbar, 1);
    tc::mbar_arrive_expect_tx(tbar, (uint32_t)sizeof(TablesT<KS>));
    tc::bulk_copy_g2s(&T, Tg, (uint32_t)sizeof(TablesT<KS>), tbar);
  }
  const int le = threadIdx.x / NG, g = threadIdx.x % NG;
  const int item = blockIdx.x * kGPElems + le;
  // cooperative load of the CTA's elements
  for (int t = threadIdx.x; t < kGPElems * NQ; t += blockDim.x) {
    const int l = t / NQ, i = t % NQ, it = blockIdx.x * kGPElems + l;
    if (it >= count) continue;
    const int e = __ldg(elems + it);
    const int n = __ldg(eq2 + (size_t)e * NQ + i);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      S.x[l][c * NQ + i] = (KS)__ldg(xg + (size_t)c * nq2 + n);
      S.z[l][c * NQ + i] = (KS)dep[(size_t)c * nq2 + n];
    }
  }
  for (int t = threadIdx.x; t < kGPElems * NL; t += blockDim.x) {
    const int l = t / NL, i = t % NL, it = blockIdx.x * kGPElems + l;
    if (it >= count) continue;
    const int e = __ldg(elems + it);
    S.p[l][i] = (KS)dep[(size_t)3 * nq2 + __ldg(elin + (size_t)e * NL + i)];
  }
  __syncthreads();
  // every thread waits for the tables (so none exits while the copy is in flight); bounded
  if (!tc::mbar_wait(tbar, 0, kTableWaitPolls)) {
    gfe_raise(err, GFE_DEVERR_TIMEOUT);
    tc::mbar_wait(tbar, 0, kTableWaitPolls);
    return;
  }
  if (item >= count) return;
  TO* o = out + (size_t)item * kGPItem + (size_t)g * kGPOut;
  if constexpr (!EXACT) {
    const KS c1 = (KS)cpar[0], c2 = (KS)cpar[1];
    GPT<KS> q;
    if (!gauss_point(T, g, S.z[le], S.x[le], S.p[le], q)) gfe_raise(err, GFE_DEVERR_JACOBIAN);
    KS sub[6][9], hyd[9], jgw;
    iron_point_tensors(q, c1, c2, sub, hyd, jgw);
    // blocks to xi space: Dxi = Zi sub Zi^T (Zi = dxi/dz); upper blocks as transposes of the lower
#pragma unroll
    for (int mh = 0; mh < 3; ++mh)
#pragma unroll
      for (int nh = 0; nh < 3; ++nh) {
        const int blk = mh == nh ? mh : (mh > nh ? 3 + (mh == 1 ? 0 : (nh == 0 ? 1 : 2))
                                                 : 3 + (nh == 1 ? 0 : (mh == 0 ? 1 : 2)));
        const bool tr = mh < nh;
        KS W[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int z = 0; z < 3; ++z) {
            KS s = KS(0);
#pragma unroll
            for (int j = 0; j < 3; ++j) s += (tr ? sub[blk][j * 3 + i] : sub[blk][i * 3 + j]) * q.Zi[z][j];
            W[i][z] = s;  // (sub Zi^T)[i][zeta]
          }
#pragma unroll
        for (int xi = 0; xi < 3; ++xi)
#pragma unroll
          for (int z = 0; z < 3; ++z)
            o[(mh * 3 + nh) * 9 + xi * 3 + z] =
                (TO)(q.Zi[xi][0] * W[0][z] + q.Zi[xi][1] * W[1][z] + q.Zi[xi][2] * W[2][z]);
      }
#pragma unroll
    for (int xi = 0; xi < 3; ++xi)
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        o[81 + xi * 3 + m] = (TO)(q.Zi[xi][0] * hyd[m * 3 + 0] + q.Zi[xi][1] * hyd[m * 3 + 1] +
                                  q.Zi[xi][2] * hyd[m * 3 + 2]);
        o[90 + xi * 3 + m] = (TO)(jgw * q.Zi[xi][m]);
      }
  } else {
    const KS c1 = (KS)cpar[0], c2 = (KS)cpar[1];
    GPInT<KS> in;
    gauss_inputs(T, g, S.z[le], S.x[le], S.p[le], in);
    float jz[10];
    if constexpr (std::is_same<KS, float>::value) jz_seeds(in.Z, jz);
    for (int seed = 0; seed < 10; ++seed) {
      KS d[9], Jz;
      point_dP(in, seed, c1, c2, d, &Jz, std::is_same<KS, float>::value ? jz : nullptr);
      if (seed < 9) {
        const int nh = seed / 3, z = seed % 3;
#pragma unroll
        for (int xi = 0; xi < 3; ++xi)
#pragma unroll
          for (int mh = 0; mh < 3; ++mh) o[(mh * 3 + nh) * 9 + xi * 3 + z] = (TO)d[xi * 3 + mh];
      } else {
#pragma unroll
        for (int k = 0; k < 9; ++k) o[81 + k] = (TO)d[k];
        KS Zi[3][3];
        const KS dz = inv3(in.Z, Zi);
        if (!(dz > KS(0)) || !isfinite(dz)) gfe_raise(err, GFE_DEVERR_JACOBIAN);
#pragma unroll
        for (int xi = 0; xi < 3; ++xi)
#pragma unroll
          for (int nh = 0; nh < 3; ++nh) o[90 + xi * 3 + nh] = (TO)(in.w * Jz * Zi[xi][nh]);
      }
    }
  }
}

constexpr int kCThreads = 256;

// u-p / p-u coefficients of one element: HvG[g][(mh,ms)] = sum_xi G[(g,xi)][ms] Hv_g[xi][mh] and
// PvG[g][(nh,ns)] = sum_xi G[(g,xi)][ns] Pv_g[xi][nh] from the Gauss-point blocks Dg[g][99].
template <typename TS, int GP>
__device__ __forceinline__ void form_up_coefficients(const TS (*G)[GP], const TS (*Dg)[kGPOut], TS (*HvG)[81],
                                                     TS (*PvG)[81]) {
  for (int t = threadIdx.x; t < NG * 81; t += blockDim.x) {
    const int g = t / 81, c = t % 81, h = c / 27, s = c % 27;
    const TS g0 = G[g * 3 + 0][s], g1 = G[g * 3 + 1][s], g2 = G[g * 3 + 2][s];
    HvG[g][c] = g0 * Dg[g][81 + h] + g1 * Dg[g][84 + h] + g2 * Dg[g][87 + h];
    PvG[g][c] = g0 * Dg[g][90 + h] + g1 * Dg[g][93 + h] + g2 * Dg[g][96 + h];
  }
}

// The u-u block of one element's 89 x 89 matrix (row-major at Ke) from the staged product
// C[(mh*3+nh)*27+ms][ns]; Iron mirrors its lower triangle into the upper one unless EXACT.  One
// warp writes each row (consecutive lanes, consecutive entries).
template <bool EXACT, typename KT, typename CT, int P>
__device__ __forceinline__ void write_uu_block(KT* __restrict__ Ke, const CT (*C)[P]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int cq[3], cr[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    cq[j] = (lane + 32 * j) / 27;
    cr[j] = (lane + 32 * j) % 27;
  }
  for (int r = warp; r < 81; r += nw) {
    const int rq = r / 27, rr = r % 27;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const int c = lane + 32 * j;
      if (c < 81) {
        const CT v = (EXACT || r >= c) ? C[(rq * 3 + cq[j]) * 27 + rr][cr[j]] : C[(cq[j] * 3 + rq) * 27 + cr[j]][rr];
        Ke[r * ND + c] = (KT)v;
      }
    }
  }
}

// The u-p and p-u blocks of one element's matrix as 27-term sums of HvG / PvG with the pressure
// basis psi, and the zero p-p block.
template <typename KT, typename CT>
__device__ __forceinline__ void write_up_blocks(KT* __restrict__ Ke, const CT (*HvG)[81], const CT (*PvG)[81],
                                                const CT (*psi)[NL]) {
  for (int t = threadIdx.x; t < 2 * 81 * NL + NL * NL; t += blockDim.x) {
    if (t < 81 * NL) {  // u rows, p columns
      const int r = t / NL, b = t % NL;
      CT s = CT(0);
      for (int g = 0; g < NG; ++g) s += HvG[g][r] * psi[g][b];
      Ke[r * ND + 81 + b] = (KT)s;
    } else if (t < 2 * 81 * NL) {  // p rows, u columns
      const int b = (t - 81 * NL) / 81, c = (t - 81 * NL) % 81;
      CT s = CT(0);
      for (int g = 0; g < NG; ++g) s += psi[g][b] * PvG[g][c];
      Ke[(81 + b) * ND + c] = (KT)s;
    } else {
      const int q = t - 2 * 81 * NL;
      Ke[(81 + q / NL) * ND + 81 + q % NL] = KT(0);
    }
  }
}

// Per element the u-u block is one product, as in the tensor-core kernel below:
//   C[(mh,nh,ms)][ns] = sum_{(g,zeta)} A[(mh,nh,ms)][(g,zeta)] G[(g,zeta)][ns],
//   A[(mh,nh,ms)][(g,zeta)] = sum_xi G[(g,xi)][ms] D_g[(mh,nh)][xi][zeta],
// 243 x 81 by 81 x 27.  A is formed in two passes of kCRows rows ([k][row] in shared memory, so a
// thread's four rows are one vector load), and each thread of the product accumulates a 4 x 4 tile
// of C in registers: two vector loads per 16 FMAs.  u-p / p-u blocks and Iron's lower-triangle
// mirror are formed from C, HvG and PvG while the element matrix is written.
constexpr int kCRows = 128;                   // rows of A per pass
constexpr int kCTileRows = kCRows / 4;        // 32 row groups of 4
constexpr int kCTileCols = 7;                 // 7 column groups of 4 (27 columns, padded to 28)

// The arrays read with vector loads (A, G) come first: their rows are multiples of 16 bytes.
template <typename TS>
struct ContractShared {
  TS A[81][kCRows];     // A[(g,zeta)][row] of the current pass
  TS G[81][28];         // G[(g,xi)][ms]; column 27 zero
  TS C[2 * kCRows][28]; // C[(mh,nh,ms)][ns]
  TS HvG[NG][81];       // sum_xi G[(g,xi)][ms] Hv[xi][mh]  -> [g][(mh,ms)]
  TS PvG[NG][81];       // sum_xi G[(g,xi)][ns] Pv[xi][nh]  -> [g][(nh,ns)]
  TS Dg[NG][kGPOut];    // this element's Gauss-point blocks
  TS psi[NG][NL];       // pressure basis at the Gauss points
};
static_assert(sizeof(float) * kCRows % 16 == 0 && sizeof(float) * 28 % 16 == 0, "vector rows");
static_assert(sizeof(float) * 81 * kCRows % 16 == 0, "G follows A on a 16-byte boundary");

template <typename TS>
__device__ __forceinline__ void load4(const TS* p, TS (&v)[4]) {
  if constexpr (std::is_same<TS, float>::value) {
    const float4 q = *reinterpret_cast<const float4*>(p);
    v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
  } else {
    const double2 a = *reinterpret_cast<const double2*>(p), b = *reinterpret_cast<const double2*>(p + 2);
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
  }
}

// Element matrices of `count` elements into Kel[e][89][89] (element number e = elems[item]).
template <typename TS, bool EXACT>
__global__ void __launch_bounds__(kCThreads)
mr_contract_kernel(const int32_t* __restrict__ elems, int32_t count, const Tables* __restrict__ Tg,
                   const TS* __restrict__ gp, TS* __restrict__ Kel) {
  extern __shared__ __align__(16) unsigned char craw[];
  ContractShared<TS>& S = *reinterpret_cast<ContractShared<TS>*>(craw);
  const int tid = threadIdx.x;
  for (int t = tid; t < 81 * 28; t += blockDim.x) {
    const int k = t / 28, ms = t % 28;
    S.G[k][ms] = ms < 27 ? (TS)Tg->dphi[k / 3][k % 3][ms] : TS(0);
  }
  for (int t = tid; t < NG * NL; t += blockDim.x) S.psi[t / NL][t % NL] = (TS)Tg->psi[t / NL][t % NL];
  const int rq = tid / kCTileCols, cq = tid % kCTileCols;  // product tile of this thread
  const bool in_product = tid < kCTileRows * kCTileCols;
  for (int item = blockIdx.x; item < count; item += gridDim.x) {
    __syncthreads();
    const TS* src = gp + (size_t)item * kGPItem;
    for (int t = tid; t < NG * kGPOut; t += blockDim.x) (&S.Dg[0][0])[t] = src[t];
    __syncthreads();
    form_up_coefficients<TS, 28>(S.G, S.Dg, S.HvG, S.PvG);
    for (int pass = 0; pass < 2; ++pass) {
      // operand rows [pass * kCRows, pass * kCRows + kCRows); rows past 242 are zero
      for (int t = tid; t < 81 * kCRows; t += blockDim.x) {
        const int k = t / kCRows, rl = t % kCRows, row = pass * kCRows + rl;
        TS v = TS(0);
        if (row < 243) {
          const int pair = row / 27, ms = row % 27, g = k / 3, zeta = k % 3;
          const TS* D = &S.Dg[g][pair * 9 + zeta];
          v = S.G[g * 3 + 0][ms] * D[0] + S.G[g * 3 + 1][ms] * D[3] + S.G[g * 3 + 2][ms] * D[6];
        }
        S.A[k][rl] = v;
      }
      __syncthreads();
      if (in_product) {
        TS acc[4][4];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) acc[a][b] = TS(0);
#pragma unroll 3
        for (int k = 0; k < 81; ++k) {
          TS av[4], bv[4];
          load4(&S.A[k][rq * 4], av);
          load4(&S.G[k][cq * 4], bv);
#pragma unroll
          for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) acc[a][b] += av[a] * bv[b];
        }
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) S.C[pass * kCRows + rq * 4 + a][cq * 4 + b] = acc[a][b];
      }
      __syncthreads();  // A is rewritten by the next pass
    }
    TS* Ke = Kel + (size_t)__ldg(elems + item) * ND * ND;
    write_up_blocks<TS, TS>(Ke, S.HvG, S.PvG, S.psi);
    write_uu_block<EXACT, TS, TS, 28>(Ke, S.C);
  }
}

// ---------------------------------------------------------------------------------------------
// Tensor-core (tcgen05, TF32) basis-gradient contraction of the element Jacobian
// ---------------------------------------------------------------------------------------------
// For every (mh, nh) displacement-component pair the u-u block is
//   K[(ms,mh),(ns,nh)] = sum_{g,zeta} A[(mh,nh,ms)][(g,zeta)] G[(g,zeta)][ns],
//   A[(mh,nh,ms)][(g,zeta)] = sum_xi G[(g,xi)][ms] D_g[(mh,nh)][xi][zeta],
// i.e. one 243 x 81 by 81 x 27 product per element.  A is formed on the CUDA cores (FP32) straight
// into shared memory in the tensor cores' operand layout; the product runs as two M = 128 halves of
// tcgen05.mma kind::tf32 (N = 32, K = 88 in 11 steps of 8) accumulating in tensor memory.  With
// SPLIT3 each operand is split into a TF32 head and a TF32 tail and the three products
// hi*hi + lo*hi + hi*lo recover about FP32 accuracy; without it the contraction is plain TF32
// (about 1e-3 relative).  u-p / p-u blocks, Iron's lower-triangle mirror and the element-matrix
// output are as in mr_contract_kernel.
constexpr int kTCThreads = 1024;               // 32 warps: every phase is latency bound
constexpr int kTCGroupWarps = kTCThreads / 32 / 16;  // warps sharing one 8-row group of the operand
constexpr int kTK = 88;                        // K = 27 Gauss points x 3, padded to 11 steps of 8
constexpr int kTKC = kTK / 4;                  // core-matrix columns along K (4 TF32 = 16 bytes)
constexpr int kTABytes = 16 * kTKC * 128;      // one M = 128 operand tile
constexpr int kTBBytes = 4 * kTKC * 128;       // the N = 32 operand
constexpr uint32_t kTLbo = 128, kTSbo = kTKC * 128;
constexpr int kTKRow = 33;                     // padded row of the staged product (no bank conflicts)
constexpr uint32_t kTWaitPolls = 1u << 24;     // bounded mbarrier wait

struct __align__(128) TCShared {
  unsigned char A[2][kTABytes];  // head, tail of the current M half
  unsigned char B[2][kTBBytes];  // G head, tail: B[ns][(g,zeta)]
  float G[81][28];               // G[(g,xi)][ms]; column 27 zero
  float psi[NG][NL];
  alignas(16) float Dg[2][kGPItem];  // Gauss-point blocks of the current and the next element (TMA)
  float K[256][kTKRow];          // product rows (mh,nh,ms), columns ns
  float HvG[NG][81];
  float PvG[NG][81];
  uint64_t mbar;
  uint64_t dbar[2];              // completion of the bulk copies into Dg[0], Dg[1]
  uint32_t tmem;
  int abort;
};

// byte offset of element (row, k) in a no-swizzle K-major operand with kTKC core columns
__device__ __forceinline__ uint32_t tc_offset(int row, int k) {
  return (uint32_t)((((row >> 3) * kTKC + (k >> 2)) * 8 + (row & 7)) * 16 + (k & 3) * 4);
}

template <bool EXACT, bool SPLIT3>
__global__ void __launch_bounds__(kTCThreads, 1)
mr_contract_tc_kernel(const int32_t* __restrict__ elems, int32_t count, const Tables* __restrict__ Tg,
                      const float* __restrict__ gp, float* __restrict__ Kel, unsigned* err) {
  static_assert(kTCThreads % (16 * 32) == 0, "whole warps per 8-row group of an M = 128 operand tile");
  extern __shared__ __align__(1024) unsigned char traw[];
  TCShared& S = *reinterpret_cast<TCShared*>(traw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // constant operands: G (FP32, for forming A) and B = G^T split into TF32 head / tail
  for (int t = tid; t < 81 * 28; t += blockDim.x) {
    const int k = t / 28, ms = t % 28;
    S.G[k][ms] = ms < 27 ? (float)Tg->dphi[k / 3][k % 3][ms] : 0.0f;
  }
  for (int t = tid; t < NG * NL; t += blockDim.x) S.psi[t / NL][t % NL] = (float)Tg->psi[t / NL][t % NL];
  for (int t = tid; t < 32 * kTK; t += blockDim.x) {
    const int n = t / kTK, k = t % kTK;
    const float v = (n < 27 && k < 81) ? (float)Tg->dphi[k / 3][k % 3][n] : 0.0f;
    const float hi = tc::to_tf32(v);
    *reinterpret_cast<float*>(S.B[0] + tc_offset(n, k)) = hi;
    *reinterpret_cast<float*>(S.B[1] + tc_offset(n, k)) = tc::to_tf32(v - hi);
  }
  if (warp == 0) tc::tmem_alloc(&S.tmem, 64);
  constexpr uint32_t kDgBytes = kGPItem * sizeof(float);
  if (tid == 0) {
    tc::mbar_init(&S.mbar, 1);
    tc::mbar_init(&S.dbar[0], 1);
    tc::mbar_init(&S.dbar[1], 1);
    S.abort = 0;
    // the first element's Gauss-point blocks: one TMA bulk copy
    if ((int)blockIdx.x < count) {
      tc::mbar_arrive_expect_tx(&S.dbar[0], kDgBytes);
      tc::bulk_copy_g2s(S.Dg[0], gp + (size_t)blockIdx.x * kGPItem, kDgBytes, &S.dbar[0]);
    }
  }
  tc::fence_proxy_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = S.tmem;
  constexpr uint32_t idesc = tc::idesc_tf32(128, 32);
  const uint32_t a_hi = tc::smem_u32(S.A[0]), a_lo = tc::smem_u32(S.A[1]);
  const uint32_t b_hi = tc::smem_u32(S.B[0]), b_lo = tc::smem_u32(S.B[1]);
  uint32_t parity = 0;
  uint32_t dpar[2] = {0u, 0u};
  bool pending[2] = {(int)blockIdx.x < count, false};  // (thread 0) copies issued and not yet waited for
  // operand formation: warp w writes the 8-row group w of the current M = 128 tile, lane l its
  // row 8 w + l / 4 and the K columns 4 kc + l % 4 (each step one core matrix, 128 bytes)
  const int r_in = lane >> 2, kq = lane & 3;

  int buf = 0;
  for (int item = blockIdx.x; item < count; item += gridDim.x, buf ^= 1) {
    __syncthreads();  // every thread is done with the previous element, whose buffer is Dg[buf ^ 1]
    const int next = item + (int)gridDim.x;
    if (tid == 0 && next < count) {
      // prefetch the next element's blocks while this one is computed
      tc::fence_proxy_async();
      tc::mbar_arrive_expect_tx(&S.dbar[buf ^ 1], kDgBytes);
      tc::bulk_copy_g2s(S.Dg[buf ^ 1], gp + (size_t)next * kGPItem, kDgBytes, &S.dbar[buf ^ 1]);
      pending[buf ^ 1] = true;
    }
    if (!tc::mbar_wait(&S.dbar[buf], dpar[buf], kTWaitPolls)) {
      gfe_raise(err, GFE_DEVERR_TIMEOUT);
      tc::mbar_wait(&S.dbar[buf], dpar[buf], kTWaitPolls);
      atomicMax(&S.abort, 1);
    }
    if (tid == 0) pending[buf] = false;
    dpar[buf] ^= 1u;
    __syncthreads();
    if (S.abort) break;
    const float(*Dg)[kGPOut] = reinterpret_cast<const float(*)[kGPOut]>(S.Dg[buf]);
    float* Ke = Kel + (size_t)__ldg(elems + item) * ND * ND;
    // warp w forms the core columns kc = w / 16, w / 16 + kTCGroupWarps, ... of the 8-row group w % 16
    const int rg = warp & 15, kc0 = warp >> 4;
    for (int half = 0; half < 2; ++half) {
      const int row = half * 128 + rg * 8 + r_in;
      const bool valid = row < 243;
      const int pair = valid ? row / 27 : 0, ms = valid ? row % 27 : 0;
      const float* Gm = &S.G[0][ms];
      const float* Dp = &Dg[0][pair * 9];
      unsigned char* a0 = S.A[0] + (rg * kTKC) * 128 + lane * 4;
      unsigned char* a1 = S.A[1] + (rg * kTKC) * 128 + lane * 4;
#pragma unroll 2
      for (int kc = kc0; kc < kTKC; kc += kTCGroupWarps) {
        const int k = kc * 4 + kq;
        float v = 0.0f;
        if (valid && k < 81) {
          const int g = k / 3, zeta = k - 3 * g;
          const float* D = Dp + g * kGPOut + zeta;
          const float* Gg = Gm + (g * 3) * 28;
          v = Gg[0] * D[0] + Gg[28] * D[3] + Gg[56] * D[6];
        }
        const float hi = tc::to_tf32(v);
        *reinterpret_cast<float*>(a0 + kc * 128) = hi;
        if (SPLIT3) *reinterpret_cast<float*>(a1 + kc * 128) = tc::to_tf32(v - hi);
      }
      tc::fence_proxy_async();
      __syncthreads();
      if (tid == 0) {
        tc::fence_after_sync();
        const uint32_t d = tmem + (uint32_t)(half * 32);
#pragma unroll 1
        for (int s = 0; s < kTK / 8; ++s) {
          const uint32_t ko = (uint32_t)(s * 256);
          tc::mma_tf32(d, tc::smem_desc(a_hi + ko, kTLbo, kTSbo), tc::smem_desc(b_hi + ko, kTLbo, kTSbo), idesc,
                       s > 0 ? 1u : 0u);
          if (SPLIT3) {
            tc::mma_tf32(d, tc::smem_desc(a_lo + ko, kTLbo, kTSbo), tc::smem_desc(b_hi + ko, kTLbo, kTSbo), idesc, 1u);
            tc::mma_tf32(d, tc::smem_desc(a_hi + ko, kTLbo, kTSbo), tc::smem_desc(b_lo + ko, kTLbo, kTSbo), idesc, 1u);
          }
        }
        tc::commit(&S.mbar);
        // the A tile is rewritten by the next half: wait (bounded) for this half's products
        if (!tc::mbar_wait(&S.mbar, parity, kTWaitPolls)) {
          // the MMAs may still be writing tensor memory: wait once more for their commit before
          // anything releases it; if that also ends without it, the tensor memory stays
          // allocated (abort = 2) rather than being freed under the MMAs
          gfe_raise(err, GFE_DEVERR_TIMEOUT);
          const bool drained = tc::mbar_wait(&S.mbar, parity, kTWaitPolls);
          S.abort = drained ? 1 : 2;
        }
      }
      // work that needs neither A nor the product runs while the tensor cores multiply
      if (half == 0) form_up_coefficients<float, 28>(S.G, Dg, S.HvG, S.PvG);
      else write_up_blocks<float, float>(Ke, S.HvG, S.PvG, S.psi);
      parity ^= 1u;
      __syncthreads();
      tc::fence_after_sync();
      if (S.abort) break;
    }
    if (S.abort) break;
    // tensor memory -> staged product: warp w < 8 reads lanes 32 (w % 4) .. of half w / 4
    if (warp < 8) {
      const int half = warp >> 2, q = warp & 3;
      float v[32];
      tc::tmem_ld_32x32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(half * 32), v);
      const int row = half * 128 + q * 32 + lane;
#pragma unroll
      for (int n = 0; n < 27; ++n) S.K[row][n] = v[n];
    }
    tc::fence_before_sync();
    __syncthreads();
    write_uu_block<EXACT, float, float, kTKRow>(Ke, S.K);
  }
  // no bulk copy may still be landing in this CTA's shared memory when it exits (bounded)
  if (tid == 0)
    for (int b = 0; b < 2; ++b)
      if (pending[b] && !tc::mbar_wait(&S.dbar[b], dpar[b], kTWaitPolls)) gfe_raise(err, GFE_DEVERR_TIMEOUT);
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0 && S.abort < 2) tc::tmem_dealloc(tmem, 64);
}

size_t residual_smem() { return sizeof(Tables) + kResWarps * sizeof(double) * (81 + 81 + 8 + NG * 9 + NG + 48); }

int check_mesh(int32_t n_elem, const int32_t* eq2, const int32_t* elin, int32_t nq2, int32_t nlin, const double* xg,
               const char* fn) {
  if (n_elem < 0 || nq2 <= 0 || nlin <= 0 || (n_elem > 0 && (!eq2 || !elin || !xg)))
    return gfe::set_error(GFE_ERR_ARG, "%s: invalid mesh arguments", fn);
  return GFE_OK;
}

int set_smem(const void* kernel, size_t bytes) {
  GFE_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  return GFE_OK;
}

}  // namespace

extern "C" int gfe_mr_residual(int32_t n_elem, const int32_t* eq2, const int32_t* elin, int32_t nq2, int32_t nlin,
                               const double* xg, const int32_t* color_elems, const int32_t* color_ptr_host,
                               int32_t n_colors, int32_t batch, const double* dep, const double* cpar, double* R,
                               void* stream) {
  const char* fn = "gfe_mr_residual";
  int rc = check_mesh(n_elem, eq2, elin, nq2, nlin, xg, fn);
  if (rc) return rc;
  if (batch <= 0 || !dep || !cpar || !R || (n_elem > 0 && (!color_elems || !color_ptr_host || n_colors <= 0)))
    return gfe::set_error(GFE_ERR_ARG, "%s: invalid arguments", fn);
  if (color_ptr_host[0] != 0 || color_ptr_host[n_colors] != n_elem)
    return gfe::set_error(GFE_ERR_ARG, "%s: colour offsets must run from 0 to n_elem", fn);
  const Tables* T = nullptr;
  if ((rc = device_tables(&T))) return rc;
  cudaStream_t s = gfe::as_stream(stream);
  const int64_t ndof = 3ll * nq2 + nlin;
  GFE_CUDA_TRY(cudaMemsetAsync(R, 0, sizeof(double) * ndof * batch, s));
  const size_t sm = residual_smem();
  if ((rc = set_smem((const void*)mr_residual_kernel, sm))) return rc;
  unsigned* err = gfe::device_error_word();
  void* prof = gfe::stage_begin(GFE_STAGE_MR_RESIDUAL, s);
  int launches = 0;
  for (int c = 0; c < n_colors; ++c) {
    const int c0 = color_ptr_host[c], cnt = color_ptr_host[c + 1] - c0;
    if (cnt <= 0) continue;
    const long long items = (long long)cnt * batch;
    const int grid = (int)std::min<long long>((items + kResWarps - 1) / kResWarps, 16ll * gfe::sm_count());
    mr_residual_kernel<<<grid, kResWarps * 32, sm, s>>>(color_elems + c0, cnt, batch, eq2, elin, nq2, nlin, xg, dep,
                                                       cpar, T, R, ndof, err);
    ++launches;
  }
  gfe::stage_end(GFE_STAGE_MR_RESIDUAL, prof, s, launches);
  GFE_LAUNCH_CHECK(fn);
  return GFE_OK;
}

extern "C" int gfe_mr_slot_map(int32_t n_elem, const int32_t* eq2, const int32_t* elin, int32_t nq2,
                               const int32_t* color_elems, const int32_t* row_ptr, const int32_t* col_idx,
                               int32_t* slots, void* stream) {
  const char* fn = "gfe_mr_slot_map";
  if (n_elem < 0 || !eq2 || !elin || !color_elems || !row_ptr || !col_idx || !slots)
    return gfe::set_error(GFE_ERR_ARG, "%s: invalid arguments", fn);
  if (n_elem == 0) return GFE_OK;
  cudaStream_t s = gfe::as_stream(stream);
  mr_slot_kernel<<<16 * gfe::sm_count(), 256, 0, s>>>(color_elems, n_elem, eq2, elin, nq2, row_ptr, col_idx, slots);
  GFE_LAUNCH_CHECK(fn);
  return GFE_OK;
}

namespace {

// Element Jacobians of one problem (mode 0: Iron's analytic tangent, 1: consistent tangent), in the
// contraction precision `precision`.  Elements in chunks of at most kElemChunk: the Gauss-point
// kernel fills a scratch array, the contraction kernel turns it into element matrices Kel (all
// elements; FP64 for GFE_FP64, else FP32); then the row gather assembles the CSR values (when
// `values`), and K_out receives the element matrices in FP64 (when given).
constexpr int kElemChunk = 1 << 16;

template <bool EXACT, bool SPLIT3>
void launch_contract_tc(int grid, cudaStream_t s, const int32_t* elems, int cnt, const Tables* T, const float* gp,
                        float* Kel, unsigned* err) {
  mr_contract_tc_kernel<EXACT, SPLIT3><<<grid, kTCThreads, sizeof(TCShared), s>>>(elems, cnt, T, gp, Kel, err);
}

// Node incidence scratch (counts, then lists) and the row gather into `values`.
template <typename TS>
int gather_rows(int32_t n_elem, const int32_t* elems, const int32_t* eq2, const int32_t* elin, int32_t nq2,
                int32_t nlin, const TS* Kel, const int32_t* slots, const int32_t* row_ptr, double* values,
                cudaStream_t s, unsigned* err) {
  const int32_t n_nodes = nq2 + nlin;
  int32_t* inc = nullptr;
  const size_t words = (size_t)n_nodes * (1 + kMaxInc);
  int rc = gfe::scratch_alloc((void**)&inc, sizeof(int32_t) * words, s, "node incidence");
  if (rc) return rc;
  int32_t* cnt = inc;
  int32_t* list = inc + n_nodes;
  cudaError_t e = cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (size_t)n_nodes, s);
  if (e != cudaSuccess) {
    gfe::scratch_free(inc, s);
    return gfe::set_error(GFE_ERR_CUDA, "node incidence: %s", cudaGetErrorString(e));
  }
  const int sms = gfe::sm_count();
  mr_incidence_fill<<<8 * sms, 256, 0, s>>>(elems, n_elem, eq2, elin, nq2, cnt, list, err);
  mr_incidence_sort<<<(n_nodes + 255) / 256, 256, 0, s>>>(n_nodes, cnt, list);
  const long long rows = 3ll * nq2 + nlin;
  const int grid = (int)std::min<long long>((rows + kRowWarps - 1) / kRowWarps, 16ll * sms);
  mr_row_gather_kernel<TS><<<grid, kRowWarps * 32, 0, s>>>(nq2, nlin, cnt, list, Kel, slots, row_ptr, values,
                                                          nullptr, err);
  gfe::scratch_free(inc, s);
  return GFE_OK;
}

template <typename TS>
int jacobian_impl(int mode, int32_t n_elem, const int32_t* eq2, const int32_t* elin, int32_t nq2, int32_t nlin,
                  const double* xg, const int32_t* elems, const double* dep, const double* cpar,
                  const int32_t* slots, const int32_t* row_ptr, double* values, double* K_out, cudaStream_t s,
                  const char* fn, int tc_mode = 0) {
  const Tables* T = nullptr;
  int rc = device_tables(&T);
  if (rc) return rc;
  // Iron's analytic tangent on the FP32 paths: FP32 kinematics from the FP32 tables
  using KF = typename std::conditional<std::is_same<TS, float>::value, float, double>::type;
  const TablesT<KF>* TK = nullptr;
  if constexpr (std::is_same<KF, float>::value) {
    if ((rc = device_tables_f(&TK))) return rc;
  } else {
    TK = T;
  }
  if (n_elem == 0) return GFE_OK;
  const size_t gsm_k = sizeof(TablesT<KF>) + sizeof(GPShared<KF>) + 16;  // + the tables' mbarrier
  const size_t csm = sizeof(ContractShared<TS>);
  const void* gk = mode == 0 ? (const void*)mr_gp_kernel<TS, false, KF> : (const void*)mr_gp_kernel<TS, true, KF>;
  const void* ck = mode == 0 ? (const void*)mr_contract_kernel<TS, false> : (const void*)mr_contract_kernel<TS, true>;
  if ((rc = set_smem(gk, gsm_k)) || (rc = set_smem(ck, csm))) return rc;
  if (tc_mode) {
    const void* tk[4] = {(const void*)mr_contract_tc_kernel<false, false>, (const void*)mr_contract_tc_kernel<false, true>,
                         (const void*)mr_contract_tc_kernel<true, false>, (const void*)mr_contract_tc_kernel<true, true>};
    for (const void* k : tk)
      if ((rc = set_smem(k, sizeof(TCShared)))) return rc;
  }
  const int chunk = std::min(n_elem, kElemChunk);
  // element matrices: straight into K_out when it has the contraction's type
  constexpr bool kDirect = std::is_same<TS, double>::value;
  TS* Kel = nullptr;
  bool own_kel = true;
  if (kDirect && K_out) {
    Kel = reinterpret_cast<TS*>(K_out);
    own_kel = false;
  } else if ((rc = gfe::scratch_alloc((void**)&Kel, sizeof(TS) * (size_t)n_elem * ND * ND, s, "element matrices"))) {
    return rc;
  }
  TS* gpbuf = nullptr;
  if ((rc = gfe::scratch_alloc((void**)&gpbuf, sizeof(TS) * (size_t)chunk * kGPItem + 16, s,
                               "Gauss-point tangent blocks"))) {
    if (own_kel) gfe::scratch_free(Kel, s);
    return rc;
  }
  unsigned* err = gfe::device_error_word();
  void* prof = gfe::stage_begin(GFE_STAGE_MR_JACOBIAN, s);
  int launches = 0;
  const int sms = gfe::sm_count();
  for (int c0 = 0; c0 < n_elem; c0 += chunk) {
    const int cnt = std::min(chunk, n_elem - c0);
    const int ggrid = (cnt + kGPElems - 1) / kGPElems;
    if (mode == 0)
      mr_gp_kernel<TS, false, KF><<<ggrid, kGPThreads, gsm_k, s>>>(elems + c0, cnt, eq2, elin, nq2, xg, dep, cpar, TK,
                                                                   gpbuf, err);
    else
      mr_gp_kernel<TS, true, KF><<<ggrid, kGPThreads, gsm_k, s>>>(elems + c0, cnt, eq2, elin, nq2, xg, dep, cpar, TK,
                                                                  gpbuf, err);
    if constexpr (std::is_same<TS, float>::value) {
      if (tc_mode) {
        const int tgrid = std::min(cnt, sms);
        if (mode == 0) {
          if (tc_mode == GFE_TC_TF32X3) launch_contract_tc<false, true>(tgrid, s, elems + c0, cnt, T, gpbuf, Kel, err);
          else launch_contract_tc<false, false>(tgrid, s, elems + c0, cnt, T, gpbuf, Kel, err);
        } else {
          if (tc_mode == GFE_TC_TF32X3) launch_contract_tc<true, true>(tgrid, s, elems + c0, cnt, T, gpbuf, Kel, err);
          else launch_contract_tc<true, false>(tgrid, s, elems + c0, cnt, T, gpbuf, Kel, err);
        }
        launches += 2;
        continue;
      }
    }
    const int cgrid = std::min(cnt, 8 * sms);
    if (mode == 0)
      mr_contract_kernel<TS, false><<<cgrid, kCThreads, csm, s>>>(elems + c0, cnt, T, gpbuf, Kel);
    else
      mr_contract_kernel<TS, true><<<cgrid, kCThreads, csm, s>>>(elems + c0, cnt, T, gpbuf, Kel);
    launches += 2;
  }
  gfe::scratch_free(gpbuf, s);
  if (values && (rc = gather_rows<TS>(n_elem, elems, eq2, elin, nq2, nlin, Kel, slots, row_ptr, values, s, err))) {
    if (own_kel) gfe::scratch_free(Kel, s);
    return rc;
  }
  if (K_out && own_kel) {
    const size_t n = (size_t)n_elem * ND * ND;
    widen_element_matrices<TS><<<8 * sms, 256, 0, s>>>(Kel, n, K_out);
    ++launches;
  }
  gfe::stage_end(GFE_STAGE_MR_JACOBIAN, prof, s, launches + (values ? 3 : 0));
  if (own_kel) gfe::scratch_free(Kel, s);
  GFE_LAUNCH_CHECK(fn);
  return GFE_OK;
}

int jacobian_entry_point(int mode, int32_t n_elem, const int32_t* eq2, const int32_t* elin, int32_t nq2, int32_t nlin,
                         const double* xg, const int32_t* color_elems, const int32_t* color_ptr_host,
                         int32_t n_colors, const double* dep, const double* cpar, const int32_t* slots,
                         const int32_t* row_ptr, double* values, int64_t nnz, double* K_out, int32_t precision,
                         void* stream, const char* fn) {
  int rc = check_mesh(n_elem, eq2, elin, nq2, nlin, xg, fn);
  if (rc) return rc;
  if (!dep || !cpar || (n_elem > 0 && (!color_elems || !color_ptr_host || n_colors <= 0)))
    return gfe::set_error(GFE_ERR_ARG, "%s: invalid arguments", fn);
  if (!K_out && !values) return gfe::set_error(GFE_ERR_ARG, "%s: need CSR values or K_out", fn);
  if (values && (!slots || !row_ptr || nnz < 0))
    return gfe::set_error(GFE_ERR_ARG, "%s: CSR values need the slot map and row_ptr", fn);
  if (color_ptr_host[0] != 0 || color_ptr_host[n_colors] != n_elem)
    return gfe::set_error(GFE_ERR_ARG, "%s: colour offsets must run from 0 to n_elem", fn);
  if (precision != GFE_FP64 && precision != GFE_MIXED && precision != GFE_TC_TF32X3 && precision != GFE_TC_TF32)
    return gfe::set_error(GFE_ERR_ARG, "%s: precision must be GFE_FP64, GFE_MIXED, GFE_TC_TF32X3 or GFE_TC_TF32", fn);
  cudaStream_t s = gfe::as_stream(stream);
  if (precision == GFE_FP64)
    return jacobian_impl<double>(mode, n_elem, eq2, elin, nq2, nlin, xg, color_elems, dep, cpar, slots, row_ptr,
                                 values, K_out, s, fn);
  return jacobian_impl<float>(mode, n_elem, eq2, elin, nq2, nlin, xg, color_elems, dep, cpar, slots, row_ptr, values,
                              K_out, s, fn, precision == GFE_MIXED ? 0 : precision);
}

}  // namespace

extern "C" int gfe_mr_jacobian(int32_t n_elem, const int32_t* eq2, const int32_t* elin, int32_t nq2, int32_t nlin,
                               const double* xg, const int32_t* color_elems, const int32_t* color_ptr_host,
                               int32_t n_colors, const double* dep, const double* cpar, const int32_t* slots,
                               const int32_t* row_ptr, double* values, int64_t nnz, double* K_out, int32_t precision,
                               void* stream) {
  return jacobian_entry_point(0, n_elem, eq2, elin, nq2, nlin, xg, color_elems, color_ptr_host, n_colors, dep, cpar,
                              slots, row_ptr, values, nnz, K_out, precision, stream, "gfe_mr_jacobian");
}

extern "C" int gfe_mr_tangent(int32_t n_elem, const int32_t* eq2, const int32_t* elin, int32_t nq2, int32_t nlin,
                              const double* xg, const int32_t* color_elems, const int32_t* color_ptr_host,
                              int32_t n_colors, const double* dep, const double* cpar, const int32_t* slots,
                              const int32_t* row_ptr, double* values, int64_t nnz, double* K_out, int32_t precision,
                              void* stream) {
  return jacobian_entry_point(1, n_elem, eq2, elin, nq2, nlin, xg, color_elems, color_ptr_host, n_colors, dep, cpar,
                              slots, row_ptr, values, nnz, K_out, precision, stream, "gfe_mr_tangent");
}

extern "C" int gfe_mr_jacobian_fd(int32_t n_elem, const int32_t* eq2, const int32_t* elin, int32_t nq2,
                                  int32_t nlin, const double* xg, const int32_t* color_elems,
                                  const int32_t* color_ptr_host, int32_t n_colors, const double* dep,
                                  const double* cpar, double step, const int32_t* slots, double* values, int64_t nnz,
                                  double* K_out, void* stream) {
  const char* fn = "gfe_mr_jacobian_fd";
  int rc = check_mesh(n_elem, eq2, elin, nq2, nlin, xg, fn);
  if (rc) return rc;
  if (!dep || !cpar || !(step > 0.0) || (n_elem > 0 && (!color_elems || !color_ptr_host || n_colors <= 0)))
    return gfe::set_error(GFE_ERR_ARG, "%s: invalid arguments", fn);
  if (!K_out && (!slots || !values)) return gfe::set_error(GFE_ERR_ARG, "%s: need CSR values + slots or K_out", fn);
  if (color_ptr_host[0] != 0 || color_ptr_host[n_colors] != n_elem)
    return gfe::set_error(GFE_ERR_ARG, "%s: colour offsets must run from 0 to n_elem", fn);
  const Tables* T = nullptr;
  if ((rc = device_tables(&T))) return rc;
  cudaStream_t s = gfe::as_stream(stream);
  const int64_t ndof = 3ll * nq2 + nlin;
  const size_t sm = sizeof(Tables) + sizeof(FDShared);
  if ((rc = set_smem((const void*)mr_jacobian_fd_kernel, sm))) return rc;
  double* parts = nullptr;
  if ((rc = gfe::scratch_alloc((void**)&parts, sizeof(double) * kNormParts, s, "FD step norm"))) return rc;
  if (values) {
    cudaError_t e = cudaMemsetAsync(values, 0, sizeof(double) * (size_t)nnz, s);
    if (e != cudaSuccess) {
      gfe::scratch_free(parts, s);
      return gfe::set_error(GFE_ERR_CUDA, "%s: %s", fn, cudaGetErrorString(e));
    }
  }
  unsigned* err = gfe::device_error_word();
  void* prof = gfe::stage_begin(GFE_STAGE_MR_JACOBIAN, s);
  sumsq_parts<<<kNormParts, 256, 0, s>>>(dep, ndof, parts);
  int launches = 1;
  for (int c = 0; c < n_colors; ++c) {
    const int c0 = color_ptr_host[c], cnt = color_ptr_host[c + 1] - c0;
    if (cnt <= 0) continue;
    const int grid = std::min(cnt, 8 * gfe::sm_count());
    mr_jacobian_fd_kernel<<<grid, kFDWarps * 32, sm, s>>>(color_elems + c0, cnt, eq2, elin, nq2, xg, dep, cpar, T,
                                                          parts, step, slots, values, K_out, err);
    ++launches;
  }
  gfe::stage_end(GFE_STAGE_MR_JACOBIAN, prof, s, launches);
  gfe::scratch_free(parts, s);
  GFE_LAUNCH_CHECK(fn);
  return GFE_OK;
}

extern "C" int gfe_mr_residual_vjp(int32_t n_elem, const int32_t* eq2, const int32_t* elin, int32_t nq2,
                                   int32_t nlin, const double* xg, const int32_t* color_elems,
                                   const int32_t* color_ptr_host, int32_t n_colors, int32_t batch, const double* dep,
                                   const double* cpar, const double* v, double* du, double* dc, void* stream) {
  const char* fn = "gfe_mr_residual_vjp";
  int rc = check_mesh(n_elem, eq2, elin, nq2, nlin, xg, fn);
  if (rc) return rc;
  if (batch <= 0 || !dep || !cpar || !v || !du || !dc || (n_elem > 0 && (!color_elems || !color_ptr_host)))
    return gfe::set_error(GFE_ERR_ARG, "%s: invalid arguments", fn);
  if (color_ptr_host[0] != 0 || color_ptr_host[n_colors] != n_elem)
    return gfe::set_error(GFE_ERR_ARG, "%s: colour offsets must run from 0 to n_elem", fn);
  const Tables* T = nullptr;
  if ((rc = device_tables(&T))) return rc;
  cudaStream_t s = gfe::as_stream(stream);
  const int64_t ndof = 3ll * nq2 + nlin;
  GFE_CUDA_TRY(cudaMemsetAsync(du, 0, sizeof(double) * ndof * batch, s));
  double* dc_elem = nullptr;
  if ((rc = gfe::scratch_alloc((void**)&dc_elem, sizeof(double) * 2 * (size_t)n_elem * batch, s, "vjp partials")))
    return rc;
  const size_t sm = sizeof(Tables) + kAdjWarps * sizeof(AdjWarpShared);
  if ((rc = set_smem((const void*)mr_vjp_reverse_kernel, sm))) { gfe::scratch_free(dc_elem, s); return rc; }
  unsigned* err = gfe::device_error_word();
  for (int c = 0; c < n_colors; ++c) {
    const int c0 = color_ptr_host[c], cnt = color_ptr_host[c + 1] - c0;
    if (cnt <= 0) continue;
    const long long items = (long long)cnt * batch;
    const int grid = (int)std::min<long long>((items + kAdjWarps - 1) / kAdjWarps, 16ll * gfe::sm_count());
    mr_vjp_reverse_kernel<<<grid, kAdjWarps * 32, sm, s>>>(color_elems + c0, cnt, batch, eq2, elin, nq2, nlin, xg,
                                                           dep, cpar, v, T, du, dc_elem, n_elem, err);
  }
  sum_dc<<<batch, 32, 0, s>>>(dc_elem, n_elem, batch, dc);
  gfe::scratch_free(dc_elem, s);
  GFE_LAUNCH_CHECK(fn);
  return GFE_OK;
}
