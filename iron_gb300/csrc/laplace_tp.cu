// laplace_tp.cu -- Laplace assembly on tensor-product Lagrange hexahedra of any order 1..3.
//
// Iron's Laplace element routine (LaplaceEquation_FiniteElementCalculate,
// src/Laplace_equations_routines.F90:433-747) works for every tensor-product Lagrange basis:
// per Gauss point it interpolates the geometry with first derivatives, forms the metrics
// (COORDINATE_METRICS_CALCULATE, src/coordinate_routines.F90:639-1026: GL = J^T J, GU = GL^-1,
// Jacobian = sqrt|det GL|) and adds
//   K(ms, ns) += sum_{mi,ni} dphi_ms/dxi_mi GU(mi,ni) dphi_ns/dxi_ni * Jacobian * w   (x kappa)
// and EquationsMatrices_ElementAdd / MATRIX_VALUES_ADD_DP2 add it into the CSR matrix.  The
// trilinear case has its own sum-factorised kernels (laplace.cu); this file covers
// (order1+1)(order2+1)(order3+1)-node elements with n1 x n2 x n3 Gauss points:
//  * basis tables (Gauss-Legendre points and weights on [0,1], closed forms for n <= 4 as in
//    Gauss_Legendre src/basis_routines.F90:6804-6890; equally spaced Lagrange polynomials as in
//    LAGRANGE_*_EVALUATE :7969-8090, node and Gauss-point numbering xi1 fastest, :3820) are built
//    on the host once per configuration, in the element arithmetic type;
//  * one CTA per element: Gauss-point threads form M_g = adj(GL) kappa w / sqrt(det GL) (= GU
//    Jacobian w kappa), then pair threads form K(m, n), m <= n, as sum_g dphi_g(m)^T M_g dphi_g(n);
//  * each pair is added at (node m, node n) and (node n, node m) of the CSR values through Iron's
//    row search (bisection to a width of 10, then a linear scan, src/matrix_vector.F90:3202-3240),
//    colour by colour, so no two elements of a launch share a row and the result is deterministic.
#include <algorithm>
#include <array>
#include <cmath>
#include <map>
#include <mutex>
#include <tuple>
#include <type_traits>
#include <vector>

#include "df.cuh"
#include "gfe_internal.cuh"
#include "tcgen05.cuh"

namespace {

constexpr int kTPThreads = 256;
constexpr int kMaxNns = 64;  // (3+1)^3
constexpr int kMaxNg = 64;   // 4^3

// Gauss-Legendre points and weights on [0, 1], n = 1..4 (closed forms of the Legendre roots).
void gauss01(int n, double* x, double* w) {
  switch (n) {
    case 1:
      x[0] = 0.5;
      w[0] = 1.0;
      break;
    case 2: {
      const double d = 0.5 / std::sqrt(3.0);
      x[0] = 0.5 - d; x[1] = 0.5 + d;
      w[0] = w[1] = 0.5;
      break;
    }
    case 3: {
      const double d = 0.5 * std::sqrt(0.6);
      x[0] = 0.5 - d; x[1] = 0.5; x[2] = 0.5 + d;
      w[0] = w[2] = 5.0 / 18.0;
      w[1] = 8.0 / 18.0;
      break;
    }
    default: {  // 4
      const double a = 0.5 * std::sqrt(3.0 / 7.0 - 2.0 / 7.0 * std::sqrt(1.2));
      const double b = 0.5 * std::sqrt(3.0 / 7.0 + 2.0 / 7.0 * std::sqrt(1.2));
      const double wa = (18.0 + std::sqrt(30.0)) / 72.0, wb = (18.0 - std::sqrt(30.0)) / 72.0;
      x[0] = 0.5 - b; x[1] = 0.5 - a; x[2] = 0.5 + a; x[3] = 0.5 + b;
      w[0] = w[3] = wb;
      w[1] = w[2] = wa;
      break;
    }
  }
}

// 1D cubic Hermite function of node a (0 or 1) and node derivative k (0 value, 1 slope) and its
// derivative, at t (the four cubics of HERMITE_CUBIC_EVALUATE, src/basis_routines.F90:7607-7701).
void hermite1d(int a, int k, double t, double* val, double* der) {
  if (a == 0 && k == 0) { *val = (2.0 * t - 3.0) * t * t + 1.0; *der = 6.0 * t * (t - 1.0); }
  else if (a == 0) { *val = ((t - 2.0) * t + 1.0) * t; *der = (3.0 * t - 4.0) * t + 1.0; }
  else if (k == 0) { *val = t * t * (3.0 - 2.0 * t); *der = 6.0 * t * (1.0 - t); }
  else { *val = t * t * (t - 1.0); *der = t * (3.0 * t - 2.0); }
}

// 1D Lagrange polynomial k of order p on the nodes j/p and its derivative, at t.
void lagrange1d(int p, int k, double t, double* val, double* der) {
  double v = 1.0, d = 0.0;
  const double tk = (double)k / p;
  for (int j = 0; j <= p; ++j) {
    if (j == k) continue;
    const double tj = (double)j / p, f = (t - tj) / (tk - tj), df = 1.0 / (tk - tj);
    d = d * f + v * df;  // product rule, accumulated factor by factor
    v *= f;
  }
  *val = v;
  *der = d;
}

// Tetrahedral simplex bases (Iron's interpolation 7 = linear, 8 = quadratic, 9 = cubic): basis
// functions are products over the four area coordinates of factors chosen by the node's position
// index (linear: 1, L; quadratic: 1, 2L, L(2L-1); cubic: 1, 3L, 3/2 L(3L-1), 1/2 L(3L-1)(3L-2)),
// the xi derivatives are d/dL4 - d/dL_i, and the Gauss points are Gauss_Simplex's tetrahedral
// rules of orders 1..5 (1, 4, 5, 11, 14 points; weights sum to 1/6)
// (src/basis_routines.F90:4813-5875, 6041-6270, 6898-7600, 8092-8313).
double simplex_factor(int interp, int pos, bool deriv, double L) {
  if (interp == 7) return pos == 1 ? (deriv ? 0.0 : 1.0) : (deriv ? 1.0 : L);
  if (interp == 9) {
    if (pos == 1) return deriv ? 0.0 : 1.0;
    if (pos == 2) return deriv ? 3.0 : 3.0 * L;
    if (pos == 3) return deriv ? 1.5 * (6.0 * L - 1.0) : 1.5 * L * (3.0 * L - 1.0);
    return deriv ? (13.5 * L - 9.0) * L + 1.0 : 0.5 * L * (3.0 * L - 1.0) * (3.0 * L - 2.0);
  }
  if (pos == 1) return deriv ? 0.0 : 1.0;
  if (pos == 2) return deriv ? 2.0 : 2.0 * L;
  return deriv ? 4.0 * L - 1.0 : L * (2.0 * L - 1.0);
}

// Symmetric point sets of the tetrahedral rules, in Gauss_Simplex's order: `four` = one area
// coordinate (1 + 3a)/4, the others (1 - a)/4, cycled; `six` = two coordinates (1 + 2b)/4 and two
// (1 - 2b)/4 over the six placements.
void simplex_four(double a, double wt, std::vector<std::array<double, 4>>& L, std::vector<double>& w) {
  const double h = (1.0 + 3.0 * a) / 4.0, o = (1.0 - a) / 4.0, r = 1.0 - h - o - o;
  const std::array<double, 4> base = {h, o, o, r};
  for (int s = 0; s < 4; ++s) {
    std::array<double, 4> p;
    for (int k = 0; k < 4; ++k) p[k] = base[(k - s + 4) % 4];
    L.push_back(p);
    w.push_back(wt / 6.0);
  }
}

void simplex_six(double b, double wt, std::vector<std::array<double, 4>>& L, std::vector<double>& w) {
  const double hi = (1.0 + 2.0 * b) / 4.0, lo = (1.0 - 2.0 * b) / 4.0, r = 1.0 - hi - hi - lo;
  // positions of the two large coordinates, in the rule's order
  static const int at[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
  for (int s = 0; s < 6; ++s) {
    std::array<double, 4> p;
    int small = 0;
    for (int k = 0; k < 4; ++k) {
      if (k == at[s][0] || k == at[s][1]) p[k] = hi;
      else p[k] = small++ == 0 ? lo : r;
    }
    L.push_back(p);
    w.push_back(wt / 6.0);
  }
}

void simplex_rule(int order, std::vector<std::array<double, 4>>& L, std::vector<double>& w) {
  if (order == 4) {
    L.push_back({0.25, 0.25, 0.25, 0.25});
    w.push_back(-148.0 / 1875.0 / 6.0);
    simplex_four(5.0 / 7.0, 343.0 / 7500.0, L, w);
    simplex_six(std::sqrt(70.0) / 28.0, 56.0 / 375.0, L, w);
    return;
  }
  if (order == 5) {
    const double two_pi = 6.283185307179586;
    const double lam =
        4.0 / 27.0 * (4.0 * std::sqrt(79.0) * std::cos((std::acos(67.0 * std::sqrt(79.0) / 24964.0) + two_pi) / 3.0) + 71.0);
    const double disc = std::sqrt(9.0 * lam * lam - 248.0 * lam + 1680.0), den = 112.0 - 10.0 * lam;
    const double a1 = (disc + 28.0 - 3.0 * lam) / den, a2 = (28.0 - 3.0 * lam - disc) / den;
    simplex_four(a1, ((21.0 - lam) * a2 - 7.0) / (420.0 * a1 * a1 * (a2 - a1)), L, w);
    simplex_four(a2, ((21.0 - lam) * a1 - 7.0) / (420.0 * a2 * a2 * (a1 - a2)), L, w);
    simplex_six(1.0 / std::sqrt(lam), lam * lam / 840.0, L, w);
    return;
  }
  if (order == 1) {
    L.push_back({0.25, 0.25, 0.25, 0.25});
    w.push_back(1.0 / 6.0);
    return;
  }
  const double a = order == 2 ? 1.0 / std::sqrt(5.0) : 1.0 / 3.0;
  const double wa = order == 2 ? 0.25 : 9.0 / 20.0;
  const double l1 = (1.0 + 3.0 * a) / 4.0, l2 = (1.0 - a) / 4.0, l3 = (1.0 - a) / 4.0, l4 = 1.0 - l1 - l2 - l3;
  if (order == 3) {
    L.push_back({0.25, 0.25, 0.25, 0.25});
    w.push_back(-4.0 / 5.0 / 6.0);
  }
  L.push_back({l1, l2, l3, l4});
  L.push_back({l4, l1, l2, l3});
  L.push_back({l3, l4, l1, l2});
  L.push_back({l2, l3, l4, l1});
  for (int k = 0; k < 4; ++k) w.push_back(wa / 6.0);
}

template <typename T>
T to_elem(double v);
template <>
double to_elem<double>(double v) { return v; }
template <>
float to_elem<float>(double v) { return (float)v; }
template <>
f2 to_elem<f2>(double v) {
  const float h = (float)v;
  return {h, (float)(v - (double)h)};
}

struct TPConfig {
  int nns, ng, npairs;
};

template <typename T>
struct TPTables {
  T* dphi = nullptr;       // [ng][3][nns]
  T* w = nullptr;          // [ng]
  int32_t* pairs = nullptr;  // [npairs]: m | n << 16, m <= n
  TPConfig cfg{};
};

std::mutex g_tp_mu;

using TPKey = std::tuple<int, int, int, int, int, int, int>;

// copy one configuration's tables to the device and cache them (caller holds g_tp_mu)
template <typename T>
int upload_tables(const TPKey& key, std::map<TPKey, TPTables<T>>& cache, int nns, int ng, const std::vector<T>& dphi,
                  const std::vector<T>& w, const TPTables<T>** out) {
  std::vector<int32_t> pairs;
  for (int m = 0; m < nns; ++m)
    for (int n = m; n < nns; ++n) pairs.push_back(m | (n << 16));
  TPTables<T> t;
  t.cfg = {nns, ng, (int)pairs.size()};
  GFE_CUDA_TRY(cudaMalloc(&t.dphi, sizeof(T) * dphi.size()));
  GFE_CUDA_TRY(cudaMalloc(&t.w, sizeof(T) * w.size()));
  GFE_CUDA_TRY(cudaMalloc(&t.pairs, sizeof(int32_t) * pairs.size()));
  GFE_CUDA_TRY(cudaMemcpy(t.dphi, dphi.data(), sizeof(T) * dphi.size(), cudaMemcpyHostToDevice));
  GFE_CUDA_TRY(cudaMemcpy(t.w, w.data(), sizeof(T) * w.size(), cudaMemcpyHostToDevice));
  GFE_CUDA_TRY(cudaMemcpy(t.pairs, pairs.data(), sizeof(int32_t) * pairs.size(), cudaMemcpyHostToDevice));
  *out = &(cache[key] = t);
  return GFE_OK;
}

template <typename T>
int tp_tables(const int32_t* order, const int32_t* ngauss, const TPTables<T>** out) {
  static std::map<TPKey, TPTables<T>> cache;
  int dev = 0;
  GFE_CUDA_TRY(cudaGetDevice(&dev));
  const auto key = std::make_tuple(dev, order[0], order[1], order[2], ngauss[0], ngauss[1], ngauss[2]);
  std::lock_guard<std::mutex> lk(g_tp_mu);
  auto it = cache.find(key);
  if (it != cache.end()) {
    *out = &it->second;
    return GFE_OK;
  }
  if (order[0] == 7 || order[0] == 8 || order[0] == 9) {
    static const int lin[4][4] = {{2, 1, 1, 1}, {1, 2, 1, 1}, {1, 1, 2, 1}, {1, 1, 1, 2}};
    static const int quad[10][4] = {{3, 1, 1, 1}, {1, 3, 1, 1}, {1, 1, 3, 1}, {1, 1, 1, 3}, {2, 2, 1, 1},
                                    {2, 1, 2, 1}, {2, 1, 1, 2}, {1, 2, 2, 1}, {1, 1, 2, 2}, {1, 2, 1, 2}};
    // cubic: vertices, the two nodes of each edge (nearer the first vertex first), the face nodes
    static const int cub[20][4] = {{4, 1, 1, 1}, {1, 4, 1, 1}, {1, 1, 4, 1}, {1, 1, 1, 4}, {3, 2, 1, 1},
                                   {2, 3, 1, 1}, {3, 1, 2, 1}, {2, 1, 3, 1}, {3, 1, 1, 2}, {2, 1, 1, 3},
                                   {1, 3, 2, 1}, {1, 2, 3, 1}, {1, 1, 3, 2}, {1, 1, 2, 3}, {1, 3, 1, 2},
                                   {1, 2, 1, 3}, {2, 2, 2, 1}, {2, 2, 1, 2}, {2, 1, 2, 2}, {1, 2, 2, 2}};
    std::vector<std::array<double, 4>> gl;
    std::vector<double> gw;
    simplex_rule(ngauss[0], gl, gw);
    const int nns = order[0] == 7 ? 4 : (order[0] == 8 ? 10 : 20), ng = (int)gl.size();
    std::vector<T> dphi((size_t)ng * 3 * nns), w(ng);
    for (int g = 0; g < ng; ++g) {
      w[g] = to_elem<T>(gw[g]);
      for (int n = 0; n < nns; ++n) {
        const int* pos = order[0] == 7 ? lin[n] : (order[0] == 8 ? quad[n] : cub[n]);
        double dL[4];
        for (int k = 0; k < 4; ++k) {
          double d = 1.0;
          for (int j = 0; j < 4; ++j) d *= simplex_factor(order[0], pos[j], j == k, gl[g][j]);
          dL[k] = d;
        }
        for (int a = 0; a < 3; ++a) dphi[((size_t)g * 3 + a) * nns + n] = to_elem<T>(dL[3] - dL[a]);
      }
    }
    return upload_tables<T>(key, cache, nns, ng, dphi, w, out);
  }
  // element parameters in Iron's order: local nodes xi1 fastest, then each node's derivatives,
  // whose count doubles for every Hermite direction in xi order (src/basis_routines.F90:2633-2662)
  int nn[3], nder = 1;
  for (int d = 0; d < 3; ++d) {
    nn[d] = order[d] == 4 ? 2 : order[d] + 1;
    if (order[d] == 4) nder *= 2;
  }
  std::vector<std::array<int, 6>> par;  // node position and node derivative per direction
  for (int a3 = 0; a3 < nn[2]; ++a3)
    for (int a2 = 0; a2 < nn[1]; ++a2)
      for (int a1 = 0; a1 < nn[0]; ++a1)
        for (int k = 0; k < nder; ++k) {
          std::array<int, 6> q = {a1, a2, a3, 0, 0, 0};
          int bit = 0;
          for (int d = 0; d < 3; ++d)
            if (order[d] == 4) q[3 + d] = (k >> bit++) & 1;
          par.push_back(q);
        }
  const int nns = (int)par.size(), ng = ngauss[0] * ngauss[1] * ngauss[2];
  double gx[3][4], gw[3][4];
  for (int d = 0; d < 3; ++d) gauss01(ngauss[d], gx[d], gw[d]);
  std::vector<T> dphi((size_t)ng * 3 * nns), w(ng);
  for (int g3 = 0; g3 < ngauss[2]; ++g3)
    for (int g2 = 0; g2 < ngauss[1]; ++g2)
      for (int g1 = 0; g1 < ngauss[0]; ++g1) {
        const int g = g1 + ngauss[0] * (g2 + ngauss[1] * g3);
        const double t[3] = {gx[0][g1], gx[1][g2], gx[2][g3]};
        w[g] = to_elem<T>(gw[0][g1] * gw[1][g2] * gw[2][g3]);
        for (int n = 0; n < nns; ++n) {
          double v[3], dv[3];
          for (int d = 0; d < 3; ++d) {
            if (order[d] == 4) hermite1d(par[n][d], par[n][3 + d], t[d], &v[d], &dv[d]);
            else lagrange1d(order[d], par[n][d], t[d], &v[d], &dv[d]);
          }
          dphi[((size_t)g * 3 + 0) * nns + n] = to_elem<T>(dv[0] * v[1] * v[2]);
          dphi[((size_t)g * 3 + 1) * nns + n] = to_elem<T>(v[0] * dv[1] * v[2]);
          dphi[((size_t)g * 3 + 2) * nns + n] = to_elem<T>(v[0] * v[1] * dv[2]);
        }
      }
  return upload_tables<T>(key, cache, nns, ng, dphi, w, out);
}

// Iron's CSR search (MATRIX_VALUES_ADD_DP2): bisection until at most 10 candidates, then a
// linear scan.  0-based position, or -1 if the column is absent.
__device__ __forceinline__ long long csr_find(const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                             int row, int col1) {
  long long lo = (long long)rp[row] - 1, hi = (long long)rp[row + 1] - 1;
  while (hi - lo > 10) {
    const long long mid = lo + (hi - lo) / 2;
    if (ci[mid] > col1) hi = mid; else lo = mid;
  }
  for (long long k = lo; k < hi; ++k)
    if (ci[k] == col1) return k;
  return -1;
}

// CSR position of element entry (m, n): from the element slot map slots[e][m][n] when given (Iron's
// search above, run once per mesh by gfe_laplace_tp_slot_map), else by the search itself.  The
// search is a chain of dependent loads per entry; for 27- to 64-node elements it dominated the
// assembly.
__device__ __forceinline__ long long entry_pos(const int32_t* __restrict__ slots, int e, int nns, int m, int n,
                                               const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                               int row, int col1) {
  if (slots) return (long long)__ldg(slots + ((size_t)e * nns + m) * nns + n);
  return csr_find(rp, ci, row, col1);
}

// Element pairs a thread scatters at a time.  Their positions, then their CSR values, are loaded
// before any value is written (the entries of one colour's elements are distinct), so a thread
// keeps several loads in flight instead of one dependent position -> value -> store chain a pair.
constexpr int kTPScatter = 4;

// Pairs t = t0, t0 + stride, ... (below total): at(t, v, pmn, pnm) gives the value and its two CSR
// positions (pnm = -2 for a diagonal pair, -1 for an absent entry).
template <typename PairAt>
__device__ __forceinline__ void scatter_batch(int t0, int stride, int total, PairAt at, double* __restrict__ values,
                                              unsigned* err) {
  long long pos[kTPScatter][2];
  double v[kTPScatter];
#pragma unroll
  for (int u = 0; u < kTPScatter; ++u) {
    const int t = t0 + u * stride;
    pos[u][0] = pos[u][1] = -2;  // nothing to add
    v[u] = 0.0;
    if (t < total) at(t, v[u], pos[u][0], pos[u][1]);
  }
  double old[kTPScatter][2];
#pragma unroll
  for (int u = 0; u < kTPScatter; ++u)
#pragma unroll
    for (int h = 0; h < 2; ++h) old[u][h] = pos[u][h] >= 0 ? values[pos[u][h]] : 0.0;
#pragma unroll
  for (int u = 0; u < kTPScatter; ++u)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      if (pos[u][h] >= 0) values[pos[u][h]] = old[u][h] + v[u];
      else if (pos[u][h] == -1) gfe_raise(err, GFE_DEVERR_SLOT);
    }
}

__global__ void tp_slot_kernel(int32_t n_elem, int32_t nns, const int32_t* __restrict__ en,
                               const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                               int32_t* __restrict__ slots) {
  const long long per = (long long)nns * nns, total = (long long)n_elem * per;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const long long e = t / per;
    const int r = (int)(t - e * per), m = r / nns, n = r % nns;
    slots[t] = (int32_t)csr_find(rp, ci, en[e * nns + m], en[e * nns + n] + 1);
  }
}

template <typename T>
__device__ __forceinline__ T tp_rsqrt(T a) {
  return rsqrt(a);
}
template <>
__device__ __forceinline__ float tp_rsqrt<float>(float a) {
  return rsqrtf(a);
}

// Element group of GROUP threads: GROUP = kTPThreads gives one element a block (triquadratic,
// tricubic and Hermite elements: up to 64 nodes, 2,080 entry pairs); GROUP = 32 gives one element
// a warp, eight a block (elements of at most kSmallNns nodes and kSmallNg Gauss points: linear and
// quadratic tetrahedra, trilinear hexahedra with other rules), whose few pairs would otherwise
// leave most of a block idle at every barrier.
constexpr int kSmallNns = 10, kSmallNg = 32;

template <int GROUP>
__device__ __forceinline__ void group_sync() {
  if constexpr (GROUP == kTPThreads) __syncthreads();
  else __syncwarp();
}

template <typename T, int GROUP, int MAXN, int MAXG>
__global__ void __launch_bounds__(kTPThreads)
laplace_tp_kernel(const int32_t* __restrict__ ce, int32_t cnt, int32_t n_nodes, const int32_t* __restrict__ en,
                  const double* __restrict__ coords, const double* __restrict__ scale,
                  const double* __restrict__ kappa, const T* __restrict__ dphi,
                  const T* __restrict__ wg, const int32_t* __restrict__ pairs, TPConfig cfg,
                  const int32_t* __restrict__ rp, const int32_t* __restrict__ ci, const int32_t* __restrict__ slots,
                  double* __restrict__ values, unsigned* err) {
  static_assert(GROUP == kTPThreads || GROUP == 32, "an element takes a block or a warp");
  constexpr int EPB = kTPThreads / GROUP;
  __shared__ T sx_all[EPB][3][MAXN];
  __shared__ T sM_all[EPB][MAXG][6];
  __shared__ int32_t snode_all[EPB][MAXN];
  __shared__ double ssf_all[EPB][MAXN];
  __shared__ T sJ_all[EPB][MAXG][9];
  const int sub = threadIdx.x % GROUP, grp = threadIdx.x / GROUP;
  T (*sJ)[9] = sJ_all[grp];
  T (*sx)[MAXN] = sx_all[grp];
  T (*sM)[6] = sM_all[grp];
  int32_t* snode = snode_all[grp];
  double* ssf = ssf_all[grp];
  const int nns = cfg.nns, ng = cfg.ng;
  // the item loop is uniform over a group (a block or a warp), so the group barriers below match
  for (int item = blockIdx.x * EPB + grp; item < cnt; item += gridDim.x * EPB) {
    const int e = ce[item];
    for (int n = sub; n < nns; n += GROUP) {
      const int node = en[(size_t)e * nns + n];
      snode[n] = node;
      // scaled geometric parameters, as FIELD_INTERPOLATION_PARAMETERS_ELEMENT_GET forms them
      const double sf = scale ? scale[(size_t)e * nns + n] : 1.0;
      if (scale) ssf[n] = sf;
#pragma unroll
      for (int c = 0; c < 3; ++c) sx[c][n] = from_double<T>(coords[(size_t)c * n_nodes + node] * sf);
    }
    const double kd = kappa ? kappa[e] : 1.0;
    if (!isfinite(kd)) gfe_raise(err, GFE_DEVERR_NONFINITE);
    const T kap = from_double<T>(kd);
    group_sync<GROUP>();
    // the 9 ng Jacobian entries dx_c/dxi_a spread over the group's lanes, then one lane a Gauss
    // point for the metric: a lane per Gauss point alone leaves most lanes idle through the
    // longest part (ng of GROUP lanes active)
    for (int q = sub; q < 9 * ng; q += GROUP) {
      const int g = q / 9, c = (q % 9) / 3, a = q % 3;
      T s = from_double<T>(0.0);
      for (int n = 0; n < nns; ++n) s = s + sx[c][n] * dphi[((size_t)g * 3 + a) * nns + n];
      sJ[g][q % 9] = s;
    }
    group_sync<GROUP>();
    for (int g = sub; g < ng; g += GROUP) {
      T J[3][3];
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int a = 0; a < 3; ++a) J[c][a] = sJ[g][c * 3 + a];
      const T G00 = J[0][0] * J[0][0] + J[1][0] * J[1][0] + J[2][0] * J[2][0];
      const T G11 = J[0][1] * J[0][1] + J[1][1] * J[1][1] + J[2][1] * J[2][1];
      const T G22 = J[0][2] * J[0][2] + J[1][2] * J[1][2] + J[2][2] * J[2][2];
      const T G01 = J[0][0] * J[0][1] + J[1][0] * J[1][1] + J[2][0] * J[2][1];
      const T G02 = J[0][0] * J[0][2] + J[1][0] * J[1][2] + J[2][0] * J[2][2];
      const T G12 = J[0][1] * J[0][2] + J[1][1] * J[1][2] + J[2][1] * J[2][2];
      const T A00 = G11 * G22 - G12 * G12, A11 = G00 * G22 - G02 * G02, A22 = G00 * G11 - G01 * G01;
      const T A01 = G02 * G12 - G01 * G22, A02 = G01 * G12 - G02 * G11, A12 = G01 * G02 - G00 * G12;
      const T det = G00 * A00 + G01 * A01 + G02 * A02;
      if (!(det > from_double<T>(0.0))) gfe_raise(err, GFE_DEVERR_JACOBIAN);
      // GU * Jacobian * w * kappa = adj(GL) / det * sqrt(det) * w * kappa
      const T sc = kap * wg[g] * tp_rsqrt(det);
      sM[g][0] = A00 * sc; sM[g][1] = A11 * sc; sM[g][2] = A22 * sc;
      sM[g][3] = A01 * sc; sM[g][4] = A02 * sc; sM[g][5] = A12 * sc;
    }
    group_sync<GROUP>();
    using Acc = typename std::conditional<std::is_same<T, double>::value, double, f2>::type;
    for (int p = sub; p < cfg.npairs; p += GROUP) {
      const int32_t mn = pairs[p];
      const int m = mn & 0xffff, n = mn >> 16;
      Acc acc = from_double<Acc>(0.0);
      for (int g = 0; g < ng; ++g) {
        const T* dg = dphi + (size_t)g * 3 * nns;
        const T am0 = dg[m], am1 = dg[nns + m], am2 = dg[2 * nns + m];
        const T an0 = dg[n], an1 = dg[nns + n], an2 = dg[2 * nns + n];
        // (M an)_a, then dm . (M an)
        const T b0 = sM[g][0] * an0 + sM[g][3] * an1 + sM[g][4] * an2;
        const T b1 = sM[g][3] * an0 + sM[g][1] * an1 + sM[g][5] * an2;
        const T b2 = sM[g][4] * an0 + sM[g][5] * an1 + sM[g][2] * an2;
        const T t = am0 * b0 + am1 * b1 + am2 * b2;
        if constexpr (std::is_same<T, float>::value) accum(acc, f2{t, 0.0f});
        else accum(acc, t);
      }
      finish(acc);
      double v = to_double(acc);
      if (scale) v = v * ssf[m] * ssf[n];  // K(ms, ns) * SF(ms) * SF(ns)
      // (staging the pair values and scattering them in batches, as the tensor-core kernel does,
      // was slower here: its shared array costs resident blocks, and the Gauss loop of the other
      // warps already hides the scatter's latency)
      const int rm = snode[m], rn = snode[n];
      const long long pmn = entry_pos(slots, e, nns, m, n, rp, ci, rm, rn + 1);
      if (pmn < 0) gfe_raise(err, GFE_DEVERR_SLOT);
      else values[pmn] += v;
      if (m != n) {
        const long long pnm = entry_pos(slots, e, nns, n, m, rp, ci, rn, rm + 1);
        if (pnm < 0) gfe_raise(err, GFE_DEVERR_SLOT);
        else values[pnm] += v;
      }
    }
    group_sync<GROUP>();
  }
}

// Linear tetrahedra, one element a thread.  GB300's FP64 pipe charges a warp instruction in full
// however few lanes it has active, so the warp-per-element path, whose Gauss-point phase runs on
// ng lanes and pair phase on 10, leaves the pipe mostly idle for a 4-node element; here every lane
// computes a whole element.  Same arithmetic, in the same order, as laplace_tp_kernel.
template <typename T>
__global__ void __launch_bounds__(kTPThreads)
laplace_tet4_kernel(const int32_t* __restrict__ ce, int32_t cnt, int32_t n_nodes, const int32_t* __restrict__ en,
                    const double* __restrict__ coords, const double* __restrict__ kappa,
                    const T* __restrict__ dphi, const T* __restrict__ wg, int ng, const int32_t* __restrict__ rp,
                    const int32_t* __restrict__ ci, double* __restrict__ values, unsigned* err) {
  using Acc = typename std::conditional<std::is_same<T, double>::value, double, f2>::type;
  for (int item = blockIdx.x * blockDim.x + threadIdx.x; item < cnt; item += gridDim.x * blockDim.x) {
    const int e = ce[item];
    int node[4];
    T x[3][4];
#pragma unroll
    for (int n = 0; n < 4; ++n) {
      node[n] = en[(size_t)e * 4 + n];
#pragma unroll
      for (int c = 0; c < 3; ++c) x[c][n] = from_double<T>(coords[(size_t)c * n_nodes + node[n]]);
    }
    const double kd = kappa ? kappa[e] : 1.0;
    if (!isfinite(kd)) gfe_raise(err, GFE_DEVERR_NONFINITE);
    const T kap = from_double<T>(kd);
    Acc K[10];
#pragma unroll
    for (int p = 0; p < 10; ++p) K[p] = from_double<Acc>(0.0);
    for (int g = 0; g < ng; ++g) {
      const T* dg = dphi + (size_t)g * 12;
      T J[3][3];
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          T s = from_double<T>(0.0);
#pragma unroll
          for (int n = 0; n < 4; ++n) s = s + x[c][n] * dg[a * 4 + n];
          J[c][a] = s;
        }
      const T G00 = J[0][0] * J[0][0] + J[1][0] * J[1][0] + J[2][0] * J[2][0];
      const T G11 = J[0][1] * J[0][1] + J[1][1] * J[1][1] + J[2][1] * J[2][1];
      const T G22 = J[0][2] * J[0][2] + J[1][2] * J[1][2] + J[2][2] * J[2][2];
      const T G01 = J[0][0] * J[0][1] + J[1][0] * J[1][1] + J[2][0] * J[2][1];
      const T G02 = J[0][0] * J[0][2] + J[1][0] * J[1][2] + J[2][0] * J[2][2];
      const T G12 = J[0][1] * J[0][2] + J[1][1] * J[1][2] + J[2][1] * J[2][2];
      const T A00 = G11 * G22 - G12 * G12, A11 = G00 * G22 - G02 * G02, A22 = G00 * G11 - G01 * G01;
      const T A01 = G02 * G12 - G01 * G22, A02 = G01 * G12 - G02 * G11, A12 = G01 * G02 - G00 * G12;
      const T det = G00 * A00 + G01 * A01 + G02 * A02;
      if (!(det > from_double<T>(0.0))) gfe_raise(err, GFE_DEVERR_JACOBIAN);
      const T sc = kap * wg[g] * tp_rsqrt(det);
      const T M0 = A00 * sc, M1 = A11 * sc, M2 = A22 * sc, M3 = A01 * sc, M4 = A02 * sc, M5 = A12 * sc;
      int p = 0;
#pragma unroll
      for (int m = 0; m < 4; ++m)
#pragma unroll
        for (int n = m; n < 4; ++n, ++p) {
          const T am0 = dg[m], am1 = dg[4 + m], am2 = dg[8 + m];
          const T an0 = dg[n], an1 = dg[4 + n], an2 = dg[8 + n];
          const T b0 = M0 * an0 + M3 * an1 + M4 * an2;
          const T b1 = M3 * an0 + M1 * an1 + M5 * an2;
          const T b2 = M4 * an0 + M5 * an1 + M2 * an2;
          const T t = am0 * b0 + am1 * b1 + am2 * b2;
          if constexpr (std::is_same<T, float>::value) accum(K[p], f2{t, 0.0f});
          else accum(K[p], t);
        }
    }
    int p = 0;
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
      for (int n = m; n < 4; ++n, ++p) {
        finish(K[p]);
        const double v = to_double(K[p]);
        const long long pmn = csr_find(rp, ci, node[m], node[n] + 1);
        if (pmn < 0) gfe_raise(err, GFE_DEVERR_SLOT);
        else values[pmn] += v;
        if (m != n) {
          const long long pnm = csr_find(rp, ci, node[n], node[m] + 1);
          if (pnm < 0) gfe_raise(err, GFE_DEVERR_SLOT);
          else values[pnm] += v;
        }
      }
  }
}

// ---------------------------------------------------------------------------------------------
// Tensor-core (tcgen05, TF32 x 3) element matrices of tensor-product hexahedra
// ---------------------------------------------------------------------------------------------
// Per element K(m, n) = sum_{g,i} C[n][(g,i)] dphi_g(i, m), C[n][(g,i)] = sum_j M_g(i, j) dphi_g(j, n),
// with M_g = GU Jacobian w kappa the symmetric Gauss-point metric of laplace_tp_kernel.  A tile stacks
// EPT = 128 / R elements (R = 32 rows for up to 32 nodes, 64 for up to 64), so one M = 128 product
// serves EPT elements: A = the stacked C, formed on the CUDA cores in FP32 and split into a TF32 head
// and tail; B[m][(g,i)] = dphi_g(i, m), the basis table (constant, K-major); N = R.  K = 3 ng runs in
// chunks through one A buffer and accumulates in tensor memory (three TF32 products a step,
// head x head + tail x head + head x tail: about FP32 accuracy).  The element pairs m <= n take
// D[(e, n)][m] and are added at (m, n) and (n, m) through the slot map or Iron's row search, colour
// by colour, as in laplace_tp_kernel.
constexpr int kTPKMax = 3 * kMaxNg;             // 192
constexpr uint32_t kTPWaitPolls = 1u << 24;     // bounded mbarrier wait

// Shape of the kernel for R rows an element: elements of up to 64 nodes take one CTA of 512
// threads an SM (16 warps: every phase is bound by load latency) and 64-column K chunks; elements
// of up to 32 nodes take two CTAs of 256 threads an SM with 32-column chunks (about 100 KB of
// shared memory each), so one CTA's barriers and MMA waits overlap the other's work.
template <int R>
struct TPTCShape {
  static constexpr int kThreads = R == 64 ? 512 : 256;  // 1,024 for 64 rows: 1-2 % faster, with spills
  static constexpr int kBlocksPerSM = R == 64 ? 1 : 2;
  static constexpr int kKChunk = R == 64 ? 64 : 32;  // K columns of A per chunk
  static constexpr int kEPT = 128 / R;               // elements a tile
  static constexpr int kDRow = R + 1;                // padded row of the staged product
};

template <int R>
struct __align__(128) TPTCShared {
  using Sh = TPTCShape<R>;
  unsigned char B[2][R * kTPKMax * 4];          // basis head, tail: [m][(g,i)], K-major core matrices
  unsigned char A[2][128 * Sh::kKChunk * 4];    // C head, tail of the current K chunk; then the product
  float sx[Sh::kEPT][3][R];
  float sJ[Sh::kEPT][kMaxNg][9];
  float sM[Sh::kEPT][kMaxNg][6];
  double ssf[Sh::kEPT][R];
  int32_t snode[Sh::kEPT][R];
  int32_t elem[Sh::kEPT];
  float kap[Sh::kEPT];
  uint64_t mbar;
  uint32_t tmem;
  int abort;
};
static_assert(sizeof(float) * 128 * TPTCShape<64>::kDRow <= sizeof(TPTCShared<64>::A), "product staged in A");
static_assert(sizeof(float) * 128 * TPTCShape<32>::kDRow <= sizeof(TPTCShared<32>::A), "product staged in A");
static_assert(2 * (sizeof(TPTCShared<32>) + 1024) <= 228 * 1024, "two CTAs an SM for up to 32 nodes");

template <int R>
__global__ void __launch_bounds__(TPTCShape<R>::kThreads, TPTCShape<R>::kBlocksPerSM)
laplace_tp_tc_kernel(const int32_t* __restrict__ ce, int32_t cnt, int32_t n_nodes, const int32_t* __restrict__ en,
                     const double* __restrict__ coords, const double* __restrict__ scale,
                     const double* __restrict__ kappa, const float* __restrict__ dphi, const float* __restrict__ wg,
                     const int32_t* __restrict__ pairs, TPConfig cfg, const int32_t* __restrict__ rp,
                     const int32_t* __restrict__ ci, const int32_t* __restrict__ slots, double* __restrict__ values,
                     unsigned* err) {
  static_assert(R == 32 || R == 64, "32 or 64 rows an element");
  using Sh = TPTCShape<R>;
  constexpr int EPT = Sh::kEPT, KCH = Sh::kKChunk;
  extern __shared__ __align__(1024) unsigned char tpraw[];
  TPTCShared<R>& S = *reinterpret_cast<TPTCShared<R>*>(tpraw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nns = cfg.nns, ng = cfg.ng, kd = 3 * ng;
  const int KP = (kd + 7) & ~7, KCB = KP / 4;  // K padded to whole MMA steps; B's core columns
  // B head / tail: row m, column (g, i) -> core matrix (m / 8, k / 4)
  for (int t = tid; t < R * KP; t += blockDim.x) {
    const int m = t / KP, k = t % KP;
    const float v = (m < nns && k < kd) ? dphi[(size_t)k * nns + m] : 0.0f;  // dphi[(g*3+i)*nns + m]
    const uint32_t off = (uint32_t)((((m >> 3) * KCB + (k >> 2)) * 8 + (m & 7)) * 16 + (k & 3) * 4);
    const float hi = tc::to_tf32(v);
    *reinterpret_cast<float*>(S.B[0] + off) = hi;
    *reinterpret_cast<float*>(S.B[1] + off) = tc::to_tf32(v - hi);
  }
  if (warp == 0) tc::tmem_alloc(&S.tmem, R);
  if (tid == 0) {
    tc::mbar_init(&S.mbar, 1);
    S.abort = 0;
  }
  tc::fence_proxy_async();  // B is read by the tensor cores
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = S.tmem;
  constexpr uint32_t idesc = tc::idesc_tf32(128, R);
  const uint32_t a_hi = tc::smem_u32(S.A[0]), a_lo = tc::smem_u32(S.A[1]);
  const uint32_t b_hi = tc::smem_u32(S.B[0]), b_lo = tc::smem_u32(S.B[1]);
  constexpr uint32_t kLbo = 128, kSboA = (KCH / 4) * 128;
  const uint32_t sbo_b = (uint32_t)KCB * 128;
  float (*D)[Sh::kDRow] = reinterpret_cast<float (*)[Sh::kDRow]>(S.A[0]);
  uint32_t parity = 0;
  bool bad = false, nonfinite = false;

  const int tiles = (cnt + EPT - 1) / EPT;
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const int item0 = tile * EPT;
    const int live_slots = min(EPT, cnt - item0);
    // element data of the tile's slots (geometry scaled as FIELD_INTERPOLATION_PARAMETERS_ELEMENT_GET)
    for (int t = tid; t < live_slots * nns; t += blockDim.x) {
      const int k = t / nns, n = t % nns;
      const int e = ce[item0 + k];
      const int node = en[(size_t)e * nns + n];
      S.snode[k][n] = node;
      const double sf = scale ? scale[(size_t)e * nns + n] : 1.0;
      S.ssf[k][n] = sf;
#pragma unroll
      for (int c = 0; c < 3; ++c) S.sx[k][c][n] = (float)(coords[(size_t)c * n_nodes + node] * sf);
    }
    if (tid < live_slots) {
      S.elem[tid] = ce[item0 + tid];
      const double kv = kappa ? kappa[ce[item0 + tid]] : 1.0;
      if (!isfinite(kv)) nonfinite = true;
      S.kap[tid] = (float)kv;
    }
    __syncthreads();
    for (int q = tid; q < live_slots * ng * 9; q += blockDim.x) {
      const int k = q / (ng * 9), r = q % (ng * 9), g = r / 9, c = (r % 9) / 3, a = r % 3;
      const float* dg = dphi + ((size_t)g * 3 + a) * nns;
      float sacc = 0.0f;
      for (int n = 0; n < nns; ++n) sacc += S.sx[k][c][n] * dg[n];
      S.sJ[k][g][r % 9] = sacc;
    }
    __syncthreads();
    for (int q = tid; q < live_slots * ng; q += blockDim.x) {
      const int k = q / ng, g = q % ng;
      float J[3][3];
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int a = 0; a < 3; ++a) J[c][a] = S.sJ[k][g][c * 3 + a];
      const float G00 = J[0][0] * J[0][0] + J[1][0] * J[1][0] + J[2][0] * J[2][0];
      const float G11 = J[0][1] * J[0][1] + J[1][1] * J[1][1] + J[2][1] * J[2][1];
      const float G22 = J[0][2] * J[0][2] + J[1][2] * J[1][2] + J[2][2] * J[2][2];
      const float G01 = J[0][0] * J[0][1] + J[1][0] * J[1][1] + J[2][0] * J[2][1];
      const float G02 = J[0][0] * J[0][2] + J[1][0] * J[1][2] + J[2][0] * J[2][2];
      const float G12 = J[0][1] * J[0][2] + J[1][1] * J[1][2] + J[2][1] * J[2][2];
      const float A00 = G11 * G22 - G12 * G12, A11 = G00 * G22 - G02 * G02, A22 = G00 * G11 - G01 * G01;
      const float A01 = G02 * G12 - G01 * G22, A02 = G01 * G12 - G02 * G11, A12 = G01 * G02 - G00 * G12;
      const float det = G00 * A00 + G01 * A01 + G02 * A02;
      if (!(det > 0.0f)) bad = true;
      const float sc = S.kap[k] * wg[g] * rsqrtf(det);
      float* M = S.sM[k][g];
      M[0] = A00 * sc; M[1] = A11 * sc; M[2] = A22 * sc; M[3] = A01 * sc; M[4] = A02 * sc; M[5] = A12 * sc;
    }
    __syncthreads();
    // the product, one K chunk at a time: warp w forms the 8-row groups w and w + 8 of A, lane l its
    // row 8 rg + l / 4 and the K column 4 kc + l % 4 of each core matrix (one 128-byte store a step)
    for (int c0 = 0; c0 < KP; c0 += KCH) {
      const int kcn = min(KCH, KP - c0) / 4;  // core columns of this chunk (even)
      // with 16 or more warps, warp w takes the core columns w / 16, w / 16 + NW / 16, ... of the
      // 8-row group w % 16; with fewer, whole groups w, w + NW, ...
      constexpr int NW = Sh::kThreads / 32, GW = NW >= 16 ? NW / 16 : 1;
      for (int rg = NW >= 16 ? warp % 16 : warp; rg < 16; rg += NW >= 16 ? 16 : NW) {
        const int row = rg * 8 + (lane >> 2), k = row / R, n = row % R;
        const bool live = k < live_slots && n < nns;
        for (int kc = NW >= 16 ? warp / 16 : 0; kc < kcn; kc += GW) {
          const int kk = c0 + kc * 4 + (lane & 3);
          float v = 0.0f;
          if (live && kk < kd) {
            const int g = kk / 3, i = kk - 3 * g;
            const float* M = S.sM[k][g];
            // M(i, j) in the packed order 00 11 22 01 02 12
            const float mi0 = i == 0 ? M[0] : (i == 1 ? M[3] : M[4]);
            const float mi1 = i == 0 ? M[3] : (i == 1 ? M[1] : M[5]);
            const float mi2 = i == 0 ? M[4] : (i == 1 ? M[5] : M[2]);
            const float* dg = dphi + (size_t)g * 3 * nns + n;
            v = mi0 * dg[0] + mi1 * dg[nns] + mi2 * dg[2 * nns];
          }
          const float hi = tc::to_tf32(v);
          const int off = (rg * (KCH / 4) + kc) * 128 + lane * 4;
          *reinterpret_cast<float*>(S.A[0] + off) = hi;
          *reinterpret_cast<float*>(S.A[1] + off) = tc::to_tf32(v - hi);
        }
      }
      tc::fence_proxy_async();
      __syncthreads();
      if (tid == 0) {
        tc::fence_after_sync();
#pragma unroll 1
        for (int st = 0; st < kcn / 2; ++st) {
          const uint32_t ao = (uint32_t)(st * 256), bo = (uint32_t)((c0 / 8 + st) * 256);
          const uint64_t ah = tc::smem_desc(a_hi + ao, kLbo, kSboA), al = tc::smem_desc(a_lo + ao, kLbo, kSboA);
          const uint64_t bh = tc::smem_desc(b_hi + bo, kLbo, sbo_b), bl = tc::smem_desc(b_lo + bo, kLbo, sbo_b);
          tc::mma_tf32(tmem, ah, bh, idesc, (c0 > 0 || st > 0) ? 1u : 0u);
          tc::mma_tf32(tmem, al, bh, idesc, 1u);
          tc::mma_tf32(tmem, ah, bl, idesc, 1u);
        }
        tc::commit(&S.mbar);
        // A is rewritten by the next chunk: wait (bounded) for this chunk's products
        if (!tc::mbar_wait(&S.mbar, parity, kTPWaitPolls)) {
          // the MMAs may still be writing tensor memory: wait once more for their commit before
          // anything releases it; if that also ends without it, the tensor memory stays allocated
          gfe_raise(err, GFE_DEVERR_TIMEOUT);
          const bool drained = tc::mbar_wait(&S.mbar, parity, kTPWaitPolls);
          S.abort = drained ? 1 : 2;
        }
      }
      parity ^= 1u;
      __syncthreads();
      tc::fence_after_sync();
      if (S.abort) break;
    }
    if (S.abort) break;
    // tensor memory -> staged product: warp w < 4 reads lanes 32 w .. 32 w + 31
    if (warp < 4) {
#pragma unroll
      for (int c0 = 0; c0 < R; c0 += 32) {
        float v[32];
        tc::tmem_ld_32x32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
        for (int j = 0; j < 32; ++j) D[warp * 32 + lane][c0 + j] = v[j];
      }
    }
    tc::fence_before_sync();
    __syncthreads();
    const int total = live_slots * cfg.npairs;
    for (int t0 = tid; t0 < total; t0 += kTPScatter * blockDim.x)
      scatter_batch(t0, blockDim.x, total, [&](int t, double& v, long long& pmn, long long& pnm) {
        const int k = t / cfg.npairs;
        const int32_t mn = pairs[t - k * cfg.npairs];
        const int m = mn & 0xffff, n = mn >> 16;
        v = (double)D[k * R + n][m];
        if (scale) v = v * S.ssf[k][m] * S.ssf[k][n];  // K(ms, ns) * SF(ms) * SF(ns)
        const int rm = S.snode[k][m], rn = S.snode[k][n];
        pmn = entry_pos(slots, S.elem[k], nns, m, n, rp, ci, rm, rn + 1);
        if (m != n) pnm = entry_pos(slots, S.elem[k], nns, n, m, rp, ci, rn, rm + 1);
      }, values, err);
    __syncthreads();  // the staged product and the element data are rewritten by the next tile
  }
  if (bad) gfe_raise(err, GFE_DEVERR_JACOBIAN);
  if (nonfinite) gfe_raise(err, GFE_DEVERR_NONFINITE);
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0 && S.abort < 2) tc::tmem_dealloc(tmem, R);
}

__global__ void values_to_fp32(const double* __restrict__ v, float* __restrict__ v32, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    v32[i] = (float)v[i];
}

template <typename T>
int launch_tp(const int32_t* order, const int32_t* ngauss, int32_t n_nodes, const int32_t* en, const double* coords,
              const double* scale, const double* kappa, const int32_t* color_elems, const int32_t* color_ptr_host, int32_t n_colors,
              const int32_t* rp, const int32_t* ci, const int32_t* slots, double* values, cudaStream_t s,
              int* launches) {
  const TPTables<T>* t = nullptr;
  if (int rc = tp_tables<T>(order, ngauss, &t)) return rc;
  unsigned* err = gfe::device_error_word();
  // linear tetrahedra (no scale factors): one element a thread
  const bool simplex_p1 = order[0] == 7 && t->cfg.nns == 4 && !scale;
  for (int c = 0; c < n_colors; ++c) {
    const int c0 = color_ptr_host[c], cnt = color_ptr_host[c + 1] - c0;
    if (cnt <= 0) continue;
    if (simplex_p1) {
      const int grid = std::min((cnt + kTPThreads - 1) / kTPThreads, 16 * gfe::sm_count());
      laplace_tet4_kernel<T><<<grid, kTPThreads, 0, s>>>(color_elems + c0, cnt, n_nodes, en, coords, kappa, t->dphi,
                                                         t->w, t->cfg.ng, rp, ci, values, err);
    } else if (t->cfg.nns <= kSmallNns && t->cfg.ng <= kSmallNg) {
      constexpr int EPB = kTPThreads / 32;
      const int grid = std::min((cnt + EPB - 1) / EPB, 8 * gfe::sm_count());
      laplace_tp_kernel<T, 32, kSmallNns, kSmallNg><<<grid, kTPThreads, 0, s>>>(
          color_elems + c0, cnt, n_nodes, en, coords, scale, kappa, t->dphi, t->w, t->pairs, t->cfg, rp, ci, slots,
          values, err);
    } else {
      const int grid = std::min(cnt, 8 * gfe::sm_count());
      laplace_tp_kernel<T, kTPThreads, kMaxNns, kMaxNg><<<grid, kTPThreads, 0, s>>>(
          color_elems + c0, cnt, n_nodes, en, coords, scale, kappa, t->dphi, t->w, t->pairs, t->cfg, rp, ci, slots,
          values, err);
    }
    ++*launches;
  }
  return GFE_OK;
}

// Tensor-core element matrices (GFE_TC_TF32X3) of hexahedral bases with up to 64 nodes and 64 Gauss
// points, colour by colour; one CTA an SM (about 186 KB of shared memory).
int launch_tp_tc(const int32_t* order, const int32_t* ngauss, int32_t n_nodes, const int32_t* en, const double* coords,
                 const double* scale, const double* kappa, const int32_t* color_elems, const int32_t* color_ptr_host,
                 int32_t n_colors, const int32_t* rp, const int32_t* ci, const int32_t* slots, double* values,
                 cudaStream_t s, int* launches) {
  const TPTables<float>* t = nullptr;
  if (int rc = tp_tables<float>(order, ngauss, &t)) return rc;
  const int nns = t->cfg.nns;
  if (nns > kMaxNns || t->cfg.ng > kMaxNg)
    return gfe::set_error(GFE_ERR_ARG, "gfe_laplace_assemble_tp: the tensor-core path takes up to %d nodes and %d "
                          "Gauss points an element", kMaxNns, kMaxNg);
  const void* k32 = (const void*)laplace_tp_tc_kernel<32>;
  const void* k64 = (const void*)laplace_tp_tc_kernel<64>;
  const size_t smem = nns <= 32 ? sizeof(TPTCShared<32>) : sizeof(TPTCShared<64>);
  GFE_CUDA_TRY(cudaFuncSetAttribute(nns <= 32 ? k32 : k64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  unsigned* err = gfe::device_error_word();
  const int ept = nns <= 32 ? TPTCShape<32>::kEPT : TPTCShape<64>::kEPT;
  const int per_sm = nns <= 32 ? TPTCShape<32>::kBlocksPerSM : TPTCShape<64>::kBlocksPerSM;
  for (int c = 0; c < n_colors; ++c) {
    const int c0 = color_ptr_host[c], cnt = color_ptr_host[c + 1] - c0;
    if (cnt <= 0) continue;
    const int grid = std::min((cnt + ept - 1) / ept, per_sm * gfe::sm_count());
    if (nns <= 32)
      laplace_tp_tc_kernel<32><<<grid, TPTCShape<32>::kThreads, smem, s>>>(
          color_elems + c0, cnt, n_nodes, en, coords, scale, kappa, t->dphi, t->w, t->pairs, t->cfg, rp, ci, slots,
          values, err);
    else
      laplace_tp_tc_kernel<64><<<grid, TPTCShape<64>::kThreads, smem, s>>>(
          color_elems + c0, cnt, n_nodes, en, coords, scale, kappa, t->dphi, t->w, t->pairs, t->cfg, rp, ci, slots,
          values, err);
    ++*launches;
  }
  return GFE_OK;
}

}  // namespace

extern "C" int gfe_laplace_tp_slot_map(int32_t n_elem, int32_t nns, const int32_t* elem_nodes, const int32_t* row_ptr,
                                       const int32_t* col_idx, int64_t nnz, int32_t* slots, void* stream) {
  const char* fn = "gfe_laplace_tp_slot_map";
  if (n_elem < 0 || nns <= 0 || nns > kMaxNns || (n_elem > 0 && (!elem_nodes || !row_ptr || !col_idx || !slots)))
    return gfe::set_error(GFE_ERR_ARG, "%s: invalid arguments", fn);
  if (nnz < 0 || nnz > INT32_MAX)
    return gfe::set_error(GFE_ERR_ARG, "%s: CSR positions must fit in int32 (nnz %lld)", fn, (long long)nnz);
  if (n_elem == 0) return GFE_OK;
  cudaStream_t s = gfe::as_stream(stream);
  tp_slot_kernel<<<16 * gfe::sm_count(), 256, 0, s>>>(n_elem, nns, elem_nodes, row_ptr, col_idx, slots);
  GFE_LAUNCH_CHECK(fn);
  return GFE_OK;
}

extern "C" int gfe_laplace_assemble_tp(const int32_t* order, const int32_t* n_gauss, int32_t n_elem, int32_t n_nodes,
                                       const int32_t* elem_nodes, const double* coords, const double* scale,
                                       const double* kappa,
                                       const int32_t* color_elems, const int32_t* color_ptr_host, int32_t n_colors,
                                       const int32_t* row_ptr, const int32_t* col_idx, int64_t nnz,
                                       const int32_t* slots, double* values, float* values32, double* rhs,
                                       int32_t precision, void* stream) {
  const char* fn = "gfe_laplace_assemble_tp";
  if (!order || !n_gauss) return gfe::set_error(GFE_ERR_ARG, "%s: order and n_gauss are required", fn);
  const bool simplex = order[0] == 7 || order[0] == 8 || order[0] == 9;
  if (simplex && (order[1] != order[0] || order[2] != order[0] || n_gauss[0] < 1 || n_gauss[0] > 5))
    return gfe::set_error(GFE_ERR_ARG, "%s: tetrahedra need the same simplex interpolation in every xi and a "
                          "Gauss_Simplex order of 1..5 in n_gauss[0]", fn);
  for (int d = 0; d < 3 && !simplex; ++d) {
    if (order[d] < 1 || order[d] > 4)
      return gfe::set_error(GFE_ERR_ARG, "%s: interpolation %d in xi%d (1..3 Lagrange, 4 cubic Hermite supported)",
                            fn, order[d], d + 1);
    if (n_gauss[d] < 1 || n_gauss[d] > 4)
      return gfe::set_error(GFE_ERR_ARG, "%s: %d Gauss points in xi%d (1..4 supported)", fn, n_gauss[d], d + 1);
  }
  if (n_elem < 0 || n_nodes <= 0 || !coords || !row_ptr || !col_idx || !values || nnz < 0 ||
      (n_elem > 0 && (!elem_nodes || !color_elems || !color_ptr_host || n_colors <= 0)))
    return gfe::set_error(GFE_ERR_ARG, "%s: invalid arguments", fn);
  if (color_ptr_host && n_colors > 0 && (color_ptr_host[0] != 0 || color_ptr_host[n_colors] != n_elem))
    return gfe::set_error(GFE_ERR_ARG, "%s: colour offsets must run from 0 to n_elem", fn);
  if (precision != GFE_FP64 && precision != GFE_MIXED && precision != GFE_MIXED_DF && precision != GFE_TC_TF32X3)
    return gfe::set_error(GFE_ERR_ARG, "%s: unknown precision %d", fn, precision);
  if (precision == GFE_TC_TF32X3 && simplex)
    return gfe::set_error(GFE_ERR_ARG, "%s: the tensor-core path covers hexahedral bases", fn);
  cudaStream_t s = gfe::as_stream(stream);
  GFE_CUDA_TRY(cudaMemsetAsync(values, 0, sizeof(double) * (size_t)nnz, s));
  if (rhs) GFE_CUDA_TRY(cudaMemsetAsync(rhs, 0, sizeof(double) * (size_t)n_nodes, s));
  void* prof = gfe::stage_begin(GFE_STAGE_LAPLACE_ELEMENTS, s);
  int launches = 0, rc;
  if (precision == GFE_FP64)
    rc = launch_tp<double>(order, n_gauss, n_nodes, elem_nodes, coords, scale, kappa, color_elems, color_ptr_host,
                           n_colors, row_ptr, col_idx, slots, values, s, &launches);
  else if (precision == GFE_MIXED)
    rc = launch_tp<float>(order, n_gauss, n_nodes, elem_nodes, coords, scale, kappa, color_elems, color_ptr_host,
                          n_colors, row_ptr, col_idx, slots, values, s, &launches);
  else if (precision == GFE_TC_TF32X3)
    rc = launch_tp_tc(order, n_gauss, n_nodes, elem_nodes, coords, scale, kappa, color_elems, color_ptr_host,
                      n_colors, row_ptr, col_idx, slots, values, s, &launches);
  else
    rc = launch_tp<f2>(order, n_gauss, n_nodes, elem_nodes, coords, scale, kappa, color_elems, color_ptr_host,
                       n_colors, row_ptr, col_idx, slots, values, s, &launches);
  gfe::stage_end(GFE_STAGE_LAPLACE_ELEMENTS, prof, s, launches);
  if (rc) return rc;
  if (values32 && nnz > 0) values_to_fp32<<<4 * gfe::sm_count(), 256, 0, s>>>(values, values32, nnz);
  GFE_LAUNCH_CHECK(fn);
  return GFE_OK;
}
