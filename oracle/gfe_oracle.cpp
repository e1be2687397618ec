// gfe_oracle.cpp -- CPU restatement of OpenCMISS-Iron's finite-element assembly hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the parity oracle for the GB300 engine in
// iron_gb300/: only tests, the smoke check and the CPU-baseline leg of bench.py load it.
// The product path never links or calls it.
//
// Iron itself (Fortran 2003 + MPI + PETSc) cannot be built in this environment, so the
// oracle restates Iron's algorithms routine by routine, citing the reference file:line
// (paths relative to the reference project root) it follows.  It is pinned against the
// reference's own fixtures and known-answer tests (tests/test_oracle_golden.py).
//
// Conventions: all node / element / DOF indices exchanged through this C ABI are 0-based;
// the CSR structure is emitted 1-based exactly as Iron stores it
// (src/types.F90:909-929, ROW_INDICES(M+1), COLUMN_INDICES(nnz)).

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace {

// ---------------------------------------------------------------------------------------
// Quadrature.  src/basis_routines.F90:6804-6890 (Gauss_Legendre): tabulated closed forms of
// the 1..4 point rules on [0,1].
// ---------------------------------------------------------------------------------------
bool gauss_legendre(int n, double* x, double* w) {
  if (n < 1 || n > 4) return false;
  const double s3 = std::sqrt(3.0), s06 = std::sqrt(0.6), s65 = std::sqrt(6.0 / 5.0), s30 = std::sqrt(30.0);
  const double loc[10] = {0.5,
                          (-1.0 / s3 + 1.0) / 2.0, (+1.0 / s3 + 1.0) / 2.0,
                          (-s06 + 1.0) / 2.0, 0.5, (+s06 + 1.0) / 2.0,
                          (-std::sqrt((3.0 + 2.0 * s65) / 7.0) + 1.0) / 2.0,
                          (-std::sqrt((3.0 - 2.0 * s65) / 7.0) + 1.0) / 2.0,
                          (+std::sqrt((3.0 - 2.0 * s65) / 7.0) + 1.0) / 2.0,
                          (+std::sqrt((3.0 + 2.0 * s65) / 7.0) + 1.0) / 2.0};
  const double wt[10] = {1.0, 0.5, 0.5, 2.5 / 9.0, 4.0 / 9.0, 2.5 / 9.0,
                         (18.0 - s30) / 72.0, (18.0 + s30) / 72.0, (18.0 + s30) / 72.0, (18.0 - s30) / 72.0};
  const int start[4] = {0, 1, 3, 6};
  for (int i = 0; i < n; ++i) {
    x[i] = loc[start[n - 1] + i];
    w[i] = wt[start[n - 1] + i];
  }
  return true;
}

// 1D Lagrange basis on [0,1]; node index a is 0-based.  deriv 0 = value, 1 = first derivative.
// src/basis_routines.F90:7969-8020 (LAGRANGE_LINEAR_EVALUATE), :8027-8090 (QUADRATIC),
// :7899-7962 (CUBIC).
double lagrange1d(int order, int a, int deriv, double xi) {
  if (order == 1) {
    if (deriv == 0) return a == 0 ? 1.0 - xi : xi;
    return a == 0 ? -1.0 : 1.0;
  }
  if (order == 2) {
    if (deriv == 0) {
      if (a == 0) return 1.0 - 3.0 * xi + 2.0 * xi * xi;
      if (a == 1) return 4.0 * xi * (1.0 - xi);
      return xi * (xi + xi - 1.0);
    }
    if (a == 0) return 4.0 * xi - 3.0;
    if (a == 1) return 4.0 - 8.0 * xi;
    return 4.0 * xi - 1.0;
  }
  if (order == 3) {
    if (deriv == 0) {
      if (a == 0) return 0.5 * (3.0 * xi - 1.0) * (3.0 * xi - 2.0) * (1.0 - xi);
      if (a == 1) return 4.5 * xi * (3.0 * xi - 2.0) * (xi - 1.0);
      if (a == 2) return 4.5 * xi * (3.0 * xi - 1.0) * (1.0 - xi);
      return 0.5 * xi * (3.0 * xi - 1.0) * (3.0 * xi - 2.0);
    }
    if (a == 0) return -13.5 * xi * xi + 18.0 * xi - 5.5;
    if (a == 1) return 40.5 * xi * xi - 45.0 * xi + 9.0;
    if (a == 2) return -40.5 * xi * xi + 36.0 * xi - 4.5;
    return 13.5 * xi * xi - 9.0 * xi + 1.0;
  }
  return 0.0;
}

// 1D cubic Hermite on [0,1], src/basis_routines.F90:7607-7701 (HERMITE_CUBIC_EVALUATE): node a
// (0-based, 0 or 1), node derivative k (0 = value, 1 = first derivative), deriv 0 = value, 1 = d/dxi.
double hermite1d(int a, int k, int deriv, double xi) {
  if (deriv == 0) {
    if (a == 0) return k == 0 ? (2.0 * xi - 3.0) * xi * xi + 1.0 : ((xi - 2.0) * xi + 1.0) * xi;
    return k == 0 ? xi * xi * (3.0 - 2.0 * xi) : xi * xi * (xi - 1.0);
  }
  if (a == 0) return k == 0 ? 6.0 * xi * (xi - 1.0) : (3.0 * xi - 4.0) * xi + 1.0;
  return k == 0 ? 6.0 * xi * (1.0 - xi) : xi * (3.0 * xi - 2.0);
}

// Tensor-product table in Iron's order: element parameter ns with xi1 fastest
// (src/basis_routines.F90:3243-3370), Gauss point ng = i + (j-1 + (k-1) n2) n1 (:3820).
// Layout of the returned table: tab[(ng * (nxi+1) + nu) * nns + ns], nu 0 = value,
// nu = 1..nxi = d/dxi_nu (Iron's partial-derivative indices 2, 4, 7: src/constants.F90:180-185).
// order[d]: Iron's interpolation specification per xi direction: 1..3 = Lagrange of that order,
// 4 = cubic Hermite (BASIS_CUBIC_HERMITE_INTERPOLATION, src/basis_routines.F90:83-86).  Element
// parameters run over the local nodes (xi1 fastest) and, within a node, over its derivatives in
// Iron's order (the count doubles for every Hermite direction in xi order, :2633-2662), so with
// three Hermite directions the derivative index is d1 + 2 d2 + 4 d3.
struct TPBasis {
  int nxi = 0, nns = 0, ng = 0;
  int nnx[3] = {1, 1, 1}, ngx[3] = {1, 1, 1}, order[3] = {1, 1, 1};
  std::vector<double> tab, wts;
};

// Tetrahedral simplex basis, src/basis_routines.F90: Basis_SimplexBasisCreate :4813-5875 (node
// positions per area coordinate: 1 absent, 2 on an edge (L for linear, 2L for quadratic),
// 3 vertex L(2L-1); SIMPLEX_LINEAR/QUADRATIC_EVALUATE :8177-8313), BASIS_SIMPLEX_BASIS_EVALUATE
// :6041-6270 (d/dxi_i = d/dL4 - d/dL_i), Gauss_Simplex :6898-7600 (tetrahedra, orders 1..5:
// 1, 4, 5, 11, 14 points in area coordinates, weights summing to 1/6).  interp 7 = linear
// (4 nodes), 8 = quadratic (10 nodes), 9 = cubic (20 nodes: vertices, two nodes on each edge,
// one on each face; positions :5236-5353, SIMPLEX_CUBIC_EVALUATE :8092-8169 with factors 1, 3L,
// 3/2 L(3L-1), 1/2 L(3L-1)(3L-2) for positions 1..4); quad_order = Gauss_Simplex order.
double simplex_factor(int interp, int pos, int deriv, double L) {
  if (interp == 7) return pos == 1 ? (deriv ? 0.0 : 1.0) : (deriv ? 1.0 : L);
  if (interp == 9) {
    switch (pos) {
      case 1: return deriv ? 0.0 : 1.0;
      case 2: return deriv ? 3.0 : 3.0 * L;
      case 3: return deriv ? 1.5 * (6.0 * L - 1.0) : 1.5 * L * (3.0 * L - 1.0);
      default: return deriv ? 13.5 * L * L - 9.0 * L + 1.0 : 0.5 * L * (3.0 * L - 1.0) * (3.0 * L - 2.0);
    }
  }
  if (pos == 1) return deriv ? 0.0 : 1.0;
  if (pos == 2) return deriv ? 2.0 : 2.0 * L;
  return deriv ? 4.0 * L - 1.0 : L * (2.0 * L - 1.0);
}

// The symmetric orbits of the tetrahedral rules, in Gauss_Simplex's point order: a = the four
// points with one area coordinate (1 + 3a)/4 and three (1 - a)/4, cycled; b = the six points with
// two coordinates (1 + 2b)/4 and two (1 - 2b)/4.
void simplex_orbit_a(double a, double wt, std::vector<std::array<double, 4>>& L, std::vector<double>& w) {
  const double l1 = (1.0 + 3.0 * a) / 4.0, l2 = (1.0 - a) / 4.0, l3 = (1.0 - a) / 4.0, l4 = 1.0 - l1 - l2 - l3;
  L.push_back({l1, l2, l3, l4});
  L.push_back({l4, l1, l2, l3});
  L.push_back({l3, l4, l1, l2});
  L.push_back({l2, l3, l4, l1});
  for (int k = 0; k < 4; ++k) w.push_back(wt / 6.0);
}

void simplex_orbit_b(double b, double wt, std::vector<std::array<double, 4>>& L, std::vector<double>& w) {
  const double p = (1.0 + 2.0 * b) / 4.0, q = (1.0 - 2.0 * b) / 4.0, r = 1.0 - p - p - q;
  L.push_back({p, p, q, r});
  L.push_back({p, q, p, r});
  L.push_back({p, q, r, p});
  L.push_back({q, p, p, r});
  L.push_back({q, p, r, p});
  L.push_back({q, r, p, p});
  for (int k = 0; k < 6; ++k) w.push_back(wt / 6.0);
}

bool make_simplex_basis(int interp, int quad_order, TPBasis& b) {
  static const int lin[4][4] = {{2, 1, 1, 1}, {1, 2, 1, 1}, {1, 1, 2, 1}, {1, 1, 1, 2}};
  static const int quad[10][4] = {{3, 1, 1, 1}, {1, 3, 1, 1}, {1, 1, 3, 1}, {1, 1, 1, 3}, {2, 2, 1, 1},
                                  {2, 1, 2, 1}, {2, 1, 1, 2}, {1, 2, 2, 1}, {1, 1, 2, 2}, {1, 2, 1, 2}};
  static const int cub[20][4] = {{4, 1, 1, 1}, {1, 4, 1, 1}, {1, 1, 4, 1}, {1, 1, 1, 4}, {3, 2, 1, 1},
                                 {2, 3, 1, 1}, {3, 1, 2, 1}, {2, 1, 3, 1}, {3, 1, 1, 2}, {2, 1, 1, 3},
                                 {1, 3, 2, 1}, {1, 2, 3, 1}, {1, 1, 3, 2}, {1, 1, 2, 3}, {1, 3, 1, 2},
                                 {1, 2, 1, 3}, {2, 2, 2, 1}, {2, 2, 1, 2}, {2, 1, 2, 2}, {1, 2, 2, 2}};
  std::vector<std::array<double, 4>> gl;
  std::vector<double> gw;
  if (quad_order == 1) {
    gl.push_back({0.25, 0.25, 0.25, 0.25});
    gw.push_back(1.0 / 6.0);
  } else if (quad_order == 2 || quad_order == 3) {
    const double a = quad_order == 2 ? 1.0 / std::sqrt(5.0) : 1.0 / 3.0;
    const double wa = quad_order == 2 ? 0.25 : 9.0 / 20.0;
    const double l1 = (1.0 + 3.0 * a) / 4.0, l2 = (1.0 - a) / 4.0, l3 = (1.0 - a) / 4.0, l4 = 1.0 - l1 - l2 - l3;
    if (quad_order == 3) {
      gl.push_back({0.25, 0.25, 0.25, 0.25});
      gw.push_back(-4.0 / 5.0 / 6.0);
    }
    gl.push_back({l1, l2, l3, l4});
    gl.push_back({l4, l1, l2, l3});
    gl.push_back({l3, l4, l1, l2});
    gl.push_back({l2, l3, l4, l1});
    for (int k = 0; k < 4; ++k) gw.push_back(wa / 6.0);
  } else if (quad_order == 4) {
    gl.push_back({0.25, 0.25, 0.25, 0.25});
    gw.push_back(-148.0 / 1875.0 / 6.0);
    simplex_orbit_a(5.0 / 7.0, 343.0 / 7500.0, gl, gw);
    simplex_orbit_b(std::sqrt(70.0) / 28.0, 56.0 / 375.0, gl, gw);
  } else if (quad_order == 5) {
    // lambda: the root of Keast's cubic that the rule's two a orbits and one b orbit are built on
    const double pi2 = 2.0 * 3.14159265358979323846;
    const double lam = 4.0 / 27.0 *
                       (4.0 * std::sqrt(79.0) * std::cos((std::acos(67.0 * std::sqrt(79.0) / 24964.0) + pi2) / 3.0) + 71.0);
    const double root = std::sqrt(9.0 * lam * lam - 248.0 * lam + 1680.0);
    const double a1 = (root + 28.0 - 3.0 * lam) / (112.0 - 10.0 * lam);
    const double a2 = (-root + 28.0 - 3.0 * lam) / (112.0 - 10.0 * lam);
    const double wa1 = ((21.0 - lam) * a2 - 7.0) / (420.0 * a1 * a1 * (a2 - a1));
    const double wa2 = ((21.0 - lam) * a1 - 7.0) / (420.0 * a2 * a2 * (a1 - a2));
    simplex_orbit_a(a1, wa1, gl, gw);
    simplex_orbit_a(a2, wa2, gl, gw);
    simplex_orbit_b(1.0 / std::sqrt(lam), lam * lam / 840.0, gl, gw);
  } else {
    return false;
  }
  if (interp != 7 && interp != 8 && interp != 9) return false;
  const int nns = interp == 7 ? 4 : (interp == 8 ? 10 : 20);
  b.nxi = 3;
  b.nns = nns;
  b.ng = (int)gl.size();
  b.tab.assign((size_t)b.ng * 4 * nns, 0.0);
  b.wts = gw;
  for (int g = 0; g < b.ng; ++g)
    for (int ns = 0; ns < nns; ++ns) {
      const int* pos = interp == 7 ? lin[ns] : (interp == 8 ? quad[ns] : cub[ns]);
      double dL[4];  // d phi / d L_k
      double v = 1.0;
      for (int k = 0; k < 4; ++k) v *= simplex_factor(interp, pos[k], 0, gl[g][k]);
      for (int k = 0; k < 4; ++k) {
        double d = 1.0;
        for (int j = 0; j < 4; ++j) d *= simplex_factor(interp, pos[j], j == k, gl[g][j]);
        dL[k] = d;
      }
      b.tab[((size_t)g * 4 + 0) * nns + ns] = v;
      for (int i = 0; i < 3; ++i) b.tab[((size_t)g * 4 + i + 1) * nns + ns] = dL[3] - dL[i];
    }
  return true;
}

// Linear triangles (interp 7 with two xi directions): area coordinates L1..L3, node n at vertex n
// (BASIS_SIMPLEX_BASIS_EVALUATE :6041-6270 with d/dxi_i = d/dL3 - d/dL_i in two dimensions), and
// Gauss_Simplex's triangle rules of orders 1..5 (:6898-7600, numberOfVertices = 3) in its point
// order: the centroid, and orbits of the three points with one coordinate (1 + 2a)/3 and two
// (1 - a)/3, cycled as (l1, l2, l3), (l3, l1, l2), (l2, l3, l1); weights sum to 1/2.
void triangle_orbit(double a, double wt, std::vector<std::array<double, 4>>& L, std::vector<double>& w) {
  const double l1 = (1.0 + 2.0 * a) / 3.0, l2 = (1.0 - a) / 3.0, l3 = 1.0 - l1 - l2;
  L.push_back({l1, l2, l3, 0.0});
  L.push_back({l3, l1, l2, 0.0});
  L.push_back({l2, l3, l1, 0.0});
  for (int k = 0; k < 3; ++k) w.push_back(wt / 2.0);
}

bool make_triangle_basis(int interp, int quad_order, TPBasis& b) {
  if (interp != 7) return false;
  std::vector<std::array<double, 4>> gl;
  std::vector<double> gw;
  const double third = 1.0 / 3.0;
  switch (quad_order) {
    case 1:
      gl.push_back({third, third, third, 0.0});
      gw.push_back(0.5);
      break;
    case 2:
      triangle_orbit(-0.5, third, gl, gw);
      break;
    case 3:
      gl.push_back({third, third, third, 0.0});
      gw.push_back(-0.75 / 2.0);
      triangle_orbit(0.4, 25.0 / 48.0, gl, gw);
      break;
    case 4: {
      const double r = std::sqrt(950.0 - 220.0 * std::sqrt(10.0));
      const double a1 = (-10.0 + 5.0 * std::sqrt(10.0) + r) / 30.0, a2 = (-10.0 + 5.0 * std::sqrt(10.0) - r) / 30.0;
      triangle_orbit(a1, (5.0 * a2 - 2.0) / (60.0 * a1 * a1 * (a2 - a1)), gl, gw);
      triangle_orbit(a2, (5.0 * a1 - 2.0) / (60.0 * a2 * a2 * (a1 - a2)), gl, gw);
      break;
    }
    case 5: {
      const double q = std::sqrt(15.0);
      gl.push_back({third, third, third, 0.0});
      gw.push_back(9.0 / 40.0 / 2.0);
      triangle_orbit((1.0 + q) / 7.0, (155.0 - q) / 1200.0, gl, gw);
      triangle_orbit((1.0 - q) / 7.0, (155.0 + q) / 1200.0, gl, gw);
      break;
    }
    default:
      return false;
  }
  b.nxi = 2;
  b.nns = 3;
  b.ng = (int)gl.size();
  b.tab.assign((size_t)b.ng * 3 * 3, 0.0);
  b.wts = gw;
  for (int g = 0; g < b.ng; ++g)
    for (int ns = 0; ns < 3; ++ns) {
      b.tab[((size_t)g * 3 + 0) * 3 + ns] = gl[g][ns];
      // d L_ns / d xi_i = d/dL3 - d/dL_i
      for (int i = 0; i < 2; ++i) b.tab[((size_t)g * 3 + i + 1) * 3 + ns] = (ns == 2 ? 1.0 : 0.0) - (ns == i ? 1.0 : 0.0);
    }
  return true;
}

bool make_tp_basis(int nxi, const int* order, const int* ngauss, TPBasis& b) {
  if (nxi == 3 && (order[0] == 7 || order[0] == 8 || order[0] == 9)) return make_simplex_basis(order[0], ngauss[0], b);
  if (nxi == 2 && (order[0] == 7 || order[0] == 8 || order[0] == 9)) return make_triangle_basis(order[0], ngauss[0], b);
  if (nxi < 1 || nxi > 3) return false;
  b.nxi = nxi;
  b.ng = 1;
  double gx[3][4], gw[3][4];
  for (int d = 0; d < 3; ++d) {
    b.nnx[d] = 1; b.ngx[d] = 1; b.order[d] = 1;
    gx[d][0] = 0.5; gw[d][0] = 1.0;
  }
  int nder = 1;  // derivatives per node
  for (int d = 0; d < nxi; ++d) {
    if (order[d] < 1 || order[d] > 4) return false;
    b.order[d] = order[d];
    b.nnx[d] = order[d] == 4 ? 2 : order[d] + 1;
    if (order[d] == 4) nder *= 2;
    b.ngx[d] = ngauss[d];
    if (!gauss_legendre(ngauss[d], gx[d], gw[d])) return false;
    b.ng *= b.ngx[d];
  }
  // element parameters: (node position, node derivative) per direction, in Iron's order
  std::vector<std::array<int, 6>> par;
  for (int a3 = 0; a3 < b.nnx[2]; ++a3)
    for (int a2 = 0; a2 < b.nnx[1]; ++a2)
      for (int a1 = 0; a1 < b.nnx[0]; ++a1)
        for (int k = 0; k < nder; ++k) {
          std::array<int, 6> q = {a1, a2, a3, 0, 0, 0};
          int bit = 0;
          for (int d = 0; d < nxi; ++d)
            if (b.order[d] == 4) q[3 + d] = (k >> bit++) & 1;
          par.push_back(q);
        }
  b.nns = (int)par.size();
  b.tab.assign((size_t)b.ng * (nxi + 1) * b.nns, 0.0);
  b.wts.assign(b.ng, 0.0);
  for (int g3 = 0; g3 < b.ngx[2]; ++g3)
    for (int g2 = 0; g2 < b.ngx[1]; ++g2)
      for (int g1 = 0; g1 < b.ngx[0]; ++g1) {
        int g = g1 + b.ngx[0] * (g2 + b.ngx[1] * g3);
        const int gi[3] = {g1, g2, g3};
        double w = 1.0;
        for (int d = 0; d < nxi; ++d) w *= gw[d][gi[d]];
        b.wts[g] = w;
        for (int ns = 0; ns < b.nns; ++ns)
          for (int nu = 0; nu <= nxi; ++nu) {
            double v = 1.0;
            for (int d = 0; d < nxi; ++d) {
              const int der = (nu == d + 1) ? 1 : 0;
              v *= b.order[d] == 4 ? hermite1d(par[ns][d], par[ns][3 + d], der, gx[d][gi[d]])
                                   : lagrange1d(b.order[d], par[ns][d], der, gx[d][gi[d]]);
            }
            b.tab[((size_t)g * (nxi + 1) + nu) * b.nns + ns] = v;
          }
      }
  return true;
}

// 3x3 / 2x2 inverse and determinant, src/maths.F90:2807-2868 (InvertFullDP).
double invert(int n, const double A[3][3], double B[3][3]) {
  double det;
  if (n == 1) {
    det = A[0][0];
    B[0][0] = 1.0 / A[0][0];
  } else if (n == 2) {
    det = A[0][0] * A[1][1] - A[1][0] * A[0][1];
    B[0][0] = A[1][1] / det; B[0][1] = -A[0][1] / det;
    B[1][0] = -A[1][0] / det; B[1][1] = A[0][0] / det;
  } else {
    det = A[0][0] * A[1][1] * A[2][2] + A[0][1] * A[1][2] * A[2][0] + A[0][2] * A[1][0] * A[2][1] -
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
  }
  return det;
}

// Metrics at one Gauss point for a rectangular-cartesian geometric field whose element
// parameters are x[comp][ns] (separated component order).  src/coordinate_routines.F90:639-1026
// (COORDINATE_METRICS_CALCULATE): DX_DXI from the interpolated first derivatives
// (src/field_routines.F90:5771-5982 / src/basis_routines.F90:2075-2130), GL = DX_DXI^T DX_DXI,
// GU = inv(GL), volume Jacobian = sqrt(|det GL|) (:818-822), DXI_DX = inv(DX_DXI) (:832).
struct Metrics {
  double dx_dxi[3][3], dxi_dx[3][3], gl[3][3], gu[3][3], jac;
};

void metrics_at(const TPBasis& b, int g, const double* const* x, int ncomp, Metrics& m) {
  const int nxi = b.nxi;
  std::memset(&m, 0, sizeof(m));
  for (int i = 0; i < ncomp; ++i)
    for (int xi = 0; xi < nxi; ++xi) {
      double s = 0.0;
      const double* t = &b.tab[((size_t)g * (nxi + 1) + xi + 1) * b.nns];
      for (int ns = 0; ns < b.nns; ++ns) s += t[ns] * x[i][ns];
      m.dx_dxi[i][xi] = s;
    }
  for (int mi = 0; mi < nxi; ++mi)
    for (int ni = 0; ni < nxi; ++ni) {
      double s = 0.0;
      for (int i = 0; i < ncomp; ++i) s += m.dx_dxi[i][mi] * m.dx_dxi[i][ni];
      m.gl[mi][ni] = s;
    }
  double detgl = invert(nxi, m.gl, m.gu);
  m.jac = std::sqrt(std::fabs(detgl));
  if (nxi == ncomp) invert(nxi, m.dx_dxi, m.dxi_dx);
}

// ---------------------------------------------------------------------------------------
// CSR value add.  src/matrix_vector.F90:3202-3240 (MATRIX_VALUES_ADD_DP2, compressed-row
// branch): bisection over the row's sorted columns until the window is <= 10 wide
// (bisectionToLinearSearchThreshold, :184), then a linear scan; error when absent.
// row/col indices here are 1-based like Iron's.
// ---------------------------------------------------------------------------------------
const int kBisectionToLinear = 10;

int csr_values_add(const int32_t* rp, const int32_t* ci, double* data, int nr, const int32_t* rows, int nc,
                   const int32_t* cols, const double* vals /* [nr][nc] row-major */) {
  int prev = -1;
  for (int i = 0; i < nr; ++i) {
    int row = rows[i];
    int lo = rp[row - 1], up = rp[row];
    for (int j = 0; j < nc; ++j) {
      int loc = 0, col = cols[j];
      if (col <= prev) lo = rp[row - 1]; else up = rp[row];
      prev = col;
      while (up - lo > kBisectionToLinear) {
        int mid = lo + (up - lo) / 2;
        if (ci[mid - 1] > col) up = mid; else lo = mid;
      }
      for (int k = lo; k <= up && k < rp[row]; ++k) {
        if (ci[k - 1] == col) { loc = k; lo = k + 1; break; }
      }
      if (loc == 0) return -1;
      data[loc - 1] += vals[(size_t)i * nc + j];
    }
  }
  return 0;
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------------------------------
// Tables
// ---------------------------------------------------------------------------------------
int orc_gauss_legendre(int n, double* x, double* w) { return gauss_legendre(n, x, w) ? 0 : -1; }

// tab: [ng][nxi+1][nns], wts: [ng].  Returns nns*1000+ng on success so callers can size arrays
// (call with tab == nullptr first).
int orc_tp_basis(int nxi, const int* order, const int* ngauss, double* tab, double* wts) {
  TPBasis b;
  if (!make_tp_basis(nxi, order, ngauss, b)) return -1;
  if (tab) std::memcpy(tab, b.tab.data(), b.tab.size() * sizeof(double));
  if (wts) std::memcpy(wts, b.wts.data(), b.wts.size() * sizeof(double));
  return b.nns * 1000 + b.ng;
}

// ---------------------------------------------------------------------------------------
// Regular generated mesh.  src/generated_mesh_routines.F90:1568-1640: elements stepped
// xi1 fastest; first element node np = 1+(ne1-1)(nn1-1)+(ne2-1)NX(nn2-1)+(ne3-1)NX NY(nn3-1);
// element nodes xi1 fastest.  Output 0-based node numbers, elem_nodes[E][nns].
// ---------------------------------------------------------------------------------------
int orc_regular_mesh(int nxi, const int* nelem, int order, int32_t* elem_nodes) {
  int ne[3] = {1, 1, 1}, nnx[3] = {1, 1, 1}, tot[3] = {1, 1, 1};
  for (int d = 0; d < nxi; ++d) {
    ne[d] = nelem[d];
    nnx[d] = order + 1;
    tot[d] = (nnx[d] - 1) * ne[d] + 1;
  }
  const int nns = nnx[0] * nnx[1] * nnx[2];
  for (int e3 = 0; e3 < ne[2]; ++e3)
    for (int e2 = 0; e2 < ne[1]; ++e2)
      for (int e1 = 0; e1 < ne[0]; ++e1) {
        int e = e1 + ne[0] * (e2 + ne[1] * e3);
        int np = e1 * (nnx[0] - 1) + e2 * tot[0] * (nnx[1] - 1) + e3 * tot[0] * tot[1] * (nnx[2] - 1);
        int nn = 0;
        for (int a3 = 0; a3 < nnx[2]; ++a3)
          for (int a2 = 0; a2 < nnx[1]; ++a2)
            for (int a1 = 0; a1 < nnx[0]; ++a1)
              elem_nodes[(size_t)e * nns + nn++] = np + a1 + a2 * tot[0] + a3 * tot[0] * tot[1];
      }
  return 0;
}

// Node coordinates of a regular mesh, separated layout coords[comp][N].
// src/generated_mesh_routines.F90:3217-3383: value = origin + (position-1) * extent/(nodes_xi-1).
int orc_regular_coords(int nxi, const int* nelem, int order, const double* origin, const double* extent,
                       double* coords) {
  int tot[3] = {1, 1, 1};
  for (int d = 0; d < nxi; ++d) tot[d] = order * nelem[d] + 1;
  const size_t N = (size_t)tot[0] * tot[1] * tot[2];
  for (int k = 0; k < tot[2]; ++k)
    for (int j = 0; j < tot[1]; ++j)
      for (int i = 0; i < tot[0]; ++i) {
        size_t n = i + (size_t)tot[0] * (j + (size_t)tot[1] * k);
        const int p[3] = {i, j, k};
        for (int c = 0; c < nxi; ++c) coords[c * N + n] = origin[c] + (double)p[c] * (extent[c] / (double)(tot[c] - 1));
      }
  return 0;
}

// Second (linear) mesh component of a mesh whose first basis is quadratic:
// src/generated_mesh_routines.F90:4941-5100 takes the corner nodes' user numbers from the first
// basis (GLOBAL_ELEMENT_NODES of the corner local nodes); the linear component's own node
// numbers are the rank of those global numbers in ascending order
// (src/mesh_routines.F90:9159-9272, tree of global nodes detached in order).
// Outputs: elem_lin[E][2^nxi] (component-local 0-based numbers), lin_to_global[n_lin]
// (0-based first-basis node), returns n_lin.
int orc_linear_component(int nxi, int n_elem, int nns_first, const int* nnx_first, const int32_t* elem_first,
                         int32_t* elem_lin, int32_t* lin_to_global) {
  const int ncorner = 1 << nxi;
  std::vector<int32_t> corners((size_t)n_elem * ncorner);
  for (int e = 0; e < n_elem; ++e) {
    int c = 0;
    for (int b3 = 0; b3 < (nxi > 2 ? 2 : 1); ++b3)
      for (int b2 = 0; b2 < (nxi > 1 ? 2 : 1); ++b2)
        for (int b1 = 0; b1 < 2; ++b1) {
          int a1 = b1 ? nnx_first[0] - 1 : 0;
          int a2 = b2 ? nnx_first[1] - 1 : 0;
          int a3 = b3 ? nnx_first[2] - 1 : 0;
          int ns = a1 + nnx_first[0] * (a2 + nnx_first[1] * a3);
          corners[(size_t)e * ncorner + c++] = elem_first[(size_t)e * nns_first + ns];
        }
  }
  std::vector<int32_t> sorted(corners);
  std::sort(sorted.begin(), sorted.end());
  sorted.erase(std::unique(sorted.begin(), sorted.end()), sorted.end());
  for (size_t i = 0; i < corners.size(); ++i)
    elem_lin[i] = (int32_t)(std::lower_bound(sorted.begin(), sorted.end(), corners[i]) - sorted.begin());
  if (lin_to_global) std::copy(sorted.begin(), sorted.end(), lin_to_global);
  return (int)sorted.size();
}

// ---------------------------------------------------------------------------------------
// CSR structure.  src/equations_matrices_routines.F90:4399-4457 (EquationsMatrix_StructureCalculate,
// FEM + compressed-row): for each row DOF, loop the surrounding elements of its node and add
// every DOF of every component of those elements; List_RemoveDuplicates sorts ascending and
// removes duplicates (src/lists.F90:2652-2700); rowIndices(i+1) = nnz+1 (1-based).
// Input: per-element DOF lists elem_dofs[E][ndpe] (0-based global DOF numbers; an element
// "surrounds" a DOF's node exactly when the DOF is in its list).
// Call with col_idx == nullptr to get nnz only.
// ---------------------------------------------------------------------------------------
int64_t orc_csr_structure(int n_elem, int ndpe, const int32_t* elem_dofs, int n_dofs, int32_t* row_ptr,
                          int32_t* col_idx) {
  std::vector<int64_t> cnt(n_dofs + 1, 0);
  for (size_t i = 0; i < (size_t)n_elem * ndpe; ++i) cnt[elem_dofs[i] + 1]++;
  for (int i = 0; i < n_dofs; ++i) cnt[i + 1] += cnt[i];
  std::vector<int32_t> dof_elems(cnt[n_dofs]);
  std::vector<int64_t> fill(cnt.begin(), cnt.end() - 1);
  for (int e = 0; e < n_elem; ++e)
    for (int k = 0; k < ndpe; ++k) dof_elems[fill[elem_dofs[(size_t)e * ndpe + k]]++] = e;
  int64_t nnz = 0;
  std::vector<int32_t> list;
  if (row_ptr) row_ptr[0] = 1;
  for (int r = 0; r < n_dofs; ++r) {
    list.clear();
    for (int64_t s = cnt[r]; s < cnt[r + 1]; ++s) {
      int e = dof_elems[s];
      for (int k = 0; k < ndpe; ++k) list.push_back(elem_dofs[(size_t)e * ndpe + k] + 1);
    }
    std::sort(list.begin(), list.end());
    list.erase(std::unique(list.begin(), list.end()), list.end());
    if (col_idx) std::copy(list.begin(), list.end(), col_idx + nnz);
    nnz += (int64_t)list.size();
    if (row_ptr) row_ptr[r + 1] = (int32_t)(nnz + 1);
  }
  return nnz;
}

// Single CSR location lookup (src/matrix_vector.F90:1724-1860 MATRIX_STORAGE_LOCATION_FIND);
// returns the 1-based location or 0 when absent.  row, col 1-based.
int64_t orc_csr_location(const int32_t* rp, const int32_t* ci, int row, int col) {
  int lo = rp[row - 1], up = rp[row];
  if (up <= lo) return 0;
  if (col < ci[lo - 1] || col > ci[up - 2]) return 0;
  while (up - lo > kBisectionToLinear) {
    int mid = lo + (up - lo) / 2;
    if (ci[mid - 1] > col) up = mid; else lo = mid;
  }
  for (int k = lo; k < up; ++k)
    if (ci[k - 1] == col) return k;
  return 0;
}

// ---------------------------------------------------------------------------------------
// Laplace element matrix.  src/Laplace_equations_routines.F90:482-552 (standard subtype):
// per Gauss point interpolate geometry with first derivatives, metrics, RWG = Jacobian*w,
// K(ms,ns) += sum_{mi,ni} dphi_ms/dxi_mi * dphi_ns/dxi_ni * GU(mi,ni) * RWG.  RHS = 0 (:546).
// Generalised subtype (:585-707) with an isotropic, element-constant conductivity kappa*I
// rotates kappa*I into xi space (unchanged, the rotation of a multiple of the identity is the
// identity) and reduces to kappa times the standard integrand; the oracle applies kappa per
// Gauss-point term.
// x: element geometric parameters x[comp][ns] (ns < nns), out: K[nns][nns] row-major.
// ---------------------------------------------------------------------------------------
void laplace_element(const TPBasis& b, const double* const* x, int ncomp, double kappa, double* K) {
  const int n = b.nns, nxi = b.nxi;
  std::fill(K, K + (size_t)n * n, 0.0);
  Metrics m;
  for (int g = 0; g < b.ng; ++g) {
    metrics_at(b, g, x, ncomp, m);
    const double rwg = m.jac * b.wts[g];
    for (int ms = 0; ms < n; ++ms) {
      double pgm[3];
      for (int i = 0; i < nxi; ++i) pgm[i] = b.tab[((size_t)g * (nxi + 1) + i + 1) * n + ms];
      for (int ns = 0; ns < n; ++ns) {
        double pgn[3];
        for (int i = 0; i < nxi; ++i) pgn[i] = b.tab[((size_t)g * (nxi + 1) + i + 1) * n + ns];
        double sum = 0.0;
        for (int mi = 0; mi < nxi; ++mi)
          for (int ni = 0; ni < nxi; ++ni) sum += pgm[mi] * pgn[ni] * m.gu[mi][ni];
        K[(size_t)ms * n + ns] += kappa * sum * rwg;
      }
    }
  }
}

// ---------------------------------------------------------------------------------------
// Generalised Laplace: a full conductivity tensor in a material frame.
// src/Laplace_equations_routines.F90:585-707 (EQUATIONS_SET_GENERALISED_LAPLACE_SUBTYPE): per
// Gauss point the materials field gives the conductivity in material coordinates (3D order
// K11 K22 K33 K12 K23 K13, 2D K11 K22 K12, :640-656), Coordinates_MaterialSystemCalculate gives
// dNudXi and dXidNu (src/coordinate_routines.F90:3841-3947), the conductivity in xi space is
// dNudXi * K * dXidNu (:665-670), and
//   K(ms,ns) += RWG * sum_{i,k,h} C(i,k) * dphi_ns/dxi_k * dphi_ms/dxi_h * GU(i,h)   (:680-693).
// The RHS is zero.
// ---------------------------------------------------------------------------------------
void normalise3(int n, const double* a, double* out) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += a[i] * a[i];
  const double l = std::sqrt(s);
  for (int i = 0; i < n; ++i) out[i] = a[i] / l;
}

void cross3(const double* a, const double* b, double* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

void matmul3(int n, const double A[3][3], const double B[3][3], double C[3][3]) {
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double s = 0.0;
      for (int k = 0; k < n; ++k) s += A[i][k] * B[k][j];
      C[i][j] = s;
    }
}

// dX/dNu of the material frame.  With fibre angles: the reference frame f = DX_DXI(:,1),
// h = f x DX_DXI(:,2), g = h x f (normalised), rotated by the fibre angle about axis 3, the
// imbrication angle about the new axis 2 and the sheet angle about the new axis 1
// (Coordinates_MaterialSystemCalculatedXdNu3D, src/coordinate_routines.F90:4020-4127); in 2D
// f = DX_DXI(:,1), g = (-f2, f1), R(angle) * [f g] with normalised columns (:3952-4000).
// Without a fibre field: the normalised columns of DX_DXI (:3879-3884).
void material_dxdnu(int nd, const Metrics& m, const double* angle, int n_angles, double dXdNu[3][3]) {
  std::memset(dXdNu, 0, sizeof(double) * 9);
  if (!angle) {
    for (int xi = 0; xi < nd; ++xi) {
      double c[3] = {m.dx_dxi[0][xi], m.dx_dxi[1][xi], m.dx_dxi[2][xi]}, o[3];
      normalise3(nd, c, o);
      for (int i = 0; i < nd; ++i) dXdNu[i][xi] = o[i];
    }
    return;
  }
  if (nd == 2) {
    double f[2] = {m.dx_dxi[0][0], m.dx_dxi[1][0]}, g[2] = {-f[1], f[0]}, fn[2], gn[2];
    normalise3(2, f, fn);
    normalise3(2, g, gn);
    const double R[3][3] = {{std::cos(angle[0]), std::sin(angle[0]), 0.0}, {-std::sin(angle[0]), std::cos(angle[0]), 0.0},
                            {0.0, 0.0, 0.0}};
    const double Rf[3][3] = {{fn[0], gn[0], 0.0}, {fn[1], gn[1], 0.0}, {0.0, 0.0, 0.0}};
    double P[3][3];
    matmul3(2, R, Rf, P);
    for (int c = 0; c < 2; ++c) {
      double col[2] = {P[0][c], P[1][c]}, o[2];
      normalise3(2, col, o);
      dXdNu[0][c] = o[0];
      dXdNu[1][c] = o[1];
    }
    return;
  }
  double a[3] = {0.0, 0.0, 0.0};
  for (int i = 0; i < n_angles && i < 3; ++i) a[i] = angle[i];
  double f[3] = {m.dx_dxi[0][0], m.dx_dxi[1][0], m.dx_dxi[2][0]};
  double d2[3] = {m.dx_dxi[0][1], m.dx_dxi[1][1], m.dx_dxi[2][1]};
  double h[3], g[3], fn[3], gn[3], hn[3];
  cross3(f, d2, h);
  cross3(h, f, g);
  normalise3(3, f, fn);
  normalise3(3, g, gn);
  normalise3(3, h, hn);
  double R0[3][3];
  for (int i = 0; i < 3; ++i) {
    R0[i][0] = fn[i];
    R0[i][1] = gn[i];
    R0[i][2] = hn[i];
  }
  const double ca = std::cos(a[0]), sa = std::sin(a[0]), cb = std::cos(a[1]), sb = std::sin(a[1]),
               cg = std::cos(a[2]), sg = std::sin(a[2]);
  const double Rz[3][3] = {{ca, -sa, 0.0}, {sa, ca, 0.0}, {0.0, 0.0, 1.0}};
  const double Ry[3][3] = {{cb, 0.0, sb}, {0.0, 1.0, 0.0}, {-sb, 0.0, cb}};
  const double Rx[3][3] = {{1.0, 0.0, 0.0}, {0.0, cg, -sg}, {0.0, sg, cg}};
  double T1[3][3], T2[3][3];
  matmul3(3, R0, Rz, T1);
  matmul3(3, T1, Ry, T2);
  matmul3(3, T2, Rx, dXdNu);
}

// Iron's material conductivity tensor from the materials field components (:640-656).
void conductivity_material(int nd, const double* k, double K[3][3]) {
  std::memset(K, 0, sizeof(double) * 9);
  if (nd == 2) {
    K[0][0] = k[0]; K[1][1] = k[1]; K[0][1] = K[1][0] = k[2];
  } else {
    K[0][0] = k[0]; K[1][1] = k[1]; K[2][2] = k[2];
    K[0][1] = K[1][0] = k[3];
    K[1][2] = K[2][1] = k[4];
    K[0][2] = K[2][0] = k[5];
  }
}

// x: element geometric parameters x[comp][ns]; cond: the element's conductivity components
// (element-constant materials field); fib: the element's fibre parameters fib[angle][ns]
// (interpolated with the element basis) or nullptr for no fibre field.
void laplace_element_generalised(const TPBasis& b, const double* const* x, const double* cond,
                                 const double* const* fib, int n_angles, double* K) {
  const int n = b.nns, nd = b.nxi;
  std::fill(K, K + (size_t)n * n, 0.0);
  Metrics m;
  double Km[3][3];
  conductivity_material(nd, cond, Km);
  for (int g = 0; g < b.ng; ++g) {
    metrics_at(b, g, x, nd, m);
    const double rwg = m.jac * b.wts[g];
    double ang[3] = {0.0, 0.0, 0.0};
    if (fib) {
      const double* phi = &b.tab[((size_t)g * (nd + 1)) * n];
      for (int a = 0; a < n_angles; ++a) {
        double s = 0.0;
        for (int ns = 0; ns < n; ++ns) s += phi[ns] * fib[a][ns];
        ang[a] = s;
      }
    }
    double dXdNu[3][3], dNudX[3][3], dNudXi[3][3], dXidNu[3][3], T[3][3], C[3][3];
    material_dxdnu(nd, m, fib ? ang : nullptr, n_angles, dXdNu);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) dNudX[i][j] = dXdNu[j][i];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) dNudXi[i][j] = i == j ? 1.0 : 0.0;
    double P[3][3];
    matmul3(nd, dNudX, m.dx_dxi, P);
    for (int i = 0; i < nd; ++i)
      for (int j = 0; j < nd; ++j) dNudXi[i][j] = P[i][j];
    invert(nd, dNudXi, dXidNu);
    matmul3(nd, dNudXi, Km, T);
    matmul3(nd, T, dXidNu, C);
    for (int ms = 0; ms < n; ++ms) {
      double pgm[3];
      for (int i = 0; i < nd; ++i) pgm[i] = b.tab[((size_t)g * (nd + 1) + i + 1) * n + ms];
      for (int ns = 0; ns < n; ++ns) {
        double pgn[3];
        for (int i = 0; i < nd; ++i) pgn[i] = b.tab[((size_t)g * (nd + 1) + i + 1) * n + ns];
        double sum = 0.0;
        for (int i = 0; i < nd; ++i)
          for (int k = 0; k < nd; ++k)
            for (int h = 0; h < nd; ++h) sum += C[i][k] * pgn[k] * pgm[h] * m.gu[i][h];
        K[(size_t)ms * n + ns] += sum * rwg;
      }
    }
  }
}

int orc_laplace_generalised_element(int nxi, const int* order, const int* ngauss, const double* xe,
                                    const double* cond, const double* fe /*[n_angles][nns] or null*/, int n_angles,
                                    double* K) {
  TPBasis b;
  if (!make_tp_basis(nxi, order, ngauss, b)) return -1;
  const double* x[3] = {xe, xe + b.nns, xe + 2 * b.nns};
  const double* f[3] = {fe, fe ? fe + b.nns : nullptr, fe ? fe + 2 * b.nns : nullptr};
  laplace_element_generalised(b, x, cond, fe ? f : nullptr, n_angles, K);
  return 0;
}

// Whole-mesh generalised assembly (the loop of orc_laplace_assemble_scaled without scale
// factors).  cond [n_elem][ncond] element-constant conductivity components; fibre [n_angles][N]
// nodal fibre angles (radians) or nullptr.
int orc_laplace_generalised_assemble(int nxi, const int* order, const int* ngauss, int n_elem, int n_nodes,
                                     const int32_t* elem_nodes, const double* coords, const double* cond,
                                     const double* fibre, int n_angles, const int32_t* row_ptr,
                                     const int32_t* col_idx, double* values, double* rhs) {
  TPBasis b;
  if (!make_tp_basis(nxi, order, ngauss, b)) return -1;
  const int n = b.nns, ncond = nxi == 2 ? 3 : 6;
  const int64_t nnz = (int64_t)row_ptr[n_nodes] - 1;
  std::fill(values, values + nnz, 0.0);
  if (rhs) std::fill(rhs, rhs + n_nodes, 0.0);
  std::vector<double> xe((size_t)nxi * n), fe((size_t)3 * n), K((size_t)n * n);
  std::vector<int32_t> dofs(n);
  const double* x[3] = {xe.data(), xe.data() + n, xe.data() + 2 * n};
  const double* f[3] = {fe.data(), fe.data() + n, fe.data() + 2 * n};
  for (int e = 0; e < n_elem; ++e) {
    for (int s = 0; s < n; ++s) {
      const int node = elem_nodes[(size_t)e * n + s];
      dofs[s] = node + 1;
      for (int c = 0; c < nxi; ++c) xe[(size_t)c * n + s] = coords[(size_t)c * n_nodes + node];
      if (fibre)
        for (int a = 0; a < n_angles; ++a) fe[(size_t)a * n + s] = fibre[(size_t)a * n_nodes + node];
    }
    laplace_element_generalised(b, x, cond + (size_t)e * ncond, fibre ? f : nullptr, n_angles, K.data());
    if (csr_values_add(row_ptr, col_idx, values, n, dofs.data(), n, dofs.data(), K.data()) != 0) return -2;
  }
  return 0;
}

// Element matrix of one element of a (possibly 2D) Lagrange mesh.
int orc_laplace_element(int nxi, const int* order, const int* ngauss, int ncomp, const double* xe /*[ncomp][nns]*/,
                        double kappa, double* K) {
  TPBasis b;
  if (!make_tp_basis(nxi, order, ngauss, b)) return -1;
  const double* x[3] = {xe, xe + b.nns, xe + 2 * b.nns};
  laplace_element(b, x, ncomp, kappa, K);
  return 0;
}

// Whole-mesh assembly, following src/equations_set_routines.F90:1203-1364
// (EquationsSet_AssembleStaticLinearFEM): zero the matrix (EquationsMatrices_VectorValuesInitialise
// :4206 of equations_matrices_routines.F90), then per element: gather element geometric parameters
// (FIELD_INTERPOLATION_PARAMETERS_ELEMENT_GET, src/field_routines.F90:8042-8260), element matrix,
// EquationsMatrices_ElementAdd (src/equations_matrices_routines.F90:1140-1265) with row DOFs =
// column DOFs = element node DOFs (one component, one domain).
// n_threads > 1: element-partitioned threads with private value copies summed at the end
// (used for the multi-core CPU baseline only).
// scale (optional) [n_elem][nns]: element parameter scale factors.  The geometric parameters are
// interpolated scaled (FIELD_INTERPOLATION_PARAMETERS_ELEMENT_GET multiplies them by the scale
// factors), and the element matrix is scaled as K(ms, ns) * SF(ms) * SF(ns)
// (src/Laplace_equations_routines.F90:555-579).  elem_nodes then holds element parameter DOFs
// and coords the parameters per DOF.
int orc_laplace_assemble_scaled(int nxi, const int* order, const int* ngauss, int n_elem, int n_nodes,
                                const int32_t* elem_nodes, const double* coords /*[nxi][N]*/, const double* scale,
                                const double* kappa, const int32_t* row_ptr, const int32_t* col_idx, double* values,
                                double* rhs, int n_threads) {
  TPBasis b;
  if (!make_tp_basis(nxi, order, ngauss, b)) return -1;
  const int n = b.nns;
  const int64_t nnz = (int64_t)row_ptr[n_nodes] - 1;
  std::fill(values, values + nnz, 0.0);
  if (rhs) std::fill(rhs, rhs + n_nodes, 0.0);
  if (n_threads < 1) n_threads = 1;
  std::vector<std::vector<double>> priv(n_threads > 1 ? n_threads : 0);
  std::vector<int> status(n_threads, 0);
  auto work = [&](int t, int e0, int e1, double* out) {
    std::vector<double> xe((size_t)nxi * n), K((size_t)n * n);
    std::vector<int32_t> dofs(n);
    const double* x[3] = {xe.data(), xe.data() + n, xe.data() + 2 * n};
    for (int e = e0; e < e1; ++e) {
      for (int s = 0; s < n; ++s) {
        int node = elem_nodes[(size_t)e * n + s];
        dofs[s] = node + 1;
        const double sf = scale ? scale[(size_t)e * n + s] : 1.0;
        for (int c = 0; c < nxi; ++c) xe[(size_t)c * n + s] = coords[(size_t)c * n_nodes + node] * sf;
      }
      laplace_element(b, x, nxi, kappa ? kappa[e] : 1.0, K.data());
      if (scale)
        for (int ms = 0; ms < n; ++ms)
          for (int ns = 0; ns < n; ++ns)
            K[(size_t)ms * n + ns] = K[(size_t)ms * n + ns] * scale[(size_t)e * n + ms] * scale[(size_t)e * n + ns];
      if (csr_values_add(row_ptr, col_idx, out, n, dofs.data(), n, dofs.data(), K.data()) != 0) {
        status[t] = -2;
        return;
      }
    }
  };
  if (n_threads == 1) {
    work(0, 0, n_elem, values);
  } else {
    std::vector<std::thread> th;
    for (int t = 0; t < n_threads; ++t) {
      priv[t].assign(nnz, 0.0);
      int e0 = (int)((int64_t)n_elem * t / n_threads), e1 = (int)((int64_t)n_elem * (t + 1) / n_threads);
      th.emplace_back(work, t, e0, e1, priv[t].data());
    }
    for (auto& x : th) x.join();
    for (int t = 0; t < n_threads; ++t)
      for (int64_t k = 0; k < nnz; ++k) values[k] += priv[t][k];
  }
  for (int s : status)
    if (s) return s;
  return 0;
}

int orc_laplace_assemble(int nxi, const int* order, const int* ngauss, int n_elem, int n_nodes,
                         const int32_t* elem_nodes, const double* coords, const double* kappa,
                         const int32_t* row_ptr, const int32_t* col_idx, double* values, double* rhs,
                         int n_threads) {
  return orc_laplace_assemble_scaled(nxi, order, ngauss, n_elem, n_nodes, elem_nodes, coords, nullptr, kappa, row_ptr,
                                     col_idx, values, rhs, n_threads);
}

// ---------------------------------------------------------------------------------------
// Sparse kernels used by the oracle's solve.  CSR 1-based.
// ---------------------------------------------------------------------------------------
void orc_csr_spmv(int n, const int32_t* rp, const int32_t* ci, const double* v, const double* x, double* y) {
  for (int r = 0; r < n; ++r) {
    double s = 0.0;
    for (int k = rp[r] - 1; k < rp[r + 1] - 1; ++k) s += v[k] * x[ci[k] - 1];
    y[r] = s;
  }
}

// ---------------------------------------------------------------------------------------
// Solver system of one linear equations set with Dirichlet conditions on one rank.
//  * Solver mapping, src/solver_mapping_routines.F90:398-520: an equations row is a solver row
//    iff its dependent DOF is free; solver rows (and, for the square system, columns) are
//    numbered in ascending global order.
//  * Structure, SOLVER_MATRIX_STRUCTURE_CALCULATE src/solver_matrices_routines.F90:1612-2431
//    (compressed-row branch): per solver row, the solver columns of the equations row's free
//    columns, then LIST_REMOVE_DUPLICATES (sort + unique), stored 1-based.
//  * Values, SOLVER_MATRIX_EQUATIONS_MATRIX_ADD src/solver_matrices_routines.F90:806-1023
//    (compressed-row branch): the zeroed solver matrix receives
//    ALPHA * K(row, col) * row_coupling * column_coupling at (solver row, solver column), found
//    by the CSR search of MATRIX_VALUES_ADD_DP2, with ALPHA = coupling coefficients = 1.
//  * Right-hand side, SOLVER_MATRICES_STATIC_ASSEMBLE src/solver_routines.F90:14025-15050 (the
//    linear branch of the RHS loop): the zeroed solver RHS receives, for each equations row r in
//    ascending order, f(r) on r's solver row (the RHS variable is free everywhere here), and, if
//    r's dependent DOF is fixed with |u(r)| >= ZERO_TOLERANCE, -1 * K(i, r) * u(r) on the solver
//    row of every row i of column r's list with |K(i, r)| >= ZERO_TOLERANCE.  Column lists hold
//    the rows of the column in ascending order, and only for columns on boundary nodes
//    (src/equations_matrices_routines.F90:4531-4561, src/boundary_condition_routines.F90:459-500);
//    col_listed (optional) marks those columns, NULL lists every column.
//  ZERO_TOLERANCE = 5 * EPSILON(1.0_DP) (src/constants.F90:69).
// rp/ci 1-based (n rows); f may be NULL (a zero equations RHS).  Outputs: solver_of_dof[n]
// (0-based solver number or -1), s_rp[n_free + 1], s_ci, s_v (capacity cap), s_rhs[n_free].
// Returns the solver nnz, or -1 if cap is too small.
// ---------------------------------------------------------------------------------------
int64_t orc_solver_system(int n, const int32_t* rp, const int32_t* ci, const double* v, const double* f,
                          const uint8_t* fixed, const uint8_t* col_listed, const double* u, int32_t* solver_of_dof,
                          int32_t* s_rp, int32_t* s_ci, double* s_v, double* s_rhs, int64_t cap, int32_t* n_free) {
  const double zero_tol = 5.0 * 2.220446049250313e-16;
  int nf = 0;
  for (int r = 0; r < n; ++r) solver_of_dof[r] = fixed[r] ? -1 : nf++;
  *n_free = nf;
  // structure
  int64_t nnz = 0;
  s_rp[0] = 1;
  std::vector<int32_t> cols;
  for (int r = 0; r < n; ++r) {
    if (fixed[r]) continue;
    cols.clear();
    for (int k = rp[r] - 1; k < rp[r + 1] - 1; ++k) {
      const int c = ci[k] - 1;
      if (!fixed[c]) cols.push_back(solver_of_dof[c] + 1);
    }
    std::sort(cols.begin(), cols.end());
    cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
    if (nnz + (int64_t)cols.size() > cap) return -1;
    for (int32_t c : cols) s_ci[nnz++] = c;
    s_rp[solver_of_dof[r] + 1] = (int32_t)(nnz + 1);
  }
  // values
  std::fill(s_v, s_v + nnz, 0.0);
  for (int r = 0; r < n; ++r) {
    if (fixed[r]) continue;
    const int sr = solver_of_dof[r] + 1;
    for (int k = rp[r] - 1; k < rp[r + 1] - 1; ++k) {
      const int c = ci[k] - 1;
      if (fixed[c]) continue;
      const double value = 1.0 * v[k] * 1.0 * 1.0;
      const int64_t loc = orc_csr_location(s_rp, s_ci, sr, solver_of_dof[c] + 1);
      if (loc == 0) return -1;
      s_v[loc - 1] += value;
    }
  }
  // right-hand side: column lists (rows ascending) of the listed fixed columns
  std::vector<std::vector<int32_t>> lists(n);
  for (int i = 0; i < n; ++i)
    for (int k = rp[i] - 1; k < rp[i + 1] - 1; ++k) {
      const int c = ci[k] - 1;
      if (fixed[c] && (!col_listed || col_listed[c])) lists[c].push_back(i);
    }
  std::fill(s_rhs, s_rhs + nf, 0.0);
  for (int r = 0; r < n; ++r) {
    if (!fixed[r]) s_rhs[solver_of_dof[r]] += (f ? f[r] : 0.0) * 1.0;
    if (!fixed[r] || !(std::fabs(u[r]) >= zero_tol)) continue;
    for (int32_t i : lists[r]) {
      const int64_t loc = orc_csr_location(rp, ci, i + 1, r + 1);
      const double kv = loc ? v[loc - 1] : 0.0;
      if (!(std::fabs(kv) >= zero_tol) || fixed[i]) continue;
      s_rhs[solver_of_dof[i]] += -1.0 * kv * u[r] * 1.0;
    }
  }
  return nnz;
}

// Dirichlet-eliminated Jacobi-preconditioned conjugate gradients in FP64.
// The solver matrix of src/solver_routines.F90:14025-15050 (SOLVER_MATRICES_STATIC_ASSEMBLE)
// removes the rows and columns of fixed DOFs and moves K_FD u_D to the right-hand side; the
// same system is solved here in the full index space with fixed DOFs masked.  Iron hands the
// system to PETSc KSP (src/solver_routines.F90:11775-11991); PETSc's CG is not restated, so the
// solve is parity-unpinned and compared by solution tolerance only.
// x: in = Dirichlet values at fixed DOFs (others ignored), out = solution.  Returns iterations
// or -1 on failure to converge.
int orc_cg_dirichlet(int n, const int32_t* rp, const int32_t* ci, const double* v, const double* f,
                     const uint8_t* fixed, double* x, double rtol, int max_it, double* final_rel) {
  std::vector<double> r(n), z(n), p(n), q(n), dinv(n), xd(n, 0.0);
  for (int i = 0; i < n; ++i) {
    if (fixed[i]) xd[i] = x[i];
    double d = 0.0;
    for (int k = rp[i] - 1; k < rp[i + 1] - 1; ++k)
      if (ci[k] - 1 == i) d = v[k];
    dinv[i] = fixed[i] ? 0.0 : 1.0 / d;
  }
  orc_csr_spmv(n, rp, ci, v, xd.data(), q.data());
  double bnorm = 0.0;
  for (int i = 0; i < n; ++i) {
    r[i] = fixed[i] ? 0.0 : (f ? f[i] : 0.0) - q[i];
    x[i] = fixed[i] ? xd[i] : 0.0;
    bnorm += r[i] * r[i];
  }
  bnorm = std::sqrt(bnorm);
  if (bnorm == 0.0) { if (final_rel) *final_rel = 0.0; return 0; }
  double rz = 0.0;
  for (int i = 0; i < n; ++i) { z[i] = dinv[i] * r[i]; p[i] = z[i]; rz += r[i] * z[i]; }
  for (int it = 1; it <= max_it; ++it) {
    for (int i = 0; i < n; ++i) xd[i] = fixed[i] ? 0.0 : p[i];
    orc_csr_spmv(n, rp, ci, v, xd.data(), q.data());
    double pq = 0.0;
    for (int i = 0; i < n; ++i) { if (fixed[i]) q[i] = 0.0; pq += p[i] * q[i]; }
    double alpha = rz / pq, rn = 0.0;
    for (int i = 0; i < n; ++i) {
      if (fixed[i]) continue;
      x[i] += alpha * p[i];
      r[i] -= alpha * q[i];
      rn += r[i] * r[i];
    }
    rn = std::sqrt(rn);
    if (rn <= rtol * bnorm) { if (final_rel) *final_rel = rn / bnorm; return it; }
    double rz2 = 0.0;
    for (int i = 0; i < n; ++i) { z[i] = dinv[i] * r[i]; rz2 += r[i] * z[i]; }
    double beta = rz2 / rz;
    rz = rz2;
    for (int i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
  }
  return -1;
}

}  // extern "C"

// =========================================================================================
// Finite elasticity, Mooney-Rivlin subtype, mixed u-p (triquadratic u + trilinear p), 3D.
// =========================================================================================
namespace {

// Voigt maps, src/constants.F90:305-306: 1=(1,1) 2=(2,2) 3=(3,3) 4=(1,2) 5=(1,3) 6=(2,3).
const int kT2V[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};
const int kV2T[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};

struct MRBases {
  TPBasis q2;  // dependent / geometric basis
  TPBasis q1;  // pressure basis (same Gauss scheme)
};

const MRBases& mr_bases(int ngauss) {
  static MRBases b2, b3, b4;
  MRBases* b = ngauss == 2 ? &b2 : (ngauss == 3 ? &b3 : &b4);
  if (b->q2.nns == 0) {
    int o2[3] = {2, 2, 2}, o1[3] = {1, 1, 1}, g[3] = {ngauss, ngauss, ngauss};
    make_tp_basis(3, o2, g, b->q2);
    make_tp_basis(3, o1, g, b->q1);
  }
  return *b;
}

void matmul3(const double A[3][3], const double B[3][3], double C[3][3]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int k = 0; k < 3; ++k) s += A[i][k] * B[k][j];
      C[i][j] = s;
    }
}

// Deformation gradient dZ/dNu, src/finite_elasticity_routines.F90:5148-5215, with the material
// frame of src/coordinate_routines.F90:3841-3947 when there is no fibre field: dX/dNu columns are
// the normalised columns of DX_DXI (geometry); dNu/dXi = (dX/dNu)^T DX_DXI; dXi/dNu = inv(dNu/dXi).
void deformation_gradient(const Metrics& mz, const Metrics& mx, double F[3][3]) {
  double dXdNu[3][3], dNudX[3][3], dNudXi[3][3], dXidNu[3][3];
  for (int xi = 0; xi < 3; ++xi) {
    double n = std::sqrt(mx.dx_dxi[0][xi] * mx.dx_dxi[0][xi] + mx.dx_dxi[1][xi] * mx.dx_dxi[1][xi] +
                         mx.dx_dxi[2][xi] * mx.dx_dxi[2][xi]);
    for (int c = 0; c < 3; ++c) dXdNu[c][xi] = mx.dx_dxi[c][xi] / n;
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) dNudX[i][j] = dXdNu[j][i];
  matmul3(dNudX, mx.dx_dxi, dNudXi);
  invert(3, dNudXi, dXidNu);
  matmul3(mz.dx_dxi, dXidNu, F);
}

// Push-forward of a Voigt 2nd-order tensor, src/finite_elasticity_routines.F90:1343-1375:
// t(i,j) = F(a_i,a_j)F(b_i,b_j) (+ F(a_i,b_j)F(b_i,a_j) for shear columns), S <- t S / J.
void push_tensor_t(const double F[3][3], double t[6][6]) {
  for (int j = 0; j < 6; ++j)
    for (int i = 0; i < 6; ++i) {
      const int ai = kV2T[i][0], bi = kV2T[i][1], aj = kV2T[j][0], bj = kV2T[j][1];
      double v = F[ai][aj] * F[bi][bj];
      if (j >= 3) v += F[ai][bj] * F[bi][aj];
      t[i][j] = v;
    }
}

void push_stress(double S[6], const double F[3][3], double J) {
  double t[6][6], out[6];
  push_tensor_t(F, t);
  for (int i = 0; i < 6; ++i) {
    double s = 0.0;
    for (int j = 0; j < 6; ++j) s += t[i][j] * S[j];
    out[i] = s / J;
  }
  for (int i = 0; i < 6; ++i) S[i] = out[i];
}

// src/finite_elasticity_routines.F90:1303-1336: D <- t D t^T / J
void push_elasticity(double D[6][6], const double F[3][3], double J) {
  double t[6][6], tmp[6][6];
  push_tensor_t(F, t);
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) {
      double s = 0.0;
      for (int k = 0; k < 6; ++k) s += t[i][k] * D[k][j];
      tmp[i][j] = s;
    }
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) {
      double s = 0.0;
      for (int k = 0; k < 6; ++k) s += tmp[i][k] * t[j][k];
      D[i][j] = s / J;
    }
}

// Cauchy stress of the MR subtype in the residual, src/finite_elasticity_routines.F90:6985-7061:
// Fbar = J^(-1/3) F, Cbar = Fbar^T Fbar, Sbar = -2 c2 Cbar + 2 (c1 + I1 c2) I (Voigt),
// sigma_bar = push(Sbar, Fbar, J), sigma = dev(sigma_bar) + p I.
void mr_cauchy_stress(const double F[3][3], double J, double p, double c1, double c2, double sig[6]) {
  double Fb[3][3], C[3][3];
  const double s = std::pow(J, -1.0 / 3.0);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) Fb[i][j] = F[i][j] * s;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double v = 0.0;
      for (int k = 0; k < 3; ++k) v += Fb[k][i] * Fb[k][j];
      C[i][j] = v;
    }
  const double I1 = C[0][0] + C[1][1] + C[2][2];
  const double t1 = -2.0 * c2, t2 = 2.0 * (c1 + I1 * c2);
  sig[0] = t1 * C[0][0] + t2; sig[1] = t1 * C[1][1] + t2; sig[2] = t1 * C[2][2] + t2;
  sig[3] = t1 * C[1][0]; sig[4] = t1 * C[2][0]; sig[5] = t1 * C[2][1];
  push_stress(sig, Fb, J);
  const double tr3 = (sig[0] + sig[1] + sig[2]) / 3.0;
  for (int i = 0; i < 3; ++i) sig[i] = sig[i] - tr3 + p;
}

struct MRPoint {
  Metrics mx, mz;
  double F[3][3], Jznu, p, dphidz[27][3], psi[8], w;
};

void mr_point(const MRBases& B, int g, const double* const* x, const double* const* z, const double* pe,
              MRPoint& P) {
  metrics_at(B.q2, g, z, 3, P.mz);
  metrics_at(B.q2, g, x, 3, P.mx);
  const int nns = B.q2.nns;
  for (int ns = 0; ns < nns; ++ns)
    for (int mh = 0; mh < 3; ++mh) {
      double s = 0.0;
      for (int mi = 0; mi < 3; ++mi) s += P.mz.dxi_dx[mi][mh] * B.q2.tab[((size_t)g * 4 + mi + 1) * nns + ns];
      P.dphidz[ns][mh] = s;
    }
  deformation_gradient(P.mz, P.mx, P.F);
  P.Jznu = P.mz.jac / P.mx.jac;
  P.w = B.q2.wts[g];
  double pv = 0.0;
  for (int ms = 0; ms < 8; ++ms) {
    P.psi[ms] = B.q1.tab[((size_t)g * 4 + 0) * 8 + ms];
    pv += P.psi[ms] * pe[ms];
  }
  P.p = pv;
}

// Element residual (89), src/finite_elasticity_routines.F90:1669-1756.
void mr_residual_element(const double* xg /*[3][27]*/, const double* zg /*[3][27]*/, const double* pe /*[8]*/,
                         double c1, double c2, double* R /*[89]*/, int ngauss = 3) {
  const MRBases& B = mr_bases(ngauss);
  const double* x[3] = {xg, xg + 27, xg + 54};
  const double* z[3] = {zg, zg + 27, zg + 54};
  std::fill(R, R + 89, 0.0);
  MRPoint P;
  for (int g = 0; g < B.q2.ng; ++g) {
    mr_point(B, g, x, z, pe, P);
    double sig[6];
    mr_cauchy_stress(P.F, P.Jznu, P.p, c1, c2, sig);
    const double jgw = P.mz.jac * P.w;
    double jgwc[3][3];
    for (int mh = 0; mh < 3; ++mh)
      for (int nh = 0; nh < 3; ++nh) jgwc[mh][nh] = jgw * sig[kT2V[mh][nh]];
    for (int mh = 0; mh < 3; ++mh)
      for (int ms = 0; ms < 27; ++ms) {
        double d = 0.0;
        for (int k = 0; k < 3; ++k) d += P.dphidz[ms][k] * jgwc[k][mh];
        R[mh * 27 + ms] += d;
      }
    const double tt = P.mx.jac * P.w * (P.Jznu - 1.0);
    for (int ms = 0; ms < 8; ++ms) R[81 + ms] += tt * P.psi[ms];
  }
}

// Iron's analytic element Jacobian (89x89, row-major K[mhs][nhs]),
// src/finite_elasticity_routines.F90:1016-1274 with FINITE_ELASTICITY_GAUSS_ELASTICITY_TENSOR :649-795.
void mr_jacobian_element(const double* xg, const double* zg, const double* pe, double c1, double c2,
                         double* K /*[89][89]*/, int ngauss = 3) {
  const MRBases& B = mr_bases(ngauss);
  const double* x[3] = {xg, xg + 27, xg + 54};
  const double* z[3] = {zg, zg + 27, zg + 54};
  std::fill(K, K + 89 * 89, 0.0);
  MRPoint P;
  for (int g = 0; g < B.q2.ng; ++g) {
    mr_point(B, g, x, z, pe, P);
    // elasticity tensor with the unmodified F (AZL = F^T F)
    double C[3][3], Ci[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double v = 0.0;
        for (int k = 0; k < 3; ++k) v += P.F[k][i] * P.F[k][j];
        C[i][j] = v;
      }
    const double I3 = invert(3, C, Ci);
    const double L[6] = {C[0][0], C[1][1], C[2][2], C[0][1], C[0][2], C[1][2]};
    const double U[6] = {Ci[0][0], Ci[1][1], Ci[2][2], Ci[0][1], Ci[0][2], Ci[1][2]};
    // I3EE filled column by column (Fortran RESHAPE), I3EE[row][col]
    const double cols[6][6] = {{0.0, 4 * L[2], 4 * L[1], 0.0, 0.0, -4 * L[5]},
                               {4 * L[2], 0.0, 4 * L[0], 0.0, -4 * L[4], 0.0},
                               {4 * L[1], 4 * L[0], 0.0, -2 * L[3], 0.0, 0.0},
                               {0.0, 0.0, -4 * L[3], -2 * L[2], 2 * L[5], 2 * L[4]},
                               {0.0, -4 * L[4], 0.0, 2 * L[5], -2 * L[1], 2 * L[3]},
                               {-4 * L[5], 0.0, 0.0, 2 * L[4], 2 * L[3], -2 * L[0]}};
    double D[6][6];
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 6; ++j) D[i][j] = 0.0;
    const double I1 = C[0][0] + C[1][1] + C[2][2];
    double S[6] = {-2 * c2 * C[0][0] + 2 * (c1 + I1 * c2), -2 * c2 * C[1][1] + 2 * (c1 + I1 * c2),
                   -2 * c2 * C[2][2] + 2 * (c1 + I1 * c2), -2 * c2 * C[1][0], -2 * c2 * C[2][0], -2 * c2 * C[2][1]};
    D[1][0] = D[2][0] = D[0][1] = D[2][1] = D[0][2] = D[1][2] = 4 * c2;
    D[3][3] = D[4][4] = D[5][5] = -2 * c2;
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 6; ++j) D[i][j] += P.p * (-2.0 * U[i] * U[j] + 0.5 * cols[j][i] / I3);
    double H[6] = {U[0], U[1], U[2], U[3], U[4], U[5]};
    push_stress(S, P.F, P.Jznu);
    push_stress(H, P.F, P.Jznu);
    push_elasticity(D, P.F, P.Jznu);
    for (int i = 0; i < 3; ++i) S[i] += P.p;
    double sig[3][3], hyd[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) { sig[i][j] = S[kT2V[i][j]]; hyd[i][j] = H[kT2V[i][j]]; }
    const double jgw = P.mz.jac * P.w;
    // diagonal component blocks, lower triangle ms >= ns
    for (int nh = 0; nh < 3; ++nh) {
      double sub[3][3];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) sub[i][j] = jgw * (D[kT2V[i][nh]][kT2V[j][nh]] + sig[i][j]);
      for (int ns = 0; ns < 27; ++ns) {
        double tv[3];
        for (int i = 0; i < 3; ++i) tv[i] = sub[i][0] * P.dphidz[ns][0] + sub[i][1] * P.dphidz[ns][1] + sub[i][2] * P.dphidz[ns][2];
        for (int ms = ns; ms < 27; ++ms)
          K[(size_t)(nh * 27 + ms) * 89 + nh * 27 + ns] +=
              P.dphidz[ms][0] * tv[0] + P.dphidz[ms][1] * tv[1] + P.dphidz[ms][2] * tv[2];
      }
    }
    // off-diagonal component blocks (nh, mh) = (1,2), (1,3), (2,3): rows mh, columns nh
    const int offn[3] = {0, 0, 1}, offm[3] = {1, 2, 2};
    for (int oh = 0; oh < 3; ++oh) {
      const int nh = offn[oh], mh = offm[oh];
      double sub[3][3];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) sub[i][j] = jgw * D[kT2V[i][mh]][kT2V[j][nh]];
      for (int ns = 0; ns < 27; ++ns) {
        double tv[3];
        for (int i = 0; i < 3; ++i) tv[i] = sub[i][0] * P.dphidz[ns][0] + sub[i][1] * P.dphidz[ns][1] + sub[i][2] * P.dphidz[ns][2];
        for (int ms = 0; ms < 27; ++ms)
          K[(size_t)(mh * 27 + ms) * 89 + nh * 27 + ns] +=
              P.dphidz[ms][0] * tv[0] + P.dphidz[ms][1] * tv[1] + P.dphidz[ms][2] * tv[2];
      }
    }
    // pressure rows, displacement columns
    for (int nh = 0; nh < 3; ++nh)
      for (int ns = 0; ns < 27; ++ns) {
        const double a = jgw * P.dphidz[ns][nh];
        for (int ms = 0; ms < 8; ++ms) K[(size_t)(81 + ms) * 89 + nh * 27 + ns] += a * P.psi[ms];
      }
    // displacement rows, pressure columns
    for (int mh = 0; mh < 3; ++mh)
      for (int ms = 0; ms < 27; ++ms) {
        const double tvm = hyd[mh][0] * P.dphidz[ms][0] + hyd[mh][1] * P.dphidz[ms][1] + hyd[mh][2] * P.dphidz[ms][2];
        const double a = jgw * tvm;
        for (int ns = 0; ns < 8; ++ns) K[(size_t)(mh * 27 + ms) * 89 + 81 + ns] += a * P.psi[ns];
      }
  }
  // mirror the displacement block's lower triangle to the upper (:1269-1274)
  for (int nhs = 1; nhs < 81; ++nhs)
    for (int mhs = 0; mhs < nhs; ++mhs) K[(size_t)mhs * 89 + nhs] = K[(size_t)nhs * 89 + mhs];
}

void mr_gather(int e, const int32_t* eq2, const int32_t* elin, int nq2, const double* xg_nodes, const double* dep,
               double* xe, double* ze, double* pe) {
  for (int s = 0; s < 27; ++s) {
    int n = eq2[(size_t)e * 27 + s];
    for (int c = 0; c < 3; ++c) {
      xe[c * 27 + s] = xg_nodes[(size_t)c * nq2 + n];
      ze[c * 27 + s] = dep[(size_t)c * nq2 + n];
    }
  }
  for (int s = 0; s < 8; ++s) pe[s] = dep[(size_t)3 * nq2 + elin[(size_t)e * 8 + s]];
}

void mr_element_dofs(int e, const int32_t* eq2, const int32_t* elin, int nq2, int32_t* dofs /*1-based*/) {
  for (int c = 0; c < 3; ++c)
    for (int s = 0; s < 27; ++s) dofs[c * 27 + s] = c * nq2 + eq2[(size_t)e * 27 + s] + 1;
  for (int s = 0; s < 8; ++s) dofs[81 + s] = 3 * nq2 + elin[(size_t)e * 8 + s] + 1;
}

}  // namespace

extern "C" {

int orc_mr_element_residual(const double* xe, const double* ze, const double* pe, double c1, double c2, double* R) {
  mr_residual_element(xe, ze, pe, c1, c2, R);
  return 0;
}

int orc_mr_element_jacobian(const double* xe, const double* ze, const double* pe, double c1, double c2, double* K) {
  mr_jacobian_element(xe, ze, pe, c1, c2, K);
  return 0;
}

// Iron's one-sided finite-difference element Jacobian, src/equations_set_routines.F90:2839-2962:
// column j = (R(u + delta e_j) - R(u)) / delta over the element's parameters in component order.
// `delta` is (1 + ||all dependent parameters||_2) * step, computed by the caller.
int orc_mr_element_jacobian_fd(const double* xe, const double* ze, const double* pe, double c1, double c2,
                               double delta, double* K) {
  double R0[89], R1[89], z[81], p[8];
  std::copy(ze, ze + 81, z);
  std::copy(pe, pe + 8, p);
  mr_residual_element(xe, z, p, c1, c2, R0);
  for (int j = 0; j < 89; ++j) {
    double* v = j < 81 ? &z[j] : &p[j - 81];
    const double orig = *v;
    *v = orig + delta;
    mr_residual_element(xe, z, p, c1, c2, R1);
    *v = orig;
    for (int i = 0; i < 89; ++i) K[(size_t)i * 89 + j] = (R1[i] - R0[i]) / delta;
  }
  return 0;
}

// Global residual (separated DOF order: z1, z2, z3 over the quadratic nodes, then p over the linear
// nodes), assembled in element order like EquationsSet_ResidualEvaluateStaticFEM
// (src/equations_set_routines.F90:5164-5286).  c: [E][2] (c10, c01) per element.
int orc_mr_assemble_residual(int n_elem, const int32_t* eq2, const int32_t* elin, int nq2, int nlin,
                             const double* xg_nodes, const double* dep, const double* c, double* R) {
  const int ndof = 3 * nq2 + nlin;
  std::fill(R, R + ndof, 0.0);
  double xe[81], ze[81], pe[8], Re[89];
  int32_t dofs[89];
  for (int e = 0; e < n_elem; ++e) {
    mr_gather(e, eq2, elin, nq2, xg_nodes, dep, xe, ze, pe);
    mr_residual_element(xe, ze, pe, c[2 * e], c[2 * e + 1], Re);
    mr_element_dofs(e, eq2, elin, nq2, dofs);
    for (int i = 0; i < 89; ++i) R[dofs[i] - 1] += Re[i];
  }
  return 0;
}

// Global analytic Jacobian into a fixed CSR structure (JacobianElementAdd,
// src/equations_matrices_routines.F90:2866-2909 -> MATRIX_VALUES_ADD_DP2).
int orc_mr_assemble_jacobian(int n_elem, const int32_t* eq2, const int32_t* elin, int nq2, int nlin,
                             const double* xg_nodes, const double* dep, const double* c, const int32_t* rp,
                             const int32_t* ci, double* values, int fd, double fd_delta) {
  const int ndof = 3 * nq2 + nlin;
  std::fill(values, values + (rp[ndof] - 1), 0.0);
  double xe[81], ze[81], pe[8];
  std::vector<double> Ke(89 * 89);
  int32_t dofs[89];
  for (int e = 0; e < n_elem; ++e) {
    mr_gather(e, eq2, elin, nq2, xg_nodes, dep, xe, ze, pe);
    if (fd) orc_mr_element_jacobian_fd(xe, ze, pe, c[2 * e], c[2 * e + 1], fd_delta, Ke.data());
    else mr_jacobian_element(xe, ze, pe, c[2 * e], c[2 * e + 1], Ke.data());
    mr_element_dofs(e, eq2, elin, nq2, dofs);
    if (csr_values_add(rp, ci, values, 89, dofs, 89, dofs, Ke.data()) != 0) return -2;
  }
  return 0;
}

}  // extern "C"
