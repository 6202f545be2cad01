// ORACLE — test infrastructure only (see oracle_core.hpp header).
//
// Part 2: superspace (local Bernstein bases, map2surface), the single-layer
// integrands of Laplace / Helmholtz / Maxwell (+ the test-only dummy operator),
// the DuffyTrick quadratures, FMM moments / transfers / transforms, the H2
// matrix assembly and matvec, and the dense Galerkin matrix.
#pragma once
#include "oracle_core.hpp"

namespace orc {

template <typename S>
struct Mat {
  int rows = 0, cols = 0;
  std::vector<S> a;  // column-major
  Mat() {}
  Mat(int r, int c) : rows(r), cols(c), a((size_t)r * c, S(0)) {}
  S& operator()(int i, int j) { return a[(size_t)j * rows + i]; }
  const S& operator()(int i, int j) const { return a[(size_t)j * rows + i]; }
  void zero() { std::fill(a.begin(), a.end(), S(0)); }
};

enum OpKind { kLaplace = 0, kHelmholtz = 1, kMaxwell = 2, kDummy = 3 };

// Dummy integrand functions of tests/DuffyTrick/test_testFunctions.hpp.
inline double dummy_fun(int which, double x0, double x1, double y0, double y1) {
  if (which == 0) {
    return std::sin(kPi * x0) * std::sin(2 * kPi * y0) * std::exp(-x1) * std::exp(y1);
  } else if (which == 1) {
    const double sigma = 1e-3;
    double c = x1 - y0;
    return std::exp(-x0 - 2 * y1) * (1. / (sigma + c * c));
  }
  return 1.0;
}

struct Operator {
  int kind = kLaplace;
  cplx kappa = 0, kappa2 = 0;
  int dummy_fun_id = 0;
  int P = 0;         // polynomial degree
  int M = 0;         // refinement level of the superspace
  int vd() const { return kind == kMaxwell ? 2 : 1; }
  int nc() const { return kind == kMaxwell ? 2 : 1; }
  int order() const { return kind == kDummy ? 0 : -1; }
  bool is_complex() const { return kind == kHelmholtz || kind == kMaxwell; }
  // LinearOperatorBase::get_FarfieldQuadratureDegree (LinearOperatorBase.hpp:56-58)
  int ffield_deg() const { return P - order() + 1; }
  // LinearOperatorBase::getNearfieldQuadratureDegree (LinearOperatorBase.hpp:69-89)
  int nfield_deg(double distance, int level) const {
    double distance_log =
        (distance * (1 << level) < 1) ? -(level * std::log(2.)) : std::log(distance);
    int alpha = 2 - order() + 2 * P;
    double numerator = (alpha + P) * level * std::log(2.) - (2 - P + order()) * distance_log;
    double denominator = (level + 2) * std::log(2.) + distance_log;
    return 0.5 * numerator / denominator;
  }
  cplx kernel_c(const V3& x, const V3& y) const {
    double r = (x - y).norm();
    return std::exp(-cplx(0., 1.) * kappa * r) / 4. / kPi / r;
  }
  double kernel_r(const V3& x, const V3& y) const { return 1. / 4. / kPi / (x - y).norm(); }
};

// ---------------------------------------------------------------------------
// SuperSpace (AnsatzSpace/SuperSpace.hpp) on top of the element tree.
struct SuperSpace {
  ElementTree et;
  int P = 0;
  int p2() const { return (P + 1) * (P + 1); }
  int ne() const { return et.nelements; }
  void init(const std::vector<Patch>& g, int M, int P_) {
    P = P_;
    et.init(g, M);
  }
  // SuperSpace::map2surface (SuperSpace.hpp:160-165)
  void map2surface(const Node& e, double xi0, double xi1, double w, SurfacePoint* sp) const {
    double h = e.h();
    et.geo[e.patch].update(sp, e.llc[0] + h * xi0, e.llc[1] + h * xi1, w, xi0, xi1);
  }
  const Node& element(int id) const { return et.nodes[et.leaves[id]]; }
  // tensor basis values, local index iy*(P+1)+ix (Spline/Basis.hpp:73-82)
  void phiphi(double s, double t, double* out) const {
    double X[32], Y[32];
    bernstein_basis(P, s, X);
    bernstein_basis(P, t, Y);
    for (int iy = 0; iy <= P; ++iy)
      for (int ix = 0; ix <= P; ++ix) out[iy * (P + 1) + ix] = X[ix] * Y[iy];
  }
  void phiphi_dx(double s, double t, double* out) const {
    double X[32], Y[32];
    bernstein_der_basis(P, s, X);
    bernstein_basis(P, t, Y);
    for (int iy = 0; iy <= P; ++iy)
      for (int ix = 0; ix <= P; ++ix) out[iy * (P + 1) + ix] = X[ix] * Y[iy];
  }
  void phiphi_dy(double s, double t, double* out) const {
    double X[32], Y[32];
    bernstein_basis(P, s, X);
    bernstein_der_basis(P, t, Y);
    for (int iy = 0; iy <= P; ++iy)
      for (int ix = 0; ix <= P; ++ix) out[iy * (P + 1) + ix] = X[ix] * Y[iy];
  }
};

// ---------------------------------------------------------------------------
// evaluateIntegrand of the operators:
//   Laplace/Helmholtz SingleLayerOperator::evaluateIntegrand_impl (:44-85),
//   Maxwell SingleLayerOperator::evaluateIntegrand_impl (:44-88),
//   DummyOperator::evaluateIntegrand_impl (Dummy/DummyOperator.hpp:62-70).
template <typename S>
inline void integrand(const Operator& op, const SuperSpace& ss, const SurfacePoint& p1,
                      const SurfacePoint& p2, Mat<S>* iv) {
  const int P = ss.P, n = ss.p2();
  double ws = p1.v[2], wt = p2.v[2];
  if (op.kind == kDummy) {
    (*iv)(0, 0) += S(dummy_fun(op.dummy_fun_id, p1.v[3], p1.v[4], p2.v[3], p2.v[4]) * ws * wt);
    return;
  }
  V3 xf = p1.x(), yf = p2.x();
  double a[64], b[64];
  ss.phiphi(p1.v[0], p1.v[1], a);
  ss.phiphi(p2.v[0], p2.v[1], b);
  (void)P;
  if (op.kind == kLaplace || op.kind == kHelmholtz) {
    double xk = p1.dx().cross(p1.dy()).norm();
    double yk = p2.dx().cross(p2.dy()).norm();
    S k;
    if constexpr (std::is_same<S, double>::value) {
      k = op.kernel_r(xf, yf);
    } else {
      k = op.kind == kLaplace ? S(op.kernel_r(xf, yf)) : S(op.kernel_c(xf, yf));
    }
    S integ = k * xk * yk * ws * wt;
    // Phi_times_Phi_ (Basis.hpp:141-164): a scaled by w first
    for (int i = 0; i < n; ++i) {
      S ai = integ * a[i];
      for (int j = 0; j < n; ++j) (*iv)(i, j) += ai * b[j];
    }
    return;
  }
  if constexpr (!std::is_same<S, double>::value) {
    // Maxwell
    double h = 1. / (1 << op.M);
    S kev = op.kernel_c(xf, yf) * ws * wt;
    S ivec = kev;
    S idiv = -kev / op.kappa2 / h / h;
    V3 xdx = p1.dx(), xdy = p1.dy(), ydx = p2.dx(), ydy = p2.dy();
    // addScaledVectorBasisInteraction (SuperSpace.hpp:236-258)
    S c00 = ivec * xdx.dot(ydx), c01 = ivec * xdx.dot(ydy);
    S c10 = ivec * xdy.dot(ydx), c11 = ivec * xdy.dot(ydy);
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        double bi = a[i] * b[j];
        (*iv)(i, j) += c00 * bi;
        (*iv)(i, j + n) += c01 * bi;
        (*iv)(i + n, j) += c10 * bi;
        (*iv)(i + n, j + n) += c11 * bi;
      }
    // Div_Phi_times_Div_Phi_ (Basis.hpp:170-200)
    double adx[64], ady[64], bdx[64], bdy[64];
    ss.phiphi_dx(p1.v[0], p1.v[1], adx);
    ss.phiphi_dy(p1.v[0], p1.v[1], ady);
    ss.phiphi_dx(p2.v[0], p2.v[1], bdx);
    ss.phiphi_dy(p2.v[0], p2.v[1], bdy);
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        (*iv)(i, j) += (idiv * adx[i]) * bdx[j];
        (*iv)(i, j + n) += (idiv * adx[i]) * bdy[j];
        (*iv)(i + n, j) += (idiv * ady[i]) * bdx[j];
        (*iv)(i + n, j + n) += (idiv * ady[i]) * bdy[j];
      }
  }
}

// ---------------------------------------------------------------------------
// DuffyTrick (DuffyTrick/*.hpp)
struct Cmp {
  int rot1, rot2, cs;
};
// compareElements (compareElements.hpp:23-69)
inline Cmp compare_elements(const Node& e1, const Node& e2, bool same, double* dist) {
  if (same) {
    *dist = 0;
    return {4, 4, 2};
  }
  *dist = (e1.mid - e2.mid).norm() - e1.radius - e2.radius;
  *dist = *dist >= 0 ? *dist : 0;
  if (*dist > .5 / (1 << e1.level)) return {4, 4, 0};
  for (int r1 = 0; r1 < 4; ++r1)
    for (int r2 = 0; r2 < 4; ++r2)
      if (e1.vert[r1] == e2.vert[r2]) {
        if (e1.vert[3] == e2.vert[(r2 + 1) % 4]) return {3, r2, 3};
        if (e1.vert[(r1 + 1) % 4] == e2.vert[(r2 + 3) % 4]) return {r1, (r2 + 3) % 4, 3};
        return {r1, r2, 4};
      }
  return {4, 4, 0};
}
// tau (tau.hpp:26-42)
inline void tau(double x, double y, int c, double* o) {
  switch (c) {
    case 1: o[0] = 1 - y; o[1] = x; return;
    case 2: o[0] = 1 - x; o[1] = 1 - y; return;
    case 3: o[0] = y; o[1] = 1 - x; return;
    default: o[0] = x; o[1] = y; return;
  }
}

// computeFfieldQnodes (farFieldQuadratureNodes.hpp:22-46)
inline std::vector<std::vector<SurfacePoint>> ffield_qnodes(const SuperSpace& ss, const Cubature& Q) {
  std::vector<std::vector<SurfacePoint>> out(ss.ne());
  double h = ss.element(0).h();
  for (int e = 0; e < ss.ne(); ++e) {
    const Node& el = ss.element(e);
    out[el.id].resize(Q.size());
    for (int k = 0; k < Q.size(); ++k) ss.map2surface(el, Q.x0[k], Q.x1[k], h * Q.w[k], &out[el.id][k]);
  }
  return out;
}

template <typename S>
inline void integrate0(const Operator& op, const SuperSpace& ss, const std::vector<SurfacePoint>& q1,
                       const std::vector<SurfacePoint>& q2, Mat<S>* iv) {
  iv->zero();
  for (size_t i = 0; i < q1.size(); ++i)
    for (size_t j = 0; j < q2.size(); ++j) integrand(op, ss, q1[i], q2[j], iv);
}
template <typename S>
inline void integrate1(const Operator& op, const SuperSpace& ss, const Node& e1, const Node& e2,
                       const Cubature& Q, Mat<S>* iv) {
  double h = e1.h();
  iv->zero();
  SurfacePoint qp1, qp2;
  for (int i = 0; i < Q.size(); ++i) {
    ss.map2surface(e1, Q.x0[i], Q.x1[i], h * Q.w[i], &qp1);
    for (int j = 0; j < Q.size(); ++j) {
      ss.map2surface(e2, Q.x0[j], Q.x1[j], h * Q.w[j], &qp2);
      integrand(op, ss, qp1, qp2, iv);
    }
  }
}
// integrate2 (integrate2.hpp:27-67): identical elements
template <typename S>
inline void integrate2(const Operator& op, const SuperSpace& ss, const Node& e1, const Cubature& Q,
                       Mat<S>* iv) {
  iv->zero();
  double h = e1.h();
  SurfacePoint qp1, qp2;
  for (int i = 0; i < Q.size(); ++i) {
    double xi0 = Q.x0[i], xi1 = Q.x1[i];
    double w = h * h * Q.w[i] * xi0 * (1 - xi0) * (1 - xi0 * xi1);
    for (int j = 0; j < Q.size(); ++j) {
      double t1 = Q.x0[j] * (1 - xi0);
      double t2 = Q.x1[j] * (1 - xi0 * xi1);
      double t3 = Q.x0[j] * (1 - xi0) + xi0;
      double t4 = Q.x1[j] * (1 - xi0 * xi1) + xi0 * xi1;
      // columns of the 2x8 point matrix
      double pts[8][2] = {{t1, t2}, {t3, t4}, {t1, t4}, {t3, t2},
                          {t2, t1}, {t4, t3}, {t2, t3}, {t4, t1}};
      for (int k = 0; k < 4; ++k) {
        ss.map2surface(e1, pts[2 * k][0], pts[2 * k][1], w, &qp1);
        ss.map2surface(e1, pts[2 * k + 1][0], pts[2 * k + 1][1], Q.w[j], &qp2);
        integrand(op, ss, qp1, qp2, iv);
        integrand(op, ss, qp2, qp1, iv);
      }
    }
  }
}
// integrate3 (integrate3.hpp:27-80): common edge
template <typename S>
inline void integrate3(const Operator& op, const SuperSpace& ss, const Node& e1, int rot1,
                       const Node& e2, int rot2, const Cubature& Q, Mat<S>* iv) {
  iv->zero();
  double h = e1.h();
  SurfacePoint qp1, qp2;
  double a[2], b[2];
  for (int i = 0; i < Q.size(); ++i) {
    double x0 = Q.x0[i], x1 = Q.x1[i];
    double w = h * h * Q.w[i] * x1 * x1;
    double t1 = x0 * (1 - x1);
    double t2 = (1 - x0) * (1 - x1);
    for (int j = 0; j < Q.size(); ++j) {
      double e0 = x1 * Q.x0[j], eo1 = x1 * Q.x1[j];
      double t3 = x0 * (1 - e0);
      double t4 = (1 - x0) * (1 - e0);
      double w2a = Q.w[j] * (1 - x1), w2b = Q.w[j] * (1 - e0);
      tau(t1, e0, rot1, a); tau(t2, eo1, rot2, b);
      ss.map2surface(e1, a[0], a[1], w, &qp1); ss.map2surface(e2, b[0], b[1], w2a, &qp2);
      integrand(op, ss, qp1, qp2, iv);
      tau(1 - t1, e0, rot1, a); tau(1 - t2, eo1, rot2, b);
      ss.map2surface(e1, a[0], a[1], w, &qp1); ss.map2surface(e2, b[0], b[1], w2a, &qp2);
      integrand(op, ss, qp1, qp2, iv);
      tau(t3, x1, rot1, a); tau(t4, eo1, rot2, b);
      ss.map2surface(e1, a[0], a[1], w, &qp1); ss.map2surface(e2, b[0], b[1], w2b, &qp2);
      integrand(op, ss, qp1, qp2, iv);
      tau(1 - t3, x1, rot1, a); tau(1 - t4, eo1, rot2, b);
      ss.map2surface(e1, a[0], a[1], w, &qp1); ss.map2surface(e2, b[0], b[1], w2b, &qp2);
      integrand(op, ss, qp1, qp2, iv);
      tau(t4, eo1, rot1, a); tau(t3, x1, rot2, b);
      ss.map2surface(e1, a[0], a[1], w, &qp1); ss.map2surface(e2, b[0], b[1], w2b, &qp2);
      integrand(op, ss, qp1, qp2, iv);
      tau(1 - t4, eo1, rot1, a); tau(1 - t3, x1, rot2, b);
      ss.map2surface(e1, a[0], a[1], w, &qp1); ss.map2surface(e2, b[0], b[1], w2b, &qp2);
      integrand(op, ss, qp1, qp2, iv);
    }
  }
}
// integrate4 (integrate4.hpp:27-64): common vertex
template <typename S>
inline void integrate4(const Operator& op, const SuperSpace& ss, const Node& e1, int rot1,
                       const Node& e2, int rot2, const Cubature& Q, Mat<S>* iv) {
  iv->zero();
  double h = e1.h();
  SurfacePoint qp1, qp2, qp3, qp4, qp5, qp6;
  double a[2];
  for (int i = 0; i < Q.size(); ++i) {
    double x0 = Q.x0[i], x1 = Q.x1[i];
    double w = h * h * Q.w[i] * std::pow(x0, 3.);
    x1 *= x0;
    tau(x0, x1, rot1, a); ss.map2surface(e1, a[0], a[1], w, &qp1);
    tau(x1, x0, rot1, a); ss.map2surface(e1, a[0], a[1], w, &qp2);
    tau(x0, x1, rot2, a); ss.map2surface(e2, a[0], a[1], w, &qp3);
    tau(x1, x0, rot2, a); ss.map2surface(e2, a[0], a[1], w, &qp4);
    for (int j = 0; j < Q.size(); ++j) {
      double e0 = x0 * Q.x0[j], eo1 = x0 * Q.x1[j];
      tau(e0, eo1, rot2, a); ss.map2surface(e2, a[0], a[1], Q.w[j], &qp5);
      tau(e0, eo1, rot1, a); ss.map2surface(e1, a[0], a[1], Q.w[j], &qp6);
      integrand(op, ss, qp1, qp5, iv);
      integrand(op, ss, qp2, qp5, iv);
      integrand(op, ss, qp6, qp3, iv);
      integrand(op, ss, qp6, qp4, iv);
    }
  }
}

// evaluateBilinearForm (evaluateBilinearForm.hpp:21-71)
template <typename S>
inline void bilinear_form(const Operator& op, const SuperSpace& ss, int id1, int id2,
                          const std::vector<std::vector<SurfacePoint>>& ffq, Mat<S>* iv) {
  const Node& e1 = ss.element(id1);
  const Node& e2 = ss.element(id2);
  double dist = 0;
  int ff = op.ffield_deg();
  Cmp cp = compare_elements(e1, e2, id1 == id2, &dist);
  int nf = op.nfield_deg(dist, e1.level);
  nf = nf >= ff ? nf : ff;
  if (nf >= kMaxQuadDeg) throw std::runtime_error("quadrature degree too large");
  const Cubature& Q = GS(nf);
  switch (cp.cs) {
    case 0:
      if (nf == ff) integrate0(op, ss, ffq[e1.id], ffq[e2.id], iv);
      else integrate1(op, ss, e1, e2, Q, iv);
      return;
    case 2: integrate2(op, ss, e1, Q, iv); return;
    case 3: integrate3(op, ss, e1, cp.rot1, e2, cp.rot2, Q, iv); return;
    case 4: integrate4(op, ss, e1, cp.rot1, e2, cp.rot2, Q, iv); return;
  }
  throw std::runtime_error("element comparison failed");
}

// ---------------------------------------------------------------------------
// H2Multipole (H2Matrix/H2Multipole.hpp)
inline std::vector<double> cheb_roots(int n) {  // ChebychevRoots :20-32
  std::vector<double> x(n);
  double alpha = kPi / (2. * double(n));
  for (int i = 0; i < n; ++i) {
    double g = double(n - i);  // LinSpaced(n,1,n).reverse()
    x[i] = 0.5 * std::cos(alpha * (2 * g - 1)) + 0.5;
  }
  return x;
}
// computeLagrangePolynomials (:39-49): Newton divided differences; L(k, i)
inline Mat<double> lagrange_newton(int n) {
  Mat<double> L(n, n);
  for (int i = 0; i < n; ++i) L(i, i) = 1;
  std::vector<double> x = cheb_roots(n);
  for (int i = 0; i < n; ++i)
    for (int j = 1; j < n; ++j)
      for (int k = n - 1; k >= j; --k) L(k, i) = (L(k, i) - L(k - 1, i)) / (x[k] - x[k - j]);
  return L;
}
// evaluatePolynomial (:55-67)
inline double eval_newton(const Mat<double>& L, int col, const std::vector<double>& x, double xi) {
  int n = L.rows;
  double r = L(n - 1, col);
  for (int i = n - 2; i >= 0; --i) r = r * (xi - x[i]) + L(i, col);
  return r;
}
// computeTransferMatrices (:76-115): np^2 x 4np^2, blocks [T0 T2 T3 T1]
inline Mat<double> transfer_matrices(int n) {
  int n2 = n * n;
  Mat<double> E(n, 2 * n), T(n2, 4 * n2);
  std::vector<double> x = cheb_roots(n);
  Mat<double> L = lagrange_newton(n);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      E(i, j) = eval_newton(L, j, x, 0.5 * x[i]);
      E(i, j + n) = eval_newton(L, j, x, 0.5 * x[i] + 0.5);
    }
  const int perm[4] = {0, 3, 1, 2};
  for (int k = 0; k < 4; ++k)
    for (int i = 0; i < n; ++i)
      for (int ii = 0; ii < n; ++ii)
        for (int j = 0; j < n; ++j)
          for (int jj = 0; jj < n; ++jj)
            T(j * n + jj, i * n + ii + n2 * perm[k]) = E(i, j + (k / 2) * n) * E(ii, jj + (k % 2) * n);
  return T;
}
// Moment1D / Moment1DDerivative (:120-218)
inline Mat<double> moment1d(int P, int cluster_level, int cluster_ref, int np, bool deriv) {
  int n = 1 << cluster_ref;
  double h = 1. / n;
  int N = 1 << cluster_level;
  double H = 1. / N;
  const Rule1D& Q = GL((int)std::ceil(0.5 * (np + P - 2)));
  std::vector<double> x = cheb_roots(np);
  Mat<double> L = lagrange_newton(np);
  Mat<double> mom(np, n * (P + 1));
  double b[32];
  for (int i = 0; i < np; ++i)
    for (int j = 0; j < n; ++j) {
      std::vector<double> iv(P + 1, 0.0);
      for (size_t k = 0; k < Q.w.size(); ++k) {
        double wk = deriv ? Q.w[k] / std::sqrt(h * H) : Q.w[k] * std::sqrt(h * H);
        double w = wk * eval_newton(L, i, x, h * (j + Q.xi[k]));
        if (deriv) bernstein_der_basis(P, Q.xi[k], b); else bernstein_basis(P, Q.xi[k], b);
        for (int m = 0; m <= P; ++m) iv[m] += w * b[m];
      }
      for (int m = 0; m <= P; ++m) mom(i, j * (P + 1) + m) = iv[m];
    }
  return mom;
}
// moment2DComputer (:224-293)
inline Mat<double> moment2d(int P, int cluster_level, int cluster_ref, int np, bool d1, bool d2) {
  int n = 1 << cluster_ref, n2 = n * n, pp = P + 1, p2 = pp * pp;
  Mat<double> m1 = moment1d(P, cluster_level, cluster_ref, np, d1);
  Mat<double> m2 = moment1d(P, cluster_level, cluster_ref, np, d2);
  std::vector<int> is(n2, 0), it(n2, 0);
  for (int j = 0; j < cluster_ref; ++j) {
    int inc = 1 << 2 * j;
    for (int i = 0; i < inc; ++i) {
      int s = is[i], t = it[i];
      is[4 * i] = 2 * s; is[4 * i + 1] = 2 * s + 1; is[4 * i + 2] = 2 * s + 1; is[4 * i + 3] = 2 * s;
      it[4 * i] = 2 * t; it[4 * i + 1] = 2 * t; it[4 * i + 2] = 2 * t + 1; it[4 * i + 3] = 2 * t + 1;
    }
  }
  Mat<double> out(np * np, m1.cols * m2.cols);
  for (int i = 0; i < np; ++i)
    for (int j = 0; j < np; ++j)
      for (int k = 0; k < n2; ++k)
        for (int a = 0; a < pp; ++a)
          for (int b = 0; b < pp; ++b)
            out(i * np + j, p2 * k + a * pp + b) = m1(i, is[k] * pp + b) * m2(j, it[k] * pp + a);
  return out;
}
// Moment2D (:301-318) and the Maxwell specialisation
// (Maxwell/SingleLayerOperator.hpp:153-183): one moment matrix per vector component.
inline std::vector<Mat<double>> moments(const Operator& op, int P, int cluster_level, int cluster_ref, int np) {
  std::vector<Mat<double>> out;
  if (op.kind != kMaxwell) {
    out.push_back(moment2d(P, cluster_level, cluster_ref, np, false, false));
    return out;
  }
  Mat<double> m = moment2d(P, cluster_level, cluster_ref, np, false, false);
  Mat<double> mdx = moment2d(P, cluster_level, cluster_ref, np, true, false);
  Mat<double> mdy = moment2d(P, cluster_level, cluster_ref, np, false, true);
  Mat<double> m1(2 * m.rows, m.cols), m2(2 * m.rows, m.cols);
  for (int j = 0; j < m.cols; ++j)
    for (int i = 0; i < m.rows; ++i) {
      m1(i, j) = m(i, j); m1(i + m.rows, j) = mdx(i, j);
      m2(i, j) = m(i, j); m2(i + m.rows, j) = mdy(i, j);
    }
  out.push_back(m1);
  out.push_back(m2);
  return out;
}

// forwardTransformation (:380-422)
template <typename S>
inline std::vector<Mat<S>> forward_transform(const Mat<double>& mom, const Mat<double>& T, int steps,
                                             const Mat<S>& X) {
  int np2 = T.rows, nc = mom.rows / np2;
  std::vector<Mat<S>> out;
  Mat<S> Y(mom.rows, X.cols);
  for (int c = 0; c < X.cols; ++c)
    for (int k = 0; k < mom.cols; ++k) {
      S xv = X(k, c);
      for (int r = 0; r < mom.rows; ++r) Y(r, c) += mom(r, k) * xv;
    }
  out.push_back(Y);
  for (int s = 0; s < steps; ++s) {
    const Mat<S>& prev = out.back();
    int R = prev.rows, C = prev.cols / 4;
    Mat<S> tr(R, C);
    // the reshape stacks the 4 children of cluster c: child k, component j
    // sits at prev(j*np2 + q, 4c + k)
    for (int c = 0; c < C; ++c)
      for (int j = 0; j < nc; ++j)
        for (int r = 0; r < np2; ++r) {
          S acc = 0;
          for (int k = 0; k < 4; ++k)
            for (int q = 0; q < np2; ++q) acc += T(r, k * np2 + q) * prev(j * np2 + q, 4 * c + k);
          tr(j * np2 + r, c) = acc;
        }
    out.push_back(tr);
  }
  return out;
}
// backwardTransformation (:428-469); Z is destroyed
template <typename S>
inline std::vector<S> backward_transform(const Mat<double>& mom, const Mat<double>& T, int steps,
                                         std::vector<Mat<S>>& Z) {
  int np2 = T.rows, nc = mom.rows / np2;
  for (int i = steps; i > 0; --i) {
    Mat<S>& cur = Z[i];
    Mat<S>& nxt = Z[i - 1];
    for (int c = 0; c < cur.cols; ++c)
      for (int j = 0; j < nc; ++j)
        for (int k = 0; k < 4; ++k)
          for (int q = 0; q < np2; ++q) {
            S acc = 0;
            for (int r = 0; r < np2; ++r) acc += T(r, k * np2 + q) * cur(j * np2 + r, c);
            nxt(j * np2 + q, 4 * c + k) += acc;
          }
  }
  const Mat<S>& Z0 = Z[0];
  std::vector<S> out((size_t)mom.cols * Z0.cols);
  for (int c = 0; c < Z0.cols; ++c)
    for (int k = 0; k < mom.cols; ++k) {
      S acc = 0;
      for (int r = 0; r < mom.rows; ++r) acc += mom(r, k) * Z0(r, c);
      out[(size_t)c * mom.cols + k] = acc;
    }
  return out;
}

// interpolationPoints2D (:324-331) and interpolateKernel (:336-375)
template <typename S>
inline Mat<S> interpolate_kernel(const Operator& op, const SuperSpace& ss, const std::vector<double>& x1d,
                                 const Node& c1, const Node& c2) {
  int np = (int)x1d.size(), n2 = np * np, vd = op.vd(), nc = op.nc();
  Mat<S> F(vd * nc * n2, vd * nc * n2);
  SurfacePoint q1, q2;
  for (int i = 0; i < n2; ++i) {
    ss.map2surface(c1, x1d[i / np], x1d[i % np], 1., &q1);
    for (int j = 0; j < n2; ++j) {
      ss.map2surface(c2, x1d[j / np], x1d[j % np], 1., &q2);
      V3 xf = q1.x(), yf = q2.x();
      if (op.kind == kMaxwell) {
        if constexpr (!std::is_same<S, double>::value) {
          S k = op.kernel_c(xf, yf);
          S out[4][4] = {};
          out[0][0] = k * q1.dx().dot(q2.dx());
          out[0][2] = k * q1.dx().dot(q2.dy());
          out[2][0] = k * q1.dy().dot(q2.dx());
          out[2][2] = k * q1.dy().dot(q2.dy());
          S d = -k / op.kappa2;
          out[1][1] = d; out[1][3] = d; out[3][1] = d; out[3][3] = d;
          for (int ii = 0; ii < vd; ++ii)
            for (int jj = 0; jj < vd; ++jj)
              for (int a = 0; a < nc; ++a)
                for (int b = 0; b < nc; ++b)
                  F(i + (ii * nc + a) * n2, j + (jj * nc + b) * n2) = out[a + ii * nc][b + jj * nc];
        }
      } else {
        double xk = q1.dx().cross(q1.dy()).norm();
        double yk = q2.dx().cross(q2.dy()).norm();
        S k;
        if constexpr (std::is_same<S, double>::value) k = op.kernel_r(xf, yf);
        else k = op.kind == kLaplace ? S(op.kernel_r(xf, yf)) : op.kernel_c(xf, yf);
        F(i, j) = k * xk * yk;
      }
    }
  }
  return F;
}

}  // namespace orc
