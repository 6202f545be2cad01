// ORACLE — test infrastructure only (see oracle_core.hpp header).
//
// Part 4: H2Matrix assembly (H2Matrix.hpp:93-250), the H2 matvec
// (EigenHelper/H2DenseProduct.hpp:33-165), the dense Galerkin matrix
// (DiscreteOperator.hpp:27-87), load vectors (DiscreteLinearForm.hpp:44-83 with
// DirichletTrace / RotatedTangentialTrace), the single-layer potential
// (DiscretePotential.hpp:49-107) and a restarted GMRES, behind a C API that the
// Python tests load with ctypes.
#include <omp.h>

#include <algorithm>
#include <chrono>
#include <limits>
#include <memory>

#include "oracle_space.hpp"

namespace orc {

template <typename S>
struct H2Leaf {
  int cc, c1, c2;              // admissibility, cluster node indices
  std::vector<Mat<S>> F;       // vd*vd blocks, index row_comp*vd + col_comp
};

struct Problem {
  SuperSpace ss;
  Operator op;
  BlockClusterTree bct;
  Sparse T;  // superspace x dofs
  int np = 9;
  Mat<double> transfer;
  std::vector<Mat<double>> mom;
  std::vector<double> x1d;
  std::vector<H2Leaf<double>> leaves_r;
  std::vector<H2Leaf<cplx>> leaves_c;
  std::vector<std::vector<SurfacePoint>> ffq;
  double t_assemble = 0;
  int leaf_stride = 1;   // assemble only leaves with index % leaf_stride == 0
  double t_leaves = 0, t_other = 0;  // split of the last product's time
  long sampled_entries = 0, total_entries = 0;
  std::string err;

  int vd() const { return op.vd(); }
  int S() const { return T.rows; }
  int N() const { return T.cols; }
  int steps() const { return std::max(0, bct.max_level - bct.mcl); }
};

template <typename S>
std::vector<H2Leaf<S>>& leaves_of(Problem& p);
template <>
std::vector<H2Leaf<double>>& leaves_of<double>(Problem& p) { return p.leaves_r; }
template <>
std::vector<H2Leaf<cplx>>& leaves_of<cplx>(Problem& p) { return p.leaves_c; }

// H2Matrix::init_H2Matrix leaf loop (H2Matrix.hpp:144-246)
template <typename S>
void assemble_h2(Problem& p) {
  const int vd = p.vd(), n = p.ss.p2();
  auto& L = leaves_of<S>(p);
  L.resize(p.bct.leaves.size());
  p.total_entries = p.sampled_entries = 0;
  for (long li = 0; li < (long)p.bct.leaves.size(); ++li) {
    const BlockLeaf& bl = p.bct.leaves[li];
    long ent = bl.cc == kDense ? (long)p.ss.et.cluster_size(bl.c1) * n * p.ss.et.cluster_size(bl.c2) * n
                               : (long)p.op.nc() * p.np * p.np * p.op.nc() * p.np * p.np;
    ent *= vd * vd;
    p.total_entries += ent;
    if (li % p.leaf_stride == 0) p.sampled_entries += ent;
  }
#pragma omp parallel for schedule(dynamic, 1)
  for (long li = 0; li < (long)p.bct.leaves.size(); ++li) {
    const BlockLeaf& bl = p.bct.leaves[li];
    H2Leaf<S>& out = L[li];
    out.cc = bl.cc;
    out.c1 = bl.c1;
    out.c2 = bl.c2;
    if (li % p.leaf_stride != 0) continue;  // sampled assembly: leaf left empty
    if (bl.cc == kDense) {
      int n1 = p.ss.et.cluster_size(bl.c1), f1 = p.ss.et.cluster_first(bl.c1);
      int n2 = p.ss.et.cluster_size(bl.c2), f2 = p.ss.et.cluster_first(bl.c2);
      out.F.assign(vd * vd, Mat<S>(n1 * n, n2 * n));
      Mat<S> iv(vd * n, vd * n);
      for (int a = 0; a < n1; ++a)
        for (int b = 0; b < n2; ++b) {
          bilinear_form<S>(p.op, p.ss, f1 + a, f2 + b, p.ffq, &iv);
          for (int i = 0; i < vd; ++i)
            for (int j = 0; j < vd; ++j)
              for (int c = 0; c < n; ++c)
                for (int r = 0; r < n; ++r) out.F[i * vd + j](a * n + r, b * n + c) = iv(i * n + r, j * n + c);
        }
    } else {
      Mat<S> F = interpolate_kernel<S>(p.op, p.ss, p.x1d, p.ss.et.nodes[bl.c1], p.ss.et.nodes[bl.c2]);
      int B = p.op.nc() * p.np * p.np;
      out.F.assign(vd * vd, Mat<S>(B, B));
      for (int i = 0; i < vd; ++i)
        for (int j = 0; j < vd; ++j)
          for (int c = 0; c < B; ++c)
            for (int r = 0; r < B; ++r) out.F[i * vd + j](r, c) = F(i * B + r, j * B + c);
    }
  }
}

// H2_time_dense_product_impl::run (H2DenseProduct.hpp:33-165), for a
// superspace vector (the T and T^T steps are applied by the caller).
template <typename S>
void h2_product_ss(Problem& p, const S* xss, S* yss) {
  const int vd = p.vd(), n = p.ss.p2(), ne = p.ss.ne();
  const int comp = ne * n;
  const int steps = p.steps();
  auto& L = leaves_of<S>(p);
  for (int i = 0; i < vd * comp; ++i) yss[i] = 0;
  for (int cc = 0; cc < vd; ++cc)
    for (int rc = 0; rc < vd; ++rc) {
      const S* xr = xss + (size_t)cc * comp;
      const Mat<double>& momc = p.mom[cc];
      Mat<S> X(momc.cols, comp / momc.cols);
      for (int i = 0; i < comp; ++i) X.a[i] = xr[i];
      std::vector<Mat<S>> fwd = forward_transform<S>(momc, p.transfer, steps, X);
      std::vector<S> dst(comp, S(0));
      auto tl0 = std::chrono::steady_clock::now();
      // The reference's OpenMP structure (H2DenseProduct.hpp:82-150): every
      // thread owns a full destination and full backward-transform targets,
      // the leaves are shared out one at a time, each thread runs its own
      // backward transform, and the destinations are summed in a critical
      // section. (The reference hands out leaves with `omp single nowait`;
      // a dynamic loop hands them out the same way with less locking.)
#pragma omp parallel
      {
        std::vector<S> mine(comp, S(0));
        std::vector<Mat<S>> bw;
        for (auto& f : fwd) bw.emplace_back(f.rows, f.cols);
#pragma omp for schedule(dynamic, 8) nowait
        for (long li = 0; li < (long)L.size(); ++li) {
          const H2Leaf<S>& lf = L[li];
          if (lf.F.empty()) continue;  // not assembled (sampled operator)
          const Mat<S>& F = lf.F[rc * vd + cc];
          const Node& c1 = p.ss.et.nodes[lf.c1];
          const Node& c2 = p.ss.et.nodes[lf.c2];
          if (lf.cc == kDense) {
            int r0 = n * p.ss.et.cluster_first(lf.c1), c0 = n * p.ss.et.cluster_first(lf.c2);
            for (int c = 0; c < F.cols; ++c) {
              S xv = xr[c0 + c];
              for (int r = 0; r < F.rows; ++r) mine[r0 + r] += F(r, c) * xv;
            }
          } else {
            int lvl = p.bct.max_level - p.bct.mcl - c1.level;
            Mat<S>& Z = bw[lvl];
            const Mat<S>& Y = fwd[lvl];
            for (int c = 0; c < F.cols; ++c) {
              S yv = Y(c, c2.id);
              for (int r = 0; r < F.rows; ++r) Z(r, c1.id) += F(r, c) * yv;
            }
          }
        }
        std::vector<S> back = backward_transform<S>(p.mom[rc], p.transfer, steps, bw);
#pragma omp critical
        for (int i = 0; i < comp; ++i) dst[i] += mine[i] + back[i];
      }
      p.t_leaves += std::chrono::duration<double>(std::chrono::steady_clock::now() - tl0).count();
      for (int i = 0; i < comp; ++i) yss[(size_t)rc * comp + i] += dst[i];
    }
}

// DiscreteOperatorComputer<MatrixXd> (DiscreteOperator.hpp:27-87): superspace
template <typename S>
void dense_ss(Problem& p, S* out) {
  const int vd = p.vd(), n = p.ss.p2(), ne = p.ss.ne();
  const long Sd = (long)vd * n * ne;
#pragma omp parallel for schedule(dynamic, 4)
  for (long e1 = 0; e1 < ne; ++e1) {
    Mat<S> iv(vd * n, vd * n);
    for (int e2 = 0; e2 < ne; ++e2) {
      bilinear_form<S>(p.op, p.ss, (int)e1, e2, p.ffq, &iv);
      for (int i = 0; i < vd; ++i)
        for (int j = 0; j < vd; ++j)
          for (int c = 0; c < n; ++c)
            for (int r = 0; r < n; ++r) {
              long row = (long)n * (i * ne + e1) + r, col = (long)n * (j * ne + e2) + c;
              out[col * Sd + row] = iv(i * n + r, j * n + c);
            }
    }
  }
}

// data functions used for load vectors (examples/Data.hpp)
struct DataFun {
  int kind = 0;  // 0: 1/(4 pi |x-x0|); 1: exp(-i k r)/(4 pi r) point source;
                 // 2: plane wave exp(-i k d.x); 3: Hertz dipole (vector)
  double prm[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  cplx kappa = 0;
  cplx scalar(const V3& x) const {
    V3 x0(prm[0], prm[1], prm[2]);
    if (kind == 0) return 1. / (4. * kPi * (x - x0).norm());
    if (kind == 1) {
      double r = (x - x0).norm();
      return std::exp(-cplx(0, 1) * kappa * r) / (4. * kPi * r);
    }
    if (kind == 2) return std::exp(-cplx(0, 1) * kappa * V3(prm[0], prm[1], prm[2]).dot(x));
    return 0;
  }
  // Data::Dipole (examples/Data.hpp:73-90)
  void vector(const V3& pt, cplx out[3]) const {
    V3 pos(prm[0], prm[1], prm[2]), len(prm[3], prm[4], prm[5]);
    const cplx i(0, 1);
    V3 c = pt - pos;
    double r = c.norm();
    V3 nn = c * (1. / r);
    cplx expc = std::exp(-i * kappa * r);
    V3 ncl = nn.cross(len).cross(nn);
    V3 hh = nn * (3 * nn.dot(len)) - len;
    cplx ec = ((1 / (r * r * r)) - (i * (-kappa) / (r * r))) * expc;
    cplx f = kappa * kappa * expc / r;
    out[0] = f * ncl.x + ec * hh.x;
    out[1] = f * ncl.y + ec * hh.y;
    out[2] = f * ncl.z + ec * hh.z;
  }
};

// DiscreteLinearForm::compute with DirichletTrace / RotatedTangentialTrace
template <typename S>
void load_vector(Problem& p, const DataFun& f, S* out) {
  const int n = p.ss.p2(), ne = p.ss.ne(), vd = p.vd();
  const Cubature& Q = GS(p.ss.P + 1);
  std::vector<S> lf((size_t)vd * n * ne, S(0));
#pragma omp parallel for schedule(static)
  for (int e = 0; e < ne; ++e) {
    const Node& el = p.ss.element(e);
    SurfacePoint qp;
    double b[64];
    for (int q = 0; q < Q.size(); ++q) {
      p.ss.map2surface(el, Q.x0[q], Q.x1[q], el.h() * Q.w[q], &qp);
      p.ss.phiphi(qp.v[0], qp.v[1], b);
      V3 dx = qp.dx(), dy = qp.dy();
      if (vd == 1) {
        double kap = dx.cross(dy).norm();
        S integ;
        if constexpr (std::is_same<S, double>::value) integ = f.scalar(qp.x()).real() * kap * qp.v[2];
        else integ = f.scalar(qp.x()) * kap * qp.v[2];
        for (int i = 0; i < n; ++i) lf[(size_t)n * el.id + i] += integ * b[i];
      } else {
        if constexpr (!std::is_same<S, double>::value) {
          V3 nrm = dx.cross(dy);
          double nn = nrm.norm();
          nrm = nrm * (1. / nn);
          cplx fv[3];
          f.vector(qp.x(), fv);
          cplx fd = fv[0] * nrm.x + fv[1] * nrm.y + fv[2] * nrm.z;
          cplx tc[3] = {(fv[0] - fd * nrm.x) * qp.v[2], (fv[1] - fd * nrm.y) * qp.v[2],
                        (fv[2] - fd * nrm.z) * qp.v[2]};
          cplx cx = dx.x * tc[0] + dx.y * tc[1] + dx.z * tc[2];
          cplx cy = dy.x * tc[0] + dy.y * tc[1] + dy.z * tc[2];
          for (int i = 0; i < n; ++i) {
            lf[(size_t)n * el.id + i] += cx * b[i];
            lf[(size_t)n * ne + (size_t)n * el.id + i] += cy * b[i];
          }
        }
      }
    }
  }
  p.T.apply_t(lf.data(), out);
}

// DiscretePotential::evaluate for the Laplace / Helmholtz single layer potential
template <typename S>
void potential(Problem& p, const S* rho, const double* pts, int npts, S* out) {
  const int n = p.ss.p2(), ne = p.ss.ne();
  std::vector<S> coef((size_t)p.S());
  p.T.apply(rho, coef.data());
  const Cubature& Q = GS(p.ss.P + 1);
  for (int i = 0; i < npts; ++i) out[i] = 0;
#pragma omp parallel
  {
    std::vector<S> mine(npts, S(0));
#pragma omp for schedule(static)
    for (int e = 0; e < ne; ++e) {
      const Node& el = p.ss.element(e);
      SurfacePoint qp;
      double b[64];
      double h = el.h();
      for (int q = 0; q < Q.size(); ++q) {
        p.ss.map2surface(el, Q.x0[q], Q.x1[q], h * h * Q.w[q], &qp);
        p.ss.phiphi(qp.v[0], qp.v[1], b);
        S cv = 0;
        for (int k = 0; k < n; ++k) cv += coef[(size_t)n * el.id + k] * b[k];
        cv = cv / h;
        double kap = qp.dx().cross(qp.dy()).norm();
        V3 xf = qp.x();
        for (int i = 0; i < npts; ++i) {
          V3 pt(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
          S k;
          if constexpr (std::is_same<S, double>::value) k = p.op.kernel_r(pt, xf);
          else k = p.op.kind == kLaplace ? S(p.op.kernel_r(pt, xf)) : p.op.kernel_c(pt, xf);
          mine[i] += k * cv * kap * qp.v[2];
        }
      }
    }
#pragma omp critical
    for (int i = 0; i < npts; ++i) out[i] += mine[i];
  }
}

// DiscretePotential::evaluate with MaxwellSingleLayerPotential::evaluateIntegrand_impl
// (Maxwell/SingleLayerPotential.hpp:44-95) and the div-conforming function
// evaluator (AnsatzSpace/FunctionEvaluatorEval.hpp:39-83): per Gauss point
// (GS[P+1], weight h^2 w), E(x) += w [k(x, y) u(y) + grad_x k(x, y) div u(y) / kappa^2]
// with u = (c0 dx + c1 dy) / h, div u = (sum c0 phi_dx + sum c1 phi_dy) / h^2.
void potential_mw(Problem& p, const cplx* rho, const double* pts, int npts, cplx* out) {
  const int n = p.ss.p2(), ne = p.ss.ne();
  std::vector<cplx> coef((size_t)p.S());
  p.T.apply(rho, coef.data());
  const cplx* c0 = coef.data();
  const cplx* c1 = coef.data() + (size_t)n * ne;
  const Cubature& Q = GS(p.ss.P + 1);
  const cplx i1(0, 1), kap = p.op.kappa, kap2 = p.op.kappa2;
  for (int i = 0; i < 3 * npts; ++i) out[i] = 0;
#pragma omp parallel
  {
    std::vector<cplx> mine(3 * (size_t)npts, cplx(0));
#pragma omp for schedule(static)
    for (int e = 0; e < ne; ++e) {
      const Node& el = p.ss.element(e);
      SurfacePoint qp;
      double b[64], bdx[64], bdy[64];
      const double h = el.h();
      for (int q = 0; q < Q.size(); ++q) {
        p.ss.map2surface(el, Q.x0[q], Q.x1[q], h * h * Q.w[q], &qp);
        p.ss.phiphi(qp.v[0], qp.v[1], b);
        p.ss.phiphi_dx(qp.v[0], qp.v[1], bdx);
        p.ss.phiphi_dy(qp.v[0], qp.v[1], bdy);
        cplx t0 = 0, t1 = 0, dv = 0;
        for (int k = 0; k < n; ++k) {
          const cplx a0 = c0[(size_t)n * el.id + k], a1 = c1[(size_t)n * el.id + k];
          t0 += a0 * b[k];
          t1 += a1 * b[k];
          dv += a0 * bdx[k] + a1 * bdy[k];
        }
        dv = dv / h / h;
        const V3 dx = qp.dx(), dy = qp.dy(), y = qp.x();
        const cplx u[3] = {(dx.x * t0 + dy.x * t1) / h, (dx.y * t0 + dy.y * t1) / h, (dx.z * t0 + dy.z * t1) / h};
        const double w = qp.v[2];
        for (int i = 0; i < npts; ++i) {
          const V3 x(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
          const V3 c = x - y;
          const double r = c.norm();
          const cplx ex = std::exp(-i1 * kap * r);
          const cplx k = ex / 4. / kPi / r;
          const cplx g = ex * (-1. - i1 * kap * r) / 4. / kPi / (r * r * r);
          const double cc[3] = {c.x, c.y, c.z};
          for (int d = 0; d < 3; ++d) mine[3 * (size_t)i + d] += (k * u[d] + 1. / kap2 * (g * cc[d]) * dv) * w;
        }
      }
    }
#pragma omp critical
    for (int i = 0; i < 3 * npts; ++i) out[i] += mine[i];
  }
}

// DOF-level product y = A x for nrhs columns (column-major, leading dim N)
template <typename S>
void h2_matvec(Problem& p, const S* x, S* y, int nrhs) {
  auto t0 = std::chrono::steady_clock::now();
  p.t_leaves = 0;
  std::vector<S> xs(p.S()), ys(p.S());
  for (int c = 0; c < nrhs; ++c) {
    p.T.apply(x + (size_t)c * p.N(), xs.data());
    h2_product_ss<S>(p, xs.data(), ys.data());
    p.T.apply_t(ys.data(), y + (size_t)c * p.N());
  }
  p.t_other = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() - p.t_leaves;
}

inline double absval(double v) { return std::fabs(v); }
inline double absval(cplx v) { return std::abs(v); }
inline double conjmul_re(double a, double b) { return a * b; }

// Restarted GMRES (Saad & Schultz 1986) with modified Gram-Schmidt and Givens
// rotations; stops when ||b - A x|| / ||b|| <= tol.
template <typename S>
int gmres(Problem& p, const S* b, S* x, double tol, int restart, int maxit) {
  const int N = p.N();
  auto dotc = [&](const std::vector<S>& u, const std::vector<S>& v) {
    S s = 0;
    for (int i = 0; i < N; ++i) {
      if constexpr (std::is_same<S, double>::value) s += u[i] * v[i];
      else s += std::conj(u[i]) * v[i];
    }
    return s;
  };
  auto nrm = [&](const std::vector<S>& u) { return std::sqrt(std::abs(dotc(u, u))); };
  std::vector<S> bv(b, b + N), r(N), Ax(N);
  double bn = nrm(bv);
  if (bn == 0) {
    for (int i = 0; i < N; ++i) x[i] = 0;
    return 0;
  }
  int it = 0;
  while (it < maxit) {
    h2_matvec<S>(p, x, Ax.data(), 1);
    for (int i = 0; i < N; ++i) r[i] = bv[i] - Ax[i];
    double beta = nrm(r);
    if (beta / bn <= tol) return it;
    std::vector<std::vector<S>> V(1, r);
    for (auto& v : V[0]) v /= beta;
    std::vector<std::vector<S>> H(restart + 1, std::vector<S>(restart, S(0)));
    std::vector<S> cs(restart), sn(restart), g(restart + 1, S(0));
    g[0] = beta;
    int j = 0;
    for (; j < restart && it < maxit; ++j, ++it) {
      std::vector<S> w(N);
      h2_matvec<S>(p, V[j].data(), w.data(), 1);
      for (int i = 0; i <= j; ++i) {
        H[i][j] = dotc(V[i], w);
        for (int k = 0; k < N; ++k) w[k] -= H[i][j] * V[i][k];
      }
      double hn = nrm(w);
      H[j + 1][j] = hn;
      for (int i = 0; i < j; ++i) {
        S t = cs[i] * H[i][j] + sn[i] * H[i + 1][j];
        if constexpr (std::is_same<S, double>::value) H[i + 1][j] = -sn[i] * H[i][j] + cs[i] * H[i + 1][j];
        else H[i + 1][j] = -std::conj(sn[i]) * H[i][j] + cs[i] * H[i + 1][j];
        H[i][j] = t;
      }
      double a = absval(H[j][j]), bb = hn;
      double den = std::sqrt(a * a + bb * bb);
      if (a == 0) {
        cs[j] = 0;
        sn[j] = 1;
      } else {
        cs[j] = a / den;
        sn[j] = (H[j][j] / a) * (S(bb) / den);
      }
      H[j][j] = cs[j] * H[j][j] + sn[j] * H[j + 1][j];
      H[j + 1][j] = 0;
      if constexpr (std::is_same<S, double>::value) g[j + 1] = -sn[j] * g[j];
      else g[j + 1] = -std::conj(sn[j]) * g[j];
      g[j] = cs[j] * g[j];
      if (hn > 0) {
        std::vector<S> vn(w);
        for (auto& v : vn) v /= hn;
        V.push_back(vn);
      }
      if (absval(g[j + 1]) / bn <= tol || hn == 0) {
        ++j;
        ++it;
        break;
      }
    }
    // solve the j x j upper triangular system and update x
    std::vector<S> yv(j);
    for (int i = j - 1; i >= 0; --i) {
      S s = g[i];
      for (int k = i + 1; k < j; ++k) s -= H[i][k] * yv[k];
      yv[i] = s / H[i][i];
    }
    for (int i = 0; i < j; ++i)
      for (int k = 0; k < N; ++k) x[k] += yv[i] * V[i][k];
  }
  return it;
}

// Conjugate gradient without preconditioning, the solver of the reference's
// Laplace example (examples/LaplaceSingleLayerH2.cpp:77-80:
// ConjugateGradient<H2Matrix<double>, Lower | Upper, IdentityPreconditioner>).
// The iteration is the published Hestenes-Stiefel CG as Eigen 3 implements it
// (Eigen/src/IterativeLinearSolvers/ConjugateGradient.h, third party, version
// not pinned by the reference): start at x = 0, stop when
// ||r||^2 < tol^2 ||b||^2, at most maxit iterations (Eigen's default is
// 2 N). Returns the iteration count; *relres gets ||r|| / ||b|| of the
// recursively updated residual, as Eigen's error() does.
int cg(Problem& p, const double* b, double* x, double tol, int maxit, double* relres) {
  const int N = p.N();
  auto dot = [&](const std::vector<double>& u, const std::vector<double>& v) {
    double s = 0;
    for (int i = 0; i < N; ++i) s += u[i] * v[i];
    return s;
  };
  std::vector<double> r(b, b + N), d(N), Ad(N);
  for (int i = 0; i < N; ++i) x[i] = 0;
  const double bn2 = dot(r, r);
  *relres = 0;
  if (bn2 == 0) return 0;
  const double threshold = std::max(tol * tol * bn2, std::numeric_limits<double>::min());
  double rn2 = bn2;
  if (rn2 < threshold) {
    *relres = std::sqrt(rn2 / bn2);
    return 0;
  }
  d = r;
  double absnew = rn2;
  int it = 0;
  while (it < maxit) {
    h2_matvec<double>(p, d.data(), Ad.data(), 1);
    const double alpha = absnew / dot(d, Ad);
    for (int i = 0; i < N; ++i) {
      x[i] += alpha * d[i];
      r[i] -= alpha * Ad[i];
    }
    rn2 = dot(r, r);
    ++it;
    if (rn2 < threshold) break;
    const double absold = absnew;
    absnew = rn2;
    const double beta = absnew / absold;
    for (int i = 0; i < N; ++i) d[i] = r[i] + beta * d[i];
  }
  *relres = std::sqrt(rn2 / bn2);
  return it;
}

}  // namespace orc

using namespace orc;

extern "C" {

const char* orc_last_error(void* h) { return static_cast<Problem*>(h)->err.c_str(); }

// Build the discrete space (AnsatzSpace), block cluster tree, FMM moments and
// transfers; assemble the H2 matrix when assemble != 0.
void* orc_create(const char* geo, int M, int P, int kind, double kre, double kim, int np, double eta,
                 int mcl, int assemble, int dummy_fun) {
  try {
    init_rules();
    auto p = std::make_unique<Problem>();
    std::vector<Patch> g = load_dat(geo);
    p->ss.init(g, M, P);
    p->op.kind = kind;
    p->op.kappa = cplx(kre, kim);
    p->op.kappa2 = p->op.kappa * p->op.kappa;
    p->op.P = P;
    p->op.M = M;
    p->op.dummy_fun_id = dummy_fun;
    p->np = np;
    p->T = transformation_matrix(p->ss, kind == kDummy ? kLaplace : kind);
    p->bct.init(p->ss.et, eta, mcl);
    int cluster_level = std::max(0, M - mcl);
    int cluster_ref = std::min(mcl, M);
    p->transfer = transfer_matrices(np);
    p->mom = moments(p->op, P, cluster_level, cluster_ref, np);
    p->x1d = cheb_roots(np);
    p->ffq = ffield_qnodes(p->ss, GS(p->op.ffield_deg()));
    if (assemble) {
      auto t0 = std::chrono::steady_clock::now();
      if (p->op.is_complex()) assemble_h2<cplx>(*p); else assemble_h2<double>(*p);
      p->t_assemble = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    return p.release();
  } catch (const std::exception& e) {
    std::fprintf(stderr, "orc_create: %s\n", e.what());
    return nullptr;
  }
}
void orc_destroy(void* h) { delete static_cast<Problem*>(h); }

// sum_i coefs[i] B_{i,p}(x) or its derivative in x (Spline/Bernstein.hpp,
// Basis::ShapeFunctionHandler::evalCoef / evalDerCoef)
double orc_bernstein(int p, const double* coefs, double x, int der) {
  std::vector<double> b(p + 1);
  if (der) bernstein_der_basis(p, x, b.data());
  else bernstein_basis(p, x, b.data());
  double r = 0;
  for (int i = 0; i <= p; ++i) r += coefs[i] * b[i];
  return r;
}

// As orc_create with assembly, but only every leaf_stride-th leaf of the block
// partition is assembled (a bounded sample of the H2 matrix for CPU timing).
void* orc_create_sampled(const char* geo, int M, int P, int kind, double kre, double kim, int np, double eta, int mcl,
                         int leaf_stride) {
  Problem* p = static_cast<Problem*>(orc_create(geo, M, P, kind, kre, kim, np, eta, mcl, 0, 0));
  if (!p) return nullptr;
  p->leaf_stride = leaf_stride < 1 ? 1 : leaf_stride;
  auto t0 = std::chrono::steady_clock::now();
  if (p->op.is_complex()) assemble_h2<cplx>(*p); else assemble_h2<double>(*p);
  p->t_assemble = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return p;
}
// times of the last product: [leaf loop s, transforms and T s, sampled entries, total entries]
void orc_last_product_split(void* h, double* out4) {
  Problem& p = *static_cast<Problem*>(h);
  out4[0] = p.t_leaves;
  out4[1] = p.t_other;
  out4[2] = (double)p.sampled_entries;
  out4[3] = (double)p.total_entries;
}

// info[0..11]: ne, S, N, n_leaves, n_dense, n_lowrank, vd, nc, np, T nnz, M, P
void orc_info(void* h, long* info) {
  Problem& p = *static_cast<Problem*>(h);
  int nd = 0, nl = 0;
  for (auto& l : p.bct.leaves) (l.cc == kDense ? nd : nl)++;
  long v[12] = {p.ss.ne(), p.S(), p.N(), (long)p.bct.leaves.size(), nd, nl, p.vd(), p.op.nc(), p.np,
                (long)p.T.val.size(), p.ss.et.max_level, p.ss.P};
  for (int i = 0; i < 12; ++i) info[i] = v[i];
}
double orc_assemble_seconds(void* h) { return static_cast<Problem*>(h)->t_assemble; }

void orc_transform_csr(void* h, int* ptr, int* idx, double* val) {
  Problem& p = *static_cast<Problem*>(h);
  std::copy(p.T.ptr.begin(), p.T.ptr.end(), ptr);
  std::copy(p.T.idx.begin(), p.T.idx.end(), idx);
  std::copy(p.T.val.begin(), p.T.val.end(), val);
}

// per element: patch, level, id, llc0, llc1, vertices[4], mid[3], radius
// the Projector matrix alone (no gluing): dims[0..2] = rows, cols, nnz; the
// CSR arrays are written when ptr is not null
void orc_projector_csr(void* h, long* dims, int* ptr, int* idx, double* val) {
  Problem& p = *static_cast<Problem*>(h);
  const Sparse P = projector_matrix(p.ss, p.op.kind == kDummy ? kLaplace : p.op.kind);
  dims[0] = P.rows;
  dims[1] = P.cols;
  dims[2] = (long)P.val.size();
  if (!ptr) return;
  std::copy(P.ptr.begin(), P.ptr.end(), ptr);
  std::copy(P.idx.begin(), P.idx.end(), idx);
  std::copy(P.val.begin(), P.val.end(), val);
}

void orc_elements(void* h, int* ints, double* dbl) {
  Problem& p = *static_cast<Problem*>(h);
  for (int e = 0; e < p.ss.ne(); ++e) {
    const Node& n = p.ss.element(e);
    int* I = ints + 7 * e;
    I[0] = n.patch; I[1] = n.level; I[2] = n.id;
    for (int k = 0; k < 4; ++k) I[3 + k] = n.vert[k];
    double* D = dbl + 6 * e;
    D[0] = n.llc[0]; D[1] = n.llc[1]; D[2] = n.mid.x; D[3] = n.mid.y; D[4] = n.mid.z; D[5] = n.radius;
  }
}

// per leaf: cc, level(c1), id(c1), id(c2), first element of c1, of c2, #elements
void orc_leaves(void* h, int* out) {
  Problem& p = *static_cast<Problem*>(h);
  for (size_t i = 0; i < p.bct.leaves.size(); ++i) {
    const BlockLeaf& l = p.bct.leaves[i];
    const Node& a = p.ss.et.nodes[l.c1];
    const Node& b = p.ss.et.nodes[l.c2];
    int* o = out + 7 * i;
    o[0] = l.cc; o[1] = a.level; o[2] = a.id; o[3] = b.id;
    o[4] = p.ss.et.cluster_first(l.c1); o[5] = p.ss.et.cluster_first(l.c2); o[6] = p.ss.et.cluster_size(l.c1);
  }
}

// one leaf's F block (row_comp, col_comp); complex values interleaved
int orc_leaf_matrix(void* h, long leaf, int rc, int cc, double* out) {
  Problem& p = *static_cast<Problem*>(h);
  int vd = p.vd();
  if (p.op.is_complex()) {
    if (p.leaves_c.empty()) return -1;
    const Mat<cplx>& F = p.leaves_c[leaf].F[rc * vd + cc];
    std::memcpy(out, F.a.data(), F.a.size() * sizeof(cplx));
  } else {
    if (p.leaves_r.empty()) return -1;
    const Mat<double>& F = p.leaves_r[leaf].F[rc * vd + cc];
    std::memcpy(out, F.a.data(), F.a.size() * sizeof(double));
  }
  return 0;
}

// Put a leaf matrix (column-major, the layout orc_leaf_matrix reads) into a
// problem created without assembly, for timing the CPU products and solves
// on entries computed elsewhere. The first call sizes the leaf table from the
// block partition.
int orc_set_leaf(void* h, long leaf, int rc, int cc, const double* in) {
  Problem& p = *static_cast<Problem*>(h);
  const int vd = p.vd(), n = p.ss.p2();
  if (leaf < 0 || leaf >= (long)p.bct.leaves.size() || rc < 0 || rc >= vd || cc < 0 || cc >= vd) return -1;
  auto fill = [&](auto& L, auto zero) -> int {
    using S = decltype(zero);
    if (L.size() != p.bct.leaves.size()) {
      L.resize(p.bct.leaves.size());
      for (size_t li = 0; li < L.size(); ++li) {
        L[li].cc = p.bct.leaves[li].cc;
        L[li].c1 = p.bct.leaves[li].c1;
        L[li].c2 = p.bct.leaves[li].c2;
      }
    }
    const BlockLeaf& bl = p.bct.leaves[leaf];
    const int rows = bl.cc == kDense ? p.ss.et.cluster_size(bl.c1) * n : p.op.nc() * p.np * p.np;
    const int cols = bl.cc == kDense ? p.ss.et.cluster_size(bl.c2) * n : p.op.nc() * p.np * p.np;
    auto& F = L[leaf].F;
    if (F.size() != (size_t)vd * vd) F.assign(vd * vd, Mat<S>(rows, cols));
    std::memcpy(static_cast<void*>(F[rc * vd + cc].a.data()), in, (size_t)rows * cols * sizeof(S));
    return 0;
  };
  if (p.op.is_complex()) return fill(p.leaves_c, cplx(0));
  return fill(p.leaves_r, 0.0);
}

// intval of evaluateBilinearForm for one element pair ((vd p^2)^2, col-major)
void orc_element_pair(void* h, int id1, int id2, double* out) {
  Problem& p = *static_cast<Problem*>(h);
  int n = p.vd() * p.ss.p2();
  if (p.op.is_complex()) {
    Mat<cplx> iv(n, n);
    bilinear_form<cplx>(p.op, p.ss, id1, id2, p.ffq, &iv);
    std::memcpy(out, iv.a.data(), iv.a.size() * sizeof(cplx));
  } else {
    Mat<double> iv(n, n);
    bilinear_form<double>(p.op, p.ss, id1, id2, p.ffq, &iv);
    std::memcpy(out, iv.a.data(), iv.a.size() * sizeof(double));
  }
}

// classification of an element pair: case, rot1, rot2, quadrature degree, dist
void orc_pair_class(void* h, int id1, int id2, int* out, double* dist) {
  Problem& p = *static_cast<Problem*>(h);
  const Node& e1 = p.ss.element(id1);
  const Node& e2 = p.ss.element(id2);
  Cmp c = compare_elements(e1, e2, id1 == id2, dist);
  int ff = p.op.ffield_deg();
  int nf = p.op.nfield_deg(*dist, e1.level);
  out[0] = c.cs; out[1] = c.rot1; out[2] = c.rot2; out[3] = nf >= ff ? nf : ff;
}

// the dummy-operator DuffyTrick integrals of tests/DuffyTrick/test_integrate*.hpp
double orc_dummy_integrate(void* h, int which, int id1, int id2, int qdeg, int rot1, int rot2) {
  Problem& p = *static_cast<Problem*>(h);
  const Cubature& Q = GS(qdeg);
  Mat<double> iv(1, 1);
  const Node& e1 = p.ss.element(id1);
  const Node& e2 = p.ss.element(id2);
  switch (which) {
    case 0: {
      auto f = ffield_qnodes(p.ss, Q);
      integrate0<double>(p.op, p.ss, f[e1.id], f[e2.id], &iv);
      break;
    }
    case 1: integrate1<double>(p.op, p.ss, e1, e2, Q, &iv); break;
    case 2: integrate2<double>(p.op, p.ss, e1, Q, &iv); break;
    case 3: integrate3<double>(p.op, p.ss, e1, rot1, e2, rot2, Q, &iv); break;
    case 4: integrate4<double>(p.op, p.ss, e1, rot1, e2, rot2, Q, &iv); break;
  }
  return iv(0, 0);
}

// single-point integrand (test_Laplace.cpp / test_Helmholtz.cpp)
void orc_point_integrand(void* h, int id, double s1, double t1, double s2, double t2, double* out) {
  Problem& p = *static_cast<Problem*>(h);
  SurfacePoint a, b;
  const Node& e = p.ss.element(id);
  p.ss.map2surface(e, s1, t1, 1, &a);
  p.ss.map2surface(e, s2, t2, 1, &b);
  int n = p.vd() * p.ss.p2();
  if (p.op.is_complex()) {
    Mat<cplx> iv(n, n);
    integrand<cplx>(p.op, p.ss, a, b, &iv);
    std::memcpy(out, iv.a.data(), iv.a.size() * sizeof(cplx));
  } else {
    Mat<double> iv(n, n);
    integrand<double>(p.op, p.ss, a, b, &iv);
    std::memcpy(out, iv.a.data(), iv.a.size() * sizeof(double));
  }
}

// Patch::updateSurfacePoint at patch coordinates (s, t)
void orc_surface_point(void* h, int patch, double s, double t, double* out12) {
  Problem& p = *static_cast<Problem*>(h);
  SurfacePoint sp;
  p.ss.et.geo[patch].update(&sp, s, t, 1, s, t);
  std::memcpy(out12, sp.v, sizeof(sp.v));
}

// FMM matrices: transfer (np^2 x 4np^2) and Moment2D for arbitrary levels
void orc_transfer_matrices(int np, double* out) {
  Mat<double> T = transfer_matrices(np);
  std::memcpy(out, T.a.data(), T.a.size() * sizeof(double));
}
void orc_moment2d(int P, int cluster_level, int cluster_ref, int np, int d1, int d2, double* out) {
  init_rules();
  Mat<double> m = moment2d(P, cluster_level, cluster_ref, np, d1 != 0, d2 != 0);
  std::memcpy(out, m.a.data(), m.a.size() * sizeof(double));
}
// moment matrix of the problem for vector component comp
void orc_moments(void* h, int comp, double* out) {
  Problem& p = *static_cast<Problem*>(h);
  std::memcpy(out, p.mom[comp].a.data(), p.mom[comp].a.size() * sizeof(double));
}
// forwardTransformation on real data: returns all levels concatenated
void orc_forward_transform(const double* mom, int mr, int mcols, const double* T, int np, int steps,
                           const double* X, int xcols, double* out) {
  Mat<double> Mm(mr, mcols), Tm(np * np, 4 * np * np), Xm(mcols, xcols);
  std::memcpy(Mm.a.data(), mom, Mm.a.size() * sizeof(double));
  std::memcpy(Tm.a.data(), T, Tm.a.size() * sizeof(double));
  std::memcpy(Xm.a.data(), X, Xm.a.size() * sizeof(double));
  auto f = forward_transform<double>(Mm, Tm, steps, Xm);
  size_t o = 0;
  for (auto& m : f) {
    std::memcpy(out + o, m.a.data(), m.a.size() * sizeof(double));
    o += m.a.size();
  }
}
// backwardTransformation on real data; Z holds steps+1 levels (level i has
// xcols / 4^i columns), concatenated
void orc_backward_transform(const double* mom, int mr, int mcols, const double* T, int np, int steps,
                            const double* Z, int xcols, double* out) {
  Mat<double> Mm(mr, mcols), Tm(np * np, 4 * np * np);
  std::memcpy(Mm.a.data(), mom, Mm.a.size() * sizeof(double));
  std::memcpy(Tm.a.data(), T, Tm.a.size() * sizeof(double));
  std::vector<Mat<double>> Zs;
  size_t o = 0;
  int c = xcols;
  for (int i = 0; i <= steps; ++i) {
    Zs.emplace_back(mr, c);
    std::memcpy(Zs.back().a.data(), Z + o, Zs.back().a.size() * sizeof(double));
    o += Zs.back().a.size();
    c /= 4;
  }
  auto v = backward_transform<double>(Mm, Tm, steps, Zs);
  std::memcpy(out, v.data(), v.size() * sizeof(double));
}

// y = A x at DOF level (complex values interleaved), nrhs columns
int orc_matvec(void* h, const double* x, double* y, int nrhs) {
  Problem& p = *static_cast<Problem*>(h);
  if (p.op.is_complex()) {
    if (p.leaves_c.empty()) return -1;
    h2_matvec<cplx>(p, reinterpret_cast<const cplx*>(x), reinterpret_cast<cplx*>(y), nrhs);
  } else {
    if (p.leaves_r.empty()) return -1;
    h2_matvec<double>(p, x, y, nrhs);
  }
  return 0;
}
// y = A_ss x at superspace level
int orc_matvec_ss(void* h, const double* x, double* y) {
  Problem& p = *static_cast<Problem*>(h);
  if (p.op.is_complex()) {
    if (p.leaves_c.empty()) return -1;
    h2_product_ss<cplx>(p, reinterpret_cast<const cplx*>(x), reinterpret_cast<cplx*>(y));
  } else {
    if (p.leaves_r.empty()) return -1;
    h2_product_ss<double>(p, x, y);
  }
  return 0;
}
// dense superspace Galerkin matrix (S x S, column-major)
void orc_dense_ss(void* h, double* out) {
  Problem& p = *static_cast<Problem*>(h);
  if (p.op.is_complex()) dense_ss<cplx>(p, reinterpret_cast<cplx*>(out));
  else dense_ss<double>(p, out);
}
// load vector for a data function (kind, params[8])
void orc_load_vector(void* h, int kind, const double* prm, double* out) {
  Problem& p = *static_cast<Problem*>(h);
  DataFun f;
  f.kind = kind;
  for (int i = 0; i < 8; ++i) f.prm[i] = prm[i];
  f.kappa = p.op.kappa;
  if (p.op.is_complex()) load_vector<cplx>(p, f, reinterpret_cast<cplx*>(out));
  else load_vector<double>(p, f, out);
}
void orc_potential(void* h, const double* rho, const double* pts, int npts, double* out) {
  Problem& p = *static_cast<Problem*>(h);
  if (p.op.kind == kMaxwell)
    potential_mw(p, reinterpret_cast<const cplx*>(rho), pts, npts, reinterpret_cast<cplx*>(out));
  else if (p.op.is_complex())
    potential<cplx>(p, reinterpret_cast<const cplx*>(rho), pts, npts, reinterpret_cast<cplx*>(out));
  else
    potential<double>(p, rho, pts, npts, out);
}
int orc_gmres(void* h, const double* b, double* x, double tol, int restart, int maxit) {
  Problem& p = *static_cast<Problem*>(h);
  if (p.op.is_complex())
    return gmres<cplx>(p, reinterpret_cast<const cplx*>(b), reinterpret_cast<cplx*>(x), tol, restart, maxit);
  return gmres<double>(p, b, x, tol, restart, maxit);
}
int orc_cg(void* h, const double* b, double* x, double tol, int maxit, double* relres) {
  Problem& p = *static_cast<Problem*>(h);
  if (p.op.is_complex()) return -1;
  return cg(p, b, x, tol, maxit, relres);
}
int orc_threads() { return omp_get_max_threads(); }

}  // extern "C"
