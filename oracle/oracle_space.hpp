// ORACLE — test infrastructure only (see oracle_core.hpp header).
//
// Part 3: the transformation matrix T = Projector * Glue of the AnsatzSpace
// (AnsatzSpace/AnsatzSpace.hpp:102-111), as a list of triplets.
#pragma once
#include "oracle_h2.hpp"

namespace orc {

struct Triplet {
  int r, c;
  double v;
};
struct Sparse {  // CSR
  int rows = 0, cols = 0;
  std::vector<int> ptr, idx;
  std::vector<double> val;
  static Sparse from_triplets(int rows, int cols, std::vector<Triplet> t) {
    std::sort(t.begin(), t.end(), [](const Triplet& a, const Triplet& b) {
      return a.r != b.r ? a.r < b.r : a.c < b.c;
    });
    Sparse s;
    s.rows = rows;
    s.cols = cols;
    s.ptr.assign(rows + 1, 0);
    for (size_t k = 0; k < t.size(); ++k) {
      if (!s.idx.empty() && k > 0 && t[k].r == t[k - 1].r && t[k].c == t[k - 1].c) {
        s.val.back() += t[k].v;  // setFromTriplets sums duplicates
        continue;
      }
      s.idx.push_back(t[k].c);
      s.val.push_back(t[k].v);
      s.ptr[t[k].r + 1]++;
    }
    for (int r = 0; r < rows; ++r) s.ptr[r + 1] += s.ptr[r];
    return s;
  }
  Sparse mul(const Sparse& B) const {  // this * B
    std::vector<Triplet> t;
    for (int r = 0; r < rows; ++r)
      for (int k = ptr[r]; k < ptr[r + 1]; ++k) {
        int m = idx[k];
        for (int l = B.ptr[m]; l < B.ptr[m + 1]; ++l) t.push_back({r, B.idx[l], val[k] * B.val[l]});
      }
    return from_triplets(rows, B.cols, t);
  }
  template <typename S>
  void apply(const S* x, S* y) const {  // y = A x
    for (int r = 0; r < rows; ++r) {
      S acc = 0;
      for (int k = ptr[r]; k < ptr[r + 1]; ++k) acc += val[k] * x[idx[k]];
      y[r] = acc;
    }
  }
  template <typename S>
  void apply_t(const S* x, S* y) const {  // y = A^T x
    for (int c = 0; c < cols; ++c) y[c] = 0;
    for (int r = 0; r < rows; ++r)
      for (int k = ptr[r]; k < ptr[r + 1]; ++k) y[idx[k]] += val[k] * x[r];
  }
};

// Knots.hpp: MakeUniformKnotVector(order, interior, repetition)
inline std::vector<double> uniform_knots(int order, int interior, int rep) {
  std::vector<double> out;
  double h = 1. / (interior + 1);
  for (int i = 0; i < order; ++i) out.push_back(0);
  for (int i = 1; i < interior + 1; ++i)
    for (int k = 0; k < rep; ++k) out.push_back(i * h);
  for (int i = 0; i < order; ++i) out.push_back(1);
  return out;
}
// DeBoor.hpp (vector version): evaluate the spline with coefficients c
inline double deboor(const std::vector<double>& c, const std::vector<double>& knots, double x) {
  int ncp = (int)c.size();
  int p = (int)knots.size() - ncp - 1;
  int l = 0;
  while (knots[l] <= x && l != ncp) l++;
  l = l - 1;
  std::vector<double> tmp(c.begin() + l - p, c.begin() + l + 1);
  for (int k = p; k != 0; k--) {
    double ws[64];
    for (int i = 0; i < k; i++)
      ws[i] = (x - knots[l - k + 1 + i]) / (knots[l + 1 + i] - knots[l - k + 1 + i]);
    for (int i = 0; i < k; i++) tmp[i] = ws[i] * tmp[1 + i] + (1 - ws[i]) * tmp[i];
  }
  return tmp[0];
}

// small dense LU with partial pivoting (row-major n x n)
struct LU {
  int n = 0;
  std::vector<double> a;
  std::vector<int> piv;
  void factor(std::vector<double> A, int n_) {
    n = n_;
    a = A;
    piv.resize(n);
    for (int k = 0; k < n; ++k) {
      int p = k;
      for (int i = k + 1; i < n; ++i)
        if (std::fabs(a[i * n + k]) > std::fabs(a[p * n + k])) p = i;
      piv[k] = p;
      if (p != k)
        for (int j = 0; j < n; ++j) std::swap(a[k * n + j], a[p * n + j]);
      for (int i = k + 1; i < n; ++i) {
        a[i * n + k] /= a[k * n + k];
        for (int j = k + 1; j < n; ++j) a[i * n + j] -= a[i * n + k] * a[k * n + j];
      }
    }
  }
  std::vector<double> solve(std::vector<double> b) const {
    for (int k = 0; k < n; ++k) std::swap(b[k], b[piv[k]]);
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < i; ++j) b[i] -= a[i * n + j] * b[j];
    for (int i = n - 1; i >= 0; --i) {
      for (int j = i + 1; j < n; ++j) b[i] -= a[i * n + j] * b[j];
      b[i] /= a[i * n + i];
    }
    return b;
  }
};

// makeLocalProjectionTriplets (AnsatzSpace/Projector.hpp:165-~340)
struct ProjInfo {
  std::vector<Triplet> t;
  int num_c_dof = 0, num_dc_dof = 0;
};
inline ProjInfo local_projection(const SuperSpace& ss, int pp1x, int pp1y, int rep_in) {
  const int M = ss.et.max_level;
  const int maxp = std::max(pp1x, pp1y);
  const int minp = std::min(pp1x, pp1y);
  const int rep = (maxp <= rep_in) ? minp : rep_in;
  const int n = 1 << M;
  const int npatch = ss.et.npatches;
  std::vector<double> kx = uniform_knots(pp1x, n - 1, rep);
  std::vector<double> ky = uniform_knots(pp1y, n - 1, rep);
  const int dx = (int)kx.size() - pp1x, dy = (int)ky.size() - pp1y, dim = dx * dy;
  std::vector<double> mask(maxp);
  {
    double h = 1. / (maxp + 1);
    for (int i = 0; i < maxp; ++i) mask[i] = (i + 1) * h;
  }
  const int ms = maxp;
  std::vector<double> sys(ms * ms * maxp * maxp);
  double vy[64], vx[64];
  for (int iy = 0; iy < maxp; ++iy) {
    bernstein_basis(maxp - 1, mask[iy], vy);
    for (int ix = 0; ix < maxp; ++ix) {
      bernstein_basis(maxp - 1, mask[ix], vx);
      for (int jy = 0; jy < maxp; ++jy)
        for (int jx = 0; jx < maxp; ++jx)
          sys[(iy * ms + ix) * (maxp * maxp) + jy * maxp + jx] = vx[jx] * vy[jy];
    }
  }
  LU lu;
  lu.factor(sys, ms * ms);
  ProjInfo out;
  for (int e = 0; e < ss.ne(); ++e) {
    const Node& el = ss.element(e);
    double px = el.llc[0], py = el.llc[1], h = el.h();
    double mx = px + .5 * h, my = py + .5 * h;
    std::vector<int> nzx, nzy;
    for (int d = 0; d < dy; ++d)
      if (ky[d] <= my && ky[d + pp1y] >= my) nzy.push_back(d);
    for (int d = 0; d < dx; ++d)
      if (kx[d] <= mx && kx[d + pp1x] >= mx) nzx.push_back(d);
    for (int dofy : nzy)
      for (int dofx : nzx) {
        std::vector<double> cx(dx, 0.0), cy(dy, 0.0);
        cx[dofx] = 1;
        cy[dofy] = 1;
        std::vector<double> vxs(ms), vys(ms);
        for (int i = 0; i < ms; ++i) {
          vxs[i] = deboor(cx, kx, px + (1.0 / n) * mask[i]);
          vys[i] = deboor(cy, ky, py + (1.0 / n) * mask[i]);
        }
        std::vector<double> rhs(ms * ms);
        for (int iy = 0; iy < ms; ++iy)
          for (int ix = 0; ix < ms; ++ix) rhs[iy * ms + ix] = vxs[ix] * vys[iy];
        std::vector<double> sol = lu.solve(rhs);
        for (int i = 0; i < maxp * maxp; ++i)
          if (std::fabs(sol[i]) > kProjectorTol)
            out.t.push_back({e * maxp * maxp + i, el.patch * dim + dx * dofy + dofx, sol[i]});
      }
  }
  out.num_c_dof = dim * npatch;
  out.num_dc_dof = maxp * maxp * n * n * npatch;
  return out;
}

// Glue.hpp: identification of dofs (DivConforming only; Discontinuous = I)
namespace glue {
inline std::vector<int> edge_dofs(int ec, int dimx, int dimy, int shift) {
  std::vector<int> out;
  switch (ec) {
    case 0: for (int i = 0; i < dimx; ++i) out.push_back(i + shift); break;
    case 1: for (int i = 0; i < dimy; ++i) out.push_back(dimx * (i + 1) - 1 + shift); break;
    case 2: for (int i = 0; i < dimx; ++i) out.push_back(dimx * (dimy - 1) + i + shift); break;
    case 3: for (int i = 0; i < dimy; ++i) out.push_back(dimx * i + shift); break;
    default: break;
  }
  return out;
}
inline bool fwd(int e) { return e == 0 || e == 1; }
inline bool inward(int e) { return e == 0 || e == 3; }
inline bool first_comp(int e) { return !(e == 0 || e == 2); }
struct DofId {
  std::vector<int> dofs;
  int coef = 1;
};
}  // namespace glue

inline Sparse glue_divconforming(const SuperSpace& ss, int rep, int pre_dofs) {
  using namespace glue;
  auto edges = ss.et.patch_topology();
  const int M = ss.et.max_level, P = ss.P, npatch = ss.et.npatches;
  const int small_dim = P + rep * ((1 << M) - 1);
  const int large_dim = P + 1 + rep * ((1 << M) - 1);
  const int per = small_dim * large_dim;
  std::vector<DofId> ids;
  for (auto& e : edges) {
    int s1 = e[0] * per + (first_comp(e[2]) ? 0 : per * npatch);
    int s2 = e[1] * per + (first_comp(e[3]) ? 0 : per * npatch);
    int xd1 = first_comp(e[2]) ? large_dim : small_dim, yd1 = first_comp(e[2]) ? small_dim : large_dim;
    int xd2 = first_comp(e[3]) ? large_dim : small_dim, yd2 = first_comp(e[3]) ? small_dim : large_dim;
    auto d1 = edge_dofs(e[2], xd1, yd1, s1);
    auto d2 = edge_dofs(e[3], xd2, yd2, s2);
    bool rev = (fwd(e[2]) && fwd(e[3])) || (!fwd(e[2]) && !fwd(e[3]));
    int coef = ((inward(e[2]) && inward(e[3])) || (!inward(e[2]) && !inward(e[3]))) ? -1 : 1;
    int sz = (int)d1.size();
    if (e[1] > -1 && e[0] > -1) {
      for (int i = 0; i < sz; ++i) {
        int j = rev ? sz - 1 - i : i;
        DofId d;
        d.dofs.push_back(std::min(d1[i], d2[j]));
        d.dofs.push_back(std::max(d1[i], d2[j]));
        d.coef = coef;
        ids.push_back(d);
      }
    } else {
      for (int i = 0; i < sz; ++i) {
        DofId d;
        d.dofs.push_back(d1[i]);
        ids.push_back(d);
      }
    }
  }
  // assembleGlueMatrix (Glue.hpp:~120-190)
  std::vector<char> is_slave(pre_dofs, 0), is_master(pre_dofs, 0);
  int nslaves = 0, nbnd = 0;
  for (auto& d : ids) {
    std::sort(d.dofs.begin(), d.dofs.end());
    is_master[d.dofs[0]] = 1;
    if (d.dofs.size() == 1) ++nbnd;
    for (size_t i = 1; i < d.dofs.size(); ++i) {
      is_slave[d.dofs[i]] = 1;
      ++nslaves;
    }
  }
  std::stable_sort(ids.begin(), ids.end(), [](const DofId& a, const DofId& b) { return a.dofs[0] < b.dofs[0]; });
  const int post = pre_dofs - nslaves - nbnd;
  const int glued = pre_dofs - nslaves;
  std::vector<Triplet> t;
  int skip = 0, mi = 0, pi = 0;
  for (int i = 0; i < glued; ++i) {
    while ((i + skip) < pre_dofs && is_slave[i + skip]) ++skip;
    int pre = i + skip;
    if (is_master[pre] && ids[mi].dofs.size() == 1) {
      ++mi;
      continue;
    }
    t.push_back({pre, pi, 1.0});
    if (is_master[pre]) {
      for (size_t j = 1; j < ids[mi].dofs.size(); ++j) t.push_back({ids[mi].dofs[j], pi, (double)ids[mi].coef});
      ++mi;
    }
    ++pi;
  }
  return Sparse::from_triplets(pre_dofs, post, t);
}

// Projector::get_projection_matrix (Projector.hpp:52-90): the spline space of
// every patch in the superspace, before any gluing; div-conforming: the two
// components (degrees (P+1, P) and (P, P+1) per direction) stacked
inline Sparse projector_matrix(const SuperSpace& ss, int kind, int rep = 1) {
  const int P = ss.P;
  if (kind != kMaxwell) {
    ProjInfo pi = local_projection(ss, P + 1, P + 1, rep);
    return Sparse::from_triplets(pi.num_dc_dof, pi.num_c_dof, pi.t);
  }
  ProjInfo a = local_projection(ss, P + 1, P, rep);
  ProjInfo b = local_projection(ss, P, P + 1, rep);
  std::vector<Triplet> t = a.t;
  for (auto x : b.t) t.push_back({x.r + a.num_dc_dof, x.c + a.num_c_dof, x.v});
  return Sparse::from_triplets(a.num_dc_dof + b.num_dc_dof, a.num_c_dof + b.num_c_dof, t);
}

// AnsatzSpace::init_AnsatzSpace (AnsatzSpace.hpp:102-111), knot repetition 1
inline Sparse transformation_matrix(const SuperSpace& ss, int kind, int rep = 1) {
  Sparse proj = projector_matrix(ss, kind, rep);
  if (kind != kMaxwell) return proj;
  Sparse g = glue_divconforming(ss, rep, proj.cols);
  return proj.mul(g);
}

}  // namespace orc
