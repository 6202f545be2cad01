// ORACLE — test infrastructure only. CPU restatement of Bembel's hot path,
// used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as
// the checker. Nothing in the bembel_gb300 package links or calls this code.
//
// Part 1: geometry (Bezier-extracted NURBS patches), element tree with the
// reference's topological vertex numbering, enclosing balls, block cluster
// partition, Gauss-Legendre rules and Bernstein bases.
//
// Parity pins: tests/test_oracle_*.py check this restatement against the
// reference's own known-answer tests (FMM identities < 1e-12, DuffyTrick
// closed-form integrals, integrand point values, sphere-panel geometry,
// H2-vs-dense < 1e-8), restated as Python tests.
#pragma once
#include <algorithm>
#include <array>
#include <cassert>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace orc {

constexpr double kPi = 3.14159265358979323846;
constexpr double kGenericTol = 1e-6;     // util/Constants.hpp:22
constexpr double kPtCompTol = 1e-9;      // util/Constants.hpp:30
constexpr double kProjectorTol = 1e-4;   // util/Constants.hpp:32
constexpr int kMaxQuadDeg = 50;          // util/Constants.hpp:25

using cplx = std::complex<double>;

struct V3 {
  double x = 0, y = 0, z = 0;
  V3() {}
  V3(double a, double b, double c) : x(a), y(b), z(c) {}
  V3 operator+(const V3& o) const { return V3(x + o.x, y + o.y, z + o.z); }
  V3 operator-(const V3& o) const { return V3(x - o.x, y - o.y, z - o.z); }
  V3 operator*(double s) const { return V3(x * s, y * s, z * s); }
  double dot(const V3& o) const { return x * o.x + y * o.y + z * o.z; }
  V3 cross(const V3& o) const {
    return V3(y * o.z - z * o.y, z * o.x - x * o.z, x * o.y - y * o.x);
  }
  double norm() const { return std::sqrt(x * x + y * y + z * z); }
};

// ---------------------------------------------------------------------------
// Bernstein polynomials (Spline/Bernstein.hpp:22-47, 164-246).
// B_{i,p}(x) = C(p,i) x^i (1-x)^(p-i); derivative p (B_{i-1,p-1} - B_{i,p-1}).
inline double binom(int n, int k) {
  double r = 1;
  for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
  return r;
}
inline double ipow(double x, int n) {
  double r = 1;
  for (int i = 0; i < n; ++i) r *= x;
  return r;
}
inline double bernstein(int i, int p, double x) {
  if (i < 0 || i > p) return 0;
  return binom(p, i) * ipow(x, i) * ipow(1. - x, p - i);
}
inline void bernstein_basis(int p, double x, double* out) {
  for (int i = 0; i <= p; ++i) out[i] = bernstein(i, p, x);
}
inline void bernstein_der_basis(int p, double x, double* out) {
  if (p == 0) {
    out[0] = 0;
    return;
  }
  for (int i = 0; i <= p; ++i)
    out[i] = p * (bernstein(i - 1, p - 1, x) - bernstein(i, p - 1, x));
}

// ---------------------------------------------------------------------------
// Gauss-Legendre on [0,1] with n points (Quadrature/GaussLegendreRule.hpp):
// nodes ascending. Restated by Newton iteration on the Legendre recurrence
// instead of the reference's hard-coded tables / Golub-Welsch eigen solve;
// both give the same nodes to within a few ulps.
struct Rule1D {
  std::vector<double> xi, w;
};
inline Rule1D gauss_legendre(int n) {
  Rule1D r;
  r.xi.resize(n);
  r.w.resize(n);
  for (int i = 0; i < n; ++i) {
    // i-th root counting from the largest on [-1,1]
    double x = std::cos(kPi * (i + 0.75) / (n + 0.5));
    double dp = 0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1, p1 = x;
      for (int k = 2; k <= n; ++k) {
        double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      if (n == 1) {
        p1 = x;
        p0 = 1;
      }
      dp = n * (x * p1 - p0) / (x * x - 1);
      double dx = p1 / dp;
      x -= dx;
      if (std::fabs(dx) < 1e-16) break;
    }
    {
      double p0 = 1, p1 = x;
      for (int k = 2; k <= n; ++k) {
        double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      dp = n * (x * p1 - p0) / (x * x - 1);
    }
    // map to [0,1], ascending order
    r.xi[n - 1 - i] = 0.5 * (x + 1);
    r.w[n - 1 - i] = 1.0 / ((1 - x * x) * dp * dp);
  }
  if (n == 1) {
    r.xi[0] = 0.5;
    r.w[0] = 1.0;
  }
  return r;
}
// GaussLegendre<..>[k] has k+1 points (Quadrature/QuadratureVector.hpp:24-30).
inline const Rule1D& GL(int k) {
  static std::vector<Rule1D> rules;
  static bool init = false;
  if (!init) {
    for (int i = 0; i <= kMaxQuadDeg + 1; ++i) rules.push_back(gauss_legendre(i + 1));
    init = true;
  }
  return rules.at(k);
}
// GaussSquare<..>[k]: (k+1)^2 points, first coordinate slowest
// (Quadrature/TensorProductQuadratureVector.hpp:23-35).
struct Cubature {
  std::vector<double> x0, x1, w;
  int size() const { return (int)w.size(); }
};
inline const Cubature& GS(int k) {
  static std::vector<Cubature> rules;
  static bool init = false;
  if (!init) {
    for (int d = 0; d <= kMaxQuadDeg; ++d) {
      const Rule1D& g = GL(d);
      Cubature c;
      int n = (int)g.xi.size();
      for (int q = 0; q < n * n; ++q) {
        c.x0.push_back(g.xi[q / n]);
        c.x1.push_back(g.xi[q % n]);
        c.w.push_back(g.w[q / n] * g.w[q % n]);
      }
      rules.push_back(c);
    }
    init = true;
  }
  return rules.at(k);
}
// Make sure the static tables are built before any OpenMP region.
inline void init_rules() {
  GL(0);
  GS(0);
}

// ---------------------------------------------------------------------------
// SurfacePoint (Geometry/SurfacePoint.hpp:15-42): [xi(2), w, x(3), dx(3), dy(3)]
struct SurfacePoint {
  double v[12];
  V3 x() const { return V3(v[3], v[4], v[5]); }
  V3 dx() const { return V3(v[6], v[7], v[8]); }
  V3 dy() const { return V3(v[9], v[10], v[11]); }
};

// Patch in Bezier form (Geometry/Patch.hpp:63-104). Only single-Bezier
// patches (knot vectors without interior knots) are supported here.
//
// face >= 0 marks an analytic cube-sphere patch instead (no reference
// counterpart; the benchmark's sphere is defined this way): the unit-sphere
// image c / |c| of c(s, t) = sg e_k + (2 s - 1) e_a + (2 t - 1) e_b on the
// cube face x_k = sg, k = face / 2, sg = +1 for even faces with (a, b) =
// (k + 1, k + 2) mod 3 and sg = -1 for odd faces with (a, b) = (k + 2, k + 1)
// mod 3; its derivatives follow from d(c / |c|) = (I - u u^T) dc / |c|.
struct Patch {
  std::vector<double> data;  // [(ix*py + iy)*4 + k], k in {x,y,z,w}
  int px = 0, py = 0;        // orders (degree + 1) in x and y
  int face = -1;

  void cube_face(double s, double t, V3* x, V3* ds, V3* dt) const {
    const int k = face / 2;
    const bool pos = face % 2 == 0;
    const int a = pos ? (k + 1) % 3 : (k + 2) % 3, b = pos ? (k + 2) % 3 : (k + 1) % 3;
    double c[3];
    c[k] = pos ? 1.0 : -1.0;
    c[a] = 2 * s - 1;
    c[b] = 2 * t - 1;
    const double ir = 1.0 / std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
    double u[3], da[3], db[3];
    for (int j = 0; j < 3; ++j) u[j] = c[j] * ir;
    for (int j = 0; j < 3; ++j) {
      da[j] = 2.0 * ((j == a ? 1.0 : 0.0) - u[j] * u[a]) * ir;
      db[j] = 2.0 * ((j == b ? 1.0 : 0.0) - u[j] * u[b]) * ir;
    }
    *x = V3(u[0], u[1], u[2]);
    *ds = V3(da[0], da[1], da[2]);
    *dt = V3(db[0], db[1], db[2]);
  }

  // Patch::eval (Patch.hpp:115-155)
  V3 eval(double s, double t) const {
    if (face >= 0) {
      V3 x, ds, dt;
      cube_face(s, t, &x, &ds, &dt);
      return x;
    }
    double xb[32], yb[32];
    bernstein_basis(px - 1, s, xb);
    bernstein_basis(py - 1, t, yb);
    double tmp[4] = {0, 0, 0, 0};
    for (int i = 0; i < px; ++i)
      for (int j = 0; j < py; ++j) {
        double b = xb[i] * yb[j];
        const double* d = &data[4 * (i * py + j)];
        for (int k = 0; k < 4; ++k) tmp[k] += d[k] * b;
      }
    return V3(tmp[0] / tmp[3], tmp[1] / tmp[3], tmp[2] / tmp[3]);
  }
  // Patch::evalJacobian (Patch.hpp:163-232)
  void jacobian(double s, double t, V3* ds, V3* dt) const {
    SurfacePoint sp;
    update(&sp, s, t, 1, 0, 0);
    *ds = sp.dx();
    *dt = sp.dy();
  }
  // Patch::updateSurfacePoint (Patch.hpp:294-365)
  void update(SurfacePoint* sp, double s, double t, double w, double xi0,
              double xi1) const {
    if (face >= 0) {
      V3 x, ds, dt;
      cube_face(s, t, &x, &ds, &dt);
      sp->v[0] = xi0;
      sp->v[1] = xi1;
      sp->v[2] = w;
      const V3* f[3] = {&x, &ds, &dt};
      for (int r = 0; r < 3; ++r) {
        sp->v[3 + 3 * r] = f[r]->x;
        sp->v[4 + 3 * r] = f[r]->y;
        sp->v[5 + 3 * r] = f[r]->z;
      }
      return;
    }
    double xb[32], yb[32], xbd[32], ybd[32];
    bernstein_basis(px - 1, s, xb);
    bernstein_basis(py - 1, t, yb);
    bernstein_der_basis(px - 1, s, xbd);
    bernstein_der_basis(py - 1, t, ybd);
    double tmp[4] = {0, 0, 0, 0}, tdx[4] = {0, 0, 0, 0}, tdy[4] = {0, 0, 0, 0};
    for (int i = 0; i < px; ++i)
      for (int j = 0; j < py; ++j) {
        double b = xb[i] * yb[j], bx = xbd[i] * yb[j], by = xb[i] * ybd[j];
        const double* d = &data[4 * (i * py + j)];
        for (int k = 0; k < 4; ++k) {
          tmp[k] += d[k] * b;
          tdx[k] += d[k] * bx;
          tdy[k] += d[k] * by;
        }
      }
    double bot = 1. / tmp[3], b2 = bot * bot;
    sp->v[0] = xi0;
    sp->v[1] = xi1;
    sp->v[2] = w;
    for (int k = 0; k < 3; ++k) {
      sp->v[3 + k] = tmp[k] * bot;
      sp->v[6 + k] = (tdx[k] * tmp[3] - tmp[k] * tdx[3]) * b2;
      sp->v[9 + k] = (tdy[k] * tmp[3] - tmp[k] * tdy[3]) * b2;
    }
  }
};

// The six analytic cube-sphere faces (see Patch::face).
inline std::vector<Patch> cube_sphere() {
  std::vector<Patch> out(6);
  for (int f = 0; f < 6; ++f) out[f].face = f;
  return out;
}

// LoadGeometryFileDAT (Geometry/GeometryIO.hpp:25-122): Octave NURBS text.
// The name "analytic:cube_sphere" selects the analytic cube sphere instead.
inline std::vector<Patch> load_dat(const std::string& path) {
  if (path == "analytic:cube_sphere") return cube_sphere();
  std::ifstream f(path);
  if (!f) throw std::runtime_error("cannot open geometry file " + path);
  std::string row;
  for (int i = 0; i < 5; ++i) std::getline(f, row);
  int info5[5];
  {
    std::istringstream is(row);
    for (int i = 0; i < 5; ++i) is >> info5[i];
  }
  std::vector<Patch> out;
  for (int pn = 0; pn < info5[2]; ++pn) {
    std::getline(f, row);  // PATCH n
    int p1, p2, n1, n2;
    std::getline(f, row);
    { std::istringstream is(row); is >> p1 >> p2; }
    std::getline(f, row);
    { std::istringstream is(row); is >> n1 >> n2; }
    std::vector<double> k1(p1 + n1 + 1), k2(p2 + n2 + 1);
    std::getline(f, row);
    { std::istringstream is(row); for (auto& v : k1) is >> v; }
    std::getline(f, row);
    { std::istringstream is(row); for (auto& v : k2) is >> v; }
    // 4 matrices, each rows = n2 (y), cols = n1 (x), row-major in the file
    std::vector<std::vector<double>> mats(4, std::vector<double>(n1 * n2));
    for (int k = 0; k < 4; ++k) {
      std::getline(f, row);
      std::istringstream is(row);
      for (int i = 0; i < n2; ++i)
        for (int j = 0; j < n1; ++j) is >> mats[k][i * n1 + j];
    }
    // only Bezier patches: knots 0..0 1..1
    for (double kv : k1)
      if (kv > kGenericTol && kv < 1 - kGenericTol)
        throw std::runtime_error("interior knots are not supported by the oracle");
    for (double kv : k2)
      if (kv > kGenericTol && kv < 1 - kGenericTol)
        throw std::runtime_error("interior knots are not supported by the oracle");
    Patch P;
    P.px = (int)k1.size() - n1;
    P.py = (int)k2.size() - n2;
    P.data.resize(4 * n1 * n2);
    // Unroll: index (x*ny + y) = matrix(y, x)
    for (int x = 0; x < n1; ++x)
      for (int y = 0; y < n2; ++y)
        for (int k = 0; k < 4; ++k) P.data[4 * (x * n2 + y) + k] = mats[k][y * n1 + x];
    out.push_back(P);
  }
  return out;
}

// ---------------------------------------------------------------------------
// Element tree (ClusterTree/ElementTree.hpp, ElementTreeNode.hpp) with the
// reference's refinement procedure and vertex numbering.
struct Node {
  int sons[4] = {-1, -1, -1, -1};
  int nsons = 0;
  int adj[4] = {-1, -1, -1, -1};
  int vert[4] = {-1, -1, -1, -1};
  V3 mid;
  double radius = INFINITY;
  double llc[2] = {0, 0};
  int id = -1, level = -1, patch = -1;
  double h() const { return 1.0 / double(1 << level); }
};

struct ElementTree {
  std::vector<Patch> geo;
  std::vector<Node> nodes;  // node 0 = root
  int max_level = 0, npoints = 0, nelements = 0, npatches = 0;
  std::vector<int> leaves;  // leaf node indices in tree order (== element id)
  std::vector<V3> points;   // generatePointList

  void update_topology(const std::vector<int>& els) {
    std::map<std::pair<int, int>, int> edges;
    for (int e : els)
      for (int j = 0; j < 4; ++j) {
        int v1 = nodes[e].vert[j], v2 = nodes[e].vert[(j + 1) % 4];
        std::pair<int, int> key(std::min(v1, v2), std::max(v1, v2));
        auto it = edges.find(key);
        if (it != edges.end()) {
          nodes[e].adj[j] = it->second;
          Node& o = nodes[it->second];
          for (int k = 0; k < 4; ++k) {
            int v3 = o.vert[k], v4 = o.vert[(k + 1) % 4];
            if (std::min(v3, v4) == key.first && std::max(v3, v4) == key.second) {
              o.adj[k] = e;
              break;
            }
          }
        } else {
          edges.insert(std::make_pair(key, e));
        }
      }
  }
  // ElementTree::refineLeaf (ElementTree.hpp:624-~720)
  void refine_leaf(int ci) {
    if (nodes[ci].nsons) return;
    int pt[5], refn[4];
    std::vector<int> els;
    for (int i = 0; i < 4; ++i) {
      refn[i] = -1;
      int a = nodes[ci].adj[i];
      if (a >= 0)
        for (int j = 0; j < 4; ++j)
          if (nodes[a].adj[j] == ci) {
            refn[i] = j;
            break;
          }
    }
    for (int i = 0; i < 4; ++i) {
      int a = nodes[ci].adj[i];
      if (a >= 0 && nodes[a].nsons) {
        int s = nodes[a].sons[refn[i]];
        pt[i] = nodes[s].vert[(refn[i] + 1) % 4];
        els.push_back(nodes[a].sons[refn[i]]);
        els.push_back(nodes[a].sons[(refn[i] + 1) % 4]);
      } else {
        pt[i] = npoints++;
      }
    }
    pt[4] = npoints++;
    static const double llcs[2][4] = {{0., .5, .5, 0.}, {0., 0., .5, .5}};
    int first = (int)nodes.size();
    for (int i = 0; i < 4; ++i) nodes.emplace_back();
    Node& c = nodes[ci];
    c.nsons = 4;
    nelements += 3;
    max_level = std::max(max_level, c.level + 1);
    for (int i = 0; i < 4; ++i) {
      Node& s = nodes[first + i];
      c.sons[i] = first + i;
      s.patch = c.patch;
      s.level = c.level + 1;
      s.id = 4 * c.id + i;
      s.llc[0] = c.llc[0] + llcs[0][i] / double(1 << c.level);
      s.llc[1] = c.llc[1] + llcs[1][i] / double(1 << c.level);
      els.push_back(first + i);
    }
    int* v = c.vert;
    int sv[4][4] = {{v[0], pt[0], pt[4], pt[3]},
                    {pt[0], v[1], pt[1], pt[4]},
                    {pt[4], pt[1], v[2], pt[2]},
                    {pt[3], pt[4], pt[2], v[3]}};
    for (int i = 0; i < 4; ++i)
      for (int k = 0; k < 4; ++k) nodes[first + i].vert[k] = sv[i][k];
    update_topology(els);
  }
  void refine_rec(int n) {
    if (nodes[n].nsons) {
      for (int i = 0; i < nodes[n].nsons; ++i) refine_rec(nodes[n].sons[i]);
    } else {
      refine_leaf(n);
    }
  }
  void collect_leaves(int n) {
    if (!nodes[n].nsons) {
      leaves.push_back(n);
      return;
    }
    for (int i = 0; i < nodes[n].nsons; ++i) collect_leaves(nodes[n].sons[i]);
  }
  // ElementTree::init_ElementTree (ElementTree.hpp:105-161)
  void init(const std::vector<Patch>& g, int M) {
    geo = g;
    npatches = (int)g.size();
    max_level = M;
    nodes.clear();
    nodes.reserve(1 + npatches * (size_t)(4 * (1 << (2 * M)) / 3 + 2));
    nodes.emplace_back();  // root
    std::vector<V3> uniq;
    npoints = 0;
    nelements = npatches;
    static const double corners[2][4] = {{0., 1., 1., 0}, {0., 0., 1., 1.}};
    std::vector<int> pats;
    for (int i = 0; i < npatches; ++i) {
      nodes.emplace_back();
      int ni = (int)nodes.size() - 1;
      Node& n = nodes[ni];
      n.id = i;
      n.level = 0;
      n.patch = i;
      for (int j = 0; j < 4; ++j) {
        V3 v = geo[i].eval(corners[0][j], corners[1][j]);
        size_t idx = 0;
        for (; idx < uniq.size(); ++idx)
          if ((uniq[idx] - v).norm() < kPtCompTol) break;
        if (idx != uniq.size()) {
          nodes[ni].vert[j] = (int)idx;
        } else {
          uniq.push_back(v);
          nodes[ni].vert[j] = npoints++;
        }
      }
      pats.push_back(ni);
    }
    nodes[0].nsons = npatches;  // root sons: patches (root has > 4 sons)
    root_sons = pats;
    update_topology(pats);
    for (int l = 0; l < M; ++l)
      for (int p : pats) refine_rec(p);
    leaves.clear();
    for (int p : pats) collect_leaves(p);
    compute_enclosings();
  }
  std::vector<int> root_sons;

  static void enclosing_ball(V3* m, double* r, const V3& m1, double r1,
                             const V3& m2, double r2) {
    V3 z = m1 - m2;
    double nrm = z.norm();
    if (nrm + r2 <= r1) {
      *m = m1;
      *r = r1;
    } else if (nrm + r1 <= r2) {
      *m = m2;
      *r = r2;
    } else {
      double s = (r1 - r2) / nrm;
      *m = V3(0.5 * (m1.x + m2.x + s * z.x), 0.5 * (m1.y + m2.y + s * z.y),
              0.5 * (m1.z + m2.z + s * z.z));
      *r = 0.5 * (r1 + r2 + nrm);
    }
  }
  void enclosing_rec(int n) {
    Node& e = nodes[n];
    V3 m1, m2;
    double r1, r2;
    if (!e.nsons) {
      enclosing_ball(&m1, &r1, points[e.vert[0]], 0, points[e.vert[2]], 0);
      enclosing_ball(&m2, &r2, points[e.vert[1]], 0, points[e.vert[3]], 0);
      enclosing_ball(&e.mid, &e.radius, m1, r1, m2, r2);
    } else {
      for (int i = 0; i < 4; ++i) enclosing_rec(e.sons[i]);
      const Node& s0 = nodes[e.sons[0]];
      const Node& s1 = nodes[e.sons[1]];
      const Node& s2 = nodes[e.sons[2]];
      const Node& s3 = nodes[e.sons[3]];
      enclosing_ball(&m1, &r1, s0.mid, s0.radius, s2.mid, s2.radius);
      enclosing_ball(&m2, &r2, s1.mid, s1.radius, s3.mid, s3.radius);
      Node& ee = nodes[n];
      enclosing_ball(&ee.mid, &ee.radius, m1, r1, m2, r2);
    }
  }
  // computeElementEnclosings (ElementTree.hpp:354-398) after generatePointList
  void compute_enclosings() {
    points.assign(npoints, V3());
    for (int li : leaves) {
      const Node& e = nodes[li];
      double h = 1.0 / double(1 << e.level);
      const Patch& P = geo[e.patch];
      points[e.vert[0]] = P.eval(e.llc[0], e.llc[1]);
      points[e.vert[1]] = P.eval(e.llc[0] + h, e.llc[1]);
      points[e.vert[2]] = P.eval(e.llc[0] + h, e.llc[1] + h);
      points[e.vert[3]] = P.eval(e.llc[0], e.llc[1] + h);
    }
    for (int p : root_sons) enclosing_rec(p);
  }
  // patchTopologyInfo (ElementTree.hpp:~490-520): [patch1, patch2, edge1, edge2]
  std::vector<std::array<int, 4>> patch_topology() const {
    std::vector<std::array<int, 4>> out;
    for (int p : root_sons) {
      const Node& n = nodes[p];
      for (int j = 0; j < 4; ++j) {
        if (n.adj[j] >= 0) {
          const Node& o = nodes[n.adj[j]];
          if (n.id < o.id) {
            int k = 0;
            for (; k < 4; ++k)
              if (o.adj[k] >= 0 && nodes[o.adj[k]].id == n.id) break;
            out.push_back({n.id, o.id, j, k});
          }
        } else {
          out.push_back({n.id, -1, j, -1});
        }
      }
    }
    return out;
  }
  // number of elements below a cluster and its first element id
  int cluster_size(int n) const {
    const Node& c = nodes[n];
    if (n == 0) return nelements;
    return 1 << (2 * (max_level - c.level));
  }
  int cluster_first(int n) const {
    const Node& c = nodes[n];
    if (n == 0) return 0;
    return c.id << (2 * (max_level - c.level));
  }
};

// ---------------------------------------------------------------------------
// Block cluster tree (H2Matrix/BlockClusterTree.hpp:154-182, 255-278).
enum { kRefine = 0, kLowRank = 1, kDense = 2 };
struct BlockLeaf {
  int c1, c2;  // node indices
  int cc;      // kLowRank or kDense
};
struct BlockClusterTree {
  double eta = 1.6;
  int mcl = 1;
  int max_level = 0;
  std::vector<BlockLeaf> leaves;  // in the reference's leaf-pointer order
  const ElementTree* et = nullptr;

  int compare(const Node& a, const Node& b) const {
    V3 d = a.mid - b.mid;
    double dist = d.norm() - a.radius - b.radius;
    dist = dist > 0 ? dist : 0;
    double maxr = a.radius > b.radius ? a.radius : b.radius;
    int r;
    if (dist < 0 || maxr >= eta * dist)
      r = kRefine;
    else
      r = kLowRank;
    if (r == kRefine && max_level - a.level <= mcl) r = kDense;
    return r;
  }
  void append(int c1, int c2) {
    const Node& a = et->nodes[c1];
    const Node& b = et->nodes[c2];
    int cc = compare(a, b);
    if (cc == kRefine) {
      std::vector<int> s1, s2;
      if (c1 == 0) s1 = et->root_sons; else s1.assign(a.sons, a.sons + a.nsons);
      if (c2 == 0) s2 = et->root_sons; else s2.assign(b.sons, b.sons + b.nsons);
      // updateLeafPointers_recursion visits sons(i, j) column by column
      for (size_t j = 0; j < s2.size(); ++j)
        for (size_t i = 0; i < s1.size(); ++i) append(s1[i], s2[j]);
    } else {
      leaves.push_back({c1, c2, cc});
    }
  }
  void init(const ElementTree& t, double eta_, int mcl_) {
    et = &t;
    eta = eta_;
    mcl = mcl_;
    max_level = t.max_level;
    leaves.clear();
    append(0, 0);
  }
};

}  // namespace orc
