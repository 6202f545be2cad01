// Host-side setup of the GB300 H2 single-layer operator (see bg_host.hpp).
#include "bg_host.hpp"

#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <fstream>
#include <map>
#include <mutex>
#include <numeric>
#include <sstream>

namespace bg {

// ---------------------------------------------------------------------------
// the next line as exactly n numbers; false when the line is missing or short
static bool read_numbers(std::istream& f, size_t n, std::vector<double>* out) {
  std::string line;
  if (!std::getline(f, line)) return false;
  std::istringstream is(line);
  out->assign(n, 0.0);
  for (double& v : *out)
    if (!(is >> v)) return false;
  return true;
}

// .dat geometry files (GeometryIO.hpp:25-122): 4 comment lines, a header line
// "2 3 npatch 0 0", then per patch: "PATCH k", degrees, control point counts,
// two knot vectors and the x, y, z, w matrices (rows = y, cols = x). Every row
// must be complete, coordinates finite and weights positive.
bool load_dat(const std::string& path, Geometry* g, std::string* err) {
  std::ifstream f(path);
  if (!f) {
    *err = "cannot open geometry file " + path;
    return false;
  }
  std::string line;
  for (int i = 0; i < 4; ++i) std::getline(f, line);
  std::getline(f, line);
  int hdr[5] = {0, 0, 0, 0, 0};
  {
    std::istringstream is(line);
    for (int& h : hdr) is >> h;
  }
  if (hdr[2] <= 0) {
    *err = "geometry file has no patches: " + path;
    return false;
  }
  g->patches.clear();
  for (int p = 0; p < hdr[2]; ++p) {
    std::vector<double> deg, ncp;
    std::getline(f, line);  // PATCH k
    if (!f || !read_numbers(f, 2, &deg) || !read_numbers(f, 2, &ncp) || deg[0] < 0 || deg[1] < 0 ||
        deg[0] > 15 || deg[1] > 15 || ncp[0] < 1 || ncp[1] < 1 || ncp[0] > 16 || ncp[1] > 16) {
      *err = "malformed patch header (degrees 0..15, control points 1..16 per direction) in " + path;
      return false;
    }
    const int nx = (int)ncp[0], ny = (int)ncp[1];
    std::vector<double> knots[2];
    for (int d = 0; d < 2; ++d) {
      if (!read_numbers(f, (size_t)deg[d] + (size_t)ncp[d] + 1, &knots[d])) {
        *err = "malformed knot vector in " + path;
        return false;
      }
      for (double k : knots[d])
        if (k > 1e-6 && k < 1 - 1e-6) {
          *err = "patches with interior knots are not supported: " + path;
          return false;
        }
    }
    std::vector<double> mat[4];
    for (int c = 0; c < 4; ++c) {
      bool ok = read_numbers(f, (size_t)nx * ny, &mat[c]);
      for (double v : mat[c]) ok = ok && std::isfinite(v) && (c < 3 || v > 0.0);
      if (!ok) {
        *err = "malformed control points (missing values, or a weight that is not positive) in " + path;
        return false;
      }
    }
    PatchData P;
    P.px = (int)knots[0].size() - nx;
    P.py = (int)knots[1].size() - ny;
    if (P.px != nx || P.py != ny) {
      *err = "only Bezier patches (no interior knots) are supported: " + path;
      return false;
    }
    P.cp.resize(4 * nx * ny);
    for (int ix = 0; ix < nx; ++ix)
      for (int iy = 0; iy < ny; ++iy)
        for (int c = 0; c < 4; ++c) P.cp[4 * (ix * ny + iy) + c] = mat[c][iy * nx + ix];
    g->patches.push_back(std::move(P));
  }
  return true;
}

bool load_igs(const std::string& path, Geometry* g, std::string* err) {
  std::ifstream f(path);
  if (!f) {
    *err = "cannot open geometry file " + path;
    return false;
  }
  std::vector<std::string> dir, par;
  std::string line;
  while (std::getline(f, line)) {
    if (!line.empty() && line.back() == '\r') line.pop_back();
    if (line.size() < 73) continue;
    if (line[72] == 'D') dir.push_back(line);
    if (line[72] == 'P') par.push_back(line);
  }
  if (dir.empty() || dir.size() % 2) {
    *err = "IGES file without a well-formed directory section: " + path;
    return false;
  }
  auto field = [](const std::string& l, int k) {  // k-th 8-column field of a directory line
    return std::atoi(l.substr(8 * k, 8).c_str());
  };
  g->patches.clear();
  for (size_t e = 0; e < dir.size(); e += 2) {
    const int type = field(dir[e], 0), first = field(dir[e], 1), count = field(dir[e + 1], 3);
    if (type != 128) {
      *err = "IGES entity " + std::to_string(type) + " is not a rational B-spline surface (128): " + path;
      return false;
    }
    if (first < 1 || count < 1 || first - 1 + count > (int)par.size()) {
      *err = "IGES parameter pointer out of range: " + path;
      return false;
    }
    // parameter data: columns 1-64 of the entity's lines, ',' between values, ';' at the end
    std::string data;
    for (int k = first - 1; k < first - 1 + count; ++k) data += par[k].substr(0, 64);
    std::vector<double> v;
    std::string tok;
    for (char c : data + ",") {
      if (c == ',' || c == ';') {
        if (!tok.empty()) {
          for (char& t : tok)
            if (t == 'D' || t == 'd') t = 'E';  // Fortran exponents
          v.push_back(std::strtod(tok.c_str(), nullptr));
        }
        tok.clear();
        if (c == ';') break;
      } else if (c != ' ') {
        tok += c;
      }
    }
    // upper indices and degrees in 0..15 (as for the .dat files), checked before any arithmetic on them
    bool in_range = v.size() >= 10 && v[0] == 128.0;
    for (int i = 1; i <= 4 && in_range; ++i) in_range = v[i] >= 0.0 && v[i] <= 15.0;
    if (!in_range) {
      *err = "malformed IGES entity 128 parameters: " + path;
      return false;
    }
    const int K1 = (int)v[1], K2 = (int)v[2], M1 = (int)v[3], M2 = (int)v[4];
    const int A = K1 + M1 + 1, B = K2 + M2 + 1, C = (K1 + 1) * (K2 + 1);  // knot counts - 1, points
    if (v.size() < (size_t)(10 + A + 1 + B + 1 + 4 * C)) {
      *err = "malformed IGES entity 128 parameters: " + path;
      return false;
    }
    if (K1 != M1 || K2 != M2) {
      *err = "patches with interior knots are not supported: " + path;
      return false;
    }
    const double* W = v.data() + 10 + A + 1 + B + 1;
    const double* X = W + C;
    for (int q = 0; q < C; ++q)
      if (!(W[q] > 0.0) || !std::isfinite(W[q]) || !std::isfinite(X[3 * q]) || !std::isfinite(X[3 * q + 1]) ||
          !std::isfinite(X[3 * q + 2])) {
        *err = "IGES control point with a weight that is not positive, or not finite: " + path;
        return false;
      }
    PatchData P;
    P.px = K1 + 1;
    P.py = K2 + 1;
    P.cp.resize(4 * C);
    for (int j = 0; j <= K2; ++j)
      for (int i = 0; i <= K1; ++i) {
        const int q = j * (K1 + 1) + i;  // IGES order: first index fastest
        const double w = W[q];
        double* c = &P.cp[4 * (i * P.py + j)];
        c[0] = X[3 * q] * w;  // homogeneous coordinates, as in the .dat files
        c[1] = X[3 * q + 1] * w;
        c[2] = X[3 * q + 2] * w;
        c[3] = w;
      }
    g->patches.push_back(std::move(P));
  }
  return true;
}

// ---------------------------------------------------------------------------
void bernstein(int p, double x, double* b) {
  // de Casteljau-style build-up: b^{k}_i = (1-x) b^{k-1}_i + x b^{k-1}_{i-1}
  b[0] = 1.0;
  for (int k = 1; k <= p; ++k) {
    double prev = 0.0;
    for (int i = 0; i < k; ++i) {
      double t = b[i];
      b[i] = prev + (1.0 - x) * t;
      prev = x * t;
    }
    b[k] = prev;
  }
}
void bernstein_der(int p, double x, double* b) {
  if (p == 0) {
    b[0] = 0.0;
    return;
  }
  double low[64];
  bernstein(p - 1, x, low);
  for (int i = 0; i <= p; ++i) {
    double a = i > 0 ? low[i - 1] : 0.0;
    double c = i < p ? low[i] : 0.0;
    b[i] = p * (a - c);
  }
}

static void patch_accumulate(const PatchData& P, double s, double t, double* h, double* hs, double* ht) {
  double bx[32], by[32], dbx[32], dby[32];
  bernstein(P.px - 1, s, bx);
  bernstein(P.py - 1, t, by);
  bernstein_der(P.px - 1, s, dbx);
  bernstein_der(P.py - 1, t, dby);
  for (int k = 0; k < 4; ++k) h[k] = hs[k] = ht[k] = 0.0;
  for (int i = 0; i < P.px; ++i)
    for (int j = 0; j < P.py; ++j) {
      const double* c = &P.cp[4 * (i * P.py + j)];
      double v = bx[i] * by[j], vs = dbx[i] * by[j], vt = bx[i] * dby[j];
      for (int k = 0; k < 4; ++k) {
        h[k] += c[k] * v;
        hs[k] += c[k] * vs;
        ht[k] += c[k] * vt;
      }
    }
}
void cube_face_frame(int face, double s, double t, double* out) {
  const int k = face / 2;
  const bool pos = face % 2 == 0;
  const int a = pos ? (k + 1) % 3 : (k + 2) % 3, b = pos ? (k + 2) % 3 : (k + 1) % 3;
  double c[3];
  c[k] = pos ? 1.0 : -1.0;
  c[a] = 2.0 * s - 1.0;
  c[b] = 2.0 * t - 1.0;
  const double ir = 1.0 / std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
  for (int j = 0; j < 3; ++j) out[j] = c[j] * ir;
  for (int j = 0; j < 3; ++j) {
    out[3 + j] = 2.0 * ((j == a ? 1.0 : 0.0) - out[j] * out[a]) * ir;
    out[6 + j] = 2.0 * ((j == b ? 1.0 : 0.0) - out[j] * out[b]) * ir;
  }
}
void cube_sphere(Geometry* g) {
  g->patches.assign(6, PatchData());
  for (int f = 0; f < 6; ++f) g->patches[f].face = f;
}
void patch_point(const PatchData& P, double s, double t, double* x3) {
  if (P.face >= 0) {
    double f[9];
    cube_face_frame(P.face, s, t, f);
    for (int k = 0; k < 3; ++k) x3[k] = f[k];
    return;
  }
  double h[4], hs[4], ht[4];
  patch_accumulate(P, s, t, h, hs, ht);
  for (int k = 0; k < 3; ++k) x3[k] = h[k] / h[3];
}
void patch_frame(const PatchData& P, double s, double t, double* out) {
  if (P.face >= 0) {
    cube_face_frame(P.face, s, t, out);
    return;
  }
  double h[4], hs[4], ht[4];
  patch_accumulate(P, s, t, h, hs, ht);
  double iw = 1.0 / h[3], iw2 = iw * iw;
  for (int k = 0; k < 3; ++k) {
    out[k] = h[k] * iw;
    out[3 + k] = (hs[k] * h[3] - h[k] * hs[3]) * iw2;
    out[6 + k] = (ht[k] * h[3] - h[k] * ht[3]) * iw2;
  }
}

// ---------------------------------------------------------------------------
// Gauss-Legendre nodes by Newton's method on the three-term Legendre
// recurrence, weights 2/((1-x^2) P_n'(x)^2), mapped to [0,1].
static Rule1D make_gauss(int n) {
  Rule1D r;
  r.x.assign(n, 0.0);
  r.w.assign(n, 0.0);
  if (n == 1) {
    r.x[0] = 0.5;
    r.w[0] = 1.0;
    return r;
  }
  for (int k = 0; k < (n + 1) / 2; ++k) {
    double z = std::cos(kPi * (k + 0.75) / (n + 0.5));
    double dp = 1.0;
    for (int it = 0; it < 64; ++it) {
      double p0 = 1.0, p1 = z;
      for (int m = 2; m <= n; ++m) {
        double p2 = ((2.0 * m - 1.0) * z * p1 - (m - 1.0) * p0) / m;
        p0 = p1;
        p1 = p2;
      }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      double dz = p1 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-17) break;
    }
    double p0 = 1.0, p1 = z;
    for (int m = 2; m <= n; ++m) {
      double p2 = ((2.0 * m - 1.0) * z * p1 - (m - 1.0) * p0) / m;
      p0 = p1;
      p1 = p2;
    }
    dp = n * (z * p1 - p0) / (z * z - 1.0);
    double w = 2.0 / ((1.0 - z * z) * dp * dp);
    // z > 0 is the (k+1)-th largest root; symmetric partner -z
    r.x[n - 1 - k] = 0.5 * (1.0 + z);
    r.w[n - 1 - k] = 0.5 * w;
    r.x[k] = 0.5 * (1.0 - z);
    r.w[k] = 0.5 * w;
  }
  if (n % 2 == 1) r.x[n / 2] = 0.5;
  return r;
}
const Rule1D& gauss_rule(int npoints) {
  static std::mutex mu;
  static std::map<int, Rule1D> cache;
  std::lock_guard<std::mutex> lock(mu);
  auto it = cache.find(npoints);
  if (it == cache.end()) it = cache.emplace(npoints, make_gauss(npoints)).first;
  return it->second;
}

// ---------------------------------------------------------------------------
int quadtree_index(int ix, int iy, int level) {
  int id = 0;
  for (int b = level - 1; b >= 0; --b) {
    int bx = (ix >> b) & 1, by = (iy >> b) & 1;
    int d = by ? (bx ? 2 : 3) : (bx ? 1 : 0);
    id = 4 * id + d;
  }
  return id;
}
void quadtree_coords(int local, int level, int* ix, int* iy) {
  int x = 0, y = 0;
  for (int b = level - 1; b >= 0; --b) {
    int d = (local >> (2 * b)) & 3;
    int bx = (d == 1 || d == 2), by = (d == 2 || d == 3);
    x = 2 * x + bx;
    y = 2 * y + by;
  }
  *ix = x;
  *iy = y;
}

struct UnionFind {
  std::vector<int> p;
  explicit UnionFind(int n) : p(n) { std::iota(p.begin(), p.end(), 0); }
  int find(int a) {
    while (p[a] != a) a = p[a] = p[p[a]];
    return a;
  }
  void unite(int a, int b) {
    a = find(a);
    b = find(b);
    if (a != b) p[std::max(a, b)] = std::min(a, b);
  }
};

static void ball_of(const double* m1, double r1, const double* m2, double r2, double* out) {
  // smallest ball around two balls (util/GeometryHelper.hpp:32-55)
  double z[3] = {m1[0] - m2[0], m1[1] - m2[1], m1[2] - m2[2]};
  double n = std::sqrt(z[0] * z[0] + z[1] * z[1] + z[2] * z[2]);
  if (n + r2 <= r1) {
    out[0] = m1[0]; out[1] = m1[1]; out[2] = m1[2]; out[3] = r1;
  } else if (n + r1 <= r2) {
    out[0] = m2[0]; out[1] = m2[1]; out[2] = m2[2]; out[3] = r2;
  } else {
    double s = (r1 - r2) / n;
    for (int k = 0; k < 3; ++k) out[k] = 0.5 * (m1[k] + m2[k] + s * z[k]);
    out[3] = 0.5 * (r1 + r2 + n);
  }
}

bool build_mesh(const Geometry& g, int M, Mesh* m, std::string* err) {
  if (M < 0 || M > 12) {
    *err = "refinement level out of range";
    return false;
  }
  const int np = (int)g.patches.size();
  const int n = 1 << M, per = (n + 1) * (n + 1);
  m->M = M;
  m->npatch = np;
  m->n1d = n;
  m->ne = np * n * n;
  // corner identification by position (tolerance 1e-9, ElementTree.hpp:130-145)
  static const int cxy[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
  std::vector<std::array<double, 3>> uniq;
  std::vector<int> corner(4 * np);
  for (int p = 0; p < np; ++p)
    for (int c = 0; c < 4; ++c) {
      double x[3];
      patch_point(g.patches[p], cxy[c][0], cxy[c][1], x);
      size_t u = 0;
      for (; u < uniq.size(); ++u) {
        double d = std::sqrt((uniq[u][0] - x[0]) * (uniq[u][0] - x[0]) + (uniq[u][1] - x[1]) * (uniq[u][1] - x[1]) +
                             (uniq[u][2] - x[2]) * (uniq[u][2] - x[2]));
        if (d < 1e-9) break;
      }
      if (u == uniq.size()) uniq.push_back({x[0], x[1], x[2]});
      corner[4 * p + c] = (int)u;
    }
  // patch edges: edge j runs from corner j to corner j+1; shared edges are
  // those with the same unordered pair of corner ids
  auto edge_point = [&](int p, int j, int t) {
    int i = 0, k = 0;
    switch (j) {
      case 0: i = t; k = 0; break;
      case 1: i = n; k = t; break;
      case 2: i = n - t; k = n; break;
      default: i = 0; k = n - t; break;
    }
    return p * per + k * (n + 1) + i;
  };
  UnionFind uf(np * per);
  for (int p = 0; p < np; ++p)
    for (int c = 0; c < 4; ++c)
      for (int q = 0; q < np; ++q)
        for (int d = 0; d < 4; ++d)
          if (corner[4 * p + c] == corner[4 * q + d])
            uf.unite(p * per + cxy[c][1] * n * (n + 1) + cxy[c][0] * n,
                     q * per + cxy[d][1] * n * (n + 1) + cxy[d][0] * n);
  std::map<std::pair<int, int>, std::pair<int, int>> first_edge;
  std::vector<std::array<int, 2>> adj(4 * np, {-1, -1});
  for (int p = 0; p < np; ++p)
    for (int j = 0; j < 4; ++j) {
      int a = corner[4 * p + j], b = corner[4 * p + (j + 1) % 4];
      std::pair<int, int> key(std::min(a, b), std::max(a, b));
      auto it = first_edge.find(key);
      if (it == first_edge.end()) {
        first_edge[key] = {p, j};
        continue;
      }
      int q = it->second.first, k = it->second.second;
      adj[4 * p + j] = {q, k};
      adj[4 * q + k] = {p, j};
      bool same_dir = corner[4 * p + j] == corner[4 * q + k];
      for (int t = 0; t <= n; ++t) uf.unite(edge_point(p, j, t), edge_point(q, k, same_dir ? t : n - t));
    }
  m->patch_edges.clear();
  for (int p = 0; p < np; ++p)
    for (int j = 0; j < 4; ++j) {
      int q = adj[4 * p + j][0];
      if (q >= 0) {
        if (p < q) m->patch_edges.push_back({p, q, j, adj[4 * p + j][1]});
      } else {
        m->patch_edges.push_back({p, -1, j, -1});
      }
    }
  std::vector<int> vid(np * per, -1);
  int nv = 0;
  for (int i = 0; i < np * per; ++i) {
    int r = uf.find(i);
    if (vid[r] < 0) vid[r] = nv++;
    vid[i] = vid[r];
  }
  m->nverts = nv;
  // element table in id order
  const double h = 1.0 / double(n);
  m->patch.resize(m->ne);
  m->ix.resize(m->ne);
  m->iy.resize(m->ne);
  m->llc.resize(2 * m->ne);
  m->vert.resize(4 * m->ne);
  for (int e = 0; e < m->ne; ++e) {
    int p = e / (n * n), x, y;
    quadtree_coords(e % (n * n), M, &x, &y);
    m->patch[e] = p;
    m->ix[e] = x;
    m->iy[e] = y;
    m->llc[2 * e] = x * h;
    m->llc[2 * e + 1] = y * h;
    m->vert[4 * e + 0] = vid[p * per + y * (n + 1) + x];
    m->vert[4 * e + 1] = vid[p * per + y * (n + 1) + x + 1];
    m->vert[4 * e + 2] = vid[p * per + (y + 1) * (n + 1) + x + 1];
    m->vert[4 * e + 3] = vid[p * per + (y + 1) * (n + 1) + x];
  }
  // vertex coordinates: later elements overwrite earlier ones
  // (ElementTree::generatePointList, ElementTree.hpp:~205-225)
  std::vector<double> pts(3 * nv, 0.0);
  for (int e = 0; e < m->ne; ++e) {
    const PatchData& P = g.patches[m->patch[e]];
    double s = m->llc[2 * e], t = m->llc[2 * e + 1];
    patch_point(P, s, t, &pts[3 * m->vert[4 * e + 0]]);
    patch_point(P, s + h, t, &pts[3 * m->vert[4 * e + 1]]);
    patch_point(P, s + h, t + h, &pts[3 * m->vert[4 * e + 2]]);
    patch_point(P, s, t + h, &pts[3 * m->vert[4 * e + 3]]);
  }
  // enclosing balls bottom-up (ElementTree.hpp:354-398)
  m->ball.assign(M + 1, {});
  m->ball[M].resize(4 * m->ne);
  for (int e = 0; e < m->ne; ++e) {
    double b1[4], b2[4];
    const int* v = &m->vert[4 * e];
    ball_of(&pts[3 * v[0]], 0, &pts[3 * v[2]], 0, b1);
    ball_of(&pts[3 * v[1]], 0, &pts[3 * v[3]], 0, b2);
    ball_of(b1, b1[3], b2, b2[3], &m->ball[M][4 * e]);
  }
  for (int l = M - 1; l >= 0; --l) {
    int nc = np << (2 * l);
    m->ball[l].resize(4 * nc);
    const std::vector<double>& s = m->ball[l + 1];
    for (int c = 0; c < nc; ++c) {
      const double* s0 = &s[4 * (4 * c + 0)];
      const double* s1 = &s[4 * (4 * c + 1)];
      const double* s2 = &s[4 * (4 * c + 2)];
      const double* s3 = &s[4 * (4 * c + 3)];
      double b1[4], b2[4];
      ball_of(s0, s0[3], s2, s2[3], b1);
      ball_of(s1, s1[3], s3, s3[3], b2);
      ball_of(b1, b1[3], b2, b2[3], &m->ball[l][4 * c]);
    }
  }
  return true;
}

// ---------------------------------------------------------------------------
namespace {
struct PartitionBuilder {
  const Mesh& m;
  double eta;
  int mcl;
  Partition* out;
  // admissibility of two clusters of the same level (BlockClusterTree.hpp:255-278)
  int compare(int level, int c1, int c2) const {
    const double* a = &m.ball[level][4 * c1];
    const double* b = &m.ball[level][4 * c2];
    double d[3] = {a[0] - b[0], a[1] - b[1], a[2] - b[2]};
    double dist = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) - a[3] - b[3];
    dist = dist > 0 ? dist : 0;
    double maxr = a[3] > b[3] ? a[3] : b[3];
    int r = (dist < 0 || maxr >= eta * dist) ? 0 : 1;
    if (r == 0 && m.M - level <= mcl) r = 2;
    return r;
  }
  void add(int cc, int level, int c1, int c2) {
    out->leaf_list.insert(out->leaf_list.end(), {cc, level, c1, c2});
    if (cc == 2) {
      out->dense_c1.push_back(c1);
      out->dense_c2.push_back(c2);
    } else {
      out->far_c1[level].push_back(c1);
      out->far_c2[level].push_back(c2);
    }
  }
  void recurse(int level, int c1, int c2) {
    int cc = compare(level, c1, c2);
    if (cc != 0) {
      add(cc, level, c1, c2);
      return;
    }
    for (int j = 0; j < 4; ++j)
      for (int i = 0; i < 4; ++i) recurse(level + 1, 4 * c1 + i, 4 * c2 + j);
  }
};
}  // namespace

void build_partition(const Mesh& m, double eta, int mcl, Partition* part) {
  *part = Partition();
  part->far_levels = std::max(m.M - mcl + 1, 0);
  part->far_c1.assign(std::max(part->far_levels, 1), {});
  part->far_c2.assign(std::max(part->far_levels, 1), {});
  PartitionBuilder b{m, eta, mcl, part};
  if (m.M + 1 <= mcl) {
    // the root block itself is dense: one cluster holding every element
    part->dense_level = -1;
    part->leaf_list = {2, -1, -1, -1};  // the root cluster has id -1
    part->dense_c1.push_back(0);
    part->dense_c2.push_back(0);
    return;
  }
  part->dense_level = m.M - mcl;
  for (int j = 0; j < m.npatch; ++j)
    for (int i = 0; i < m.npatch; ++i) b.recurse(0, i, j);
}

// ---------------------------------------------------------------------------
PairClass classify_pair(const Mesh& m, int e1, int e2, int P) {
  PairClass pc{0, 4, 4, 0};
  const int M = m.M;
  double dist = 0.0;
  if (e1 == e2) {
    pc.cs = 2;
  } else {
    const double* a = &m.ball[M][4 * e1];
    const double* b = &m.ball[M][4 * e2];
    double d[3] = {a[0] - b[0], a[1] - b[1], a[2] - b[2]};
    dist = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) - a[3] - b[3];
    dist = dist >= 0 ? dist : 0;
    pc.cs = 0;
    if (!(dist > .5 / (1 << M))) {
      const int* v1 = &m.vert[4 * e1];
      const int* v2 = &m.vert[4 * e2];
      bool found = false;
      for (int r1 = 0; r1 < 4 && !found; ++r1)
        for (int r2 = 0; r2 < 4 && !found; ++r2)
          if (v1[r1] == v2[r2]) {
            found = true;
            if (v1[3] == v2[(r2 + 1) % 4]) pc = {3, 3, r2, 0};
            else if (v1[(r1 + 1) % 4] == v2[(r2 + 3) % 4]) pc = {3, r1, (r2 + 3) % 4, 0};
            else pc = {4, r1, r2, 0};
          }
    }
  }
  // quadrature degree, operator order -1 (LinearOperatorBase.hpp:56-89)
  const int order = -1, level = M;
  double distance_log = (dist * (1 << level) < 1) ? -(level * std::log(2.)) : std::log(dist);
  int alpha = 2 - order + 2 * P;
  double numerator = (alpha + P) * level * std::log(2.) - (2 - P + order) * distance_log;
  double denominator = (level + 2) * std::log(2.) + distance_log;
  int nf = (int)(0.5 * numerator / denominator);
  int ff = P - order + 1;
  pc.deg = nf >= ff ? nf : ff;
  return pc;
}

// ---------------------------------------------------------------------------
// B-spline N_{i,o} (order o) by the Cox-de Boor recursion.
static double bspline(const std::vector<double>& knots, int i, int o, double x) {
  double N[64];
  for (int k = 0; k < o; ++k) {
    double a = knots[i + k], b = knots[i + k + 1];
    bool last = (b == knots.back()) && (x == b) && (a < b);
    N[k] = ((a <= x && x < b) || last) ? 1.0 : 0.0;
  }
  for (int d = 1; d < o; ++d)
    for (int k = 0; k < o - d; ++k) {
      double l = 0.0, r = 0.0;
      double den1 = knots[i + k + d] - knots[i + k];
      double den2 = knots[i + k + d + 1] - knots[i + k + 1];
      if (den1 > 0) l = (x - knots[i + k]) / den1 * N[k];
      if (den2 > 0) r = (knots[i + k + d + 1] - x) / den2 * N[k + 1];
      N[k] = l + r;
    }
  return N[0];
}

// 1D extraction: coefficients of the order-o B-splines supported on element
// e (of n uniform elements) in the degree-D Bernstein basis of the element,
// obtained by interpolation at the points (k+1)/(D+2) as in
// Projector.hpp:200-300 (which solves the tensor version of this system).
// out[(b) * (D+1) + a]: B-spline e+b, Bernstein a.
static void extraction_1d(int o, int n, int D, int e, std::vector<double>* out, int* first_dof) {
  std::vector<double> knots;
  for (int i = 0; i < o; ++i) knots.push_back(0.0);
  for (int i = 1; i < n; ++i) knots.push_back(double(i) / n);
  for (int i = 0; i < o; ++i) knots.push_back(1.0);
  const int m = D + 1;
  std::vector<double> pts(m), V(m * m);
  double hgrid = 1.0 / (D + 2);
  for (int k = 0; k < m; ++k) pts[k] = (k + 1) * hgrid;
  double b[64];
  for (int k = 0; k < m; ++k) {
    bernstein(D, pts[k], b);
    for (int a = 0; a < m; ++a) V[k * m + a] = b[a];
  }
  // Gaussian elimination with partial pivoting on V (m x m), m right-hand sides
  int ndof = (int)knots.size() - o;
  double mid = (e + 0.5) / n;
  std::vector<int> dofs;
  for (int d = 0; d < ndof; ++d)
    if (knots[d] <= mid && knots[d + o] >= mid) dofs.push_back(d);
  *first_dof = dofs.empty() ? 0 : dofs[0];
  out->assign(dofs.size() * m, 0.0);
  for (size_t q = 0; q < dofs.size(); ++q) {
    std::vector<double> A = V, r(m);
    for (int k = 0; k < m; ++k) r[k] = bspline(knots, dofs[q], o, double(e) / n + pts[k] / n);
    for (int c = 0; c < m; ++c) {
      int piv = c;
      for (int k = c + 1; k < m; ++k)
        if (std::fabs(A[k * m + c]) > std::fabs(A[piv * m + c])) piv = k;
      if (piv != c) {
        for (int a = 0; a < m; ++a) std::swap(A[c * m + a], A[piv * m + a]);
        std::swap(r[c], r[piv]);
      }
      for (int k = c + 1; k < m; ++k) {
        double f = A[k * m + c] / A[c * m + c];
        for (int a = c; a < m; ++a) A[k * m + a] -= f * A[c * m + a];
        r[k] -= f * r[c];
      }
    }
    for (int c = m - 1; c >= 0; --c) {
      double s = r[c];
      for (int a = c + 1; a < m; ++a) s -= A[c * m + a] * (*out)[q * m + a];
      (*out)[q * m + c] = s / A[c * m + c];
    }
  }
}

struct Trip {
  int r, c;
  double v;
};
static Csr csr_from(int rows, int cols, std::vector<Trip> t) {
  std::sort(t.begin(), t.end(), [](const Trip& a, const Trip& b) { return a.r != b.r ? a.r < b.r : a.c < b.c; });
  Csr A;
  A.rows = rows;
  A.cols = cols;
  A.ptr.assign(rows + 1, 0);
  for (size_t k = 0; k < t.size(); ++k) {
    if (k > 0 && t[k].r == t[k - 1].r && t[k].c == t[k - 1].c) {
      A.val.back() += t[k].v;
      continue;
    }
    A.idx.push_back(t[k].c);
    A.val.push_back(t[k].v);
    A.ptr[t[k].r + 1]++;
  }
  for (int r = 0; r < rows; ++r) A.ptr[r + 1] += A.ptr[r];
  return A;
}
Csr transpose(const Csr& A) {
  std::vector<Trip> t;
  for (int r = 0; r < A.rows; ++r)
    for (int k = A.ptr[r]; k < A.ptr[r + 1]; ++k) t.push_back({A.idx[k], r, A.val[k]});
  return csr_from(A.cols, A.rows, t);
}

// patchwise projection for one vector component with orders (ox, oy) into the
// degree-P Bernstein superspace; rows offset by row0, columns by col0.
static int add_projection(const Mesh& m, int P, int ox, int oy, int row0, int col0, std::vector<Trip>* t) {
  const int n = m.n1d, D = P, pp = P + 1;
  const int dimx = n + ox - 1, dimy = n + oy - 1, dim = dimx * dimy;
  std::vector<std::vector<double>> ex(n), ey(n);
  std::vector<int> fx(n), fy(n);
  for (int e = 0; e < n; ++e) {
    extraction_1d(ox, n, D, e, &ex[e], &fx[e]);
    extraction_1d(oy, n, D, e, &ey[e], &fy[e]);
  }
  for (int e = 0; e < m.ne; ++e) {
    int x = m.ix[e], y = m.iy[e], p = m.patch[e];
    int nbx = (int)ex[x].size() / pp, nby = (int)ey[y].size() / pp;
    for (int by = 0; by < nby; ++by)
      for (int bx = 0; bx < nbx; ++bx)
        for (int ay = 0; ay < pp; ++ay)
          for (int ax = 0; ax < pp; ++ax) {
            double v = ex[x][bx * pp + ax] * ey[y][by * pp + ay];
            if (std::fabs(v) > 1e-4)  // Constants::projector_tolerance
              t->push_back({row0 + e * pp * pp + ay * pp + ax, col0 + p * dim + dimx * (fy[y] + by) + fx[x] + bx, v});
          }
  }
  return dim * m.npatch;
}

// Glue of div-conforming spaces (Glue.hpp): the normal component is
// continuous across patch interfaces. Dofs of a patch component are numbered
// x-fastest; edge k of a patch selects the dofs on that side.
static Csr glue_divconforming(const Mesh& m, int P, int pre) {
  const int n = m.n1d;
  const int small_dim = P + (n - 1), large_dim = P + 1 + (n - 1), per = small_dim * large_dim;
  auto first_comp = [](int e) { return e == 1 || e == 3; };
  auto edge_dofs = [](int e, int dx, int dy, int shift) {
    std::vector<int> d;
    if (e == 0) for (int i = 0; i < dx; ++i) d.push_back(shift + i);
    if (e == 1) for (int i = 0; i < dy; ++i) d.push_back(shift + dx * (i + 1) - 1);
    if (e == 2) for (int i = 0; i < dx; ++i) d.push_back(shift + dx * (dy - 1) + i);
    if (e == 3) for (int i = 0; i < dy; ++i) d.push_back(shift + dx * i);
    return d;
  };
  // partner[d] = (master, sign) for slaves; boundary dofs are dropped
  std::vector<int> partner(pre, -1), sign(pre, 1);
  std::vector<char> drop(pre, 0), is_master(pre, 0);
  for (const auto& ed : m.patch_edges) {
    int p = ed[0], q = ed[1], j = ed[2], k = ed[3];
    int s1 = p * per + (first_comp(j) ? 0 : per * m.npatch);
    std::vector<int> d1 = edge_dofs(j, first_comp(j) ? large_dim : small_dim, first_comp(j) ? small_dim : large_dim, s1);
    if (q < 0) {
      for (int d : d1) drop[d] = 1;
      continue;
    }
    int s2 = q * per + (first_comp(k) ? 0 : per * m.npatch);
    std::vector<int> d2 = edge_dofs(k, first_comp(k) ? large_dim : small_dim, first_comp(k) ? small_dim : large_dim, s2);
    bool fj = (j == 0 || j == 1), fk = (k == 0 || k == 1);
    bool rev = (fj == fk);
    bool ij = (j == 0 || j == 3), ik = (k == 0 || k == 3);
    int coef = (ij == ik) ? -1 : 1;
    int sz = (int)d1.size();
    for (int i = 0; i < sz; ++i) {
      int a = d1[i], b = d2[rev ? sz - 1 - i : i];
      int lo = std::min(a, b), hi = std::max(a, b);
      is_master[lo] = 1;
      partner[hi] = lo;
      sign[hi] = coef;
    }
  }
  std::vector<int> col(pre, -1);
  int post = 0;
  for (int d = 0; d < pre; ++d)
    if (partner[d] < 0 && !drop[d]) col[d] = post++;
  std::vector<Trip> t;
  for (int d = 0; d < pre; ++d) {
    if (col[d] >= 0) t.push_back({d, col[d], 1.0});
    else if (partner[d] >= 0 && col[partner[d]] >= 0) t.push_back({d, col[partner[d]], (double)sign[d]});
  }
  return csr_from(pre, post, t);
}

static Csr multiply(const Csr& A, const Csr& B) {
  std::vector<Trip> t;
  for (int r = 0; r < A.rows; ++r)
    for (int k = A.ptr[r]; k < A.ptr[r + 1]; ++k) {
      int mid = A.idx[k];
      for (int l = B.ptr[mid]; l < B.ptr[mid + 1]; ++l) t.push_back({r, B.idx[l], A.val[k] * B.val[l]});
    }
  return csr_from(A.rows, B.cols, t);
}

bool build_transform(const Mesh& m, int P, bool div_conforming, Csr* T, std::string* err) {
  const int pp = P + 1, ss = m.ne * pp * pp;
  std::vector<Trip> t;
  if (!div_conforming) {
    int nc = add_projection(m, P, P + 1, P + 1, 0, 0, &t);
    *T = csr_from(ss, nc, t);
    return true;
  }
  if (P < 1) {
    *err = "div-conforming spaces need P >= 1";
    return false;
  }
  int c0 = add_projection(m, P, P + 1, P, 0, 0, &t);
  int c1 = add_projection(m, P, P, P + 1, ss, c0, &t);
  Csr proj = csr_from(2 * ss, c0 + c1, t);
  *T = multiply(proj, glue_divconforming(m, P, c0 + c1));
  return true;
}

// ---------------------------------------------------------------------------
std::vector<double> cheb_points(int np) {
  std::vector<double> x(np);
  double alpha = kPi / (2. * double(np));
  for (int i = 0; i < np; ++i) x[i] = 0.5 * std::cos(alpha * (2.0 * double(np - i) - 1.0)) + 0.5;
  return x;
}
// Lagrange basis in Newton form on the Chebyshev points: coef[k * np + j] is the
// k-th divided-difference coefficient of L_j (H2Multipole.hpp:39-67)
static std::vector<double> newton_coefficients(int np, const std::vector<double>& x) {
  std::vector<double> c(np * np, 0.0);
  for (int j = 0; j < np; ++j) {
    c[j * np + j] = 1.0;
    for (int d = 1; d < np; ++d)
      for (int k = np - 1; k >= d; --k) c[k * np + j] = (c[k * np + j] - c[(k - 1) * np + j]) / (x[k] - x[k - d]);
  }
  return c;
}
static double lagrange_value(const std::vector<double>& c, const std::vector<double>& x, int np, int j, double t) {
  double v = c[(np - 1) * np + j];
  for (int k = np - 2; k >= 0; --k) v = v * (t - x[k]) + c[k * np + j];
  return v;
}
std::vector<double> transfer_factors(int np) {
  std::vector<double> x = cheb_points(np), c = newton_coefficients(np, x);
  // E0[i][j] = L_j(x_i / 2), E1[i][j] = L_j(x_i / 2 + 1/2), stored [E0 | E1]
  std::vector<double> E(2 * (size_t)np * np);
  for (int i = 0; i < np; ++i)
    for (int j = 0; j < np; ++j) {
      E[i * np + j] = lagrange_value(c, x, np, j, 0.5 * x[i]);
      E[(size_t)np * np + i * np + j] = lagrange_value(c, x, np, j, 0.5 * x[i] + 0.5);
    }
  return E;
}
std::vector<double> transfer_matrix(int np) {
  const int n2 = np * np;
  const std::vector<double> E = transfer_factors(np);
  const double* E0 = E.data();
  const double* E1 = E.data() + n2;
  // child k (son order) sits in the s-half sx and t-half sy
  static const int sx[4] = {0, 1, 1, 0}, sy[4] = {0, 0, 1, 1};
  std::vector<double> T((size_t)n2 * 4 * n2);
  for (int k = 0; k < 4; ++k) {
    const double* Es = sx[k] ? E1 : E0;
    const double* Et = sy[k] ? E1 : E0;
    for (int ps = 0; ps < np; ++ps)
      for (int pt = 0; pt < np; ++pt)
        for (int cs = 0; cs < np; ++cs)
          for (int ct = 0; ct < np; ++ct)
            T[(size_t)(ps * np + pt) * 4 * n2 + k * n2 + cs * np + ct] = Es[cs * np + ps] * Et[ct * np + pt];
  }
  return T;
}
// 1D moments: mom[i][j*(P+1) + m] = sum_k w_k s L_i(h (j + xi_k)) B_m(xi_k), s = sqrt(hH)
// (or the derivative basis with 1/sqrt(hH)).
static std::vector<double> moment_1d(int P, int cluster_level, int cluster_ref, int np, bool deriv) {
  int n = 1 << cluster_ref;
  double h = 1. / n, H = 1. / (1 << cluster_level);
  const Rule1D& Q = gauss_rule((int)std::ceil(0.5 * (np + P - 2)) + 1);
  std::vector<double> x = cheb_points(np), c = newton_coefficients(np, x);
  std::vector<double> mom((size_t)np * n * (P + 1), 0.0);
  double b[64];
  double scale = deriv ? 1.0 / std::sqrt(h * H) : std::sqrt(h * H);
  for (int i = 0; i < np; ++i)
    for (int j = 0; j < n; ++j)
      for (size_t k = 0; k < Q.x.size(); ++k) {
        double w = Q.w[k] * scale * lagrange_value(c, x, np, i, h * (j + Q.x[k]));
        if (deriv) bernstein_der(P, Q.x[k], b); else bernstein(P, Q.x[k], b);
        for (int m = 0; m <= P; ++m) mom[(size_t)i * n * (P + 1) + j * (P + 1) + m] += w * b[m];
      }
  return mom;
}
static std::vector<double> moment_2d(int P, int cl, int cr, int np, bool ds, bool dt) {
  int n = 1 << cr, pp = P + 1, p2 = pp * pp, ncl = n * n;
  std::vector<double> ms = moment_1d(P, cl, cr, np, ds), mt = moment_1d(P, cl, cr, np, dt);
  int cols = ncl * p2, w1 = n * pp;
  std::vector<double> out((size_t)np * np * cols);
  for (int k = 0; k < ncl; ++k) {
    int ex, ey;
    quadtree_coords(k, cr, &ex, &ey);
    for (int i = 0; i < np; ++i)
      for (int j = 0; j < np; ++j)
        for (int ay = 0; ay < pp; ++ay)
          for (int ax = 0; ax < pp; ++ax)
            out[(size_t)(i * np + j) * cols + p2 * k + ay * pp + ax] =
                ms[(size_t)i * w1 + ex * pp + ax] * mt[(size_t)j * w1 + ey * pp + ay];
  }
  return out;
}
void moment_factors(int P, int cl, int cr, int np, std::vector<double>* ms, std::vector<double>* mt,
                    std::vector<int>* cmap) {
  const int n = 1 << cr, pp = P + 1, p2 = pp * pp;
  *ms = moment_1d(P, cl, cr, np, false);
  *mt = moment_1d(P, cl, cr, np, false);
  cmap->assign((size_t)n * n * p2, 0);
  for (int k = 0; k < n * n; ++k) {
    int ex, ey;
    quadtree_coords(k, cr, &ex, &ey);
    for (int ay = 0; ay < pp; ++ay)
      for (int ax = 0; ax < pp; ++ax) (*cmap)[p2 * k + ay * pp + ax] = (ex * pp + ax) | ((ey * pp + ay) << 8);
  }
}
std::vector<std::vector<double>> moment_matrices(bool maxwell, int P, int cl, int cr, int np) {
  std::vector<std::vector<double>> out;
  std::vector<double> m = moment_2d(P, cl, cr, np, false, false);
  if (!maxwell) {
    out.push_back(m);
    return out;
  }
  std::vector<double> mdx = moment_2d(P, cl, cr, np, true, false), mdy = moment_2d(P, cl, cr, np, false, true);
  std::vector<double> a = m, b = m;
  a.insert(a.end(), mdx.begin(), mdx.end());
  b.insert(b.end(), mdy.begin(), mdy.end());
  out.push_back(a);
  out.push_back(b);
  return out;
}

}  // namespace bg
