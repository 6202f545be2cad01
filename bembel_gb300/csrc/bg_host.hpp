// Host-side setup of the GB300 H2 single-layer operator: geometry, element
// table, cluster balls, block partition, element-pair classification,
// quadrature rules, the transformation matrix T and the FMM moment/transfer
// matrices. Everything here is computed once per operator and uploaded as
// flat tables; the hot path (assembly, matvec, solve) runs on the device.
#pragma once
#include <array>
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

namespace bg {

constexpr double kPi = 3.14159265358979323846;

// One rational Bezier patch in homogeneous coordinates:
// cp[4 * (ix * py + iy) + k], k = x, y, z, w; px/py = number of control
// points (degree + 1) per direction (Geometry/Patch.hpp:63-104).
//
// A patch with face >= 0 is instead the analytic cube-sphere map of face
// `face` (no control points): the unit-sphere image x / |x| of one face of
// the cube [-1, 1]^3 (see cube_face_frame). The reference's patches are all
// rational B-splines (Patch.hpp:63-104); this kind is an addition.
struct PatchData {
  int px = 0, py = 0;
  std::vector<double> cp;
  int face = -1;
};
struct Geometry {
  std::vector<PatchData> patches;
};
// Parse an Octave-NURBS .dat file (Geometry/GeometryIO.hpp:25-122). Patches
// with interior knots are rejected (the H2 path uses Bezier patches).
bool load_dat(const std::string& path, Geometry* g, std::string* err);
// Parse the rational B-spline surfaces (entity 128) of an IGES file
// (Geometry/GeometryIGS.hpp:25-151): fixed 80-column records, section letter
// in column 73, two directory lines per entity, parameter data in columns
// 1-64. Single-span (Bezier) surfaces only, like load_dat.
bool load_igs(const std::string& path, Geometry* g, std::string* err);

void bernstein(int p, double x, double* b);      // degree p, p+1 values
void bernstein_der(int p, double x, double* b);  // derivative, p+1 values
// Patch::eval (point only, division by the weight; Patch.hpp:115-155)
void patch_point(const PatchData& P, double s, double t, double* x3);
// Patch::updateSurfacePoint (Patch.hpp:294-365): out[0..8] = x, dx, dy
void patch_frame(const PatchData& P, double s, double t, double* out9);
// The unit sphere as six analytic patches: face f lies on the cube plane
// x_k = sg (k = f / 2, sg = +1 for even f, -1 for odd f) and is parametrised
// by c(s, t) = sg e_k + (2 s - 1) e_a + (2 t - 1) e_b with (a, b) = (k + 1,
// k + 2) mod 3 for sg = +1 and (k + 2, k + 1) mod 3 for sg = -1, so that
// e_a x e_b is the outward normal; the surface point is c / |c|.
void cube_sphere(Geometry* g);
// x, dx/ds, dx/dt of face f at (s, t): x = c / |c|,
// dx/ds = 2 (e_a - x x_a) / |c|, dx/dt = 2 (e_b - x x_b) / |c|.
void cube_face_frame(int face, double s, double t, double* out9);

// Gauss-Legendre rule with n points on [0,1], ascending nodes.
struct Rule1D {
  std::vector<double> x, w;
};
const Rule1D& gauss_rule(int npoints);

// Uniformly refined mesh: element id = patch * 4^M + quadtree index with the
// son order (0,0), (1,0), (1,1), (0,1) of ElementTree::refineLeaf
// (ElementTree.hpp:706-711).
struct Mesh {
  int M = 0, npatch = 0, ne = 0, n1d = 1, nverts = 0;
  std::vector<int> patch;   // per element
  std::vector<int> ix, iy;  // grid position in its patch
  std::vector<double> llc;  // 2 per element (patch coordinates)
  std::vector<int> vert;    // 4 per element: corners (0,0),(1,0),(1,1),(0,1)
  // enclosing balls per level l = 0..M, cluster c in [0, npatch*4^l):
  // ball[l][4c + 0..2] midpoint, ball[l][4c + 3] radius
  std::vector<std::vector<double>> ball;
  // patch adjacency [patch, neighbour patch or -1, edge, neighbour edge]
  std::vector<std::array<int, 4>> patch_edges;
};
bool build_mesh(const Geometry& g, int M, Mesh* mesh, std::string* err);
int quadtree_index(int ix, int iy, int level);  // (ix, iy) -> local id
void quadtree_coords(int local, int level, int* ix, int* iy);

// Block partition (BlockClusterTree.hpp:154-182, 255-278).
struct Partition {
  int dense_level = 0;  // level of all dense leaves: max(M - mcl, 0)
  int far_levels = 0;   // low-rank leaves exist on levels 0 .. far_levels-1
  std::vector<int> dense_c1, dense_c2;               // cluster ids at dense_level
  std::vector<std::vector<int>> far_c1, far_c2;      // per level
  // leaf list in tree order for inspection: cc, level, c1, c2
  std::vector<int> leaf_list;
};
void build_partition(const Mesh& m, double eta, int mcl, Partition* part);

// DuffyTrick classification of an element pair (compareElements.hpp:23-69 and
// the degree rule of LinearOperatorBase.hpp:56-89 with operator order -1).
struct PairClass {
  int cs, rot1, rot2, deg;
};
PairClass classify_pair(const Mesh& m, int e1, int e2, int P);

// Sparse matrix in CSR.
struct Csr {
  int rows = 0, cols = 0;
  std::vector<int> ptr, idx;
  std::vector<double> val;
};
// T = Projector * Glue (AnsatzSpace.hpp:102-111) for knot repetition 1:
// discontinuous patchwise B-splines (Laplace/Helmholtz) or div-conforming
// vector B-splines (Maxwell).
bool build_transform(const Mesh& m, int P, bool div_conforming, Csr* T, std::string* err);
Csr transpose(const Csr& A);

// FMM: Chebyshev roots on [0,1] (H2Multipole.hpp:20-32), transfer matrix
// (np^2 x 4np^2, row-major, blocks [T0 T2 T3 T1], H2Multipole.hpp:76-115) and
// moment matrices (rows nc*np^2, cols 4^mcl p^2, row-major) per vector
// component (H2Multipole.hpp:120-318, Maxwell/SingleLayerOperator.hpp:153-183).
std::vector<double> cheb_points(int np);
std::vector<double> transfer_matrix(int np);
std::vector<std::vector<double>> moment_matrices(bool maxwell, int P, int cluster_level, int cluster_ref, int np);
// The 1-D factors of the transfer and (scalar) moment matrices above:
// E = [E0 | E1] (np x np each, E_h[c][p] = L_p(x_c / 2 + h / 2)); ms, mt the
// 1-D moments (np x w1, w1 = 2^cluster_ref (P + 1)); cmap[q] = a | (b << 8)
// for superspace row q of a leaf cluster, so that
// moments[(i np + j)][q] = ms[i][a] mt[j][b].
std::vector<double> transfer_factors(int np);
void moment_factors(int P, int cluster_level, int cluster_ref, int np, std::vector<double>* ms, std::vector<double>* mt,
                    std::vector<int>* cmap);

}  // namespace bg
