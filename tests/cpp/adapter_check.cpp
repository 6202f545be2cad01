// Checks of the header-style C++ front end (include/bembel_gb300/H2MatrixGPU.hpp)
// through the C ABI. Usage: adapter_check <sphere.dat> [gpu]
//  - host: geometry from a .dat file and from its own Bezier data give the
//    same surface points; operator sizes; errors arrive as exceptions.
//  - gpu: assemble a small Laplace operator and compare the FP64 and the
//    FP32 product (relative difference below 1e-5).
#include <bembel_gb300/H2MatrixGPU.hpp>

#include <cmath>
#include <complex>
#include <cstdio>
#include <vector>

using namespace bembel_gb300;

static int fail(const char* what) {
  std::printf("FAIL %s\n", what);
  return 1;
}

int main(int argc, char** argv) {
  if (argc < 2) return fail("usage");
  const bool gpu = argc > 2 && std::string(argv[2]) == "gpu";
  Context ctx(gpu ? 0 : -1);
  Geometry g = Geometry::from_dat(ctx, argv[1]);
  const int np = g.num_patches();
  std::vector<int> px, py;
  std::vector<double> data;
  for (int p = 0; p < np; ++p) {
    int a = 0, b = 0;
    std::vector<double> d = g.patch_data(p, &a, &b);
    px.push_back(a);
    py.push_back(b);
    data.insert(data.end(), d.begin(), d.end());
  }
  Geometry h = Geometry::from_bezier(ctx, px, py, data);
  if (h.num_patches() != np) return fail("patch count");
  double worst = 0.0;
  for (int p = 0; p < np; ++p)
    for (int i = 0; i <= 4; ++i)
      for (int j = 0; j <= 4; ++j) {
        double u[12], v[12];
        if (bg_geometry_surface_point(g.get(), p, 0.25 * i, 0.25 * j, u) != BG_OK) return fail("surface point");
        if (bg_geometry_surface_point(h.get(), p, 0.25 * i, 0.25 * j, v) != BG_OK) return fail("surface point");
        for (int k = 0; k < 12; ++k) worst = std::fmax(worst, std::fabs(u[k] - v[k]));
      }
  if (worst != 0.0) return fail("surface points differ");
  Operator<double> A(h, 3, 1, BG_LAPLACE_SL);
  if (A.rows() != 6 * 9 * 9) return fail("dofs at M=3, P=1");
  bool threw = false;
  try {
    Operator<std::complex<double>> bad(h, 2, 1, BG_LAPLACE_SL);
  } catch (const Error& e) {
    threw = e.status() == BG_INVALID_ARG;
  }
  if (!threw) return fail("scalar mismatch not reported");
  threw = false;
  try {
    std::vector<double> neg(data);
    neg[3] = -1.0;  // weight of the first control point
    Geometry::from_bezier(ctx, px, py, neg);
  } catch (const Error& e) {
    threw = e.status() == BG_INVALID_ARG && std::string(e.what()).find("weight") != std::string::npos;
  }
  if (!threw) return fail("invalid weight not reported");
  // launch plans are operator state: set, read back, refused when out of range
  A.set_plan(32, BG_PREC_FP32, bg_launch_plan{2, 608, 1});
  const bg_launch_plan lp = A.plan(32, BG_PREC_FP32);
  if (lp.near_kernel != 2 || lp.split_k_batches != 608 || lp.far_order != 1) return fail("launch plan round trip");
  if (A.plan(32, BG_PREC_MIXED).split_k_batches != -1) return fail("built-in plan");
  threw = false;
  try {
    A.set_plan(32, BG_PREC_FP32, bg_launch_plan{0, -1, 3});
  } catch (const Error& e) {
    threw = e.status() == BG_INVALID_ARG;
  }
  if (!threw) return fail("invalid launch plan not reported");
  // the analytic cube sphere: six patches without control data, an operator
  // on it has the same unknowns as on the NURBS sphere
  Geometry cs = Geometry::cube_sphere(ctx);
  if (cs.num_patches() != 6) return fail("cube sphere patches");
  threw = false;
  try {
    int a = 0, b = 0;
    cs.patch_data(0, &a, &b);
  } catch (const Error& e) {
    threw = e.status() == BG_UNSUPPORTED;
  }
  if (!threw) return fail("cube sphere patch data not refused");
  Operator<double> C(cs, 3, 1, BG_LAPLACE_SL);
  if (C.rows() != A.rows()) return fail("cube sphere dofs");
  if (gpu) {
    Operator<double> B(h, 2, 1, BG_LAPLACE_SL);
    B.assemble();
    const long n = B.rows();
    std::vector<double> x(2 * n), y64(2 * n), y32(2 * n);
    for (long i = 0; i < 2 * n; ++i) x[i] = std::sin(0.37 * i) + 0.5;
    B.matvec(x.data(), n, y64.data(), n, 2);
    B.matvec(x.data(), n, y32.data(), n, 2, 1.0, 0.0, BG_PREC_FP32);
    double num = 0.0, den = 0.0;
    for (long i = 0; i < 2 * n; ++i) {
      num += (y64[i] - y32[i]) * (y64[i] - y32[i]);
      den += y64[i] * y64[i];
    }
    if (!(std::sqrt(num / den) < 1e-5)) return fail("FP32 product differs from FP64");
    std::vector<double> sol(2 * n);
    bg_solve_stats st = B.solve(y64.data(), sol.data(), 2);
    double e2 = 0.0, x2 = 0.0;
    for (long i = 0; i < 2 * n; ++i) {
      e2 += (sol[i] - x[i]) * (sol[i] - x[i]);
      x2 += x[i] * x[i];
    }
    if (!(st.final_relres <= 1e-8)) return fail("solve residual");
    std::printf("gpu: N=%ld, FP32 vs FP64 %.2e, solve rel. error %.2e\n", n, std::sqrt(num / den), std::sqrt(e2 / x2));
  }
  std::printf("OK\n");
  return 0;
}
