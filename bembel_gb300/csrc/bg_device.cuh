// Device helpers shared by the GB300 kernels: complex arithmetic, the FP64
// reciprocal square root, Bernstein bases and the surface map of a rational
// Bezier patch (Patch::updateSurfacePoint, Geometry/Patch.hpp:294-365).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace bg {

struct cd {  // complex<double>, interleaved
  double re, im;
};
struct cf {  // complex<float>
  float re, im;
};
struct __align__(32) d4 {  // point + weight, one 32-byte load
  double x, y, z, w;
};
__host__ __device__ inline cd operator+(cd a, cd b) { return {a.re + b.re, a.im + b.im}; }
__host__ __device__ inline cd operator-(cd a, cd b) { return {a.re - b.re, a.im - b.im}; }
__host__ __device__ inline cd operator*(cd a, cd b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__host__ __device__ inline cd operator*(cd a, double s) { return {a.re * s, a.im * s}; }
__host__ __device__ inline cf operator+(cf a, cf b) { return {a.re + b.re, a.im + b.im}; }
__host__ __device__ inline cf operator*(cf a, cf b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__host__ __device__ inline cf operator*(cf a, float s) { return {a.re * s, a.im * s}; }

// zero / fma helpers working for real and complex scalars
template <typename S> __device__ inline S zero();
template <> __device__ inline double zero<double>() { return 0.0; }
template <> __device__ inline float zero<float>() { return 0.0f; }
template <> __device__ inline cd zero<cd>() { return {0.0, 0.0}; }
template <> __device__ inline cf zero<cf>() { return {0.0f, 0.0f}; }
__device__ inline double fmac(double acc, double a, double b) { return fma(a, b, acc); }
__device__ inline float fmac(float acc, float a, float b) { return fmaf(a, b, acc); }
__device__ inline cd fmac(cd acc, cd a, cd b) {
  return {fma(a.re, b.re, fma(-a.im, b.im, acc.re)), fma(a.re, b.im, fma(a.im, b.re, acc.im))};
}
__device__ inline cf fmac(cf acc, cf a, cf b) {
  return {fmaf(a.re, b.re, fmaf(-a.im, b.im, acc.re)), fmaf(a.re, b.im, fmaf(a.im, b.re, acc.im))};
}
__device__ inline cd fmac(cd acc, double a, cd b) { return {fma(a, b.re, acc.re), fma(a, b.im, acc.im)}; }
__device__ inline cf fmac(cf acc, float a, cf b) { return {fmaf(a, b.re, acc.re), fmaf(a, b.im, acc.im)}; }
__device__ inline cd fmac(cd acc, cd a, double b) { return {fma(a.re, b, acc.re), fma(a.im, b, acc.im)}; }
__device__ inline cf fmac(cf acc, cf a, float b) { return {fmaf(a.re, b, acc.re), fmaf(a.im, b, acc.im)}; }

// 1/sqrt(x) in FP64: single-precision estimate refined by two Newton-Raphson
// steps y <- y (3 - x y^2) / 2 for f(y) = y^-2 - x. Each step squares the
// relative error, so the FP32 seed (rel. error ~1e-7) reaches FP64 accuracy.
// Valid for normal x in the FP32 range (all distances here).
__device__ inline double rsqrt_nr(double x) {
  double y = (double)rsqrtf((float)x);
  double hx = 0.5 * x;
  y = y * fma(-hx * y, y, 1.5);
  y = y * fma(-hx * y, y, 1.5);
  return y;
}

// 1/x in FP64: single-precision estimate refined by two Newton-Raphson steps
// y <- y (2 - x y); valid for normal x in the FP32 range.
__device__ inline double rcp_nr(double x) {
  double y = (double)__frcp_rn((float)x);
  y = y * fma(-x, y, 2.0);
  y = y * fma(-x, y, 2.0);
  return y;
}

// Bernstein basis of degree p at x (p <= N-1), built by the triangular
// recurrence b_i <- (1-x) b_i + x b_{i-1}.
template <int N>
__device__ inline void bern(int p, double x, double* b) {
  b[0] = 1.0;
#pragma unroll
  for (int k = 1; k < N; ++k) {
    if (k <= p) {
      double prev = 0.0;
#pragma unroll
      for (int i = 0; i < k; ++i) {
        double t = b[i];
        b[i] = fma(1.0 - x, t, prev);
        prev = x * t;
      }
      b[k] = prev;
    }
  }
}
// Bernstein basis and its derivative, degree p (p <= N-1)
template <int N>
__device__ inline void bern_der(int p, double x, double* b, double* db) {
  double lo[N];
  bern<N>(p - 1 < 0 ? 0 : p - 1, x, lo);
  if (p == 0) {
    b[0] = 1.0;
    db[0] = 0.0;
    return;
  }
#pragma unroll
  for (int i = 0; i < N; ++i) {
    if (i <= p) {
      double a = i > 0 ? lo[i - 1] : 0.0;
      double c = i < p ? lo[i] : 0.0;
      db[i] = p * (a - c);
    }
  }
  bern<N>(p, x, b);
}

// Patches on the device: orders px, py <= G; control points at cp + off
// (4 doubles per point, index 4 * (ix * py + iy) + k).
struct PatchTable {
  const int* meta;     // per patch: px, py, offset (in doubles)
  const double* cp;
};

// Analytic cube-sphere face f (meta px = 0, py = f): the unit-sphere image
// c / |c| of c(s, t) = sg e_k + (2 s - 1) e_a + (2 t - 1) e_b, k = f / 2,
// sg = +1 for even f (a, b = k + 1, k + 2 mod 3), -1 for odd f (a, b =
// k + 2, k + 1 mod 3), so e_a x e_b points outwards;
// dx/ds = 2 (e_a - x x_a) / |c|, dx/dt = 2 (e_b - x x_b) / |c|.
__device__ inline void cube_face_frame(int f, double s, double t, double* x, double* dx, double* dy) {
  const int k = f >> 1;
  const bool pos = (f & 1) == 0;
  const int a = pos ? (k + 1) % 3 : (k + 2) % 3, b = pos ? (k + 2) % 3 : (k + 1) % 3;
  double c[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) c[j] = j == k ? (pos ? 1.0 : -1.0) : (j == a ? fma(2.0, s, -1.0) : fma(2.0, t, -1.0));
  const double ir = rsqrt_nr(fma(c[0], c[0], fma(c[1], c[1], c[2] * c[2])));
#pragma unroll
  for (int j = 0; j < 3; ++j) x[j] = c[j] * ir;
  const double xa = x[0] * (a == 0) + x[1] * (a == 1) + x[2] * (a == 2);
  const double xb = x[0] * (b == 0) + x[1] * (b == 1) + x[2] * (b == 2);
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    dx[j] = 2.0 * ((j == a ? 1.0 : 0.0) - x[j] * xa) * ir;
    dy[j] = 2.0 * ((j == b ? 1.0 : 0.0) - x[j] * xb) * ir;
  }
}

// Surface point at patch coordinates (s, t): x, dx, dy (9 doubles)
template <int G>
__device__ inline void surface_frame(const PatchTable& pt, int patch, double s, double t, double* x, double* dx,
                                     double* dy) {
  const int px = __ldg(&pt.meta[3 * patch]), py = __ldg(&pt.meta[3 * patch + 1]);
  if (px == 0) {
    cube_face_frame(py, s, t, x, dx, dy);
    return;
  }
  const double* cp = pt.cp + __ldg(&pt.meta[3 * patch + 2]);
  double bs[G], dbs[G], bt[G], dbt[G];
  bern_der<G>(px - 1, s, bs, dbs);
  bern_der<G>(py - 1, t, bt, dbt);
  double h[4] = {0, 0, 0, 0}, hs[4] = {0, 0, 0, 0}, ht[4] = {0, 0, 0, 0};
#pragma unroll
  for (int i = 0; i < G; ++i) {
    if (i < px) {
      // inner sum over t first: q = sum_j bt_j P_ij, qt = sum_j dbt_j P_ij
      double q[4] = {0, 0, 0, 0}, qt[4] = {0, 0, 0, 0};
#pragma unroll
      for (int j = 0; j < G; ++j) {
        if (j < py) {
          const d4 c = *reinterpret_cast<const d4*>(cp + 4 * (i * py + j));
          q[0] = fma(c.x, bt[j], q[0]); q[1] = fma(c.y, bt[j], q[1]);
          q[2] = fma(c.z, bt[j], q[2]); q[3] = fma(c.w, bt[j], q[3]);
          qt[0] = fma(c.x, dbt[j], qt[0]); qt[1] = fma(c.y, dbt[j], qt[1]);
          qt[2] = fma(c.z, dbt[j], qt[2]); qt[3] = fma(c.w, dbt[j], qt[3]);
        }
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        h[k] = fma(bs[i], q[k], h[k]);
        hs[k] = fma(dbs[i], q[k], hs[k]);
        ht[k] = fma(bs[i], qt[k], ht[k]);
      }
    }
  }
  const double iw = rcp_nr(h[3]);
  const double iw2 = iw * iw;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    x[k] = h[k] * iw;
    dx[k] = (hs[k] * h[3] - h[k] * hs[3]) * iw2;
    dy[k] = (ht[k] * h[3] - h[k] * ht[3]) * iw2;
  }
}

// Surface points along a line of one fixed patch coordinate: the control
// points are contracted along the fixed direction once (values with the
// Bernstein basis and its derivative there), so every point of the line
// costs one G-term contraction instead of G^2 (the sums of
// Patch::updateSurfacePoint, Patch.hpp:294-365, associated the other way).
// Analytic patches keep the fixed coordinate and evaluate in closed form.
template <int G>
struct SurfaceLine {
  double q[G][4], qd[G][4];  // q_m = sum_n B_n(fixed) P, qd_m = sum_n B'_n(fixed) P
  double c;                  // the fixed coordinate
  int n, face;               // terms along the free direction; n = 0: analytic face
  bool fix_s;
};

template <int G>
__device__ inline void surface_line(const PatchTable& pt, int patch, bool fix_s, double c, SurfaceLine<G>& L) {
  const int px = __ldg(&pt.meta[3 * patch]), py = __ldg(&pt.meta[3 * patch + 1]);
  L.fix_s = fix_s;
  L.c = c;
  if (px == 0) {
    L.n = 0;
    L.face = py;
    return;
  }
  const double* cp = pt.cp + __ldg(&pt.meta[3 * patch + 2]);
  const int nf = fix_s ? px : py;
  L.n = fix_s ? py : px;
  double b[G], db[G];
  bern_der<G>(nf - 1, c, b, db);
#pragma unroll
  for (int m = 0; m < G; ++m) {
#pragma unroll
    for (int k = 0; k < 4; ++k) L.q[m][k] = L.qd[m][k] = 0.0;
    if (m < L.n) {
#pragma unroll
      for (int n = 0; n < G; ++n) {
        if (n < nf) {
          const d4 P = *reinterpret_cast<const d4*>(cp + 4 * (fix_s ? n * py + m : m * py + n));
          L.q[m][0] = fma(P.x, b[n], L.q[m][0]); L.q[m][1] = fma(P.y, b[n], L.q[m][1]);
          L.q[m][2] = fma(P.z, b[n], L.q[m][2]); L.q[m][3] = fma(P.w, b[n], L.q[m][3]);
          L.qd[m][0] = fma(P.x, db[n], L.qd[m][0]); L.qd[m][1] = fma(P.y, db[n], L.qd[m][1]);
          L.qd[m][2] = fma(P.z, db[n], L.qd[m][2]); L.qd[m][3] = fma(P.w, db[n], L.qd[m][3]);
        }
      }
    }
  }
}

// x, dx/ds, dx/dt at the free coordinate v of the line
template <int G>
__device__ inline void surface_line_point(const SurfaceLine<G>& L, double v, double* x, double* dx, double* dy) {
  if (L.n == 0) {
    if (L.fix_s) cube_face_frame(L.face, L.c, v, x, dx, dy);
    else cube_face_frame(L.face, v, L.c, x, dx, dy);
    return;
  }
  double b[G], db[G];
  bern_der<G>(L.n - 1, v, b, db);
  double h[4] = {0, 0, 0, 0}, hf[4] = {0, 0, 0, 0}, hv[4] = {0, 0, 0, 0};
#pragma unroll
  for (int m = 0; m < G; ++m) {
    if (m < L.n) {
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        h[k] = fma(b[m], L.q[m][k], h[k]);
        hf[k] = fma(b[m], L.qd[m][k], hf[k]);
        hv[k] = fma(db[m], L.q[m][k], hv[k]);
      }
    }
  }
  const double iw = rcp_nr(h[3]);
  const double iw2 = iw * iw;
  const double hs3 = L.fix_s ? hf[3] : hv[3], ht3 = L.fix_s ? hv[3] : hf[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double hsk = L.fix_s ? hf[k] : hv[k], htk = L.fix_s ? hv[k] : hf[k];
    x[k] = h[k] * iw;
    dx[k] = (hsk * h[3] - h[k] * hs3) * iw2;
    dy[k] = (htk * h[3] - h[k] * ht3) * iw2;
  }
}

// surface measure |dx x dy|
__device__ inline double surface_measure(const double* dx, const double* dy) {
  double n0 = dx[1] * dy[2] - dx[2] * dy[1];
  double n1 = dx[2] * dy[0] - dx[0] * dy[2];
  double n2 = dx[0] * dy[1] - dx[1] * dy[0];
  double n2s = n0 * n0 + n1 * n1 + n2 * n2;
  return n2s * rsqrt_nr(n2s);
}

// tensor Bernstein basis of degree P at (s, t), local index iy*(P+1)+ix
template <int P>
__device__ inline void tensor_basis(double s, double t, double* phi) {
  double bs[P + 1], bt[P + 1];
  bern<P + 1>(P, s, bs);
  bern<P + 1>(P, t, bt);
#pragma unroll
  for (int iy = 0; iy <= P; ++iy)
#pragma unroll
    for (int ix = 0; ix <= P; ++ix) phi[iy * (P + 1) + ix] = bs[ix] * bt[iy];
}

// tensor Bernstein basis and its two partial derivatives in the element
// coordinates (Basis.hpp:170-200 uses them for the divergence of the
// div-conforming Maxwell basis); same local index as tensor_basis
template <int P>
__device__ inline void tensor_basis_grad(double s, double t, double* phi, double* phx, double* phy) {
  double bs[P + 1], dbs[P + 1], bt[P + 1], dbt[P + 1];
  bern_der<P + 1>(P, s, bs, dbs);
  bern_der<P + 1>(P, t, bt, dbt);
#pragma unroll
  for (int iy = 0; iy <= P; ++iy)
#pragma unroll
    for (int ix = 0; ix <= P; ++ix) {
      phi[iy * (P + 1) + ix] = bs[ix] * bt[iy];
      phx[iy * (P + 1) + ix] = dbs[ix] * bt[iy];
      phy[iy * (P + 1) + ix] = bs[ix] * dbt[iy];
    }
}

// the DuffyTrick rotation tau (DuffyTrick/tau.hpp:26-42)
__device__ inline void tau(double x, double y, int c, double* o) {
  if (c == 1) { o[0] = 1 - y; o[1] = x; }
  else if (c == 2) { o[0] = 1 - x; o[1] = 1 - y; }
  else if (c == 3) { o[0] = y; o[1] = 1 - x; }
  else { o[0] = x; o[1] = y; }
}

}  // namespace bg
