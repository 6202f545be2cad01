// Load vectors and potentials on GB300.
//
// bg_load_vector: DiscreteLinearForm<DirichletTrace<S>, Op>::compute
// (LinearForm/DiscreteLinearForm.hpp:44-83, LinearForm/DirichletTrace.hpp:38-66):
// per element the (P+2)^2-point tensor Gauss rule, weight h*w, integrand
// u(x) |dx x dy| phi_a, then the transpose of the transformation matrix.
// bg_potential: DiscretePotential::evaluate (Potential/DiscretePotential.hpp:49-107)
// for the Laplace / Helmholtz single layer potential.
#include <algorithm>
#include <complex>
#include <vector>

#include "bg_operator.hpp"

using namespace bg;

namespace {

constexpr double kInv4Pi = 0.07957747154594767;

// analytic Dirichlet data (examples/Data.hpp), kind 0/1/2, per right-hand side
__device__ inline cd data_value(int kind, const double* prm, const double* x, double kre, double kim) {
  if (kind == 2) {
    const double dx = prm[0] * x[0] + prm[1] * x[1] + prm[2] * x[2];
    // exp(-i k d.x), k = kre + i kim
    double sn, cs;
    sincos(kre * dx, &sn, &cs);
    const double a = kim != 0.0 ? exp(kim * dx) : 1.0;
    return {cs * a, -sn * a};
  }
  const double d0 = x[0] - prm[0], d1 = x[1] - prm[1], d2 = x[2] - prm[2];
  const double r2 = d0 * d0 + d1 * d1 + d2 * d2;
  const double inv = rsqrt_nr(r2);
  if (kind == 0) return {inv * kInv4Pi, 0.0};
  const double r = r2 * inv;
  double sn, cs;
  sincos(kre * r, &sn, &cs);
  const double a = (kim != 0.0 ? exp(kim * r) : 1.0) * inv * kInv4Pi;
  return {cs * a, -sn * a};
}

// thread per (element, rhs); output superspace rows e*p2 + a, row-major k
template <int G, int P, bool CPLX>
__global__ void k_load(PatchTable pt, ElementTable et, int ne, const double* __restrict__ gx,
                       const double* __restrict__ gw, int n1, int kind, const double* __restrict__ prm, int k,
                       double kre, double kim, double* __restrict__ out) {
  constexpr int P2 = (P + 1) * (P + 1);
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)ne * k) return;
  const int e = (int)(t / k), c = (int)(t % k);
  const double h = et.h;
  double acc_re[P2], acc_im[P2];
#pragma unroll
  for (int a = 0; a < P2; ++a) acc_re[a] = acc_im[a] = 0.0;
  for (int q = 0; q < n1 * n1; ++q) {
    const double u = gx[q / n1], v = gx[q % n1], w = gw[q / n1] * gw[q % n1];
    double x[3], dx[3], dy[3], phi[P2];
    surface_frame<G>(pt, et.patch[e], et.llc[2 * e] + h * u, et.llc[2 * e + 1] + h * v, x, dx, dy);
    const double wk = h * w * surface_measure(dx, dy);
    const cd f = data_value(kind, prm + 3 * c, x, kre, kim);
    tensor_basis<P>(u, v, phi);
#pragma unroll
    for (int a = 0; a < P2; ++a) {
      acc_re[a] = fma(f.re * wk, phi[a], acc_re[a]);
      acc_im[a] = fma(f.im * wk, phi[a], acc_im[a]);
    }
  }
#pragma unroll
  for (int a = 0; a < P2; ++a) {
    const long o = ((long)e * P2 + a) * k + c;
    if (CPLX) {
      out[2 * o] = acc_re[a];
      out[2 * o + 1] = acc_im[a];
    } else {
      out[o] = acc_re[a];
    }
  }
}

// Maxwell excitation: the field of a Hertz dipole (examples/Data.hpp:73-90),
// prm = position (3), moment (3), and its tangential part integrated against
// the two tangent directions of the vector basis
// (LinearForm/RotatedTangentialTrace.hpp:30-87): per Gauss point with weight
// h w, t = (f - (f.n) n) h w, then dx.t phi_a into component 0 and dy.t phi_a
// into component 1 of the superspace vector.
__device__ inline void dipole_field(const double* prm, const double* x, double kre, double kim, cd* f) {
  const double c0 = x[0] - prm[0], c1 = x[1] - prm[1], c2 = x[2] - prm[2];
  const double r2 = c0 * c0 + c1 * c1 + c2 * c2;
  const double ir = rsqrt_nr(r2), r = r2 * ir;
  const double n[3] = {c0 * ir, c1 * ir, c2 * ir};
  const double* len = prm + 3;
  // (n x len) x n and 3 n (n.len) - len
  const double nl[3] = {n[1] * len[2] - n[2] * len[1], n[2] * len[0] - n[0] * len[2], n[0] * len[1] - n[1] * len[0]};
  const double ncl[3] = {nl[1] * n[2] - nl[2] * n[1], nl[2] * n[0] - nl[0] * n[2], nl[0] * n[1] - nl[1] * n[0]};
  const double ndl = n[0] * len[0] + n[1] * len[1] + n[2] * len[2];
  // exp(-i kappa r) with kappa = kre + i kim
  double sn, cs;
  sincos(kre * r, &sn, &cs);
  const double a = kim != 0.0 ? exp(kim * r) : 1.0;
  const cd ex{cs * a, -sn * a};
  // ec = (1/r^3 + i kappa / r^2) exp(-i kappa r), fk = kappa^2 exp(-i kappa r) / r
  const cd ec = cd{ir * ir * ir - kim * ir * ir, kre * ir * ir} * ex;
  const cd fk = cd{kre * kre - kim * kim, 2 * kre * kim} * ex * ir;
#pragma unroll
  for (int k = 0; k < 3; ++k) f[k] = fk * ncl[k] + ec * (3 * n[k] * ndl - len[k]);
}

template <int G, int P>
__global__ void k_load_mw(PatchTable pt, ElementTable et, int ne, const double* __restrict__ gx,
                          const double* __restrict__ gw, int n1, const double* __restrict__ prm, int k, double kre,
                          double kim, cd* __restrict__ out) {
  constexpr int P2 = (P + 1) * (P + 1);
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)ne * k) return;
  const int e = (int)(t / k), c = (int)(t % k);
  const double h = et.h;
  cd acc0[P2], acc1[P2];
#pragma unroll
  for (int a = 0; a < P2; ++a) acc0[a] = acc1[a] = zero<cd>();
  for (int q = 0; q < n1 * n1; ++q) {
    const double u = gx[q / n1], v = gx[q % n1], w = h * gw[q / n1] * gw[q % n1];
    double x[3], dx[3], dy[3], phi[P2];
    surface_frame<G>(pt, et.patch[e], et.llc[2 * e] + h * u, et.llc[2 * e + 1] + h * v, x, dx, dy);
    double n[3] = {dx[1] * dy[2] - dx[2] * dy[1], dx[2] * dy[0] - dx[0] * dy[2], dx[0] * dy[1] - dx[1] * dy[0]};
    const double in = rsqrt_nr(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    n[0] *= in;
    n[1] *= in;
    n[2] *= in;
    cd f[3];
    dipole_field(prm + 6 * c, x, kre, kim, f);
    const cd fd = f[0] * n[0] + f[1] * n[1] + f[2] * n[2];
    cd tc[3];
#pragma unroll
    for (int m = 0; m < 3; ++m) tc[m] = (f[m] - fd * n[m]) * w;
    const cd cx = tc[0] * dx[0] + tc[1] * dx[1] + tc[2] * dx[2];
    const cd cy = tc[0] * dy[0] + tc[1] * dy[1] + tc[2] * dy[2];
    tensor_basis<P>(u, v, phi);
#pragma unroll
    for (int a = 0; a < P2; ++a) {
      acc0[a] = fmac(acc0[a], cx, phi[a]);
      acc1[a] = fmac(acc1[a], cy, phi[a]);
    }
  }
#pragma unroll
  for (int a = 0; a < P2; ++a) {
    out[((long)e * P2 + a) * k + c] = acc0[a];
    out[((long)(ne + e) * P2 + a) * k + c] = acc1[a];
  }
}

template <int G>
cudaError_t load_mw_p(int P, const PatchTable& pt, const ElementTable& et, int ne, const double* gx, const double* gw,
                      int n1, const double* prm, int k, double kre, double kim, cd* out, cudaStream_t s) {
  const unsigned g = (unsigned)(((long)ne * k + 127) / 128);
  switch (P) {
    case 1: k_load_mw<G, 1><<<g, 128, 0, s>>>(pt, et, ne, gx, gw, n1, prm, k, kre, kim, out); break;
    case 2: k_load_mw<G, 2><<<g, 128, 0, s>>>(pt, et, ne, gx, gw, n1, prm, k, kre, kim, out); break;
    case 3: k_load_mw<G, 3><<<g, 128, 0, s>>>(pt, et, ne, gx, gw, n1, prm, k, kre, kim, out); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}
cudaError_t launch_load_mw(int G, int P, const PatchTable& pt, const ElementTable& et, int ne, const double* gx,
                           const double* gw, int n1, const double* prm, int k, double kre, double kim, cd* out,
                           cudaStream_t s) {
  switch (G) {
    case 2: return load_mw_p<2>(P, pt, et, ne, gx, gw, n1, prm, k, kre, kim, out, s);
    case 3: return load_mw_p<3>(P, pt, et, ne, gx, gw, n1, prm, k, kre, kim, out, s);
    case 4: return load_mw_p<4>(P, pt, et, ne, gx, gw, n1, prm, k, kre, kim, out, s);
    case 5: return load_mw_p<5>(P, pt, et, ne, gx, gw, n1, prm, k, kre, kim, out, s);
    case 6: return load_mw_p<6>(P, pt, et, ne, gx, gw, n1, prm, k, kre, kim, out, s);
    default: return cudaErrorInvalidValue;
  }
}

// CTA per evaluation point: threads over (element, Gauss point) sum
// k(x, y_q) c_q rho(y_q) with c_q = h w |J| and rho = sum_a coef phi_a (the
// 1/h of FunctionEvaluatorEval and the h^2 of the weight leave h).
template <int P, bool CPLX>
__global__ void k_potential(const d4* __restrict__ tab, int ne, int Q, const double* __restrict__ basis,
                            const double* __restrict__ coef, int k, const double* __restrict__ pts, double kre,
                            double kim, double* __restrict__ out) {
  constexpr int P2 = (P + 1) * (P + 1);
  __shared__ double red_re[256], red_im[256];
  const int p = blockIdx.x;
  const double px = pts[3 * p], py = pts[3 * p + 1], pz = pts[3 * p + 2];
  for (int c = 0; c < k; ++c) {
    double sre = 0, sim = 0;
    for (long t = threadIdx.x; t < (long)ne * Q; t += blockDim.x) {
      const int e = (int)(t / Q), q = (int)(t % Q);
      const d4 y = tab[t];
      const double d0 = px - y.x, d1 = py - y.y, d2 = pz - y.z;
      const double r2 = d0 * d0 + d1 * d1 + d2 * d2;
      const double inv = rsqrt_nr(r2);
      double kr = inv * kInv4Pi * y.w, ki = 0.0;
      if (CPLX) {
        const double r = r2 * inv;
        double sn, cs;
        sincos(kre * r, &sn, &cs);
        const double a = kim != 0.0 ? exp(kim * r) : 1.0;
        ki = -sn * a * kr;
        kr = cs * a * kr;
      }
      double rre = 0, rim = 0;
#pragma unroll
      for (int a = 0; a < P2; ++a) {
        const long o = ((long)e * P2 + a) * k + c;
        const double b = basis[q * P2 + a];
        if (CPLX) {
          rre = fma(coef[2 * o], b, rre);
          rim = fma(coef[2 * o + 1], b, rim);
        } else {
          rre = fma(coef[o], b, rre);
        }
      }
      sre += kr * rre - ki * rim;
      sim += kr * rim + ki * rre;
    }
    red_re[threadIdx.x] = sre;
    red_im[threadIdx.x] = sim;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
      if (threadIdx.x < w) {
        red_re[threadIdx.x] += red_re[threadIdx.x + w];
        red_im[threadIdx.x] += red_im[threadIdx.x + w];
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      if (CPLX) {
        out[2 * ((long)c * gridDim.x + p)] = red_re[0];
        out[2 * ((long)c * gridDim.x + p) + 1] = red_im[0];
      } else {
        out[(long)c * gridDim.x + p] = red_re[0];
      }
    }
    __syncthreads();
  }
}

// Maxwell field (Maxwell/SingleLayerPotential.hpp:44-95 with the div-conforming
// evaluator of AnsatzSpace/FunctionEvaluatorEval.hpp:39-83): CTA per evaluation
// point x; threads over (element, Gauss point y) sum, with weight h^2 w,
//   k(x, y) u(y) + grad_x k(x, y) div u(y) / kappa^2,
// u = (c0 dx + c1 dy) / h, div u = (sum c0 d/ds phi + sum c1 d/dt phi) / h^2,
// c0, c1 the superspace coefficients of the two components at the element.
// tab holds x, dx, dy and h w per Gauss point; basis3 = [phi | d/ds phi | d/dt phi].
// Output: 3 complex values per point and right-hand side, [rhs][point][xyz].
template <int P>
__global__ void __launch_bounds__(256) k_potential_mw(const MwPt* __restrict__ tab, int ne, int Q, double h,
                                                      const double* __restrict__ basis3, const cd* __restrict__ coef,
                                                      int k, const double* __restrict__ pts, double kre, double kim,
                                                      cd inv_k2, cd* __restrict__ out) {
  constexpr int P2 = (P + 1) * (P + 1);
  __shared__ double red[6][256];
  const int p = blockIdx.x;
  const double px = pts[3 * p], py = pts[3 * p + 1], pz = pts[3 * p + 2];
  for (int c = 0; c < k; ++c) {
    cd acc[3] = {zero<cd>(), zero<cd>(), zero<cd>()};
    for (long t = threadIdx.x; t < (long)ne * Q; t += blockDim.x) {
      const int e = (int)(t / Q), q = (int)(t % Q);
      const MwPt y = tab[t];
      cd t0 = zero<cd>(), t1 = zero<cd>(), dv = zero<cd>();
#pragma unroll
      for (int a = 0; a < P2; ++a) {
        const cd a0 = coef[((long)e * P2 + a) * k + c], a1 = coef[((long)(ne + e) * P2 + a) * k + c];
        t0 = fmac(t0, a0, basis3[q * P2 + a]);
        t1 = fmac(t1, a1, basis3[q * P2 + a]);
        dv = fmac(dv, a0, basis3[(Q + q) * P2 + a]);
        dv = fmac(dv, a1, basis3[(2 * Q + q) * P2 + a]);
      }
      const double w = y.w * h;  // h^2 w
      const double ih = 1.0 / h;
      const double d0 = px - y.x[0], d1 = py - y.x[1], d2 = pz - y.x[2];
      const double r2 = fma(d0, d0, fma(d1, d1, d2 * d2));
      const double ir = rsqrt_nr(r2), r = r2 * ir;
      double sn, cs;
      sincos(kre * r, &sn, &cs);
      const double amp = (kim != 0.0 ? exp(kim * r) : 1.0) * kInv4Pi * ir;
      const cd kv{cs * amp, -sn * amp};                      // exp(-i kappa r) / (4 pi r)
      // grad_x: exp(-i kappa r) (-1 - i kappa r) / (4 pi r^3) (x - y), kappa = kre + i kim
      const cd gk = kv * cd{-1.0 + kim * r, -kre * r} * (ir * ir);
      const cd dq = dv * inv_k2 * (ih * ih);
      const double dd[3] = {d0, d1, d2};
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        const cd u = (t0 * y.dx[m] + t1 * y.dy[m]) * ih;
        acc[m] = acc[m] + (kv * u + gk * dq * dd[m]) * w;
      }
    }
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      red[2 * m][threadIdx.x] = acc[m].re;
      red[2 * m + 1][threadIdx.x] = acc[m].im;
    }
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s)
#pragma unroll
        for (int v = 0; v < 6; ++v) red[v][threadIdx.x] += red[v][threadIdx.x + s];
      __syncthreads();
    }
    if (threadIdx.x == 0)
#pragma unroll
      for (int m = 0; m < 3; ++m) out[((long)c * gridDim.x + p) * 3 + m] = cd{red[2 * m][0], red[2 * m + 1][0]};
    __syncthreads();
  }
}

cudaError_t launch_potential_mw(int P, const MwPt* tab, int ne, int Q, double h, const double* basis3,
                                const cd* coef, int k, const double* pts, int npts, double kre, double kim, cd inv_k2,
                                cd* out, cudaStream_t s) {
  switch (P) {
    case 1: k_potential_mw<1><<<npts, 256, 0, s>>>(tab, ne, Q, h, basis3, coef, k, pts, kre, kim, inv_k2, out); break;
    case 2: k_potential_mw<2><<<npts, 256, 0, s>>>(tab, ne, Q, h, basis3, coef, k, pts, kre, kim, inv_k2, out); break;
    case 3: k_potential_mw<3><<<npts, 256, 0, s>>>(tab, ne, Q, h, basis3, coef, k, pts, kre, kim, inv_k2, out); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <int G, int P>
cudaError_t run_load(bool cplx, const PatchTable& pt, const ElementTable& et, int ne, const double* gx,
                     const double* gw, int n1, int kind, const double* prm, int k, double kre, double kim, double* out,
                     cudaStream_t s) {
  const long n = (long)ne * k;
  const unsigned g = (unsigned)((n + 127) / 128);
  if (cplx) k_load<G, P, true><<<g, 128, 0, s>>>(pt, et, ne, gx, gw, n1, kind, prm, k, kre, kim, out);
  else k_load<G, P, false><<<g, 128, 0, s>>>(pt, et, ne, gx, gw, n1, kind, prm, k, kre, kim, out);
  return cudaGetLastError();
}
template <int G>
cudaError_t load_p(int P, bool cplx, const PatchTable& pt, const ElementTable& et, int ne, const double* gx,
                   const double* gw, int n1, int kind, const double* prm, int k, double kre, double kim, double* out,
                   cudaStream_t s) {
  switch (P) {
    case 0: return run_load<G, 0>(cplx, pt, et, ne, gx, gw, n1, kind, prm, k, kre, kim, out, s);
    case 1: return run_load<G, 1>(cplx, pt, et, ne, gx, gw, n1, kind, prm, k, kre, kim, out, s);
    case 2: return run_load<G, 2>(cplx, pt, et, ne, gx, gw, n1, kind, prm, k, kre, kim, out, s);
    case 3: return run_load<G, 3>(cplx, pt, et, ne, gx, gw, n1, kind, prm, k, kre, kim, out, s);
    default: return cudaErrorInvalidValue;
  }
}
cudaError_t launch_load(int G, int P, bool cplx, const PatchTable& pt, const ElementTable& et, int ne,
                        const double* gx, const double* gw, int n1, int kind, const double* prm, int k, double kre,
                        double kim, double* out, cudaStream_t s) {
  switch (G) {
    case 2: return load_p<2>(P, cplx, pt, et, ne, gx, gw, n1, kind, prm, k, kre, kim, out, s);
    case 3: return load_p<3>(P, cplx, pt, et, ne, gx, gw, n1, kind, prm, k, kre, kim, out, s);
    case 4: return load_p<4>(P, cplx, pt, et, ne, gx, gw, n1, kind, prm, k, kre, kim, out, s);
    case 5: return load_p<5>(P, cplx, pt, et, ne, gx, gw, n1, kind, prm, k, kre, kim, out, s);
    case 6: return load_p<6>(P, cplx, pt, et, ne, gx, gw, n1, kind, prm, k, kre, kim, out, s);
    default: return cudaErrorInvalidValue;
  }
}
cudaError_t launch_potential(int P, bool cplx, const d4* tab, int ne, int Q, const double* basis, const double* coef,
                             int k, const double* pts, int npts, double kre, double kim, double* out, cudaStream_t s) {
#define BG_POT(PP)                                                                                              \
  case PP:                                                                                                      \
    if (cplx) k_potential<PP, true><<<npts, 256, 0, s>>>(tab, ne, Q, basis, coef, k, pts, kre, kim, out);      \
    else k_potential<PP, false><<<npts, 256, 0, s>>>(tab, ne, Q, basis, coef, k, pts, kre, kim, out);          \
    break;
  switch (P) {
    BG_POT(0)
    BG_POT(1)
    BG_POT(2)
    BG_POT(3)
    default: return cudaErrorInvalidValue;
  }
#undef BG_POT
  return cudaGetLastError();
}

}  // namespace

extern "C" bg_status bg_load_vector(bg_operator* op, int kind, const double* prm, int nrhs, void* out, int on_device) {
  if (!op || nrhs < 0 || kind < 0 || kind > 3) return BG_INVALID_ARG;
  if (nrhs == 0) return BG_OK;  // no columns
  if (!prm || !out) return BG_INVALID_ARG;
  if (op->ctx->device < 0) return set_error(op->ctx, BG_UNSUPPORTED, "host-only context: load vectors need a GPU");
  if ((op->vd == 2) != (kind == 3))
    return set_error(op->ctx, BG_INVALID_ARG, "the Maxwell operator takes dipole data (kind 3) and only it");
  const int npr = kind == 3 ? 6 : 3;  // parameters per right-hand side
  if (!op->cplx && kind != 0) return set_error(op->ctx, BG_INVALID_ARG, "complex data for a real operator");
  cudaSetDevice(op->ctx->device);
  if (op->kbatched()) {
    // batched wavenumbers: column block q with wavenumber q
    const int nk = (int)op->kslots.size();
    if (nrhs % nk)
      return set_error(op->ctx, BG_INVALID_ARG, "batched wavenumbers: columns must be a multiple of the wavenumbers");
    const int nr = nrhs / nk;
    bg_status st = BG_OK;
    for (int q = 0; q < nk && st == BG_OK; ++q) {
      op->activate_slot(q);
      st = bg_load_vector(op, kind, prm + (size_t)npr * q * nr, nr, static_cast<char*>(out) + (size_t)q * nr * op->N * 16,
                          on_device);
    }
    op->activate_slot(-1);
    return st;
  }
  cudaStream_t s = op->ctx->stream;
  const size_t usz = op->cplx ? 16 : 8;
  const Rule1D& gr = gauss_rule(op->P + 2);
  PatchTable pt{op->d_patch_meta.as<int>(), op->d_patch_cp.as<double>()};
  ElementTable et{op->d_el_patch.as<int>(), op->d_el_llc.as<double>(), 1.0 / double(1 << op->M)};
  for (int c0 = 0; c0 < nrhs; c0 += 32) {
    const int k = std::min(32, nrhs - c0);
    bg_status st = ensure_work(op, k);
    if (st != BG_OK) return st;
    DevBuf gx, gw, dp, dout;
    std::vector<double> p(prm + npr * c0, prm + npr * (c0 + k));
    cudaError_t e = gx.upload(gr.x, s);
    if (e == cudaSuccess) e = gw.upload(gr.w, s);
    if (e == cudaSuccess) e = dp.upload(p, s);
    if (e == cudaSuccess && kind == 3)
      e = launch_load_mw(op->G, op->P, pt, et, op->ne, gx.as<double>(), gw.as<double>(), op->P + 2, dp.as<double>(),
                         k, op->kre, op->kim, op->w_yss.as<cd>(), s);
    else if (e == cudaSuccess)
      e = launch_load(op->G, op->P, op->cplx, pt, et, op->ne, gx.as<double>(), gw.as<double>(), op->P + 2, kind,
                      dp.as<double>(), k, op->kre, op->kim, op->w_yss.as<double>(), s);
    if (e == cudaSuccess)
      e = launch_csr_apply(op->stype(false), op->d_Tt_ptr.as<int>(), op->d_Tt_idx.as<int>(), op->d_Tt_val.as<double>(),
                           op->N, op->w_yss.p, op->w_ydof.p, k, s);
    void* dst = static_cast<char*>(out) + (size_t)c0 * op->N * usz;
    void* dd = dst;
    if (!on_device && e == cudaSuccess) {
      e = dout.alloc((size_t)op->N * k * usz);
      dd = dout.p;
    }
    const double one[2] = {1, 0}, zero2[2] = {0, 0};
    if (e == cudaSuccess) e = launch_scatter_out(op->stype(false), op->w_ydof.p, op->N, k, dd, op->N, one, zero2, s);
    if (!on_device && e == cudaSuccess) e = cudaMemcpyAsync(dst, dd, (size_t)op->N * k * usz, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_status(op->ctx, e, "load vector");
  }
  return BG_OK;
}

// Maxwell: the field (3 complex values per point)
static bg_status potential_mw(bg_operator* op, const void* rho, int nrhs, const double* pts, int npts, void* out) {
  cudaStream_t s = op->ctx->stream;
  const int n1 = op->P + 2, Q = n1 * n1;
  const Rule1D& gr = gauss_rule(n1);
  const std::vector<double> basis3 = basis3_table(op->P, gr);
  PatchTable pt{op->d_patch_meta.as<int>(), op->d_patch_cp.as<double>()};
  const double h = 1.0 / double(1 << op->M);
  ElementTable et{op->d_el_patch.as<int>(), op->d_el_llc.as<double>(), h};
  const std::complex<double> kap(op->kre, op->kim), ik2 = 1.0 / (kap * kap);
  DevBuf gx, gw, tab, dbas, dpts, drho, dout;
  std::vector<double> P3(pts, pts + 3 * npts);
  cudaError_t e = gx.upload(gr.x, s);
  if (e == cudaSuccess) e = gw.upload(gr.w, s);
  if (e == cudaSuccess) e = dbas.upload(basis3, s);
  if (e == cudaSuccess) e = dpts.upload(P3, s);
  if (e == cudaSuccess) e = tab.alloc((size_t)op->ne * Q * sizeof(MwPt));
  if (e == cudaSuccess)
    e = launch_quad_table_mw(op->G, pt, et, op->ne, gx.as<double>(), gw.as<double>(), n1, tab.as<MwPt>(), s);
  if (e != cudaSuccess) return cuda_status(op->ctx, e, "potential setup");
  for (int c0 = 0; c0 < nrhs; c0 += 32) {
    const int k = std::min(32, nrhs - c0);
    bg_status st = ensure_work(op, k);
    if (st != BG_OK) return st;
    e = drho.alloc((size_t)op->N * k * 16);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(drho.p, static_cast<const char*>(rho) + (size_t)c0 * op->N * 16, (size_t)op->N * k * 16,
                          cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = launch_gather_in(1, 1, drho.p, op->N, op->N, k, op->w_xdof.p, s);
    if (e == cudaSuccess)
      e = launch_csr_apply(1, op->d_T_ptr.as<int>(), op->d_T_idx.as<int>(), op->d_T_val.as<double>(), op->S,
                           op->w_xdof.p, op->w_xss.p, k, s);
    if (e == cudaSuccess) e = dout.alloc((size_t)npts * 3 * k * 16);
    if (e == cudaSuccess)
      e = launch_potential_mw(op->P, tab.as<MwPt>(), op->ne, Q, h, dbas.as<double>(), op->w_xss.as<cd>(), k,
                              dpts.as<double>(), npts, op->kre, op->kim, cd{ik2.real(), ik2.imag()},
                              dout.as<cd>(), s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(static_cast<char*>(out) + (size_t)c0 * npts * 3 * 16, dout.p, (size_t)npts * 3 * k * 16,
                          cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_status(op->ctx, e, "potential");
  }
  return BG_OK;
}

extern "C" bg_status bg_potential(bg_operator* op, const void* rho, int nrhs, const double* pts, int npts, void* out) {
  if (!op || nrhs < 0 || npts < 0) return BG_INVALID_ARG;
  if (nrhs == 0 || npts == 0) return BG_OK;  // nothing to evaluate
  if (!rho || !pts || !out) return BG_INVALID_ARG;
  if (op->ctx->device < 0) return set_error(op->ctx, BG_UNSUPPORTED, "host-only context: potentials need a GPU");
  cudaSetDevice(op->ctx->device);
  if (op->kbatched()) {
    // batched wavenumbers: column block q with wavenumber q
    const int nk = (int)op->kslots.size();
    if (nrhs % nk)
      return set_error(op->ctx, BG_INVALID_ARG, "batched wavenumbers: columns must be a multiple of the wavenumbers");
    const int nr = nrhs / nk;
    bg_status st = BG_OK;
    for (int q = 0; q < nk && st == BG_OK; ++q) {
      op->activate_slot(q);
      st = bg_potential(op, static_cast<const char*>(rho) + (size_t)q * nr * op->N * 16, nr, pts, npts,
                        static_cast<char*>(out) + (size_t)q * nr * npts * 16);
    }
    op->activate_slot(-1);
    return st;
  }
  if (op->maxwell()) return potential_mw(op, rho, nrhs, pts, npts, out);
  cudaStream_t s = op->ctx->stream;
  const size_t usz = op->cplx ? 16 : 8;
  const int n1 = op->P + 2, Q = n1 * n1, p2 = op->p2;
  const Rule1D& gr = gauss_rule(n1);
  std::vector<double> basis((size_t)Q * p2);
  for (int q = 0; q < Q; ++q) {
    double bs[8], bt[8];
    bernstein(op->P, gr.x[q / n1], bs);
    bernstein(op->P, gr.x[q % n1], bt);
    for (int iy = 0; iy <= op->P; ++iy)
      for (int ix = 0; ix <= op->P; ++ix) basis[(size_t)q * p2 + iy * (op->P + 1) + ix] = bs[ix] * bt[iy];
  }
  PatchTable pt{op->d_patch_meta.as<int>(), op->d_patch_cp.as<double>()};
  ElementTable et{op->d_el_patch.as<int>(), op->d_el_llc.as<double>(), 1.0 / double(1 << op->M)};
  DevBuf gx, gw, tab, dbas, dpts, drho, dout;
  std::vector<double> P3(pts, pts + 3 * npts);
  cudaError_t e = gx.upload(gr.x, s);
  if (e == cudaSuccess) e = gw.upload(gr.w, s);
  if (e == cudaSuccess) e = dbas.upload(basis, s);
  if (e == cudaSuccess) e = dpts.upload(P3, s);
  if (e == cudaSuccess) e = tab.alloc((size_t)op->ne * Q * sizeof(d4));
  if (e == cudaSuccess) e = launch_quad_table(op->G, pt, et, op->ne, gx.as<double>(), gw.as<double>(), n1, tab.as<d4>(), s);
  if (e != cudaSuccess) return cuda_status(op->ctx, e, "potential setup");
  for (int c0 = 0; c0 < nrhs; c0 += 32) {
    const int k = std::min(32, nrhs - c0);
    bg_status st = ensure_work(op, k);
    if (st != BG_OK) return st;
    e = drho.alloc((size_t)op->N * k * usz);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(drho.p, static_cast<const char*>(rho) + (size_t)c0 * op->N * usz, (size_t)op->N * k * usz,
                          cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = launch_gather_in(op->stype(false), op->stype(false), drho.p, op->N, op->N, k, op->w_xdof.p, s);
    if (e == cudaSuccess)
      e = launch_csr_apply(op->stype(false), op->d_T_ptr.as<int>(), op->d_T_idx.as<int>(), op->d_T_val.as<double>(),
                           op->S, op->w_xdof.p, op->w_xss.p, k, s);
    if (e == cudaSuccess) e = dout.alloc((size_t)npts * k * usz);
    if (e == cudaSuccess)
      e = launch_potential(op->P, op->cplx, tab.as<d4>(), op->ne, Q, dbas.as<double>(), op->w_xss.as<double>(), k,
                           dpts.as<double>(), npts, op->kre, op->kim, dout.as<double>(), s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(static_cast<char*>(out) + (size_t)c0 * npts * usz, dout.p, (size_t)npts * k * usz,
                          cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_status(op->ctx, e, "potential");
  }
  return BG_OK;
}
