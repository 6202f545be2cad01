// Near-field assembly on GB300 (FP64): the element-pair blocks of the dense
// leaves of the H2 matrix (H2Matrix.hpp:163-212 via
// DuffyTrick::evaluateBilinearForm, evaluateBilinearForm.hpp:21-71).
//
// Regular pairs (integrate0 / integrate1) use per-element tables of surface
// points at the Gauss nodes, shared by every pair that needs the same degree,
// and the factorisation  I = U diag(c1) K diag(c2) U^T  of the tensor
// quadrature: per pair only the kernel matrix K is evaluated.
// Singular pairs (integrate2/3/4) evaluate the Duffy-transformed points on the
// fly; each warp owns one outer Gauss point and its lanes sweep the inner
// points, and the (p^2 x p^2) accumulator is distributed over the lanes.
#include <cstdio>

#include "bg_kernels.cuh"

namespace bg {

constexpr double kInv4Pi = 0.07957747154594767;  // 1 / (4 pi)

// Laplace 1/(4 pi r) and Helmholtz exp(-i k r)/(4 pi r) from r^2
// (Laplace/SingleLayerOperator.hpp:115-118, Helmholtz/SingleLayerOperator.hpp:115-120)
template <typename S>
__device__ inline S kernel_val(double r2, double kre, double kim);
template <>
__device__ inline double kernel_val<double>(double r2, double, double) {
  return rsqrt_nr(r2) * kInv4Pi;
}
template <>
__device__ inline cd kernel_val<cd>(double r2, double kre, double kim) {
  double inv = rsqrt_nr(r2);
  double r = r2 * inv;
  double sn, cs;
  sincos(kre * r, &sn, &cs);
  double amp = inv * kInv4Pi;
  if (kim != 0.0) amp *= exp(kim * r);
  return {cs * amp, -sn * amp};
}

__device__ inline double scale_of(double v, double s) { return v * s; }
__device__ inline cd scale_of(cd v, double s) { return v * s; }

// ---------------------------------------------------------------------------
template <int G>
__global__ void k_quad_table(PatchTable pt, ElementTable et, int ne, const double* __restrict__ gx,
                             const double* __restrict__ gw, int n1, d4* __restrict__ out) {
  const int Q = n1 * n1;
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long)ne * Q) return;
  const int e = (int)(idx / Q), q = (int)(idx % Q);
  const double u = gx[q / n1], v = gx[q % n1], w = gw[q / n1] * gw[q % n1];
  const double h = et.h;
  double x[3], dx[3], dy[3];
  surface_frame<G>(pt, et.patch[e], et.llc[2 * e] + h * u, et.llc[2 * e + 1] + h * v, x, dx, dy);
  out[idx] = d4{x[0], x[1], x[2], h * w * surface_measure(dx, dy)};
}

cudaError_t launch_quad_table(int G, const PatchTable& pt, const ElementTable& et, int ne, const double* gx,
                              const double* gw, int n1, d4* out, cudaStream_t s) {
  const long n = (long)ne * n1 * n1;
  const int bs = 128;
  const unsigned grid = (unsigned)((n + bs - 1) / bs);
  switch (G) {
    case 2: k_quad_table<2><<<grid, bs, 0, s>>>(pt, et, ne, gx, gw, n1, out); break;
    case 3: k_quad_table<3><<<grid, bs, 0, s>>>(pt, et, ne, gx, gw, n1, out); break;
    case 4: k_quad_table<4><<<grid, bs, 0, s>>>(pt, et, ne, gx, gw, n1, out); break;
    case 5: k_quad_table<5><<<grid, bs, 0, s>>>(pt, et, ne, gx, gw, n1, out); break;
    case 6: k_quad_table<6><<<grid, bs, 0, s>>>(pt, et, ne, gx, gw, n1, out); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Regular pairs. One CTA per pair. Phase 1: thread per Gauss point i of e1
// computes W_i[b] = sum_j k(x_i, y_j) c_j phi_b(y_j). Phase 2: thread per
// entry (a, b) sums c_i phi_a(x_i) W_i[b] over i.
template <int P, typename S>
__global__ void __launch_bounds__(128) k_near_regular(const NearPair* __restrict__ pairs, const d4* __restrict__ tab,
                                                      int n1, const double* __restrict__ basis, double kre, double kim,
                                                      S* __restrict__ out, int B) {
  constexpr int P2 = (P + 1) * (P + 1);
  const int Q = n1 * n1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  d4* ys = reinterpret_cast<d4*>(smem_raw);
  double* U = reinterpret_cast<double*>(ys + Q);
  double* ci = U + Q * P2;
  S* W = reinterpret_cast<S*>(ci + Q);
  const NearPair pr = pairs[blockIdx.x];
  for (int q = threadIdx.x; q < Q; q += blockDim.x) ys[q] = tab[(long)pr.e2 * Q + q];
  for (int k = threadIdx.x; k < Q * P2; k += blockDim.x) U[k] = basis[k];
  __syncthreads();
  for (int i = threadIdx.x; i < Q; i += blockDim.x) {
    const d4 xi = tab[(long)pr.e1 * Q + i];
    S w[P2];
#pragma unroll
    for (int b = 0; b < P2; ++b) w[b] = zero<S>();
    for (int j = 0; j < Q; ++j) {
      const d4 yj = ys[j];
      const double d0 = xi.x - yj.x, d1 = xi.y - yj.y, d2 = xi.z - yj.z;
      const double r2 = fma(d0, d0, fma(d1, d1, d2 * d2));
      const S kv = scale_of(kernel_val<S>(r2, kre, kim), yj.w);
#pragma unroll
      for (int b = 0; b < P2; ++b) w[b] = fmac(w[b], kv, U[j * P2 + b]);
    }
#pragma unroll
    for (int b = 0; b < P2; ++b) W[i * P2 + b] = w[b];
    ci[i] = xi.w;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < P2 * P2; e += blockDim.x) {
    const int a = e % P2, b = e / P2;
    S acc = zero<S>();
    for (int i = 0; i < Q; ++i) acc = fmac(acc, W[i * P2 + b], ci[i] * U[i * P2 + a]);
    out[pr.dst + (long)b * B + a] = acc;
  }
}

template <int P, typename S>
static cudaError_t run_regular(const NearPair* pairs, int npairs, const d4* tab, int n1, const double* basis,
                               double kre, double kim, S* out, int B, cudaStream_t s) {
  constexpr int P2 = (P + 1) * (P + 1);
  const int Q = n1 * n1;
  size_t smem = Q * sizeof(d4) + Q * P2 * sizeof(double) + Q * sizeof(double) + Q * P2 * sizeof(S);
  if (smem > 200 * 1024) return cudaErrorInvalidConfiguration;
  auto kfn = k_near_regular<P, S>;
  cudaError_t err = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return err;
  if (npairs == 0) return cudaSuccess;
  kfn<<<npairs, 128, smem, s>>>(pairs, tab, n1, basis, kre, kim, out, B);
  return cudaGetLastError();
}

cudaError_t launch_near_regular(int P, bool cplx, const NearPair* pairs, int npairs, const d4* tab, int n1,
                                const double* basis, double kre, double kim, void* out, int B, cudaStream_t s) {
#define BG_REG(PP)                                                                                          \
  case PP:                                                                                                  \
    return cplx ? run_regular<PP, cd>(pairs, npairs, tab, n1, basis, kre, kim, static_cast<cd*>(out), B, s) \
                : run_regular<PP, double>(pairs, npairs, tab, n1, basis, kre, kim, static_cast<double*>(out), B, s);
  switch (P) {
    BG_REG(0)
    BG_REG(1)
    BG_REG(2)
    BG_REG(3)
    default: return cudaErrorInvalidValue;
  }
#undef BG_REG
}

// ---------------------------------------------------------------------------
// Singular pairs.
struct PointEval {
  double x[3];
  double c;  // quadrature weight times surface measure
};

template <int G, int P>
__device__ inline void eval_point(const PatchTable& pt, int patch, double l0, double l1, double h, double u, double v,
                                  double w, PointEval* pe, double* phi) {
  double dx[3], dy[3];
  surface_frame<G>(pt, patch, l0 + h * u, l1 + h * v, pe->x, dx, dy);
  pe->c = w * surface_measure(dx, dy);
  tensor_basis<P>(u, v, phi);
}

template <int P, typename S>
struct WarpAcc {
  static constexpr int P2 = (P + 1) * (P + 1);
  static constexpr int NE = P2 * P2;
  static constexpr int PER = (NE + 31) / 32;
  S acc[PER];
  __device__ void init() {
#pragma unroll
    for (int m = 0; m < PER; ++m) acc[m] = zero<S>();
  }
  // add the 32 staged samples c_s phi_a(s) phi_b(s) (+ transposed when sym)
  __device__ void add(const S* sc, const double* sa, const double* sb, bool sym, int lane) {
    for (int s = 0; s < 32; ++s) {
      const S c = sc[s];
#pragma unroll
      for (int m = 0; m < PER; ++m) {
        const int e = lane + 32 * m;
        if (e < NE) {
          const int a = e % P2, b = e / P2;
          double v = sa[s * P2 + a] * sb[s * P2 + b];
          if (sym) v = fma(sb[s * P2 + a], sa[s * P2 + b], v);
          acc[m] = fmac(acc[m], c, v);
        }
      }
    }
  }
};

template <int G, int P, typename S, int CS>
__global__ void __launch_bounds__(128) k_near_duffy(PatchTable pt, ElementTable et, const NearPair* __restrict__ pairs,
                                                    const double* __restrict__ gx, const double* __restrict__ gw, int n1,
                                                    double kre, double kim, S* __restrict__ out, int B) {
  constexpr int P2 = (P + 1) * (P + 1);
  constexpr int NE = P2 * P2;
  constexpr int NW = 4;
  __shared__ S st_c[NW][32];
  __shared__ double st_a[NW][32 * P2];
  __shared__ double st_b[NW][32 * P2];
  __shared__ PointEval vp[NW][4];        // per-i points of the common-vertex rule
  __shared__ double vphi[NW][4][P2];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const NearPair pr = pairs[blockIdx.x];
  const int rot1 = pr.rot & 15, rot2 = pr.rot >> 4;
  const int p1 = et.patch[pr.e1], p2 = et.patch[pr.e2];
  const double a0 = et.llc[2 * pr.e1], a1 = et.llc[2 * pr.e1 + 1];
  const double b0 = et.llc[2 * pr.e2], b1 = et.llc[2 * pr.e2 + 1];
  const double h = et.h;
  const int Q = n1 * n1;
  WarpAcc<P, S> acc;
  acc.init();
  S* sc = st_c[warp];
  double* sa = st_a[warp];
  double* sb = st_b[warp];
  for (int i = warp; i < Q; i += NW) {
    const double x0 = gx[i / n1], x1 = gx[i % n1], wi = gw[i / n1] * gw[i % n1];
    double w = 0;
    if (CS == 2) w = h * h * wi * x0 * (1 - x0) * (1 - x0 * x1);
    if (CS == 3) w = h * h * wi * x1 * x1;
    if (CS == 4) {
      w = h * h * wi * (x0 * x0 * x0);
      const double y1 = x1 * x0;
      if (lane < 4) {
        double uv[2];
        const int r = (lane < 2) ? rot1 : rot2;
        if (lane == 0 || lane == 2) tau(x0, y1, r, uv); else tau(y1, x0, r, uv);
        if (lane < 2) eval_point<G, P>(pt, p1, a0, a1, h, uv[0], uv[1], w, &vp[warp][lane], vphi[warp][lane]);
        else eval_point<G, P>(pt, p2, b0, b1, h, uv[0], uv[1], w, &vp[warp][lane], vphi[warp][lane]);
      }
      __syncwarp();
    }
    for (int jj = 0; jj < Q; jj += 32) {
      const int j = jj + lane;
      const bool valid = j < Q;
      const double e0 = valid ? gx[j / n1] : 0.5, e1 = valid ? gx[j % n1] : 0.5;
      const double wj = valid ? gw[j / n1] * gw[j % n1] : 0.0;
      constexpr int NK = CS == 2 ? 4 : (CS == 3 ? 6 : 4);
      // common-vertex: the inner points are shared by the four samples
      PointEval q5, q6;
      double phi5[P2], phi6[P2];
      if (CS == 4) {
        double uv[2];
        tau(x0 * e0, x0 * e1, rot2, uv);
        eval_point<G, P>(pt, p2, b0, b1, h, uv[0], uv[1], wj, &q5, phi5);
        tau(x0 * e0, x0 * e1, rot1, uv);
        eval_point<G, P>(pt, p1, a0, a1, h, uv[0], uv[1], wj, &q6, phi6);
      }
#pragma unroll 1
      for (int k = 0; k < NK; ++k) {
        PointEval A, Bp;
        double* pa = sa + lane * P2;
        double* pb = sb + lane * P2;
        if (CS == 2) {
          // integrate2.hpp:41-60: point pairs of the identical-element rule
          const double t1 = e0 * (1 - x0), t2 = e1 * (1 - x0 * x1);
          const double t3 = e0 * (1 - x0) + x0, t4 = e1 * (1 - x0 * x1) + x0 * x1;
          double u1, v1, u2, v2;
          if (k == 0) { u1 = t1; v1 = t2; u2 = t3; v2 = t4; }
          else if (k == 1) { u1 = t1; v1 = t4; u2 = t3; v2 = t2; }
          else if (k == 2) { u1 = t2; v1 = t1; u2 = t4; v2 = t3; }
          else { u1 = t2; v1 = t3; u2 = t4; v2 = t1; }
          eval_point<G, P>(pt, p1, a0, a1, h, u1, v1, w, &A, pa);
          eval_point<G, P>(pt, p1, a0, a1, h, u2, v2, wj, &Bp, pb);
        } else if (CS == 3) {
          // integrate3.hpp:45-76: six point pairs of the common-edge rule
          const double f0 = x1 * e0, f1 = x1 * e1;
          const double t1 = x0 * (1 - x1), t2 = (1 - x0) * (1 - x1);
          const double t3 = x0 * (1 - f0), t4 = (1 - x0) * (1 - f0);
          double ua, va, ub, vb, wb;
          if (k == 0) { ua = t1; va = f0; ub = t2; vb = f1; wb = wj * (1 - x1); }
          else if (k == 1) { ua = 1 - t1; va = f0; ub = 1 - t2; vb = f1; wb = wj * (1 - x1); }
          else if (k == 2) { ua = t3; va = x1; ub = t4; vb = f1; wb = wj * (1 - f0); }
          else if (k == 3) { ua = 1 - t3; va = x1; ub = 1 - t4; vb = f1; wb = wj * (1 - f0); }
          else if (k == 4) { ua = t4; va = f1; ub = t3; vb = x1; wb = wj * (1 - f0); }
          else { ua = 1 - t4; va = f1; ub = 1 - t3; vb = x1; wb = wj * (1 - f0); }
          double uv1[2], uv2[2];
          tau(ua, va, rot1, uv1);
          tau(ub, vb, rot2, uv2);
          eval_point<G, P>(pt, p1, a0, a1, h, uv1[0], uv1[1], w, &A, pa);
          eval_point<G, P>(pt, p2, b0, b1, h, uv2[0], uv2[1], wb, &Bp, pb);
        } else {
          // integrate4.hpp:49-58: (qp1,qp5), (qp2,qp5), (qp6,qp3), (qp6,qp4)
          const PointEval* v = vp[warp];
          if (k < 2) {
            A = v[k];
            Bp = q5;
#pragma unroll
            for (int t = 0; t < P2; ++t) { pa[t] = vphi[warp][k][t]; pb[t] = phi5[t]; }
          } else {
            A = q6;
            Bp = v[k];
#pragma unroll
            for (int t = 0; t < P2; ++t) { pa[t] = phi6[t]; pb[t] = vphi[warp][k][t]; }
          }
        }
        const double d0 = A.x[0] - Bp.x[0], d1 = A.x[1] - Bp.x[1], d2 = A.x[2] - Bp.x[2];
        const double r2 = fma(d0, d0, fma(d1, d1, d2 * d2));
        S c = scale_of(kernel_val<S>(r2, kre, kim), A.c * Bp.c);
        if (!valid) c = zero<S>();
        sc[lane] = c;
        __syncwarp();
        acc.add(sc, sa, sb, CS == 2, lane);
        __syncwarp();
      }
    }
    if (CS == 4) __syncwarp();
  }
  // reduce the warps' accumulators (staging memory reused: NE * sizeof(S)
  // <= 32 * P2 * sizeof(double) for P <= 3) and write the block
  static_assert(NE * sizeof(S) <= 32 * P2 * sizeof(double), "reduction buffer too small");
  __syncthreads();
  S* red = reinterpret_cast<S*>(&st_a[0][0]);
  const int stride = 32 * P2 * sizeof(double) / sizeof(S);
#pragma unroll
  for (int m = 0; m < WarpAcc<P, S>::PER; ++m) {
    const int e = lane + 32 * m;
    if (e < NE) red[warp * stride + e] = acc.acc[m];
  }
  __syncthreads();
  for (int e = threadIdx.x; e < NE; e += blockDim.x) {
    S v = red[e];
#pragma unroll
    for (int w2 = 1; w2 < NW; ++w2) v = v + red[w2 * stride + e];
    const int a = e % P2, b = e / P2;
    out[pr.dst + (long)b * B + a] = v;
  }
}

template <int G, int P, typename S>
static cudaError_t run_duffy(int cs, const PatchTable& pt, const ElementTable& et, const NearPair* pairs, int npairs,
                             const double* gx, const double* gw, int n1, double kre, double kim, S* out, int B,
                             cudaStream_t s) {
  if (npairs == 0) return cudaSuccess;
  if (cs == 2) k_near_duffy<G, P, S, 2><<<npairs, 128, 0, s>>>(pt, et, pairs, gx, gw, n1, kre, kim, out, B);
  else if (cs == 3) k_near_duffy<G, P, S, 3><<<npairs, 128, 0, s>>>(pt, et, pairs, gx, gw, n1, kre, kim, out, B);
  else if (cs == 4) k_near_duffy<G, P, S, 4><<<npairs, 128, 0, s>>>(pt, et, pairs, gx, gw, n1, kre, kim, out, B);
  else return cudaErrorInvalidValue;
  return cudaGetLastError();
}

template <int G>
static cudaError_t duffy_p(int P, bool cplx, int cs, const PatchTable& pt, const ElementTable& et,
                           const NearPair* pairs, int npairs, const double* gx, const double* gw, int n1, double kre,
                           double kim, void* out, int B, cudaStream_t s) {
#define BG_DUF(PP)                                                                                               \
  case PP:                                                                                                       \
    return cplx ? run_duffy<G, PP, cd>(cs, pt, et, pairs, npairs, gx, gw, n1, kre, kim, static_cast<cd*>(out), B, s) \
                : run_duffy<G, PP, double>(cs, pt, et, pairs, npairs, gx, gw, n1, kre, kim,                      \
                                           static_cast<double*>(out), B, s);
  switch (P) {
    BG_DUF(0)
    BG_DUF(1)
    BG_DUF(2)
    BG_DUF(3)
    default: return cudaErrorInvalidValue;
  }
#undef BG_DUF
}

cudaError_t launch_near_duffy(int G, int P, bool cplx, int cs, const PatchTable& pt, const ElementTable& et,
                              const NearPair* pairs, int npairs, const double* gx, const double* gw, int n1,
                              double kre, double kim, void* out, int B, cudaStream_t s) {
  switch (G) {
    case 2: return duffy_p<2>(P, cplx, cs, pt, et, pairs, npairs, gx, gw, n1, kre, kim, out, B, s);
    case 3: return duffy_p<3>(P, cplx, cs, pt, et, pairs, npairs, gx, gw, n1, kre, kim, out, B, s);
    case 5: return duffy_p<5>(P, cplx, cs, pt, et, pairs, npairs, gx, gw, n1, kre, kim, out, B, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace bg
