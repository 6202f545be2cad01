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
  cudaError_t err = smem_limit(kfn, smem);
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
  // NK accumulators at once: acc[k] += c_k(s) phi_a(s) phi_b(s) for the 32
  // staged samples, sc[k * 32 + s] (the basis products are formed once)
  template <int NK>
  static __device__ void add_multi(WarpAcc* acc, const S* sc, const double* sa, const double* sb, bool sym,
                                   int lane) {
    for (int s = 0; s < 32; ++s) {
#pragma unroll
      for (int m = 0; m < PER; ++m) {
        const int e = lane + 32 * m;
        if (e < NE) {
          const int a = e % P2, b = e / P2;
          double v = sa[s * P2 + a] * sb[s * P2 + b];
          if (sym) v = fma(sb[s * P2 + a], sa[s * P2 + b], v);
#pragma unroll
          for (int k = 0; k < NK; ++k) acc[k].acc[m] = fmac(acc[k].acc[m], sc[k * 32 + s], v);
        }
      }
    }
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

// Several wavenumbers per launch (KBatch, NK of them): every Duffy sample's
// points, surface measures and basis values are evaluated once and shared;
// each wavenumber has its own kernel values, accumulators and output.
template <typename S, int NK>
struct KBatch {
  double kre[NK], kim[NK];
  S* out[NK];
};

template <int G, int P, typename S, int CS, int NK>
__global__ void __launch_bounds__(128) k_near_duffy(PatchTable pt, ElementTable et, const NearPair* __restrict__ pairs,
                                                    const double* __restrict__ gx, const double* __restrict__ gw, int n1,
                                                    KBatch<S, NK> kb, int B) {
  constexpr int P2 = (P + 1) * (P + 1);
  constexpr int NE = P2 * P2;
  constexpr int NW = 4;
  __shared__ S st_c[NW][NK * 32];
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
  WarpAcc<P, S> acc[NK];
#pragma unroll
  for (int k = 0; k < NK; ++k) acc[k].init();
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
      constexpr int NSUB = CS == 2 ? 4 : (CS == 3 ? 6 : 4);  // point pairs per (outer, inner) sample
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
      for (int k = 0; k < NSUB; ++k) {
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
#pragma unroll
        for (int q = 0; q < NK; ++q) {
          S c = scale_of(kernel_val<S>(r2, kb.kre[q], kb.kim[q]), A.c * Bp.c);
          if (!valid) c = zero<S>();
          sc[q * 32 + lane] = c;
        }
        __syncwarp();
        if (NK == 1) acc[0].add(sc, sa, sb, CS == 2, lane);
        else WarpAcc<P, S>::template add_multi<NK>(acc, sc, sa, sb, CS == 2, lane);
        __syncwarp();
      }
    }
    if (CS == 4) __syncwarp();
  }
  // reduce the warps' accumulators (staging memory reused: NE * sizeof(S)
  // <= 32 * P2 * sizeof(double) for P <= 3) and write the block
  static_assert(NE * sizeof(S) <= 32 * P2 * sizeof(double), "reduction buffer too small");
  S* red = reinterpret_cast<S*>(&st_a[0][0]);
  const int stride = 32 * P2 * sizeof(double) / sizeof(S);
#pragma unroll
  for (int q = 0; q < NK; ++q) {
    __syncthreads();
#pragma unroll
    for (int m = 0; m < WarpAcc<P, S>::PER; ++m) {
      const int e = lane + 32 * m;
      if (e < NE) red[warp * stride + e] = acc[q].acc[m];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < NE; e += blockDim.x) {
      S v = red[e];
#pragma unroll
      for (int w2 = 1; w2 < NW; ++w2) v = v + red[w2 * stride + e];
      const int a = e % P2, b = e / P2;
      kb.out[q][pr.dst + (long)b * B + a] = v;
    }
  }
}

// ---------------------------------------------------------------------------
// Common-edge and common-vertex pairs with the inner sum factorised (one
// wavenumber per launch, P <= 2, n1 <= 16).
//
// Common edge (integrate3.hpp:45-76): with outer node (x0, x1) and inner
// node (e0, e1), every one of the six point pairs has one point that does not
// depend on e1: sub-rules 0-3 the point on the first element, ((1 -) x0 (1 -
// x1), x1 e0) and ((1 -) x0 (1 - x1 e0), x1), sub-rules 4, 5 the point on the
// second, ((1 -) x0 (1 - x1 e0), x1). So each sub-rule's contribution is
//   sum_e0 phi(fixed(e0)) (x) [sum_e1 c(e0, e1) phi(varying(e0, e1))],
// a rank-one update per (outer node, e0, sub-rule) instead of one per sample:
// one fixed point evaluation and one basis outer product per n1 samples. In
// sub-rules 0, 1 the varying point depends on e1 alone and is evaluated once
// per outer node (a per-warp cache). The weights are split the same way: the
// fixed point carries the outer weight, the e0 weight and the (1 - x1) or
// (1 - x1 e0) factor, the varying point the e1 weight.
// Common vertex (integrate4.hpp:49-58): the four pairs are (qp1, qp5), (qp2,
// qp5), (qp6, qp3), (qp6, qp4), where qp1-qp4 depend on the outer node only;
// so sum_j c_k(j) phi(qp5 or qp6 at j) is accumulated per lane over all inner
// nodes and each outer node ends with four rank-one updates.
// The sums are the reference's in another order: leaf blocks agree with the
// per-sample kernel to rounding.
constexpr int kEdgeNW = 4;

__device__ inline double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ inline cd warp_sum(cd v) { return {warp_sum(v.re), warp_sum(v.im)}; }
__device__ inline double shfl_xor(double v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ inline cd shfl_xor(cd v, int o) { return {shfl_xor(v.re, o), shfl_xor(v.im, o)}; }

template <int P, typename S>
struct RankOneStage {
  static constexpr int P2 = (P + 1) * (P + 1);
  double f[kEdgeNW][32 * P2];  // basis values of the fixed point per lane
  S v[kEdgeNW][32 * P2];       // inner sums per lane
  int o[kEdgeNW][32];          // 0: fixed point on the first element (rows), 1: on the second (columns)
};

// acc(a, b) += f_s(a) v_s(b) (o = 0) or v_s(a) f_s(b) (o = 1) for the 32
// staged lanes s of this warp; the p^2 x p^2 block is distributed over the
// lanes, entry lane + 32 m.
template <int P, typename S, int PER>
__device__ inline void add_rank_one(S* acc, const RankOneStage<P, S>& st, int warp, int lane) {
  constexpr int P2 = (P + 1) * (P + 1);
  constexpr int NE = P2 * P2;
  for (int s = 0; s < 32; ++s) {
    const int o = st.o[warp][s];
    const double* f = &st.f[warp][s * P2];
    const S* v = &st.v[warp][s * P2];
#pragma unroll
    for (int m = 0; m < PER; ++m) {
      const int e = lane + 32 * m;
      if (e < NE) {
        const int a = e % P2, b = e / P2;
        acc[m] = o ? fmac(acc[m], v[a], f[b]) : fmac(acc[m], v[b], f[a]);
      }
    }
  }
}

template <int P, typename S>
__device__ inline void stage_rank_one(RankOneStage<P, S>& st, int warp, int lane, bool act, int o, const double* f,
                                      const S* v) {
  constexpr int P2 = (P + 1) * (P + 1);
  st.o[warp][lane] = act ? o : 0;
#pragma unroll
  for (int t = 0; t < P2; ++t) {
    st.f[warp][lane * P2 + t] = act ? f[t] : 0.0;
    st.v[warp][lane * P2 + t] = act ? v[t] : zero<S>();
  }
}

// sum the warps' accumulators (staging memory reused) and write the block
template <int P, typename S, int PER>
__device__ inline void write_block(S* acc, RankOneStage<P, S>& st, int warp, int lane, S* out, long long dst, int B) {
  constexpr int P2 = (P + 1) * (P + 1);
  constexpr int NE = P2 * P2;
  static_assert(NE <= 32 * P2, "reduction buffer too small");
  S* red = &st.v[0][0];
  __syncthreads();
#pragma unroll
  for (int m = 0; m < PER; ++m) {
    const int e = lane + 32 * m;
    if (e < NE) red[warp * 32 * P2 + e] = acc[m];
  }
  __syncthreads();
  for (int e = threadIdx.x; e < NE; e += blockDim.x) {
    S v = red[e];
#pragma unroll
    for (int w2 = 1; w2 < kEdgeNW; ++w2) v = v + red[w2 * 32 * P2 + e];
    out[dst + (long)(e / P2) * B + e % P2] = v;
  }
}

template <int G, int P, typename S>
__global__ void __launch_bounds__(128) k_near_edge(PatchTable pt, ElementTable et, const NearPair* __restrict__ pairs,
                                                   const double* __restrict__ gx, const double* __restrict__ gw,
                                                   int n1, double kre, double kim, S* __restrict__ out, int B) {
  constexpr int P2 = (P + 1) * (P + 1);
  constexpr int NE = P2 * P2;
  constexpr int PER = (NE + 31) / 32;
  __shared__ RankOneStage<P, S> st;
  __shared__ PointEval cpt[kEdgeNW][32];  // sub-rules 0, 1: the e1-only points on the second element
  __shared__ double cphi[kEdgeNW][32 * P2];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const NearPair pr = pairs[blockIdx.x];
  const int rot1 = pr.rot & 15, rot2 = pr.rot >> 4;
  const int p1 = et.patch[pr.e1], p2 = et.patch[pr.e2];
  const double a0 = et.llc[2 * pr.e1], a1 = et.llc[2 * pr.e1 + 1];
  const double b0 = et.llc[2 * pr.e2], b1 = et.llc[2 * pr.e2 + 1];
  const double h = et.h;
  const int Q = n1 * n1;
  S acc[PER];
#pragma unroll
  for (int m = 0; m < PER; ++m) acc[m] = zero<S>();
  // sub-rules 0, 1: a warp per outer node; lane = (sub-rule, e0 node) for the
  // fixed point, cache lane = (sub-rule, e1 node) for the varying one
  for (int i = warp; i < Q; i += kEdgeNW) {
    const double x0 = gx[i / n1], x1 = gx[i % n1], wi = gw[i / n1] * gw[i % n1];
    const double w = h * h * wi * x1 * x1;
    const double t1 = x0 * (1 - x1), t2 = (1 - x0) * (1 - x1);
    const bool act = lane < 2 * n1;
    const int k = act ? lane / n1 : 0, m0 = act ? lane % n1 : 0;
    double uv[2];
    if (act) {
      tau(k ? 1 - t2 : t2, x1 * gx[m0], rot2, uv);
      eval_point<G, P>(pt, p2, b0, b1, h, uv[0], uv[1], gw[m0], &cpt[warp][lane], &cphi[warp][lane * P2]);
    }
    __syncwarp();
    tau(k ? 1 - t1 : t1, x1 * gx[m0], rot1, uv);
    PointEval F;
    double phF[P2];
    eval_point<G, P>(pt, p1, a0, a1, h, uv[0], uv[1], w * gw[m0] * (1 - x1), &F, phF);
    S v[P2];
#pragma unroll
    for (int t = 0; t < P2; ++t) v[t] = zero<S>();
    if (act) {
      for (int m = 0; m < n1; ++m) {
        const PointEval& V = cpt[warp][k * n1 + m];
        const double d0 = F.x[0] - V.x[0], d1 = F.x[1] - V.x[1], d2 = F.x[2] - V.x[2];
        const S c = scale_of(kernel_val<S>(fma(d0, d0, fma(d1, d1, d2 * d2)), kre, kim), F.c * V.c);
        const double* ph = &cphi[warp][(k * n1 + m) * P2];
#pragma unroll
        for (int t = 0; t < P2; ++t) v[t] = fmac(v[t], c, ph[t]);
      }
    }
    stage_rank_one<P, S>(st, warp, lane, act, 0, phF, v);
    __syncwarp();
    add_rank_one<P, S, PER>(acc, st, warp, lane);
    __syncwarp();
  }
  // sub-rules 2-5: units (outer node, e0 node, sub-rule) over all threads
  const int U = Q * n1 * 4;
  for (int base = 0; base < U; base += blockDim.x) {
    const int u = base + threadIdx.x;
    const bool act = u < U;
    const int uu = act ? u : 0;
    const int i = uu / (4 * n1), rem = uu % (4 * n1), m0 = rem >> 2, k = (rem & 3) + 2;
    const double x0 = gx[i / n1], x1 = gx[i % n1], wi = gw[i / n1] * gw[i % n1];
    const double w = h * h * wi * x1 * x1;
    const double f0 = x1 * gx[m0];
    const double t3 = x0 * (1 - f0), t4 = (1 - x0) * (1 - f0);
    // sub-rules 2, 3: fixed on the first element at ((1 -) t3, x1), varying on
    // the second at ((1 -) t4, x1 e1); sub-rules 4, 5: the other way round
    const bool flip = k & 1, onA = k < 4;
    const int pf = onA ? p1 : p2, pv = onA ? p2 : p1, rf = onA ? rot1 : rot2, rv = onA ? rot2 : rot1;
    const double lf0 = onA ? a0 : b0, lf1 = onA ? a1 : b1, lv0 = onA ? b0 : a0, lv1 = onA ? b1 : a1;
    const double vt = flip ? 1 - t4 : t4;
    double uv[2];
    tau(flip ? 1 - t3 : t3, x1, rf, uv);
    PointEval F;
    double phF[P2];
    eval_point<G, P>(pt, pf, lf0, lf1, h, uv[0], uv[1], w * gw[m0] * (1 - f0), &F, phF);
    // the varying points (vt, x1 e1) lie on one line of the patch: rotations
    // 1 and 3 fix the patch's t, the others its s
    const bool fs = !(rv == 1 || rv == 3);
    tau(vt, 0.0, rv, uv);
    SurfaceLine<G> line;
    surface_line<G>(pt, pv, fs, fs ? lv0 + h * uv[0] : lv1 + h * uv[1], line);
    S v[P2];
#pragma unroll
    for (int t = 0; t < P2; ++t) v[t] = zero<S>();
    for (int m = 0; m < n1; ++m) {
      tau(vt, x1 * gx[m], rv, uv);
      PointEval V;
      double phV[P2];
      {
        double dx[3], dy[3];
        surface_line_point<G>(line, fs ? lv1 + h * uv[1] : lv0 + h * uv[0], V.x, dx, dy);
        V.c = gw[m] * surface_measure(dx, dy);
        tensor_basis<P>(uv[0], uv[1], phV);
      }
      const double d0 = F.x[0] - V.x[0], d1 = F.x[1] - V.x[1], d2 = F.x[2] - V.x[2];
      const S c = scale_of(kernel_val<S>(fma(d0, d0, fma(d1, d1, d2 * d2)), kre, kim), F.c * V.c);
#pragma unroll
      for (int t = 0; t < P2; ++t) v[t] = fmac(v[t], c, phV[t]);
    }
    stage_rank_one<P, S>(st, warp, lane, act, onA ? 0 : 1, phF, v);
    __syncwarp();
    add_rank_one<P, S, PER>(acc, st, warp, lane);
    __syncwarp();
  }
  write_block<P, S, PER>(acc, st, warp, lane, out, pr.dst, B);
}

template <int G, int P, typename S>
__global__ void __launch_bounds__(128) k_near_vertex(PatchTable pt, ElementTable et, const NearPair* __restrict__ pairs,
                                                     const double* __restrict__ gx, const double* __restrict__ gw,
                                                     int n1, double kre, double kim, S* __restrict__ out, int B) {
  constexpr int P2 = (P + 1) * (P + 1);
  constexpr int NE = P2 * P2;
  constexpr int PER = (NE + 31) / 32;
  __shared__ RankOneStage<P, S> st;  // only st.v (inner sums of the 4 pairs) and the final reduction
  __shared__ PointEval vp[kEdgeNW][4];
  __shared__ double vphi[kEdgeNW][4 * P2];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const NearPair pr = pairs[blockIdx.x];
  const int rot1 = pr.rot & 15, rot2 = pr.rot >> 4;
  const int p1 = et.patch[pr.e1], p2 = et.patch[pr.e2];
  const double a0 = et.llc[2 * pr.e1], a1 = et.llc[2 * pr.e1 + 1];
  const double b0 = et.llc[2 * pr.e2], b1 = et.llc[2 * pr.e2 + 1];
  const double h = et.h;
  const int Q = n1 * n1;
  S acc[PER];
#pragma unroll
  for (int m = 0; m < PER; ++m) acc[m] = zero<S>();
  S* sv = &st.v[warp][0];
  for (int i = warp; i < Q; i += kEdgeNW) {
    const double x0 = gx[i / n1], x1 = gx[i % n1], wi = gw[i / n1] * gw[i % n1];
    const double w = h * h * wi * (x0 * x0 * x0);
    const double y1 = x1 * x0;
    if (lane < 4) {
      double uv[2];
      const int r = (lane < 2) ? rot1 : rot2;
      if (lane == 0 || lane == 2) tau(x0, y1, r, uv); else tau(y1, x0, r, uv);
      if (lane < 2) eval_point<G, P>(pt, p1, a0, a1, h, uv[0], uv[1], w, &vp[warp][lane], &vphi[warp][lane * P2]);
      else eval_point<G, P>(pt, p2, b0, b1, h, uv[0], uv[1], w, &vp[warp][lane], &vphi[warp][lane * P2]);
    }
    __syncwarp();
    // pass 0: qp5 (second element) against qp1, qp2; pass 1: qp6 (first
    // element) against qp3, qp4 -- every inner point is evaluated once
#pragma unroll 1
    for (int pass = 0; pass < 2; ++pass) {
      S v[2][P2];
#pragma unroll
      for (int k = 0; k < 2; ++k)
#pragma unroll
        for (int t = 0; t < P2; ++t) v[k][t] = zero<S>();
      for (int jj = 0; jj < Q; jj += 32) {
        const int j = jj + lane;
        const bool valid = j < Q;
        const double e0 = valid ? gx[j / n1] : 0.5, e1 = valid ? gx[j % n1] : 0.5;
        const double wj = valid ? gw[j / n1] * gw[j % n1] : 0.0;
        double uv[2];
        PointEval q;
        double phq[P2];
        tau(x0 * e0, x0 * e1, pass ? rot1 : rot2, uv);
        eval_point<G, P>(pt, pass ? p1 : p2, pass ? a0 : b0, pass ? a1 : b1, h, uv[0], uv[1], wj, &q, phq);
#pragma unroll
        for (int k = 0; k < 2; ++k) {
          const PointEval& Fk = vp[warp][2 * pass + k];
          const double d0 = Fk.x[0] - q.x[0], d1 = Fk.x[1] - q.x[1], d2 = Fk.x[2] - q.x[2];
          S c = scale_of(kernel_val<S>(fma(d0, d0, fma(d1, d1, d2 * d2)), kre, kim), Fk.c * q.c);
          if (!valid) c = zero<S>();
#pragma unroll
          for (int t = 0; t < P2; ++t) v[k][t] = fmac(v[k][t], c, phq[t]);
        }
      }
      // sum the lanes' inner sums (every lane ends with the totals)
#pragma unroll
      for (int k = 0; k < 2; ++k)
#pragma unroll
        for (int t = 0; t < P2; ++t) v[k][t] = warp_sum(v[k][t]);
#pragma unroll
      for (int q = 0; q < 2 * P2; ++q)
        if ((q & 31) == lane) sv[2 * pass * P2 + q] = v[q / P2][q % P2];
    }
    __syncwarp();
    // pairs 0, 1: fixed point on the first element; 2, 3: on the second
#pragma unroll
    for (int m = 0; m < PER; ++m) {
      const int e = lane + 32 * m;
      if (e < NE) {
        const int a = e % P2, b = e / P2;
        const double* f = vphi[warp];
        acc[m] = fmac(acc[m], sv[b], f[a]);
        acc[m] = fmac(acc[m], sv[P2 + b], f[P2 + a]);
        acc[m] = fmac(acc[m], sv[2 * P2 + a], f[2 * P2 + b]);
        acc[m] = fmac(acc[m], sv[3 * P2 + a], f[3 * P2 + b]);
      }
    }
    __syncwarp();
  }
  write_block<P, S, PER>(acc, st, warp, lane, out, pr.dst, B);
}

// Identical element (integrate2.hpp:41-60), one wavenumber, P <= 2,
// n1 <= 16. With t1 = e0 (1 - x0), t3 = t1 + x0 (depending on e0) and
// t2 = e1 (1 - x0 x1), t4 = t2 + x0 x1 (depending on e1), the four point
// pairs are A = (t1, t2), B = (t3, t4); A = (t1, t4), B = (t3, t2);
// A = (t2, t1), B = (t4, t3); A = (t2, t3), B = (t4, t1). For a fixed
// (outer node, e0) every point lies on one of four patch lines (s fixed at
// t1 or t3, or t fixed at t1 or t3), contracted once (SurfaceLine), and each
// basis product splits into an e0 part and an e1 part, e.g. pair 0:
// phi_a(A) phi_b(B) = [B_ax(t1) B_bx(t3)] [B_ay(t2) B_by(t4)]. So the e1 sums
// are accumulated as three p^2-vectors per (outer node, e0) and added to the
// block as Kronecker products; the symmetric half (the pairs with A and B
// exchanged) is the transpose, added once at the end. A half-warp takes one
// e0 node, its lanes the e1 nodes.
template <int G, int P, typename S>
__global__ void __launch_bounds__(128) k_near_identical(PatchTable pt, ElementTable et,
                                                        const NearPair* __restrict__ pairs,
                                                        const double* __restrict__ gx, const double* __restrict__ gw,
                                                        int n1, double kre, double kim, S* __restrict__ out, int B) {
  constexpr int P1 = P + 1, P2 = P1 * P1, NE = P2 * P2;
  constexpr int PER = (NE + 31) / 32;
  __shared__ RankOneStage<P, S> st;  // final reduction only
  __shared__ SurfaceLine<G> lines[kEdgeNW][2][4];
  __shared__ double fb[kEdgeNW][2][2 * P1];  // per half: Bernstein values at t1, t3
  __shared__ S fv[kEdgeNW][2][3 * P2];       // per half: the three e1 sums
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, half = lane >> 4, l16 = lane & 15;
  const NearPair pr = pairs[blockIdx.x];
  const int p1 = et.patch[pr.e1];
  const double a0 = et.llc[2 * pr.e1], a1 = et.llc[2 * pr.e1 + 1];
  const double h = et.h;
  const int Q = n1 * n1;
  S acc[PER];
#pragma unroll
  for (int m = 0; m < PER; ++m) acc[m] = zero<S>();
  for (int i = warp; i < Q; i += kEdgeNW) {
    const double x0 = gx[i / n1], x1 = gx[i % n1], wi = gw[i / n1] * gw[i % n1];
    const double w = h * h * wi * x0 * (1 - x0) * (1 - x0 * x1);
    for (int e0b = 0; e0b < n1; e0b += 2) {
      const int m0 = e0b + half;
      const bool act0 = m0 < n1;
      const double t1 = act0 ? gx[m0] * (1 - x0) : 0.5, t3 = t1 + x0;
      // lines 0: s = t1, 1: s = t3, 2: t = t1, 3: t = t3 (element coordinates)
      if (act0 && l16 < 4)
        surface_line<G>(pt, p1, l16 < 2, (l16 < 2 ? a0 : a1) + h * ((l16 & 1) ? t3 : t1), lines[warp][half][l16]);
      if (act0 && l16 >= 4 && l16 < 6) {
        double b[P1];
        bern<P1>(P, l16 == 4 ? t1 : t3, b);
#pragma unroll
        for (int q = 0; q < P1; ++q) fb[warp][half][(l16 - 4) * P1 + q] = b[q];
      }
      __syncwarp();
      const bool act = act0 && l16 < n1;
      const int m1 = act ? l16 : 0;
      const double t2 = gx[m1] * (1 - x0 * x1), t4 = t2 + x0 * x1;
      const double wj = act ? w * gw[m0 < n1 ? m0 : 0] * gw[m1] : 0.0;
      S vL[P2], v2[P2], v3[P2];
#pragma unroll
      for (int q = 0; q < P2; ++q) vL[q] = v2[q] = v3[q] = zero<S>();
      if (act) {
        const SurfaceLine<G>* L = lines[warp][half];
        // points and surface measures: L1(t2), L3(t4), L1(t4), L3(t2), M1(t2), M3(t4), M3(t2), M1(t4)
        double X[8][3], J[8];
        const int li[8] = {0, 1, 0, 1, 2, 3, 3, 2};
        const double tv[8] = {t2, t4, t4, t2, t2, t4, t2, t4};
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          double dx[3], dy[3];
          surface_line_point<G>(L[li[k]], (li[k] < 2 ? a1 : a0) + h * tv[k], X[k], dx, dy);
          J[k] = surface_measure(dx, dy);
        }
        double b2[P1], b4[P1];
        bern<P1>(P, t2, b2);
        bern<P1>(P, t4, b4);
        S c[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const int ia = 2 * k, ib = 2 * k + 1;
          const double d0 = X[ia][0] - X[ib][0], d1 = X[ia][1] - X[ib][1], d2 = X[ia][2] - X[ib][2];
          c[k] = scale_of(kernel_val<S>(fma(d0, d0, fma(d1, d1, d2 * d2)), kre, kim), wj * J[ia] * J[ib]);
        }
#pragma unroll
        for (int ya = 0; ya < P1; ++ya)
#pragma unroll
          for (int yb = 0; yb < P1; ++yb) {
            const int q = ya * P1 + yb;
            // pairs 0, 1 vary in the second coordinate: (A, B) = (t2, t4) and (t4, t2)
            vL[q] = fmac(fmac(vL[q], c[0], b2[ya] * b4[yb]), c[1], b4[ya] * b2[yb]);
            // pairs 2, 3 vary in the first coordinate: (A, B) = (t2, t4)
            v2[q] = fmac(v2[q], c[2], b2[ya] * b4[yb]);
            v3[q] = fmac(v3[q], c[3], b2[ya] * b4[yb]);
          }
      }
      // sums over the half-warp's e1 nodes
#pragma unroll
      for (int q = 0; q < P2; ++q) {
#pragma unroll
        for (int o = 8; o; o >>= 1) {
          vL[q] = vL[q] + shfl_xor(vL[q], o);
          v2[q] = v2[q] + shfl_xor(v2[q], o);
          v3[q] = v3[q] + shfl_xor(v3[q], o);
        }
      }
      if (l16 == 0 && act0) {
#pragma unroll
        for (int q = 0; q < P2; ++q) {
          fv[warp][half][q] = vL[q];
          fv[warp][half][P2 + q] = v2[q];
          fv[warp][half][2 * P2 + q] = v3[q];
        }
      }
      __syncwarp();
      // block S(a, b), a = ay P1 + ax, b = by P1 + bx:
      //   F_L(ax, bx) vL(ay, by) + v2(ax, bx) F2(ay, by) + v3(ax, bx) F3(ay, by)
      // with F_L(x, y) = F2(x, y) = B_x(t1) B_y(t3), F3(x, y) = B_x(t3) B_y(t1)
#pragma unroll
      for (int hf = 0; hf < 2; ++hf) {
        if (e0b + hf >= n1) break;
        const double* f1 = fb[warp][hf];
        const double* f3 = f1 + P1;
        const S* v = fv[warp][hf];
#pragma unroll
        for (int m = 0; m < PER; ++m) {
          const int e = lane + 32 * m;
          if (e < NE) {
            const int a = e % P2, b = e / P2;
            const int ax = a % P1, ay = a / P1, bx = b % P1, by = b / P1;
            acc[m] = fmac(acc[m], v[ay * P1 + by], f1[ax] * f3[bx]);
            acc[m] = fmac(acc[m], v[P2 + ax * P1 + bx], f1[ay] * f3[by]);
            acc[m] = fmac(acc[m], v[2 * P2 + ax * P1 + bx], f3[ay] * f1[by]);
          }
        }
      }
      __syncwarp();
    }
  }
  // sum the warps, then add the transpose (the pairs with A and B exchanged)
  S* red = &st.v[0][0];
  __syncthreads();
#pragma unroll
  for (int m = 0; m < PER; ++m) {
    const int e = lane + 32 * m;
    if (e < NE) red[warp * 32 * P2 + e] = acc[m];
  }
  __syncthreads();
  for (int e = threadIdx.x; e < NE; e += blockDim.x) {
    const int a = e % P2, b = e / P2, et2 = b + a * P2;
    S v = red[e] + red[et2];
#pragma unroll
    for (int w2 = 1; w2 < kEdgeNW; ++w2) v = v + red[w2 * 32 * P2 + e] + red[w2 * 32 * P2 + et2];
    out[pr.dst + (long)b * B + a] = v;
  }
}

template <int G, int P, typename S, int NK>
static cudaError_t run_duffy_k(int cs, const PatchTable& pt, const ElementTable& et, const NearPair* pairs,
                               int npairs, const double* gx, const double* gw, int n1, const KBatch<S, NK>& kb, int B,
                               cudaStream_t s) {
  if constexpr (NK == 1 && P <= 2) {
    // factorised common-edge / common-vertex kernels (cache of 2 n1 points per warp)
    if (cs == 3 && 2 * n1 <= 32) {
      k_near_edge<G, P, S><<<npairs, 128, 0, s>>>(pt, et, pairs, gx, gw, n1, kb.kre[0], kb.kim[0], kb.out[0], B);
      return cudaGetLastError();
    }
    if (cs == 4) {
      k_near_vertex<G, P, S><<<npairs, 128, 0, s>>>(pt, et, pairs, gx, gw, n1, kb.kre[0], kb.kim[0], kb.out[0], B);
      return cudaGetLastError();
    }
    if (cs == 2 && 2 * n1 <= 32) {
      k_near_identical<G, P, S><<<npairs, 128, 0, s>>>(pt, et, pairs, gx, gw, n1, kb.kre[0], kb.kim[0], kb.out[0], B);
      return cudaGetLastError();
    }
  }
  if (cs == 2) k_near_duffy<G, P, S, 2, NK><<<npairs, 128, 0, s>>>(pt, et, pairs, gx, gw, n1, kb, B);
  else if (cs == 3) k_near_duffy<G, P, S, 3, NK><<<npairs, 128, 0, s>>>(pt, et, pairs, gx, gw, n1, kb, B);
  else if (cs == 4) k_near_duffy<G, P, S, 4, NK><<<npairs, 128, 0, s>>>(pt, et, pairs, gx, gw, n1, kb, B);
  else return cudaErrorInvalidValue;
  return cudaGetLastError();
}

template <int G, int P, typename S>
static cudaError_t run_duffy(int cs, const PatchTable& pt, const ElementTable& et, const NearPair* pairs, int npairs,
                             const double* gx, const double* gw, int n1, double kre, double kim, S* out, int B,
                             cudaStream_t s) {
  if (npairs == 0) return cudaSuccess;
  KBatch<S, 1> kb{{kre}, {kim}, {out}};
  return run_duffy_k<G, P, S, 1>(cs, pt, et, pairs, npairs, gx, gw, n1, kb, B, s);
}

// complex kernels, nk (1 .. kDuffyMaxWavenumbers) wavenumbers per launch
template <int G, int P>
static cudaError_t run_duffy_multi(int cs, const PatchTable& pt, const ElementTable& et, const NearPair* pairs,
                                   int npairs, const double* gx, const double* gw, int n1, int nk, const double* kre,
                                   const double* kim, void* const* out, int B, cudaStream_t s) {
  if (npairs == 0) return cudaSuccess;
  switch (nk) {
#define BG_DUFK(NKV)                                                                               \
  case NKV: {                                                                                      \
    KBatch<cd, NKV> kb;                                                                            \
    for (int q = 0; q < NKV; ++q) {                                                                \
      kb.kre[q] = kre[q];                                                                          \
      kb.kim[q] = kim[q];                                                                          \
      kb.out[q] = static_cast<cd*>(out[q]);                                                        \
    }                                                                                              \
    return run_duffy_k<G, P, cd, NKV>(cs, pt, et, pairs, npairs, gx, gw, n1, kb, B, s);            \
  }
    BG_DUFK(1)
    BG_DUFK(2)
    BG_DUFK(3)
    BG_DUFK(4)
#undef BG_DUFK
    default: return cudaErrorInvalidValue;
  }
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

template <int G>
static cudaError_t duffy_multi_p(int P, int cs, const PatchTable& pt, const ElementTable& et, const NearPair* pairs,
                                 int npairs, const double* gx, const double* gw, int n1, int nk, const double* kre,
                                 const double* kim, void* const* out, int B, cudaStream_t s) {
  switch (P) {
    case 1: return run_duffy_multi<G, 1>(cs, pt, et, pairs, npairs, gx, gw, n1, nk, kre, kim, out, B, s);
    case 2: return run_duffy_multi<G, 2>(cs, pt, et, pairs, npairs, gx, gw, n1, nk, kre, kim, out, B, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_near_duffy_multi(int G, int P, int cs, const PatchTable& pt, const ElementTable& et,
                                    const NearPair* pairs, int npairs, const double* gx, const double* gw, int n1,
                                    int nk, const double* kre, const double* kim, void* const* out, int B,
                                    cudaStream_t s) {
  switch (G) {
    case 2: return duffy_multi_p<2>(P, cs, pt, et, pairs, npairs, gx, gw, n1, nk, kre, kim, out, B, s);
    case 3: return duffy_multi_p<3>(P, cs, pt, et, pairs, npairs, gx, gw, n1, nk, kre, kim, out, B, s);
    case 5: return duffy_multi_p<5>(P, cs, pt, et, pairs, npairs, gx, gw, n1, nk, kre, kim, out, B, s);
    default: return cudaErrorInvalidValue;
  }
}

// ---------------------------------------------------------------------------
// Maxwell single layer (Maxwell/SingleLayerOperator.hpp:44-88 with
// SuperSpace::addScaledVectorBasisInteraction, SuperSpace.hpp:236-258, and
// Div_Phi_times_Div_Phi_, Basis.hpp:170-200). Per point pair, with
// c = k(x, y) w_x w_y and t_0 = dx, t_1 = dy the patch tangents, block
// (rc, cc) of the element pair gains
//   c (t_rc(x) . t_cc(y)) phi_a(x) phi_b(y) + c idiv D_rc phi_a(x) D_cc phi_b(y)
// where D_0, D_1 are the element-coordinate derivatives and
// idiv = -1 / (kappa^2 h^2).

template <int G>
__global__ void k_quad_table_mw(PatchTable pt, ElementTable et, int ne, const double* __restrict__ gx,
                                const double* __restrict__ gw, int n1, MwPt* __restrict__ out) {
  const int Q = n1 * n1;
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long)ne * Q) return;
  const int e = (int)(idx / Q), q = (int)(idx % Q);
  const double u = gx[q / n1], v = gx[q % n1], w = gw[q / n1] * gw[q % n1];
  const double h = et.h;
  MwPt p;
  surface_frame<G>(pt, et.patch[e], et.llc[2 * e] + h * u, et.llc[2 * e + 1] + h * v, p.x, p.dx, p.dy);
  p.w = h * w;
  out[idx] = p;
}

cudaError_t launch_quad_table_mw(int G, const PatchTable& pt, const ElementTable& et, int ne, const double* gx,
                                 const double* gw, int n1, MwPt* out, cudaStream_t s) {
  const long n = (long)ne * n1 * n1;
  const unsigned grid = (unsigned)((n + 127) / 128);
  switch (G) {
    case 2: k_quad_table_mw<2><<<grid, 128, 0, s>>>(pt, et, ne, gx, gw, n1, out); break;
    case 3: k_quad_table_mw<3><<<grid, 128, 0, s>>>(pt, et, ne, gx, gw, n1, out); break;
    case 4: k_quad_table_mw<4><<<grid, 128, 0, s>>>(pt, et, ne, gx, gw, n1, out); break;
    case 5: k_quad_table_mw<5><<<grid, 128, 0, s>>>(pt, et, ne, gx, gw, n1, out); break;
    case 6: k_quad_table_mw<6><<<grid, 128, 0, s>>>(pt, et, ne, gx, gw, n1, out); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// Regular pairs, one CTA per pair, the tensor rule factorised as in
// k_near_regular. The Gauss points i of e1 go in chunks of kMwChunk:
//  A) Kt[i][j] = k(x_i, y_j) w_i w_j for the chunk;
//  B) thread (i, cc, m) sums W[i][cc][m][b] = sum_j Kt[i][j] f_m(y_j) g_b(y_j)
//     with (f_m, g) = (t_cc,m, phi) for m < 3 and (idiv, D_cc phi) for m = 3;
//  C) thread per entry (rc, cc, a, b) adds
//     sum_i phi_a(x_i) t_rc(x_i) . W[i][cc][0..2][b] + D_rc phi_a(x_i) W[i][cc][3][b].
// basis3 holds phi, D_0 phi, D_1 phi at the Q points ([3][Q][P2]).
constexpr int kMwChunk = 16;

template <int P>
__global__ void __launch_bounds__(128) k_near_regular_mw(const NearPairV* __restrict__ pairs,
                                                         const MwPt* __restrict__ tab, int n1,
                                                         const double* __restrict__ basis3, double kre, double kim,
                                                         cd idiv, cd* __restrict__ out, int B) {
  constexpr int P2 = (P + 1) * (P + 1);
  constexpr int NB = P2 * P2;
  constexpr int NE = 4 * NB;
  constexpr int PER = (NE + 127) / 128;
  const int Q = n1 * n1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cd* Kt = reinterpret_cast<cd*>(smem_raw);  // [kMwChunk][Q]
  cd* Ws = Kt + kMwChunk * Q;                // [kMwChunk][2][4][P2]
  MwPt* ys = reinterpret_cast<MwPt*>(Ws + kMwChunk * 8 * P2);
  MwPt* xs = ys + Q;  // [kMwChunk]
  double* U = reinterpret_cast<double*>(xs + kMwChunk);
  const NearPairV pr = pairs[blockIdx.x];
  const int tid = threadIdx.x;
  for (int q = tid; q < Q; q += blockDim.x) ys[q] = tab[(long)pr.e2 * Q + q];
  for (int k = tid; k < 3 * Q * P2; k += blockDim.x) U[k] = basis3[k];
  cd acc[PER];
#pragma unroll
  for (int m = 0; m < PER; ++m) acc[m] = zero<cd>();
  for (int i0 = 0; i0 < Q; i0 += kMwChunk) {
    const int ic = min(kMwChunk, Q - i0);
    __syncthreads();
    if (tid < ic) xs[tid] = tab[(long)pr.e1 * Q + i0 + tid];
    __syncthreads();
    for (int e = tid; e < ic * Q; e += blockDim.x) {
      const int ii = e / Q, j = e % Q;
      const double d0 = xs[ii].x[0] - ys[j].x[0], d1 = xs[ii].x[1] - ys[j].x[1], d2 = xs[ii].x[2] - ys[j].x[2];
      const double r2 = fma(d0, d0, fma(d1, d1, d2 * d2));
      Kt[e] = kernel_val<cd>(r2, kre, kim) * (xs[ii].w * ys[j].w);
    }
    __syncthreads();
    for (int t = tid; t < ic * 8; t += blockDim.x) {
      const int ii = t >> 3, cc = (t >> 2) & 1, m = t & 3;
      const double* g = m < 3 ? U : U + (1 + cc) * Q * P2;
      cd w[P2];
#pragma unroll
      for (int b = 0; b < P2; ++b) w[b] = zero<cd>();
      for (int j = 0; j < Q; ++j) {
        const double f = m < 3 ? (cc == 0 ? ys[j].dx[m] : ys[j].dy[m]) : 1.0;
        const cd kk = Kt[ii * Q + j] * f;
#pragma unroll
        for (int b = 0; b < P2; ++b) w[b] = fmac(w[b], kk, g[j * P2 + b]);
      }
      cd* o = Ws + (ii * 8 + cc * 4 + m) * P2;
#pragma unroll
      for (int b = 0; b < P2; ++b) o[b] = m < 3 ? w[b] : w[b] * idiv;
    }
    __syncthreads();
#pragma unroll
    for (int m = 0; m < PER; ++m) {
      const int e = tid + 128 * m;
      if (e < NE) {
        const int comp = e / NB, wi = e % NB;
        const int a = wi % P2, b = wi / P2, rc = comp >> 1, cc = comp & 1;
        const double* Da = U + (1 + rc) * Q * P2;
        cd v = acc[m];
        for (int ii = 0; ii < ic; ++ii) {
          const int i = i0 + ii;
          const double* t = rc == 0 ? xs[ii].dx : xs[ii].dy;
          const cd* wv = Ws + (ii * 8 + cc * 4) * P2 + b;
          cd tv = wv[0] * t[0];
          tv = fmac(tv, t[1], wv[P2]);
          tv = fmac(tv, t[2], wv[2 * P2]);
          v = fmac(v, U[i * P2 + a], tv);
          v = fmac(v, Da[i * P2 + a], wv[3 * P2]);
        }
        acc[m] = v;
      }
    }
  }
#pragma unroll
  for (int m = 0; m < PER; ++m) {
    const int e = tid + 128 * m;
    if (e < NE) {
      const int comp = e / NB, wi = e % NB;
      const int a = wi % P2, b = wi / P2;
      out[pr.dst[comp] + (long)b * B + a] = acc[m];
    }
  }
}

template <int P>
static size_t regular_mw_smem(int Q) {
  constexpr int P2 = (P + 1) * (P + 1);
  return (size_t)kMwChunk * Q * sizeof(cd) + (size_t)kMwChunk * 8 * P2 * sizeof(cd) + (size_t)Q * sizeof(MwPt) +
         (size_t)kMwChunk * sizeof(MwPt) + (size_t)3 * Q * P2 * sizeof(double);
}

template <int P>
static cudaError_t run_regular_mw(const NearPairV* pairs, int npairs, const MwPt* tab, int n1, const double* basis3,
                                  double kre, double kim, cd idiv, cd* out, int B, cudaStream_t s) {
  const size_t smem = regular_mw_smem<P>(n1 * n1);
  if (smem > 220 * 1024) return cudaErrorInvalidConfiguration;
  auto kfn = k_near_regular_mw<P>;
  cudaError_t err = smem_limit(kfn, smem);
  if (err != cudaSuccess) return err;
  if (npairs == 0) return cudaSuccess;
  kfn<<<npairs, 128, smem, s>>>(pairs, tab, n1, basis3, kre, kim, idiv, out, B);
  return cudaGetLastError();
}

cudaError_t launch_near_regular_mw(int P, const NearPairV* pairs, int npairs, const MwPt* tab, int n1,
                                   const double* basis3, double kre, double kim, cd idiv, cd* out, int B,
                                   cudaStream_t s) {
  switch (P) {
    case 1: return run_regular_mw<1>(pairs, npairs, tab, n1, basis3, kre, kim, idiv, out, B, s);
    case 2: return run_regular_mw<2>(pairs, npairs, tab, n1, basis3, kre, kim, idiv, out, B, s);
    case 3: return run_regular_mw<3>(pairs, npairs, tab, n1, basis3, kre, kim, idiv, out, B, s);
    default: return cudaErrorInvalidValue;
  }
}


// Singular pairs of the Maxwell operator: the quadratures of k_near_duffy, with
// the samples of a warp staged as c = k w_x w_y, c idiv, the four tangent
// products T[rc][cc] = t_rc(x) . t_cc(y) and (phi, D_0 phi, D_1 phi) at both
// points; each lane accumulates its share of the 4 p^4 entries.
template <int G, int P>
__device__ inline void eval_point_mw(const PatchTable& pt, int patch, double l0, double l1, double h, double u,
                                     double v, double w, MwPt* pe, double* phi3) {
  constexpr int P2 = (P + 1) * (P + 1);
  surface_frame<G>(pt, patch, l0 + h * u, l1 + h * v, pe->x, pe->dx, pe->dy);
  pe->w = w;
  tensor_basis_grad<P>(u, v, phi3, phi3 + P2, phi3 + 2 * P2);
}

template <int P>
struct MwWarpLayout {
  static constexpr int P2 = (P + 1) * (P + 1);
  // per warp, in doubles: sc, sd (32 complex each), st (32 x 4), sa, sb
  // (32 x 3 P2 each), vp (4 points), vphi (4 x 3 P2)
  static constexpr int SC = 0, SD = 64, ST = 128, SA = 256, SB = SA + 32 * 3 * P2, VP = SB + 32 * 3 * P2,
                       VPHI = VP + 4 * 10, WORDS = VPHI + 4 * 3 * P2;
};

template <int G, int P, int CS>
__global__ void __launch_bounds__(128) k_near_duffy_mw(PatchTable pt, ElementTable et,
                                                       const NearPairV* __restrict__ pairs,
                                                       const double* __restrict__ gx, const double* __restrict__ gw,
                                                       int n1, double kre, double kim, cd idiv, cd* __restrict__ out,
                                                       int B) {
  using L = MwWarpLayout<P>;
  constexpr int P2 = L::P2;
  constexpr int NB = P2 * P2;
  constexpr int NE = 4 * NB;
  constexpr int PER = (NE + 31) / 32;
  constexpr int NW = 4;
  extern __shared__ __align__(16) double dsm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* wb = dsm + warp * L::WORDS;
  cd* sc = reinterpret_cast<cd*>(wb + L::SC);
  cd* sd = reinterpret_cast<cd*>(wb + L::SD);
  double* st = wb + L::ST;
  double* sa = wb + L::SA;
  double* sb = wb + L::SB;
  MwPt* vp = reinterpret_cast<MwPt*>(wb + L::VP);
  double* vphi = wb + L::VPHI;
  const NearPairV pr = pairs[blockIdx.x];
  const int rot1 = pr.rot & 15, rot2 = pr.rot >> 4;
  const int p1 = et.patch[pr.e1], p2 = et.patch[pr.e2];
  const double a0 = et.llc[2 * pr.e1], a1 = et.llc[2 * pr.e1 + 1];
  const double b0 = et.llc[2 * pr.e2], b1 = et.llc[2 * pr.e2 + 1];
  const double h = et.h;
  const int Q = n1 * n1;
  cd acc[PER];
#pragma unroll
  for (int m = 0; m < PER; ++m) acc[m] = zero<cd>();
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
        if (lane < 2) eval_point_mw<G, P>(pt, p1, a0, a1, h, uv[0], uv[1], w, &vp[lane], vphi + lane * 3 * P2);
        else eval_point_mw<G, P>(pt, p2, b0, b1, h, uv[0], uv[1], w, &vp[lane], vphi + lane * 3 * P2);
      }
      __syncwarp();
    }
    for (int jj = 0; jj < Q; jj += 32) {
      const int j = jj + lane;
      const bool valid = j < Q;
      const double e0 = valid ? gx[j / n1] : 0.5, e1 = valid ? gx[j % n1] : 0.5;
      const double wj = valid ? gw[j / n1] * gw[j % n1] : 0.0;
      constexpr int NK = CS == 2 ? 4 : (CS == 3 ? 6 : 4);
#pragma unroll 1
      for (int k = 0; k < NK; ++k) {
        MwPt A, Bp;
        double* pa = sa + lane * 3 * P2;
        double* pb = sb + lane * 3 * P2;
        if (CS == 2) {
          // integrate2.hpp:41-60
          const double t1 = e0 * (1 - x0), t2 = e1 * (1 - x0 * x1);
          const double t3 = e0 * (1 - x0) + x0, t4 = e1 * (1 - x0 * x1) + x0 * x1;
          double u1, v1, u2, v2;
          if (k == 0) { u1 = t1; v1 = t2; u2 = t3; v2 = t4; }
          else if (k == 1) { u1 = t1; v1 = t4; u2 = t3; v2 = t2; }
          else if (k == 2) { u1 = t2; v1 = t1; u2 = t4; v2 = t3; }
          else { u1 = t2; v1 = t3; u2 = t4; v2 = t1; }
          eval_point_mw<G, P>(pt, p1, a0, a1, h, u1, v1, w, &A, pa);
          eval_point_mw<G, P>(pt, p1, a0, a1, h, u2, v2, wj, &Bp, pb);
        } else if (CS == 3) {
          // integrate3.hpp:45-76
          const double f0 = x1 * e0, f1 = x1 * e1;
          const double t1 = x0 * (1 - x1), t2 = (1 - x0) * (1 - x1);
          const double t3 = x0 * (1 - f0), t4 = (1 - x0) * (1 - f0);
          double ua, va, ub, vb, wbb;
          if (k == 0) { ua = t1; va = f0; ub = t2; vb = f1; wbb = wj * (1 - x1); }
          else if (k == 1) { ua = 1 - t1; va = f0; ub = 1 - t2; vb = f1; wbb = wj * (1 - x1); }
          else if (k == 2) { ua = t3; va = x1; ub = t4; vb = f1; wbb = wj * (1 - f0); }
          else if (k == 3) { ua = 1 - t3; va = x1; ub = 1 - t4; vb = f1; wbb = wj * (1 - f0); }
          else if (k == 4) { ua = t4; va = f1; ub = t3; vb = x1; wbb = wj * (1 - f0); }
          else { ua = 1 - t4; va = f1; ub = 1 - t3; vb = x1; wbb = wj * (1 - f0); }
          double uv1[2], uv2[2];
          tau(ua, va, rot1, uv1);
          tau(ub, vb, rot2, uv2);
          eval_point_mw<G, P>(pt, p1, a0, a1, h, uv1[0], uv1[1], w, &A, pa);
          eval_point_mw<G, P>(pt, p2, b0, b1, h, uv2[0], uv2[1], wbb, &Bp, pb);
        } else {
          // integrate4.hpp:49-58: (qp1,qp5), (qp2,qp5), (qp6,qp3), (qp6,qp4)
          double uv[2];
          if (k < 2) {
            tau(x0 * e0, x0 * e1, rot2, uv);
            eval_point_mw<G, P>(pt, p2, b0, b1, h, uv[0], uv[1], wj, &Bp, pb);
            A = vp[k];
#pragma unroll
            for (int t = 0; t < 3 * P2; ++t) pa[t] = vphi[k * 3 * P2 + t];
          } else {
            tau(x0 * e0, x0 * e1, rot1, uv);
            eval_point_mw<G, P>(pt, p1, a0, a1, h, uv[0], uv[1], wj, &A, pa);
            Bp = vp[k];
#pragma unroll
            for (int t = 0; t < 3 * P2; ++t) pb[t] = vphi[k * 3 * P2 + t];
          }
        }
        const double d0 = A.x[0] - Bp.x[0], d1 = A.x[1] - Bp.x[1], d2 = A.x[2] - Bp.x[2];
        const double r2 = fma(d0, d0, fma(d1, d1, d2 * d2));
        cd c = kernel_val<cd>(r2, kre, kim) * (A.w * Bp.w);
        if (!valid) c = zero<cd>();
        sc[lane] = c;
        sd[lane] = c * idiv;
        double* tl = st + 4 * lane;
        const double* ta[2] = {A.dx, A.dy};
        const double* tb[2] = {Bp.dx, Bp.dy};
#pragma unroll
        for (int r = 0; r < 2; ++r)
#pragma unroll
          for (int q = 0; q < 2; ++q)
            tl[2 * r + q] = fma(ta[r][0], tb[q][0], fma(ta[r][1], tb[q][1], ta[r][2] * tb[q][2]));
        __syncwarp();
        for (int smp = 0; smp < 32; ++smp) {
          const cd cs = sc[smp], ds = sd[smp];
          const double* T = st + 4 * smp;
          const double* fa = sa + smp * 3 * P2;
          const double* fb = sb + smp * 3 * P2;
#pragma unroll
          for (int m = 0; m < PER; ++m) {
            const int e = lane + 32 * m;
            if (e < NE) {
              const int comp = e / NB, wi = e % NB;
              const int a = wi % P2, b = wi / P2, rc = comp >> 1, cc = comp & 1;
              double v = T[comp] * fa[a] * fb[b];
              double dv = fa[(1 + rc) * P2 + a] * fb[(1 + cc) * P2 + b];
              if (CS == 2) {
                // integrand(qp2, qp1) of the identical-element rule
                v = fma(T[2 * cc + rc] * fb[a], fa[b], v);
                dv = fma(fb[(1 + rc) * P2 + a], fa[(1 + cc) * P2 + b], dv);
              }
              acc[m] = fmac(fmac(acc[m], cs, v), ds, dv);
            }
          }
        }
        __syncwarp();
      }
    }
    if (CS == 4) __syncwarp();
  }
  // reduce the warps' accumulators through the staging memory
  static_assert(NE * 2 <= L::WORDS, "reduction buffer too small");
  __syncthreads();
  cd* red = reinterpret_cast<cd*>(dsm);
  const int stride = L::WORDS / 2;
#pragma unroll
  for (int m = 0; m < PER; ++m) {
    const int e = lane + 32 * m;
    if (e < NE) red[warp * stride + e] = acc[m];
  }
  __syncthreads();
  for (int e = threadIdx.x; e < NE; e += blockDim.x) {
    cd v = red[e];
#pragma unroll
    for (int w2 = 1; w2 < NW; ++w2) v = v + red[w2 * stride + e];
    const int comp = e / NB, wi = e % NB;
    const int a = wi % P2, b = wi / P2;
    out[pr.dst[comp] + (long)b * B + a] = v;
  }
}

template <int G, int P>
static cudaError_t run_duffy_mw(int cs, const PatchTable& pt, const ElementTable& et, const NearPairV* pairs,
                                int npairs, const double* gx, const double* gw, int n1, double kre, double kim,
                                cd idiv, cd* out, int B, cudaStream_t s) {
  const size_t smem = 4 * MwWarpLayout<P>::WORDS * sizeof(double);
#define BG_DMW(CSV)                                                                                      \
  {                                                                                                      \
    auto kfn = k_near_duffy_mw<G, P, CSV>;                                                               \
    cudaError_t err = smem_limit(kfn, smem); \
    if (err != cudaSuccess) return err;                                                                  \
    if (npairs == 0) return cudaSuccess;                                                                 \
    kfn<<<npairs, 128, smem, s>>>(pt, et, pairs, gx, gw, n1, kre, kim, idiv, out, B);                    \
    return cudaGetLastError();                                                                           \
  }
  if (cs == 2) BG_DMW(2)
  if (cs == 3) BG_DMW(3)
  if (cs == 4) BG_DMW(4)
#undef BG_DMW
  return cudaErrorInvalidValue;
}

template <int G>
static cudaError_t duffy_mw_p(int P, int cs, const PatchTable& pt, const ElementTable& et, const NearPairV* pairs,
                              int npairs, const double* gx, const double* gw, int n1, double kre, double kim, cd idiv,
                              cd* out, int B, cudaStream_t s) {
  switch (P) {
    case 1: return run_duffy_mw<G, 1>(cs, pt, et, pairs, npairs, gx, gw, n1, kre, kim, idiv, out, B, s);
    case 2: return run_duffy_mw<G, 2>(cs, pt, et, pairs, npairs, gx, gw, n1, kre, kim, idiv, out, B, s);
    case 3: return run_duffy_mw<G, 3>(cs, pt, et, pairs, npairs, gx, gw, n1, kre, kim, idiv, out, B, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_near_duffy_mw(int G, int P, int cs, const PatchTable& pt, const ElementTable& et,
                                 const NearPairV* pairs, int npairs, const double* gx, const double* gw, int n1,
                                 double kre, double kim, cd idiv, cd* out, int B, cudaStream_t s) {
  switch (G) {
    case 2: return duffy_mw_p<2>(P, cs, pt, et, pairs, npairs, gx, gw, n1, kre, kim, idiv, out, B, s);
    case 3: return duffy_mw_p<3>(P, cs, pt, et, pairs, npairs, gx, gw, n1, kre, kim, idiv, out, B, s);
    case 5: return duffy_mw_p<5>(P, cs, pt, et, pairs, npairs, gx, gw, n1, kre, kim, idiv, out, B, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace bg
