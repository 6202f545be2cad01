// FMM forward and backward transforms (H2Multipole.hpp:380-469) as two fused
// launches per product, applied through their tensor-product factors.
//
// The reference builds both FMM matrices as tensor products of 1-D matrices
// (H2Multipole.hpp:76-115 and :224-293):
//   transfer  T_k[(ps,pt)][(cs,ct)] = Es_k[cs][ps] Et_k[ct][pt], child k of a
//             parent (son order), Es_k / Et_k the Lagrange values of the parent
//             polynomials at the child's points on the s / t half of the
//             parent interval (E0: lower half, E1: upper half);
//   moments   Mom[(i,j)][(e,ay,ax)] = Ms[i][a] Mt[j][b], a = ex_e (P+1) + ax,
//             b = ey_e (P+1) + ay for element e of the leaf cluster at
//             (ex_e, ey_e).
// Applying the factors one direction at a time gives the same products as
// the assembled np^2 x 4np^2 and np^2 x Bq matrices, with rounding as the only
// difference, in a fraction of the operations (per parent and column
// 8 np^3 instead of 4 np^4 multiply-adds; n_p = 9: 5832 instead of 26244).
//
// Forward (k_fmm_up): one CTA per FMM parent of the leaf clusters and per 32
// columns. It computes the moments of its 4 leaf clusters, writes them
// (Y_L), and transfers them to the parent (Y_{L-1}). The parent's 4 siblings
// meet in a counter: the CTA that arrives last transfers the 4 of them one
// level up, and so on to level 0 (the threadfence-reduction pattern; no CTA
// ever waits for another). The last arriver puts the counter back to zero.
//
// Backward (k_fmm_down): one CTA per FMM parent of the leaf clusters and per
// 32 columns. It walks the path from its level-0 ancestor down, adding the
// transposed transfer of the ancestor's full coefficient to each level's
// far-field result (every CTA recomputes its own ancestors: a chain of L - 1
// one-child transfers, cheap in factored form, and no inter-CTA
// dependencies), then for each of its 4 leaf clusters adds the transfer from
// the parent and applies the transposed moments, accumulating into the
// superspace result.
//
// Layout: panels in shared memory are [row][32 columns], lane = column, so a
// warp reads a row without bank conflicts and the 1-D factors are broadcast.
// Warp w owns output rows w, w + 8, ... of every stage.
#include <algorithm>
#include <cstdint>
#include <type_traits>

#include "bg_kernels.cuh"

namespace bg {

namespace {

constexpr int kFmmThreads = 256;
constexpr int kFmmWarps = kFmmThreads / 32;
constexpr int kFmmCols = 32;
constexpr int kMaxAcc = (kFmmMaxNp * kFmmMaxNp + kFmmWarps - 1) / kFmmWarps;

// son order (0,0), (1,0), (1,1), (0,1) (ElementTree.hpp:706-711): halves of child k
__device__ __forceinline__ int half_s(int k) { return (k == 1 || k == 2) ? 1 : 0; }
__device__ __forceinline__ int half_t(int k) { return k >> 1; }

template <typename T>
struct FmmSmem {
  T* E;    // [2][np][np]: E_h[c][p] = L_p(x_c / 2 + h / 2)
  T* Ms;   // [np][w1]
  T* Mt;   // [np][w1]
  int* q_of;  // [w1][w1]: superspace row of the leaf cluster holding (a, b)
  T* X;    // [4 Bq][32] leaf inputs (up) / unused (down)
  T* W;    // [max(np w1, np^2)][32] stage scratch
  T* V;    // [np^2][32] stage scratch
  T* C;    // [np^2][32] current child / leaf coefficients
  T* Zf;   // [np^2][32] (down) the parent's full coefficients
};

template <typename T>
__device__ __forceinline__ size_t align16(size_t n) { return (n * sizeof(T) + 15) / 16 * 16 / sizeof(T); }

template <typename T>
__device__ FmmSmem<T> carve(unsigned char* base, int np, int w1, int Bq, bool with_x) {
  FmmSmem<T> s;
  const int np2 = np * np, wrows = max(np * w1, np2);
  T* p = reinterpret_cast<T*>(base);
  s.E = p;
  p += align16<T>(2 * np2);
  s.Ms = p;
  p += align16<T>(np * w1);
  s.Mt = p;
  p += align16<T>(np * w1);
  s.X = p;
  if (with_x) p += (size_t)4 * Bq * kFmmCols;
  s.W = p;
  p += (size_t)wrows * kFmmCols;
  s.V = p;
  p += (size_t)np2 * kFmmCols;
  s.C = p;
  p += (size_t)np2 * kFmmCols;
  s.Zf = p;
  p += (size_t)np2 * kFmmCols;
  s.q_of = reinterpret_cast<int*>(p);
  return s;
}

template <typename T>
__device__ void load_factors(const FmmSmem<T>& s, const T* fac, const int* cmap, int np, int w1, int Bq) {
  const int np2 = np * np;
  for (int t = threadIdx.x; t < 2 * np2; t += blockDim.x) s.E[t] = fac[t];
  for (int t = threadIdx.x; t < np * w1; t += blockDim.x) {
    s.Ms[t] = fac[2 * np2 + t];
    s.Mt[t] = fac[2 * np2 + np * w1 + t];
  }
  for (int q = threadIdx.x; q < Bq; q += blockDim.x) {
    const int ab = cmap[q];
    s.q_of[(ab & 0xFF) * w1 + (ab >> 8)] = q;
  }
}

// V[cs][pt] = sum_ct Et[ct][pt] C[cs][ct]   (transfer up, stage 1, t direction)
template <typename T>
__device__ __forceinline__ void up_stage1(const T* Et, const T* C, T* V, int np, int w, int lane) {
  const int np2 = np * np;
  for (int o = w; o < np2; o += kFmmWarps) {
    const int cs = o / np, pt = o - cs * np;
    T acc = T(0);
    for (int ct = 0; ct < np; ++ct) acc = fma(Et[ct * np + pt], C[(cs * np + ct) * kFmmCols + lane], acc);
    V[o * kFmmCols + lane] = acc;
  }
}
// acc[u] += sum_cs Es[cs][ps] V[cs][pt], output row o = w + 8u = ps np + pt
template <typename T>
__device__ __forceinline__ void up_stage2(const T* Es, const T* V, T* acc, int np, int w, int lane) {
  const int np2 = np * np;
#pragma unroll
  for (int u = 0; u < kMaxAcc; ++u) {
    const int o = w + kFmmWarps * u;
    if (o < np2) {
      const int ps = o / np, pt = o - ps * np;
      T a = acc[u];
      for (int cs = 0; cs < np; ++cs) a = fma(Es[cs * np + ps], V[(cs * np + pt) * kFmmCols + lane], a);
      acc[u] = a;
    }
  }
}

// one level of the upward pass for parent `par` of level l from its 4
// children at level l + 1, read from global memory (ld.global.cg: written by
// other CTAs of this launch)
template <typename T>
__device__ void transfer_up_from_global(const FmmSmem<T>& s, const T* ychild, T* ypar, int par, int np, int kk,
                                        int c0) {
  const int np2 = np * np, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool on = c0 + lane < kk;
  T acc[kMaxAcc];
#pragma unroll
  for (int u = 0; u < kMaxAcc; ++u) acc[u] = T(0);
  for (int k = 0; k < 4; ++k) {
    const T* src = ychild + ((size_t)(4 * par + k) * np2) * kk + c0 + lane;
    for (int o = w; o < np2; o += kFmmWarps) s.C[o * kFmmCols + lane] = on ? __ldcg(src + (size_t)o * kk) : T(0);
    __syncthreads();
    up_stage1(s.E + half_t(k) * np2, s.C, s.V, np, w, lane);
    __syncthreads();
    up_stage2(s.E + half_s(k) * np2, s.V, acc, np, w, lane);
    __syncthreads();
  }
  T* dst = ypar + ((size_t)par * np2) * kk + c0 + lane;
#pragma unroll
  for (int u = 0; u < kMaxAcc; ++u) {
    const int o = w + kFmmWarps * u;
    if (o < np2 && on) dst[(size_t)o * kk] = acc[u];
  }
}

template <typename T>
__global__ void __launch_bounds__(kFmmThreads) k_fmm_up(FmmLevels<T> a) {
  extern __shared__ __align__(16) unsigned char fmm_smem[];
  const int np = a.np, np2 = np * np, w1 = a.w1, Bq = a.Bq, kk = a.kk;
  const FmmSmem<T> s = carve<T>(fmm_smem, np, w1, Bq, true);
  const int P = blockIdx.x, chunk = blockIdx.y, c0 = chunk * kFmmCols;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool on = c0 + lane < kk;
  const int L = a.L;
  load_factors(s, a.fac, a.cmap, np, w1, Bq);
  // the 4 leaf clusters' superspace panels
  for (int r = w; r < 4 * Bq; r += kFmmWarps)
    s.X[r * kFmmCols + lane] = on ? a.x[((size_t)4 * P * Bq + r) * kk + c0 + lane] : T(0);
  __syncthreads();
  T acc[kMaxAcc];
#pragma unroll
  for (int u = 0; u < kMaxAcc; ++u) acc[u] = T(0);
  for (int j = 0; j < 4; ++j) {
    const T* Xj = s.X + (size_t)j * Bq * kFmmCols;
    // moments, s direction: W[i][b] = sum_a Ms[i][a] X[q(a, b)]
    for (int o = w; o < np * w1; o += kFmmWarps) {
      const int i = o / w1, b = o - i * w1;
      T v = T(0);
      for (int aa = 0; aa < w1; ++aa) v = fma(s.Ms[i * w1 + aa], Xj[s.q_of[aa * w1 + b] * kFmmCols + lane], v);
      s.W[o * kFmmCols + lane] = v;
    }
    __syncthreads();
    // moments, t direction: C[i][i2] = sum_b W[i][b] Mt[i2][b]; written out as Y_L
    T* yl = a.y[L] + ((size_t)(4 * P + j) * np2) * kk + c0 + lane;
    for (int o = w; o < np2; o += kFmmWarps) {
      const int i = o / np, i2 = o - i * np;
      T v = T(0);
      for (int b = 0; b < w1; ++b) v = fma(s.W[(i * w1 + b) * kFmmCols + lane], s.Mt[i2 * w1 + b], v);
      s.C[o * kFmmCols + lane] = v;
      if (on) yl[(size_t)o * kk] = v;
    }
    __syncthreads();
    up_stage1(s.E + half_t(j) * np2, s.C, s.V, np, w, lane);
    __syncthreads();
    up_stage2(s.E + half_s(j) * np2, s.V, acc, np, w, lane);
  }
  {
    T* dst = a.y[L - 1] + ((size_t)P * np2) * kk + c0 + lane;
#pragma unroll
    for (int u = 0; u < kMaxAcc; ++u) {
      const int o = w + kFmmWarps * u;
      if (o < np2 && on) dst[(size_t)o * kk] = acc[u];
    }
  }
  // climb: the last of 4 siblings to finish transfers them to their parent
  __shared__ int last;
  int cur = P;
  for (int l = L - 2; l >= 0; --l) {
    __syncthreads();  // every store of level l + 1 issued
    if (threadIdx.x == 0) {
      __threadfence();
      int* cnt = a.cnt + a.cnt_off[l] + (size_t)chunk * a.cnt_stride + (cur >> 2);
      const int old = atomicAdd(cnt, 1);
      last = old == 3;
      if (last) {
        *cnt = 0;  // ready for the next launch
        __threadfence();
      }
    }
    __syncthreads();
    if (!last) return;
    cur >>= 2;
    transfer_up_from_global(s, a.y[l + 1], a.y[l], cur, np, kk, c0);
  }
}

// W[ps][ct] = sum_pt Et[ct][pt] Z[ps][pt]   (transposed transfer, t direction)
template <typename T>
__device__ __forceinline__ void down_stage1(const T* Et, const T* Z, T* W, int np, int w, int lane) {
  const int np2 = np * np;
  for (int o = w; o < np2; o += kFmmWarps) {
    const int ps = o / np, ct = o - ps * np;
    T v = T(0);
    for (int pt = 0; pt < np; ++pt) v = fma(Et[ct * np + pt], Z[(ps * np + pt) * kFmmCols + lane], v);
    W[o * kFmmCols + lane] = v;
  }
}
// out[cs][ct] = base[cs][ct] + sum_ps Es[cs][ps] W[ps][ct]  (s direction);
// base read from global (this level's far-field result)
template <typename T>
__device__ __forceinline__ void down_stage2(const T* Es, const T* W, const T* base, int kk, bool on, T* out, int np,
                                            int w, int lane) {
  const int np2 = np * np;
  for (int o = w; o < np2; o += kFmmWarps) {
    const int cs = o / np, ct = o - cs * np;
    T v = on ? base[(size_t)o * kk] : T(0);
    for (int ps = 0; ps < np; ++ps) v = fma(Es[cs * np + ps], W[(ps * np + ct) * kFmmCols + lane], v);
    out[o * kFmmCols + lane] = v;
  }
}

template <typename T>
__global__ void __launch_bounds__(kFmmThreads) k_fmm_down(FmmLevels<T> a) {
  extern __shared__ __align__(16) unsigned char fmm_smem[];
  const int np = a.np, np2 = np * np, w1 = a.w1, Bq = a.Bq, kk = a.kk;
  const FmmSmem<T> s = carve<T>(fmm_smem, np, w1, Bq, false);
  const int P = blockIdx.x, c0 = blockIdx.y * kFmmCols;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool on = c0 + lane < kk;
  const int L = a.L;
  load_factors(s, a.fac, a.cmap, np, w1, Bq);
  // full coefficients of the level-0 ancestor: its far-field result
  {
    const T* z0 = a.z[0] + ((size_t)(P >> (2 * (L - 1))) * np2) * kk + c0 + lane;
    for (int o = w; o < np2; o += kFmmWarps) s.Zf[o * kFmmCols + lane] = on ? z0[(size_t)o * kk] : T(0);
  }
  __syncthreads();
  // down the ancestor path to the parent P at level L - 1
  for (int l = 1; l <= L - 1; ++l) {
    const int al = P >> (2 * (L - 1 - l)), k = al & 3;
    down_stage1(s.E + half_t(k) * np2, s.Zf, s.W, np, w, lane);
    __syncthreads();
    down_stage2(s.E + half_s(k) * np2, s.W, a.z[l] + ((size_t)al * np2) * kk + c0 + lane, kk, on, s.Zf, np, w,
                lane);
    __syncthreads();
  }
  for (int j = 0; j < 4; ++j) {
    const int leaf = 4 * P + j;
    down_stage1(s.E + half_t(j) * np2, s.Zf, s.W, np, w, lane);
    __syncthreads();
    down_stage2(s.E + half_s(j) * np2, s.W, a.z[L] + ((size_t)leaf * np2) * kk + c0 + lane, kk, on, s.C, np, w,
                lane);
    __syncthreads();
    // transposed moments, t direction: V[i][b] = sum_j Mt[j][b] C[i][j]
    for (int o = w; o < np * w1; o += kFmmWarps) {
      const int i = o / w1, b = o - i * w1;
      T v = T(0);
      for (int jj = 0; jj < np; ++jj) v = fma(s.Mt[jj * w1 + b], s.C[(i * np + jj) * kFmmCols + lane], v);
      s.V[o * kFmmCols + lane] = v;
    }
    __syncthreads();
    // s direction: y[q(a, b)] += sum_i Ms[i][a] V[i][b]
    T* yo = a.out + ((size_t)leaf * Bq) * kk + c0 + lane;
    for (int o = w; o < w1 * w1; o += kFmmWarps) {
      const int aa = o / w1, b = o - aa * w1;
      T v = T(0);
      for (int i = 0; i < np; ++i) v = fma(s.Ms[i * w1 + aa], s.V[(i * w1 + b) * kFmmCols + lane], v);
      if (on) {
        T* dst = yo + (size_t)s.q_of[o] * kk;
        *dst += v;
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// The same two passes with the sizes fixed at compile time (n_p and the 1-D
// moment width w1 of the common discretisations). The 1-D factors travel in
// the kernel parameters, so with every loop unrolled each multiply-add takes
// its factor straight from the constant bank; a warp owns one row (or column)
// of the 2-D coefficient grid per stage and keeps that row's data in
// registers, so shared memory is read once per operand row, not per
// multiply-add. One warp per point row: NP warps.
template <typename T, int NP, int W1>
struct FmmFactors {
  T E[2][NP * NP];  // E[h][c * NP + p]
  T Ms[NP * W1];    // Ms[i * W1 + a]
  T Mt[NP * W1];
};

// V[cs][pt] = sum_ct E_H[ct][pt] C[cs][ct]; warp = cs
template <typename T, int NP, int W1, int H>
__device__ __forceinline__ void tup1(const FmmFactors<T, NP, W1>& f, const T* C, T* V, int w, int lane) {
  if (w >= NP) return;
  T c[NP];
#pragma unroll
  for (int ct = 0; ct < NP; ++ct) c[ct] = C[(w * NP + ct) * kFmmCols + lane];
#pragma unroll
  for (int pt = 0; pt < NP; ++pt) {
    T v = T(0);
#pragma unroll
    for (int ct = 0; ct < NP; ++ct) v = fma(f.E[H][ct * NP + pt], c[ct], v);
    V[(w * NP + pt) * kFmmCols + lane] = v;
  }
}
// acc[ps] += sum_cs E_H[cs][ps] V[cs][pt]; warp = pt
template <typename T, int NP, int W1, int H>
__device__ __forceinline__ void tup2(const FmmFactors<T, NP, W1>& f, const T* V, T* acc, int w, int lane) {
  if (w >= NP) return;
  T v[NP];
#pragma unroll
  for (int cs = 0; cs < NP; ++cs) v[cs] = V[(cs * NP + w) * kFmmCols + lane];
#pragma unroll
  for (int ps = 0; ps < NP; ++ps) {
    T a = acc[ps];
#pragma unroll
    for (int cs = 0; cs < NP; ++cs) a = fma(f.E[H][cs * NP + ps], v[cs], a);
    acc[ps] = a;
  }
}
// child K of a parent: both transfer stages, summed into acc
template <typename T, int NP, int W1, int K>
__device__ __forceinline__ void tup_child(const FmmFactors<T, NP, W1>& f, const T* C, T* V, T* acc, int w,
                                          int lane) {
  constexpr int HT = K >> 1, HS = (K == 1 || K == 2) ? 1 : 0;
  tup1<T, NP, W1, HT>(f, C, V, w, lane);
  __syncthreads();
  tup2<T, NP, W1, HS>(f, V, acc, w, lane);
  __syncthreads();
}
// moments of one leaf cluster: W[i][b] = sum_a Ms[i][a] X[q(a, b)] (warp = b),
// then C[i][i2] = sum_b Mt[i2][b] W[i][b] (warp = i), written to yout too
template <typename T, int NP, int W1>
__device__ __forceinline__ void tmom(const FmmFactors<T, NP, W1>& f, const T* X, const int* q_of, T* W, T* C,
                                     T* yout, int kk, bool on, int w, int lane) {
  if (w < W1) {
    T x[W1];
#pragma unroll
    for (int a = 0; a < W1; ++a) x[a] = X[q_of[a * W1 + w] * kFmmCols + lane];
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      T v = T(0);
#pragma unroll
      for (int a = 0; a < W1; ++a) v = fma(f.Ms[i * W1 + a], x[a], v);
      W[(i * W1 + w) * kFmmCols + lane] = v;
    }
  }
  __syncthreads();
  if (w < NP) {
    T wv[W1];
#pragma unroll
    for (int b = 0; b < W1; ++b) wv[b] = W[(w * W1 + b) * kFmmCols + lane];
#pragma unroll
    for (int i2 = 0; i2 < NP; ++i2) {
      T v = T(0);
#pragma unroll
      for (int b = 0; b < W1; ++b) v = fma(f.Mt[i2 * W1 + b], wv[b], v);
      C[(w * NP + i2) * kFmmCols + lane] = v;
      if (on) yout[(size_t)(w * NP + i2) * kk] = v;
    }
  }
  __syncthreads();
}

template <typename T, int NP, int W1>
__global__ void __launch_bounds__(32 * NP) k_fmm_up_t(const __grid_constant__ FmmLevels<T> a, const __grid_constant__ FmmFactors<T, NP, W1> f) {
  extern __shared__ __align__(16) unsigned char fmm_smem[];
  constexpr int NP2 = NP * NP, BQ = W1 * W1, NW = NP;
  // X [4 BQ][32] | W [NP W1][32] | C [NP2][32], then V [NP2][32] after
  // FRONT rows; the climb reuses the front as Cg [4 NP2][32]
  constexpr int FRONT = (4 * BQ + NP * W1 + NP2) > 4 * NP2 ? (4 * BQ + NP * W1 + NP2) : 4 * NP2;
  T* X = reinterpret_cast<T*>(fmm_smem);
  T* W = X + 4 * BQ * kFmmCols;
  T* C = W + NP * W1 * kFmmCols;
  T* V = X + FRONT * kFmmCols;
  int* q_of = reinterpret_cast<int*>(V + NP2 * kFmmCols);
  T* Cg = X;
  const int P = blockIdx.x, chunk = blockIdx.y, c0 = chunk * kFmmCols, kk = a.kk, L = a.L;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool on = c0 + lane < kk;
  for (int q = threadIdx.x; q < BQ; q += blockDim.x) {
    const int ab = a.cmap[q];
    q_of[(ab & 0xFF) * W1 + (ab >> 8)] = q;
  }
  for (int r = w; r < 4 * BQ; r += NW)
    X[r * kFmmCols + lane] = on ? a.x[((size_t)4 * P * BQ + r) * kk + c0 + lane] : T(0);
  __syncthreads();
  T acc[NP];
#pragma unroll
  for (int u = 0; u < NP; ++u) acc[u] = T(0);
  auto leaf = [&](auto kc) {
    constexpr int K = decltype(kc)::value;
    tmom<T, NP, W1>(f, X + K * BQ * kFmmCols, q_of, W, C, a.y[L] + ((size_t)(4 * P + K) * NP2) * kk + c0 + lane,
                    kk, on, w, lane);
    tup_child<T, NP, W1, K>(f, C, V, acc, w, lane);
  };
  leaf(std::integral_constant<int, 0>());
  leaf(std::integral_constant<int, 1>());
  leaf(std::integral_constant<int, 2>());
  leaf(std::integral_constant<int, 3>());
  // warp pt holds column pt of the parent's coefficients
  auto store = [&](T* dst) {
    if (w < NP && on)
#pragma unroll
      for (int ps = 0; ps < NP; ++ps) dst[(size_t)(ps * NP + w) * kk] = acc[ps];
  };
  store(a.y[L - 1] + ((size_t)P * NP2) * kk + c0 + lane);
  __shared__ int last;
  int cur = P;
  for (int l = L - 2; l >= 0; --l) {
    __syncthreads();  // every store of level l + 1 issued
    if (threadIdx.x == 0) {
      __threadfence();
      int* cnt = a.cnt + a.cnt_off[l] + (size_t)chunk * a.cnt_stride + (cur >> 2);
      const int old = atomicAdd(cnt, 1);
      last = old == 3;
      if (last) {
        *cnt = 0;  // ready for the next launch
        __threadfence();
      }
    }
    __syncthreads();
    if (!last) return;
    cur >>= 2;
    const T* src = a.y[l + 1] + ((size_t)4 * cur * NP2) * kk + c0 + lane;
    for (int r = w; r < 4 * NP2; r += NW) Cg[r * kFmmCols + lane] = on ? __ldcg(src + (size_t)r * kk) : T(0);
    __syncthreads();
#pragma unroll
    for (int u = 0; u < NP; ++u) acc[u] = T(0);
    tup_child<T, NP, W1, 0>(f, Cg, V, acc, w, lane);
    tup_child<T, NP, W1, 1>(f, Cg + NP2 * kFmmCols, V, acc, w, lane);
    tup_child<T, NP, W1, 2>(f, Cg + 2 * NP2 * kFmmCols, V, acc, w, lane);
    tup_child<T, NP, W1, 3>(f, Cg + 3 * NP2 * kFmmCols, V, acc, w, lane);
    store(a.y[l] + ((size_t)cur * NP2) * kk + c0 + lane);
  }
}

// W[ps][ct] = sum_pt E_H[ct][pt] Z[ps][pt]; warp = ps
template <typename T, int NP, int W1, int H>
__device__ __forceinline__ void tdown1(const FmmFactors<T, NP, W1>& f, const T* Z, T* W, int w, int lane) {
  if (w >= NP) return;
  T z[NP];
#pragma unroll
  for (int pt = 0; pt < NP; ++pt) z[pt] = Z[(w * NP + pt) * kFmmCols + lane];
#pragma unroll
  for (int ct = 0; ct < NP; ++ct) {
    T v = T(0);
#pragma unroll
    for (int pt = 0; pt < NP; ++pt) v = fma(f.E[H][ct * NP + pt], z[pt], v);
    W[(w * NP + ct) * kFmmCols + lane] = v;
  }
}
// out[cs][ct] = base[cs] + sum_ps E_H[cs][ps] W[ps][ct]; warp = ct, base[cs]
// the far-field result of row (cs, ct), already in registers
template <typename T, int NP, int W1, int H>
__device__ __forceinline__ void tdown2(const FmmFactors<T, NP, W1>& f, const T* W, const T* base, T* out, int w,
                                       int lane) {
  if (w >= NP) return;
  T v[NP];
#pragma unroll
  for (int ps = 0; ps < NP; ++ps) v[ps] = W[(ps * NP + w) * kFmmCols + lane];
#pragma unroll
  for (int cs = 0; cs < NP; ++cs) {
    T o = base[cs];
#pragma unroll
    for (int ps = 0; ps < NP; ++ps) o = fma(f.E[H][cs * NP + ps], v[ps], o);
    out[(cs * NP + w) * kFmmCols + lane] = o;
  }
}
template <typename T, int NP, int W1, int K>
__device__ __forceinline__ void tdown_child(const FmmFactors<T, NP, W1>& f, const T* Zp, T* W, const T* base, T* out,
                                            int w, int lane) {
  constexpr int HT = K >> 1, HS = (K == 1 || K == 2) ? 1 : 0;
  tdown1<T, NP, W1, HT>(f, Zp, W, w, lane);
  __syncthreads();
  tdown2<T, NP, W1, HS>(f, W, base, out, w, lane);
  __syncthreads();
}

// The downward pass as one sequence of steps: the L - 1 ancestors below
// level 0 (full coefficients in Zf, updated in place), then the 4 leaf
// clusters (into C, then the transposed moments). Each step's far-field rows
// are loaded into registers one step ahead, and each leaf's superspace rows
// before its transfer, so that global-memory latency overlaps the arithmetic.
template <typename T, int NP, int W1>
__global__ void __launch_bounds__(32 * NP) k_fmm_down_t(const __grid_constant__ FmmLevels<T> a, const __grid_constant__ FmmFactors<T, NP, W1> f) {
  extern __shared__ __align__(16) unsigned char fmm_smem[];
  constexpr int NP2 = NP * NP, BQ = W1 * W1, NW = NP;
  // Zf [NP2][32] | W [NP2][32] | C [NP2][32] | V [NP W1][32]
  T* Zf = reinterpret_cast<T*>(fmm_smem);
  T* W = Zf + NP2 * kFmmCols;
  T* C = W + NP2 * kFmmCols;
  T* V = C + NP2 * kFmmCols;
  int* q_of = reinterpret_cast<int*>(V + NP * W1 * kFmmCols);
  const int P = blockIdx.x, c0 = blockIdx.y * kFmmCols, kk = a.kk, L = a.L;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool on = c0 + lane < kk;
  for (int q = threadIdx.x; q < BQ; q += blockDim.x) {
    const int ab = a.cmap[q];
    q_of[(ab & 0xFF) * W1 + (ab >> 8)] = q;
  }
  {
    const T* z0 = a.z[0] + ((size_t)(P >> (2 * (L - 1))) * NP2) * kk + c0 + lane;
    for (int r = w; r < NP2; r += NW) Zf[r * kFmmCols + lane] = on ? z0[(size_t)r * kk] : T(0);
  }
  const int nsteps = L - 1 + 4;
  // far-field rows (cs, w) of step st: ancestor level st + 1, then leaf st - (L - 1)
  auto rows_of = [&](int st) -> const T* {
    if (st < L - 1) {
      const int l = st + 1;
      return a.z[l] + ((size_t)(P >> (2 * (L - 1 - l))) * NP2) * kk + c0 + lane;
    }
    return a.z[L] + ((size_t)(4 * P + st - (L - 1)) * NP2) * kk + c0 + lane;
  };
  T nb[NP];
  auto load_rows = [&](int st) {
    const T* p = rows_of(st);
#pragma unroll
    for (int cs = 0; cs < NP; ++cs) nb[cs] = (on && w < NP) ? p[(size_t)(cs * NP + w) * kk] : T(0);
  };
  load_rows(0);
  __syncthreads();
  for (int st = 0; st < nsteps; ++st) {
    T cb[NP];
#pragma unroll
    for (int cs = 0; cs < NP; ++cs) cb[cs] = nb[cs];
    if (st + 1 < nsteps) load_rows(st + 1);
    const bool leaf = st >= L - 1;
    const int lf = 4 * P + st - (L - 1);
    // this leaf's superspace rows, read-modify-written by warp b < W1
    T yv[W1];
    T* yo = a.out + ((size_t)lf * BQ) * kk + c0 + lane;
    if (leaf && w < W1 && on) {
#pragma unroll
      for (int aa = 0; aa < W1; ++aa) yv[aa] = yo[(size_t)q_of[aa * W1 + w] * kk];
    }
    const int k = leaf ? st - (L - 1) : ((P >> (2 * (L - 2 - st))) & 3);
    T* dst = leaf ? C : Zf;
    switch (k) {
      case 0: tdown_child<T, NP, W1, 0>(f, Zf, W, cb, dst, w, lane); break;
      case 1: tdown_child<T, NP, W1, 1>(f, Zf, W, cb, dst, w, lane); break;
      case 2: tdown_child<T, NP, W1, 2>(f, Zf, W, cb, dst, w, lane); break;
      default: tdown_child<T, NP, W1, 3>(f, Zf, W, cb, dst, w, lane); break;
    }
    if (!leaf) continue;
    // transposed moments: V[i][b] = sum_j Mt[j][b] C[i][j] (warp = i), then
    // y[q(a, b)] += sum_i Ms[i][a] V[i][b] (warp = b)
    if (w < NP) {
      T c[NP];
#pragma unroll
      for (int j = 0; j < NP; ++j) c[j] = C[(w * NP + j) * kFmmCols + lane];
#pragma unroll
      for (int b = 0; b < W1; ++b) {
        T v = T(0);
#pragma unroll
        for (int j = 0; j < NP; ++j) v = fma(f.Mt[j * W1 + b], c[j], v);
        V[(w * W1 + b) * kFmmCols + lane] = v;
      }
    }
    __syncthreads();
    if (w < W1) {
      T v[NP];
#pragma unroll
      for (int i = 0; i < NP; ++i) v[i] = V[(i * W1 + w) * kFmmCols + lane];
#pragma unroll
      for (int aa = 0; aa < W1; ++aa) {
        T o = T(0);
#pragma unroll
        for (int i = 0; i < NP; ++i) o = fma(f.Ms[i * W1 + aa], v[i], o);
        if (on) yo[(size_t)q_of[aa * W1 + w] * kk] = yv[aa] + o;
      }
    }
    __syncthreads();
  }
}

template <typename T, int NP, int W1>
cudaError_t fmm_launch_t(bool up, const FmmLevels<T>& a, const double* hfac, int nparents, cudaStream_t s) {
  constexpr int NP2 = NP * NP, BQ = W1 * W1;
  FmmFactors<T, NP, W1> f;
  for (int h = 0; h < 2; ++h)
    for (int e = 0; e < NP2; ++e) f.E[h][e] = (T)hfac[h * NP2 + e];
  for (int e = 0; e < NP * W1; ++e) {
    f.Ms[e] = (T)hfac[2 * NP2 + e];
    f.Mt[e] = (T)hfac[2 * NP2 + NP * W1 + e];
  }
  constexpr int FRONT = (4 * BQ + NP * W1 + NP2) > 4 * NP2 ? (4 * BQ + NP * W1 + NP2) : 4 * NP2;
  const size_t smem = up ? sizeof(T) * kFmmCols * (FRONT + NP2) + sizeof(int) * BQ
                         : sizeof(T) * kFmmCols * (3 * NP2 + NP * W1) + sizeof(int) * BQ;
  const dim3 grid(nparents, (a.kk + kFmmCols - 1) / kFmmCols);
  if (up) {
    cudaError_t e = smem_limit(k_fmm_up_t<T, NP, W1>, smem);
    if (e != cudaSuccess) return e;
    k_fmm_up_t<T, NP, W1><<<grid, 32 * NP, smem, s>>>(a, f);
  } else {
    cudaError_t e = smem_limit(k_fmm_down_t<T, NP, W1>, smem);
    if (e != cudaSuccess) return e;
    k_fmm_down_t<T, NP, W1><<<grid, 32 * NP, smem, s>>>(a, f);
  }
  return cudaGetLastError();
}

template <typename T>
size_t fmm_smem_bytes(int np, int w1, int Bq, bool with_x) {
  auto a16 = [](size_t n) { return (n * sizeof(T) + 15) / 16 * 16; };
  const int np2 = np * np, wrows = std::max(np * w1, np2);
  return a16(2 * np2) + 2 * a16(np * w1) +
         sizeof(T) * kFmmCols * ((with_x ? (size_t)4 * Bq : 0) + wrows + 3 * (size_t)np2) +
         sizeof(int) * (size_t)w1 * w1;
}

template <typename T>
cudaError_t fmm_launch(bool up, const FmmLevels<T>& a, const double* hfac, int nparents, cudaStream_t s) {
  if (nparents == 0 || a.kk == 0) return cudaSuccess;
  if (a.L < 1 || a.L >= kMaxFarLevels || a.np < 2 || a.np > kFmmMaxNp || a.w1 < 1 || a.w1 * a.w1 != a.Bq ||
      a.w1 > 16)
    return cudaErrorInvalidValue;
  // compiled sizes: n_p 6, 9, 10 with P = 1, 2 (w1 = 4, 6)
  if (hfac) {
#define BG_FMM_T(NPV, W1V) \
  if (a.np == NPV && a.w1 == W1V) return fmm_launch_t<T, NPV, W1V>(up, a, hfac, nparents, s);
    BG_FMM_T(6, 4) BG_FMM_T(6, 6) BG_FMM_T(9, 4) BG_FMM_T(9, 6) BG_FMM_T(10, 4) BG_FMM_T(10, 6)
#undef BG_FMM_T
  }
  const size_t smem = fmm_smem_bytes<T>(a.np, a.w1, a.Bq, up);
  if (smem > 200 * 1024) return cudaErrorInvalidValue;
  auto kf = up ? k_fmm_up<T> : k_fmm_down<T>;
  cudaError_t e = smem_limit(kf, smem);
  if (e != cudaSuccess) return e;
  const dim3 grid(nparents, (a.kk + kFmmCols - 1) / kFmmCols);
  kf<<<grid, kFmmThreads, smem, s>>>(a);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_fmm_up(int S, const FmmLevelsAny& a, const double* hfac, int nparents, cudaStream_t s) {
  if (S < 2) return fmm_launch<double>(true, a.f64, hfac, nparents, s);
  return fmm_launch<float>(true, a.f32, hfac, nparents, s);
}
cudaError_t launch_fmm_down(int S, const FmmLevelsAny& a, const double* hfac, int nparents, cudaStream_t s) {
  if (S < 2) return fmm_launch<double>(false, a.f64, hfac, nparents, s);
  return fmm_launch<float>(false, a.f32, hfac, nparents, s);
}

}  // namespace bg
