// Krylov solve, load vectors and potential evaluation on GB300.
//
// bg_solve: restarted GMRES (Saad & Schultz 1986) batched over right-hand
// sides with classical Gram-Schmidt applied twice and an FP64 Krylov basis.
// FP64 path: GMRES on the FP64 H2 matrix. Mixed path: flexible GMRES (Saad
// 1993) on the FP64 operator whose right preconditioner is an inner GMRES solve
// with a low-precision operator (BG_PREC_MIXED: FP64 near field, FP32 far
// field; BG_PREC_FP32: both in FP32): every outer step
// is one FP64 residual-consistent product, the inner steps are cheap, and the
// outer Krylov space recovers the FP64 solution. Replaces the Eigen solvers
// used at examples/LaplaceSingleLayerH2.cpp:78-81 and
// examples/HelmholtzSingleLayerH2.cpp:82-85.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

#include "bg_operator.hpp"

using namespace bg;

namespace {

template <typename S> __device__ inline S conj_mul(S a, S b);
template <> __device__ inline double conj_mul<double>(double a, double b) { return a * b; }
template <> __device__ inline cd conj_mul<cd>(cd a, cd b) { return {a.re * b.re + a.im * b.im, a.re * b.im - a.im * b.re}; }
__device__ inline double sub(double a, double b) { return a - b; }
__device__ inline cd sub(cd a, cd b) { return a - b; }
__device__ inline double addv(double a, double b) { return a + b; }
__device__ inline cd addv(cd a, cd b) { return a + b; }

// out[i][c] = sum_n conj(V[i][n][c]) w[n][c] for i < nv (one CTA per i)
// (any k: with more columns than threads each thread sums whole columns)
template <typename S>
__global__ void k_mdot(const S* __restrict__ V, long vstride, const S* __restrict__ w, int N, int k, S* __restrict__ out) {
  __shared__ S red[256];
  const int i = blockIdx.x;
  const int kp = k;  // columns
  if (kp > (int)blockDim.x) {
    const S* v = V + (long)i * vstride;
    for (int c = threadIdx.x; c < kp; c += blockDim.x) {
      S acc = zero<S>();
      for (int n = 0; n < N; ++n) acc = addv(acc, conj_mul(v[(long)n * k + c], w[(long)n * k + c]));
      out[(long)i * k + c] = acc;
    }
    return;
  }
  const int groups = blockDim.x / kp;
  const int c = threadIdx.x % kp, g = threadIdx.x / kp;
  S acc = zero<S>();
  if (g < groups) {
    const S* v = V + (long)i * vstride;
    for (int n = g; n < N; n += groups) acc = addv(acc, conj_mul(v[(long)n * k + c], w[(long)n * k + c]));
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.x < kp) {
    S s = zero<S>();
    for (int gg = 0; gg < groups; ++gg) s = addv(s, red[gg * kp + threadIdx.x]);
    out[(long)i * k + threadIdx.x] = s;
  }
}
// Blocked dot products for many vectors at once: CTA (i, chunk) reduces rows
// [chunk*rows_per, ...) of V_i^H w for all k columns into part[(i*nch + chunk)*k + c];
// k_reduce_parts then sums the chunks in a fixed order (deterministic).
template <typename S>
__global__ void k_mdot_part(const S* __restrict__ V, long vstride, const S* __restrict__ w, int N, int k, int rows_per,
                            S* __restrict__ part) {
  __shared__ S red[256];
  const int i = blockIdx.x, ch = blockIdx.y, nch = gridDim.y;
  const int n0 = ch * rows_per, n1 = min(N, n0 + rows_per);
  if (k > (int)blockDim.x) {  // more columns than threads: each thread sums whole columns of the chunk
    const S* v = V + (long)i * vstride;
    for (int c = threadIdx.x; c < k; c += blockDim.x) {
      S acc = zero<S>();
      for (int n = n0; n < n1; ++n) acc = addv(acc, conj_mul(v[(long)n * k + c], w[(long)n * k + c]));
      part[((long)i * nch + ch) * k + c] = acc;
    }
    return;
  }
  const int groups = blockDim.x / k;
  const int c = threadIdx.x % k, g = threadIdx.x / k;
  S acc = zero<S>();
  if (g < groups) {
    const S* v = V + (long)i * vstride;
    for (int n = n0 + g; n < n1; n += groups) acc = addv(acc, conj_mul(v[(long)n * k + c], w[(long)n * k + c]));
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.x < k) {
    S s2 = zero<S>();
    for (int gg = 0; gg < groups; ++gg) s2 = addv(s2, red[gg * k + threadIdx.x]);
    part[((long)i * nch + ch) * k + threadIdx.x] = s2;
  }
}
template <typename S>
__global__ void k_reduce_parts(const S* __restrict__ part, int nv, int nch, int k, S* __restrict__ out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nv * k) return;
  const int i = t / k, c = t % k;
  S s2 = zero<S>();
  for (int ch = 0; ch < nch; ++ch) s2 = addv(s2, part[((long)i * nch + ch) * k + c]);
  out[(long)i * k + c] = s2;
}

// w[n][c] -= sum_{i<nv} V[i][n][c] h[i][c]
template <typename S>
__global__ void k_vupdate(const S* __restrict__ V, long vstride, int nv, const S* __restrict__ h, int N, int k,
                          S* __restrict__ w) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)N * k) return;
  const int c = (int)(t % k);
  S acc = w[t];
  for (int i = 0; i < nv; ++i) acc = sub(acc, V[(long)i * vstride + t] * h[(long)i * k + c]);
  w[t] = acc;
}
// inv[c] = 1 / sqrt(|d[c]|) (0 when d[c] == 0), from a Gram column of w with itself
template <typename S>
__global__ void k_inv_norm(const S* __restrict__ d, int k, double* __restrict__ inv);
template <>
__global__ void k_inv_norm<double>(const double* __restrict__ d, int k, double* __restrict__ inv) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < k) inv[c] = d[c] > 0 ? 1.0 / sqrt(d[c]) : 0.0;
}
template <>
__global__ void k_inv_norm<cd>(const cd* __restrict__ d, int k, double* __restrict__ inv) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < k) inv[c] = d[c].re > 0 ? 1.0 / sqrt(d[c].re) : 0.0;
}
// V_next[n][c] = w[n][c] * inv[c]
template <typename S>
__global__ void k_vscale(const S* __restrict__ w, const double* __restrict__ inv, int N, int k, S* __restrict__ out) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)N * k) return;
  out[t] = w[t] * inv[t % k];
}
// x[n][c] += sum_i V[i][n][c] y[i][c]
template <typename S>
__global__ void k_xupdate(const S* __restrict__ V, long vstride, int nv, const S* __restrict__ y, int N, int k,
                          S* __restrict__ x) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)N * k) return;
  const int c = (int)(t % k);
  S acc = x[t];
  for (int i = 0; i < nv; ++i) acc = addv(acc, V[(long)i * vstride + t] * y[(long)i * k + c]);
  x[t] = acc;
}
// r = b - r (in place on r)
template <typename S>
__global__ void k_residual(const S* __restrict__ b, long n, S* __restrict__ r) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) r[t] = sub(b[t], r[t]);
}
inline unsigned nblk(long n) { return (unsigned)((n + 255) / 256); }

}  // namespace

// ---------------------------------------------------------------------------
namespace {

struct Krylov {
  bg_operator* op;
  int N, k, m;
  bool flexible;          // store the preconditioned directions Z
  DevBuf V, Z, w, hdev, inv, ydev, part, r;
  size_t hpin_bytes = 0;
  // two pinned slots for the Hessenberg column of an Arnoldi step (h1, h2,
  // norm), each with an event, so the host reads step j while step j+1 runs
  void* hpin = nullptr;
  size_t slot_bytes = 0;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  Krylov() {}
  Krylov(const Krylov&) = delete;
  Krylov& operator=(const Krylov&) = delete;
  ~Krylov() {
    if (hpin) cudaFreeHost(hpin);
    for (auto& x : ev)
      if (x) cudaEventDestroy(x);
  }
  bg_status init(bg_operator* o, int kk, int mm, bool flex, size_t sb) {
    op = o;
    N = o->N;
    k = kk;
    m = mm;
    flexible = flex;
    const long nk = (long)N * k;
    cudaError_t e = V.alloc((size_t)(m + 1) * nk * sb);
    if (e == cudaSuccess && flex) e = Z.alloc((size_t)m * nk * sb);
    if (e == cudaSuccess) e = w.alloc(nk * sb);
    if (e == cudaSuccess) e = hdev.alloc((size_t)3 * (m + 1) * k * sb);
    if (e == cudaSuccess) e = part.alloc((size_t)(m + 1) * 64 * k * sb);
    if (e == cudaSuccess) e = inv.alloc(k * sizeof(double));
    if (e == cudaSuccess) e = ydev.alloc((size_t)(m + 1) * k * sb);
    if (e == cudaSuccess) e = r.alloc(nk * sb);
    // buffers are kept between solves and grown only when needed
    slot_bytes = (size_t)(2 * (m + 1) + 1) * k * sb;
    if (e == cudaSuccess && 2 * slot_bytes > hpin_bytes) {
      if (hpin) cudaFreeHost(hpin);
      hpin = nullptr;
      hpin_bytes = 0;
      e = cudaMallocHost(&hpin, 2 * slot_bytes);
      if (e == cudaSuccess) hpin_bytes = 2 * slot_bytes;
    }
    for (auto& x : ev)
      if (e == cudaSuccess && !x) e = cudaEventCreateWithFlags(&x, cudaEventDisableTiming);
    return cuda_status(o->ctx, e, "solver workspace");
  }
};

// Solver workspaces of an operator, kept between bg_solve calls so that a
// solve allocates nothing once the sizes have been seen (and no cudaFree
// synchronises the device inside a solve)
struct SolverWS {
  Krylov plain, outer, inner;
  DevBuf bw, xw, bu, xu;
};
void free_solver_ws(void* p) { delete static_cast<SolverWS*>(p); }
size_t krylov_bytes(const Krylov& k) {
  return k.V.bytes + k.Z.bytes + k.w.bytes + k.hdev.bytes + k.inv.bytes + k.ydev.bytes + k.part.bytes + k.r.bytes;
}
size_t solver_ws_bytes(const void* p) {
  const SolverWS* w = static_cast<const SolverWS*>(p);
  return krylov_bytes(w->plain) + krylov_bytes(w->outer) + krylov_bytes(w->inner) + w->bw.bytes + w->xw.bytes +
         w->bu.bytes + w->xu.bytes;
}
SolverWS* get_ws(bg_operator* op) {
  if (!op->solver_ws) {
    op->solver_ws = new SolverWS();
    op->solver_ws_free = free_solver_ws;
    op->solver_ws_bytes = solver_ws_bytes;
  }
  return static_cast<SolverWS*>(op->solver_ws);
}

template <typename S>
using HostS = typename std::conditional<std::is_same<S, double>::value, double, std::complex<double>>::type;
inline double cj(double v) { return v; }
inline std::complex<double> cj(std::complex<double> v) { return std::conj(v); }

// column norms of a row-major N x k block (FP64 work vector)
template <typename S>
bg_status col_norms(Krylov& K, const void* x, std::vector<double>* out) {
  cudaStream_t s = K.op->ctx->stream;
  timed_launch(K.op->ctx, KC_KRYLOV, [&] {
    k_mdot<S><<<1, 256, 0, s>>>(static_cast<const S*>(x), 0, static_cast<const S*>(x), K.N, K.k, K.hdev.as<S>());
    return cudaGetLastError();
  });
  std::vector<HostS<S>> h(K.k);
  cudaError_t e = cudaMemcpyAsync(h.data(), K.hdev.p, K.k * sizeof(S), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_status(K.op->ctx, e, "norms");
  out->resize(K.k);
  for (int c = 0; c < K.k; ++c) (*out)[c] = std::sqrt(std::abs(h[c]));
  return BG_OK;
}

struct Counters {
  int fp64_mv = 0, mixed_mv = 0, inner_it = 0, outer_it = 0;
};

// Right-preconditioned restarted (F)GMRES for A x = b on row-major FP64 work
// vectors; x must be zero on entry and is updated in place. A is the operator
// of precision prec. With a preconditioner (inner != nullptr)
// z_j = M^-1 v_j is an inner GMRES solve on the low-precision operator and the
// directions z_j are kept (flexible GMRES); otherwise z_j = v_j. Stops when
// every column's residual estimate is below tol * ||b_c||.
template <typename S>
bg_status fgmres(Krylov& K, int prec, Krylov* inner, int inner_prec, double inner_tol, int inner_max, const void* b,
                 void* x, double tol, int max_iter, Counters* cnt, std::vector<double>* relres, int gs_passes = 2) {
  const bool low = prec != BG_PREC_FP64;
  typedef HostS<S> H;
  bg_operator* op = K.op;
  cudaStream_t s = op->ctx->stream;
  const int N = K.N, k = K.k, m = K.m;
  const long nk = (long)N * k, vstride = nk;
  std::vector<double> bn;
  bg_status st = col_norms<S>(K, b, &bn);
  if (st != BG_OK) return st;
  DevBuf& r = K.r;
  cudaError_t e = cudaSuccess;
  std::vector<H> Hm((size_t)(m + 1) * m * k), g((size_t)(m + 1) * k), cs((size_t)m * k), sn((size_t)m * k);
  std::vector<H> hcol((size_t)(m + 1) * k);
  std::vector<double> inv(k), beta;
  int it = 0;
  bool first_cycle = true;
  while (true) {
    // true residual r = b - A x (x is zero on entry, so the first one is b)
    if (first_cycle) {
      e = cudaMemcpyAsync(r.p, b, nk * sizeof(S), cudaMemcpyDeviceToDevice, s);
      if (e != cudaSuccess) return cuda_status(op->ctx, e, "gmres");
      first_cycle = false;
    } else {
      if ((st = apply_operator(op, k, prec, x, r.p)) != BG_OK) return st;
      ++(low ? cnt->mixed_mv : cnt->fp64_mv);
      timed_launch(op->ctx, KC_KRYLOV, [&] {
        k_residual<S><<<nblk(nk), 256, 0, s>>>(static_cast<const S*>(b), nk, r.as<S>());
        return cudaGetLastError();
      });
    }
    if ((st = col_norms<S>(K, r.p, &beta)) != BG_OK) return st;
    bool done = true;
    for (int c = 0; c < k; ++c)
      if (beta[c] > tol * bn[c] && bn[c] > 0) done = false;
    if (relres) {
      relres->resize(k);
      for (int c = 0; c < k; ++c) (*relres)[c] = bn[c] > 0 ? beta[c] / bn[c] : 0.0;
    }
    if (done || it >= max_iter) break;
    for (int c = 0; c < k; ++c) inv[c] = beta[c] > 0 ? 1.0 / beta[c] : 0.0;
    e = cudaMemcpyAsync(K.inv.p, inv.data(), k * sizeof(double), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_status(op->ctx, e, "gmres");
    timed_launch(op->ctx, KC_KRYLOV, [&] {
      k_vscale<S><<<nblk(nk), 256, 0, s>>>(r.as<S>(), K.inv.as<double>(), N, k, K.V.as<S>());
      return cudaGetLastError();
    });
    std::fill(Hm.begin(), Hm.end(), H(0));
    std::fill(g.begin(), g.end(), H(0));
    for (int c = 0; c < k; ++c) g[c] = beta[c];
    // step count at which each column met the tolerance in this cycle (-1:
    // not yet): its update uses those steps only, so that columns that
    // converge early are not iterated further on a basis that keeps growing
    // for the others (with one Gram-Schmidt pass and a low-precision operator
    // that extra iteration spoils their directions)
    std::vector<int> jconv(k, -1);
    for (int c = 0; c < k; ++c)
      if (!(beta[c] > tol * bn[c] && bn[c] > 0)) jconv[c] = 0;
    // Arnoldi steps with the host one step behind (without an inner solve):
    // step jj+1 is launched (it needs only device data) before the host reads
    // step jj's Hessenberg column from its pinned slot, so the GPU does not wait
    // for the host. A step launched after the last needed one is wasted,
    // nothing else; its pinned slot is the other one of the two.
    const int it0 = it;
    auto launch_step = [&](int jj) -> bg_status {
        S* vj = K.V.as<S>() + (long)jj * vstride;
        const S* zj = vj;
        if (inner) {
          S* zdst = K.Z.as<S>() + (long)jj * vstride;
          e = cudaMemsetAsync(zdst, 0, nk * sizeof(S), s);
          if (e != cudaSuccess) return cuda_status(op->ctx, e, "gmres");
          Counters ic;
          // the inner solve only preconditions (tolerance ~1e-3): one Gram-Schmidt pass
          if ((st = fgmres<S>(*inner, inner_prec, nullptr, 0, 0, 0, vj, zdst, inner_tol, inner_max, &ic, nullptr, 1)) !=
              BG_OK)
            return st;
          cnt->mixed_mv += ic.mixed_mv;
          cnt->inner_it += ic.outer_it;
          zj = zdst;
        }
        if ((st = apply_operator(op, k, prec, zj, K.w.p)) != BG_OK) return st;
        ++(low ? cnt->mixed_mv : cnt->fp64_mv);
        // classical Gram-Schmidt (gs_passes passes: two for the outer and the plain
        // FP64 solve, one for the inner preconditioning solve) and the norm, on the device;
        // one copy brings the Hessenberg column back
        S* h1 = K.hdev.as<S>();
        S* h2 = h1 + (size_t)(m + 1) * k;
        S* h3 = h2 + (size_t)(m + 1) * k;
        for (int pass = 0; pass < gs_passes; ++pass) {
          S* hp = pass == 0 ? h1 : h2;
          // split the rows over enough CTAs to fill the GPU
          const int nch = std::max(1, std::min(64, (4 * 152 + jj) / (jj + 1)));
          const int rows_per = (N + nch - 1) / nch;
          timed_launch(op->ctx, KC_KRYLOV, [&] {
            k_mdot_part<S><<<dim3(jj + 1, nch), 256, 0, s>>>(K.V.as<S>(), vstride, K.w.as<S>(), N, k, rows_per,
                                                            K.part.as<S>());
            return cudaGetLastError();
          });
          timed_launch(op->ctx, KC_KRYLOV, [&] {
            k_reduce_parts<S><<<((jj + 1) * k + 255) / 256, 256, 0, s>>>(K.part.as<S>(), jj + 1, nch, k, hp);
            return cudaGetLastError();
          });
          timed_launch(op->ctx, KC_KRYLOV, [&] {
            k_vupdate<S><<<nblk(nk), 256, 0, s>>>(K.V.as<S>(), vstride, jj + 1, hp, N, k, K.w.as<S>());
            return cudaGetLastError();
          });
        }
        {
          const int nch = 64, rows_per = (N + nch - 1) / nch;
          timed_launch(op->ctx, KC_KRYLOV, [&] {
            k_mdot_part<S><<<dim3(1, nch), 256, 0, s>>>(K.w.as<S>(), 0, K.w.as<S>(), N, k, rows_per, K.part.as<S>());
            return cudaGetLastError();
          });
          timed_launch(op->ctx, KC_KRYLOV, [&] {
            k_reduce_parts<S><<<(k + 255) / 256, 256, 0, s>>>(K.part.as<S>(), 1, nch, k, h3);
            return cudaGetLastError();
          });
        }
        timed_launch(op->ctx, KC_KRYLOV, [&] {
          k_inv_norm<S><<<(k + 63) / 64, 64, 0, s>>>(h3, k, K.inv.as<double>());
          return cudaGetLastError();
        });
        timed_launch(op->ctx, KC_KRYLOV, [&] {
          k_vscale<S><<<nblk(nk), 256, 0, s>>>(K.w.as<S>(), K.inv.as<double>(), N, k, K.V.as<S>() + (long)(jj + 1) * vstride);
          return cudaGetLastError();
        });
      unsigned char* slot = static_cast<unsigned char*>(K.hpin) + (jj & 1) * K.slot_bytes;
      e = cudaMemcpyAsync(slot, h1, (size_t)(jj + 1) * k * sizeof(S), cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess && gs_passes > 1)
        e = cudaMemcpyAsync(slot + (size_t)(m + 1) * k * sizeof(S), h2, (size_t)(jj + 1) * k * sizeof(S),
                            cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(slot + (size_t)2 * (m + 1) * k * sizeof(S), h3, k * sizeof(S), cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaEventRecord(K.ev[jj & 1], s);
      return cuda_status(op->ctx, e, "gmres orthogonalisation");
    };
    auto process_column = [&](int j, bool* all_done_out) -> bg_status {
      cudaError_t ee = cudaEventSynchronize(K.ev[j & 1]);
      if (ee != cudaSuccess) return cuda_status(op->ctx, ee, "gmres orthogonalisation");
      const H* slot = reinterpret_cast<const H*>(static_cast<unsigned char*>(K.hpin) + (j & 1) * K.slot_bytes);
      std::vector<H> hp1(slot, slot + (size_t)(j + 1) * k), hp2((size_t)(j + 1) * k, H(0)), hp3(k);
      if (gs_passes > 1) std::copy(slot + (size_t)(m + 1) * k, slot + (size_t)(m + 1) * k + (size_t)(j + 1) * k, hp2.begin());
      std::copy(slot + (size_t)2 * (m + 1) * k, slot + (size_t)2 * (m + 1) * k + k, hp3.begin());
      for (size_t q = 0; q < hp1.size(); ++q) hcol[q] = hp1[q] + hp2[q];
      std::vector<double> hn(k);
      for (int c = 0; c < k; ++c) hn[c] = std::sqrt(std::abs(hp3[c]));
      bool all_done = true;
      for (int c = 0; c < k; ++c) {
        H* hc = &Hm[(size_t)c * (m + 1) * m];
        for (int i = 0; i <= j; ++i) hc[(size_t)j * (m + 1) + i] = hcol[(size_t)i * k + c];
        hc[(size_t)j * (m + 1) + j + 1] = hn[c];
        for (int i = 0; i < j; ++i) {  // previous Givens rotations
          H a = hc[(size_t)j * (m + 1) + i], bb = hc[(size_t)j * (m + 1) + i + 1];
          H cc = cs[(size_t)c * m + i], ss = sn[(size_t)c * m + i];
          hc[(size_t)j * (m + 1) + i] = cc * a + ss * bb;
          hc[(size_t)j * (m + 1) + i + 1] = -cj(ss) * a + cc * bb;
        }
        H a = hc[(size_t)j * (m + 1) + j];
        double hb = hn[c], aa = std::abs(a);
        double den = std::sqrt(aa * aa + hb * hb);
        H cc, ss;
        if (den == 0) { cc = 1; ss = 0; }
        else if (aa == 0) { cc = 0; ss = 1; }
        else { cc = aa / den; ss = (a / aa) * (hb / den); }
        cs[(size_t)c * m + j] = cc;
        sn[(size_t)c * m + j] = ss;
        hc[(size_t)j * (m + 1) + j] = cc * a + ss * hb;
        hc[(size_t)j * (m + 1) + j + 1] = 0;
        H gj = g[(size_t)j * k + c];
        g[(size_t)(j + 1) * k + c] = -cj(ss) * gj;
        g[(size_t)j * k + c] = cc * gj;
        if (jconv[c] < 0 && !(std::abs(g[(size_t)(j + 1) * k + c]) > tol * bn[c] && hn[c] > 0)) jconv[c] = j + 1;
        if (jconv[c] < 0) all_done = false;
      }
      *all_done_out = all_done;
      return BG_OK;
    };
    auto can_launch = [&](int q) { return q < m && it0 + q < max_iter; };
    // a flexible step contains an inner solve: too costly to launch speculatively
    const bool speculate = inner == nullptr;
    int launched = 0, j = 0;
    if (can_launch(0)) {
      if ((st = launch_step(0)) != BG_OK) return st;
      launched = 1;
    }
    while (j < launched) {
      if (speculate && can_launch(launched)) {
        if ((st = launch_step(launched)) != BG_OK) return st;
        ++launched;
      }
      bool all_done = false;
      if ((st = process_column(j, &all_done)) != BG_OK) return st;
      ++j;
      if (all_done) break;
      if (!speculate && can_launch(launched)) {
        if ((st = launch_step(launched)) != BG_OK) return st;
        ++launched;
      }
    }
    it = it0 + j;
    // y = R^-1 g per column; x += [V or Z] y
    std::vector<H> y((size_t)j * k, H(0));
    for (int c = 0; c < k; ++c) {
      const H* hc = &Hm[(size_t)c * (m + 1) * m];
      const int jc = jconv[c] >= 0 ? std::min(jconv[c], j) : j;
      for (int i = jc - 1; i >= 0; --i) {
        H acc = g[(size_t)i * k + c];
        for (int q = i + 1; q < jc; ++q) acc -= hc[(size_t)q * (m + 1) + i] * y[(size_t)q * k + c];
        H diag = hc[(size_t)i * (m + 1) + i];
        y[(size_t)i * k + c] = std::abs(diag) > 0 ? acc / diag : H(0);
      }
    }
    e = cudaMemcpyAsync(K.ydev.p, y.data(), y.size() * sizeof(S), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_status(op->ctx, e, "gmres update");
    timed_launch(op->ctx, KC_KRYLOV, [&] {
      k_xupdate<S><<<nblk(nk), 256, 0, s>>>(inner ? K.Z.as<S>() : K.V.as<S>(), vstride, j, K.ydev.as<S>(), N, k,
                                          static_cast<S*>(x));
      return cudaGetLastError();
    });
  }
  cnt->outer_it += it;
  return BG_OK;
}

template <typename S>
bg_status solve_typed(bg_operator* op, const void* bdof, void* xdof, int k, const bg_solve_params& prm,
                      bg_solve_stats* stats) {
  cudaStream_t s = op->ctx->stream;
  const long nk = (long)op->N * k;
  cudaError_t e = cudaMemsetAsync(xdof, 0, nk * sizeof(S), s);
  if (e != cudaSuccess) return cuda_status(op->ctx, e, "solve");
  const bool mixed = prm.inner_precision != BG_PREC_FP64;
  Counters cnt;
  std::vector<double> relres;
  bg_status st;
  if (!mixed) {
    Krylov& K = get_ws(op)->plain;
    if ((st = K.init(op, k, std::max(2, prm.restart), false, sizeof(S))) != BG_OK) return st;
    st = fgmres<S>(K, BG_PREC_FP64, nullptr, 0, 0, 0, bdof, xdof, prm.tol, prm.max_iter, &cnt, &relres);
    cnt.inner_it = cnt.outer_it;
  } else {
    // outer FP64 flexible GMRES; each direction is an inner mixed GMRES solve
    Krylov& outer = get_ws(op)->outer;
    Krylov& inner = get_ws(op)->inner;
    const int mo = std::max(2, prm.max_refinements);
    if ((st = outer.init(op, k, mo, true, sizeof(S))) != BG_OK) return st;
    if ((st = inner.init(op, k, std::max(2, prm.restart), false, sizeof(S))) != BG_OK) return st;
    st = fgmres<S>(outer, BG_PREC_FP64, &inner, prm.inner_precision, prm.inner_tol, prm.max_iter, bdof, xdof, prm.tol,
                   mo, &cnt, &relres);
  }
  if (st != BG_OK) return st;
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_status(op->ctx, e, "solve");
  double worst = 0;
  for (double r : relres) worst = std::max(worst, r);
  bg_solve_stats loc;
  loc.iterations = cnt.inner_it;
  loc.refinements = mixed ? cnt.outer_it : 0;
  loc.fp64_matvecs = cnt.fp64_mv;
  loc.low_matvecs = cnt.mixed_mv;
  loc.final_relres = worst;
  if (stats) *stats = loc;
  return worst <= prm.tol ? BG_OK : set_error(op->ctx, BG_NOT_CONVERGED, "solver did not reach the tolerance");
}

}  // namespace

static bg_status solve_chunks(bg_operator* op, const void* b, void* x, int nrhs, const bg_solve_params& prm,
                              bg_solve_stats* stats, int on_device, int chunk);

// Batched wavenumbers: the columns form nk blocks of nr, block q with
// wavenumber q, and every batch the solver runs must hold an equal slice of
// every block in block order (the product maps its columns that way). The
// columns are permuted on the device so that slice j (columns c0 .. c0 + w - 1
// of every block) is contiguous, solved in chunks of nk w columns (at most
// 256), and permuted back.
static bg_status solve_wavenumber_slices(bg_operator* op, const void* b, void* x, int nrhs, const bg_solve_params& prm,
                                         bg_solve_stats* stats, int on_device) {
  const int nk = (int)op->kslots.size();
  if (nrhs % nk)
    return set_error(op->ctx, BG_INVALID_ARG, "batched wavenumbers: columns must be a multiple of the wavenumbers");
  const int nr = nrhs / nk, w = std::max(1, std::min(nr, 256 / nk));
  cudaStream_t s = op->ctx->stream;
  const size_t col = (size_t)op->N * (op->cplx ? 16 : 8);
  DevBuf bp, xp;
  cudaError_t e = bp.alloc(col * nrhs);
  if (e == cudaSuccess) e = xp.alloc(col * nrhs);
  if (e != cudaSuccess) return cuda_status(op->ctx, e, "solve staging");
  // block q, columns c0 .. c0 + ws - 1  <->  permuted columns c0 nk + q ws
  auto permute = [&](bool in) -> cudaError_t {
    for (int c0 = 0; c0 < nr; c0 += w) {
      const int ws = std::min(w, nr - c0);
      for (int q = 0; q < nk; ++q) {
        const size_t user = (size_t)(q * nr + c0) * col, perm = (size_t)(c0 * nk + q * ws) * col;
        cudaError_t ee =
            in ? cudaMemcpyAsync(static_cast<char*>(bp.p) + perm, static_cast<const char*>(b) + user, ws * col,
                                 on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s)
               : cudaMemcpyAsync(static_cast<char*>(x) + user, static_cast<const char*>(xp.p) + perm, ws * col,
                                 on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s);
        if (ee != cudaSuccess) return ee;
      }
    }
    return cudaSuccess;
  };
  if ((e = permute(true)) != cudaSuccess) return cuda_status(op->ctx, e, "solve staging");
  const bg_status st = solve_chunks(op, bp.p, xp.p, nrhs, prm, stats, 1, nk * w);
  if (st != BG_OK && st != BG_NOT_CONVERGED && st != BG_TIMEOUT) return st;
  if ((e = permute(false)) == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_status(op->ctx, e, "solve copy-out");
  return st;
}

extern "C" bg_status bg_solve(bg_operator* op, const void* b, void* x, int nrhs, const bg_solve_params* params,
                              bg_solve_stats* stats, int on_device) {
  if (!op || nrhs < 0) return BG_INVALID_ARG;
  if (nrhs == 0) {  // no right-hand sides: nothing to solve
    if (stats) *stats = bg_solve_stats{};
    return BG_OK;
  }
  if (!b || !x) return BG_INVALID_ARG;
  if (op->ctx->device < 0) return set_error(op->ctx, BG_UNSUPPORTED, "host-only context: solves need a GPU");
  if (!op->assembled) return set_error(op->ctx, BG_INVALID_ARG, "operator not assembled");
  bg_solve_params prm;
  bg_solve_params_default(&prm);
  if (params) prm = *params;
  if (prm.tol <= 0 || prm.restart < 1 || prm.max_iter < 1 || prm.inner_precision < BG_PREC_FP64 ||
      prm.inner_precision > BG_PREC_FP32)
    return set_error(op->ctx, BG_INVALID_ARG, "solve parameters");
  cudaSetDevice(op->ctx->device);
  if (op->kbatched()) return solve_wavenumber_slices(op, b, x, nrhs, prm, stats, on_device);
  return solve_chunks(op, b, x, nrhs, prm, stats, on_device, 32);
}

// Column chunks of at most `chunk` columns, each solved as one batch.
static bg_status solve_chunks(bg_operator* op, const void* b, void* x, int nrhs, const bg_solve_params& prm,
                              bg_solve_stats* stats, int on_device, int chunk) {
  cudaStream_t s = op->ctx->stream;
  const size_t usz = op->cplx ? 16 : 8;
  bg_solve_stats total{0, 0, 0, 0, 0.0};
  bg_status result = BG_OK;
  for (int c0 = 0; c0 < nrhs; c0 += chunk) {
    const int k = std::min(chunk, nrhs - c0);
    bg_status st = ensure_work(op, k);
    if (st != BG_OK) return st;
    const long nk = (long)op->N * k;
    DevBuf& bw = get_ws(op)->bw;
    DevBuf& xw = get_ws(op)->xw;
    DevBuf& bu = get_ws(op)->bu;
    cudaError_t e = bw.alloc(nk * usz);
    if (e == cudaSuccess) e = xw.alloc(nk * usz);
    const void* bsrc = static_cast<const char*>(b) + (size_t)c0 * op->N * usz;
    if (!on_device) {
      if (e == cudaSuccess) e = bu.alloc(nk * usz);
      if (e == cudaSuccess) e = cudaMemcpyAsync(bu.p, bsrc, nk * usz, cudaMemcpyHostToDevice, s);
      bsrc = bu.p;
    }
    if (e != cudaSuccess) return cuda_status(op->ctx, e, "solve staging");
    // user column-major -> row-major work
    if ((st = cuda_status(op->ctx, launch_gather_in(op->cplx ? 1 : 0, op->cplx ? 1 : 0, bsrc, op->N, op->N, k, bw.p, s),
                          "gather b")) != BG_OK)
      return st;
    bg_solve_stats part;
    st = op->cplx ? solve_typed<cd>(op, bw.p, xw.p, k, prm, &part) : solve_typed<double>(op, bw.p, xw.p, k, prm, &part);
    if (st != BG_OK && st != BG_NOT_CONVERGED) return st;
    if (st == BG_NOT_CONVERGED) result = st;
    total.iterations += part.iterations;
    total.refinements = std::max(total.refinements, part.refinements);
    total.fp64_matvecs += part.fp64_matvecs;
    total.low_matvecs += part.low_matvecs;
    total.final_relres = std::max(total.final_relres, part.final_relres);
    const double one[2] = {1, 0}, zero2[2] = {0, 0};
    void* xdst = static_cast<char*>(x) + (size_t)c0 * op->N * usz;
    DevBuf& xu = get_ws(op)->xu;
    void* xd = xdst;
    if (!on_device) {
      if ((e = xu.alloc(nk * usz)) != cudaSuccess) return cuda_status(op->ctx, e, "solve staging");
      xd = xu.p;
    }
    if ((st = cuda_status(op->ctx, launch_scatter_out(op->cplx ? 1 : 0, xw.p, op->N, k, xd, op->N, one, zero2, s),
                          "scatter x")) != BG_OK)
      return st;
    if (!on_device) {
      e = cudaMemcpyAsync(xdst, xd, nk * usz, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) return cuda_status(op->ctx, e, "solve copy-out");
    }
  }
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_status(op->ctx, e, "solve");
  if (stats) *stats = total;
  const bg_status flag = check_device_flag(op);
  return flag != BG_OK ? flag : result;
}
