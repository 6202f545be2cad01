// Krylov solve, load vectors and potential evaluation on GB300.
//
// bg_solve: restarted GMRES (Saad & Schultz 1986) batched over right-hand
// sides with classical Gram-Schmidt applied twice, FP64 Krylov basis, wrapped
// in iterative refinement: every refinement step evaluates the FP64 residual
// b - A x with the FP64 operator and solves for the correction with the inner
// operator (FP64, or the FP32 fused far field). Replaces the Eigen solvers
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
template <typename S>
__global__ void k_mdot(const S* __restrict__ V, long vstride, const S* __restrict__ w, int N, int k, S* __restrict__ out) {
  __shared__ S red[256];
  const int i = blockIdx.x;
  const int kp = k;  // columns
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
template <typename S>
__global__ void k_axpy(S* __restrict__ x, const S* __restrict__ d, long n) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) x[t] = addv(x[t], d[t]);
}

inline unsigned nblk(long n) { return (unsigned)((n + 255) / 256); }

}  // namespace

// ---------------------------------------------------------------------------
namespace {

struct Krylov {
  bg_operator* op;
  int N, k, m;
  bool cplx;
  size_t sb;  // FP64 scalar bytes
  DevBuf V, w, hdev, tmp32a, tmp32b, inv, ydev;
};

// w = A v with the requested precision (FP64 work vectors in and out)
bg_status apply_prec(Krylov& K, bool fp32, const void* v, void* w) {
  bg_operator* op = K.op;
  cudaStream_t s = op->ctx->stream;
  if (!fp32) return apply_operator(op, K.k, false, v, w);
  const long n = (long)K.N * K.k;
  const int S64 = op->stype(false), S32 = op->stype(true);
  bg_status st = cuda_status(op->ctx, launch_convert(S64, S32, v, n, K.tmp32a.p, s), "convert");
  if (st != BG_OK) return st;
  if ((st = apply_operator(op, K.k, true, K.tmp32a.p, K.tmp32b.p)) != BG_OK) return st;
  return cuda_status(op->ctx, launch_convert(S32, S64, K.tmp32b.p, n, w, s), "convert");
}

template <typename S>
using HostS = typename std::conditional<std::is_same<S, double>::value, double, std::complex<double>>::type;
inline double cj(double v) { return v; }
inline std::complex<double> cj(std::complex<double> v) { return std::conj(v); }

// column norms of a row-major N x k block (FP64 work vector)
template <typename S>
bg_status col_norms(Krylov& K, const void* x, std::vector<double>* out) {
  cudaStream_t s = K.op->ctx->stream;
  k_mdot<S><<<1, 256, 0, s>>>(static_cast<const S*>(x), 0, static_cast<const S*>(x), K.N, K.k, K.hdev.as<S>());
  std::vector<HostS<S>> h(K.k);
  cudaError_t e = cudaMemcpyAsync(h.data(), K.hdev.p, K.k * sizeof(S), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_status(K.op->ctx, e, "norms");
  out->resize(K.k);
  for (int c = 0; c < K.k; ++c) (*out)[c] = std::sqrt(std::abs(h[c]));
  return BG_OK;
}

// GMRES on A (precision fp32 or fp64) for the row-major FP64 rhs r (N x k):
// solves A d = r to relative tolerance tol per column; d accumulates.
template <typename S>
bg_status gmres_cycles(Krylov& K, bool fp32, const void* r, void* d, double tol, int max_iter, int* iters,
                       int* matvecs) {
  typedef HostS<S> H;
  bg_operator* op = K.op;
  cudaStream_t s = op->ctx->stream;
  const int N = K.N, k = K.k, m = K.m;
  const long nk = (long)N * k;
  const long vstride = nk;
  std::vector<double> rn;
  bg_status st = col_norms<S>(K, r, &rn);
  if (st != BG_OK) return st;
  // residual vector of the correction system: rc = r - A d (d starts at 0)
  DevBuf rc;
  cudaError_t e = rc.alloc(nk * sizeof(S));
  if (e == cudaSuccess) e = cudaMemcpyAsync(rc.p, r, nk * sizeof(S), cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(d, 0, nk * sizeof(S), s);
  if (e != cudaSuccess) return cuda_status(op->ctx, e, "gmres setup");
  int it = 0;
  std::vector<H> Hm((size_t)(m + 1) * m * k), g((size_t)(m + 1) * k), cs((size_t)m * k), sn((size_t)m * k);
  std::vector<H> hcol((size_t)(m + 1) * k);
  std::vector<double> inv(k);
  while (it < max_iter) {
    std::vector<double> beta;
    if ((st = col_norms<S>(K, rc.p, &beta)) != BG_OK) return st;
    bool done = true;
    for (int c = 0; c < k; ++c)
      if (beta[c] > tol * rn[c] && rn[c] > 0) done = false;
    if (done) break;
    for (int c = 0; c < k; ++c) inv[c] = beta[c] > 0 ? 1.0 / beta[c] : 0.0;
    e = cudaMemcpyAsync(K.inv.p, inv.data(), k * sizeof(double), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_status(op->ctx, e, "gmres");
    k_vscale<S><<<nblk(nk), 256, 0, s>>>(rc.as<S>(), K.inv.as<double>(), N, k, K.V.as<S>());
    std::fill(Hm.begin(), Hm.end(), H(0));
    std::fill(g.begin(), g.end(), H(0));
    for (int c = 0; c < k; ++c) g[c] = beta[c];
    std::vector<char> active(k, 1);
    int j = 0;
    for (; j < m && it < max_iter; ++j, ++it) {
      S* vj = K.V.as<S>() + (long)j * vstride;
      if ((st = apply_prec(K, fp32, vj, K.w.p)) != BG_OK) return st;
      ++*matvecs;
      // CGS2: two Gram-Schmidt passes
      std::fill(hcol.begin(), hcol.end(), H(0));
      for (int pass = 0; pass < 2; ++pass) {
        k_mdot<S><<<j + 1, 256, 0, s>>>(K.V.as<S>(), vstride, K.w.as<S>(), N, k, K.hdev.as<S>());
        k_vupdate<S><<<nblk(nk), 256, 0, s>>>(K.V.as<S>(), vstride, j + 1, K.hdev.as<S>(), N, k, K.w.as<S>());
        std::vector<H> hp((size_t)(j + 1) * k);
        e = cudaMemcpyAsync(hp.data(), K.hdev.p, hp.size() * sizeof(S), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return cuda_status(op->ctx, e, "gmres orthogonalisation");
        for (size_t q = 0; q < hp.size(); ++q) hcol[q] += hp[q];
      }
      std::vector<double> hn;
      if ((st = col_norms<S>(K, K.w.p, &hn)) != BG_OK) return st;
      for (int c = 0; c < k; ++c) inv[c] = hn[c] > 0 ? 1.0 / hn[c] : 0.0;
      e = cudaMemcpyAsync(K.inv.p, inv.data(), k * sizeof(double), cudaMemcpyHostToDevice, s);
      if (e != cudaSuccess) return cuda_status(op->ctx, e, "gmres");
      k_vscale<S><<<nblk(nk), 256, 0, s>>>(K.w.as<S>(), K.inv.as<double>(), N, k, K.V.as<S>() + (long)(j + 1) * vstride);
      bool all_done = true;
      for (int c = 0; c < k; ++c) {
        H* hc = &Hm[(size_t)c * (m + 1) * m];
        for (int i = 0; i <= j; ++i) hc[(size_t)j * (m + 1) + i] = hcol[(size_t)i * k + c];
        hc[(size_t)j * (m + 1) + j + 1] = hn[c];
        // apply the previous Givens rotations to the new column
        for (int i = 0; i < j; ++i) {
          H a = hc[(size_t)j * (m + 1) + i], b = hc[(size_t)j * (m + 1) + i + 1];
          H cc = cs[(size_t)c * m + i], ss = sn[(size_t)c * m + i];
          hc[(size_t)j * (m + 1) + i] = cc * a + ss * b;
          hc[(size_t)j * (m + 1) + i + 1] = -cj(ss) * a + cc * b;
        }
        H a = hc[(size_t)j * (m + 1) + j];
        double bb = hn[c], aa = std::abs(a);
        double den = std::sqrt(aa * aa + bb * bb);
        H cc, ss;
        if (den == 0) { cc = 1; ss = 0; }
        else if (aa == 0) { cc = 0; ss = 1; }
        else { cc = aa / den; ss = (a / aa) * (bb / den); }
        cs[(size_t)c * m + j] = cc;
        sn[(size_t)c * m + j] = ss;
        hc[(size_t)j * (m + 1) + j] = cc * a + ss * bb;
        hc[(size_t)j * (m + 1) + j + 1] = 0;
        H gj = g[(size_t)j * k + c];
        g[(size_t)(j + 1) * k + c] = -cj(ss) * gj;
        g[(size_t)j * k + c] = cc * gj;
        if (std::abs(g[(size_t)(j + 1) * k + c]) > tol * rn[c] && hn[c] > 0) all_done = false;
      }
      if (all_done) {
        ++j;
        ++it;
        break;
      }
    }
    // y = R^-1 g per column, d += V y
    std::vector<H> y((size_t)j * k, H(0));
    for (int c = 0; c < k; ++c) {
      const H* hc = &Hm[(size_t)c * (m + 1) * m];
      for (int i = j - 1; i >= 0; --i) {
        H acc = g[(size_t)i * k + c];
        for (int q = i + 1; q < j; ++q) acc -= hc[(size_t)q * (m + 1) + i] * y[(size_t)q * k + c];
        H diag = hc[(size_t)i * (m + 1) + i];
        y[(size_t)i * k + c] = std::abs(diag) > 0 ? acc / diag : H(0);
      }
    }
    e = cudaMemcpyAsync(K.ydev.p, y.data(), y.size() * sizeof(S), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_status(op->ctx, e, "gmres update");
    k_xupdate<S><<<nblk(nk), 256, 0, s>>>(K.V.as<S>(), vstride, j, K.ydev.as<S>(), N, k, static_cast<S*>(d));
    // true residual of the correction system for the restart
    if ((st = apply_prec(K, fp32, d, rc.p)) != BG_OK) return st;
    ++*matvecs;
    k_residual<S><<<nblk(nk), 256, 0, s>>>(static_cast<const S*>(r), nk, rc.as<S>());
  }
  *iters += it;
  return BG_OK;
}

template <typename S>
bg_status solve_typed(bg_operator* op, const void* bdof, void* xdof, int k, const bg_solve_params& prm,
                      bg_solve_stats* stats) {
  cudaStream_t s = op->ctx->stream;
  Krylov K;
  K.op = op;
  K.N = op->N;
  K.k = k;
  K.m = std::max(2, prm.restart);
  K.cplx = op->cplx;
  K.sb = sizeof(S);
  const long nk = (long)K.N * k;
  cudaError_t e = K.V.alloc((size_t)(K.m + 1) * nk * sizeof(S));
  if (e == cudaSuccess) e = K.w.alloc(nk * sizeof(S));
  if (e == cudaSuccess) e = K.hdev.alloc((size_t)(K.m + 1) * k * sizeof(S));
  if (e == cudaSuccess) e = K.tmp32a.alloc(nk * sizeof(S));
  if (e == cudaSuccess) e = K.tmp32b.alloc(nk * sizeof(S));
  if (e == cudaSuccess) e = K.inv.alloc(k * sizeof(double));
  if (e == cudaSuccess) e = K.ydev.alloc((size_t)(K.m + 1) * k * sizeof(S));
  DevBuf r, d;
  if (e == cudaSuccess) e = r.alloc(nk * sizeof(S));
  if (e == cudaSuccess) e = d.alloc(nk * sizeof(S));
  if (e == cudaSuccess) e = cudaMemsetAsync(xdof, 0, nk * sizeof(S), s);
  if (e != cudaSuccess) return cuda_status(op->ctx, e, "solver workspace");
  std::vector<double> bn;
  bg_status st = col_norms<S>(K, bdof, &bn);
  if (st != BG_OK) return st;
  const bool inner32 = prm.inner_precision == BG_PREC_FP32;
  bg_solve_stats loc{0, 0, 0, 0, 0.0};
  int fp64_mv = 0, low_mv = 0;
  double worst = 0;
  for (int ref = 0; ref <= prm.max_refinements; ++ref) {
    // FP64 residual r = b - A x
    if (ref == 0) {
      e = cudaMemcpyAsync(r.p, bdof, nk * sizeof(S), cudaMemcpyDeviceToDevice, s);
      if (e != cudaSuccess) return cuda_status(op->ctx, e, "residual");
    } else {
      if ((st = apply_operator(op, k, false, xdof, r.p)) != BG_OK) return st;
      ++fp64_mv;
      k_residual<S><<<nblk(nk), 256, 0, s>>>(static_cast<const S*>(bdof), nk, r.as<S>());
    }
    std::vector<double> rn;
    if ((st = col_norms<S>(K, r.p, &rn)) != BG_OK) return st;
    worst = 0;
    for (int c = 0; c < k; ++c) worst = std::max(worst, bn[c] > 0 ? rn[c] / bn[c] : 0.0);
    loc.refinements = ref;
    if (worst <= prm.tol) break;
    if (ref == prm.max_refinements || loc.iterations >= prm.max_iter) break;
    // inner tolerance relative to the current residual, but never asking for
    // more than the target on the full system
    double itol = inner32 ? prm.inner_tol : prm.tol;
    double need = 0;
    for (int c = 0; c < k; ++c) need = std::max(need, rn[c] > 0 ? prm.tol * bn[c] / rn[c] : 0.0);
    itol = std::max(itol, 0.5 * need);
    int mv = 0;
    if ((st = gmres_cycles<S>(K, inner32, r.p, d.p, itol, prm.max_iter - loc.iterations, &loc.iterations, &mv)) != BG_OK)
      return st;
    (inner32 ? low_mv : fp64_mv) += mv;
    k_axpy<S><<<nblk(nk), 256, 0, s>>>(static_cast<S*>(xdof), d.as<S>(), nk);
  }
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_status(op->ctx, e, "solve");
  loc.final_relres = worst;
  loc.fp64_matvecs = fp64_mv;
  loc.low_matvecs = low_mv;
  if (stats) *stats = loc;
  return worst <= prm.tol ? BG_OK : set_error(op->ctx, BG_NOT_CONVERGED, "solver did not reach the tolerance");
}

}  // namespace

extern "C" bg_status bg_solve(bg_operator* op, const void* b, void* x, int nrhs, const bg_solve_params* params,
                              bg_solve_stats* stats, int on_device) {
  if (!op || !b || !x || nrhs <= 0) return BG_INVALID_ARG;
  if (op->ctx->device < 0) return set_error(op->ctx, BG_UNSUPPORTED, "host-only context: solves need a GPU");
  if (!op->assembled) return set_error(op->ctx, BG_INVALID_ARG, "operator not assembled");
  bg_solve_params prm;
  bg_solve_params_default(&prm);
  if (params) prm = *params;
  if (prm.tol <= 0 || prm.restart < 1 || prm.max_iter < 1) return set_error(op->ctx, BG_INVALID_ARG, "solve parameters");
  cudaSetDevice(op->ctx->device);
  cudaStream_t s = op->ctx->stream;
  const size_t usz = op->cplx ? 16 : 8;
  bg_solve_stats total{0, 0, 0, 0, 0.0};
  bg_status result = BG_OK;
  for (int c0 = 0; c0 < nrhs; c0 += 32) {
    const int k = std::min(32, nrhs - c0);
    bg_status st = ensure_work(op, k);
    if (st != BG_OK) return st;
    const long nk = (long)op->N * k;
    DevBuf bw, xw, bu;
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
    DevBuf xu;
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
  return result;
}
