// The H2 matvec on GB300 (H2_time_dense_product_impl::run,
// EigenHelper/H2DenseProduct.hpp:33-165), batched over right-hand sides:
//   x_ss = T x                          (sparse gather, :52-53)
//   Y_leaf = Mom X_ss, Y_l = T_fmm Y_l+1 (forwardTransformation, H2Multipole.hpp:380-422)
//   y_ss = sum_dense F x_ss[c2]          (dense leaves, :107-115)
//   Z_l[c1] = sum_lowrank F Y_l[c2]      (low-rank leaves, :117-135)
//   Z_l+1 += T_fmm^T Z_l, y_ss += Mom^T Z_leaf (backwardTransformation, :428-469)
//   y = T^T y_ss                         (:161-162)
// Work vectors are row-major with the right-hand sides contiguous, so every
// coupling entry streamed from HBM is reused across all right-hand sides.
#include <type_traits>

#include "bg_kernels.cuh"

namespace bg {

template <typename S> struct RealOf;
template <> struct RealOf<double> { typedef double T; };
template <> struct RealOf<cd> { typedef double T; };
template <> struct RealOf<float> { typedef float T; };
template <> struct RealOf<cf> { typedef float T; };

__device__ inline double to_d(double v) { return v; }
__device__ inline double to_d(float v) { return (double)v; }

template <typename A, typename B> struct Conv;
template <typename A> struct Conv<A, A> { __device__ static A run(A v) { return v; } };
template <> struct Conv<double, float> { __device__ static float run(double v) { return (float)v; } };
template <> struct Conv<float, double> { __device__ static double run(float v) { return (double)v; } };
template <> struct Conv<cd, cf> { __device__ static cf run(cd v) { return {(float)v.re, (float)v.im}; } };
template <> struct Conv<cf, cd> { __device__ static cd run(cf v) { return {(double)v.re, (double)v.im}; } };

__device__ inline double add(double a, double b) { return a + b; }
__device__ inline float add(float a, float b) { return a + b; }
__device__ inline cd add(cd a, cd b) { return a + b; }
__device__ inline cf add(cf a, cf b) { return a + b; }

// ---------------------------------------------------------------------------
template <typename S>
__global__ void k_csr_apply(const int* __restrict__ ptr, const int* __restrict__ idx, const double* __restrict__ val,
                            int rows, const S* __restrict__ x, S* __restrict__ y, int nrhs) {
  typedef typename RealOf<S>::T R;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)rows * nrhs) return;
  const int r = (int)(t / nrhs), k = (int)(t % nrhs);
  S acc = zero<S>();
  for (int p = ptr[r]; p < ptr[r + 1]; ++p) acc = fmac(acc, x[(long)idx[p] * nrhs + k], (R)val[p]);
  y[t] = acc;
}

// Block-sparse rows: CTA per block row, thread i < B owns row i of the block
// and all right-hand sides; F blocks are column-major so a warp reads
// consecutive entries of one column (coalesced), x is staged in shared memory.
template <typename S, int NR>
__global__ void k_bsr(const int* __restrict__ row_ptr, const int* __restrict__ col, const S* __restrict__ blocks,
                      int B, const S* __restrict__ x, S* __restrict__ y, int nrhs, int accumulate) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  S* xs = reinterpret_cast<S*>(smem_raw);
  const int row = blockIdx.x;
  const int i = threadIdx.x;
  S acc[NR];
#pragma unroll
  for (int c = 0; c < NR; ++c) acc[c] = zero<S>();
  for (int k = row_ptr[row]; k < row_ptr[row + 1]; ++k) {
    const long xoff = (long)col[k] * B * nrhs;
    __syncthreads();
    for (int t = threadIdx.x; t < B * nrhs; t += blockDim.x) xs[t] = x[xoff + t];
    __syncthreads();
    if (i < B) {
      const S* F = blocks + (long)k * B * B + i;
      for (int j = 0; j < B; ++j) {
        const S f = F[(long)j * B];
#pragma unroll
        for (int c = 0; c < NR; ++c)
          if (c < nrhs) acc[c] = fmac(acc[c], f, xs[j * nrhs + c]);
      }
    }
  }
  if (i < B) {
    S* yo = y + ((long)row * B + i) * nrhs;
#pragma unroll
    for (int c = 0; c < NR; ++c)
      if (c < nrhs) yo[c] = accumulate ? add(yo[c], acc[c]) : acc[c];
  }
}

// Y[c][r][k] = sum_q Mom[r][q] X[c*Bq + q][k]
template <typename S>
__global__ void k_moment_fwd(const typename RealOf<S>::T* __restrict__ mom, int R, int Bq,
                             const S* __restrict__ xss, S* __restrict__ y, int nrhs) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  S* xs = reinterpret_cast<S*>(smem_raw);
  const int c = blockIdx.x;
  for (int t = threadIdx.x; t < Bq * nrhs; t += blockDim.x) xs[t] = xss[(long)c * Bq * nrhs + t];
  __syncthreads();
  for (int t = threadIdx.x; t < R * nrhs; t += blockDim.x) {
    const int r = t / nrhs, k = t % nrhs;
    S acc = zero<S>();
    for (int q = 0; q < Bq; ++q) acc = fmac(acc, xs[q * nrhs + k], mom[r * Bq + q]);
    y[(long)c * R * nrhs + t] = acc;
  }
}
// Yss[c*Bq + q][k] += sum_r Mom[r][q] Z[c][r][k]
template <typename S>
__global__ void k_moment_bwd(const typename RealOf<S>::T* __restrict__ mom, int R, int Bq, const S* __restrict__ z,
                             S* __restrict__ yss, int nrhs) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  S* zs = reinterpret_cast<S*>(smem_raw);
  const int c = blockIdx.x;
  for (int t = threadIdx.x; t < R * nrhs; t += blockDim.x) zs[t] = z[(long)c * R * nrhs + t];
  __syncthreads();
  for (int t = threadIdx.x; t < Bq * nrhs; t += blockDim.x) {
    const int q = t / nrhs, k = t % nrhs;
    S acc = zero<S>();
    for (int r = 0; r < R; ++r) acc = fmac(acc, zs[r * nrhs + k], mom[r * Bq + q]);
    const long o = (long)c * Bq * nrhs + t;
    yss[o] = add(yss[o], acc);
  }
}
// parent[p][comp*np2 + r][k] = sum_{ch, q} T[r][ch*np2 + q] child[4p+ch][comp*np2 + q][k]
template <typename S>
__global__ void k_transfer_fwd(const typename RealOf<S>::T* __restrict__ T, int np2, int nc,
                               const S* __restrict__ ychild, S* __restrict__ yparent, int nrhs) {
  const int p = blockIdx.x, R = nc * np2;
  for (int t = threadIdx.x; t < R * nrhs; t += blockDim.x) {
    const int row = t / nrhs, k = t % nrhs;
    const int comp = row / np2, r = row % np2;
    S acc = zero<S>();
    for (int ch = 0; ch < 4; ++ch) {
      const S* src = ychild + ((long)(4 * p + ch) * R + comp * np2) * nrhs + k;
      const typename RealOf<S>::T* Tr = T + (long)r * 4 * np2 + ch * np2;
      for (int q = 0; q < np2; ++q) acc = fmac(acc, src[(long)q * nrhs], Tr[q]);
    }
    yparent[(long)p * R * nrhs + t] = acc;
  }
}
// child[4p+ch][comp*np2 + q][k] += sum_r T[r][ch*np2 + q] parent[p][comp*np2 + r][k]
template <typename S>
__global__ void k_transfer_bwd(const typename RealOf<S>::T* __restrict__ T, int np2, int nc,
                               const S* __restrict__ zparent, S* __restrict__ zchild, int nrhs) {
  const int p = blockIdx.x, R = nc * np2;
  for (int t = threadIdx.x; t < 4 * R * nrhs; t += blockDim.x) {
    const int row = t / nrhs, k = t % nrhs;  // row over 4 children
    const int ch = row / R, cr = row % R;
    const int comp = cr / np2, q = cr % np2;
    const S* src = zparent + ((long)p * R + comp * np2) * nrhs + k;
    S acc = zero<S>();
    for (int r = 0; r < np2; ++r) acc = fmac(acc, src[(long)r * nrhs], T[(long)r * 4 * np2 + ch * np2 + q]);
    const long o = ((long)(4 * p + ch) * R + cr) * nrhs + k;
    zchild[o] = add(zchild[o], acc);
  }
}

// Fused FP32 far field: the coupling F_ij = k(x_i, y_j) |J_i| |J_j| is
// generated from the clusters' interpolation points inside the product.
template <bool CPLX, int NR>
__global__ void k_far_fused(const float4* __restrict__ prow, const float4* __restrict__ pcol,
                            const int* __restrict__ row_ptr, const int* __restrict__ col, int np2, float kre, float kim,
                            const void* __restrict__ yv, void* __restrict__ zv, int nrhs) {
  typedef typename std::conditional<CPLX, cf, float>::type S;
  const S* y = static_cast<const S*>(yv);
  S* z = static_cast<S*>(zv);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float4* ps = reinterpret_cast<float4*>(smem_raw);
  S* ys = reinterpret_cast<S*>(ps + np2);
  const int row = blockIdx.x, i = threadIdx.x;
  float4 xi = make_float4(0, 0, 0, 0);
  if (i < np2) xi = prow[(long)row * np2 + i];
  S acc[NR];
#pragma unroll
  for (int c = 0; c < NR; ++c) acc[c] = zero<S>();
  for (int k = row_ptr[row]; k < row_ptr[row + 1]; ++k) {
    const int c2 = col[k];
    __syncthreads();
    for (int t = threadIdx.x; t < np2; t += blockDim.x) ps[t] = pcol[(long)c2 * np2 + t];
    for (int t = threadIdx.x; t < np2 * nrhs; t += blockDim.x) ys[t] = y[(long)c2 * np2 * nrhs + t];
    __syncthreads();
    if (i < np2) {
      for (int j = 0; j < np2; ++j) {
        const float4 yj = ps[j];
        const float d0 = xi.x - yj.x, d1 = xi.y - yj.y, d2 = xi.z - yj.z;
        const float r2 = fmaf(d0, d0, fmaf(d1, d1, d2 * d2));
        const float inv = rsqrtf(r2);
        const float amp = inv * 0.0795774715f * xi.w * yj.w;
        if constexpr (CPLX) {
          const float r = r2 * inv;
          float sn, cs;
          sincosf(kre * r, &sn, &cs);
          float a = amp;
          if (kim != 0.0f) a *= expf(kim * r);
          const cf f = {cs * a, -sn * a};
#pragma unroll
          for (int c = 0; c < NR; ++c)
            if (c < nrhs) acc[c] = fmac(acc[c], f, ys[j * nrhs + c]);
        } else {
#pragma unroll
          for (int c = 0; c < NR; ++c)
            if (c < nrhs) acc[c] = fmac(acc[c], amp, ys[j * nrhs + c]);
        }
      }
    }
  }
  if (i < np2) {
    S* zo = z + ((long)row * np2 + i) * nrhs;
#pragma unroll
    for (int c = 0; c < NR; ++c)
      if (c < nrhs) zo[c] = acc[c];
  }
}

template <typename Sin, typename Sout>
__global__ void k_gather_in(const Sin* __restrict__ user, long ld, int rows, int nrhs, Sout* __restrict__ work) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)rows * nrhs) return;
  const int r = (int)(t / nrhs), k = (int)(t % nrhs);
  work[t] = Conv<Sin, Sout>::run(user[r + k * ld]);
}
template <typename S>
__global__ void k_scatter_out_real(const S* __restrict__ work, int rows, int nrhs, double* __restrict__ user, long ld,
                                   double alpha, double beta) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)rows * nrhs) return;
  const int r = (int)(t / nrhs), k = (int)(t % nrhs);
  double* u = user + r + k * ld;
  const double v = alpha * to_d(work[t]);
  *u = beta == 0.0 ? v : fma(beta, *u, v);
}
template <typename S>
__global__ void k_scatter_out_cplx(const S* __restrict__ work, int rows, int nrhs, cd* __restrict__ user, long ld,
                                   cd alpha, cd beta) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)rows * nrhs) return;
  const int r = (int)(t / nrhs), k = (int)(t % nrhs);
  cd* u = user + r + k * ld;
  const cd w = Conv<S, cd>::run(work[t]);
  cd v = alpha * w;
  if (beta.re != 0.0 || beta.im != 0.0) v = v + beta * (*u);
  *u = v;
}
template <typename Sin, typename Sout>
__global__ void k_convert(const Sin* __restrict__ in, long n, Sout* __restrict__ out) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) out[t] = Conv<Sin, Sout>::run(in[t]);
}

// ---------------------------------------------------------------------------
static inline unsigned blocks_for(long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

cudaError_t launch_csr_apply(int S, const int* ptr, const int* idx, const double* val, int rows, const void* x,
                             void* y, int nrhs, cudaStream_t s) {
  const long n = (long)rows * nrhs;
  if (n == 0) return cudaSuccess;
  const unsigned g = blocks_for(n, 256);
  switch (S) {
    case 0: k_csr_apply<double><<<g, 256, 0, s>>>(ptr, idx, val, rows, (const double*)x, (double*)y, nrhs); break;
    case 1: k_csr_apply<cd><<<g, 256, 0, s>>>(ptr, idx, val, rows, (const cd*)x, (cd*)y, nrhs); break;
    case 2: k_csr_apply<float><<<g, 256, 0, s>>>(ptr, idx, val, rows, (const float*)x, (float*)y, nrhs); break;
    case 3: k_csr_apply<cf><<<g, 256, 0, s>>>(ptr, idx, val, rows, (const cf*)x, (cf*)y, nrhs); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <typename S>
static cudaError_t bsr_typed(const int* row_ptr, const int* col, const S* blocks, int nrows, int B, const S* x, S* y,
                             int nrhs, int accumulate, cudaStream_t s) {
  if (nrows == 0) return cudaSuccess;
  const int bs = ((B + 31) / 32) * 32;
  if (bs > 1024) return cudaErrorInvalidValue;
  const size_t smem = (size_t)B * nrhs * sizeof(S);
#define BG_BSR(NRV)                                                                                          \
  {                                                                                                          \
    auto kf = k_bsr<S, NRV>;                                                                                 \
    cudaError_t e = cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);        \
    if (e != cudaSuccess) return e;                                                                          \
    kf<<<nrows, bs, smem, s>>>(row_ptr, col, blocks, B, x, y, nrhs, accumulate);                             \
    return cudaGetLastError();                                                                               \
  }
  if (nrhs <= 1) BG_BSR(1)
  if (nrhs <= 2) BG_BSR(2)
  if (nrhs <= 4) BG_BSR(4)
  if (nrhs <= 8) BG_BSR(8)
  if (nrhs <= 16) BG_BSR(16)
  if (nrhs <= 32) BG_BSR(32)
#undef BG_BSR
  return cudaErrorInvalidValue;
}
cudaError_t launch_bsr(int S, const int* row_ptr, const int* col, const void* blocks, int nrows, int B, const void* x,
                       void* y, int nrhs, int accumulate, cudaStream_t s) {
  switch (S) {
    case 0: return bsr_typed<double>(row_ptr, col, (const double*)blocks, nrows, B, (const double*)x, (double*)y, nrhs, accumulate, s);
    case 1: return bsr_typed<cd>(row_ptr, col, (const cd*)blocks, nrows, B, (const cd*)x, (cd*)y, nrhs, accumulate, s);
    case 2: return bsr_typed<float>(row_ptr, col, (const float*)blocks, nrows, B, (const float*)x, (float*)y, nrhs, accumulate, s);
    case 3: return bsr_typed<cf>(row_ptr, col, (const cf*)blocks, nrows, B, (const cf*)x, (cf*)y, nrhs, accumulate, s);
    default: return cudaErrorInvalidValue;
  }
}

template <typename S>
static cudaError_t mom_fwd_t(const void* mom, int R, int Bq, int ncl, const void* xss, void* y, int nrhs, cudaStream_t s) {
  if (ncl == 0) return cudaSuccess;
  const size_t smem = (size_t)Bq * nrhs * sizeof(S);
  auto kf = k_moment_fwd<S>;
  cudaError_t e = cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  kf<<<ncl, 256, smem, s>>>((const typename RealOf<S>::T*)mom, R, Bq, (const S*)xss, (S*)y, nrhs);
  return cudaGetLastError();
}
cudaError_t launch_moment_fwd(int S, const void* mom, int R, int Bq, int ncl, const void* xss, void* y, int nrhs,
                              cudaStream_t s) {
  switch (S) {
    case 0: return mom_fwd_t<double>(mom, R, Bq, ncl, xss, y, nrhs, s);
    case 1: return mom_fwd_t<cd>(mom, R, Bq, ncl, xss, y, nrhs, s);
    case 2: return mom_fwd_t<float>(mom, R, Bq, ncl, xss, y, nrhs, s);
    case 3: return mom_fwd_t<cf>(mom, R, Bq, ncl, xss, y, nrhs, s);
    default: return cudaErrorInvalidValue;
  }
}
template <typename S>
static cudaError_t mom_bwd_t(const void* mom, int R, int Bq, int ncl, const void* z, void* yss, int nrhs, cudaStream_t s) {
  if (ncl == 0) return cudaSuccess;
  const size_t smem = (size_t)R * nrhs * sizeof(S);
  auto kf = k_moment_bwd<S>;
  cudaError_t e = cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  kf<<<ncl, 256, smem, s>>>((const typename RealOf<S>::T*)mom, R, Bq, (const S*)z, (S*)yss, nrhs);
  return cudaGetLastError();
}
cudaError_t launch_moment_bwd(int S, const void* mom, int R, int Bq, int ncl, const void* z, void* yss, int nrhs,
                              cudaStream_t s) {
  switch (S) {
    case 0: return mom_bwd_t<double>(mom, R, Bq, ncl, z, yss, nrhs, s);
    case 1: return mom_bwd_t<cd>(mom, R, Bq, ncl, z, yss, nrhs, s);
    case 2: return mom_bwd_t<float>(mom, R, Bq, ncl, z, yss, nrhs, s);
    case 3: return mom_bwd_t<cf>(mom, R, Bq, ncl, z, yss, nrhs, s);
    default: return cudaErrorInvalidValue;
  }
}
cudaError_t launch_transfer_fwd(int S, const void* T, int np2, int nc, int np_, const void* yc, void* yp, int nrhs,
                                cudaStream_t s) {
  if (np_ == 0) return cudaSuccess;
  switch (S) {
    case 0: k_transfer_fwd<double><<<np_, 256, 0, s>>>((const double*)T, np2, nc, (const double*)yc, (double*)yp, nrhs); break;
    case 1: k_transfer_fwd<cd><<<np_, 256, 0, s>>>((const double*)T, np2, nc, (const cd*)yc, (cd*)yp, nrhs); break;
    case 2: k_transfer_fwd<float><<<np_, 256, 0, s>>>((const float*)T, np2, nc, (const float*)yc, (float*)yp, nrhs); break;
    case 3: k_transfer_fwd<cf><<<np_, 256, 0, s>>>((const float*)T, np2, nc, (const cf*)yc, (cf*)yp, nrhs); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}
cudaError_t launch_transfer_bwd(int S, const void* T, int np2, int nc, int np_, const void* zp, void* zc, int nrhs,
                                cudaStream_t s) {
  if (np_ == 0) return cudaSuccess;
  switch (S) {
    case 0: k_transfer_bwd<double><<<np_, 256, 0, s>>>((const double*)T, np2, nc, (const double*)zp, (double*)zc, nrhs); break;
    case 1: k_transfer_bwd<cd><<<np_, 256, 0, s>>>((const double*)T, np2, nc, (const cd*)zp, (cd*)zc, nrhs); break;
    case 2: k_transfer_bwd<float><<<np_, 256, 0, s>>>((const float*)T, np2, nc, (const float*)zp, (float*)zc, nrhs); break;
    case 3: k_transfer_bwd<cf><<<np_, 256, 0, s>>>((const float*)T, np2, nc, (const cf*)zp, (cf*)zc, nrhs); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <bool CPLX>
static cudaError_t far_fused_t(const float4* prow, const float4* pcol, const int* row_ptr, const int* col, int nrows,
                               int np2, float kre, float kim, const void* y, void* z, int nrhs, cudaStream_t s) {
  if (nrows == 0) return cudaSuccess;
  const int bs = ((np2 + 31) / 32) * 32;
  const size_t smem = np2 * sizeof(float4) + (size_t)np2 * nrhs * (CPLX ? sizeof(cf) : sizeof(float));
#define BG_FF(NRV)                                                                                          \
  {                                                                                                         \
    auto kf = k_far_fused<CPLX, NRV>;                                                                       \
    cudaError_t e = cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);       \
    if (e != cudaSuccess) return e;                                                                         \
    kf<<<nrows, bs, smem, s>>>(prow, pcol, row_ptr, col, np2, kre, kim, y, z, nrhs);                        \
    return cudaGetLastError();                                                                              \
  }
  if (nrhs <= 1) BG_FF(1)
  if (nrhs <= 2) BG_FF(2)
  if (nrhs <= 4) BG_FF(4)
  if (nrhs <= 8) BG_FF(8)
  if (nrhs <= 16) BG_FF(16)
  if (nrhs <= 32) BG_FF(32)
#undef BG_FF
  return cudaErrorInvalidValue;
}
cudaError_t launch_far_fused(bool cplx, const float4* prow, const float4* pcol, const int* row_ptr, const int* col,
                             int nrows, int np2, float kre, float kim, const void* y, void* z, int nrhs,
                             cudaStream_t s) {
  return cplx ? far_fused_t<true>(prow, pcol, row_ptr, col, nrows, np2, kre, kim, y, z, nrhs, s)
              : far_fused_t<false>(prow, pcol, row_ptr, col, nrows, np2, kre, kim, y, z, nrhs, s);
}

cudaError_t launch_gather_in(int Sin, int Sout, const void* user, long ld, int rows, int nrhs, void* work,
                             cudaStream_t s) {
  const long n = (long)rows * nrhs;
  if (n == 0) return cudaSuccess;
  const unsigned g = blocks_for(n, 256);
  if (Sin == 0 && Sout == 0) k_gather_in<double, double><<<g, 256, 0, s>>>((const double*)user, ld, rows, nrhs, (double*)work);
  else if (Sin == 0 && Sout == 2) k_gather_in<double, float><<<g, 256, 0, s>>>((const double*)user, ld, rows, nrhs, (float*)work);
  else if (Sin == 1 && Sout == 1) k_gather_in<cd, cd><<<g, 256, 0, s>>>((const cd*)user, ld, rows, nrhs, (cd*)work);
  else if (Sin == 1 && Sout == 3) k_gather_in<cd, cf><<<g, 256, 0, s>>>((const cd*)user, ld, rows, nrhs, (cf*)work);
  else return cudaErrorInvalidValue;
  return cudaGetLastError();
}
cudaError_t launch_scatter_out(int Sw, const void* work, int rows, int nrhs, void* user, long ld, const double* alpha,
                               const double* beta, cudaStream_t s) {
  const long n = (long)rows * nrhs;
  if (n == 0) return cudaSuccess;
  const unsigned g = blocks_for(n, 256);
  const cd a = {alpha[0], alpha[1]}, b = {beta[0], beta[1]};
  switch (Sw) {
    case 0: k_scatter_out_real<double><<<g, 256, 0, s>>>((const double*)work, rows, nrhs, (double*)user, ld, alpha[0], beta[0]); break;
    case 2: k_scatter_out_real<float><<<g, 256, 0, s>>>((const float*)work, rows, nrhs, (double*)user, ld, alpha[0], beta[0]); break;
    case 1: k_scatter_out_cplx<cd><<<g, 256, 0, s>>>((const cd*)work, rows, nrhs, (cd*)user, ld, a, b); break;
    case 3: k_scatter_out_cplx<cf><<<g, 256, 0, s>>>((const cf*)work, rows, nrhs, (cd*)user, ld, a, b); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}
cudaError_t launch_convert(int Sin, int Sout, const void* in, long n, void* out, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const unsigned g = blocks_for(n, 256);
  if (Sin == 0 && Sout == 2) k_convert<double, float><<<g, 256, 0, s>>>((const double*)in, n, (float*)out);
  else if (Sin == 1 && Sout == 3) k_convert<cd, cf><<<g, 256, 0, s>>>((const cd*)in, n, (cf*)out);
  else if (Sin == 2 && Sout == 0) k_convert<float, double><<<g, 256, 0, s>>>((const float*)in, n, (double*)out);
  else if (Sin == 3 && Sout == 1) k_convert<cf, cd><<<g, 256, 0, s>>>((const cf*)in, n, (cd*)out);
  else return cudaErrorInvalidValue;
  return cudaGetLastError();
}

}  // namespace bg
