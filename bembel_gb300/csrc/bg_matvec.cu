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
#include <algorithm>
#include <type_traits>

#include <mutex>
#include <unordered_map>

#include "bg_kernels.cuh"

namespace bg {

cudaError_t raise_smem_limit(const void* func, size_t bytes) {
  static std::mutex mu;
  static std::unordered_map<const void*, size_t> limit;
  std::lock_guard<std::mutex> lk(mu);
  size_t& cur = limit[func];
  if (bytes <= cur) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) cur = bytes;
  return e;
}


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

// Neumaier's compensated summation step: sum + comp carries the running total
__device__ inline void neumaier_add(float& sum, float& comp, float v) {
  const float t = sum + v;
  comp += (fabsf(sum) >= fabsf(v)) ? ((sum - t) + v) : ((v - t) + sum);
  sum = t;
}
__device__ inline void neumaier_add(cf& sum, cf& comp, cf v) {
  neumaier_add(sum.re, comp.re, v.re);
  neumaier_add(sum.im, comp.im, v.im);
}

__device__ inline void cp_async16(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem));
}
__device__ inline void cp_async8(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem));
}
__device__ inline void cp_async4(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem));
}
__device__ inline void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ inline void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

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

// Pipelined block-sparse product for FP64 / complex FP64 blocks. Thread t
// owns row t % B and the NCOL right-hand sides of column group t / B. The
// next block (coupling matrix and its x panel) is staged with cp.async while
// the current one is multiplied from shared memory.
template <typename S, int NCOL>
__global__ void k_bsr_pipe(const int* __restrict__ row_ptr, const int* __restrict__ col, const S* __restrict__ blocks,
                           long bstride, int B, const S* __restrict__ x, S* __restrict__ y, int nrhs, int accumulate) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const long fsz = (B * B * (long)sizeof(S) + 15) / 16 * 16;  // bytes per staged block
  const long xsz = (B * nrhs * (long)sizeof(S) + 15) / 16 * 16;
  unsigned char* st[2] = {smem_raw, smem_raw + fsz + xsz};
  const int row = blockIdx.x, t = threadIdx.x;
  const int i = t % B, cg = t / B;
  const int c0 = cg * NCOL;
  const bool active = c0 < nrhs && cg * B + i == t;
  S acc[NCOL];
#pragma unroll
  for (int c = 0; c < NCOL; ++c) acc[c] = zero<S>();
  const int kb = row_ptr[row], ke = row_ptr[row + 1];
  auto issue = [&](int k, unsigned char* dst) {
    const unsigned char* F = reinterpret_cast<const unsigned char*>(blocks + (long)k * bstride);
    const long fbytes = (long)B * B * sizeof(S);
    for (long off = 16L * t; off < fbytes; off += 16L * blockDim.x) cp_async16(dst + off, F + off);
    const S* xs = x + (long)col[k] * B * nrhs;
    S* xd = reinterpret_cast<S*>(dst + fsz);
    for (int e = t; e < B * nrhs; e += blockDim.x) {
      if (sizeof(S) == 16) cp_async16(xd + e, xs + e);
      else if (sizeof(S) == 8) cp_async8(xd + e, xs + e);
      else cp_async4(xd + e, xs + e);
    }
    cp_async_commit();
  };
  if (kb < ke) issue(kb, st[0]);
  for (int k = kb; k < ke; ++k) {
    const int s = (k - kb) & 1;
    if (k + 1 < ke) {
      issue(k + 1, st[s ^ 1]);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    if (active) {
      const S* F = reinterpret_cast<const S*>(st[s]);
      const S* xs = reinterpret_cast<const S*>(st[s] + fsz);
      for (int j = 0; j < B; ++j) {
        const S f = F[j * B + i];
#pragma unroll
        for (int c = 0; c < NCOL; ++c)
          if (c0 + c < nrhs) acc[c] = fmac(acc[c], f, xs[j * nrhs + c0 + c]);
      }
    }
    __syncthreads();
  }
  if (active) {
    S* yo = y + ((long)row * B + i) * nrhs;
#pragma unroll
    for (int c = 0; c < NCOL; ++c)
      if (c0 + c < nrhs) yo[c0 + c] = accumulate ? add(yo[c0 + c], acc[c]) : acc[c];
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

// Batched small GEMM with one shared real matrix (FMM moments and transfers):
//   C[b] (=, +=) op(A) B[b],  op(A) = A (Mo x Ki) or A^T (A stored Ki x Mo),
// B[b]: Ki x kk row-major, C[b]: Mo x kk row-major; complex vectors are real
// matrices with kk = 2 * nrhs. Persistent CTAs stage A in shared memory once
// (when it fits) and loop over batch items; each thread owns an RT x CT tile.
template <typename T, bool TA, bool ACC, bool STAGE_A, int RT, int CT>
__global__ void __launch_bounds__(256) k_bgemm(const T* __restrict__ A, int Mo, int Ki, const T* __restrict__ B,
                                               long bstride, T* __restrict__ C, long cstride, int nbatch, int kk) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* As = reinterpret_cast<T*>(smem_raw);              // [q][i] (= op(A)^T), when staged
  T* Bs = As + (STAGE_A ? (size_t)Mo * Ki : 0);        // [q][c]
  if (STAGE_A) {
    for (int t = threadIdx.x; t < Mo * Ki; t += blockDim.x) {
      const int q = t / Mo, i = t - q * Mo;
      As[t] = TA ? A[(long)q * Mo + i] : A[(long)i * Ki + q];
    }
  }
  const int rtiles = (Mo + RT - 1) / RT, ctiles = (kk + CT - 1) / CT;
  for (int b = blockIdx.x; b < nbatch; b += gridDim.x) {
    __syncthreads();
    const T* Bb = B + (long)b * bstride;
    for (int t = threadIdx.x; t < Ki * kk; t += blockDim.x) Bs[t] = Bb[t];
    __syncthreads();
    T* Cb = C + (long)b * cstride;
    for (int tile = threadIdx.x; tile < rtiles * ctiles; tile += blockDim.x) {
      const int i0 = (tile / ctiles) * RT, c0 = (tile % ctiles) * CT;
      T acc[RT][CT];
#pragma unroll
      for (int r = 0; r < RT; ++r)
#pragma unroll
        for (int c = 0; c < CT; ++c) acc[r][c] = (T)0;
      for (int q = 0; q < Ki; ++q) {
        T a[RT], bv[CT];
#pragma unroll
        for (int r = 0; r < RT; ++r) {
          const int i = i0 + r < Mo ? i0 + r : Mo - 1;
          a[r] = STAGE_A ? As[(long)q * Mo + i] : (TA ? __ldg(&A[(long)q * Mo + i]) : __ldg(&A[(long)i * Ki + q]));
        }
#pragma unroll
        for (int c = 0; c < CT; ++c) bv[c] = Bs[q * kk + (c0 + c < kk ? c0 + c : kk - 1)];
#pragma unroll
        for (int r = 0; r < RT; ++r)
#pragma unroll
          for (int c = 0; c < CT; ++c) acc[r][c] = fmac(acc[r][c], a[r], bv[c]);
      }
#pragma unroll
      for (int r = 0; r < RT; ++r)
#pragma unroll
        for (int c = 0; c < CT; ++c)
          if (i0 + r < Mo && c0 + c < kk) {
            T* o = Cb + (long)(i0 + r) * kk + c0 + c;
            *o = ACC ? *o + acc[r][c] : acc[r][c];
          }
    }
  }
}

// K-chunked variant: one CTA per batch item, A and B staged KC rows of the
// inner dimension at a time (small shared footprint, many CTAs per SM).
template <typename T, bool TA, bool ACC, int RT, int CT, int KC>
__global__ void __launch_bounds__(256) k_bgemm_kc(const T* __restrict__ A, int Mo, int Ki, const T* __restrict__ B,
                                                  long bstride, T* __restrict__ C, long cstride, int kk) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* As = reinterpret_cast<T*>(smem_raw);  // [q][i], KC x Mo
  T* Bs = As + (size_t)KC * Mo;            // [q][c], KC x kk
  const int b = blockIdx.x;
  const T* Bb = B + (long)b * bstride;
  T* Cb = C + (long)b * cstride;
  const int rtiles = (Mo + RT - 1) / RT, ctiles = (kk + CT - 1) / CT, ntiles = rtiles * ctiles;
  constexpr int MAXT = 4;  // tiles per thread
  T acc[MAXT][RT][CT];
#pragma unroll
  for (int u = 0; u < MAXT; ++u)
#pragma unroll
    for (int r = 0; r < RT; ++r)
#pragma unroll
      for (int c = 0; c < CT; ++c) acc[u][r][c] = (T)0;
  for (int q0 = 0; q0 < Ki; q0 += KC) {
    const int qn = min(KC, Ki - q0);
    __syncthreads();
    for (int t = threadIdx.x; t < qn * Mo; t += blockDim.x) {
      const int q = t / Mo, i = t - q * Mo;
      As[t] = TA ? A[(long)(q0 + q) * Mo + i] : A[(long)i * Ki + q0 + q];
    }
    for (int t = threadIdx.x; t < qn * kk; t += blockDim.x) Bs[t] = Bb[(long)q0 * kk + t];
    __syncthreads();
#pragma unroll
    for (int u = 0; u < MAXT; ++u) {
      const int tile = threadIdx.x + u * blockDim.x;
      if (tile < ntiles) {
        const int i0 = (tile / ctiles) * RT, c0 = (tile % ctiles) * CT;
        for (int q = 0; q < qn; ++q) {
          T a[RT], bv[CT];
#pragma unroll
          for (int r = 0; r < RT; ++r) a[r] = As[q * Mo + min(i0 + r, Mo - 1)];
#pragma unroll
          for (int c = 0; c < CT; ++c) bv[c] = Bs[q * kk + min(c0 + c, kk - 1)];
#pragma unroll
          for (int r = 0; r < RT; ++r)
#pragma unroll
            for (int c = 0; c < CT; ++c) acc[u][r][c] = fmac(acc[u][r][c], a[r], bv[c]);
        }
      }
    }
  }
#pragma unroll
  for (int u = 0; u < MAXT; ++u) {
    const int tile = threadIdx.x + u * blockDim.x;
    if (tile < ntiles) {
      const int i0 = (tile / ctiles) * RT, c0 = (tile % ctiles) * CT;
#pragma unroll
      for (int r = 0; r < RT; ++r)
#pragma unroll
        for (int c = 0; c < CT; ++c)
          if (i0 + r < Mo && c0 + c < kk) {
            T* o = Cb + (long)(i0 + r) * kk + c0 + c;
            *o = ACC ? *o + acc[u][r][c] : acc[u][r][c];
          }
    }
  }
}

template <typename T>
static cudaError_t bgemm(bool ta, bool acc, const T* A, int Mo, int Ki, const T* B, long bstride, T* C, long cstride,
                         int nbatch, int kk, cudaStream_t s) {
  if (nbatch == 0) return cudaSuccess;
  constexpr int RT = 3, CT = 4, KC = 32;
  const long ntiles = (long)((Mo + RT - 1) / RT) * ((kk + CT - 1) / CT);
  if (ntiles > 4 * 256) {
    // large outputs: persistent kernel with the whole A staged
    const size_t a_bytes = (size_t)Mo * Ki * sizeof(T), b_bytes = (size_t)Ki * kk * sizeof(T);
    const bool stage = a_bytes + b_bytes <= 200 * 1024;
    if (!stage && b_bytes > 200 * 1024) return cudaErrorInvalidValue;
    const size_t smem = (stage ? a_bytes : 0) + b_bytes;
    const int grid = std::min(nbatch, 4 * 152);
#define BG_GEMM(TA_, AC_, ST_)                                                                             \
    {                                                                                                      \
      auto kf = k_bgemm<T, TA_, AC_, ST_, 3, 4>;                                                           \
      cudaError_t e = smem_limit(kf, smem);    \
      if (e != cudaSuccess) return e;                                                                      \
      kf<<<grid, 256, smem, s>>>(A, Mo, Ki, B, bstride, C, cstride, nbatch, kk);                           \
      return cudaGetLastError();                                                                           \
    }
    if (!ta && !acc && stage) BG_GEMM(false, false, true)
    if (!ta && !acc && !stage) BG_GEMM(false, false, false)
    if (ta && acc && stage) BG_GEMM(true, true, true)
    if (ta && acc && !stage) BG_GEMM(true, true, false)
#undef BG_GEMM
    return cudaErrorInvalidValue;
  }
  const size_t smem = (size_t)KC * (Mo + kk) * sizeof(T);
#define BG_KC(TA_, AC_)                                                                                    \
  {                                                                                                        \
    auto kf = k_bgemm_kc<T, TA_, AC_, RT, CT, KC>;                                                         \
    cudaError_t e = smem_limit(kf, smem);      \
    if (e != cudaSuccess) return e;                                                                        \
    kf<<<nbatch, 256, smem, s>>>(A, Mo, Ki, B, bstride, C, cstride, kk);                                   \
    return cudaGetLastError();                                                                             \
  }
  if (!ta && !acc) BG_KC(false, false)
  if (ta && acc) BG_KC(true, true)
#undef BG_KC
  return cudaErrorInvalidValue;
}

// FMM transforms as batched GEMMs with one shared matrix:
//   C[b] (=, +=) op(A) B[b]   (op(A): Mo x Ki; B[b]: Ki x kk; C[b]: Mo x kk)
// op(A) is given transposed and padded, AT[q][i] with row length ld (a
// multiple of 4 and at least Mo rounded up to 3, zero beyond Mo), so its
// chunks stage with coalesced 16-byte cp.async. One CTA per batch item and 32
// columns; K is staged 16 rows at a time, double-buffered; each thread owns up
// to 4 tiles of 3 rows x 4 columns.
template <typename T>
__device__ __forceinline__ void load4(const T* p, T* v) {
  if constexpr (sizeof(T) == 4) {
    const float4 q = *reinterpret_cast<const float4*>(p);
    v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
  } else {
    const double2 q0 = *reinterpret_cast<const double2*>(p), q1 = *reinterpret_cast<const double2*>(p + 2);
    v[0] = q0.x; v[1] = q0.y; v[2] = q1.x; v[3] = q1.y;
  }
}

template <typename T, bool ACC, int MAXT>
__global__ void __launch_bounds__(256) k_tgemm(const T* __restrict__ AT, int ld, int Mo, int Ki,
                                               const T* __restrict__ B, long bstride, T* __restrict__ C, long cstride,
                                               int kk, int vec_b) {
  constexpr int KC = 16, RT = 3, CT = 4, NCOL = 32;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* As = reinterpret_cast<T*>(smem_raw);  // [2][KC][ld]
  T* Bs = As + 2 * KC * ld;                // [2][KC][NCOL]
  const int b = blockIdx.x, cbase = NCOL * blockIdx.y;
  const int ncol = min(NCOL, kk - cbase);
  const T* Bb = B + (long)b * bstride + cbase;
  const int tid = threadIdx.x;
  // columns beyond ncol are never copied into: zero them once in both buffers
  if (ncol < NCOL)
    for (int t = tid; t < 2 * KC * NCOL; t += blockDim.x)
      if ((t % NCOL) >= ncol) Bs[t] = (T)0;
  auto stage = [&](int q0, int buf) {
    const int qn = min(KC, Ki - q0);
    const unsigned char* asrc = reinterpret_cast<const unsigned char*>(AT + (long)q0 * ld);
    unsigned char* adst = reinterpret_cast<unsigned char*>(As + buf * KC * ld);
    const int abytes = qn * ld * (int)sizeof(T);
    for (int o = 16 * tid; o < abytes; o += 16 * blockDim.x) cp_async16(adst + o, asrc + o);
    T* bdst = Bs + buf * KC * NCOL;
    if (vec_b) {
      const int per_row = ncol * (int)sizeof(T) / 16;
      for (int t = tid; t < qn * per_row; t += blockDim.x) {
        const int q = t / per_row, v = t - q * per_row;
        cp_async16(reinterpret_cast<unsigned char*>(bdst + q * NCOL) + 16 * v,
                   reinterpret_cast<const unsigned char*>(Bb + (long)(q0 + q) * kk) + 16 * v);
      }
    } else {
      for (int t = tid; t < qn * ncol; t += blockDim.x) {
        const int q = t / ncol, c = t - q * ncol;
        bdst[q * NCOL + c] = Bb[(long)(q0 + q) * kk + c];
      }
    }
    cp_async_commit();
  };
  const int rtiles = (Mo + RT - 1) / RT, ctiles = (ncol + CT - 1) / CT, ntiles = rtiles * ctiles;
  T acc[MAXT][RT][CT];
#pragma unroll
  for (int u = 0; u < MAXT; ++u)
#pragma unroll
    for (int r = 0; r < RT; ++r)
#pragma unroll
      for (int c = 0; c < CT; ++c) acc[u][r][c] = (T)0;
  stage(0, 0);
  const int nchunks = (Ki + KC - 1) / KC;
  for (int ch = 0; ch < nchunks; ++ch) {
    const int buf = ch & 1, q0 = ch * KC, qn = min(KC, Ki - q0);
    cp_async_wait<0>();
    __syncthreads();  // chunk ch staged; everyone is done with buffer buf^1
    if (ch + 1 < nchunks) stage(q0 + KC, buf ^ 1);
    const T* as = As + buf * KC * ld;
    const T* bs = Bs + buf * KC * NCOL;
#pragma unroll
    for (int u = 0; u < MAXT; ++u) {
      const int tile = tid + u * blockDim.x;
      if (tile < ntiles) {
        const int i0 = (tile / ctiles) * RT, c0 = (tile % ctiles) * CT;
        for (int q = 0; q < qn; ++q) {
          T a[RT], bv[CT];
#pragma unroll
          for (int r = 0; r < RT; ++r) a[r] = as[q * ld + i0 + r];
          load4(bs + q * NCOL + c0, bv);
#pragma unroll
          for (int r = 0; r < RT; ++r)
#pragma unroll
            for (int c = 0; c < CT; ++c) acc[u][r][c] = fma(a[r], bv[c], acc[u][r][c]);
        }
      }
    }
  }
  T* Cb = C + (long)b * cstride + cbase;
#pragma unroll
  for (int u = 0; u < MAXT; ++u) {
    const int tile = tid + u * blockDim.x;
    if (tile < ntiles) {
      const int i0 = (tile / ctiles) * RT, c0 = (tile % ctiles) * CT;
#pragma unroll
      for (int r = 0; r < RT; ++r)
#pragma unroll
        for (int c = 0; c < CT; ++c)
          if (i0 + r < Mo && c0 + c < ncol) {
            T* o = Cb + (long)(i0 + r) * kk + c0 + c;
            *o = ACC ? *o + acc[u][r][c] : acc[u][r][c];
          }
    }
  }
}

// Few batch items (coarse FMM levels): one CTA of up to 1024 threads per item
// and 32 columns stages all of op(A)^T and B at once, then splits K across
// ksplit thread groups; partial tiles are added in a fixed order, so the result
// does not depend on scheduling.
template <bool ACC>
__global__ void __launch_bounds__(1024) k_tgemm_small(const float* __restrict__ AT, int ld, int Mo, int Ki,
                                                      const float* __restrict__ B, long bstride, float* __restrict__ C,
                                                      long cstride, int kk, int vec_b, int ksplit) {
  constexpr int RT = 3, CT = 4, NCOL = 32;
  extern __shared__ __align__(16) float smg[];
  float* As = smg;                     // [Ki][ld]
  float* Bs = As + (size_t)Ki * ld;    // [Ki][NCOL]
  float* red = Bs + (size_t)Ki * NCOL; // [ksplit - 1][ntiles][RT * CT]
  const int b = blockIdx.x, cbase = NCOL * blockIdx.y, tid = threadIdx.x;
  const int ncol = min(NCOL, kk - cbase);
  const float* Bb = B + (long)b * bstride + cbase;
  for (int o = 4 * tid; o < Ki * ld; o += 4 * blockDim.x) cp_async16(As + o, AT + o);
  if (vec_b) {
    const int per_row = ncol / 4;
    for (int t = tid; t < Ki * per_row; t += blockDim.x) {
      const int q = t / per_row, v = t - q * per_row;
      cp_async16(Bs + q * NCOL + 4 * v, Bb + (long)q * kk + 4 * v);
    }
  } else {
    for (int t = tid; t < Ki * ncol; t += blockDim.x) {
      const int q = t / ncol, c = t - q * ncol;
      Bs[q * NCOL + c] = Bb[(long)q * kk + c];
    }
  }
  if (ncol < NCOL)
    for (int t = tid; t < Ki * NCOL; t += blockDim.x)
      if (t % NCOL >= ncol) Bs[t] = 0.0f;
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();
  const int rtiles = (Mo + RT - 1) / RT, ctiles = (ncol + CT - 1) / CT, ntiles = rtiles * ctiles;
  const int tile = tid % ntiles, kq = tid / ntiles;
  const bool active = kq < ksplit;
  float acc[RT][CT];
#pragma unroll
  for (int r = 0; r < RT; ++r)
#pragma unroll
    for (int c = 0; c < CT; ++c) acc[r][c] = 0.0f;
  const int i0 = (tile / ctiles) * RT, c0 = (tile % ctiles) * CT;
  if (active) {
    const int q0 = (int)((long)kq * Ki / ksplit), q1 = (int)((long)(kq + 1) * Ki / ksplit);
    for (int q = q0; q < q1; ++q) {
      float a[RT], bv[CT];
#pragma unroll
      for (int r = 0; r < RT; ++r) a[r] = As[q * ld + i0 + r];
      load4(Bs + q * NCOL + c0, bv);
#pragma unroll
      for (int r = 0; r < RT; ++r)
#pragma unroll
        for (int c = 0; c < CT; ++c) acc[r][c] = fmaf(a[r], bv[c], acc[r][c]);
    }
    if (kq > 0) {
      float* rp = red + ((size_t)(kq - 1) * ntiles + tile) * (RT * CT);
#pragma unroll
      for (int r = 0; r < RT; ++r)
#pragma unroll
        for (int c = 0; c < CT; ++c) rp[r * CT + c] = acc[r][c];
    }
  }
  __syncthreads();
  if (active && kq == 0) {
    for (int g = 1; g < ksplit; ++g) {
      const float* rp = red + ((size_t)(g - 1) * ntiles + tile) * (RT * CT);
#pragma unroll
      for (int r = 0; r < RT; ++r)
#pragma unroll
        for (int c = 0; c < CT; ++c) acc[r][c] += rp[r * CT + c];
    }
    float* Cb = C + (long)b * cstride + cbase;
#pragma unroll
    for (int r = 0; r < RT; ++r)
#pragma unroll
      for (int c = 0; c < CT; ++c)
        if (i0 + r < Mo && c0 + c < ncol) {
          float* o = Cb + (long)(i0 + r) * kk + c0 + c;
          *o = ACC ? *o + acc[r][c] : acc[r][c];
        }
  }
}

template <typename T>
static cudaError_t tgemm_t(bool acc, const TGemmA& A, const T* B, long bstride, T* C, long cstride, int nbatch, int kk,
                           cudaStream_t s, int split_k_batches) {
  if constexpr (sizeof(T) == 4) {
    // coarse levels: fewer CTAs than SMs -> whole-operand staging and split K
    const long ctas = (long)nbatch * ((kk + 31) / 32);
    const long split_max = split_k_batches < 0 ? 152 : split_k_batches;
    const int ntiles = ((A.Mo + 2) / 3) * 8;
    if (nbatch > 0 && ctas <= split_max && ntiles <= 1024 && A.ld % 4 == 0 && A.ld >= (A.Mo + 2) / 3 * 3) {
      const int ksplit = std::max(1, std::min(8, 1024 / ntiles));
      const int threads = std::min(1024, (ntiles * ksplit + 31) / 32 * 32);
      const size_t smem = ((size_t)A.Ki * A.ld + (size_t)A.Ki * 32 + (size_t)(ksplit - 1) * ntiles * 12) * 4;
      if (smem <= 200 * 1024) {
        const int vec_b = (kk % 4) == 0 && (bstride % 4) == 0 && (reinterpret_cast<uintptr_t>(B) % 16) == 0;
        auto kf = acc ? k_tgemm_small<true> : k_tgemm_small<false>;
        cudaError_t e = smem_limit(kf, smem);
        if (e != cudaSuccess) return e;
        kf<<<dim3(nbatch, (kk + 31) / 32), threads, smem, s>>>(reinterpret_cast<const float*>(A.at), A.ld, A.Mo, A.Ki,
                                                                reinterpret_cast<const float*>(B), bstride,
                                                                reinterpret_cast<float*>(C), cstride, kk, vec_b, ksplit);
        return cudaGetLastError();
      }
    }
  }
  if (nbatch == 0) return cudaSuccess;
  const int rtiles = (A.Mo + 2) / 3;
  // up to 4 (or, for op(A) of up to 512 rows, 6) tiles of 3 x 4 per thread
  if (rtiles * 8 > 6 * 256 || A.ld < rtiles * 3 || A.ld % 4 != 0) return cudaErrorInvalidValue;
  const size_t smem = (size_t)2 * 16 * (A.ld + 32) * sizeof(T);
  const int vec_b = (kk * sizeof(T)) % 16 == 0 && (bstride * sizeof(T)) % 16 == 0 &&
                    (reinterpret_cast<uintptr_t>(B) % 16) == 0;
  const dim3 grid(nbatch, (kk + 31) / 32);
  const bool big = rtiles * 8 > 4 * 256;
  auto kf = big ? (acc ? k_tgemm<T, true, 6> : k_tgemm<T, false, 6>) : (acc ? k_tgemm<T, true, 4> : k_tgemm<T, false, 4>);
  cudaError_t e = smem_limit(kf, smem);
  if (e != cudaSuccess) return e;
  kf<<<grid, 256, smem, s>>>(static_cast<const T*>(A.at), A.ld, A.Mo, A.Ki, B, bstride, C, cstride, kk, vec_b);
  return cudaGetLastError();
}

cudaError_t launch_tgemm(int S, bool acc, const TGemmA& A, const void* B, long bstride_rows, void* C,
                         long cstride_rows, int nbatch, int nrhs, cudaStream_t s, int split_k_batches) {
  // complex vectors are real matrices with 2 nrhs columns
  const int kk = (S & 1) ? 2 * nrhs : nrhs;
  if (S < 2)
    return tgemm_t<double>(acc, A, static_cast<const double*>(B), bstride_rows * kk, static_cast<double*>(C),
                           cstride_rows * kk, nbatch, kk, s, split_k_batches);
  return tgemm_t<float>(acc, A, static_cast<const float*>(B), bstride_rows * kk, static_cast<float*>(C),
                        cstride_rows * kk, nbatch, kk, s, split_k_batches);
}

// Fused FP32 far field: the coupling F_ij = k(x_i, y_j) |J_i| |J_j| is
// generated from the clusters' interpolation points inside the product, so the
// far field is never stored. One CTA (128 threads) per block row (cluster c1).
// Per block: the next block's points and right-hand sides are prefetched with
// cp.async while the CTA writes the np2 x np2 coupling tile to shared memory
// ([j][i], conflict-free) and contracts it; each thread owns ROWS rows x NC
// right-hand sides. Block results are summed with Neumaier compensation.
// Points are FP32 offsets from FP64 cluster centres (centre differences in
// FP64), which keeps near-admissible distances accurate to FP32 rounding.
template <bool CPLX, int NP2, int NC>
__global__ void __launch_bounds__(128) k_far_fused(const float4* __restrict__ pts, const d4* __restrict__ centres,
                                                   const int* __restrict__ row_ptr, const int* __restrict__ col,
                                                   float kre, float kim, const void* __restrict__ yv,
                                                   void* __restrict__ zv, int nrhs) {
  typedef typename std::conditional<CPLX, cf, float>::type S;
  typedef typename std::conditional<CPLX, float2, float>::type FT;
  constexpr int ROWS = (NP2 + 31) / 32;
  constexpr int LD = 4 * NC;  // padded right-hand-side row length
  const S* y = static_cast<const S*>(yv);
  S* z = static_cast<S*>(zv);
  __shared__ float4 prs[NP2];
  __shared__ float4 pcs[2][NP2];
  __shared__ __align__(16) S ys[2][NP2 * LD];
  extern __shared__ __align__(16) unsigned char smem_raw[];
  FT* F = reinterpret_cast<FT*>(smem_raw);  // [j][i]
  const int row = blockIdx.x;
  const int lane = threadIdx.x & 31, cg = threadIdx.x >> 5;
  const int c0 = cg * NC;
  for (int t = threadIdx.x; t < NP2; t += blockDim.x) prs[t] = pts[(long)row * NP2 + t];
  const d4 crow = centres[row];
  const bool dense_rhs = (nrhs == LD);
  auto issue = [&](int k, int b) {
    const int c2 = col[k];
    for (int t = threadIdx.x; t < NP2; t += blockDim.x) cp_async16(&pcs[b][t], &pts[(long)c2 * NP2 + t]);
    const S* src = y + (long)c2 * NP2 * nrhs;
    if (dense_rhs) {
      constexpr int CH = (int)(NP2 * LD * sizeof(S) / 16);
      for (int t = threadIdx.x; t < CH; t += blockDim.x)
        cp_async16(reinterpret_cast<unsigned char*>(ys[b]) + 16 * t, reinterpret_cast<const unsigned char*>(src) + 16 * t);
    } else {
      for (int t = threadIdx.x; t < NP2 * LD; t += blockDim.x) {
        const int j = t / LD, c = t - j * LD;
        if (c < nrhs) {
          if (sizeof(S) == 8) cp_async8(&ys[b][t], &src[j * nrhs + c]);
          else ys[b][t] = src[j * nrhs + c];
        } else {
          ys[b][t] = zero<S>();
        }
      }
    }
    cp_async_commit();
  };
  S sum[ROWS][NC], cmp[ROWS][NC];
#pragma unroll
  for (int r = 0; r < ROWS; ++r)
#pragma unroll
    for (int c = 0; c < NC; ++c) sum[r][c] = cmp[r][c] = zero<S>();
  const int kb = row_ptr[row], ke = row_ptr[row + 1];
  if (kb < ke) issue(kb, 0);
  for (int k = kb; k < ke; ++k) {
    const int b = (k - kb) & 1;
    cp_async_wait<0>();
    __syncthreads();  // block k staged; every thread is done with F and buffer b^1
    if (k + 1 < ke) issue(k + 1, b ^ 1);
    const d4 ccol = centres[col[k]];
    const float dcx = (float)(crow.x - ccol.x), dcy = (float)(crow.y - ccol.y), dcz = (float)(crow.z - ccol.z);
    for (int e = threadIdx.x; e < NP2 * NP2; e += blockDim.x) {
      const int j = e / NP2, i = e - j * NP2;
      const float4 xi = prs[i], yj = pcs[b][j];
      const float d0 = dcx + (xi.x - yj.x), d1 = dcy + (xi.y - yj.y), d2 = dcz + (xi.z - yj.z);
      const float r2 = fmaf(d0, d0, fmaf(d1, d1, d2 * d2));
      const float inv = rsqrtf(r2);
      const float amp = inv * 0.0795774715f * xi.w * yj.w;
      if constexpr (CPLX) {
        const float r = r2 * inv;
        float sn, cs;
        sincosf(kre * r, &sn, &cs);
        float a = amp;
        if (kim != 0.0f) a *= expf(kim * r);
        F[e] = make_float2(cs * a, -sn * a);
      } else {
        F[e] = amp;
      }
    }
    __syncthreads();  // coupling tile complete
    S acc[ROWS][NC];
#pragma unroll
    for (int r = 0; r < ROWS; ++r)
#pragma unroll
      for (int c = 0; c < NC; ++c) acc[r][c] = zero<S>();
#pragma unroll 3
    for (int j = 0; j < NP2; ++j) {
      S yl[NC];
      if constexpr ((NC * sizeof(S)) % 16 == 0) {
        const float4* src = reinterpret_cast<const float4*>(&ys[b][j * LD + c0]);
#pragma unroll
        for (int v = 0; v < (int)(NC * sizeof(S) / 16); ++v) {
          const float4 q = src[v];
          float* d = reinterpret_cast<float*>(yl) + 4 * v;
          d[0] = q.x; d[1] = q.y; d[2] = q.z; d[3] = q.w;
        }
      } else {
#pragma unroll
        for (int c = 0; c < NC; ++c) yl[c] = ys[b][j * LD + c0 + c];
      }
#pragma unroll
      for (int r = 0; r < ROWS; ++r) {
        const int i = lane + 32 * r;
        if (i < NP2) {
          const FT f = F[j * NP2 + i];
#pragma unroll
          for (int c = 0; c < NC; ++c) {
            if constexpr (CPLX) acc[r][c] = fmac(acc[r][c], cf{f.x, f.y}, yl[c]);
            else acc[r][c] = fmac(acc[r][c], f, yl[c]);
          }
        }
      }
    }
#pragma unroll
    for (int r = 0; r < ROWS; ++r)
#pragma unroll
      for (int c = 0; c < NC; ++c) neumaier_add(sum[r][c], cmp[r][c], acc[r][c]);
  }
#pragma unroll
  for (int r = 0; r < ROWS; ++r) {
    const int i = lane + 32 * r;
    if (i < NP2) {
      S* zo = z + ((long)row * NP2 + i) * nrhs;
#pragma unroll
      for (int c = 0; c < NC; ++c)
        if (c0 + c < nrhs) zo[c0 + c] = add(sum[r][c], cmp[r][c]);
    }
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
template <typename S64, typename S32>
__global__ void k_add_low(const S32* __restrict__ in, long n, S64* __restrict__ out) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) out[t] = add(out[t], Conv<S32, S64>::run(in[t]));
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
    cudaError_t e = smem_limit(kf, smem);        \
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
static cudaError_t bsr_pipe_typed(const int* row_ptr, const int* col, const S* blocks, long bstride, int nrows, int B,
                                  const S* x, S* y, int nrhs, int accumulate, cudaStream_t s) {
  if (nrows == 0) return cudaSuccess;
  // column groups: enough threads to cover B rows x nrhs, at most 1024 threads
  int ncol = nrhs <= 1 ? 1 : (nrhs <= 2 ? 2 : (nrhs <= 4 ? 4 : 8));
  int groups = (nrhs + ncol - 1) / ncol;
  while (B * groups > 1024) {
    ncol *= 2;
    groups = (nrhs + ncol - 1) / ncol;
  }
  if (ncol > 32) return cudaErrorInvalidValue;
  const int threads = ((B * groups + 31) / 32) * 32;
  const size_t fsz = ((size_t)B * B * sizeof(S) + 15) / 16 * 16, xsz = ((size_t)B * nrhs * sizeof(S) + 15) / 16 * 16;
  const size_t smem = 2 * (fsz + xsz);
  if (smem > 220 * 1024) {
    // too large to double-buffer: single-stage kernel on contiguous blocks
    if (bstride != (long)B * B) return cudaErrorInvalidValue;
    return bsr_typed<S>(row_ptr, col, blocks, nrows, B, x, y, nrhs, accumulate, s);
  }
#define BG_PIPE(NC)                                                                                         \
  if (ncol == NC) {                                                                                         \
    auto kf = k_bsr_pipe<S, NC>;                                                                            \
    cudaError_t e = smem_limit(kf, smem);       \
    if (e != cudaSuccess) return e;                                                                         \
    kf<<<nrows, threads, smem, s>>>(row_ptr, col, blocks, bstride, B, x, y, nrhs, accumulate);              \
    return cudaGetLastError();                                                                              \
  }
  BG_PIPE(1)
  BG_PIPE(2)
  BG_PIPE(4)
  BG_PIPE(8)
  BG_PIPE(16)
  BG_PIPE(32)
#undef BG_PIPE
  return cudaErrorInvalidValue;
}
cudaError_t launch_bsr_fp64(bool cplx, const int* row_ptr, const int* col, const void* blocks, long bstride, int nrows,
                            int B, const void* x, void* y, int nrhs, int accumulate, cudaStream_t s) {
  if (cplx)
    return bsr_pipe_typed<cd>(row_ptr, col, (const cd*)blocks, bstride, nrows, B, (const cd*)x, (cd*)y, nrhs, accumulate, s);
  return bsr_pipe_typed<double>(row_ptr, col, (const double*)blocks, bstride, nrows, B, (const double*)x, (double*)y,
                                nrhs, accumulate, s);
}
// Double-float block-sparse product for real operators. Blocks are stored as
// FP32 pairs (hi, lo) with hi + lo equal to the FP64 coupling to 2^-48 and x
// arrives split the same way (launch_split_df). Every multiply-add forms
// hi*hi exactly (product plus its fmaf error), adds the cross terms
// hi*lo + lo*hi, and sums with TwoSum into an FP32 pair per output, so the
// result matches the FP64 product to about 1e-14 relative while running on
// the FP32 pipes (GB300's FP64 rate is 1/64 of its FP32 rate).
// Thread t owns row t % B and NCOL right-hand sides of column group t / B.
// The block is read from global memory directly (each element once per
// column group, coalesced along a block column; the groups share it through
// L1); only the x panels are staged, double-buffered with cp.async, so
// several CTAs fit on an SM.
template <int NCOL, bool FULL>
__global__ void __launch_bounds__(352) k_bsr_df(const int* __restrict__ row_ptr, const int* __restrict__ col,
                                                const float2* __restrict__ blocks, long bstride, int B,
                                                const float2* __restrict__ x, double* __restrict__ y, int nrhs,
                                                int ldy, int y0, int accumulate) {
  extern __shared__ __align__(16) float2 xsm[];  // [2][B * nrhs]
  const int row = blockIdx.x, t = threadIdx.x;
  const int i = t % B, cg = t / B, c0 = cg * NCOL;
  const bool active = c0 < nrhs && cg * B + i == t;
  const int panel = B * nrhs;
  float s[NCOL], cc[NCOL];
#pragma unroll
  for (int c = 0; c < NCOL; ++c) s[c] = cc[c] = 0.0f;
  const int kb = row_ptr[row], ke = row_ptr[row + 1];
  auto issue = [&](int k, int buf) {
    const float2* src = x + (long)col[k] * panel;
    float2* dst = xsm + buf * panel;
    if ((panel & 1) == 0) {
      for (int e = 2 * t; e < panel; e += 2 * blockDim.x) cp_async16(dst + e, src + e);
    } else {
      for (int e = t; e < panel; e += blockDim.x) cp_async8(dst + e, src + e);
    }
    cp_async_commit();
  };
  if (kb < ke) issue(kb, 0);
  for (int k = kb; k < ke; ++k) {
    const int buf = (k - kb) & 1;
    cp_async_wait<0>();
    __syncthreads();  // panel k staged; everyone is done with panel k-1
    if (k + 1 < ke) issue(k + 1, buf ^ 1);
    if (active) {
      const float2* F = blocks + (long)k * bstride + i;
      const float2* xp = xsm + buf * panel + c0;
      auto madd = [&](const float2 f, const float2* xv) {
#pragma unroll
        for (int c = 0; c < NCOL; ++c) {
          if (FULL || c0 + c < nrhs) {
            const float2 b = xv[c];
            const float p = f.x * b.x;
            float e = fmaf(f.x, b.x, -p);
            e = fmaf(f.x, b.y, e);
            e = fmaf(f.y, b.x, e);
            const float tt = s[c] + p, z = tt - s[c];
            cc[c] += ((s[c] - (tt - z)) + (p - z)) + e;
            s[c] = tt;
          }
        }
      };
      // block columns in groups of 4, the next group's couplings loaded
      // while the current one is multiplied
      constexpr int G = 4;
      const int jg = B / G * G;
      float2 fa[G], fb[G];
#pragma unroll
      for (int u = 0; u < G; ++u) fa[u] = u < jg ? __ldg(F + (long)u * B) : make_float2(0.f, 0.f);
      for (int j = 0; j < jg; j += G) {
#pragma unroll
        for (int u = 0; u < G; ++u) fb[u] = j + G + u < jg ? __ldg(F + (long)(j + G + u) * B) : make_float2(0.f, 0.f);
#pragma unroll
        for (int u = 0; u < G; ++u) madd(fa[u], xp + (j + u) * nrhs);
#pragma unroll
        for (int u = 0; u < G; ++u) fa[u] = fb[u];
      }
      for (int j = jg; j < B; ++j) madd(__ldg(F + (long)j * B), xp + j * nrhs);
    }
  }
  if (active) {
    double* yo = y + ((long)row * B + i) * ldy + y0;
#pragma unroll
    for (int c = 0; c < NCOL; ++c)
      if (FULL || c0 + c < nrhs) {
        const double v = (double)s[c] + (double)cc[c];
        yo[c0 + c] = accumulate ? yo[c0 + c] + v : v;
      }
  }
}

// FP64-accurate near field for 32 right-hand sides on both pipes at once:
// the double-float arithmetic of k_bsr_df runs on the FP32 pipe and the FP64
// pipe sits idle, so a quarter of the columns (24 .. 31) go to native FP64
// fma on the FP64 pipe in warps of their own. Per CTA (one block row):
// warps 0-3 are the double-float role (thread = block row i x 8 of columns
// 0 .. 23, 3 B threads active), warps 4-5 the FP64 role (thread = block row
// i x columns 24 .. 31). Both read the same block: its (hi, lo) pairs and its
// FP64 entries (same element stride); x arrives split (columns 0 .. 23) and in
// FP64 (columns 24 .. 31), both panels double-buffered with cp.async.
constexpr int kMixThreads = 192, kMixDfThreads = 128, kMixCols = 32, kMixDfCols = 24;
__global__ void __launch_bounds__(kMixThreads) k_bsr_near_mix(const int* __restrict__ row_ptr,
                                                             const int* __restrict__ col,
                                                             const float2* __restrict__ pairs,
                                                             const double* __restrict__ blocks64, long bstride,
                                                             int B, const float2* __restrict__ xdf,
                                                             const double* __restrict__ x64,
                                                             double* __restrict__ y) {
  extern __shared__ __align__(16) unsigned char mix_smem[];
  float2* xs = reinterpret_cast<float2*>(mix_smem);  // [2][B][24] split x
  double* xd = reinterpret_cast<double*>(xs + 2 * B * kMixDfCols);  // [2][B][8] FP64 x
  constexpr int NF = kMixCols - kMixDfCols;
  const int row = blockIdx.x, t = threadIdx.x;
  const int kb = row_ptr[row], ke = row_ptr[row + 1];
  auto issue = [&](int k, int buf) {
    const long r0 = (long)col[k] * B;
    // split columns 0 .. 23: 24 pairs = 192 bytes per row, 12 x 16 bytes
    for (int e = t; e < B * 12; e += kMixThreads) {
      const int r = e / 12, q = e - r * 12;
      cp_async16(xs + (buf * B + r) * kMixDfCols + 2 * q, xdf + (r0 + r) * kMixCols + 2 * q);
    }
    // FP64 columns 24 .. 31: 64 bytes per row, 4 x 16 bytes
    for (int e = t; e < B * 4; e += kMixThreads) {
      const int r = e >> 2, q = e & 3;
      cp_async16(xd + (buf * B + r) * NF + 2 * q, x64 + (r0 + r) * kMixCols + kMixDfCols + 2 * q);
    }
    cp_async_commit();
  };
  const bool df = t < kMixDfThreads;
  const int tt = df ? t : t - kMixDfThreads;
  const int i = df ? tt % B : tt, cg = df ? tt / B : 0;
  const bool active = df ? (tt < 3 * B) : (tt < B);
  float s[8], cc[8];
  double a[NF];
#pragma unroll
  for (int c = 0; c < 8; ++c) s[c] = cc[c] = 0.0f;
#pragma unroll
  for (int c = 0; c < NF; ++c) a[c] = 0.0;
  if (kb < ke) issue(kb, 0);
  for (int k = kb; k < ke; ++k) {
    const int buf = (k - kb) & 1;
    cp_async_wait<0>();
    __syncthreads();  // panels k staged; everyone is done with panels k-1
    if (k + 1 < ke) issue(k + 1, buf ^ 1);
    if (active && df) {
      const float2* F = pairs + (long)k * bstride + i;
      const float2* xp = xs + buf * B * kMixDfCols + 8 * cg;
      for (int j = 0; j < B; ++j) {
        const float2 f = __ldg(F + (long)j * B);
        const float2* xv = xp + j * kMixDfCols;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          const float2 b = xv[c];
          const float p = f.x * b.x;
          float e = fmaf(f.x, b.x, -p);
          e = fmaf(f.x, b.y, e);
          e = fmaf(f.y, b.x, e);
          const float ts = s[c] + p, z = ts - s[c];
          cc[c] += ((s[c] - (ts - z)) + (p - z)) + e;
          s[c] = ts;
        }
      }
    } else if (active) {
      const double* F = blocks64 + (long)k * bstride + i;
      const double* xp = xd + buf * B * NF;
      for (int j = 0; j < B; ++j) {
        const double f = __ldg(F + (long)j * B);
#pragma unroll
        for (int c = 0; c < NF; ++c) a[c] = fma(f, xp[j * NF + c], a[c]);
      }
    }
  }
  if (!active) return;
  double* yo = y + ((long)row * B + i) * kMixCols;
  if (df) {
#pragma unroll
    for (int c = 0; c < 8; ++c) yo[8 * cg + c] = (double)s[c] + (double)cc[c];
  } else {
#pragma unroll
    for (int c = 0; c < NF; ++c) yo[kMixDfCols + c] = a[c];
  }
}

cudaError_t launch_bsr_near_mix(const int* row_ptr, const int* col, const void* pairs, const void* blocks64,
                                long bstride, int nrows, int B, const void* xdf, const void* x64, void* y,
                                cudaStream_t s) {
  if (nrows == 0) return cudaSuccess;
  if (B < 1 || 3 * B > kMixDfThreads || B > kMixThreads - kMixDfThreads) return cudaErrorInvalidValue;
  const size_t smem = (size_t)2 * B * (kMixDfCols * sizeof(float2) + (kMixCols - kMixDfCols) * sizeof(double));
  cudaError_t e = smem_limit(k_bsr_near_mix, smem);
  if (e != cudaSuccess) return e;
  k_bsr_near_mix<<<nrows, kMixThreads, smem, s>>>(row_ptr, col, static_cast<const float2*>(pairs),
                                                  static_cast<const double*>(blocks64), bstride, B,
                                                  static_cast<const float2*>(xdf), static_cast<const double*>(x64),
                                                  static_cast<double*>(y));
  return cudaGetLastError();
}

cudaError_t launch_bsr_df(const int* row_ptr, const int* col, const void* blocks, long bstride, int nrows, int B,
                          const void* x, void* y, int nrhs, int accumulate, cudaStream_t s) {
  return launch_bsr_df_cols(row_ptr, col, blocks, bstride, nrows, B, x, y, nrhs, nrhs, 0, accumulate, s);
}
cudaError_t launch_bsr_df_cols(const int* row_ptr, const int* col, const void* blocks, long bstride, int nrows, int B,
                               const void* x, void* y, int nrhs, int ldy, int y0, int accumulate, cudaStream_t s) {
  if (nrows == 0) return cudaSuccess;
  if (y0 < 0 || y0 + nrhs > ldy) return cudaErrorInvalidValue;
  int ncol = nrhs <= 1 ? 1 : (nrhs <= 2 ? 2 : (nrhs <= 4 ? 4 : 8));
  int groups = (nrhs + ncol - 1) / ncol;
  while (B * groups > 352) {
    ncol *= 2;
    groups = (nrhs + ncol - 1) / ncol;
  }
  if (ncol > 32) return cudaErrorInvalidValue;
  const int threads = ((B * groups + 31) / 32) * 32;
  const size_t smem = (size_t)2 * B * nrhs * sizeof(float2);
  if (smem > 227 * 1024) return cudaErrorInvalidValue;
  const bool full = nrhs % ncol == 0;
  const float2* bl = static_cast<const float2*>(blocks);
  const float2* xx = static_cast<const float2*>(x);
  double* yy = static_cast<double*>(y);
#define BG_DF(NC, FU)                                                                                       \
  if (ncol == NC && full == FU) {                                                                           \
    auto kf = k_bsr_df<NC, FU>;                                                                             \
    cudaError_t e = smem_limit(kf, smem);       \
    if (e != cudaSuccess) return e;                                                                         \
    kf<<<nrows, threads, smem, s>>>(row_ptr, col, bl, bstride, B, xx, yy, nrhs, ldy, y0, accumulate);      \
    return cudaGetLastError();                                                                              \
  }
  BG_DF(1, true)
  BG_DF(2, true)
  BG_DF(2, false)
  BG_DF(4, true)
  BG_DF(4, false)
  BG_DF(8, true)
  BG_DF(8, false)
  BG_DF(16, true)
  BG_DF(16, false)
  BG_DF(32, true)
  BG_DF(32, false)
#undef BG_DF
  return cudaErrorInvalidValue;
}

__global__ void k_split_df(const double* __restrict__ in, long n, float2* __restrict__ out) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const double v = in[t];
  const float h = (float)v;
  out[t] = make_float2(h, (float)(v - (double)h));
}
// complex columns c0 .. c0 + nc - 1 of rows of ld complex entries, times 1 or
// times i, as interleaved (re, im) double-float pairs: out[(r nc + c) 2 + {0, 1}]
__global__ void k_split_df_cols(const double2* __restrict__ in, long rows, int ld, int c0, int nc, int times_i,
                                float2* __restrict__ out) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= rows * nc) return;
  const long r = t / nc;
  const int c = (int)(t % nc);
  const double2 v = in[r * ld + c0 + c];
  const double re = times_i ? -v.y : v.x, im = times_i ? v.x : v.y;
  const float hr = (float)re, hi = (float)im;
  out[2 * t] = make_float2(hr, (float)(re - (double)hr));
  out[2 * t + 1] = make_float2(hi, (float)(im - (double)hi));
}
cudaError_t launch_split_df_cols(const void* in, long rows, int ld, int c0, int nc, int times_i, void* out,
                                 cudaStream_t s) {
  const long n = rows * nc;
  if (n == 0) return cudaSuccess;
  if (c0 < 0 || nc < 1 || c0 + nc > ld) return cudaErrorInvalidValue;
  k_split_df_cols<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(static_cast<const double2*>(in), rows, ld, c0, nc,
                                                                times_i, static_cast<float2*>(out));
  return cudaGetLastError();
}
// complex FP64 blocks -> double-float pairs of the real parts (out) and of the
// imaginary parts (out + nblocks * sout); sout pairs between blocks
__global__ void k_split_df_cplx_blocks(const double2* __restrict__ in, long sin, long B2, long nblocks, long sout,
                                       float2* __restrict__ out) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nblocks * B2) return;
  const long b = t / B2, e = t % B2;
  const double2 v = in[b * sin + e];
  const float hr = (float)v.x, hi = (float)v.y;
  out[b * sout + e] = make_float2(hr, (float)(v.x - (double)hr));
  out[(nblocks + b) * sout + e] = make_float2(hi, (float)(v.y - (double)hi));
}
cudaError_t launch_split_df_cplx_blocks(const void* in, long sin, long B2, long nblocks, long sout, void* out,
                                        cudaStream_t s) {
  const long n = nblocks * B2;
  if (n == 0) return cudaSuccess;
  k_split_df_cplx_blocks<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(static_cast<const double2*>(in), sin, B2,
                                                                       nblocks, sout, static_cast<float2*>(out));
  return cudaGetLastError();
}
cudaError_t launch_split_df(const void* in, long n, void* out, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  k_split_df<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(static_cast<const double*>(in), n,
                                                           static_cast<float2*>(out));
  return cudaGetLastError();
}

// FP32 block-sparse product with register tiles: thread t owns rows
// 4 (t / (nrhs/4)) .. +3 and right-hand sides 4 (t % (nrhs/4)) .. +3, so every
// block column costs two 16-byte shared loads for 16 FMAs. Blocks and x panels
// are staged with cp.async, double-buffered. Needs B % 4 == 0, nrhs % 4 == 0
// and a 16-byte block stride.
__global__ void __launch_bounds__(128) k_bsr32_tile(const int* __restrict__ row_ptr, const int* __restrict__ col,
                                                    const float* __restrict__ blocks, long bstride, int B,
                                                    const float* __restrict__ x, float* __restrict__ y, int nrhs,
                                                    int accumulate) {
  extern __shared__ __align__(16) float sm32[];
  const int fsz = B * B, xsz = B * nrhs;
  float* st[2] = {sm32, sm32 + fsz + xsz};
  const int row = blockIdx.x, t = threadIdx.x;
  const int cq = nrhs >> 2;
  const int i0 = 4 * (t / cq), c0 = 4 * (t % cq);
  const bool active = t < (B >> 2) * cq;
  float acc[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[r][c] = 0.0f;
  const int kb = row_ptr[row], ke = row_ptr[row + 1];
  auto issue = [&](int k, float* dst) {
    const float* F = blocks + (long)k * bstride;
    for (int e = 4 * t; e < fsz; e += 4 * blockDim.x) cp_async16(dst + e, F + e);
    const float* xs = x + (long)col[k] * xsz;
    for (int e = 4 * t; e < xsz; e += 4 * blockDim.x) cp_async16(dst + fsz + e, xs + e);
    cp_async_commit();
  };
  if (kb < ke) issue(kb, st[0]);
  for (int k = kb; k < ke; ++k) {
    const int sb = (k - kb) & 1;
    cp_async_wait<0>();
    __syncthreads();  // block k staged; everyone is done with block k-1
    if (k + 1 < ke) issue(k + 1, st[sb ^ 1]);
    if (active) {
      const float* F = st[sb];
      const float* xs = st[sb] + fsz;
#pragma unroll 4
      for (int j = 0; j < B; ++j) {
        const float4 f = *reinterpret_cast<const float4*>(F + j * B + i0);
        const float4 v = *reinterpret_cast<const float4*>(xs + j * nrhs + c0);
        const float fr[4] = {f.x, f.y, f.z, f.w}, xv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
          for (int c = 0; c < 4; ++c) acc[r][c] = fmaf(fr[r], xv[c], acc[r][c]);
      }
    }
  }
  if (active) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      float* yo = y + ((long)row * B + i0 + r) * nrhs + c0;
#pragma unroll
      for (int c = 0; c < 4; ++c) yo[c] = accumulate ? yo[c] + acc[r][c] : acc[r][c];
    }
  }
}

// Complex FP32 block-sparse product with register tiles: thread t owns RT rows
// and 2 complex right-hand sides (columns 2 (t % (nrhs/2)) ..), so a block
// column costs RT/2 + 1 16-byte shared loads for 2 RT complex multiply-adds.
// Blocks and x panels staged with cp.async, double-buffered, as k_bsr32_tile.
template <int RT>
__global__ void __launch_bounds__(256) k_bsr32c_tile(const int* __restrict__ row_ptr, const int* __restrict__ col,
                                                     const float2* __restrict__ blocks, long bstride, int B,
                                                     const float2* __restrict__ x, float2* __restrict__ y, int nrhs,
                                                     int accumulate) {
  extern __shared__ __align__(16) float2 smc[];
  const int fsz = B * B, xsz = B * nrhs;
  float2* st[2] = {smc, smc + fsz + xsz};
  const int row = blockIdx.x, t = threadIdx.x;
  const int cq = nrhs >> 1;
  const int i0 = RT * (t / cq), c0 = 2 * (t % cq);
  const bool active = t < (B / RT) * cq;
  float2 acc[RT][2];
#pragma unroll
  for (int r = 0; r < RT; ++r) acc[r][0] = acc[r][1] = make_float2(0.0f, 0.0f);
  const int kb = row_ptr[row], ke = row_ptr[row + 1];
  auto issue = [&](int k, float2* dst) {
    const float2* F = blocks + (long)k * bstride;
    for (int e = 2 * t; e < fsz; e += 2 * blockDim.x) cp_async16(dst + e, F + e);
    const float2* xs = x + (long)col[k] * xsz;
    for (int e = 2 * t; e < xsz; e += 2 * blockDim.x) cp_async16(dst + fsz + e, xs + e);
    cp_async_commit();
  };
  if (kb < ke) issue(kb, st[0]);
  for (int k = kb; k < ke; ++k) {
    const int sb = (k - kb) & 1;
    cp_async_wait<0>();
    __syncthreads();  // block k staged; everyone is done with block k-1
    if (k + 1 < ke) issue(k + 1, st[sb ^ 1]);
    if (active) {
      const float2* F = st[sb];
      const float2* xs = st[sb] + fsz;
#pragma unroll 4
      for (int j = 0; j < B; ++j) {
        float2 f[RT];
#pragma unroll
        for (int h = 0; h < RT / 2; ++h) {
          const float4 q = *reinterpret_cast<const float4*>(F + j * B + i0 + 2 * h);
          f[2 * h] = make_float2(q.x, q.y);
          f[2 * h + 1] = make_float2(q.z, q.w);
        }
        const float4 v = *reinterpret_cast<const float4*>(xs + j * nrhs + c0);
        const float2 xv[2] = {make_float2(v.x, v.y), make_float2(v.z, v.w)};
#pragma unroll
        for (int r = 0; r < RT; ++r)
#pragma unroll
          for (int c = 0; c < 2; ++c) {
            acc[r][c].x = fmaf(f[r].x, xv[c].x, fmaf(-f[r].y, xv[c].y, acc[r][c].x));
            acc[r][c].y = fmaf(f[r].x, xv[c].y, fmaf(f[r].y, xv[c].x, acc[r][c].y));
          }
      }
    }
  }
  if (active) {
#pragma unroll
    for (int r = 0; r < RT; ++r) {
      float2* yo = y + ((long)row * B + i0 + r) * nrhs + c0;
#pragma unroll
      for (int c = 0; c < 2; ++c)
        yo[c] = accumulate ? make_float2(yo[c].x + acc[r][c].x, yo[c].y + acc[r][c].y) : acc[r][c];
    }
  }
}

cudaError_t launch_bsr_fp32(bool cplx, const int* row_ptr, const int* col, const void* blocks, long bstride, int nrows,
                            int B, const void* x, void* y, int nrhs, int accumulate, cudaStream_t s, int variant) {
  if (variant != 1 && cplx && nrows > 0 && B % 2 == 0 && nrhs % 2 == 0 && bstride % 2 == 0 &&
      (reinterpret_cast<uintptr_t>(blocks) % 16) == 0 && (reinterpret_cast<uintptr_t>(x) % 16) == 0) {
    int rt = (B % 4 == 0 && (B / 4) * (nrhs / 2) >= 64) ? 4 : 2;
    if (variant == 2) rt = 2;
    if (variant == 3 && B % 4 == 0) rt = 4;
    const int nthr = (B / rt) * (nrhs / 2);
    const size_t smem = (size_t)2 * (B * B + B * nrhs) * sizeof(float2);
    if (nthr <= 256 && smem <= 100 * 1024) {
      const int threads = (nthr + 31) / 32 * 32;
      auto kf = rt == 4 ? k_bsr32c_tile<4> : k_bsr32c_tile<2>;
      cudaError_t e = smem_limit(kf, smem);
      if (e != cudaSuccess) return e;
      kf<<<nrows, threads, smem, s>>>(row_ptr, col, static_cast<const float2*>(blocks), bstride, B,
                                      static_cast<const float2*>(x), static_cast<float2*>(y), nrhs, accumulate);
      return cudaGetLastError();
    }
  }
  if (variant != 1 && !cplx && nrows > 0 && B % 4 == 0 && nrhs % 4 == 0 && bstride % 4 == 0 &&
      (B / 4) * (nrhs / 4) <= 128) {
    const size_t smem = (size_t)2 * (B * B + B * nrhs) * sizeof(float);
    if (smem <= 100 * 1024) {
      const int threads = (((B / 4) * (nrhs / 4)) + 31) / 32 * 32;
      cudaError_t e = smem_limit(k_bsr32_tile, smem);
      if (e != cudaSuccess) return e;
      k_bsr32_tile<<<nrows, threads, smem, s>>>(row_ptr, col, static_cast<const float*>(blocks), bstride, B,
                                                static_cast<const float*>(x), static_cast<float*>(y), nrhs, accumulate);
      return cudaGetLastError();
    }
  }
  if (cplx)
    return bsr_pipe_typed<cf>(row_ptr, col, (const cf*)blocks, bstride, nrows, B, (const cf*)x, (cf*)y, nrhs, accumulate, s);
  return bsr_pipe_typed<float>(row_ptr, col, (const float*)blocks, bstride, nrows, B, (const float*)x, (float*)y,
                               nrhs, accumulate, s);
}

// FP32 copy of FP64 blocks with a different block stride (in scalars)
template <typename S64, typename S32>
__global__ void k_convert_blocks(const S64* __restrict__ in, long sin, S32* __restrict__ out, long sout, long B2,
                                 long nblocks) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nblocks * B2) return;
  const long b = t / B2, e = t % B2;
  out[b * sout + e] = Conv<S64, S32>::run(in[b * sin + e]);
}
cudaError_t launch_convert_blocks(bool cplx, const void* in, long sin, void* out, long sout, long B2, long nblocks,
                                  cudaStream_t s) {
  const long n = nblocks * B2;
  if (n == 0) return cudaSuccess;
  const unsigned g = (unsigned)((n + 255) / 256);
  if (cplx) k_convert_blocks<cd, cf><<<g, 256, 0, s>>>((const cd*)in, sin, (cf*)out, sout, B2, nblocks);
  else k_convert_blocks<double, float><<<g, 256, 0, s>>>((const double*)in, sin, (float*)out, sout, B2, nblocks);
  return cudaGetLastError();
}

cudaError_t launch_moment_fwd_acc(int S, bool acc, const void* mom, int R, int Bq, int ncl, const void* xss, void* y,
                                  int nrhs, cudaStream_t s) {
  const int kk = (S & 1) ? 2 * nrhs : nrhs;
  if (S < 2) return bgemm<double>(false, acc, (const double*)mom, R, Bq, (const double*)xss, (long)Bq * kk, (double*)y,
                                  (long)R * kk, ncl, kk, s);
  return bgemm<float>(false, acc, (const float*)mom, R, Bq, (const float*)xss, (long)Bq * kk, (float*)y, (long)R * kk,
                      ncl, kk, s);
}
cudaError_t launch_moment_fwd(int S, const void* mom, int R, int Bq, int ncl, const void* xss, void* y, int nrhs,
                              cudaStream_t s) {
  // Y[c] (R x k) = Mom (R x Bq) X[c] (Bq x k); complex vectors as 2k real columns
  const int kk = (S & 1) ? 2 * nrhs : nrhs;
  if (S < 2) return bgemm<double>(false, false, (const double*)mom, R, Bq, (const double*)xss, (long)Bq * kk, (double*)y,
                                  (long)R * kk, ncl, kk, s);
  return bgemm<float>(false, false, (const float*)mom, R, Bq, (const float*)xss, (long)Bq * kk, (float*)y, (long)R * kk,
                      ncl, kk, s);
}
cudaError_t launch_moment_bwd(int S, const void* mom, int R, int Bq, int ncl, const void* z, void* yss, int nrhs,
                              cudaStream_t s) {
  // Yss[c] (Bq x k) += Mom^T (Bq x R) Z[c] (R x k)
  const int kk = (S & 1) ? 2 * nrhs : nrhs;
  if (S < 2) return bgemm<double>(true, true, (const double*)mom, Bq, R, (const double*)z, (long)R * kk, (double*)yss,
                                  (long)Bq * kk, ncl, kk, s);
  return bgemm<float>(true, true, (const float*)mom, Bq, R, (const float*)z, (long)R * kk, (float*)yss, (long)Bq * kk,
                      ncl, kk, s);
}
cudaError_t launch_transfer_fwd(int S, const void* T, int np2, int nc, int np_, const void* yc, void* yp, int nrhs,
                                cudaStream_t s) {
  if (np_ == 0) return cudaSuccess;
  if (nc == 1) {
    // parent p (np2 x k) = T (np2 x 4np2) [children 4p..4p+3 stacked] (4np2 x k)
    const int kk = (S & 1) ? 2 * nrhs : nrhs;
    if (S < 2)
      return bgemm<double>(false, false, (const double*)T, np2, 4 * np2, (const double*)yc, 4L * np2 * kk, (double*)yp,
                           (long)np2 * kk, np_, kk, s);
    return bgemm<float>(false, false, (const float*)T, np2, 4 * np2, (const float*)yc, 4L * np2 * kk, (float*)yp,
                        (long)np2 * kk, np_, kk, s);
  }
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
  if (nc == 1) {
    // children 4p..4p+3 stacked (4np2 x k) += T^T (4np2 x np2) parent p (np2 x k)
    const int kk = (S & 1) ? 2 * nrhs : nrhs;
    if (S < 2)
      return bgemm<double>(true, true, (const double*)T, 4 * np2, np2, (const double*)zp, (long)np2 * kk, (double*)zc,
                           4L * np2 * kk, np_, kk, s);
    return bgemm<float>(true, true, (const float*)T, 4 * np2, np2, (const float*)zp, (long)np2 * kk, (float*)zc,
                        4L * np2 * kk, np_, kk, s);
  }
  switch (S) {
    case 0: k_transfer_bwd<double><<<np_, 256, 0, s>>>((const double*)T, np2, nc, (const double*)zp, (double*)zc, nrhs); break;
    case 1: k_transfer_bwd<cd><<<np_, 256, 0, s>>>((const double*)T, np2, nc, (const cd*)zp, (cd*)zc, nrhs); break;
    case 2: k_transfer_bwd<float><<<np_, 256, 0, s>>>((const float*)T, np2, nc, (const float*)zp, (float*)zc, nrhs); break;
    case 3: k_transfer_bwd<cf><<<np_, 256, 0, s>>>((const float*)T, np2, nc, (const cf*)zp, (cf*)zc, nrhs); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <bool CPLX, int NP2>
static cudaError_t far_fused_t(const float4* pts, const d4* centres, const int* row_ptr, const int* col, int nrows,
                               float kre, float kim, const void* y, void* z, int nrhs, cudaStream_t s) {
  const size_t smem = (size_t)NP2 * NP2 * (CPLX ? sizeof(float2) : sizeof(float));
#define BG_FF(NCV)                                                                                          \
  {                                                                                                         \
    auto kf = k_far_fused<CPLX, NP2, NCV>;                                                                  \
    cudaError_t e = smem_limit(kf, smem);       \
    if (e != cudaSuccess) return e;                                                                         \
    kf<<<nrows, 128, smem, s>>>(pts, centres, row_ptr, col, kre, kim, y, z, nrhs);                          \
    return cudaGetLastError();                                                                              \
  }
  if (nrhs <= 4) BG_FF(1)
  if (nrhs <= 8) BG_FF(2)
  if (nrhs <= 16) BG_FF(4)
  if (nrhs <= 32) BG_FF(8)
#undef BG_FF
  return cudaErrorInvalidValue;
}
cudaError_t launch_far_fused(bool cplx, const float4* pts, const d4* centres, const int* row_ptr, const int* col,
                             int nrows, int np2, float kre, float kim, const void* y, void* z, int nrhs, cudaStream_t s) {
  if (nrows == 0) return cudaSuccess;
#define BG_FR(N2)                                                                                    \
  case N2:                                                                                           \
    return cplx ? far_fused_t<true, N2>(pts, centres, row_ptr, col, nrows, kre, kim, y, z, nrhs, s)  \
                : far_fused_t<false, N2>(pts, centres, row_ptr, col, nrows, kre, kim, y, z, nrhs, s);
  switch (np2) {
    BG_FR(16)
    BG_FR(25)
    BG_FR(36)
    BG_FR(49)
    BG_FR(64)
    BG_FR(81)
    BG_FR(100)
    BG_FR(121)
    default: return cudaErrorInvalidValue;
  }
#undef BG_FR
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
cudaError_t launch_add_low(bool cplx, const void* in32, long n, void* out64, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const unsigned g = blocks_for(n, 256);
  if (cplx) k_add_low<cd, cf><<<g, 256, 0, s>>>((const cf*)in32, n, (cd*)out64);
  else k_add_low<double, float><<<g, 256, 0, s>>>((const float*)in32, n, (double*)out64);
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
