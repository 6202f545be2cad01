// FP64-accurate near-field product on the tensor cores (the near field of
// the mixed inner operator, H2DenseProduct.hpp:122-150 for the dense leaves).
//
// GB300's FP64 pipe runs at 1/64 of its FP32 rate, so the FP64 near-field
// product is emulated exactly with integer slices on the FP16 tensor cores
// (Ozaki's error-free splitting, fixed-point variant):
//  - every row i of a block row of the near field gets an exponent e_i with
//    |A_ij| <= 2^(e_i - 1) over the whole block row; every right-hand-side
//    column c an exponent f_c with |x_jc| <= 2^(f_c - 1) over all rows;
//  - A_ij = 2^e_i sum_s a_s 2^(-7 (s + 1)), x_jc = 2^f_c sum_t x_t 2^(-7 (t + 1)),
//    s, t = 0 .. 7, with integer digits |a_s|, |x_t| <= 64 (56 bits; FP16
//    holds them exactly);
//  - y_ic = 2^(e_i + f_c - 14) sum_d 2^(-7 d) acc_d with acc_d = sum_j
//    sum_{s + t = d} a_s x_t for d = 0 .. 7 (the dropped d >= 8 terms are
//    below 2^-53 of sum_j |A_ij| |x_jc|). Every product is at most 2^12 and a
//    diagonal holds at most 8 of them per j, so acc_d stays an exact integer
//    in FP32 (below 2^24) over up to 512 / B blocks: the tensor cores' FP32
//    accumulation is exact here, whatever its rounding;
//  - the epilogue turns each acc_d into a 64-bit fixed-point integer (unit
//    2^-34 of the leading digit product), sums them over diagonals and
//    chunks of blocks, and converts once to FP64 with the two exponents.
// The result is the FP64 product to about 1e-16 relative to sum_j |A_ij| |x_jc|.
//
// MMA shape (tcgen05.mma kind::f16, cta_group::1, M = 128, N = B padded to
// 16, K = B padded to 16): the x digits form the A operand, rows (t, c) in
// blocks of 32 columns per digit t, stacked as [0, 0, 0, x_0, .., x_7]; the
// coupling digits a_s are the B operand (N = rows i of the block, K = j).
// For digit s the A operand starts at the row block of x_{4 g - s}, so that
// tensor-memory accumulator g (g = 0, 1) gets sum_t a_s x_t in its row block
// d - 4 g for every diagonal d = s + t in [4 g, 4 g + 4); row blocks with
// t < 0 read the zero blocks. 12 MMA chains of K steps per block.
//
// Roles per CTA (persistent, one per SM): warp 0 lane 0 moves each block's
// 8 coupling digit tiles and its column cluster's 8 x digit tiles with 1-D
// TMA bulk copies into 3 shared-memory stages; warp 1 lane 0 issues the
// MMAs into one of two tensor-memory buffers per chunk of blocks; warps 2-5
// (tensor-memory lane quadrant d mod 4) fold each chunk into per-row 64-bit
// sums and, at the end of a block row, reduce the four quadrants in shared
// memory and write y in FP64. Every wait is bounded; on timeout the kernel
// records an error code in err and returns.
#include <cuda_fp16.h>

#include <algorithm>
#include <climits>
#include <cstdint>

#include "bg_kernels.cuh"
#include "bg_tcgen05.cuh"

namespace bg {

namespace {

using namespace tc;

constexpr int kOzDigits = 8;      // digits per operand, 7 bits each
constexpr int kOzCols = 32;       // right-hand sides per pass
constexpr int kOzZero = 3;        // zero row blocks before x_0 in the A operand
constexpr int kOzStages = 3;
constexpr int kOzThreads = 192;   // producer, MMA issuer, 4 epilogue warps
constexpr uint32_t kOzTmemCols = 256;
constexpr int kOzUnit = 34;       // fixed point: acc_0 << 34

template <int B>
struct OzShape {
  static constexpr int KP = (B + 15) / 16 * 16;  // MMA K; x tiles store all of it (zero beyond B)
  static constexpr int KA = (B + 7) / 8 * 8;     // K stored in the coupling tiles
  static constexpr int NA = (B + 7) / 8 * 8;     // rows stored in the coupling tiles
  static constexpr int NM = (B + 15) / 16 * 16;  // MMA N
  static constexpr uint32_t SBO_A = KA / 8 * 128;
  static constexpr uint32_t SLICE_A = NA / 8 * SBO_A;
  static constexpr uint32_t BLOCK_A = kOzDigits * SLICE_A;
  static constexpr uint32_t SBO_X = KP / 8 * 128;
  static constexpr uint32_t XBLK = 4 * SBO_X;  // 32 rows (one digit, 32 columns)
  static constexpr uint32_t PANEL_X = kOzDigits * XBLK;
  static constexpr uint32_t ZERO_X = kOzZero * XBLK;
  static constexpr uint32_t STAGE = BLOCK_A + ZERO_X + PANEL_X;  // [coupling digits][zeros][x digits]
  static constexpr uint32_t COPY = BLOCK_A + PANEL_X;
  static constexpr int CHUNK = (1 << 24) / (kOzDigits * 4096 * B);  // blocks per exact accumulation
  static constexpr uint32_t RED = 4u * B * kOzCols * 8u;
  static constexpr uint32_t SMEM = kOzStages * STAGE + RED;
  // the B operand of the last digit reads NM rows and KP columns from its
  // start: at most into the zero blocks that follow the coupling tiles
  static constexpr uint32_t B_READ = (kOzDigits - 1) * SLICE_A + (NM / 8) * SBO_A + (KP - KA) / 8 * 128;
  static_assert(B_READ <= BLOCK_A + ZERO_X, "coupling tiles: over-read leaves the stage");
  static_assert(NM <= 64, "two accumulators of N columns per 128-column buffer");
  static_assert(CHUNK >= 1, "block too large for exact FP32 accumulation");
  static_assert(BLOCK_A % 16 == 0 && PANEL_X % 16 == 0 && STAGE % 16 == 0, "bulk copies need 16-byte sizes");
};

// 8 signed base-128 digits of round(|v| 2^(56 - f)) (|v| <= 2^(f - 1)): the
// top digit in [0, 64], the others in [-64, 63], then the sign of v. Integer
// arithmetic only (the FP64 pipe is the slow one).
__device__ __forceinline__ void oz_digits(double v, int f, int* d) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
  const int be = (int)((bits >> 52) & 0x7FF);
  const unsigned long long mant = bits & ((1ull << 52) - 1);
  unsigned long long m = be ? (mant | (1ull << 52)) : mant;
  const int sh = (be ? be - 1075 : -1074) - f + 56;  // |v| 2^(56 - f) = m 2^sh, sh <= 2
  unsigned long long V;
  if (m == 0) V = 0;
  else if (sh >= 0) V = m << sh;
  else if (sh > -63) V = (m + (1ull << (-sh - 1))) >> (-sh);
  else V = 0;
  int carry = 0;
#pragma unroll
  for (int k = kOzDigits - 1; k >= 1; --k) {
    int dk = (int)((V >> (7 * (kOzDigits - 1 - k))) & 127) + carry;
    carry = dk >= 64;
    d[k] = carry ? dk - 128 : dk;
  }
  d[0] = (int)(V >> (7 * (kOzDigits - 1))) + carry;
  if (bits >> 63) {
#pragma unroll
    for (int k = 0; k < kOzDigits; ++k) d[k] = -d[k];
  }
}

// v 2^k as FP64 for a 64-bit integer v (round to nearest even); integer
// arithmetic except outside the normal range
__device__ __forceinline__ double oz_to_double(long long v, int k) {
  if (v == 0) return 0.0;
  const unsigned long long sgn = v < 0 ? (1ull << 63) : 0ull;
  const unsigned long long a = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
  int top = 63 - __clzll((long long)a);
  unsigned long long m;
  if (top > 52) {
    const int sh = top - 52;
    const unsigned long long rem = a & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    m = a >> sh;
    if (rem > half || (rem == half && (m & 1))) {
      ++m;
      if (m == (1ull << 53)) {
        m >>= 1;
        ++top;
      }
    }
  } else {
    m = a << (52 - top);
  }
  const int ex = top + k + 1023;
  if (ex <= 0 || ex >= 2047) return ldexp((double)v, k);
  return __longlong_as_double((long long)(sgn | ((unsigned long long)ex << 52) | (m & ((1ull << 52) - 1))));
}

__device__ __forceinline__ long long oz_fix(float acc, int sh) {
  const long long v = (long long)__float2int_rn(acc);  // an exact integer below 2^24
  return sh >= 0 ? v * (1ll << sh) : ((v + (1ll << (-sh - 1))) >> (-sh));
}

__device__ __forceinline__ void epi_sync() { asm volatile("bar.sync 1, 128;\n" ::: "memory"); }

// one byte offset of element (row, k) in a K-major core-matrix tile
__device__ __forceinline__ uint32_t kmajor_off(int row, int k, uint32_t sbo) {
  return (uint32_t)(row >> 3) * sbo + (uint32_t)(k >> 3) * 128u + (uint32_t)(row & 7) * 16u + (uint32_t)(k & 7) * 2u;
}

}  // namespace

// Row exponents: e[r B + i] = (largest biased exponent over row i of block
// row r) - 1021, so that |A_ij| <= 2^(e - 1). One CTA per block row.
__global__ void k_oz_row_exp(const int* __restrict__ row_ptr, const double* __restrict__ blocks, long bstride, int B,
                             int* __restrict__ e) {
  extern __shared__ int emax[];
  const int r = blockIdx.x;
  for (int i = threadIdx.x; i < B; i += blockDim.x) emax[i] = 0;
  __syncthreads();
  const int kb = row_ptr[r], ke = row_ptr[r + 1];
  for (int k = kb; k < ke; ++k) {
    const double* F = blocks + (long)k * bstride;
    for (int q = threadIdx.x; q < B * B; q += blockDim.x) {  // column-major: q = i + j B
      const int be = (int)(((unsigned long long)__double_as_longlong(F[q]) >> 52) & 0x7FF);
      atomicMax(&emax[q % B], be);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < B; i += blockDim.x) e[(long)r * B + i] = emax[i] - 1021;
}

// Coupling digit tiles: block k of block row r, digit s, entry (i, j) at
// k BLOCK_A + s SLICE_A + kmajor_off(i, j, SBO_A). Padding stays as zeroed.
template <int B>
__global__ void k_oz_build(const int* __restrict__ row_ptr, const double* __restrict__ blocks, long bstride,
                           const int* __restrict__ e, __half* __restrict__ tiles) {
  using G = OzShape<B>;
  const int r = blockIdx.x;
  const int kb = row_ptr[r], ke = row_ptr[r + 1];
  for (int k = kb; k < ke; ++k) {
    const double* F = blocks + (long)k * bstride;
    unsigned char* base = reinterpret_cast<unsigned char*>(tiles) + (size_t)k * G::BLOCK_A;
    for (int q = threadIdx.x; q < B * B; q += blockDim.x) {
      const int i = q % B, j = q / B;
      int d[kOzDigits];
      oz_digits(F[q], e[(long)r * B + i], d);
      const uint32_t off = kmajor_off(i, j, G::SBO_A);
#pragma unroll
      for (int s = 0; s < kOzDigits; ++s)
        *reinterpret_cast<__half*>(base + s * G::SLICE_A + off) = __int2half_rn(d[s]);
    }
  }
}

// Column exponents of x (rows x ld, columns c0 .. c0 + nc - 1): fmax[c] =
// the largest biased exponent (fmax zeroed before)
__global__ void k_oz_col_exp(const double* __restrict__ x, long rows, int ld, int c0, int nc, int* __restrict__ fmax) {
  __shared__ int red[kOzCols];
  const int c = threadIdx.x & 31;
  if (threadIdx.x < kOzCols) red[threadIdx.x] = 0;
  __syncthreads();
  int mx = 0;
  if (c < nc) {
    for (long r = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < rows;
         r += (long)gridDim.x * (blockDim.x >> 5)) {
      const int be = (int)(((unsigned long long)__double_as_longlong(x[r * ld + c0 + c]) >> 52) & 0x7FF);
      mx = max(mx, be);
    }
  }
  atomicMax(&red[c], mx);
  __syncthreads();
  if (threadIdx.x < kOzCols) atomicMax(&fmax[threadIdx.x], red[threadIdx.x]);
}

// x digit tiles: cluster J = row / B, local row j = row % B, digit t, column
// c at J PANEL_X + t XBLK + kmajor_off(c, j, SBO_X); columns >= nc and rows
// j >= B of a cluster get zeros. A thread takes 8 consecutive rows of one
// column (one 16-byte core-matrix row per digit), so a warp's stores are
// whole 128-byte core matrices and its loads whole rows of x.
template <int B>
__global__ void k_oz_split_x(const double* __restrict__ x, long rows, int ld, int c0, int nc,
                             const int* __restrict__ fmax, __half* __restrict__ panels) {
  using G = OzShape<B>;
  constexpr int NG = (B + 7) / 8;  // groups of 8 rows holding the cluster's rows
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long ncl = rows / B;
  if (t >= ncl * NG * kOzCols) return;
  const int c = (int)(t & 31);
  const long q = t >> 5;
  const long J = q / NG;
  const int g = (int)(q - J * NG);
  const int f = fmax[c] - 1021;
  uint32_t w[kOzDigits][4];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int j = g * 8 + i;
    const double v = (j < B && c < nc) ? x[(J * B + j) * ld + c0 + c] : 0.0;
    int d[kOzDigits];
    oz_digits(v, f, d);
#pragma unroll
    for (int s = 0; s < kOzDigits; ++s) {
      const uint32_t h = (uint32_t)__half_as_ushort(__int2half_rn(d[s]));
      if (i & 1) w[s][i >> 1] |= h << 16;
      else w[s][i >> 1] = h;
    }
  }
  unsigned char* base = reinterpret_cast<unsigned char*>(panels) + (size_t)J * G::PANEL_X + kmajor_off(c, g * 8, G::SBO_X);
#pragma unroll
  for (int s = 0; s < kOzDigits; ++s)
    *reinterpret_cast<uint4*>(base + s * G::XBLK) = make_uint4(w[s][0], w[s][1], w[s][2], w[s][3]);
}

template <int B>
__global__ void __launch_bounds__(kOzThreads, 1)
    k_near_oz(const int* __restrict__ row_ptr, const int* __restrict__ col, int nrows,
              const unsigned char* __restrict__ atiles, const unsigned char* __restrict__ xpanels,
              const int* __restrict__ rexp, const int* __restrict__ fmax, double* __restrict__ y, int ldy, int y0,
              int nc, int* __restrict__ err) {
  using G = OzShape<B>;
  constexpr int S = kOzStages;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t full_bar[S], done_bar[S], acc_full[2], acc_free[2], fin_bar;
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag, ep_stop;
  volatile int* abort_v = &abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  long long* red = reinterpret_cast<long long*>(smem + S * G::STAGE);

  // the zero row blocks of every stage (generic-proxy writes, made visible
  // to the tensor cores by the proxy fence)
  for (int st = 0; st < S; ++st) {
    uint4* z = reinterpret_cast<uint4*>(smem + st * G::STAGE + G::BLOCK_A);
    for (uint32_t q = tid; q < G::ZERO_X / 16; q += kOzThreads) z[q] = make_uint4(0, 0, 0, 0);
  }
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_slot)),
                 "r"(kOzTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  if (tid == 0) {
    for (int b = 0; b < S; ++b) {
      mbar_init(&full_bar[b], 1);
      mbar_init(&done_bar[b], 1);
    }
    mbar_init(&acc_full[0], 1);
    mbar_init(&acc_full[1], 1);
    mbar_init(&acc_free[0], 4);
    mbar_init(&acc_free[1], 4);
    mbar_init(&fin_bar, 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_slot;

  if (warp == 0) {
    // ---- producer ----
    if (lane == 0) {
      int it = 0;
      for (int r = blockIdx.x; r < nrows && !*abort_v; r += gridDim.x) {
        const int kb = row_ptr[r], ke = row_ptr[r + 1];
        for (int k = kb; k < ke; ++k, ++it) {
          const int st = it % S;
          if (it >= S && !mbar_wait(&done_bar[st], (uint32_t)((it / S - 1) & 1))) {
            *abort_v = 1;
            atomicExch(err, 11);
            break;
          }
          if (*abort_v) break;
          unsigned char* sm = smem + st * G::STAGE;
          mbar_expect_tx(&full_bar[st], G::COPY);
          bulk_g2s(sm, atiles + (size_t)k * G::BLOCK_A, G::BLOCK_A, &full_bar[st]);
          bulk_g2s(sm + G::BLOCK_A + G::ZERO_X, xpanels + (size_t)col[k] * G::PANEL_X, G::PANEL_X, &full_bar[st]);
        }
      }
      // after an abort, the copies still in flight land before the CTA exits
      if (*abort_v)
        for (int j = max(0, it - S); j < it; ++j) mbar_wait(&full_bar[j % S], (uint32_t)((j / S) & 1));
    }
  } else if (warp == 1) {
    // ---- MMA issuer ----
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_f16(128, G::NM);
      const uint32_t base = smem_u32(smem);
      int it = 0, ch = 0;
      bool issued = false;
      for (int r = blockIdx.x; r < nrows && !*abort_v; r += gridDim.x) {
        const int kb = row_ptr[r], ke = row_ptr[r + 1];
        for (int cb = kb; cb < ke && !*abort_v; cb += G::CHUNK, ++ch) {
          const int ce = min(ke, cb + G::CHUNK), buf = ch & 1;
          if (ch >= 2 && !mbar_wait(&acc_free[buf], (uint32_t)(((ch >> 1) - 1) & 1))) {
            *abort_v = 1;
            atomicExch(err, 12);
            break;
          }
          for (int k = cb; k < ce; ++k, ++it) {
            const int st = it % S;
            if (!mbar_wait(&full_bar[st], (uint32_t)((it / S) & 1))) {
              *abort_v = 1;
              atomicExch(err, 13);
              break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t sa = base + st * G::STAGE;               // coupling digits (B operand)
            const uint32_t sx = sa + G::BLOCK_A;                    // zero blocks, then x digits (A operand)
#pragma unroll 1
            for (int s = 0; s < kOzDigits; ++s) {
#pragma unroll
              for (int g = 0; g < 2; ++g) {
                if (g == 0 && s > 3) continue;  // diagonals 0 .. 3 get nothing from digits s > 3
                uint64_t ad = umma_desc(sx + (uint32_t)(kOzZero - s + 4 * g) * G::XBLK, 128, G::SBO_X);
                uint64_t bd = umma_desc(sa + (uint32_t)s * G::SLICE_A, 128, G::SBO_A);
                const uint32_t dd = tmem + (uint32_t)(128 * buf + 64 * g);
#pragma unroll
                for (int ks = 0; ks < G::KP / 16; ++ks) {
                  mma_f16(dd, ad, bd, idesc, (k > cb || s > 0 || ks > 0) ? 1u : 0u);
                  ad += 16;  // next K step: two core matrices = 256 bytes
                  bd += 16;
                }
              }
            }
            issued = true;
            mma_commit(&done_bar[st]);
          }
          if (*abort_v) break;
          mma_commit(&acc_full[buf]);
        }
      }
      if (issued) {
        // every MMA of this CTA complete before the tensor memory is freed
        mma_commit(&fin_bar);
        if (!mbar_wait(&fin_bar, 0)) atomicExch(err, 14);
      }
    }
  } else {
    // ---- epilogue warps 2-5: lane quadrant q = diagonals q and 4 + q ----
    // The four warps meet at named barriers; whether to stop is decided once
    // per block row from a value every one of them reads after the barrier.
    const int q = warp & 3, et = tid - 64;
    const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16);
    const int sh0 = kOzUnit - 7 * q, sh1 = kOzUnit - 7 * (4 + q);
    int ch = 0;
    for (int r = blockIdx.x; r < nrows; r += gridDim.x) {
      if (et == 0) ep_stop = *abort_v;
      epi_sync();
      if (ep_stop) break;
      const int kb = row_ptr[r], ke = row_ptr[r + 1];
      long long P[B];
#pragma unroll
      for (int i = 0; i < B; ++i) P[i] = 0;
      for (int cb = kb; cb < ke; cb += G::CHUNK, ++ch) {
        const int buf = ch & 1;
        int got = 0;
        if (lane == 0 && !*abort_v) got = mbar_wait(&acc_full[buf], (uint32_t)((ch >> 1) & 1)) ? 1 : 0;
        got = __shfl_sync(0xffffffffu, got, 0);
        if (!got) {
          if (lane == 0) {
            *abort_v = 1;
            atomicExch(err, 15);
          }
          continue;  // the row is finished without data; the next one stops
        }
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
#pragma unroll
        for (int g = 0; g < 2; ++g) {
          const uint32_t ta = lane_base + (uint32_t)(128 * buf + 64 * g);
          const int sh = g ? sh1 : sh0;
#pragma unroll
          for (int i0 = 0; i0 < B; i0 += 8) {
            float v[8];
            tmem_ld8(ta + (uint32_t)i0, v);
#pragma unroll
            for (int u = 0; u < 8; ++u)
              if (i0 + u < B) P[i0 + u] += oz_fix(v[u], sh);
          }
        }
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive(&acc_free[buf]);
      }
      // reduce the four quadrants and write y rows r B .. r B + B - 1
#pragma unroll
      for (int i = 0; i < B; ++i) red[(q * B + i) * kOzCols + lane] = P[i];
      epi_sync();
      for (int idx = et; idx < B * kOzCols; idx += 128) {
        const int i = idx >> 5, c = idx & 31;
        if (c < nc) {
          const long long V = red[(0 * B + i) * kOzCols + c] + red[(1 * B + i) * kOzCols + c] +
                              red[(2 * B + i) * kOzCols + c] + red[(3 * B + i) * kOzCols + c];
          const int k2 = rexp[(long)r * B + i] + (fmax[c] - 1021) - 14 - kOzUnit;
          // a column holding Inf or NaN gives NaN, as the FP64 product would
          y[((long)r * B + i) * ldy + y0 + c] = fmax[c] == 2047 ? __longlong_as_double(0x7FF8000000000000ll)
                                                                : oz_to_double(V, k2);
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kOzTmemCols));
}

#define BG_OZ_SIZES(X) X(4) X(16) X(36)

bool oz_supported(int B) {
  switch (B) {
#define BG_C(N) case N:
    BG_OZ_SIZES(BG_C)
#undef BG_C
    return true;
    default: return false;
  }
}

size_t oz_tile_bytes(int B, long nblocks) {
  switch (B) {
#define BG_C(N) \
  case N: return (size_t)nblocks * OzShape<N>::BLOCK_A;
    BG_OZ_SIZES(BG_C)
#undef BG_C
    default: return 0;
  }
}

size_t oz_panel_bytes(int B, long nclusters) {
  switch (B) {
#define BG_C(N) \
  case N: return (size_t)nclusters * OzShape<N>::PANEL_X;
    BG_OZ_SIZES(BG_C)
#undef BG_C
    default: return 0;
  }
}

cudaError_t launch_oz_build(const int* row_ptr, const double* blocks, long bstride, int nrows, int B, int* rexp,
                            void* tiles, long nblocks, cudaStream_t s) {
  if (!oz_supported(B)) return cudaErrorInvalidValue;
  if (nrows == 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(tiles, 0, oz_tile_bytes(B, nblocks), s);
  if (e != cudaSuccess) return e;
  k_oz_row_exp<<<nrows, 256, B * sizeof(int), s>>>(row_ptr, blocks, bstride, B, rexp);
  switch (B) {
#define BG_C(N) \
  case N: k_oz_build<N><<<nrows, 256, 0, s>>>(row_ptr, blocks, bstride, rexp, static_cast<__half*>(tiles)); break;
    BG_OZ_SIZES(BG_C)
#undef BG_C
  }
  return cudaGetLastError();
}

cudaError_t launch_near_oz(const int* row_ptr, const int* col, int nrows, int B, const void* tiles,
                           const int* rexp, const double* x, long xrows, int ldx, void* panels, int* fmax,
                           double* y, int ldy, int nrhs, int* err, cudaStream_t s) {
  if (!oz_supported(B)) return cudaErrorInvalidValue;
  if (nrows == 0 || nrhs == 0) return cudaSuccess;
  int dev = 0, nsm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  for (int c0 = 0; c0 < nrhs; c0 += kOzCols) {
    const int nc = std::min(kOzCols, nrhs - c0);
    e = cudaMemsetAsync(fmax, 0, kOzCols * sizeof(int), s);
    if (e != cudaSuccess) return e;
    k_oz_col_exp<<<2 * nsm, 256, 0, s>>>(x, xrows, ldx, c0, nc, fmax);
    const long nt = (xrows / B) * ((B + 7) / 8) * kOzCols;
    const unsigned blocks = (unsigned)((nt + 255) / 256);
    switch (B) {
#define BG_C(N)                                                                                                 \
  case N: {                                                                                                     \
    using G = OzShape<N>;                                                                                       \
    k_oz_split_x<N><<<blocks, 256, 0, s>>>(x, xrows, ldx, c0, nc, fmax, static_cast<__half*>(panels));          \
    e = smem_limit(k_near_oz<N>, G::SMEM);                                                                      \
    if (e != cudaSuccess) return e;                                                                             \
    k_near_oz<N><<<std::min(nrows, nsm), kOzThreads, G::SMEM, s>>>(                                            \
        row_ptr, col, nrows, static_cast<const unsigned char*>(tiles), static_cast<const unsigned char*>(panels), \
        rexp, fmax, y, ldy, c0, nc, err);                                                                       \
    break;                                                                                                      \
  }
      BG_OZ_SIZES(BG_C)
#undef BG_C
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace bg
