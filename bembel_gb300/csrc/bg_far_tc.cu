// Far-field product on the 5th-generation tensor cores (tcgen05, sm_103a).
//
// For every target cluster row i of every FMM level:
//   Z_i = sum_j F_ij Y_j,  F_ij[m][k] = |J(x_m)| |J(y_k)| / (4 pi |x_m - y_k|)
// (H2Multipole.hpp:336-375 for the couplings, H2DenseProduct.hpp:88-121 for
// the product), with F_ij generated on the fly in FP32 and never stored.
//
// One CTA per (level, row) from a work list sorted by block count, all levels
// in one launch. Warp roles: 16 generator warps and one MMA warp.
//  - Generators write the n_p^2 x n_p^2 coupling tile of each far-field block
//    straight into shared memory in the UMMA K-major no-swizzle core-matrix
//    layout (8 rows x 16 bytes per core matrix, core matrices contiguous along
//    K), split into a TF32 high part and an FP32 remainder; Y_j (staged one
//    block ahead with cp.async) is split the same way. Point arrays are padded
//    with distant zero-weight points, so the padded rows and columns of a tile
//    come out as exact zeros without branches.
//  - The MMA warp issues tcgen05.mma kind::tf32 (M = 128, N = 32, K = 8) for
//    hi*hi and, into a second accumulator, hi*lo + lo*hi, which keeps about 21
//    bits of every product.
//  - The tensor core's FP32 accumulation is not round-to-nearest, so chains
//    are kept short: every block starts fresh tensor-memory accumulators (two
//    buffers alternate) and the generators fold each finished block into
//    per-row register sums with Neumaier compensation (each thread owns 8 of
//    the 32 columns of one row) while later blocks run.
// Two shared-memory stages let the generation of block k+1 overlap the MMAs
// of block k; mbarriers hand stages between the roles (full: all generator
// threads arrive; done: tcgen05.commit). Every wait is bounded: on timeout the
// kernel records an error code, waits (bounded) for its MMAs, frees its tensor
// memory and returns.
#include <cuda_fp16.h>

#include <algorithm>
#include <cstdint>

#include "bg_kernels.cuh"
#include "bg_tcgen05.cuh"

namespace bg {

namespace {

using namespace tc;

constexpr int kGenWarps = 16;                 // warps generating the tiles
constexpr int kGenThreads = 32 * kGenWarps;   // the MMA warp follows them
constexpr int kThreads = kGenThreads + 32;
constexpr int kN = 32;                        // MMA N: right-hand sides per tile
constexpr int kYStride = 40;                  // floats per staged Y_j row (conflict-free reads)
// FP32 accumulators: 2 buffers x {hi*hi, hi*lo + lo*hi} x 32 columns
constexpr uint32_t kTmemCols = 128;
constexpr float kFar = 1.0e18f;                  // padding points: finite r^2 (< 1.2e37), weight 0

// round to the nearest TF32 value (10 explicit mantissa bits), ties away
__device__ __forceinline__ float tf32_hi(float x) {
  return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_u32(smem)), "l"(gmem));
}
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(smem_u32(smem)), "l"(gmem));
}

__device__ __forceinline__ void gen_sync() { asm volatile("bar.sync 1, %0;\n" ::"n"(kGenThreads) : "memory"); }

// 1/sqrt(x) by the hardware approximation (relative error below 2^-22); x is
// a squared distance of admissible clusters or a padding value, never subnormal
__device__ __forceinline__ float rsqrt_approx(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;\n" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ void neumaier(float& sum, float& comp, float v) {
  const float t = sum + v;
  comp += fabsf(sum) >= fabsf(v) ? (sum - t) + v : (v - t) + sum;
  sum = t;
}

// Generator warp w owns tensor-memory lanes 32 (w % 4) .. +31 (the lanes its
// warp may access) and columns 8 (w / 4) .. +7: fold accumulator buffer buf
// (one finished block) into its row sums.
__device__ __forceinline__ void drain_block(uint32_t tmem, int warp, int buf, float* sum, float* comp) {
  float hh[8], cr[8];
  const uint32_t base = tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(64 * buf + 8 * (warp >> 2));
  tmem_ld8(base, hh);
  tmem_ld8(base + 32, cr);
#pragma unroll
  for (int n = 0; n < 8; ++n) neumaier(sum[n], comp[n], hh[n] + cr[n]);
}

// Compile-time tile geometry and shared-memory plan (bytes) for n_p^2 = NP2.
// An A tile holds MG row groups of 8; the tensor core also reads row groups
// MG..15 (rows beyond n_p^2, whose results are discarded), which land in the
// following buffers or the tail, always inside the allocation (TOTAL >= NEED).
template <int NP2>
struct TcShape {
  static constexpr int KP = (NP2 + 7) / 8 * 8;  // K padded to the MMA K step
  static constexpr int KC = KP / 4;             // 16-byte core-matrix columns along K
  static constexpr int MG = (NP2 + 7) / 8;      // 8-row groups holding the targets
  static constexpr uint32_t SBO = KC * 128;
  static constexpr uint32_t A_BYTES = MG * SBO, B_BYTES = 4 * SBO;
  static constexpr uint32_t STAGE = 2 * A_BYTES + 2 * B_BYTES, TILES = 2 * STAGE;
  static constexpr uint32_t NEED = STAGE + A_BYTES + 16 * SBO;
  static constexpr int NPRS = (MG + 1) * 8;     // padded target points (one spare group)
  static constexpr uint32_t PTS_OFF = TILES;    // prs [NPRS], pcs [2][KP]
  static constexpr uint32_t YS_OFF = PTS_OFF + (NPRS + 2 * KP) * 16;
  static constexpr uint32_t END = YS_OFF + 2 * KP * kYStride * 4;
  static constexpr uint32_t TOTAL = END > NEED ? END : NEED;
};

}  // namespace

template <int NP2>
__global__ void __launch_bounds__(kThreads, 1)
    k_far_tc(FarTcLevels L, const int2* __restrict__ work, int nrhs, int* __restrict__ err) {
  using G = TcShape<NP2>;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t full_bar[2], done_bar[2];
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;
  volatile int* abort_v = &abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int2 w = work[blockIdx.x];
  const int lev = w.x, row = w.y;
  const int* row_ptr = L.row_ptr[lev];
  const int kb = row_ptr[row], ke = row_ptr[row + 1];
  float* z = L.z[lev];
  if (kb == ke) {  // no far-field block in this row (uniform over the CTA)
    for (int e = tid; e < NP2 * nrhs; e += kThreads) z[(long)row * NP2 * nrhs + e] = 0.0f;
    return;
  }
  const int* col = L.col[lev];
  const float4* pts = L.pts[lev];
  const d4* cen = L.cen[lev];
  const float* y = L.y[lev];
  float4* prs = reinterpret_cast<float4*>(smem + G::PTS_OFF);
  float4* pcs = prs + G::NPRS;                             // [2][KP]
  float* ys = reinterpret_cast<float*>(smem + G::YS_OFF);  // [2][KP][kYStride]
  const int nblk = ke - kb;

  // stage the source points and Y_j of block column c2 into stage st
  auto issue_stage = [&](int st, int c2) {
    float4* pd = pcs + st * G::KP;
    for (int t = tid; t < NP2; t += kGenThreads) cp_async16(&pd[t], &pts[(long)c2 * NP2 + t]);
    float* yd = ys + st * G::KP * kYStride;
    const float* src = y + (long)c2 * NP2 * nrhs;
    if (nrhs == kN) {
      for (int t = tid; t < NP2 * (kN / 4); t += kGenThreads) {
        const int k = t >> 3, q = t & 7;
        cp_async16(yd + k * kYStride + 4 * q, src + k * kN + 4 * q);
      }
    } else {
      for (int t = tid; t < NP2 * nrhs; t += kGenThreads) {
        const int k = t / nrhs, n = t - k * nrhs;
        cp_async4(yd + k * kYStride + n, src + t);
      }
    }
  };

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_slot)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  if (tid == 0) {
    mbar_init(&full_bar[0], kGenThreads);
    mbar_init(&full_bar[1], kGenThreads);
    mbar_init(&done_bar[0], 1);
    mbar_init(&done_bar[1], 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (tid < kGenThreads) {
    // padded points, and the zero padding of the Y staging (never copied into)
    for (int t = tid; t < G::NPRS; t += kGenThreads)
      prs[t] = t < NP2 ? pts[(long)row * NP2 + t] : make_float4(kFar, kFar, kFar, 0.0f);
    if constexpr (G::KP > NP2) {
      constexpr int PAD = G::KP - NP2;
      for (int t = tid; t < 2 * PAD; t += kGenThreads)
        pcs[(t / PAD) * G::KP + NP2 + t % PAD] = make_float4(-kFar, -kFar, -kFar, 0.0f);
    }
    for (int t = tid; t < 2 * G::KP * kYStride; t += kGenThreads) {
      const int k = (t / kYStride) % G::KP, n = t % kYStride;
      if (k >= NP2 || n >= nrhs) ys[t] = 0.0f;
    }
    issue_stage(0, col[kb]);
    asm volatile("cp.async.commit_group;\n" ::);
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();  // the only CTA-wide barrier: the MMA warp leaves after its loop
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_slot;

  if (warp == kGenWarps) {
    // ---- MMA warp: one thread issues every tensor-core instruction ----
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_tf32(128, kN);
      const uint32_t base = smem_u32(smem);
      for (int it = 0; it < nblk; ++it) {
        const int s = it & 1;
        if (!mbar_wait(&full_bar[s], (uint32_t)((it >> 1) & 1))) {
          *abort_v = 1;
          atomicExch(err, 3);
          break;
        }
        if (*abort_v) break;
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const uint32_t a0 = base + s * G::STAGE, a1 = a0 + G::A_BYTES;
        const uint32_t b0 = a0 + 2 * G::A_BYTES, b1 = b0 + G::B_BYTES;
        const uint32_t d_hh = tmem + (uint32_t)(64 * s), d_cr = d_hh + 32;
#pragma unroll
        for (int pass = 0; pass < 3; ++pass) {
          uint64_t ad = umma_desc(pass == 2 ? a1 : a0, 128, G::SBO);
          uint64_t bd = umma_desc(pass == 1 ? b1 : b0, 128, G::SBO);
          const uint32_t dd = pass == 0 ? d_hh : d_cr;
#pragma unroll
          for (int ks = 0; ks < G::KP / 8; ++ks) {
            mma_tf32(dd, ad, bd, idesc, (pass == 2 || ks != 0) ? 1u : 0u);
            ad += 16;  // next K step: 256 bytes, in 16-byte units of the start-address field
            bd += 16;
          }
        }
        mma_commit(&done_bar[s]);
      }
    }
    return;
  }

  // ---- generator warps ----
  float sum[8], comp[8];  // this thread's row (lane) and 8 of the 32 columns
#pragma unroll
  for (int n = 0; n < 8; ++n) sum[n] = comp[n] = 0.0f;
  const d4 crow = cen[row];
  constexpr int AU = G::MG * G::KC, BU = 4 * G::KC;  // core matrices of A and B
  const int a_begin = (warp * AU) / kGenWarps, a_end = ((warp + 1) * AU) / kGenWarps;
  const int b_begin = (warp * BU) / kGenWarps, b_end = ((warp + 1) * BU) / kGenWarps;
  int it = 0;
  bool aborted = false;
  for (; it < nblk; ++it) {
    const int s = it & 1, k = kb + it;
    if (tid == 0 && it >= 2 && !mbar_wait(&done_bar[s], (uint32_t)(((it >> 1) - 1) & 1))) {
      *abort_v = 1;
      atomicExch(err, 1);
    }
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    gen_sync();  // stage s and accumulator buffer s free; block k staged; abort flag visible
    if (*abort_v) {
      aborted = true;
      break;
    }
    if (it >= 2) {  // block it-2 is complete: fold buffer s into the row sums
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      drain_block(tmem, warp, s, sum, comp);
    }
    if (it + 1 < nblk) issue_stage(s ^ 1, col[k + 1]);
    asm volatile("cp.async.commit_group;\n" ::);
    float* ahi = reinterpret_cast<float*>(smem + s * G::STAGE);
    float* alo = ahi + G::A_BYTES / 4;
    float* bhi = ahi + 2 * (G::A_BYTES / 4);
    float* blo = bhi + G::B_BYTES / 4;
    // B = Y_j^T (N x K, K-major): core matrix cm = ng * KC + kg, lane = 4 (n % 8) + kk % 4
    {
      const float* yst = ys + s * G::KP * kYStride + (lane & 3) * kYStride + (lane >> 2);
#pragma unroll 2
      for (int cm = b_begin; cm < b_end; ++cm) {
        const int ng = cm / G::KC, kg = cm - ng * G::KC;
        const float v = yst[kg * 4 * kYStride + ng * 8];
        const float h = tf32_hi(v);
        bhi[cm * 32 + lane] = h;
        blo[cm * 32 + lane] = v - h;
      }
    }
    // A = F_ij (M x K, K-major): core matrix cm = mg * KC + kg, lane = 4 (m % 8) + kk % 4
    {
      const float4* pc = pcs + s * G::KP + (lane & 3);
      const d4 ccol = cen[col[k]];
      const float dcx = (float)(crow.x - ccol.x), dcy = (float)(crow.y - ccol.y), dcz = (float)(crow.z - ccol.z);
      // this warp's core matrices [a_begin, a_end) as segments of whole or
      // partial row groups
      int cm = a_begin;
      int mg = cm / G::KC, kg = cm - mg * G::KC;
      while (cm < a_end) {
        const float4 xi = prs[mg * 8 + (lane >> 2)];
        const float x0 = dcx + xi.x, x1 = dcy + xi.y, x2 = dcz + xi.z, wm = xi.w * 0.0795774715f;
        const int kend = min(G::KC, kg + (a_end - cm));
        float* ph = ahi + cm * 32 + lane;
        float* pl = alo + cm * 32 + lane;
        const float4* py = pc + kg * 4;
        const int cnt = kend - kg;
#pragma unroll 4
        for (int q = 0; q < cnt; ++q) {
          const float4 yj = py[4 * q];
          const float d0 = x0 - yj.x, d1 = x1 - yj.y, d2 = x2 - yj.z;
          const float r2 = fmaf(d0, d0, fmaf(d1, d1, d2 * d2));
          const float f = rsqrt_approx(r2) * (wm * yj.w);
          const float h = tf32_hi(f);
          ph[32 * q] = h;
          pl[32 * q] = f - h;
        }
        cm += cnt;
        kg = 0;
        ++mg;
      }
    }
    // publish stage s to the tensor core: every generator thread arrives
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    mbar_arrive(&full_bar[s]);
  }
  // wait for the tensor core: the last block's commit covers every earlier MMA
  if (tid == 0 && it > 0) {
    const int last = it - 1;
    if (!mbar_wait(&done_bar[last & 1], (uint32_t)((last >> 1) & 1))) {
      *abort_v = 1;
      atomicExch(err, 2);
    }
  }
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
  gen_sync();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  if (!aborted && !*abort_v) {
    // blocks not folded in the loop: nblk-2 (if any) and nblk-1
    for (int b = nblk >= 2 ? nblk - 2 : 0; b < nblk; ++b) drain_block(tmem, warp, b & 1, sum, comp);
    const int m = (warp & 3) * 32 + lane, c0 = 8 * (warp >> 2);
    if (m < NP2) {
      float* zo = z + ((long)row * NP2 + m) * nrhs + c0;
#pragma unroll
      for (int n = 0; n < 8; ++n)
        if (c0 + n < nrhs) zo[n] = sum[n] + comp[n];
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  gen_sync();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTmemCols));
}

template <int NP2>
static cudaError_t launch_np(const FarTcLevels& L, const int2* work, int nwork, int nrhs, int* err, cudaStream_t s) {
  constexpr uint32_t smem = TcShape<NP2>::TOTAL;
  static_assert(smem <= 227 * 1024, "tensor-core far field: shared memory plan too large");
  cudaError_t e = smem_limit(k_far_tc<NP2>, smem);
  if (e != cudaSuccess) return e;
  k_far_tc<NP2><<<nwork, kThreads, smem, s>>>(L, work, nrhs, err);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Stored-tile helpers: 1-D TMA bulk copies and wide tensor-memory loads.
constexpr int kStoredThreads = 192;

// ---------------------------------------------------------------------------
// FP16 stored-tile variant (the one the product uses). Each low-rank block is
// scaled by a power of two sA (largest coupling in [2^13, 2^14)) and split into
// FP16 hi + lo, which keeps 22 bits of every coupling at 4 bytes per entry;
// each right-hand-side column of a cluster is scaled and split the same way
// (sB[n]). tcgen05.mma kind::f16 (M = 128, N = 32, K = 16) forms hi*hi and
// hi*lo + lo*hi exactly into FP32 tensor memory; the epilogue multiplies by
// 1/(sA sB[n]) (exact) before the compensated row sums. Four shared-memory
// stages of tiles move by 1-D TMA bulk copies; two accumulator buffers.
constexpr int kH16Stages = 4;

// The coupling (A) tiles store K padded only to the 8-element core-matrix
// width, KA, while the MMA steps K by 16 up to KP. Where KA < KP the last
// K step reads one core-matrix column past a row group's end: the first
// column of the next row group (or, after the last row group, of the next
// tile in the stage), finite data that meets the zero rows KA .. KP - 1 of
// the right-hand-side (B) tiles, which keep the full KP. Rows beyond the
// stored row groups (M = 128 reads 16) only feed output rows >= NP2, which
// are never read.
// EDGE (real operators, n_p^2 >= 16): the MMA covers K = KM, n_p^2 rounded
// down to the K step of 16, and the last E = n_p^2 - KM source columns are
// applied on the CUDA cores in FP32: their couplings follow the tiles of a
// block in global memory (EDGE_BYTES, [e][m]), read by the epilogue, so no
// K padding is stored or streamed (n_p = 9: 80 + 1 columns; 28 496 bytes
// per block instead of 30 976).
template <int NP2, int NSTAGE = kH16Stages, bool EDGE = false>
struct H16Shape {
  static constexpr bool SPLIT = EDGE && NP2 >= 16;
  static constexpr int KP = SPLIT ? NP2 / 16 * 16 : (NP2 + 15) / 16 * 16;  // K of the MMA steps and B tiles
  static constexpr int E = SPLIT ? NP2 - KP : 0;                            // source columns on the CUDA cores
  static constexpr int KC = KP / 8;                // 16-byte core-matrix columns (8 halves) of a B tile
  static constexpr int KA = SPLIT ? KP : (NP2 + 7) / 8 * 8;  // K stored in the A tiles
  static constexpr int KCA = KA / 8;
  static constexpr int MG = (NP2 + 7) / 8;
  static constexpr uint32_t SBO = KC * 128;        // B tiles: bytes between 8-row groups
  static constexpr uint32_t SBOA = KCA * 128;      // A tiles
  static constexpr uint32_t A_BYTES = MG * SBOA, B_BYTES = 4 * SBO;
  static constexpr uint32_t A2 = 2 * A_BYTES, B2 = 2 * B_BYTES;
  static constexpr uint32_t EDGE_BYTES = (uint32_t)(E * NP2 * 4 + 15) / 16 * 16;
  static constexpr uint32_t ASTRIDE = A2 + EDGE_BYTES;  // global bytes per block: hi, lo, edge couplings
  static constexpr uint32_t STAGE = A2 + B2;
  static constexpr uint32_t TILES = NSTAGE * STAGE;
  // furthest byte an M = 128 A operand reads, from its start
  static constexpr uint32_t A_READ = 15 * SBOA + KC * 128;
  static constexpr uint32_t NEED = (NSTAGE - 1) * STAGE + A_BYTES + A_READ;
  static constexpr uint32_t SMEM = TILES > NEED ? TILES : NEED;
  static_assert(KP - KA <= 8, "one aliased core-matrix column at most");
};

// power of two s with max_abs * s in [2^13, 2^14) (1 for zero or non-finite)
__device__ __forceinline__ float h16_scale(float max_abs) {
  if (!(max_abs > 0.0f) || !isfinite(max_abs)) return 1.0f;
  int e;
  frexpf(max_abs, &e);  // max_abs = f 2^e, f in [0.5, 1)
  return ldexpf(1.0f, 14 - e);
}

// NSTAGE shared-memory stages, MINB CTAs per SM: 4 stages and one CTA per SM,
// or 2 stages and two CTAs per SM (two producers, issuers and epilogues per
// SM, twice the blocks in flight: 0.469 -> 0.363 ms per launch at c2). The
// built-in choice takes two CTAs per SM when there are at least as many rows
// as CTAs (launch plan far_ctas)
// HI: the hi coupling tiles only (hi*hi and hi*lo, the lo tiles not read)
template <int NP2, int NSTAGE, int MINB, bool HI>
__global__ void __launch_bounds__(kStoredThreads, MINB)
    k_far_h16(FarH16Tiles T, const int2* __restrict__ work, int nwork, int nrhs, int* __restrict__ err) {
  // Persistent: CTA c takes the rows c, c + gridDim.x, ... of the work list
  // (sorted by block count) and all three roles walk the same flattened
  // sequence of blocks, so the copy pipeline runs on across row boundaries.
  using G = H16Shape<NP2, NSTAGE, true>;
  constexpr int S = NSTAGE;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t full_bar[S], done_bar[S], free_bar[2];
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;
  volatile int* abort_v = &abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_slot)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  if (tid == 0) {
    for (int b = 0; b < S; ++b) {
      mbar_init(&full_bar[b], 1);
      mbar_init(&done_bar[b], 1);
    }
    mbar_init(&free_bar[0], 4);
    mbar_init(&free_bar[1], 4);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_slot;

  if (warp == 0) {
    // ---- producer: whole tiles by 1-D TMA bulk copies ----
    if (lane == 0) {
      int it = 0;
      for (int wi = blockIdx.x; wi < nwork && !*abort_v; wi += gridDim.x) {
        const int lev = work[wi].x, row = work[wi].y;
        const int kb = T.row_ptr[lev][row], ke = T.row_ptr[lev][row + 1];
        const int* col = T.col[lev];
        const unsigned char* atiles = T.a[lev];
        const unsigned char* btiles = T.b[lev];
        for (int k = kb; k < ke; ++k, ++it) {
          const int st = it % S;
          if (it >= S && !mbar_wait(&done_bar[st], (uint32_t)((it / S - 1) & 1))) {
            *abort_v = 1;
            atomicExch(err, 4);
            break;
          }
          if (*abort_v) break;
          unsigned char* sm = smem + st * G::STAGE;
          const unsigned char* ga = atiles + (size_t)k * G::ASTRIDE;
          const unsigned char* gb = btiles + (size_t)col[k] * G::B2;
          // hi and lo tiles are contiguous in global and shared memory: one copy each for A and B
          mbar_expect_tx(&full_bar[st], (HI ? G::A_BYTES : G::A2) + G::B2);
          bulk_g2s(sm, ga, HI ? G::A_BYTES : G::A2, &full_bar[st]);
          bulk_g2s(sm + G::A2, gb, G::B2, &full_bar[st]);
        }
      }
    }
  } else if (warp == 1) {
    // ---- MMA issuer ----
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_f16(128, kN);
      const uint32_t base = smem_u32(smem);
      int it = 0;
      for (int wi = blockIdx.x; wi < nwork && !*abort_v; wi += gridDim.x) {
        const int lev = work[wi].x, row = work[wi].y;
        const int nb = T.row_ptr[lev][row + 1] - T.row_ptr[lev][row];
        for (int q = 0; q < nb; ++q, ++it) {
          const int st = it % S, ab = it & 1;
          if (!mbar_wait(&full_bar[st], (uint32_t)((it / S) & 1))) {
            *abort_v = 1;
            atomicExch(err, 5);
            break;
          }
          if (it >= 2 && !mbar_wait(&free_bar[ab], (uint32_t)(((it >> 1) - 1) & 1))) {
            *abort_v = 1;
            atomicExch(err, 6);
            break;
          }
          if (*abort_v) break;
          asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
          const uint32_t a0 = base + st * G::STAGE, a1 = a0 + G::A_BYTES;
          const uint32_t b0 = a0 + G::A2, b1 = b0 + G::B_BYTES;
          const uint32_t d_hh = tmem + (uint32_t)(64 * ab), d_cr = d_hh + 32;
#pragma unroll
          for (int pass = 0; pass < (HI ? 2 : 3); ++pass) {
            uint64_t ad = umma_desc(pass == 2 ? a1 : a0, 128, G::SBOA);
            uint64_t bd = umma_desc(pass == 1 ? b1 : b0, 128, G::SBO);
            const uint32_t dd = pass == 0 ? d_hh : d_cr;
#pragma unroll
            for (int ks = 0; ks < G::KP / 16; ++ks) {
              mma_f16(dd, ad, bd, idesc, (pass == 2 || ks != 0) ? 1u : 0u);
              ad += 16;  // next K step: two core matrices = 256 bytes
              bd += 16;
            }
          }
          mma_commit(&done_bar[st]);
        }
      }
    }
  } else {
    // ---- epilogue warps 2-5: tensor-memory lanes 32 (warp % 4) .. +31 ----
    const uint32_t lane_base = tmem + ((uint32_t)((warp & 3) * 32) << 16);
    const int m = (warp & 3) * 32 + lane;
    int it = 0;
    bool ok = true;
    for (int wi = blockIdx.x; wi < nwork && ok; wi += gridDim.x) {
      const int lev = work[wi].x, row = work[wi].y;
      const int kb = T.row_ptr[lev][row], ke = T.row_ptr[lev][row + 1];
      const int* col = T.col[lev];
      const float* ainv = T.ainv[lev];
      const float* binv = T.binv[lev];
      const unsigned char* atiles = T.a[lev];
      const float* ylev = T.y[lev];
      float sum[32], comp[32];
#pragma unroll
      for (int n = 0; n < 32; ++n) sum[n] = comp[n] = 0.0f;
      for (int k = kb; k < ke; ++k, ++it) {
        const int st = it % S, ab = it & 1;
        // the block's scales and edge columns do not depend on its MMAs: load
        // them first, so that their latency overlaps the wait for the
        // accumulators
        const float sa = __ldg(&ainv[k]);
        float4 bsc[8];
        {
          const float4* sb = reinterpret_cast<const float4*>(binv + (long)col[k] * kN);
#pragma unroll
          for (int q = 0; q < 8; ++q) bsc[q] = __ldg(&sb[q]);
        }
        // source columns KP .. NP2 - 1 in FP32, f Y[KP + e][n] added to the
        // compensation term of the row sums (the edge is a 1 / n_p^2 share of
        // a block's contribution, so plain FP32 sums keep its error below
        // the tiles' own)
        if (G::E > 0) {
          const float* edge = reinterpret_cast<const float*>(atiles + (size_t)k * G::ASTRIDE + G::A2);
          const float* ye = ylev + ((long)col[k] * NP2 + G::KP) * nrhs;
#pragma unroll
          for (int e = 0; e < G::E; ++e) {
            const float f = m < NP2 ? __ldg(edge + e * NP2 + m) : 0.0f;
            if (nrhs == kN) {
              const float4* y4 = reinterpret_cast<const float4*>(ye + e * kN);
#pragma unroll
              for (int q = 0; q < 8; ++q) {
                const float4 v = __ldg(&y4[q]);
                comp[4 * q + 0] = fmaf(f, v.x, comp[4 * q + 0]);
                comp[4 * q + 1] = fmaf(f, v.y, comp[4 * q + 1]);
                comp[4 * q + 2] = fmaf(f, v.z, comp[4 * q + 2]);
                comp[4 * q + 3] = fmaf(f, v.w, comp[4 * q + 3]);
              }
            } else {
#pragma unroll
              for (int n = 0; n < 32; ++n)
                if (n < nrhs) comp[n] = fmaf(f, __ldg(ye + e * nrhs + n), comp[n]);
            }
          }
        }
        int got = 1;
        if (lane == 0) got = mbar_wait(&done_bar[st], (uint32_t)((it / S) & 1)) ? 1 : 0;
        got = __shfl_sync(0xffffffffu, got, 0);
        if (!got) {
          if (lane == 0) {
            *abort_v = 1;
            atomicExch(err, 7);
          }
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        float hh[32], cr[32];
        tmem_ld32(lane_base + (uint32_t)(64 * ab), hh);
        tmem_ld32(lane_base + (uint32_t)(64 * ab + 32), cr);
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive(&free_bar[ab]);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const float4 b4 = bsc[q];
          neumaier(sum[4 * q + 0], comp[4 * q + 0], (hh[4 * q + 0] + cr[4 * q + 0]) * (sa * b4.x));
          neumaier(sum[4 * q + 1], comp[4 * q + 1], (hh[4 * q + 1] + cr[4 * q + 1]) * (sa * b4.y));
          neumaier(sum[4 * q + 2], comp[4 * q + 2], (hh[4 * q + 2] + cr[4 * q + 2]) * (sa * b4.z));
          neumaier(sum[4 * q + 3], comp[4 * q + 3], (hh[4 * q + 3] + cr[4 * q + 3]) * (sa * b4.w));
        }
      }
      if (ok && m < NP2) {  // rows without blocks come out as zeros
        float* zo = T.z[lev] + ((long)row * NP2 + m) * nrhs;
#pragma unroll
        for (int n = 0; n < 32; ++n)
          if (n < nrhs) zo[n] = sum[n] + comp[n];
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTmemCols));
}

// A tiles of nblocks FP64 blocks (column-major, stride bstride): one CTA per
// block finds the largest coupling, picks sA, writes [hi tile][lo tile] with
// entry (m, k) in core matrix (m / 8) * KCA + k / 8 at row m % 8, element k % 8,
// and 1/sA to ainv[b].
template <int NP2>
__global__ void __launch_bounds__(256) k_build_h16_atiles(const double* __restrict__ F, long bstride,
                                                          __half* __restrict__ tiles, float* __restrict__ ainv) {
  using G = H16Shape<NP2, kH16Stages, true>;
  constexpr int AH = G::A_BYTES / 2;  // halves per tile
  __shared__ float red[8];
  const long b = blockIdx.x;
  const double* Fb = F + b * bstride;
  float mx = 0.0f;
  for (int e = threadIdx.x; e < NP2 * NP2; e += blockDim.x) mx = fmaxf(mx, (float)fabs(Fb[e]));
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
  __syncthreads();
  mx = red[0];
  for (int i = 1; i < (int)(blockDim.x >> 5); ++i) mx = fmaxf(mx, red[i]);
  const float sa = h16_scale(mx * 1.0000001f);
  __half* out = tiles + b * (G::ASTRIDE / 2);
  for (int e = threadIdx.x; e < AH; e += blockDim.x) {
    const int cm = e >> 6, r = (e >> 3) & 7, c = e & 7;
    const int m = (cm / G::KCA) * 8 + r, k = (cm % G::KCA) * 8 + c;
    const double v = (m < NP2 && k < NP2) ? Fb[(long)k * NP2 + m] * (double)sa : 0.0;
    const __half h = __double2half(v);
    out[e] = h;
    out[AH + e] = __double2half(v - (double)__half2float(h));
  }
  // the edge columns KP .. NP2 - 1, unscaled FP32, [e][m]
  float* edge = reinterpret_cast<float*>(out + 2 * AH);
  for (int t = threadIdx.x; t < G::E * NP2; t += blockDim.x) edge[t] = (float)Fb[(long)G::KP * NP2 + t];
  if (threadIdx.x == 0) ainv[b] = 1.0f / sa;
}

// B tiles of every cluster of every level (one CTA each): per right-hand-side
// column n a scale sB[n], Y_c^T scaled and split into [hi tile][lo tile], and
// 1/sB[n] to binv (32 per cluster, zero-padded columns have scale 1).
template <int NP2>
__global__ void __launch_bounds__(256) k_build_h16_btiles(FarH16Tiles T, int nlev, int nrhs) {
  using G = H16Shape<NP2, kH16Stages, true>;
  constexpr int BH = G::B_BYTES / 2;
  __shared__ float cmax[8][kN];
  __shared__ float scale[kN];
  int c = blockIdx.x, lev = 0;
  while (lev + 1 < nlev && c >= T.ncl[lev]) c -= T.ncl[lev++];
  const float* y = T.y[lev] + (long)c * NP2 * nrhs;
  // column maxima: thread (q, n) scans rows q, q + 8, ...
  {
    const int n = threadIdx.x & 31, q = threadIdx.x >> 5;
    float mx = 0.0f;
    if (n < nrhs)
      for (int k = q; k < NP2; k += 8) mx = fmaxf(mx, fabsf(y[k * nrhs + n]));
    cmax[q][n] = mx;
  }
  __syncthreads();
  if (threadIdx.x < kN) {
    float mx = 0.0f;
    for (int q = 0; q < 8; ++q) mx = fmaxf(mx, cmax[q][threadIdx.x]);
    const float sb = h16_scale(mx * 1.0000001f);
    scale[threadIdx.x] = sb;
    T.binv[lev][(long)c * kN + threadIdx.x] = 1.0f / sb;
  }
  __syncthreads();
  __half* out = reinterpret_cast<__half*>(T.b[lev]) + (long)c * 2 * BH;
  for (int e = threadIdx.x; e < BH; e += blockDim.x) {
    const int cm = e >> 6, r = (e >> 3) & 7, cc = e & 7;
    const int n = (cm / G::KC) * 8 + r, k = (cm % G::KC) * 8 + cc;
    const float v = (n < nrhs && k < NP2) ? y[k * nrhs + n] * scale[n] : 0.0f;
    const __half h = __float2half_rn(v);
    out[e] = h;
    out[BH + e] = __float2half_rn(v - __half2float(h));
  }
}

#define BG_H16_SHAPES(X) X(4) X(9) X(16) X(25) X(36) X(49) X(64) X(81)

size_t far_h16_atile_bytes(int np2) {
  switch (np2) {
#define BG_T(N) \
  case N: return H16Shape<N, kH16Stages, true>::ASTRIDE;
    BG_H16_SHAPES(BG_T)
#undef BG_T
    default: return 0;
  }
}
size_t far_h16_btile_bytes(int np2) {
  switch (np2) {
#define BG_T(N) \
  case N: return H16Shape<N, kH16Stages, true>::B2;
    BG_H16_SHAPES(BG_T)
#undef BG_T
    default: return 0;
  }
}

cudaError_t launch_build_h16_atiles(int np2, const double* F, long bstride, long nblocks, void* tiles, float* ainv,
                                    cudaStream_t s) {
  if (nblocks == 0) return cudaSuccess;
  switch (np2) {
#define BG_T(N)                                                                                               \
  case N:                                                                                                     \
    k_build_h16_atiles<N><<<(unsigned)nblocks, 256, 0, s>>>(F, bstride, static_cast<__half*>(tiles), ainv); \
    break;
    BG_H16_SHAPES(BG_T)
#undef BG_T
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_build_h16_btiles(const FarH16Tiles& T, int nlev, int np2, int nrhs, cudaStream_t s) {
  if (nlev < 1 || nlev > kMaxTileLevels || nrhs < 1 || nrhs > kN) return cudaErrorInvalidValue;
  int ncl_total = 0;
  for (int l = 0; l < nlev; ++l) ncl_total += T.ncl[l];
  if (ncl_total == 0) return cudaSuccess;
  switch (np2) {
#define BG_T(N) \
  case N: k_build_h16_btiles<N><<<ncl_total, 256, 0, s>>>(T, nlev, nrhs); break;
    BG_H16_SHAPES(BG_T)
#undef BG_T
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <int N, bool HI>
static cudaError_t far_h16_launch(const FarH16Tiles& T, const int2* work, int nwork, int nrhs, int* err,
                                  cudaStream_t s, int ctas_per_sm, int nsm) {
  if (ctas_per_sm == 2) {
    constexpr uint32_t smem = H16Shape<N, 2, true>::SMEM;
    static_assert(2 * smem <= 220 * 1024, "FP16 far field: two CTAs per SM do not fit");
    cudaError_t e = smem_limit(k_far_h16<N, 2, 2, HI>, smem);
    if (e != cudaSuccess) return e;
    k_far_h16<N, 2, 2, HI><<<std::min(nwork, 2 * nsm), kStoredThreads, smem, s>>>(T, work, nwork, nrhs, err);
    return cudaGetLastError();
  }
  constexpr uint32_t smem = H16Shape<N, kH16Stages, true>::SMEM;
  static_assert(smem <= 227 * 1024, "FP16 far field: shared memory plan too large");
  cudaError_t e = smem_limit(k_far_h16<N, kH16Stages, 1, HI>, smem);
  if (e != cudaSuccess) return e;
  k_far_h16<N, kH16Stages, 1, HI><<<std::min(nwork, nsm), kStoredThreads, smem, s>>>(T, work, nwork, nrhs, err);
  return cudaGetLastError();
}

cudaError_t launch_far_h16(const FarH16Tiles& T, const int2* work, int nwork, int np2, int nrhs, int* err,
                           cudaStream_t s, int ctas_per_sm, bool hi_only) {
  if (nwork == 0) return cudaSuccess;
  if (!far_tc_supported(false, np2, nrhs)) return cudaErrorInvalidValue;
  // persistent CTAs: one or two per SM
  int dev = 0, nsm = 0;
  cudaError_t ea = cudaGetDevice(&dev);
  if (ea == cudaSuccess) ea = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (ea != cudaSuccess) return ea;
  // built-in: two CTAs per SM when every CTA still gets a row
  if (ctas_per_sm != 1 && ctas_per_sm != 2) ctas_per_sm = nwork >= 2 * nsm ? 2 : 1;
  switch (np2) {
#define BG_T(N)                                                                                            \
  case N:                                                                                                  \
    return hi_only ? far_h16_launch<N, true>(T, work, nwork, nrhs, err, s, ctas_per_sm, nsm)              \
                   : far_h16_launch<N, false>(T, work, nwork, nrhs, err, s, ctas_per_sm, nsm);
    BG_H16_SHAPES(BG_T)
#undef BG_T
    default: return cudaErrorInvalidValue;
  }
}

// ---------------------------------------------------------------------------
// Complex stored-tile variant (Helmholtz and Maxwell kernels exp(-i k r)/(4 pi r)).
// A block K = Kr + i Ki is stored as four FP16 tiles [Kr hi][Kr lo][Ki hi][Ki lo]
// under one power-of-two scale; the right-hand sides of a cluster (up to 16
// complex columns) as one real tile pair of 32 columns [Re Y | Im Y], each
// column with its own scale. Per block the MMA warp forms P = Kr [Re Y | Im Y]
// and Q = Ki [Re Y | Im Y] (hi*hi and hi*lo + lo*hi each, so four FP32
// accumulators of 32 columns, two buffers: 256 tensor-memory columns), and the
// epilogue folds Re Z = P_re - Q_im, Im Z = P_im + Q_re into compensated sums.
// Two shared-memory stages (a stage holds 80 KB at n_p = 9, 105 KB at 10).
constexpr int kH16CStages = 2;
constexpr int kNC = 16;                // complex columns per launch
constexpr uint32_t kTmemColsC = 256;

template <int NP2>
struct H16CShape {
  using R = H16Shape<NP2>;
  static constexpr uint32_t SBO = R::SBO, SBOA = R::SBOA, A_BYTES = R::A_BYTES, B_BYTES = R::B_BYTES;
  static constexpr uint32_t A4 = 4 * A_BYTES, B2 = 2 * B_BYTES;
  static constexpr uint32_t STAGE = A4 + B2;
  static constexpr uint32_t TILES = kH16CStages * STAGE;
  // an M = 128 operand read starting at the last A tile of the last stage
  static constexpr uint32_t NEED = (kH16CStages - 1) * STAGE + 3 * A_BYTES + R::A_READ;
  static constexpr uint32_t SMEM = TILES > NEED ? TILES : NEED;
};

template <int NP2>
__global__ void __launch_bounds__(kStoredThreads, 1)
    k_far_h16c(FarH16Tiles T, const int2* __restrict__ work, int nwork, int ldz, int z0, int nc,
               int* __restrict__ err) {
  using G = H16CShape<NP2>;
  constexpr int S = kH16CStages;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t full_bar[S], done_bar[S], free_bar[2];
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;
  volatile int* abort_v = &abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_slot)),
                 "r"(kTmemColsC));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  if (tid == 0) {
    for (int b = 0; b < S; ++b) {
      mbar_init(&full_bar[b], 1);
      mbar_init(&done_bar[b], 1);
    }
    mbar_init(&free_bar[0], 4);
    mbar_init(&free_bar[1], 4);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_slot;

  if (warp == 0) {
    // ---- producer: 4 coupling tiles + 2 right-hand-side tiles per block ----
    if (lane == 0) {
      int it = 0;
      for (int wi = blockIdx.x; wi < nwork && !*abort_v; wi += gridDim.x) {
        const int lev = work[wi].x, row = work[wi].y;
        const int kb = T.row_ptr[lev][row], ke = T.row_ptr[lev][row + 1];
        const int* col = T.col[lev];
        for (int k = kb; k < ke; ++k, ++it) {
          const int st = it % S;
          if (it >= S && !mbar_wait(&done_bar[st], (uint32_t)((it / S - 1) & 1))) {
            *abort_v = 1;
            atomicExch(err, 14);
            break;
          }
          if (*abort_v) break;
          unsigned char* sm = smem + st * G::STAGE;
          const unsigned char* ga = T.a[lev] + (size_t)k * G::A4;
          const unsigned char* gb = T.b[lev] + (size_t)col[k] * G::B2;
          // the four coupling tiles and the two right-hand-side tiles are contiguous: two copies
          mbar_expect_tx(&full_bar[st], G::STAGE);
          bulk_g2s(sm, ga, G::A4, &full_bar[st]);
          bulk_g2s(sm + G::A4, gb, G::B2, &full_bar[st]);
        }
      }
    }
  } else if (warp == 1) {
    // ---- MMA issuer ----
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_f16(128, kN);
      const uint32_t base = smem_u32(smem);
      int it = 0;
      for (int wi = blockIdx.x; wi < nwork && !*abort_v; wi += gridDim.x) {
        const int lev = work[wi].x, row = work[wi].y;
        const int nb = T.row_ptr[lev][row + 1] - T.row_ptr[lev][row];
        for (int q = 0; q < nb; ++q, ++it) {
          const int st = it % S, ab = it & 1;
          if (!mbar_wait(&full_bar[st], (uint32_t)((it / S) & 1))) {
            *abort_v = 1;
            atomicExch(err, 15);
            break;
          }
          if (it >= 2 && !mbar_wait(&free_bar[ab], (uint32_t)(((it >> 1) - 1) & 1))) {
            *abort_v = 1;
            atomicExch(err, 16);
            break;
          }
          if (*abort_v) break;
          asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
          const uint32_t a0 = base + st * G::STAGE;
          const uint32_t b0 = a0 + G::A4, b1 = b0 + G::B_BYTES;
#pragma unroll
          for (int part = 0; part < 2; ++part) {  // 0: Kr -> P, 1: Ki -> Q
            const uint32_t ahi = a0 + (2 * part) * G::A_BYTES, alo = ahi + G::A_BYTES;
            const uint32_t d_hh = tmem + (uint32_t)(128 * ab + 64 * part), d_cr = d_hh + 32;
#pragma unroll
            for (int pass = 0; pass < 3; ++pass) {
              uint64_t ad = umma_desc(pass == 2 ? alo : ahi, 128, G::SBOA);
              uint64_t bd = umma_desc(pass == 1 ? b1 : b0, 128, G::SBO);
              const uint32_t dd = pass == 0 ? d_hh : d_cr;
#pragma unroll
              for (int ks = 0; ks < H16Shape<NP2>::KP / 16; ++ks) {
                mma_f16(dd, ad, bd, idesc, (pass == 2 || ks != 0) ? 1u : 0u);
                ad += 16;
                bd += 16;
              }
            }
          }
          mma_commit(&done_bar[st]);
        }
      }
    }
  } else {
    // ---- epilogue warps 2-5: tensor-memory lanes 32 (warp % 4) .. +31 ----
    const uint32_t lane_base = tmem + ((uint32_t)((warp & 3) * 32) << 16);
    const int m = (warp & 3) * 32 + lane;
    int it = 0;
    bool ok = true;
    for (int wi = blockIdx.x; wi < nwork && ok; wi += gridDim.x) {
      const int lev = work[wi].x, row = work[wi].y;
      const int kb = T.row_ptr[lev][row], ke = T.row_ptr[lev][row + 1];
      const int* col = T.col[lev];
      const float* ainv = T.ainv[lev];
      const float* binv = T.binv[lev];
      float sre[kNC], cre[kNC], sim[kNC], cim[kNC];
#pragma unroll
      for (int n = 0; n < kNC; ++n) sre[n] = cre[n] = sim[n] = cim[n] = 0.0f;
      for (int k = kb; k < ke; ++k, ++it) {
        const int st = it % S, ab = it & 1;
        // the block's scales, loaded before the wait for its accumulators
        const float sa = __ldg(&ainv[k]);
        float sbv[32];
        {
          const float4* sb4 = reinterpret_cast<const float4*>(binv + (long)col[k] * kN);
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const float4 b4 = __ldg(&sb4[q]);
            sbv[4 * q] = sa * b4.x;
            sbv[4 * q + 1] = sa * b4.y;
            sbv[4 * q + 2] = sa * b4.z;
            sbv[4 * q + 3] = sa * b4.w;
          }
        }
        int got = 1;
        if (lane == 0) got = mbar_wait(&done_bar[st], (uint32_t)((it / S) & 1)) ? 1 : 0;
        got = __shfl_sync(0xffffffffu, got, 0);
        if (!got) {
          if (lane == 0) {
            *abort_v = 1;
            atomicExch(err, 17);
          }
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        float p[32];
        {
          float hh[32], cr[32];
          tmem_ld32(lane_base + (uint32_t)(128 * ab), hh);
          tmem_ld32(lane_base + (uint32_t)(128 * ab + 32), cr);
#pragma unroll
          for (int n = 0; n < 32; ++n) p[n] = (hh[n] + cr[n]) * sbv[n];
        }
        float hh[32], cr[32];
        tmem_ld32(lane_base + (uint32_t)(128 * ab + 64), hh);
        tmem_ld32(lane_base + (uint32_t)(128 * ab + 96), cr);
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive(&free_bar[ab]);
#pragma unroll
        for (int n = 0; n < kNC; ++n) {
          const float q_re = (hh[n] + cr[n]) * sbv[n];
          const float q_im = (hh[kNC + n] + cr[kNC + n]) * sbv[kNC + n];
          neumaier(sre[n], cre[n], p[n] - q_im);
          neumaier(sim[n], cim[n], p[kNC + n] + q_re);
        }
      }
      if (ok && m < NP2) {
        float2* zo = reinterpret_cast<float2*>(T.z[lev]) + ((long)row * NP2 + m) * ldz + z0;
#pragma unroll
        for (int n = 0; n < kNC; ++n)
          if (n < nc) zo[n] = make_float2(sre[n] + cre[n], sim[n] + cim[n]);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTmemColsC));
}

// Complex A tiles: one scale per block from the largest |Re| or |Im|.
template <int NP2>
__global__ void __launch_bounds__(256) k_build_h16c_atiles(const double2* __restrict__ F, long bstride,
                                                           __half* __restrict__ tiles, float* __restrict__ ainv) {
  using G = H16Shape<NP2>;
  constexpr int AH = G::A_BYTES / 2;
  __shared__ float red[8];
  const long b = blockIdx.x;
  const double2* Fb = F + b * bstride;
  float mx = 0.0f;
  for (int e = threadIdx.x; e < NP2 * NP2; e += blockDim.x) {
    const double2 v = Fb[e];
    mx = fmaxf(mx, fmaxf((float)fabs(v.x), (float)fabs(v.y)));
  }
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
  __syncthreads();
  mx = red[0];
  for (int i = 1; i < (int)(blockDim.x >> 5); ++i) mx = fmaxf(mx, red[i]);
  const float sa = h16_scale(mx * 1.0000001f);
  __half* out = tiles + b * 4 * AH;
  for (int e = threadIdx.x; e < AH; e += blockDim.x) {
    const int cm = e >> 6, r = (e >> 3) & 7, c = e & 7;
    const int m = (cm / G::KCA) * 8 + r, k = (cm % G::KCA) * 8 + c;
    double2 v = make_double2(0.0, 0.0);
    if (m < NP2 && k < NP2) v = Fb[(long)k * NP2 + m];
    const double vr = v.x * (double)sa, vi = v.y * (double)sa;
    const __half hr = __double2half(vr), hi = __double2half(vi);
    out[e] = hr;
    out[AH + e] = __double2half(vr - (double)__half2float(hr));
    out[2 * AH + e] = hi;
    out[3 * AH + e] = __double2half(vi - (double)__half2float(hi));
  }
  if (threadIdx.x == 0) ainv[b] = 1.0f / sa;
}

// Complex B tiles of every cluster of every level: real columns n < 16 hold
// Re Y[:, y0 + n], columns 16 + n hold Im Y[:, y0 + n] (n < nc; others zero).
// Y rows have ldy complex entries.
template <int NP2>
__global__ void __launch_bounds__(256) k_build_h16c_btiles(FarH16Tiles T, int nlev, int ldy, int y0, int nc) {
  using G = H16Shape<NP2>;
  constexpr int BH = G::B_BYTES / 2;
  __shared__ float cmax[8][kN];
  __shared__ float scale[kN];
  int c = blockIdx.x, lev = 0;
  while (lev + 1 < nlev && c >= T.ncl[lev]) c -= T.ncl[lev++];
  const float2* y = reinterpret_cast<const float2*>(T.y[lev]) + (long)c * NP2 * ldy + y0;
  auto val = [&](int k, int n) -> float {
    const int j = n & (kNC - 1);
    if (j >= nc || k >= NP2) return 0.0f;
    const float2 v = y[(long)k * ldy + j];
    return n < kNC ? v.x : v.y;
  };
  {
    const int n = threadIdx.x & 31, q = threadIdx.x >> 5;
    float mx = 0.0f;
    for (int k = q; k < NP2; k += 8) mx = fmaxf(mx, fabsf(val(k, n)));
    cmax[q][n] = mx;
  }
  __syncthreads();
  if (threadIdx.x < kN) {
    float mx = 0.0f;
    for (int q = 0; q < 8; ++q) mx = fmaxf(mx, cmax[q][threadIdx.x]);
    const float sb = h16_scale(mx * 1.0000001f);
    scale[threadIdx.x] = sb;
    T.binv[lev][(long)c * kN + threadIdx.x] = 1.0f / sb;
  }
  __syncthreads();
  __half* out = reinterpret_cast<__half*>(T.b[lev]) + (long)c * 2 * BH;
  for (int e = threadIdx.x; e < BH; e += blockDim.x) {
    const int cm = e >> 6, r = (e >> 3) & 7, cc = e & 7;
    const int n = (cm / G::KC) * 8 + r, k = (cm % G::KC) * 8 + cc;
    const float v = val(k, n) * scale[n];
    const __half h = __float2half_rn(v);
    out[e] = h;
    out[BH + e] = __float2half_rn(v - __half2float(h));
  }
}

#define BG_H16C_SHAPES(X) X(4) X(9) X(16) X(25) X(36) X(49) X(64) X(81) X(100)

size_t far_h16c_atile_bytes(int np2) {
  switch (np2) {
#define BG_T(N) \
  case N: return H16CShape<N>::A4;
    BG_H16C_SHAPES(BG_T)
#undef BG_T
    default: return 0;
  }
}
size_t far_h16c_btile_bytes(int np2) {
  switch (np2) {
#define BG_T(N) \
  case N: return H16CShape<N>::B2;
    BG_H16C_SHAPES(BG_T)
#undef BG_T
    default: return 0;
  }
}

cudaError_t launch_build_h16c_atiles(int np2, const void* F, long bstride, long nblocks, void* tiles, float* ainv,
                                     cudaStream_t s) {
  if (nblocks == 0) return cudaSuccess;
  switch (np2) {
#define BG_T(N)                                                                                          \
  case N:                                                                                                \
    k_build_h16c_atiles<N><<<(unsigned)nblocks, 256, 0, s>>>(static_cast<const double2*>(F), bstride,    \
                                                             static_cast<__half*>(tiles), ainv);         \
    break;
    BG_H16C_SHAPES(BG_T)
#undef BG_T
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_build_h16c_btiles(const FarH16Tiles& T, int nlev, int np2, int ldy, int y0, int nc,
                                     cudaStream_t s) {
  if (nlev < 1 || nlev > kMaxTileLevels || nc < 1 || nc > kNC || y0 < 0 || y0 + nc > ldy) return cudaErrorInvalidValue;
  int ncl_total = 0;
  for (int l = 0; l < nlev; ++l) ncl_total += T.ncl[l];
  if (ncl_total == 0) return cudaSuccess;
  switch (np2) {
#define BG_T(N) \
  case N: k_build_h16c_btiles<N><<<ncl_total, 256, 0, s>>>(T, nlev, ldy, y0, nc); break;
    BG_H16C_SHAPES(BG_T)
#undef BG_T
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_far_h16c(const FarH16Tiles& T, const int2* work, int nwork, int np2, int ldz, int z0, int nc,
                            int* err, cudaStream_t s) {
  if (nwork == 0) return cudaSuccess;
  if (far_h16c_atile_bytes(np2) == 0 || nc < 1 || nc > kNC || z0 < 0 || z0 + nc > ldz) return cudaErrorInvalidValue;
  int dev = 0, nsm = 0;
  cudaError_t ea = cudaGetDevice(&dev);
  if (ea == cudaSuccess) ea = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (ea != cudaSuccess) return ea;
  switch (np2) {
#define BG_T(N)                                                                                              \
  case N: {                                                                                                  \
    constexpr uint32_t smem = H16CShape<N>::SMEM;                                                            \
    static_assert(smem <= 220 * 1024, "complex FP16 far field: shared memory plan too large");               \
    cudaError_t e = smem_limit(k_far_h16c<N>, smem); \
    if (e != cudaSuccess) return e;                                                                          \
    k_far_h16c<N><<<std::min(nwork, nsm), kStoredThreads, smem, s>>>(T, work, nwork, ldz, z0, nc, err);     \
    return cudaGetLastError();                                                                               \
  }
    BG_H16C_SHAPES(BG_T)
#undef BG_T
    default: return cudaErrorInvalidValue;
  }
}

// ---------------------------------------------------------------------------
// Watchdog self-test: one thread waits on an mbarrier that nothing completes,
// with a wait bounded by `limit` clock cycles, the same bounded wait the
// tensor-core kernels use; when it runs out the kernel records code 99 in the
// error flag and returns normally.
__global__ void k_wait_selftest(long long limit, int* __restrict__ err) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    const uint32_t a = smem_u32(&bar);
    const long long t0 = clock64();
    bool done = false;
    while (!done && clock64() - t0 <= limit) {
      uint32_t d;
      asm volatile(
          "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
          : "=r"(d)
          : "r"(a), "r"(0u)
          : "memory");
      done = d != 0;
    }
    if (!done) atomicExch(err, 99);
  }
}

cudaError_t launch_wait_selftest(long long limit_cycles, int* err, cudaStream_t s) {
  if (limit_cycles <= 0 || limit_cycles > 4000000000LL) return cudaErrorInvalidValue;
  k_wait_selftest<<<1, 32, 0, s>>>(limit_cycles, err);
  return cudaGetLastError();
}

bool far_tc_supported(bool cplx, int np2, int nrhs) {
  const bool shape = np2 == 4 || np2 == 9 || np2 == 16 || np2 == 25 || np2 == 36 || np2 == 49 || np2 == 64 || np2 == 81;
  return !cplx && shape && nrhs >= 1 && nrhs <= kN;
}

cudaError_t launch_far_tc(const FarTcLevels& L, const int2* work, int nwork, int np2, int nrhs, int* err,
                          cudaStream_t s) {
  if (nwork == 0) return cudaSuccess;
  if (!far_tc_supported(false, np2, nrhs)) return cudaErrorInvalidValue;
  switch (np2) {
    case 4: return launch_np<4>(L, work, nwork, nrhs, err, s);
    case 9: return launch_np<9>(L, work, nwork, nrhs, err, s);
    case 16: return launch_np<16>(L, work, nwork, nrhs, err, s);
    case 25: return launch_np<25>(L, work, nwork, nrhs, err, s);
    case 36: return launch_np<36>(L, work, nwork, nrhs, err, s);
    case 49: return launch_np<49>(L, work, nwork, nrhs, err, s);
    case 64: return launch_np<64>(L, work, nwork, nrhs, err, s);
    case 81: return launch_np<81>(L, work, nwork, nrhs, err, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace bg
