// bg_matvec_noalloc: one H2 product y = A x that allocates no device memory.
//
// Some callers of this library may not call cudaMalloc at the time they need a
// product: a host that hands the library a fixed memory budget up front and
// counts every allocation, code running inside a stream-ordered or pooled
// allocator it must not disturb, or a serving loop that forbids allocation
// after warm-up (an allocation can synchronise the device and stall every
// other stream on it). bg_matvec grows per-operator work vectors on demand, so
// it may allocate on its first call with a new right-hand-side count; this
// entry point instead takes all its intermediate vectors from one fixed
// device array that lives in this file and exists for the life of the process.
//
// Limits and rules (also stated at the declaration in bembel_gb300.h):
//  - one right-hand side per call, x and y device pointers of N scalars;
//  - the intermediate vectors must fit kNoallocScratchBytes (16 MiB); larger
//    operators are rejected with BG_INVALID_ARG before any device work;
//  - every call, from any context or thread, shares the one array per device:
//    calls that overlap on the GPU race and give wrong results;
//  - the first call on a device looks the array's device address up
//    (cudaGetSymbolAddress) and caches it; make that first call before any
//    stream capture. The cached address belongs to the device's primary
//    context, the one the CUDA runtime uses: after cudaDeviceReset on that
//    device it is stale, so do not call this entry point after a reset;
//  - the call selects the operator's device for its duration and restores
//    the caller's current device before it returns.
// Nothing in the array needs to start at zero: every buffer carved from it is
// fully written before it is read, and the FP32 accumulator of the mixed path
// is cleared with cudaMemsetAsync on each call.
//
// The FP64 far field follows bg_matvec: real operators multiply the
// double-float (hi, lo) copies of the couplings when they exist, complex ones
// the split real and imaginary pairs, and only operators without those copies
// read the FP64 blocks. Operators assembled with keep_fp64_blocks = 0 (as the
// serving cache builds them) have released the FP64 blocks and always take
// the double-float route; an operator holding neither is refused with
// BG_UNSUPPORTED before any device work.
#include <cstdint>
#include <mutex>

#include "bg_operator.hpp"

using namespace bg;

namespace {

constexpr size_t kNoallocScratchBytes = size_t(16) << 20;
constexpr int kMaxDevices = 64;

// Every GPU that loads the library holds this array until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

std::mutex g_scratch_mutex;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on `device` (which must be current).
// In host code the array's name only stands for the symbol; its device
// address comes from the runtime.
cudaError_t scratch_address(int device, void** out) {
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_addr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[device] = p;
  }
  *out = g_scratch_addr[device];
  return cudaSuccess;
}

size_t round256(size_t n) { return (n + 255) & ~size_t(255); }

// Carving of the scratch array for one right-hand side.
struct ScratchPlan {
  size_t xss = 0, yss = 0, xss32 = 0, yss32 = 0;
  std::vector<size_t> y, z;  // per FMM level
  std::vector<size_t> ydf;   // per FMM level: double-float split of y (FP64 product on the pairs)
  size_t total = 0;
};

bool has_far(const bg_operator* op) {
  for (const auto& f : op->far)
    if (!f.col.empty()) return true;
  return false;
}

ScratchPlan plan_scratch(const bg_operator* op, bool mixed) {
  ScratchPlan sp;
  const size_t sb = op->scalar_bytes(false);
  size_t off = 0;
  auto take = [&](size_t n) {
    const size_t at = off;
    off += round256(n);
    return at;
  };
  sp.xss = take((size_t)op->S * sb);
  sp.yss = take((size_t)op->S * sb);
  if (has_far(op)) {
    if (mixed) {
      sp.xss32 = take((size_t)op->S * sb / 2);
      sp.yss32 = take((size_t)op->S * sb / 2);
    }
    const size_t fsb = op->scalar_bytes(mixed);
    for (int l = 0; l <= op->leaf_level; ++l) {
      const size_t n = (size_t)op->vd * op->nclusters(l) * op->R * fsb;
      sp.y.push_back(take(n));
      sp.z.push_back(take(n));
      // one (hi, lo) float pair per real entry of y: one pair for a real
      // coupling column, two (re, im) for a complex one
      // (the size check runs before the assembled check, so the per-level
      // buffers may not exist yet)
      const bool df = !mixed && !op->far[l].col.empty() && l < (int)op->d_far_df.size() && op->d_far_df[l]->p;
      const size_t ndf = df ? (size_t)op->nclusters(l) * op->R * (op->cplx ? 2 : 1) * sizeof(float2) : 0;
      sp.ydf.push_back(ndf ? take(ndf) : 0);
    }
  }
  sp.total = off;
  return sp;
}

}  // namespace

#define NA_CHECK(expr, what)                              \
  do {                                                    \
    bg_status _st = cuda_status(op->ctx, (expr), (what)); \
    if (_st != BG_OK) return _st;                         \
  } while (0)

// y = A x for one right-hand side with every intermediate vector in the
// scratch array; the launch sequence is the one of the multi-column product
// (H2DenseProduct.hpp:33-165): T x, near field, forward transforms, far field
// per level, backward transforms, T^T.
static bg_status product_in_scratch(bg_operator* op, bool mixed, const ScratchPlan& sp, char* base, const void* x,
                                    void* y) {
  cudaStream_t s = op->ctx->stream;
  const int S64 = op->stype(false), Sfar = op->stype(mixed);
  const size_t sfar = op->scalar_bytes(mixed);
  const int np2 = op->np * op->np;
  const long ss_n = op->S;
  void* xss = base + sp.xss;
  void* yss = base + sp.yss;
  NA_CHECK(launch_csr_apply(S64, op->d_T_ptr.as<int>(), op->d_T_idx.as<int>(), op->d_T_val.as<double>(), op->S, x,
                            xss, 1, s),
           "T x");
  NA_CHECK(launch_bsr_fp64(op->cplx, op->dense.d_row_ptr.as<int>(), op->dense.d_col.as<int>(), op->d_dense64.p,
                           op->block_stride(op->dense.B), op->dense.nrows, op->dense.B, xss, yss, 1, 0, s),
           "near-field product");
  if (!sp.y.empty()) {
    const long comp_ss = (long)op->ne * op->p2;
    const void* xfar = xss;
    void* yfar = yss;
    if (mixed) {
      if (op->vd != 1 || op->nc != 1) return set_error(op->ctx, BG_UNSUPPORTED, "mixed far field of vector operators");
      NA_CHECK(launch_convert(S64, Sfar, xss, ss_n, base + sp.xss32, s), "x to FP32");
      NA_CHECK(cudaMemsetAsync(base + sp.yss32, 0, ss_n * sfar, s), "far field");
      xfar = base + sp.xss32;
      yfar = base + sp.yss32;
    } else if (!op->store_far) {
      return set_error(op->ctx, BG_UNSUPPORTED, "the FP64 product needs the stored far field");
    }
    const int Ll = op->leaf_level;
    auto Y = [&](int l) { return base + sp.y[l]; };
    auto Z = [&](int l) { return base + sp.z[l]; };
    for (int c = 0; c < op->vd; ++c) {
      const void* mom = mixed ? op->d_mom32[c]->p : op->d_mom64[c]->p;
      NA_CHECK(launch_moment_fwd(Sfar, mom, op->R, op->Bq, op->nleaf_cl,
                                 static_cast<const char*>(xfar) + c * comp_ss * sfar,
                                 Y(Ll) + (size_t)c * op->nleaf_cl * op->R * sfar, 1, s),
               "forward moments");
      for (int l = Ll - 1; l >= 0; --l) {
        const int ncl = op->nclusters(l);
        NA_CHECK(launch_transfer_fwd(Sfar, mixed ? op->d_tr32.p : op->d_tr64.p, np2, op->nc, ncl,
                                     Y(l + 1) + (size_t)c * 4 * ncl * op->R * sfar,
                                     Y(l) + (size_t)c * ncl * op->R * sfar, 1, s),
                 "forward transfer");
      }
    }
    for (int l = 0; l <= Ll; ++l) {
      const BsrSegment& f = op->far[l];
      if (f.col.empty()) {
        NA_CHECK(cudaMemsetAsync(Z(l), 0, (size_t)f.nrows * f.B * sfar, s), "far field");
        continue;
      }
      if (mixed)
        NA_CHECK(launch_far_fused(op->cplx, op->d_pts32[l]->as<float4>(), op->d_centres[l]->as<d4>(),
                                  f.d_row_ptr.as<int>(), f.d_col.as<int>(), f.nrows, np2, (float)op->kre,
                                  (float)op->kim, Y(l), Z(l), 1, s),
                 "far-field product (FP32 fused)");
      else if (op->d_far_df[l]->p && op->cplx) {
        // Re K split(y) + Im K split(i y), the second pass accumulating
        const long sdf = ((long)f.B * f.B + 1) / 2 * 2;
        const float2* kr = op->d_far_df[l]->as<float2>();
        const float2* ki = kr + (long)f.col.size() * sdf;
        const long rows = (long)op->nclusters(l) * f.B;
        for (int part = 0; part < 2; ++part) {
          NA_CHECK(launch_split_df_cols(Y(l), rows, 1, 0, 1, part, base + sp.ydf[l], s), "far-field split of Y");
          NA_CHECK(launch_bsr_df_cols(f.d_row_ptr.as<int>(), f.d_col.as<int>(), part ? ki : kr, sdf, f.nrows, f.B,
                                      base + sp.ydf[l], Z(l), 2, 2, 0, part, s),
                   "far-field product (complex double-float)");
        }
      } else if (op->d_far_df[l]->p) {
        NA_CHECK(launch_split_df(Y(l), (long)op->nclusters(l) * op->R, base + sp.ydf[l], s), "far-field split of Y");
        NA_CHECK(launch_bsr_df(f.d_row_ptr.as<int>(), f.d_col.as<int>(), op->d_far_df[l]->p, op->block_stride(f.B),
                               f.nrows, f.B, base + sp.ydf[l], Z(l), 1, 0, s),
                 "far-field product (double-float)");
      } else {
        NA_CHECK(launch_bsr_fp64(op->cplx, f.d_row_ptr.as<int>(), f.d_col.as<int>(), op->d_far64[l]->p,
                                 op->block_stride(f.B), f.nrows, f.B, Y(l), Z(l), 1, 0, s),
                 "far-field product");
      }
    }
    for (int c = 0; c < op->vd; ++c) {
      for (int l = 0; l < Ll; ++l) {
        const int ncl = op->nclusters(l);
        NA_CHECK(launch_transfer_bwd(Sfar, mixed ? op->d_tr32.p : op->d_tr64.p, np2, op->nc, ncl,
                                     Z(l) + (size_t)c * ncl * op->R * sfar,
                                     Z(l + 1) + (size_t)c * 4 * ncl * op->R * sfar, 1, s),
                 "backward transfer");
      }
      const void* mom = mixed ? op->d_mom32[c]->p : op->d_mom64[c]->p;
      NA_CHECK(launch_moment_bwd(Sfar, mom, op->R, op->Bq, op->nleaf_cl,
                                 Z(Ll) + (size_t)c * op->nleaf_cl * op->R * sfar,
                                 static_cast<char*>(yfar) + c * comp_ss * sfar, 1, s),
               "backward moments");
    }
    if (mixed) NA_CHECK(launch_add_low(op->cplx, base + sp.yss32, ss_n, yss, s), "far field to FP64");
  }
  NA_CHECK(launch_csr_apply(S64, op->d_Tt_ptr.as<int>(), op->d_Tt_idx.as<int>(), op->d_Tt_val.as<double>(), op->N,
                            yss, y, 1, s),
           "T^T y");
  return BG_OK;
}

extern "C" bg_status bg_matvec_noalloc(bg_operator* op, const void* x, void* y, int precision) {
  if (!op || !x || !y) return BG_INVALID_ARG;
  if (op->ctx->device < 0) return set_error(op->ctx, BG_UNSUPPORTED, "host-only context: products need a GPU");
  if (op->ctx->device >= kMaxDevices) return set_error(op->ctx, BG_UNSUPPORTED, "device ordinal too large");
  if (precision != BG_PREC_FP64 && precision != BG_PREC_MIXED) return set_error(op->ctx, BG_INVALID_ARG, "precision");
  if (op->maxwell())
    return set_error(op->ctx, BG_UNSUPPORTED, "bg_matvec_noalloc: the Maxwell operator is not supported; use bg_matvec");
  if (op->kbatched())
    return set_error(op->ctx, BG_UNSUPPORTED, "bg_matvec_noalloc: batched wavenumbers are not supported; use bg_matvec");
  const bool mixed = precision == BG_PREC_MIXED;
  const ScratchPlan sp = plan_scratch(op, mixed);
  if (sp.total > kNoallocScratchBytes)
    return set_error(op->ctx, BG_INVALID_ARG,
                     "bg_matvec_noalloc: operator needs " + std::to_string(sp.total) +
                         " bytes of scratch, above the fixed maximum of " + std::to_string(kNoallocScratchBytes) +
                         " bytes (16 MiB); use bg_matvec");
  if (!op->assembled) return set_error(op->ctx, BG_INVALID_ARG, "operator not assembled");
  const uintptr_t align = op->cplx ? 16 : 8;
  if (reinterpret_cast<uintptr_t>(x) % align || reinterpret_cast<uintptr_t>(y) % align)
    return set_error(op->ctx, BG_INVALID_ARG, "bg_matvec_noalloc: x and y must be aligned to their scalar type");
  if (!mixed && has_far(op))
    for (int l = 0; l <= op->leaf_level; ++l)
      if (!op->far[l].col.empty() && !op->d_far_df[l]->p && !op->d_far64[l]->p)
        return set_error(op->ctx, BG_UNSUPPORTED,
                         "bg_matvec_noalloc: the FP64 product needs the stored far field (FP64 blocks or their "
                         "double-float copies); use bg_matvec");
  int caller_device = -1;
  NA_CHECK(cudaGetDevice(&caller_device), "current device");
  NA_CHECK(cudaSetDevice(op->ctx->device), "select device");
  void* scratch = nullptr;
  bg_status st = cuda_status(op->ctx, scratch_address(op->ctx->device, &scratch),
                             "scratch address (cudaGetSymbolAddress)");
  if (st == BG_OK) st = product_in_scratch(op, mixed, sp, static_cast<char*>(scratch), x, y);
  if (st == BG_OK) st = cuda_status(op->ctx, cudaStreamSynchronize(op->ctx->stream), "H2 matvec (no allocation)");
  // the caller's device comes back whatever happened above
  const cudaError_t back = cudaSetDevice(caller_device);
  if (st == BG_OK) st = cuda_status(op->ctx, back, "restore the caller's device");
  return st;
}
