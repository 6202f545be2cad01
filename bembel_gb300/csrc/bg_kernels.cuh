// Kernel interfaces of the GB300 H2 single-layer operator. Implementations in
// bg_nearfield.cu (near-field assembly), bg_farfield.cu (cluster points and
// far-field assembly) and bg_matvec.cu (transforms, block-sparse products,
// the fused FP32 far field and the Krylov vector kernels).
#pragma once
#include <cuda_runtime.h>

#include "bg_device.cuh"

namespace bg {

// Raise the dynamic shared-memory limit of a kernel to at least bytes. The
// limit is one value per kernel for the whole process and launches from
// several host threads (the serving workers) may use different sizes, so it
// only ever grows: lowering it between another thread's call and launch would
// make that launch fail.
cudaError_t raise_smem_limit(const void* func, size_t bytes);
template <typename K>
inline cudaError_t smem_limit(K* func, size_t bytes) {
  return raise_smem_limit(reinterpret_cast<const void*>(func), bytes);
}

// element pair of a dense leaf: output block position dst (scalars) inside
// the dense-block pool; rot packs rot1 | rot2 << 4
struct NearPair {
  int e1, e2, rot, pad;
  long long dst;
};

// element pair of a dense leaf of the Maxwell operator: one destination per
// component pair (rc, cc) at dst[2 * rc + cc]
struct NearPairV {
  int e1, e2, rot, pad;
  long long dst[4];
};

// a Gauss point of the Maxwell quadrature tables: surface point, the two
// tangents of the patch parametrisation and the weight h * w (no surface
// measure: the vector basis carries the Jacobian)
struct MwPt {
  double x[3], dx[3], dy[3], w;
};

struct ElementTable {
  const int* patch;    // per element
  const double* llc;   // 2 per element
  double h;            // element size in patch coordinates
};

// ---- near field ----
// per element e and 2D Gauss point q of an n1 x n1 rule: x, y, z, h*w*|dx x dy|
cudaError_t launch_quad_table(int G, const PatchTable& pt, const ElementTable& et, int ne, const double* gx,
                              const double* gw, int n1, d4* out, cudaStream_t s);
// regular pairs (integrate0 / integrate1 of the DuffyTrick) from quad tables
cudaError_t launch_near_regular(int P, bool cplx, const NearPair* pairs, int npairs, const d4* tab, int n1,
                                const double* basis, double kre, double kim, void* out, int B, cudaStream_t s);
// identical (cs = 2), common edge (3), common vertex (4) pairs
cudaError_t launch_near_duffy(int G, int P, bool cplx, int cs, const PatchTable& pt, const ElementTable& et,
                              const NearPair* pairs, int npairs, const double* gx, const double* gw, int n1,
                              double kre, double kim, void* out, int B, cudaStream_t s);

// Maxwell single layer (Maxwell/SingleLayerOperator.hpp:44-88): the four
// component blocks of every element pair, idiv = -1 / (kappa^2 h^2)
cudaError_t launch_quad_table_mw(int G, const PatchTable& pt, const ElementTable& et, int ne, const double* gx,
                                 const double* gw, int n1, MwPt* out, cudaStream_t s);
// complex (Helmholtz) singular pairs for nk wavenumbers at once
// (1 <= nk <= kDuffyMaxWavenumbers, P = 1 or 2): out[q] receives the blocks of
// wavenumber kre[q] + i kim[q]
constexpr int kDuffyMaxWavenumbers = 4;
cudaError_t launch_near_duffy_multi(int G, int P, int cs, const PatchTable& pt, const ElementTable& et,
                                    const NearPair* pairs, int npairs, const double* gx, const double* gw, int n1,
                                    int nk, const double* kre, const double* kim, void* const* out, int B,
                                    cudaStream_t s);
cudaError_t launch_near_regular_mw(int P, const NearPairV* pairs, int npairs, const MwPt* tab, int n1,
                                   const double* basis3, double kre, double kim, cd idiv, cd* out, int B,
                                   cudaStream_t s);
cudaError_t launch_near_duffy_mw(int G, int P, int cs, const PatchTable& pt, const ElementTable& et,
                                 const NearPairV* pairs, int npairs, const double* gx, const double* gw, int n1,
                                 double kre, double kim, cd idiv, cd* out, int B, cudaStream_t s);

// ---- far field ----
// interpolation points of every cluster of a level: x, y, z, |dx x dy| (FP64 and FP32)
// With tan64 set (Maxwell) the weight is 1 and the two tangents dx, dy of every
// point go to tan64 (6 doubles) and tan32 (6 floats).
cudaError_t launch_cluster_points(int G, const PatchTable& pt, int level, int nclusters, const double* cheb, int np,
                                  const d4* centres, d4* out64, float4* out32, double* tan64, float* tan32,
                                  cudaStream_t s);
// Maxwell far field through the scalar kernel matrix K of each cluster pair
// (Maxwell/SingleLayerOperator.hpp:90-120 couples the tangential parts by
// k t_rc(x).t_cc(y) and the divergence parts by -k / kappa^2). The moments of
// a level are three channels, each [cluster][np2][nrhs]: Yphi_0, Yphi_1 (the
// tangential parts of the two components) and Ydiv (the divergence parts of
// both components summed; the transfers are linear, so the sum is formed at
// the leaves). mw_far_in forms, per cluster point j and right-hand side r of
// the chunk [r0, r0 + nr), the four columns v_q = sum_cc t_cc,q(y_j) Yphi_cc
// (q < 3) and v_3 = Ydiv into Yv ([cluster][np2][4 nr]); mw_far_out maps
// Zv = K Yv back to the channels of Z: Zphi_rc = sum_q t_rc,q(x_i) Zv_q and
// Zdiv = m Zv_3 (shared by both row components).
cudaError_t launch_mw_far_in(int S, int ncl, int np2, const void* y, int nrhs, int r0, int nr, const void* tan,
                             void* yv, cudaStream_t s);
cudaError_t launch_mw_far_out(int S, int ncl, int np2, const void* zv, int nrhs, int r0, int nr, const void* tan,
                              double mre, double mim, void* z, cudaStream_t s);
// F blocks (B x B, column-major) for the listed cluster pairs of one level
// block k written at out + k * bstride scalars
cudaError_t launch_far_assemble(bool cplx, const d4* pts, const int2* pairs, int nblocks, int B, long bstride,
                                double kre, double kim, void* out, cudaStream_t s);

// ---- matvec building blocks (row-major work vectors, nrhs contiguous) ----
// S: 0 double, 1 complex double, 2 float, 3 complex float
cudaError_t launch_csr_apply(int S, const int* ptr, const int* idx, const double* val, int rows, const void* x,
                             void* y, int nrhs, cudaStream_t s);
cudaError_t launch_bsr(int S, const int* row_ptr, const int* col, const void* blocks, int nrows, int B, const void* x,
                       void* y, int nrhs, int accumulate, cudaStream_t s);
// FP64 (cplx: complex FP64) block-sparse product with a cp.async pipeline;
// block k starts at blocks + k * bstride scalars (bstride * sizeof >= 16 B multiple)
cudaError_t launch_bsr_fp64(bool cplx, const int* row_ptr, const int* col, const void* blocks, long bstride, int nrows,
                            int B, const void* x, void* y, int nrhs, int accumulate, cudaStream_t s);
// as launch_moment_fwd, adding to y when acc is set
cudaError_t launch_moment_fwd_acc(int S, bool acc, const void* mom, int R, int Bq, int nclusters, const void* xss,
                                  void* y, int nrhs, cudaStream_t s);
cudaError_t launch_moment_fwd(int S, const void* mom, int R, int Bq, int nclusters, const void* xss, void* y, int nrhs,
                              cudaStream_t s);
cudaError_t launch_moment_bwd(int S, const void* mom, int R, int Bq, int nclusters, const void* z, void* yss, int nrhs,
                              cudaStream_t s);
cudaError_t launch_transfer_fwd(int S, const void* T, int np2, int nc, int nparents, const void* ychild, void* yparent,
                                int nrhs, cudaStream_t s);
cudaError_t launch_transfer_bwd(int S, const void* T, int np2, int nc, int nparents, const void* zparent, void* zchild,
                                int nrhs, cudaStream_t s);
// fused FP32 far field: for each listed block, generate the coupling from
// cluster points on the fly and accumulate into the row cluster's output
// (points are FP32 offsets from the FP64 cluster centres)
// Per-level tables of the tensor-core far-field product (one launch for all
// FMM levels). y/z: FP32 coefficient blocks [cluster][n_p^2][nrhs].
constexpr int kMaxFarLevels = 12;
struct FarTcLevels {
  const int* row_ptr[kMaxFarLevels];
  const int* col[kMaxFarLevels];
  const float4* pts[kMaxFarLevels];
  const d4* cen[kMaxFarLevels];
  const float* y[kMaxFarLevels];
  float* z[kMaxFarLevels];
};
// Stored-tile far field, per level: the low-rank blocks' scaled FP16 hi/lo
// tiles (a) and their inverse scales (ainv, one per block), the right-hand-side
// tiles of every cluster (b) and inverse column scales (binv, 32 per cluster),
// both rebuilt per product from y by launch_build_h16_btiles, the product's
// output (z) and the cluster count (ncl). A "level" here may also be one
// level of one wavenumber of a batch (index q (L + 1) + l), hence the larger
// bound (the structure is a kernel parameter of about 4.4 KB).
constexpr int kMaxTileLevels = 64;
struct FarH16Tiles {
  const int* row_ptr[kMaxTileLevels];
  const int* col[kMaxTileLevels];
  const unsigned char* a[kMaxTileLevels];
  const float* ainv[kMaxTileLevels];
  unsigned char* b[kMaxTileLevels];
  float* binv[kMaxTileLevels];
  const float* y[kMaxTileLevels];
  float* z[kMaxTileLevels];
  int ncl[kMaxTileLevels];
};
size_t far_h16_atile_bytes(int np2);  // per low-rank block (0: shape not supported)
size_t far_h16_btile_bytes(int np2);  // per cluster
cudaError_t launch_build_h16_atiles(int np2, const double* F, long bstride, long nblocks, void* tiles, float* ainv,
                                    cudaStream_t s);
cudaError_t launch_build_h16_btiles(const FarH16Tiles& T, int nlev, int np2, int nrhs, cudaStream_t s);
// ctas_per_sm: 1 one CTA of four stages per SM, 2 two CTAs of two stages,
// otherwise the built-in choice (2 when there are at least 2 x SMs rows)
// hi_only: the FP16 hi coupling tiles only (two products per block instead of three)
cudaError_t launch_far_h16(const FarH16Tiles& T, const int2* work, int nwork, int np2, int nrhs, int* err,
                           cudaStream_t s, int ctas_per_sm = 0, bool hi_only = false);
// watchdog self-test: a bounded wait that cannot complete; sets *err = 99 when it runs out
cudaError_t launch_wait_selftest(long long limit_cycles, int* err, cudaStream_t s);
// real kernels, n_p^2 <= 128 within the shared-memory limit, nrhs <= 32
bool far_tc_supported(bool cplx, int np2, int nrhs);
// Complex kernels (Helmholtz, Maxwell): a holds [Re hi][Re lo][Im hi][Im lo]
// per block (built from complex FP64 blocks), b a real tile pair of 32 columns
// per cluster ([Re Y | Im Y] of up to 16 complex columns y0 .. y0 + nc - 1 of
// rows with ldy entries); the product writes columns z0 .. z0 + nc - 1 of z
// (rows of ldz complex entries). n_p^2 in {4, 9, ..., 81, 100}.
size_t far_h16c_atile_bytes(int np2);  // per low-rank block (0: shape not supported)
size_t far_h16c_btile_bytes(int np2);  // per cluster
cudaError_t launch_build_h16c_atiles(int np2, const void* F, long bstride, long nblocks, void* tiles, float* ainv,
                                     cudaStream_t s);
cudaError_t launch_build_h16c_btiles(const FarH16Tiles& T, int nlev, int np2, int ldy, int y0, int nc,
                                     cudaStream_t s);
cudaError_t launch_far_h16c(const FarH16Tiles& T, const int2* work, int nwork, int np2, int ldz, int z0, int nc,
                            int* err, cudaStream_t s);

// work: (level, row) per CTA, every row of every level in L exactly once;
// err: set to a nonzero code if a bounded wait of the kernel ran out
cudaError_t launch_far_tc(const FarTcLevels& L, const int2* work, int nwork, int np2, int nrhs, int* err,
                          cudaStream_t s);
cudaError_t launch_far_fused(bool cplx, const float4* pts, const d4* centres, const int* row_ptr, const int* col,
                             int nrows, int np2, float kre, float kim, const void* y, void* z, int nrhs, cudaStream_t s);
// user column-major block (ld) <-> row-major work vector, with precision change
cudaError_t launch_gather_in(int Sin, int Sout, const void* user, long ld, int rows, int nrhs, void* work,
                             cudaStream_t s);
cudaError_t launch_scatter_out(int Swork, const void* work, int rows, int nrhs, void* user, long ld, const double* alpha,
                               const double* beta, cudaStream_t s);
// Double-float product of real FP64 blocks stored as FP32 (hi, lo) pairs
// (launch_split_df), FP64 x and y; bstride in pairs, even
cudaError_t launch_bsr_df(const int* row_ptr, const int* col, const void* blocks, long bstride, int nrows, int B,
                          const void* x, void* y, int nrhs, int accumulate, cudaStream_t s);
// out[t] = (hi, lo) of in[t] (FP64), t < n
cudaError_t launch_split_df(const void* in, long n, void* out, cudaStream_t s);
// FP64-accurate near field on the tensor cores (bg_near_tc.cu) for real
// operators with leaf blocks of B = 4, 16 or 36 rows: oz_supported(B);
// bytes of the digit tiles of nblocks blocks and of the x digit panels of
// nclusters clusters; launch_oz_build turns the FP64 blocks (column-major,
// stride bstride) into row exponents rexp [nrows * B] and digit tiles;
// launch_near_oz writes y (rows of ldy entries, nrhs columns) = A x for x
// FP64 [xrows][ldx], panels and fmax (32 ints) its scratch, err the bounded
// waits' flag
bool oz_supported(int B);
size_t oz_tile_bytes(int B, long nblocks);
size_t oz_panel_bytes(int B, long nclusters);
cudaError_t launch_oz_build(const int* row_ptr, const double* blocks, long bstride, int nrows, int B, int* rexp,
                            void* tiles, long nblocks, cudaStream_t s);
cudaError_t launch_near_oz(const int* row_ptr, const int* col, int nrows, int B, const void* tiles,
                           const int* rexp, const double* x, long xrows, int ldx, void* panels, int* fmax,
                           double* y, int ldy, int nrhs, int* err, cudaStream_t s);
// FP64-accurate near field of real operators for exactly 32 right-hand
// sides (B <= 42): columns 0 .. 23 in double-float from the (hi, lo) pairs
// and the split x, columns 24 .. 31 in FP64 from blocks64 and x64 (row-major
// [rows][32], 16-byte aligned); y written (not accumulated)
cudaError_t launch_bsr_near_mix(const int* row_ptr, const int* col, const void* pairs, const void* blocks64,
                                long bstride, int nrows, int B, const void* xdf, const void* x64, void* y,
                                cudaStream_t s);
// as launch_bsr_df, writing columns y0 .. y0 + nrhs - 1 of y rows of ldy entries
cudaError_t launch_bsr_df_cols(const int* row_ptr, const int* col, const void* blocks, long bstride, int nrows, int B,
                               const void* x, void* y, int nrhs, int ldy, int y0, int accumulate, cudaStream_t s);
// Complex double-float product, Re y + i Im y = Kr split(x) + Ki split(i x) with
// complex columns seen as interleaved real pairs: the column split of x (times
// 1 or times i) and the split of complex blocks into Kr pairs followed by Ki pairs
cudaError_t launch_split_df_cols(const void* in, long rows, int ld, int c0, int nc, int times_i, void* out,
                                 cudaStream_t s);
cudaError_t launch_split_df_cplx_blocks(const void* in, long sin, long B2, long nblocks, long sout, void* out,
                                        cudaStream_t s);
// Fused FMM transforms through the tensor-product factors (bg_fmm.cu).
// fac: [E0 np x np][E1 np x np][Ms np x w1][Mt np x w1] with E_h[c][p] the
// parent polynomial p at child point c of half h, Ms / Mt the 1-D moments;
// cmap[q] = a | (b << 8): the (s, t) 1-D moment columns of superspace row q of
// a leaf cluster (Bq = w1^2 rows). y[l] / z[l]: coefficients of level l
// ([cluster][np^2][kk]); x / out: superspace panels ([leaf cluster][Bq][kk]),
// out accumulated. cnt: arrival counters of the upward pass, zero between
// launches, at cnt_off[l] + chunk * cnt_stride + parent for parents at levels
// 0 .. L - 2 and column chunks of 32.
constexpr int kFmmMaxNp = 12;
template <typename T>
struct FmmLevels {
  const T* fac;
  const int* cmap;
  const T* x;
  T* out;
  T* y[kMaxFarLevels];
  const T* z[kMaxFarLevels];
  int* cnt;
  long cnt_off[kMaxFarLevels];
  long cnt_stride;
  int np, w1, Bq, L, kk;
};
struct FmmLevelsAny {
  FmmLevels<double> f64;
  FmmLevels<float> f32;
};
// upward pass (moments of the leaf clusters, transfers to level 0) and
// downward pass (transposed transfers, transposed moments added to out);
// nparents = clusters of level L - 1; S the bg vector type of the pass;
// hfac the factors on the host (FP64, layout of fac) for the compiled sizes,
// whose kernels take them as launch parameters (nullptr: generic kernels)
cudaError_t launch_fmm_up(int S, const FmmLevelsAny& a, const double* hfac, int nparents, cudaStream_t s);
cudaError_t launch_fmm_down(int S, const FmmLevelsAny& a, const double* hfac, int nparents, cudaStream_t s);
// op(A) of an FMM transform, stored transposed: AT[q][i], q < Ki, i < ld
// (ld a multiple of 4, at least Mo rounded up to 3, zero beyond Mo)
struct TGemmA {
  const void* at;
  int ld, Mo, Ki;
};
// C[b] (=, += if acc) op(A) B[b] for nbatch items; B[b] = B + b * bstride_rows
// rows of the vector type S (bg stype), C likewise; nrhs columns. FP32
// launches of at most split_k_batches CTAs (-1: 152) use the split-K kernel.
cudaError_t launch_tgemm(int S, bool acc, const TGemmA& A, const void* B, long bstride_rows, void* C,
                         long cstride_rows, int nbatch, int nrhs, cudaStream_t s, int split_k_batches = -1);
// FP32 / complex-FP32 blocks; same layout rules as launch_bsr_fp64. variant
// (bg_launch_plan::near_kernel): 0 built-in, 1 pipelined, 2 register tiles
// (complex: 2 rows per thread), 3 complex tiles of 4 rows
cudaError_t launch_bsr_fp32(bool cplx, const int* row_ptr, const int* col, const void* blocks, long bstride, int nrows,
                            int B, const void* x, void* y, int nrhs, int accumulate, cudaStream_t s, int variant = 0);
// out[b*sout + e] = (FP32) in[b*sin + e], e < B2, b < nblocks
cudaError_t launch_convert_blocks(bool cplx, const void* in, long sin, void* out, long sout, long B2, long nblocks,
                                  cudaStream_t s);
cudaError_t launch_convert(int Sin, int Sout, const void* in, long n, void* out, cudaStream_t s);
// out64[t] += (FP64) in32[t]
cudaError_t launch_add_low(bool cplx, const void* in32, long n, void* out64, cudaStream_t s);

}  // namespace bg
