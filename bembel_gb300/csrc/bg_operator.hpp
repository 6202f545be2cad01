// Operator state shared by the C-ABI translation units.
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <set>
#include <string>
#include <vector>

#include "../../include/bembel_gb300.h"
#include "bg_host.hpp"
#include "bg_kernels.cuh"

// owning device allocation
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() {}
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), bytes(o.bytes) {
    o.p = nullptr;
    o.bytes = 0;
  }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      release();
      p = o.p;
      bytes = o.bytes;
      o.p = nullptr;
      o.bytes = 0;
    }
    return *this;
  }
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  cudaError_t alloc(size_t n) {
    if (n <= bytes && p) return cudaSuccess;
    release();
    if (n == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc(&p, n);
    if (e == cudaSuccess) bytes = n;
    else p = nullptr;
    return e;
  }
  template <typename T>
  cudaError_t upload(const std::vector<T>& v, cudaStream_t s) {
    cudaError_t e = alloc(v.size() * sizeof(T));
    if (e != cudaSuccess || v.empty()) return e;
    return cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s);
  }
  template <typename T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

struct bg_context {
  int device = -1;  // -1: host-only context (setup and inspection, no device work)
  int children = 0;      // live geometries and operators
  bool closing = false;  // bg_context_destroy was called; free with the last child
  cudaStream_t stream = nullptr;
  std::string err;
  DevBuf stage_in, stage_out;   // device staging of host operands
  void* pinned = nullptr;       // pinned host staging
  size_t pinned_bytes = 0;
  // kernel-class timing with CUDA events on `stream` (bg_profile)
  bool profiling = false;
  unsigned profile_mask = 0xFFu;  // kernel classes bracketed with events while profiling
  long launches = 0;
  std::vector<cudaEvent_t> event_pool;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending[8];
  double class_ms[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  long class_launches[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  cudaEvent_t get_event() {
    if (event_pool.empty()) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      return e;
    }
    cudaEvent_t e = event_pool.back();
    event_pool.pop_back();
    return e;
  }
};

// kernel classes reported by bg_profile_read
enum { KC_NEAR = 0, KC_FAR64 = 1, KC_FAR_FUSED = 2, KC_TRANSFORM = 3, KC_TAPPLY = 4, KC_KRYLOV = 5, KC_OTHER = 6,
       KC_ASSEMBLY = 7 };

// launch f() on ctx->stream, counting it and, when profiling, bracketing it
// with events of class cls
template <typename F>
cudaError_t timed_launch(bg_context* ctx, int cls, F&& f) {
  ++ctx->launches;
  ++ctx->class_launches[cls];
  if (!ctx->profiling || !(ctx->profile_mask & (1u << cls))) return f();
  cudaEvent_t a = ctx->get_event(), b = ctx->get_event();
  cudaEventRecord(a, ctx->stream);
  cudaError_t e = f();
  cudaEventRecord(b, ctx->stream);
  ctx->pending[cls].push_back({a, b});
  return e;
}

struct bg_geometry {
  bg::Geometry g;
  bg_context* ctx = nullptr;
};

// block-sparse row structure of one segment (dense leaves or one far level)
struct BsrSegment {
  int nrows = 0;   // block rows (component-major: rc * nclusters + c)
  int B = 0;       // block size
  std::vector<int> row_ptr, col;
  std::vector<int> leaf;  // leaf index (into the partition's leaf list) per block
  std::vector<int> comp;  // rc * vd + cc per block
  DevBuf d_row_ptr, d_col;
};

struct bg_operator {
  bg_context* ctx = nullptr;
  int kind = 0, M = 0, P = 0, vd = 1, nc = 1, np = 9, mcl = 1, G = 2;
  double eta = 1.6;
  bool cplx = false, store_far = true;
  double kre = 0.0, kim = 0.0;
  bg::Geometry geo;
  bg::Mesh mesh;
  bg::Partition part;
  bg::Csr T, Tt;
  int p2 = 1, ne = 0, S = 0, N = 0;
  int leaf_level = 0;       // FMM leaf cluster level (M - mcl, or 0)
  int nleaf_cl = 0;         // clusters at the leaf level
  int Bq = 0;               // superspace rows per FMM leaf cluster (4^mcl p^2)
  int R = 0;                // rows per cluster coefficient block (nc np^2)
  BsrSegment dense;
  std::vector<BsrSegment> far;  // per level 0..leaf_level
  long near_pairs = 0;
  bool assembled = false;
  double t_near = 0, t_far = 0, t_total = 0;
  double t_prepare = 0;  // seconds of the last bg_operator_prepare_wavenumbers
  // near fields prepared for several wavenumbers in one pass
  // (bg_operator_prepare_wavenumbers); bg_operator_assemble copies the one of
  // the current wavenumber instead of running the quadrature
  struct NearCacheEntry {
    double kre, kim;
    DevBuf* blocks;
  };
  std::vector<NearCacheEntry> near_cache;

  // Several wavenumbers assembled side by side (bg_operator_assemble_wavenumbers):
  // slot q holds wavenumber q's near field, far field and tensor-core tiles.
  // While no slot is active, products, load vectors, potentials and solves
  // take nslots column blocks of equal width and apply slot q to block q, by
  // swapping the slot's fields into the operator's (activate_slot).
  struct KSlot {
    double kre = 0.0, kim = 0.0;
    DevBuf dense64, dense32;
    std::vector<DevBuf*> far64, far_df, atiles, ainv;
    bool far_tiles = false;
  };
  std::vector<KSlot> kslots;
  int kslot_active = -1;
  DevBuf w_kx, w_ky;  // one column block of a batched product (row-major dof vectors)
  // the batched product in one pass over all wavenumbers (kb_nwork > 0): per
  // (wavenumber q, level l), index q (leaf_level + 1) + l, the right-hand-side
  // tiles of the tensor-core far field; its work list over those indexes;
  // superspace column blocks for the per-wavenumber near fields
  std::vector<DevBuf*> kb_btiles, kb_binv;
  DevBuf kb_work, kb_xs, kb_ys;
  int kb_nwork = 0;
  bool kbatched() const { return !kslots.empty() && kslot_active < 0; }
  void swap_slot(int q) {
    KSlot& k = kslots[q];
    std::swap(kre, k.kre);
    std::swap(kim, k.kim);
    std::swap(d_dense64, k.dense64);
    std::swap(d_dense32, k.dense32);
    std::swap(d_far64, k.far64);
    std::swap(d_far_df, k.far_df);
    std::swap(d_far_atiles, k.atiles);
    std::swap(d_far_ainv, k.ainv);
    std::swap(far_tiles, k.far_tiles);
  }
  void activate_slot(int q) {
    if (q == kslot_active) return;
    if (kslot_active >= 0) swap_slot(kslot_active);
    if (q >= 0) swap_slot(q);
    kslot_active = q;
  }
  void free_slots() {
    activate_slot(-1);
    for (auto& k : kslots)
      for (auto v : {&k.far64, &k.far_df, &k.atiles, &k.ainv})
        for (auto b : *v) delete b;
    kslots.clear();
    for (auto v : {&kb_btiles, &kb_binv}) {
      for (auto b : *v) delete b;
      v->clear();
    }
    kb_work.release();
    kb_xs.release();
    kb_ys.release();
    kb_nwork = 0;
  }

  // device tables
  DevBuf d_patch_meta, d_patch_cp, d_el_patch, d_el_llc;
  DevBuf d_T_ptr, d_T_idx, d_T_val, d_Tt_ptr, d_Tt_idx, d_Tt_val;
  DevBuf d_cheb;
  std::vector<DevBuf*> d_pts64, d_pts32, d_centres;  // per level
  std::vector<DevBuf*> d_tan64, d_tan32;             // per level, Maxwell: tangents dx, dy of every point
  DevBuf d_dense64;                       // dense blocks (FP64)
  DevBuf d_dense32;                       // FP32 copy of the dense blocks (BG_PREC_FP32)
  DevBuf d_dense_df;                      // real operators: FP32 (hi, lo) pairs of the dense blocks, the
                                          // near field of BG_PREC_MIXED products (double-float, FP64 accuracy)
  // real operators, leaf blocks of 4, 16 or 36 rows: the near field as 8
  // FP16 integer digits per entry in tensor-core tiles (bg_near_tc.cu), the
  // exponent of every block-row row, and the per-product x digit panels and
  // column exponents
  DevBuf d_oz_tiles, d_oz_rexp, w_oz_panels, w_oz_fmax;
  std::vector<DevBuf*> d_far64;           // per level
  std::vector<DevBuf*> d_far_df;          // per level: FP32 (hi, lo) pairs of d_far64 (real operators)
  std::vector<DevBuf*> d_far_atiles;      // per level: FP16 hi/lo tensor-core tiles of the low-rank blocks
  std::vector<DevBuf*> d_far_ainv;        // per level: inverse power-of-two scale of every tile
  bool far_tiles = false;                 // every far-field level has its tiles
  bool keep_far64 = true;                 // keep d_far64 after assembly (else released)
  std::vector<DevBuf*> d_mom64, d_mom32;  // per vector component
  DevBuf d_tr64, d_tr32;
  // FMM matrices transposed and padded for launch_tgemm, per precision
  // (0 FP64, 1 FP32): moments forward/backward per component, transfers
  // Maxwell: the np^2 x Bq moment blocks phi, d/ds phi, d/dt phi of the
  // three transform channels (forward and backward)
  struct TransformMats {
    DevBuf mom_f[2], mom_b[2], tr_f, tr_b, mw_f[3], mw_b[3];
    bg::TGemmA a_mom_f[2], a_mom_b[2], a_tr_f, a_tr_b, a_mw_f[3], a_mw_b[3];
  };
  TransformMats tm[2];
  bool use_tgemm = false;
  // fused FMM transforms through the tensor-product factors (scalar
  // operators): factors per precision ([E0|E1|Ms|Mt]), the superspace-row map
  // of a leaf cluster, and the upward pass's arrival counters (zero between
  // launches; fmm_cnt_chunks column chunks of 32)
  bool fmm_fused = false;
  int fmm_w1 = 0;
  DevBuf d_fmm_fac64, d_fmm_fac32, d_fmm_cmap, d_fmm_cnt;
  std::vector<double> fmm_hfac;  // the same factors on the host (launch parameters of the compiled sizes)
  long fmm_cnt_off[bg::kMaxFarLevels] = {};
  long fmm_cnt_stride = 0;
  int fmm_cnt_chunks = 0;
  // tensor-core far field: (level, row) work list, heaviest rows first, and
  // the two alternative orders of bg_launch_plan::far_order (built only when
  // there are more rows than persistent CTAs)
  DevBuf d_far_work;
  DevBuf d_far_work_alt[2];
  int n_far_work = 0;
  const int2* far_work(int order) const {
    if ((order == 1 || order == 2) && d_far_work_alt[order - 1].p) return d_far_work_alt[order - 1].as<int2>();
    return d_far_work.as<int2>();
  }
  DevBuf d_err;  // int: nonzero after a bounded device wait ran out
  // work vectors (sized for the largest nrhs seen)
  int cap = 0;
  DevBuf w_xdof, w_xss, w_yss, w_ydof, w_xss32, w_yss32;
  DevBuf w_xss_df;                // real operators: FP32 (hi, lo) split of w_xss for the double-float near field
  std::vector<DevBuf*> w_y, w_z;  // per level
  std::vector<DevBuf*> w_ydf;     // per level: FP32 (hi, lo) split of w_y for the double-float product
  std::vector<DevBuf*> w_yv, w_zv;  // per level, Maxwell: the four kernel columns per right-hand side
  std::vector<DevBuf*> w_btiles;  // per level: FP16 hi/lo right-hand-side tiles of every cluster
  std::vector<DevBuf*> w_binv;    // per level: inverse column scales of those tiles (32 per cluster)

  // CUDA graphs of the product's middle part, per (nrhs, precision)
  struct ProductGraph {
    cudaGraphExec_t exec = nullptr;
    long launches = 0;
    long class_launches[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  };
  std::map<long, ProductGraph> graphs;
  std::set<long> graph_seen;  // shapes run once directly (captured on the next product)
  bool use_graphs = true;
  void drop_graphs() {
    for (auto& kv : graphs)
      if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
    graphs.clear();
    graph_seen.clear();
  }

  // launch plans per (nrhs, precision), keyed as the graphs
  std::map<long, bg_launch_plan> plans;
  static long plan_key(int nrhs, int prec) { return (long)nrhs * 4 + prec; }
  static bg_launch_plan builtin_plan() { return bg_launch_plan{0, -1, 0, 0, 0, 0, 0}; }
  bg_launch_plan plan_for(int nrhs, int prec) const {
    auto it = plans.find(plan_key(nrhs, prec));
    return it == plans.end() ? builtin_plan() : it->second;
  }

  // solver workspaces kept between bg_solve calls (owned by the solver)
  void* solver_ws = nullptr;
  void (*solver_ws_free)(void*) = nullptr;
  size_t (*solver_ws_bytes)(const void*) = nullptr;

  ~bg_operator() {
    drop_graphs();
    free_slots();
    if (solver_ws && solver_ws_free) solver_ws_free(solver_ws);
    for (auto v : {&d_pts64, &d_pts32, &d_centres, &d_tan64, &d_tan32, &d_far64, &d_far_df, &d_far_atiles, &d_far_ainv,
                   &d_mom64, &d_mom32, &w_y, &w_z, &w_ydf, &w_btiles, &w_binv, &w_yv, &w_zv})
      for (auto b : *v) delete b;
    for (auto& c : near_cache) delete c.blocks;
  }
  size_t scalar_bytes(bool fp32) const { return (cplx ? 2 : 1) * (fp32 ? 4 : 8); }
  // scalars between consecutive stored FP64 blocks of size B x B: rounded up
  // so that every block starts on a 16-byte boundary
  long block_stride(int B) const { return cplx ? (long)B * B : ((long)B * B + 1) / 2 * 2; }
  // FP32 blocks: stride a multiple of 16 bytes
  long block_stride32(int B) const { return cplx ? ((long)B * B + 1) / 2 * 2 : ((long)B * B + 3) / 4 * 4; }
  int stype(bool fp32) const { return (fp32 ? 2 : 0) + (cplx ? 1 : 0); }
  // Maxwell: the far field is stored as the scalar kernel matrix of each
  // cluster pair (np^2 x np^2) and applied to kMwRhsChunk right-hand sides at a time
  bool maxwell() const { return vd == 2; }
  static constexpr int kMwRhsChunk = 8;
  int nclusters(int level) const { return level < 0 ? 1 : mesh.npatch << (2 * level); }
};

bg_status set_error(bg_context* ctx, bg_status st, const std::string& msg);
std::vector<double> basis3_table(int P, const bg::Rule1D& gr);
// child bookkeeping: a context is released only after its last child
void context_retain(bg_context* ctx);
void context_release(bg_context* ctx);
bg_status cuda_status(bg_context* ctx, cudaError_t e, const char* what);
bg_status ensure_work(bg_operator* op, int nrhs);
bg_status check_device_flag(bg_operator* op);
// y_dof = A x_dof on row-major FP64 work vectors. prec (bg_precision):
// BG_PREC_FP64 the FP64 H2 matrix (stored far field); BG_PREC_MIXED FP64 near
// field plus the FP32 fused far field (forward/backward transforms in FP32);
// BG_PREC_FP32 as MIXED with the near field in FP32 as well.
bg_status apply_operator(bg_operator* op, int nrhs, int prec, const void* xdof, void* ydof);
