// Operator state shared by the C-ABI translation units.
#pragma once
#include <cuda_runtime.h>

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
  cudaStream_t stream = nullptr;
  std::string err;
  DevBuf stage_in, stage_out;   // device staging of host operands
  void* pinned = nullptr;       // pinned host staging
  size_t pinned_bytes = 0;
};

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

  // device tables
  DevBuf d_patch_meta, d_patch_cp, d_el_patch, d_el_llc;
  DevBuf d_T_ptr, d_T_idx, d_T_val, d_Tt_ptr, d_Tt_idx, d_Tt_val;
  DevBuf d_cheb;
  std::vector<DevBuf*> d_pts64, d_pts32;  // per level
  DevBuf d_dense64, d_dense32;            // dense blocks
  std::vector<DevBuf*> d_far64;           // per level
  std::vector<DevBuf*> d_mom64, d_mom32;  // per vector component
  DevBuf d_tr64, d_tr32;
  // work vectors (sized for the largest nrhs seen)
  int cap = 0;
  DevBuf w_xdof, w_xss, w_yss, w_ydof;
  std::vector<DevBuf*> w_y, w_z;  // per level

  ~bg_operator() {
    for (auto v : {&d_pts64, &d_pts32, &d_far64, &d_mom64, &d_mom32, &w_y, &w_z})
      for (auto b : *v) delete b;
  }
  size_t scalar_bytes(bool fp32) const { return (cplx ? 2 : 1) * (fp32 ? 4 : 8); }
  int stype(bool fp32) const { return (fp32 ? 2 : 0) + (cplx ? 1 : 0); }
  int nclusters(int level) const { return level < 0 ? 1 : mesh.npatch << (2 * level); }
};

bg_status set_error(bg_context* ctx, bg_status st, const std::string& msg);
bg_status cuda_status(bg_context* ctx, cudaError_t e, const char* what);
bg_status ensure_work(bg_operator* op, int nrhs);
// y_dof (row-major work, FP64 or FP32 per precision) = A x_dof
bg_status apply_operator(bg_operator* op, int nrhs, bool fp32, const void* xdof, void* ydof);
