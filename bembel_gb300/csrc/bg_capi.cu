// C ABI of the GB300 H2 single-layer operator (include/bembel_gb300.h):
// context, geometry and operator lifecycle, device tables, assembly and the
// batched H2 matvec.
#include <algorithm>
#include <array>
#include <chrono>
#include <complex>
#include <cstring>
#include <map>
#include <new>

#include "bg_operator.hpp"

using namespace bg;

static void context_free(bg_context* ctx) {
  if (ctx->device >= 0) {
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    ctx->stage_in.release();
    ctx->stage_out.release();
    for (int c = 0; c < 8; ++c)
      for (auto& pr : ctx->pending[c]) {
        cudaEventDestroy(pr.first);
        cudaEventDestroy(pr.second);
      }
    for (auto ev : ctx->event_pool) cudaEventDestroy(ev);
    if (ctx->pinned) cudaFreeHost(ctx->pinned);
    cudaStreamDestroy(ctx->stream);
  }
  delete ctx;
}
void context_retain(bg_context* ctx) { ++ctx->children; }
void context_release(bg_context* ctx) {
  if (--ctx->children == 0 && ctx->closing) context_free(ctx);
}

bg_status set_error(bg_context* ctx, bg_status st, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return st;
}
bg_status cuda_status(bg_context* ctx, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return BG_OK;
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) return set_error(ctx, BG_OOM, m);
  return set_error(ctx, BG_DEVICE_ERROR, m);
}
#define BG_CHECK(expr, what)                                   \
  do {                                                         \
    bg_status _st = cuda_status(op->ctx, (expr), (what));      \
    if (_st != BG_OK) return _st;                              \
  } while (0)

extern "C" {

void bg_h2_params_default(bg_h2_params* p) {
  if (!p) return;
  p->n_p = 9;
  p->eta = 1.6;
  p->min_cluster_level = 1;
  p->store_fp64_far = 1;
  p->keep_fp64_blocks = 1;
}
void bg_solve_params_default(bg_solve_params* p) {
  if (!p) return;
  p->tol = 1e-8;
  p->restart = 200;
  p->max_iter = 2000;
  p->inner_precision = BG_PREC_FP32;
  p->inner_tol = 2e-3;
  p->max_refinements = 12;
}

bg_status bg_context_create(int device, bg_context** out) {
  if (!out) return BG_INVALID_ARG;
  *out = nullptr;
  bg_context* ctx = new (std::nothrow) bg_context();
  if (!ctx) return BG_OOM;
  ctx->device = device;
  if (device >= 0) {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || device >= n) {
      delete ctx;
      return BG_DEVICE_ERROR;
    }
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete ctx;
      return BG_DEVICE_ERROR;
    }
  }
  *out = ctx;
  return BG_OK;
}
bg_status bg_context_destroy(bg_context* ctx) {
  if (!ctx || ctx->closing) return BG_INVALID_ARG;
  ctx->closing = true;
  if (ctx->children == 0) context_free(ctx);
  return BG_OK;
}
const char* bg_last_error_string(bg_context* ctx) { return ctx ? ctx->err.c_str() : "no context"; }

bg_status bg_context_get_stream(bg_context* ctx, void** stream) {
  if (!ctx || !stream) return BG_INVALID_ARG;
  *stream = (void*)ctx->stream;
  return BG_OK;
}
bg_status bg_profile_enable(bg_context* ctx, int enable) {
  if (!ctx) return BG_INVALID_ARG;
  if (ctx->device < 0) return set_error(ctx, BG_UNSUPPORTED, "host-only context");
  ctx->profiling = enable != 0;
  return BG_OK;
}
bg_status bg_profile_classes(bg_context* ctx, unsigned mask) {
  if (!ctx) return BG_INVALID_ARG;
  ctx->profile_mask = mask;
  return BG_OK;
}
bg_status bg_profile_read(bg_context* ctx, double* ms8, long* launches8) {
  if (!ctx || !ms8 || !launches8) return BG_INVALID_ARG;
  if (ctx->device < 0) return set_error(ctx, BG_UNSUPPORTED, "host-only context");
  cudaSetDevice(ctx->device);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_status(ctx, e, "profile");
  for (int c = 0; c < 8; ++c) {
    for (auto& pr : ctx->pending[c]) {
      float ms = 0;
      cudaEventElapsedTime(&ms, pr.first, pr.second);
      ctx->class_ms[c] += ms;
      ctx->event_pool.push_back(pr.first);
      ctx->event_pool.push_back(pr.second);
    }
    ctx->pending[c].clear();
    ms8[c] = ctx->class_ms[c];
    launches8[c] = ctx->class_launches[c];
    ctx->class_ms[c] = 0;
    ctx->class_launches[c] = 0;
  }
  return BG_OK;
}

bg_status bg_geometry_load_dat(bg_context* ctx, const char* path, bg_geometry** out) {
  if (!ctx || !path || !out || ctx->closing) return BG_INVALID_ARG;
  *out = nullptr;
  bg_geometry* g = new (std::nothrow) bg_geometry();
  if (!g) return BG_OOM;
  std::string err;
  if (!load_dat(path, &g->g, &err)) {
    delete g;
    return set_error(ctx, BG_INVALID_ARG, err);
  }
  g->ctx = ctx;
  context_retain(ctx);
  *out = g;
  return BG_OK;
}
bg_status bg_geometry_load_igs(bg_context* ctx, const char* path, bg_geometry** out) {
  if (!ctx || !path || !out || ctx->closing) return BG_INVALID_ARG;
  *out = nullptr;
  bg_geometry* g = new (std::nothrow) bg_geometry();
  if (!g) return BG_OOM;
  std::string err;
  if (!load_igs(path, &g->g, &err)) {
    delete g;
    return set_error(ctx, BG_INVALID_ARG, err);
  }
  g->ctx = ctx;
  context_retain(ctx);
  *out = g;
  return BG_OK;
}
bg_status bg_geometry_from_bezier(bg_context* ctx, int npatch, const int* px, const int* py, const double* data,
                                  bg_geometry** out) {
  if (!ctx || !out || npatch <= 0 || !px || !py || !data || ctx->closing) return BG_INVALID_ARG;
  *out = nullptr;
  bg_geometry* g = new (std::nothrow) bg_geometry();
  if (!g) return BG_OOM;
  long off = 0;
  for (int p = 0; p < npatch; ++p) {
    if (px[p] < 1 || py[p] < 1 || px[p] > 16 || py[p] > 16) {
      delete g;
      return set_error(ctx, BG_INVALID_ARG, "patch " + std::to_string(p) + ": control points per direction out of 1..16");
    }
    PatchData P;
    P.px = px[p];
    P.py = py[p];
    P.cp.assign(data + off, data + off + 4L * px[p] * py[p]);
    off += 4L * px[p] * py[p];
    for (int c = 0; c < px[p] * py[p]; ++c)
      if (!(P.cp[4 * c + 3] > 0.0) || !std::isfinite(P.cp[4 * c]) || !std::isfinite(P.cp[4 * c + 1]) ||
          !std::isfinite(P.cp[4 * c + 2])) {
        delete g;
        return set_error(ctx, BG_INVALID_ARG, "patch " + std::to_string(p) + ": non-finite point or weight <= 0");
      }
    g->g.patches.push_back(std::move(P));
  }
  g->ctx = ctx;
  context_retain(ctx);
  *out = g;
  return BG_OK;
}
bg_status bg_geometry_cube_sphere(bg_context* ctx, bg_geometry** out) {
  if (!ctx || !out || ctx->closing) return BG_INVALID_ARG;
  *out = nullptr;
  bg_geometry* g = new (std::nothrow) bg_geometry();
  if (!g) return BG_OOM;
  cube_sphere(&g->g);
  g->ctx = ctx;
  context_retain(ctx);
  *out = g;
  return BG_OK;
}
bg_status bg_geometry_patch_data(const bg_geometry* g, int patch, int* px, int* py, double* data) {
  if (!g || !px || !py || patch < 0 || patch >= (int)g->g.patches.size()) return BG_INVALID_ARG;
  const PatchData& P = g->g.patches[patch];
  if (P.face >= 0) return BG_UNSUPPORTED;  // analytic patch: no control points
  *px = P.px;
  *py = P.py;
  if (data) std::copy(P.cp.begin(), P.cp.end(), data);
  return BG_OK;
}
bg_status bg_geometry_num_patches(const bg_geometry* g, int* n) {
  if (!g || !n) return BG_INVALID_ARG;
  *n = (int)g->g.patches.size();
  return BG_OK;
}
bg_status bg_geometry_destroy(bg_geometry* g) {
  if (!g) return BG_INVALID_ARG;
  bg_context* ctx = g->ctx;
  delete g;
  if (ctx) context_release(ctx);
  return BG_OK;
}
bg_status bg_geometry_surface_point(const bg_geometry* g, int patch, double s, double t, double* out12) {
  if (!g || !out12 || patch < 0 || patch >= (int)g->g.patches.size()) return BG_INVALID_ARG;
  out12[0] = s;
  out12[1] = t;
  out12[2] = 1.0;
  patch_frame(g->g.patches[patch], s, t, out12 + 3);
  return BG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
static void build_segments(bg_operator* op) {
  const Partition& pt = op->part;
  const int vd = op->vd;
  // dense leaves
  {
    BsrSegment& s = op->dense;
    const int ncl = op->nclusters(pt.dense_level);
    const int ecl = pt.dense_level < 0 ? op->ne : (1 << (2 * (op->M - pt.dense_level)));
    s.B = ecl * op->p2;
    s.nrows = vd * ncl;
    std::vector<std::vector<std::pair<int, int>>> rows(s.nrows);  // (col block, block id)
    int li = 0, di = 0;
    std::vector<int> leaf_index_of_dense;
    for (size_t k = 0; k < pt.leaf_list.size(); k += 4, ++li)
      if (pt.leaf_list[k] == 2) {
        for (int rc = 0; rc < vd; ++rc)
          for (int cc = 0; cc < vd; ++cc)
            rows[rc * ncl + pt.dense_c1[di]].push_back({cc * ncl + pt.dense_c2[di], (li << 4) | (rc * vd + cc)});
        ++di;
      }
    s.row_ptr.assign(1, 0);
    for (auto& r : rows) {
      std::stable_sort(r.begin(), r.end());
      for (auto& e : r) {
        s.col.push_back(e.first);
        s.leaf.push_back(e.second >> 4);
        s.comp.push_back(e.second & 15);
      }
      s.row_ptr.push_back((int)s.col.size());
    }
  }
  // far levels
  op->far.clear();
  op->far.resize(op->leaf_level + 1);
  // Maxwell far blocks are one scalar kernel matrix per cluster pair
  const int vdf = op->maxwell() ? 1 : vd;
  std::vector<std::vector<std::vector<std::pair<int, int>>>> rows(op->leaf_level + 1);
  for (int l = 0; l <= op->leaf_level; ++l) rows[l].resize(vdf * op->nclusters(l));
  std::vector<int> pos(op->leaf_level + 1, 0);
  int li = 0;
  for (size_t k = 0; k < pt.leaf_list.size(); k += 4, ++li)
    if (pt.leaf_list[k] == 1) {
      const int l = pt.leaf_list[k + 1], c1 = pt.leaf_list[k + 2], c2 = pt.leaf_list[k + 3];
      const int ncl = op->nclusters(l);
      for (int rc = 0; rc < vdf; ++rc)
        for (int cc = 0; cc < vdf; ++cc) rows[l][rc * ncl + c1].push_back({cc * ncl + c2, (li << 4) | (rc * vd + cc)});
    }
  for (int l = 0; l <= op->leaf_level; ++l) {
    BsrSegment& s = op->far[l];
    s.B = op->maxwell() ? op->np * op->np : op->R;
    s.nrows = vdf * op->nclusters(l);
    s.row_ptr.assign(1, 0);
    for (auto& r : rows[l]) {
      std::stable_sort(r.begin(), r.end());
      for (auto& e : r) {
        s.col.push_back(e.first);
        s.leaf.push_back(e.second >> 4);
        s.comp.push_back(e.second & 15);
      }
      s.row_ptr.push_back((int)s.col.size());
    }
  }
}


// Alternative orders of the heaviest-first far-field rows for a persistent
// kernel whose CTA b takes list items b, b + G, b + 2G, ...: order 1 reverses
// every second round of G items (serpentine); order 2 gives each round's
// items, heaviest first, to the CTAs with the least work so far (work of a
// row: its blocks + 1). Both only permute items within a round. Returns false
// unless the result is a permutation of the rows.
static bool far_row_order(const std::vector<std::pair<int, int2>>& sorted, int G, int order, std::vector<int2>* out) {
  const size_t n = sorted.size();
  std::vector<long> pos(n, -1);  // list position of sorted item i
  std::vector<long> load(G, 0);
  std::vector<int> cta(G);
  for (size_t r0 = 0; r0 < n; r0 += G) {
    const int m = (int)std::min<size_t>(G, n - r0);
    for (int j = 0; j < m; ++j) cta[j] = j;
    if (order == 1) {
      if ((r0 / G) % 2 == 1) std::reverse(cta.begin(), cta.begin() + m);
    } else {
      std::stable_sort(cta.begin(), cta.begin() + m, [&](int a, int b) { return load[a] < load[b]; });
    }
    for (int j = 0; j < m; ++j) {
      pos[r0 + j] = (long)r0 + cta[j];
      load[cta[j]] += sorted[r0 + j].first + 1;
    }
  }
  out->assign(n, make_int2(-1, -1));
  std::vector<char> used(n, 0);
  for (size_t i = 0; i < n; ++i) {
    if (pos[i] < 0 || pos[i] >= (long)n || used[pos[i]]) return false;
    used[pos[i]] = 1;
    (*out)[pos[i]] = sorted[i].second;
  }
  return true;
}

static bg_status upload_tables(bg_operator* op) {
  cudaStream_t s = op->ctx->stream;
  std::vector<int> meta;
  std::vector<double> cp;
  for (const auto& P : op->geo.patches) {
    // analytic cube-sphere face: px = 0 marks it, py holds the face
    if (P.face >= 0) meta.insert(meta.end(), {0, P.face, 0});
    else meta.insert(meta.end(), {P.px, P.py, (int)cp.size()});
    cp.insert(cp.end(), P.cp.begin(), P.cp.end());
    while (cp.size() % 4) cp.push_back(0.0);
  }
  BG_CHECK(op->d_patch_meta.upload(meta, s), "upload patches");
  BG_CHECK(op->d_patch_cp.upload(cp, s), "upload patches");
  BG_CHECK(op->d_el_patch.upload(op->mesh.patch, s), "upload elements");
  BG_CHECK(op->d_el_llc.upload(op->mesh.llc, s), "upload elements");
  BG_CHECK(op->d_T_ptr.upload(op->T.ptr, s), "upload T");
  BG_CHECK(op->d_T_idx.upload(op->T.idx, s), "upload T");
  BG_CHECK(op->d_T_val.upload(op->T.val, s), "upload T");
  BG_CHECK(op->d_Tt_ptr.upload(op->Tt.ptr, s), "upload T");
  BG_CHECK(op->d_Tt_idx.upload(op->Tt.idx, s), "upload T");
  BG_CHECK(op->d_Tt_val.upload(op->Tt.val, s), "upload T");
  BG_CHECK(op->d_cheb.upload(cheb_points(op->np), s), "upload FMM");
  BG_CHECK(op->dense.d_row_ptr.upload(op->dense.row_ptr, s), "upload partition");
  BG_CHECK(op->dense.d_col.upload(op->dense.col, s), "upload partition");
  for (auto& f : op->far) {
    BG_CHECK(f.d_row_ptr.upload(f.row_ptr, s), "upload partition");
    BG_CHECK(f.d_col.upload(f.col, s), "upload partition");
  }
  std::vector<std::vector<double>> mom = moment_matrices(op->kind == BG_MAXWELL_SL, op->P, op->leaf_level,
                                                         std::min(op->mcl, op->M), op->np);
  std::vector<double> tr = transfer_matrix(op->np);
  for (auto& m : mom) {
    DevBuf* a = new DevBuf();
    DevBuf* b = new DevBuf();
    op->d_mom64.push_back(a);
    op->d_mom32.push_back(b);
    BG_CHECK(a->upload(m, s), "upload moments");
    std::vector<float> mf(m.begin(), m.end());
    BG_CHECK(b->upload(mf, s), "upload moments");
  }
  BG_CHECK(op->d_tr64.upload(tr, s), "upload transfer");
  std::vector<float> tf(tr.begin(), tr.end());
  BG_CHECK(op->d_tr32.upload(tf, s), "upload transfer");
  {
    // transposed, padded copies for launch_tgemm: AT[q][i] = op(A)[i][q]
    const int R = op->R, Bq = op->Bq, np2 = op->np * op->np;
    auto ld_for = [](int Mo) { const int r = (Mo + 2) / 3 * 3; return (r + 3) / 4 * 4; };
    auto build = [&](int Mo, int Ki, auto opA, DevBuf* d64, DevBuf* d32, TGemmA* a64, TGemmA* a32) -> bg_status {
      const int ld = ld_for(Mo);
      std::vector<double> at((size_t)Ki * ld, 0.0);
      for (int q = 0; q < Ki; ++q)
        for (int i = 0; i < Mo; ++i) at[(size_t)q * ld + i] = opA(i, q);
      std::vector<float> af(at.begin(), at.end());
      BG_CHECK(d64->upload(at, s), "upload transforms");
      BG_CHECK(d32->upload(af, s), "upload transforms");
      *a64 = TGemmA{d64->p, ld, Mo, Ki};
      *a32 = TGemmA{d32->p, ld, Mo, Ki};
      return BG_OK;
    };
    bg_status st;
    for (size_t c = 0; c < mom.size() && c < 2; ++c) {
      const std::vector<double>& m = mom[c];  // R x Bq, row-major
      if ((st = build(R, Bq, [&](int i, int q) { return m[(size_t)i * Bq + q]; }, &op->tm[0].mom_f[c],
                      &op->tm[1].mom_f[c], &op->tm[0].a_mom_f[c], &op->tm[1].a_mom_f[c])) != BG_OK)
        return st;
      if ((st = build(Bq, R, [&](int i, int q) { return m[(size_t)q * Bq + i]; }, &op->tm[0].mom_b[c],
                      &op->tm[1].mom_b[c], &op->tm[0].a_mom_b[c], &op->tm[1].a_mom_b[c])) != BG_OK)
        return st;
    }
    // transfer matrix np2 x 4 np2, row-major
    if ((st = build(np2, 4 * np2, [&](int i, int q) { return tr[(size_t)i * 4 * np2 + q]; }, &op->tm[0].tr_f,
                    &op->tm[1].tr_f, &op->tm[0].a_tr_f, &op->tm[1].a_tr_f)) != BG_OK)
      return st;
    if ((st = build(4 * np2, np2, [&](int i, int q) { return tr[(size_t)q * 4 * np2 + i]; }, &op->tm[0].tr_b,
                    &op->tm[1].tr_b, &op->tm[0].a_tr_b, &op->tm[1].a_tr_b)) != BG_OK)
      return st;
    if (op->maxwell()) {
      // channel blocks: phi (rows 0..np2-1 of either component's matrix),
      // d/ds phi (component 0) and d/dt phi (component 1), rows np2..2 np2-1
      const double* sub[3] = {mom[0].data(), mom[0].data() + (size_t)np2 * Bq, mom[1].data() + (size_t)np2 * Bq};
      for (int c = 0; c < 3; ++c) {
        const double* m = sub[c];
        if ((st = build(np2, Bq, [&](int i, int q) { return m[(size_t)i * Bq + q]; }, &op->tm[0].mw_f[c],
                        &op->tm[1].mw_f[c], &op->tm[0].a_mw_f[c], &op->tm[1].a_mw_f[c])) != BG_OK)
          return st;
        if ((st = build(Bq, np2, [&](int i, int q) { return m[(size_t)q * Bq + i]; }, &op->tm[0].mw_b[c],
                        &op->tm[1].mw_b[c], &op->tm[0].a_mw_b[c], &op->tm[1].a_mw_b[c])) != BG_OK)
          return st;
      }
    }
    // every output row tile count within the kernel's 6 x 256 tiles of 3 x 4
    auto fits = [&](int Mo) { return (Mo + 2) / 3 * 8 <= 6 * 256; };
    op->use_tgemm = (op->maxwell() || (op->nc == 1 && mom.size() <= 2 && fits(R))) && fits(Bq) && fits(np2) &&
                    fits(4 * np2);
  }
  {
    // tensor-product factors of the transfer and moment matrices for the
    // fused transforms (scalar operators with a transfer level); used only if
    // they rebuild the assembled matrices to rounding
    op->fmm_fused = false;
    const int cr = std::min(op->mcl, op->M), np = op->np, np2 = np * np;
    if (!op->maxwell() && op->vd == 1 && op->nc == 1 && op->leaf_level >= 1 && op->leaf_level < kMaxFarLevels &&
        np <= kFmmMaxNp) {
      std::vector<double> E = transfer_factors(np), ms, mt;
      std::vector<int> cmap;
      moment_factors(op->P, op->leaf_level, cr, np, &ms, &mt, &cmap);
      const int w1 = (1 << cr) * (op->P + 1);
      bool ok = w1 <= 16 && w1 * w1 == op->Bq && (int)cmap.size() == op->Bq && mom.size() == 1;
      double dev = 0.0, big = 0.0;
      static const int sx[4] = {0, 1, 1, 0}, sy[4] = {0, 0, 1, 1};
      for (int k = 0; ok && k < 4; ++k)
        for (int o = 0; o < np2; ++o)
          for (int q = 0; q < np2; ++q) {
            const double f = E[sx[k] * np2 + (q / np) * np + o / np] * E[sy[k] * np2 + (q % np) * np + o % np];
            const double t = tr[(size_t)o * 4 * np2 + k * np2 + q];
            dev = std::max(dev, std::fabs(f - t));
            big = std::max(big, std::fabs(t));
          }
      double mdev = 0.0, mbig = 0.0;
      for (int o = 0; ok && o < np2; ++o)
        for (int q = 0; q < op->Bq; ++q) {
          const int a = cmap[q] & 0xFF, b = cmap[q] >> 8;
          const double f = ms[(o / np) * w1 + a] * mt[(o % np) * w1 + b];
          const double t = mom[0][(size_t)o * op->Bq + q];
          mdev = std::max(mdev, std::fabs(f - t));
          mbig = std::max(mbig, std::fabs(t));
        }
      ok = ok && dev <= 1e-14 * big && mdev <= 1e-14 * mbig;
      if (ok) {
        std::vector<double> fac(E);
        fac.insert(fac.end(), ms.begin(), ms.end());
        fac.insert(fac.end(), mt.begin(), mt.end());
        std::vector<float> f32(fac.begin(), fac.end());
        BG_CHECK(op->d_fmm_fac64.upload(fac, s), "upload transforms");
        BG_CHECK(op->d_fmm_fac32.upload(f32, s), "upload transforms");
        BG_CHECK(op->d_fmm_cmap.upload(cmap, s), "upload transforms");
        op->fmm_hfac = fac;
        op->fmm_w1 = w1;
        op->fmm_fused = true;
      }
    }
  }
  {
    // every row of every far-field level, rows with more blocks first so the
    // longest CTAs start in the first wave
    std::vector<std::pair<int, int2>> items;
    for (int l = 0; l < (int)op->far.size() && l < kMaxFarLevels; ++l)
      for (int r = 0; r < op->far[l].nrows; ++r)
        items.push_back({op->far[l].row_ptr[r + 1] - op->far[l].row_ptr[r], make_int2(l, r)});
    std::stable_sort(items.begin(), items.end(), [](const auto& a, const auto& b) { return a.first > b.first; });
    std::vector<int2> work(items.size());
    for (size_t i = 0; i < items.size(); ++i) work[i] = items[i].second;
    BG_CHECK(op->d_far_work.upload(work, s), "far-field work list");
    op->n_far_work = (int)work.size();
    // alternative orders for the persistent far-field kernels (one CTA per SM)
    int nsm = 0;
    BG_CHECK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, op->ctx->device), "device attributes");
    for (int o = 0; o < 2; ++o) op->d_far_work_alt[o].release();
    if (nsm > 0 && (long)items.size() > nsm)
      for (int o = 1; o <= 2; ++o) {
        std::vector<int2> alt;
        if (!far_row_order(items, nsm, o, &alt))
          return set_error(op->ctx, BG_DEVICE_ERROR, "far-field schedule is not a permutation of the rows");
        BG_CHECK(op->d_far_work_alt[o - 1].upload(alt, s), "far-field work list");
      }
  }
  BG_CHECK(op->d_err.alloc(sizeof(int)), "error flag");
  BG_CHECK(cudaMemsetAsync(op->d_err.p, 0, sizeof(int), s), "error flag");
  BG_CHECK(cudaStreamSynchronize(s), "upload tables");
  return BG_OK;
}

extern "C" bg_status bg_operator_create(bg_context* ctx, const bg_geometry* g, int M, int P, int op_kind,
                                        const bg_h2_params* params, bg_operator** out) {
  if (!ctx || !g || !out || ctx->closing) return BG_INVALID_ARG;
  *out = nullptr;
  if (M < 0 || M > 9) return set_error(ctx, BG_INVALID_ARG, "refinement level must be in [0, 9]");
  if (P < 0 || P > 3) return set_error(ctx, BG_UNSUPPORTED, "polynomial degree must be in [0, 3]");
  if (op_kind != BG_LAPLACE_SL && op_kind != BG_HELMHOLTZ_SL && op_kind != BG_MAXWELL_SL)
    return set_error(ctx, BG_INVALID_ARG, "unknown operator kind");
  bg_h2_params prm;
  bg_h2_params_default(&prm);
  if (params) prm = *params;
  if (prm.n_p < 2 || prm.n_p > 12 || prm.eta <= 0 || prm.min_cluster_level < 0 || prm.min_cluster_level > 3)
    return set_error(ctx, BG_INVALID_ARG, "invalid H2 parameters");
  bg_operator* op = new (std::nothrow) bg_operator();
  if (!op) return BG_OOM;
  op->ctx = ctx;
  op->kind = op_kind;
  op->M = M;
  op->P = P;
  op->np = prm.n_p;
  op->eta = prm.eta;
  op->mcl = prm.min_cluster_level;
  op->store_far = prm.store_fp64_far != 0;
  op->keep_far64 = prm.keep_fp64_blocks != 0;
  op->cplx = op_kind != BG_LAPLACE_SL;
  op->vd = op_kind == BG_MAXWELL_SL ? 2 : 1;
  op->nc = op_kind == BG_MAXWELL_SL ? 2 : 1;
  op->geo = g->g;
  op->G = 2;
  for (const auto& p : op->geo.patches) op->G = std::max(op->G, std::max(p.px, p.py));
  if (op->G > 6) {
    delete op;
    return set_error(ctx, BG_UNSUPPORTED, "patch degree above 5 is not supported");
  }
  std::string err;
  if (!build_mesh(op->geo, M, &op->mesh, &err) || !build_transform(op->mesh, P, op->vd == 2, &op->T, &err)) {
    delete op;
    return set_error(ctx, BG_INVALID_ARG, err);
  }
  op->Tt = transpose(op->T);
  build_partition(op->mesh, op->eta, op->mcl, &op->part);
  op->p2 = (P + 1) * (P + 1);
  op->ne = op->mesh.ne;
  op->S = op->T.rows;
  op->N = op->T.cols;
  op->leaf_level = std::max(M - op->mcl, 0);
  op->nleaf_cl = op->nclusters(op->leaf_level);
  op->Bq = (1 << (2 * std::min(op->mcl, M))) * op->p2;
  op->R = op->nc * op->np * op->np;
  build_segments(op);
  if (ctx->device >= 0) {
    cudaSetDevice(ctx->device);
    bg_status st = upload_tables(op);
    if (st != BG_OK) {
      delete op;
      return st;
    }
  }
  context_retain(ctx);
  *out = op;
  return BG_OK;
}

extern "C" bg_status bg_operator_destroy(bg_operator* op) {
  if (!op) return BG_INVALID_ARG;
  bg_context* ctx = op->ctx;
  if (ctx && ctx->device >= 0) {
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
  }
  delete op;
  if (ctx) context_release(ctx);
  return BG_OK;
}

extern "C" bg_status bg_operator_set_wavenumber(bg_operator* op, double re, double im) {
  if (!op) return BG_INVALID_ARG;
  if (op->kind == BG_LAPLACE_SL) return set_error(op->ctx, BG_INVALID_ARG, "the Laplace operator has no wavenumber");
  if (op->kind == BG_MAXWELL_SL && re == 0.0 && im == 0.0)
    return set_error(op->ctx, BG_INVALID_ARG, "the Maxwell operator needs a nonzero wavenumber");
  op->kre = re;
  op->kim = im;
  op->assembled = false;
  return BG_OK;
}

extern "C" bg_status bg_operator_info(const bg_operator* op, long* info) {
  if (!op || !info) return BG_INVALID_ARG;
  long nd = 0, nl = 0;
  for (size_t k = 0; k < op->part.leaf_list.size(); k += 4) (op->part.leaf_list[k] == 2 ? nd : nl)++;
  long far_bytes = 0;
  for (const auto& f : op->far) far_bytes += (long)f.col.size() * op->block_stride(f.B) * 8 * (op->cplx ? 2 : 1);
  if (!op->store_far) far_bytes = 0;
  const long near_bytes = (long)op->dense.col.size() * op->block_stride(op->dense.B) * (long)op->scalar_bytes(false);
  long v[16] = {op->N, op->S, op->ne, nd, nl, op->vd, op->nc, op->np, op->cplx ? 1 : 0, op->M, op->P,
                op->dense.B / std::max(op->p2, 1), (long)op->T.val.size(), far_bytes, near_bytes, op->near_pairs};
  std::memcpy(info, v, sizeof(v));
  return BG_OK;
}
// bg_watchdog_selftest: CUDA errors are reported against the context
#define WD_CHECK(expr, what)                                   \
  do {                                                         \
    bg_status _st = cuda_status(ctx, (expr), (what));          \
    if (_st != BG_OK) return _st;                              \
  } while (0)
extern "C" bg_status bg_watchdog_selftest(bg_context* ctx, long long limit_cycles) {
  if (!ctx || limit_cycles <= 0) return BG_INVALID_ARG;
  if (ctx->device < 0) return set_error(ctx, BG_UNSUPPORTED, "host-only context: the self-test needs a GPU");
  cudaSetDevice(ctx->device);
  DevBuf flag;
  WD_CHECK(flag.alloc(sizeof(int)), "watchdog self-test");
  WD_CHECK(cudaMemsetAsync(flag.p, 0, sizeof(int), ctx->stream), "watchdog self-test");
  WD_CHECK(launch_wait_selftest(limit_cycles, flag.as<int>(), ctx->stream), "watchdog self-test");
  int code = 0;
  WD_CHECK(cudaMemcpyAsync(&code, flag.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream), "watchdog self-test");
  WD_CHECK(cudaStreamSynchronize(ctx->stream), "watchdog self-test");
  if (code != 0)
    return set_error(ctx, BG_TIMEOUT, "watchdog self-test: the bounded device wait ran out (code " +
                                           std::to_string(code) + ")");
  return BG_OK;
}
#undef WD_CHECK

extern "C" bg_status bg_operator_memory(const bg_operator* op, size_t* allocated, size_t* estimate) {
  if (!op || !allocated || !estimate) return BG_INVALID_ARG;
  size_t a = 0;
  for (const DevBuf* b : {&op->d_patch_meta, &op->d_patch_cp, &op->d_el_patch, &op->d_el_llc, &op->d_T_ptr,
                          &op->d_T_idx, &op->d_T_val, &op->d_Tt_ptr, &op->d_Tt_idx, &op->d_Tt_val, &op->d_cheb,
                          &op->d_dense64, &op->d_dense32, &op->d_dense_df, &op->d_oz_tiles, &op->d_oz_rexp,
                          &op->w_oz_panels, &op->w_oz_fmax, &op->d_tr64, &op->d_tr32,
                          &op->d_far_work, &op->d_err, &op->w_xdof, &op->w_xss, &op->w_yss, &op->w_ydof,
                          &op->w_xss32, &op->w_yss32, &op->w_xss_df,
                          &op->dense.d_row_ptr, &op->dense.d_col})
    a += b->bytes;
  for (const auto* v : {&op->d_pts64, &op->d_pts32, &op->d_centres, &op->d_tan64, &op->d_tan32, &op->d_far64,
                        &op->d_far_df, &op->d_far_atiles, &op->d_far_ainv, &op->d_mom64, &op->d_mom32, &op->w_y,
                        &op->w_z, &op->w_ydf, &op->w_yv, &op->w_zv, &op->w_btiles, &op->w_binv})
    for (const DevBuf* b : *v) a += b->bytes;
  for (const auto& tm : op->tm)
    for (const DevBuf* b : {&tm.mom_f[0], &tm.mom_f[1], &tm.mom_b[0], &tm.mom_b[1], &tm.tr_f, &tm.tr_b, &tm.mw_f[0],
                            &tm.mw_f[1], &tm.mw_f[2], &tm.mw_b[0], &tm.mw_b[1], &tm.mw_b[2]})
      a += b->bytes;
  for (const auto& f : op->far) a += f.d_row_ptr.bytes + f.d_col.bytes;
  for (const auto& c : op->near_cache) a += c.blocks->bytes;
  for (const auto& k : op->kslots) {  // batched wavenumbers (the active slot's fields are counted above)
    if (&k == &op->kslots[0] + op->kslot_active) continue;
    a += k.dense64.bytes + k.dense32.bytes;
    for (const auto* v : {&k.far64, &k.far_df, &k.atiles, &k.ainv})
      for (const DevBuf* b : *v) a += b->bytes;
  }
  a += op->w_kx.bytes + op->w_ky.bytes;
  if (op->solver_ws && op->solver_ws_bytes) a += op->solver_ws_bytes(op->solver_ws);
  *allocated = a;
  // stored fields once assembled
  const size_t sb = op->scalar_bytes(false);
  const int np2 = op->np * op->np;
  size_t e = (size_t)op->dense.col.size() * op->block_stride(op->dense.B) * sb +
             (size_t)op->dense.col.size() * op->block_stride32(op->dense.B) * sb / 2;
  if (!op->cplx) e += (size_t)op->dense.col.size() * op->block_stride(op->dense.B) * sizeof(float2);  // double-float
  if (!op->cplx && oz_supported(op->dense.B))  // tensor-core digit tiles, row exponents, x digit panels
    e += oz_tile_bytes(op->dense.B, (long)op->dense.col.size()) + (size_t)op->dense.nrows * op->dense.B * sizeof(int) +
         oz_panel_bytes(op->dense.B, op->S / op->dense.B) + 32 * sizeof(int);
  for (int l = 0; l <= op->leaf_level && l < (int)op->far.size(); ++l) {
    const size_t nb = op->far[l].col.size();
    const size_t ncl = (size_t)op->nclusters(l);
    e += ncl * np2 * (sizeof(d4) + sizeof(float4) + (op->maxwell() ? 6 * (sizeof(double) + sizeof(float)) : 0));
    if (!op->store_far) continue;
    if (op->keep_far64) e += nb * op->block_stride(op->far[l].B) * sb;  // FP64 couplings
    e += nb * op->block_stride(op->far[l].B) * 8 * (op->cplx ? 2 : 1);  // double-float pairs
    e += nb * (op->cplx ? far_h16c_atile_bytes(np2) : far_h16_atile_bytes(np2)) + nb * sizeof(float);
  }
  // work vectors and solver workspaces for 32 right-hand sides: superspace and
  // level vectors, and three Krylov bases (restart 200) of N x 32
  const size_t k = 32;
  size_t lev = 0;
  for (int l = 0; l <= op->leaf_level; ++l) lev += (size_t)op->vd * op->nclusters(l) * op->R;
  e += 9 * (size_t)op->S * k * sb + 4 * lev * k * sb + 3 * 202 * (size_t)op->N * k * sb;
  *estimate = std::max(e, a);
  return BG_OK;
}

extern "C" bg_status bg_operator_assembly_times(const bg_operator* op, double* t3) {
  if (!op || !t3) return BG_INVALID_ARG;
  t3[0] = op->t_near;
  t3[1] = op->t_far;
  t3[2] = op->t_total;
  return BG_OK;
}

extern "C" bg_status bg_operator_elements(const bg_operator* op, int* ints5, double* dbl6) {
  if (!op || !ints5 || !dbl6) return BG_INVALID_ARG;
  const Mesh& m = op->mesh;
  for (int e = 0; e < m.ne; ++e) {
    ints5[5 * e] = m.patch[e];
    for (int k = 0; k < 4; ++k) ints5[5 * e + 1 + k] = m.vert[4 * e + k];
    dbl6[6 * e] = m.llc[2 * e];
    dbl6[6 * e + 1] = m.llc[2 * e + 1];
    for (int k = 0; k < 4; ++k) dbl6[6 * e + 2 + k] = m.ball[m.M][4 * e + k];
  }
  return BG_OK;
}
extern "C" bg_status bg_operator_leaves(const bg_operator* op, int* out4) {
  if (!op || !out4) return BG_INVALID_ARG;
  std::copy(op->part.leaf_list.begin(), op->part.leaf_list.end(), out4);
  return BG_OK;
}
extern "C" bg_status bg_operator_transform(const bg_operator* op, int* ptr, int* idx, double* val) {
  if (!op || !ptr || !idx || !val) return BG_INVALID_ARG;
  std::copy(op->T.ptr.begin(), op->T.ptr.end(), ptr);
  std::copy(op->T.idx.begin(), op->T.idx.end(), idx);
  std::copy(op->T.val.begin(), op->T.val.end(), val);
  return BG_OK;
}

// The (rc, cc) block of a Maxwell low-rank leaf in the reference layout
// (interpolateKernel, H2Multipole.hpp:336-375, with the 4 x 4 coupling of
// Maxwell/SingleLayerOperator.hpp:90-120): [K o (t_rc . t_cc), 0; 0, -K / kappa^2]
// over the np^2 points, rebuilt from the stored kernel matrix K and the tangents.
static bg_status maxwell_far_block(const bg_operator* op, long leaf, long k, int rc, int cc, double* out) {
  const int l = op->part.leaf_list[4 * leaf + 1], c1 = op->part.leaf_list[4 * leaf + 2],
            c2 = op->part.leaf_list[4 * leaf + 3];
  const int np2 = op->np * op->np, R = 2 * np2;
  std::vector<double> K(2 * (size_t)np2 * np2), t1(6 * (size_t)np2), t2(6 * (size_t)np2);
  cudaSetDevice(op->ctx->device);
  cudaError_t e = cudaMemcpy(K.data(), static_cast<const char*>(op->d_far64[l]->p) + k * op->block_stride(np2) * 16,
                             K.size() * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess)
    e = cudaMemcpy(t1.data(), op->d_tan64[l]->as<double>() + 6L * c1 * np2, t1.size() * sizeof(double),
                   cudaMemcpyDeviceToHost);
  if (e == cudaSuccess)
    e = cudaMemcpy(t2.data(), op->d_tan64[l]->as<double>() + 6L * c2 * np2, t2.size() * sizeof(double),
                   cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_status(op->ctx, e, "copy leaf block");
  const std::complex<double> kap(op->kre, op->kim), mk2 = -1.0 / (kap * kap);
  std::fill(out, out + 2 * (size_t)R * R, 0.0);
  for (int j = 0; j < np2; ++j)
    for (int i = 0; i < np2; ++i) {
      const std::complex<double> kv(K[2 * ((size_t)j * np2 + i)], K[2 * ((size_t)j * np2 + i) + 1]);
      const double* ti = &t1[6 * i + 3 * rc];
      const double* tj = &t2[6 * j + 3 * cc];
      const std::complex<double> a = kv * (ti[0] * tj[0] + ti[1] * tj[1] + ti[2] * tj[2]), d = kv * mk2;
      out[2 * ((size_t)j * R + i)] = a.real();
      out[2 * ((size_t)j * R + i) + 1] = a.imag();
      out[2 * ((size_t)(np2 + j) * R + np2 + i)] = d.real();
      out[2 * ((size_t)(np2 + j) * R + np2 + i) + 1] = d.imag();
    }
  return BG_OK;
}

extern "C" bg_status bg_operator_leaf_block(const bg_operator* op, long leaf, int rc, int cc, double* out) {
  if (!op || !out || leaf < 0 || 4 * leaf >= (long)op->part.leaf_list.size() || rc < 0 || cc < 0 || rc >= op->vd ||
      cc >= op->vd)
    return BG_INVALID_ARG;
  if (op->ctx->device < 0 || !op->assembled) return set_error(op->ctx, BG_INVALID_ARG, "operator not assembled");
  if (op->kbatched())
    return set_error(op->ctx, BG_UNSUPPORTED, "leaf blocks of batched wavenumbers: assemble one wavenumber to inspect");
  const int cls = op->part.leaf_list[4 * leaf];
  const BsrSegment* seg = nullptr;
  const DevBuf* data = nullptr;
  if (cls == 2) {
    seg = &op->dense;
    data = &op->d_dense64;
  } else {
    if (!op->store_far) return set_error(op->ctx, BG_INVALID_ARG, "far field is not stored");
    const int l = op->part.leaf_list[4 * leaf + 1];
    if (!op->d_far64[l]->p)
      return set_error(op->ctx, BG_INVALID_ARG, "the FP64 coupling blocks were released after assembly");
    seg = &op->far[l];
    data = op->d_far64[l];
  }
  const bool mw_far = cls != 2 && op->maxwell();
  long k = -1;
  for (size_t i = 0; i < seg->leaf.size(); ++i)
    if (seg->leaf[i] == leaf && (mw_far || seg->comp[i] == rc * op->vd + cc)) k = (long)i;
  if (k < 0) return set_error(op->ctx, BG_INVALID_ARG, "leaf not found");
  if (mw_far) return maxwell_far_block(op, leaf, k, rc, cc, out);
  const size_t sb = op->scalar_bytes(false);
  const size_t bytes = (size_t)seg->B * seg->B * sb;
  const size_t stride = (size_t)op->block_stride(seg->B) * sb;
  cudaSetDevice(op->ctx->device);
  cudaError_t e = cudaMemcpy(out, static_cast<const char*>(data->p) + k * stride, bytes, cudaMemcpyDeviceToHost);
  return cuda_status(op->ctx, e, "copy leaf block");
}

// ---------------------------------------------------------------------------
// Assembly (H2Matrix::init_H2Matrix, H2Matrix.hpp:93-250)
static bg_status assemble_far(bg_operator* op) {
  cudaStream_t s = op->ctx->stream;
  PatchTable pt{op->d_patch_meta.as<int>(), op->d_patch_cp.as<double>()};
  const int np2 = op->np * op->np;
  bool any_far = false;
  int far_levels = 0, tiled_levels = 0;
  for (const auto& f : op->far) {
    any_far |= !f.col.empty();
    far_levels += !f.col.empty();
  }
  op->far_tiles = false;
  if (!any_far) return BG_OK;
  for (int l = 0; l <= op->leaf_level; ++l) {
    if ((int)op->d_pts64.size() <= l) {
      op->d_pts64.push_back(new DevBuf());
      op->d_pts32.push_back(new DevBuf());
      op->d_centres.push_back(new DevBuf());
      op->d_far64.push_back(new DevBuf());
      op->d_far_df.push_back(new DevBuf());
      op->d_far_atiles.push_back(new DevBuf());
      op->d_far_ainv.push_back(new DevBuf());
      op->d_tan64.push_back(new DevBuf());
      op->d_tan32.push_back(new DevBuf());
    }
    const int ncl = op->nclusters(l);
    std::vector<double> cen(4 * (size_t)ncl);
    for (int c = 0; c < ncl; ++c)
      for (int q = 0; q < 3; ++q) cen[4 * c + q] = op->mesh.ball[l][4 * c + q];
    BG_CHECK(op->d_centres[l]->upload(cen, s), "cluster centres");
    BG_CHECK(op->d_pts64[l]->alloc((size_t)ncl * np2 * sizeof(d4)), "cluster points");
    BG_CHECK(op->d_pts32[l]->alloc((size_t)ncl * np2 * sizeof(float4)), "cluster points");
    if (op->maxwell()) {
      BG_CHECK(op->d_tan64[l]->alloc((size_t)ncl * np2 * 6 * sizeof(double)), "cluster tangents");
      BG_CHECK(op->d_tan32[l]->alloc((size_t)ncl * np2 * 6 * sizeof(float)), "cluster tangents");
    }
    BG_CHECK(timed_launch(op->ctx, KC_ASSEMBLY, [&] { return launch_cluster_points(op->G, pt, l, ncl, op->d_cheb.as<double>(), op->np, op->d_centres[l]->as<d4>(),
                                   op->d_pts64[l]->as<d4>(), op->d_pts32[l]->as<float4>(),
                                   op->maxwell() ? op->d_tan64[l]->as<double>() : nullptr,
                                   op->maxwell() ? op->d_tan32[l]->as<float>() : nullptr, s); }),
             "cluster points");
    if (!op->store_far || op->far[l].col.empty()) continue;
    const BsrSegment& f = op->far[l];
    std::vector<int2> pairs(f.col.size());
    for (int r = 0; r < f.nrows; ++r)
      for (int k = f.row_ptr[r]; k < f.row_ptr[r + 1]; ++k) pairs[k] = make_int2(r, f.col[k]);
    DevBuf dp;
    BG_CHECK(dp.upload(pairs, s), "far pairs");
    const size_t bytes = (size_t)f.col.size() * op->block_stride(f.B) * op->scalar_bytes(false);
    BG_CHECK(op->d_far64[l]->alloc(bytes), "far field storage");
    BG_CHECK(timed_launch(op->ctx, KC_ASSEMBLY, [&] { return launch_far_assemble(op->cplx, op->d_pts64[l]->as<d4>(), dp.as<int2>(), (int)pairs.size(), f.B,
                                 op->block_stride(f.B), op->kre, op->kim, op->d_far64[l]->p, s); }),
             "far-field assembly");
    if (op->cplx) {
      // double-float pairs of Re and Im for the complex FP64 product
      const long sdf = ((long)f.B * f.B + 1) / 2 * 2;
      BG_CHECK(op->d_far_df[l]->alloc(2 * f.col.size() * sdf * sizeof(float2)), "far field storage");
      BG_CHECK(launch_split_df_cplx_blocks(op->d_far64[l]->p, op->block_stride(f.B), (long)f.B * f.B, (long)f.col.size(),
                                           sdf, op->d_far_df[l]->p, s),
               "far-field split");
      // scaled FP16 hi / lo tiles of Re and Im for the complex tensor-core product
      const size_t tb = far_h16c_atile_bytes(np2);
      if (tb > 0) {
        BG_CHECK(op->d_far_atiles[l]->alloc(tb * f.col.size()), "far field tiles");
        BG_CHECK(op->d_far_ainv[l]->alloc(sizeof(float) * f.col.size()), "far field tiles");
        BG_CHECK(launch_build_h16c_atiles(np2, op->d_far64[l]->p, op->block_stride(f.B), (long)f.col.size(),
                                          op->d_far_atiles[l]->p, op->d_far_ainv[l]->as<float>(), s),
                 "far-field tiles");
        ++tiled_levels;
      }
    } else {
      // (hi, lo) FP32 pairs of the same blocks for the double-float FP64 product
      BG_CHECK(op->d_far_df[l]->alloc(bytes), "far field storage");
      BG_CHECK(launch_split_df(op->d_far64[l]->p, (long)f.col.size() * op->block_stride(f.B), op->d_far_df[l]->p, s),
               "far-field split");
      // scaled FP16 hi / lo tiles in the tensor-core operand layout
      const size_t tb = far_h16_atile_bytes(np2);
      if (tb > 0 && op->vd == 1 && op->nc == 1) {
        BG_CHECK(op->d_far_atiles[l]->alloc(tb * f.col.size()), "far field tiles");
        BG_CHECK(op->d_far_ainv[l]->alloc(sizeof(float) * f.col.size()), "far field tiles");
        BG_CHECK(launch_build_h16_atiles(np2, op->d_far64[l]->as<double>(), op->block_stride(f.B), (long)f.col.size(),
                                         op->d_far_atiles[l]->p, op->d_far_ainv[l]->as<float>(), s),
                 "far-field tiles");
        ++tiled_levels;
      }
    }
    BG_CHECK(cudaStreamSynchronize(s), "far-field assembly");
    // the products read the double-float pairs and the tiles, not the FP64 blocks
    if (!op->keep_far64 && op->d_far_df[l]->p) op->d_far64[l]->release();
  }
  op->far_tiles = tiled_levels == far_levels && op->leaf_level < kMaxFarLevels;
  return BG_OK;
}

// phi, d/ds phi, d/dt phi of the degree-P tensor Bernstein basis at the
// points of the n1 x n1 tensor rule gr, as [3][n1^2][(P+1)^2]
std::vector<double> basis3_table(int P, const Rule1D& gr) {
  const int n1 = (int)gr.x.size(), Q = n1 * n1, p2 = (P + 1) * (P + 1);
  std::vector<double> basis3((size_t)3 * Q * p2);
  for (int q = 0; q < Q; ++q) {
    double bs[8], bt[8], ds[8], dt[8];
    const double u = gr.x[q / n1], v = gr.x[q % n1];
    bernstein(P, u, bs);
    bernstein(P, v, bt);
    bernstein_der(P, u, ds);
    bernstein_der(P, v, dt);
    for (int iy = 0; iy <= P; ++iy)
      for (int ix = 0; ix <= P; ++ix) {
        const size_t o = (size_t)q * p2 + iy * (P + 1) + ix;
        basis3[o] = bs[ix] * bt[iy];
        basis3[(size_t)Q * p2 + o] = ds[ix] * bt[iy];
        basis3[(size_t)2 * Q * p2 + o] = bs[ix] * dt[iy];
      }
  }
  return basis3;
}

// Dense leaves of the Maxwell operator: every element pair fills its four
// component blocks at once (H2Matrix.hpp:195-205 scatters them per component).
static bg_status assemble_near_mw(bg_operator* op) {
  cudaStream_t s = op->ctx->stream;
  const BsrSegment& D = op->dense;
  const int B = D.B, p2 = op->p2, P = op->P;
  const int ecl = B / p2;
  const int ncl = D.nrows / 2;
  const long bstride = op->block_stride(B);
  BG_CHECK(op->d_dense64.alloc((size_t)D.col.size() * bstride * 16), "near-field storage");
  BG_CHECK(cudaMemsetAsync(op->d_dense64.p, 0, (size_t)D.col.size() * bstride * 16, s), "near-field storage");
  // block index of every (leaf, component pair)
  std::map<int, std::array<long, 4>> where;
  for (size_t k = 0; k < D.col.size(); ++k) {
    auto it = where.find(D.leaf[k]);
    if (it == where.end()) it = where.emplace(D.leaf[k], std::array<long, 4>{-1, -1, -1, -1}).first;
    it->second[D.comp[k]] = (long)k;
  }
  std::map<int, std::vector<NearPairV>> regular;
  std::map<std::pair<int, int>, std::vector<NearPairV>> singular;
  long npairs = 0;
  for (int r = 0; r < ncl; ++r)
    for (int k = D.row_ptr[r]; k < D.row_ptr[r + 1]; ++k) {
      if (D.comp[k] != 0) continue;
      const std::array<long, 4>& kk = where[D.leaf[k]];
      if (kk[0] < 0 || kk[1] < 0 || kk[2] < 0 || kk[3] < 0)
        return set_error(op->ctx, BG_DEVICE_ERROR, "incomplete component blocks of a dense leaf");
      const int c1 = r, c2 = D.col[k];
      for (int b = 0; b < ecl; ++b)
        for (int a = 0; a < ecl; ++a) {
          const int e1 = c1 * ecl + a, e2 = c2 * ecl + b;
          PairClass pc = classify_pair(op->mesh, e1, e2, op->P);
          NearPairV np;
          np.e1 = e1;
          np.e2 = e2;
          np.rot = (pc.rot1 & 15) | ((pc.rot2 & 15) << 4);
          np.pad = 0;
          for (int c = 0; c < 4; ++c) np.dst[c] = (long long)kk[c] * bstride + (long long)(b * p2) * B + a * p2;
          if (pc.cs == 0) regular[pc.deg].push_back(np);
          else singular[{pc.cs, pc.deg}].push_back(np);
          ++npairs;
        }
    }
  op->near_pairs = npairs;
  PatchTable pt{op->d_patch_meta.as<int>(), op->d_patch_cp.as<double>()};
  const double h = 1.0 / double(1 << op->M);
  ElementTable et{op->d_el_patch.as<int>(), op->d_el_llc.as<double>(), h};
  // idiv = -1 / (kappa^2 h^2) (Maxwell/SingleLayerOperator.hpp:71-76)
  const std::complex<double> kap(op->kre, op->kim), idv = -1.0 / (kap * kap * h * h);
  const cd idiv{idv.real(), idv.imag()};
  cd* out = op->d_dense64.as<cd>();
  std::vector<DevBuf*> keep;
  auto cleanup = [&]() {
    cudaStreamSynchronize(s);
    for (auto b : keep) delete b;
  };
  bg_status st = BG_OK;
  for (auto& kv : regular) {
    const int deg = kv.first, n1 = deg + 1, Q = n1 * n1;
    const Rule1D& gr = gauss_rule(n1);
    const std::vector<double> basis3 = basis3_table(P, gr);
    DevBuf *dgx = new DevBuf(), *dgw = new DevBuf(), *dtab = new DevBuf(), *dbas = new DevBuf(), *dpairs = new DevBuf();
    keep.insert(keep.end(), {dgx, dgw, dtab, dbas, dpairs});
    cudaError_t e = dgx->upload(gr.x, s);
    if (e == cudaSuccess) e = dgw->upload(gr.w, s);
    if (e == cudaSuccess) e = dbas->upload(basis3, s);
    if (e == cudaSuccess) e = dpairs->upload(kv.second, s);
    if (e == cudaSuccess) e = dtab->alloc((size_t)op->ne * Q * sizeof(MwPt));
    if (e == cudaSuccess)
      e = launch_quad_table_mw(op->G, pt, et, op->ne, dgx->as<double>(), dgw->as<double>(), n1, dtab->as<MwPt>(), s);
    if (e == cudaSuccess)
      e = launch_near_regular_mw(P, dpairs->as<NearPairV>(), (int)kv.second.size(), dtab->as<MwPt>(), n1,
                                 dbas->as<double>(), op->kre, op->kim, idiv, out, B, s);
    if ((st = cuda_status(op->ctx, e, "near-field regular pairs (Maxwell)")) != BG_OK) {
      cleanup();
      return st;
    }
  }
  for (auto& kv : singular) {
    const int cs = kv.first.first, deg = kv.first.second, n1 = deg + 1;
    const Rule1D& gr = gauss_rule(n1);
    DevBuf *dgx = new DevBuf(), *dgw = new DevBuf(), *dpairs = new DevBuf();
    keep.insert(keep.end(), {dgx, dgw, dpairs});
    cudaError_t e = dgx->upload(gr.x, s);
    if (e == cudaSuccess) e = dgw->upload(gr.w, s);
    if (e == cudaSuccess) e = dpairs->upload(kv.second, s);
    if (e == cudaSuccess)
      e = launch_near_duffy_mw(op->G, P, cs, pt, et, dpairs->as<NearPairV>(), (int)kv.second.size(),
                               dgx->as<double>(), dgw->as<double>(), n1, op->kre, op->kim, idiv, out, B, s);
    if ((st = cuda_status(op->ctx, e, "near-field singular pairs (Maxwell)")) != BG_OK) {
      cleanup();
      return st;
    }
  }
  cudaError_t e = cudaStreamSynchronize(s);
  cleanup();
  return cuda_status(op->ctx, e, "near-field assembly");
}

// Element pairs of the dense leaves of a scalar operator, classified on the
// host (FP64, as the reference): regular pairs by quadrature degree, singular
// pairs by (case, degree); dst is the entry offset of the pair's block.
struct NearWork {
  std::map<int, std::vector<NearPair>> regular;
  std::map<std::pair<int, int>, std::vector<NearPair>> singular;
  long npairs = 0;
};
static NearWork near_work(const bg_operator* op) {
  NearWork w;
  const BsrSegment& D = op->dense;
  const int B = D.B, p2 = op->p2, ecl = B / p2;
  const long bstride = op->block_stride(B);
  for (int r = 0; r < D.nrows; ++r)
    for (int k = D.row_ptr[r]; k < D.row_ptr[r + 1]; ++k) {
      const int c1 = r, c2 = D.col[k];
      for (int b = 0; b < ecl; ++b)
        for (int a = 0; a < ecl; ++a) {
          const int e1 = c1 * ecl + a, e2 = c2 * ecl + b;
          PairClass pc = classify_pair(op->mesh, e1, e2, op->P);
          NearPair np;
          np.e1 = e1;
          np.e2 = e2;
          np.rot = (pc.rot1 & 15) | ((pc.rot2 & 15) << 4);
          np.pad = 0;
          np.dst = (long long)k * bstride + (long long)(b * p2) * B + a * p2;
          if (pc.cs == 0) w.regular[pc.deg].push_back(np);
          else w.singular[{pc.cs, pc.deg}].push_back(np);
          ++w.npairs;
        }
    }
  return w;
}

// Quadrature of the dense leaves for nk wavenumbers into out[q] (zeroed
// block pools). The regular pairs' per-element tables of surface points are
// built once per degree and shared; the singular (Duffy) pairs of complex
// operators evaluate each sample's points, measures and basis values once for
// up to kDuffyMaxWavenumbers wavenumbers per launch.
static bg_status near_quadrature(bg_operator* op, const NearWork& w, int nk, const double* kre, const double* kim,
                                 void* const* out) {
  cudaStream_t s = op->ctx->stream;
  const int B = op->dense.B, p2 = op->p2;
  PatchTable pt{op->d_patch_meta.as<int>(), op->d_patch_cp.as<double>()};
  ElementTable et{op->d_el_patch.as<int>(), op->d_el_llc.as<double>(), 1.0 / double(1 << op->M)};
  std::vector<DevBuf*> keep;  // buffers alive until the stream drains
  auto cleanup = [&]() {
    cudaStreamSynchronize(s);
    for (auto b : keep) delete b;
  };
  bg_status st = BG_OK;
  for (auto& kv : w.regular) {
    const int deg = kv.first, n1 = deg + 1, Q = n1 * n1;
    const Rule1D& gr = gauss_rule(n1);
    std::vector<double> basis((size_t)Q * p2);
    for (int q = 0; q < Q; ++q) {
      double bs[8], bt[8];
      bernstein(op->P, gr.x[q / n1], bs);
      bernstein(op->P, gr.x[q % n1], bt);
      for (int iy = 0; iy <= op->P; ++iy)
        for (int ix = 0; ix <= op->P; ++ix) basis[(size_t)q * p2 + iy * (op->P + 1) + ix] = bs[ix] * bt[iy];
    }
    DevBuf *dgx = new DevBuf(), *dgw = new DevBuf(), *dtab = new DevBuf(), *dbas = new DevBuf(), *dpairs = new DevBuf();
    keep.insert(keep.end(), {dgx, dgw, dtab, dbas, dpairs});
    cudaError_t e = dgx->upload(gr.x, s);
    if (e == cudaSuccess) e = dgw->upload(gr.w, s);
    if (e == cudaSuccess) e = dbas->upload(basis, s);
    if (e == cudaSuccess) e = dpairs->upload(kv.second, s);
    if (e == cudaSuccess) e = dtab->alloc((size_t)op->ne * Q * sizeof(d4));
    if (e == cudaSuccess) e = launch_quad_table(op->G, pt, et, op->ne, dgx->as<double>(), dgw->as<double>(), n1, dtab->as<d4>(), s);
    for (int q = 0; q < nk && e == cudaSuccess; ++q)
      e = launch_near_regular(op->P, op->cplx, dpairs->as<NearPair>(), (int)kv.second.size(), dtab->as<d4>(), n1,
                              dbas->as<double>(), kre[q], kim[q], out[q], B, s);
    if ((st = cuda_status(op->ctx, e, "near-field regular pairs")) != BG_OK) {
      cleanup();
      return st;
    }
  }
  const bool multi = op->cplx && nk > 1 && (op->P == 1 || op->P == 2);
  for (auto& kv : w.singular) {
    const int cs = kv.first.first, deg = kv.first.second, n1 = deg + 1;
    const Rule1D& gr = gauss_rule(n1);
    DevBuf *dgx = new DevBuf(), *dgw = new DevBuf(), *dpairs = new DevBuf();
    keep.insert(keep.end(), {dgx, dgw, dpairs});
    cudaError_t e = dgx->upload(gr.x, s);
    if (e == cudaSuccess) e = dgw->upload(gr.w, s);
    if (e == cudaSuccess) e = dpairs->upload(kv.second, s);
    // the common-edge and common-vertex rules have factorised one-wavenumber
    // kernels (P <= 2, n1 <= 16), faster than sharing per-sample work over
    // several wavenumbers; the identical-element rule shares it
    const bool factorised = (cs == 3 || cs == 4) && op->P <= 2 && 2 * n1 <= 32;
    for (int q0 = 0; q0 < nk && e == cudaSuccess;) {
      const bool mk = multi && !factorised;
      const int nb = mk ? std::min(kDuffyMaxWavenumbers, nk - q0) : 1;
      if (mk)
        e = launch_near_duffy_multi(op->G, op->P, cs, pt, et, dpairs->as<NearPair>(), (int)kv.second.size(),
                                    dgx->as<double>(), dgw->as<double>(), n1, nb, kre + q0, kim + q0, out + q0, B, s);
      else
        e = launch_near_duffy(op->G, op->P, op->cplx, cs, pt, et, dpairs->as<NearPair>(), (int)kv.second.size(),
                              dgx->as<double>(), dgw->as<double>(), n1, kre[q0], kim[q0], out[q0], B, s);
      q0 += nb;
    }
    if ((st = cuda_status(op->ctx, e, "near-field singular pairs")) != BG_OK) {
      cleanup();
      return st;
    }
  }
  cudaError_t e = cudaStreamSynchronize(s);
  cleanup();
  return cuda_status(op->ctx, e, "near-field assembly");
}

static void fresh_far_fields(bg_operator* op);

static bg_status assemble_near(bg_operator* op) {
  if (op->maxwell()) return assemble_near_mw(op);
  cudaStream_t s = op->ctx->stream;
  const BsrSegment& D = op->dense;
  if (op->vd != 1) return set_error(op->ctx, BG_UNSUPPORTED, "near field of vector operators");
  const size_t bytes = (size_t)D.col.size() * op->block_stride(D.B) * op->scalar_bytes(false);
  BG_CHECK(op->d_dense64.alloc(bytes), "near-field storage");
  // a near field prepared for this wavenumber (bg_operator_prepare_wavenumbers)
  for (const auto& c : op->near_cache)
    if (c.kre == op->kre && c.kim == op->kim && c.blocks->bytes == bytes) {
      BG_CHECK(cudaMemcpyAsync(op->d_dense64.p, c.blocks->p, bytes, cudaMemcpyDeviceToDevice, s), "near field");
      BG_CHECK(cudaStreamSynchronize(s), "near field");
      return BG_OK;
    }
  BG_CHECK(cudaMemsetAsync(op->d_dense64.p, 0, bytes, s), "near-field storage");
  const NearWork w = near_work(op);
  op->near_pairs = w.npairs;
  void* out = op->d_dense64.p;
  return near_quadrature(op, w, 1, &op->kre, &op->kim, &out);
}

extern "C" bg_status bg_operator_quadrature_counts(const bg_operator* op, long* counts8) {
  if (!op || !counts8) return BG_INVALID_ARG;
  for (int i = 0; i < 8; ++i) counts8[i] = 0;
  if (op->maxwell() || op->vd != 1)
    return set_error(op->ctx, BG_UNSUPPORTED, "quadrature counts: scalar operators only");
  const NearWork w = near_work(op);
  for (const auto& kv : w.regular) {
    const long q = (long)(kv.first + 1) * (kv.first + 1);
    counts8[0] += (long)kv.second.size();
    counts8[1] += (long)kv.second.size() * q * q;
  }
  // point pairs per (outer, inner) Gauss sample of the reference's rules:
  // identical 8 (integrate2.hpp), common edge 6 (integrate3.hpp), common vertex 4 (integrate4.hpp)
  for (const auto& kv : w.singular) {
    const int cs = kv.first.first;
    const long q = (long)(kv.first.second + 1) * (kv.first.second + 1);
    const int slot = cs == 2 ? 2 : (cs == 3 ? 4 : 6);
    const long per = cs == 2 ? 8 : (cs == 3 ? 6 : 4);
    counts8[slot] += (long)kv.second.size();
    counts8[slot + 1] += (long)kv.second.size() * q * q * per;
  }
  return BG_OK;
}

extern "C" bg_status bg_operator_prepare_wavenumbers(bg_operator* op, const double* kre, const double* kim, int n) {
  if (!op || n < 0 || (n > 0 && (!kre || !kim))) return BG_INVALID_ARG;
  if (op->ctx->device < 0) return set_error(op->ctx, BG_UNSUPPORTED, "host-only context: assembly needs a GPU");
  if (!op->cplx || op->maxwell() || op->vd != 1)
    return set_error(op->ctx, BG_UNSUPPORTED, "prepared wavenumbers: Helmholtz single layer only");
  for (int q = 0; q < n; ++q)
    if (!std::isfinite(kre[q]) || !std::isfinite(kim[q]))
      return set_error(op->ctx, BG_INVALID_ARG, "prepared wavenumbers: wavenumbers must be finite");
  cudaSetDevice(op->ctx->device);
  cudaStream_t s = op->ctx->stream;
  auto t0 = std::chrono::steady_clock::now();
  const size_t bytes = (size_t)op->dense.col.size() * op->block_stride(op->dense.B) * op->scalar_bytes(false);
  std::vector<DevBuf*> bufs;
  std::vector<void*> outs;
  auto drop = [&]() {
    for (auto b : bufs) delete b;
  };
  for (int q = 0; q < n; ++q) {
    DevBuf* b = new DevBuf();
    bufs.push_back(b);
    cudaError_t e = b->alloc(bytes);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->p, 0, bytes, s);
    if (e != cudaSuccess) {
      drop();
      return cuda_status(op->ctx, e, "prepared near fields");
    }
    outs.push_back(b->p);
  }
  if (n > 0) {
    const NearWork w = near_work(op);
    op->near_pairs = w.npairs;
    bg_status st = near_quadrature(op, w, n, kre, kim, outs.data());
    if (st != BG_OK) {
      drop();
      return st;
    }
  }
  for (int q = 0; q < n; ++q) {
    // replace an entry of the same wavenumber
    for (size_t i = 0; i < op->near_cache.size(); ++i)
      if (op->near_cache[i].kre == kre[q] && op->near_cache[i].kim == kim[q]) {
        delete op->near_cache[i].blocks;
        op->near_cache.erase(op->near_cache.begin() + i);
        break;
      }
    op->near_cache.push_back({kre[q], kim[q], bufs[q]});
  }
  op->t_prepare = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return BG_OK;
}

extern "C" bg_status bg_operator_release_wavenumbers(bg_operator* op) {
  if (!op) return BG_INVALID_ARG;
  for (auto& c : op->near_cache) delete c.blocks;
  op->near_cache.clear();
  if (!op->kslots.empty()) {
    op->drop_graphs();
    op->free_slots();
    fresh_far_fields(op);
    op->assembled = false;
  }
  return BG_OK;
}

extern "C" bg_status bg_operator_assemble(bg_operator* op);

// Batched products in one pass over all wavenumbers: right-hand-side tile
// buffers per (wavenumber, level) and the far-field work list over those
// indexes (every row of every wavenumber, heaviest first as in the
// one-wavenumber list). Left unset, so that low-precision products go one
// wavenumber at a time, when a wavenumber has no tiles or the indexes exceed
// the tile bound.
static bg_status setup_kbatch(bg_operator* op) {
  const int nk = (int)op->kslots.size(), nlev = op->leaf_level + 1, np2 = op->np * op->np;
  op->kb_nwork = 0;
  if (op->n_far_work == 0 || nk * nlev > kMaxTileLevels) return BG_OK;
  for (const auto& k : op->kslots)
    if (!k.far_tiles) return BG_OK;
  const size_t tb = far_h16c_btile_bytes(np2);
  if (tb == 0) return BG_OK;
  for (int q = 0; q < nk; ++q)
    for (int l = 0; l < nlev; ++l) {
      op->kb_btiles.push_back(new DevBuf());
      op->kb_binv.push_back(new DevBuf());
      BG_CHECK(op->kb_btiles.back()->alloc(tb * op->nclusters(l)), "batched right-hand-side tiles");
      BG_CHECK(op->kb_binv.back()->alloc(sizeof(float) * 32 * op->nclusters(l)), "batched right-hand-side tiles");
    }
  std::vector<int2> base(op->n_far_work), work;
  BG_CHECK(cudaMemcpy(base.data(), op->d_far_work.p, base.size() * sizeof(int2), cudaMemcpyDeviceToHost),
           "far-field work list");
  work.reserve(base.size() * nk);
  for (const int2& it : base)
    for (int q = 0; q < nk; ++q) work.push_back(make_int2(q * nlev + it.x, it.y));
  BG_CHECK(op->kb_work.upload(work, op->ctx->stream), "far-field work list");
  BG_CHECK(cudaStreamSynchronize(op->ctx->stream), "far-field work list");
  op->kb_nwork = (int)work.size();
  return BG_OK;
}

extern "C" bg_status bg_operator_assemble_wavenumbers(bg_operator* op) {
  if (!op) return BG_INVALID_ARG;
  if (op->ctx->device < 0) return set_error(op->ctx, BG_UNSUPPORTED, "host-only context: assembly needs a GPU");
  if (!op->cplx || op->maxwell() || op->vd != 1)
    return set_error(op->ctx, BG_UNSUPPORTED, "batched wavenumbers: Helmholtz single layer only");
  if (op->near_cache.empty())
    return set_error(op->ctx, BG_INVALID_ARG, "batched wavenumbers: prepare the wavenumbers first");
  std::vector<std::pair<double, double>> ks;
  for (const auto& c : op->near_cache) ks.emplace_back(c.kre, c.kim);
  const double kre0 = op->kre, kim0 = op->kim;
  std::vector<bg_operator::KSlot> slots;
  auto fail = [&](bg_status st) {
    for (auto& k : slots)
      for (auto v : {&k.far64, &k.far_df, &k.atiles, &k.ainv})
        for (auto b : *v) delete b;
    op->kre = kre0;
    op->kim = kim0;
    op->assembled = false;
    return st;
  };
  double t_far = 0, t_near = 0;
  for (const auto& k : ks) {
    op->kre = k.first;
    op->kim = k.second;
    bg_status st = bg_operator_assemble(op);  // copies the prepared near field, assembles the far field
    if (st != BG_OK) return fail(st);
    t_far += op->t_far;
    t_near += op->t_near;
    bg_operator::KSlot slot;
    slot.kre = k.first;
    slot.kim = k.second;
    std::swap(slot.dense64, op->d_dense64);
    std::swap(slot.dense32, op->d_dense32);
    std::swap(slot.far64, op->d_far64);
    std::swap(slot.far_df, op->d_far_df);
    std::swap(slot.atiles, op->d_far_atiles);
    std::swap(slot.ainv, op->d_far_ainv);
    slot.far_tiles = op->far_tiles;
    fresh_far_fields(op);
    // the prepared copy of this near field is no longer needed
    for (size_t i = 0; i < op->near_cache.size(); ++i)
      if (op->near_cache[i].kre == k.first && op->near_cache[i].kim == k.second) {
        delete op->near_cache[i].blocks;
        op->near_cache.erase(op->near_cache.begin() + i);
        break;
      }
    slots.push_back(std::move(slot));
  }
  op->drop_graphs();
  op->kslots = std::move(slots);
  op->kslot_active = -1;
  op->kre = kre0;
  op->kim = kim0;
  if (bg_status st = setup_kbatch(op)) {
    op->free_slots();
    op->assembled = false;
    return st;
  }
  op->t_far = t_far;
  op->t_near = t_near;
  op->t_total = t_far + t_near;
  op->assembled = true;
  return BG_OK;
}

extern "C" bg_status bg_operator_num_wavenumbers(const bg_operator* op, int* n, double* kre, double* kim) {
  if (!op || !n) return BG_INVALID_ARG;
  *n = (int)op->kslots.size();
  for (int q = 0; q < *n; ++q) {
    // the active slot's wavenumber sits in the operator while it is swapped in
    const bool act = q == op->kslot_active;
    if (kre) kre[q] = act ? op->kre : op->kslots[q].kre;
    if (kim) kim[q] = act ? op->kim : op->kslots[q].kim;
  }
  return BG_OK;
}

// the per-level far-field buffers of the current wavenumber, empty (after
// they moved into a wavenumber slot or the slots were freed)
static void fresh_far_fields(bg_operator* op) {
  const size_t L = op->d_pts64.size();
  for (auto v : {&op->d_far64, &op->d_far_df, &op->d_far_atiles, &op->d_far_ainv}) {
    for (auto b : *v) delete b;
    v->clear();
    for (size_t l = 0; l < L; ++l) v->push_back(new DevBuf());
  }
  op->far_tiles = false;
  op->d_dense64.release();
  op->d_dense32.release();
}

extern "C" bg_status bg_operator_assemble(bg_operator* op) {
  if (!op) return BG_INVALID_ARG;
  if (op->ctx->device < 0) return set_error(op->ctx, BG_UNSUPPORTED, "host-only context: assembly needs a GPU");
  if (op->maxwell() && (op->P < 1 || op->P > 3))
    return set_error(op->ctx, BG_UNSUPPORTED, "the Maxwell operator needs a polynomial degree in [1, 3]");
  if (op->maxwell() && op->kre == 0.0 && op->kim == 0.0)
    return set_error(op->ctx, BG_INVALID_ARG, "the Maxwell operator needs a nonzero wavenumber");
  cudaSetDevice(op->ctx->device);
  op->assembled = false;
  op->drop_graphs();  // assembly may move the stored fields
  if (!op->kslots.empty()) {
    op->free_slots();
    fresh_far_fields(op);
  }
  auto t0 = std::chrono::steady_clock::now();
  bg_status st = assemble_far(op);
  if (st != BG_OK) return st;
  auto t1 = std::chrono::steady_clock::now();
  st = assemble_near(op);
  if (st != BG_OK) return st;
  {
    // FP32 copy of the near field for BG_PREC_FP32 products
    const long nb = (long)op->dense.col.size(), B = op->dense.B;
    cudaError_t e = op->d_dense32.alloc((size_t)nb * op->block_stride32((int)B) * op->scalar_bytes(true));
    if (e == cudaSuccess)
      e = launch_convert_blocks(op->cplx, op->d_dense64.p, op->block_stride((int)B), op->d_dense32.p,
                                op->block_stride32((int)B), B * B, nb, op->ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(op->ctx->stream);
    if ((st = cuda_status(op->ctx, e, "FP32 near field")) != BG_OK) return st;
    // (hi, lo) FP32 pairs of the real blocks: the FP64-accurate near field of
    // BG_PREC_MIXED products runs on the FP32 pipes
    if (!op->cplx && nb > 0) {
      const long n = nb * op->block_stride((int)B);
      e = op->d_dense_df.alloc((size_t)n * sizeof(float2));
      if (e == cudaSuccess) e = launch_split_df(op->d_dense64.p, n, op->d_dense_df.p, op->ctx->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(op->ctx->stream);
      if ((st = cuda_status(op->ctx, e, "double-float near field")) != BG_OK) return st;
    }
    // integer digits of the real blocks for the tensor-core near field of
    // BG_PREC_MIXED products (and their per-product scratch: x digit panels,
    // zero where no digit is written, and column exponents)
    if (!op->cplx && nb > 0 && oz_supported((int)B) && (long)op->dense.nrows * B == (long)op->S) {
      const int nrows = op->dense.nrows;
      e = op->d_oz_tiles.alloc(oz_tile_bytes((int)B, nb));
      if (e == cudaSuccess) e = op->d_oz_rexp.alloc((size_t)nrows * B * sizeof(int));
      if (e == cudaSuccess) e = op->w_oz_panels.alloc(oz_panel_bytes((int)B, op->S / B));
      if (e == cudaSuccess) e = op->w_oz_fmax.alloc(32 * sizeof(int));
      if (e == cudaSuccess) e = cudaMemsetAsync(op->w_oz_panels.p, 0, op->w_oz_panels.bytes, op->ctx->stream);
      if (e == cudaSuccess)
        e = launch_oz_build(op->dense.d_row_ptr.as<int>(), op->d_dense64.as<double>(), op->block_stride((int)B), nrows,
                            (int)B, op->d_oz_rexp.as<int>(), op->d_oz_tiles.p, nb, op->ctx->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(op->ctx->stream);
      if ((st = cuda_status(op->ctx, e, "tensor-core near field digits")) != BG_OK) return st;
    }
  }
  auto t2 = std::chrono::steady_clock::now();
  op->t_far = std::chrono::duration<double>(t1 - t0).count();
  op->t_near = std::chrono::duration<double>(t2 - t1).count();
  op->t_total = op->t_far + op->t_near;
  op->assembled = true;
  return BG_OK;
}

// ---------------------------------------------------------------------------
bg_status ensure_work(bg_operator* op, int nrhs) {
  if (nrhs <= op->cap) return BG_OK;
  op->drop_graphs();  // the buffers below move
  const size_t sb = op->scalar_bytes(false);  // FP64 sizes cover the FP32 path
  BG_CHECK(op->w_xdof.alloc((size_t)op->N * nrhs * sb), "work vectors");
  BG_CHECK(op->w_ydof.alloc((size_t)op->N * nrhs * sb), "work vectors");
  BG_CHECK(op->w_xss.alloc((size_t)op->S * nrhs * sb), "work vectors");
  BG_CHECK(op->w_yss.alloc((size_t)op->S * nrhs * sb), "work vectors");
  BG_CHECK(op->w_xss32.alloc((size_t)op->S * nrhs * sb / 2), "work vectors");
  BG_CHECK(op->w_yss32.alloc((size_t)op->S * nrhs * sb / 2), "work vectors");
  if (!op->cplx) BG_CHECK(op->w_xss_df.alloc((size_t)op->S * nrhs * sizeof(float2)), "work vectors");
  while ((int)op->w_y.size() <= op->leaf_level) {
    op->w_y.push_back(new DevBuf());
    op->w_z.push_back(new DevBuf());
    op->w_ydf.push_back(new DevBuf());
    op->w_btiles.push_back(new DevBuf());
    op->w_binv.push_back(new DevBuf());
    op->w_yv.push_back(new DevBuf());
    op->w_zv.push_back(new DevBuf());
  }
  for (int l = 0; l <= op->leaf_level; ++l) {
    const size_t n = (size_t)op->vd * op->nclusters(l) * op->R * nrhs * sb;
    BG_CHECK(op->w_y[l]->alloc(n), "work vectors");
    BG_CHECK(op->w_z[l]->alloc(n), "work vectors");
    // double-float split of y (complex: 16 columns at a time)
    BG_CHECK(op->w_ydf[l]->alloc(op->cplx ? (size_t)op->nclusters(l) * op->np * op->np * 32 * sizeof(float2) : n),
             "work vectors");
    const size_t tb = op->cplx ? far_h16c_btile_bytes(op->np * op->np) : far_h16_btile_bytes(op->np * op->np);
    if (op->maxwell()) {
      const size_t nv = (size_t)op->nclusters(l) * op->np * op->np * 4 * std::min(nrhs, (int)bg_operator::kMwRhsChunk) * sb;
      BG_CHECK(op->w_yv[l]->alloc(nv), "work vectors");
      BG_CHECK(op->w_zv[l]->alloc(nv), "work vectors");
    }
    if (tb > 0) {
      BG_CHECK(op->w_btiles[l]->alloc(tb * op->nclusters(l)), "work vectors");
      BG_CHECK(op->w_binv[l]->alloc(sizeof(float) * 32 * op->nclusters(l)), "work vectors");
    }
  }
  if (op->fmm_fused) {
    // arrival counters of the fused upward pass: parents at levels
    // 0 .. L - 2, per 32-column chunk of the widest product (complex: 2 nrhs)
    const int chunks = ((op->cplx ? 2 : 1) * nrhs + 31) / 32;
    long stride = 0;
    for (int l = 0; l + 2 <= op->leaf_level; ++l) {
      op->fmm_cnt_off[l] = stride;
      stride += op->nclusters(l);
    }
    op->fmm_cnt_stride = stride;
    if (stride > 0) {
      BG_CHECK(op->d_fmm_cnt.alloc((size_t)chunks * stride * sizeof(int)), "work vectors");
      BG_CHECK(cudaMemsetAsync(op->d_fmm_cnt.p, 0, (size_t)chunks * stride * sizeof(int), op->ctx->stream),
               "work vectors");
    }
    op->fmm_cnt_chunks = chunks;
  }
  op->cap = nrhs;
  return BG_OK;
}

// Tables of the fused FMM transforms for one product: x / out the
// superspace panels, y / z the level coefficients of the operator's work
// vectors, kk real columns (complex vectors: 2 per right-hand side).
template <typename T>
static void fill_fmm(const bg_operator* op, const void* fac, int kk, const void* x, void* out, FmmLevels<T>* f) {
  f->fac = static_cast<const T*>(fac);
  f->cmap = op->d_fmm_cmap.as<int>();
  f->x = static_cast<const T*>(x);
  f->out = static_cast<T*>(out);
  for (int l = 0; l <= op->leaf_level; ++l) {
    f->y[l] = static_cast<T*>(op->w_y[l]->p);
    f->z[l] = static_cast<const T*>(op->w_z[l]->p);
  }
  f->cnt = op->d_fmm_cnt.as<int>();
  for (int l = 0; l < kMaxFarLevels; ++l) f->cnt_off[l] = op->fmm_cnt_off[l];
  f->cnt_stride = op->fmm_cnt_stride;
  f->np = op->np;
  f->w1 = op->fmm_w1;
  f->Bq = op->Bq;
  f->L = op->leaf_level;
  f->kk = kk;
}

// One H2 product on row-major FP64 work vectors (H2DenseProduct.hpp:33-165).
// The product between T x and T^T y: superspace x in w_xss to superspace y in
// w_yss, only on the operator's own work buffers (so it can be captured as a
// CUDA graph and replayed).
static bg_status apply_middle(bg_operator* op, int nrhs, int prec) {
  cudaStream_t s = op->ctx->stream;
  const bool mixed = prec != BG_PREC_FP64;   // far field and transforms in FP32
  const bool near32 = prec == BG_PREC_FP32;  // near field in FP32 too
  const int S64 = op->stype(false), Sfar = op->stype(mixed);
  const size_t sfar = op->scalar_bytes(mixed);
  const int np2 = op->np * op->np;
  const long ss_n = (long)op->S * nrhs;
  const bg_launch_plan pl = op->plan_for(nrhs, prec);
  bool any_far = false;
  for (const auto& f : op->far) any_far |= !f.col.empty();
  if (op->kbatched()) {
    // batched wavenumbers: wavenumber q's near field on column block q (the
    // block is copied out of the row-major superspace vectors and back)
    const int nk = (int)op->kslots.size(), nr = nrhs / nk;
    if (near32)
      BG_CHECK(timed_launch(op->ctx, KC_OTHER, [&] { return launch_convert(S64, Sfar, op->w_xss.p, ss_n, op->w_xss32.p, s); }), "x to FP32");
    const size_t es = op->scalar_bytes(near32);
    const char* xs = static_cast<const char*>(near32 ? op->w_xss32.p : op->w_xss.p);
    char* ys = static_cast<char*>(near32 ? op->w_yss32.p : op->w_yss.p);
    for (int q = 0; q < nk; ++q) {
      BG_CHECK(cudaMemcpy2DAsync(op->kb_xs.p, nr * es, xs + (size_t)q * nr * es, (size_t)nrhs * es, nr * es, op->S,
                                 cudaMemcpyDeviceToDevice, s), "near-field column block");
      const bg_operator::KSlot& k = op->kslots[q];
      BG_CHECK(timed_launch(op->ctx, KC_NEAR, [&] {
                 return near32 ? launch_bsr_fp32(true, op->dense.d_row_ptr.as<int>(), op->dense.d_col.as<int>(), k.dense32.p,
                                                 op->block_stride32(op->dense.B), op->dense.nrows, op->dense.B,
                                                 op->kb_xs.p, op->kb_ys.p, nr, 0, s, pl.near_kernel)
                               : launch_bsr_fp64(true, op->dense.d_row_ptr.as<int>(), op->dense.d_col.as<int>(), k.dense64.p,
                                                 op->block_stride(op->dense.B), op->dense.nrows, op->dense.B,
                                                 op->kb_xs.p, op->kb_ys.p, nr, 0, s); }),
               "near-field product (batched wavenumbers)");
      BG_CHECK(cudaMemcpy2DAsync(ys + (size_t)q * nr * es, (size_t)nrhs * es, op->kb_ys.p, nr * es, nr * es, op->S,
                                 cudaMemcpyDeviceToDevice, s), "near-field column block");
    }
  } else if (near32) {
    // FP32 near field into the FP32 accumulator the far field adds to
    BG_CHECK(timed_launch(op->ctx, KC_OTHER, [&] { return launch_convert(S64, Sfar, op->w_xss.p, ss_n, op->w_xss32.p, s); }), "x to FP32");
    BG_CHECK(timed_launch(op->ctx, KC_NEAR, [&] { return launch_bsr_fp32(op->cplx, op->dense.d_row_ptr.as<int>(), op->dense.d_col.as<int>(), op->d_dense32.p,
                        op->block_stride32(op->dense.B), op->dense.nrows, op->dense.B, op->w_xss32.p, op->w_yss32.p, nrhs, 0, s, pl.near_kernel); }),
             "near-field product (FP32)");
  } else if (mixed && !op->cplx && op->d_oz_tiles.p && pl.mixed_near == 0) {
    // FP64-accurate near field on the tensor cores: 8 integer digits of 7
    // bits per operand, exact integer accumulation, one rounding at the end
    BG_CHECK(timed_launch(op->ctx, KC_NEAR, [&] {
               return launch_near_oz(op->dense.d_row_ptr.as<int>(), op->dense.d_col.as<int>(), op->dense.nrows,
                                     op->dense.B, op->d_oz_tiles.p, op->d_oz_rexp.as<int>(), op->w_xss.as<double>(),
                                     op->S, nrhs, op->w_oz_panels.p, op->w_oz_fmax.as<int>(), op->w_yss.as<double>(),
                                     nrhs, nrhs, op->d_err.as<int>(), s); }),
             "near-field product (tensor cores, integer digits)");
  } else if (mixed && !op->cplx && op->d_dense_df.p) {
    // FP64-accurate near field in double-float: blocks and x as FP32 (hi, lo)
    // pairs, exact products and compensated sums (about 1e-14 relative)
    BG_CHECK(timed_launch(op->ctx, KC_OTHER, [&] { return launch_split_df(op->w_xss.p, ss_n, op->w_xss_df.p, s); }),
             "near-field split of x");
    // launch plan: 32 columns with a quarter of them on the FP64 pipe, the
    // rest in double-float
    const bool both_pipes = pl.mixed_near == 2 && nrhs == 32 && op->dense.B <= 42;
    BG_CHECK(timed_launch(op->ctx, KC_NEAR, [&] {
               return both_pipes
                          ? launch_bsr_near_mix(op->dense.d_row_ptr.as<int>(), op->dense.d_col.as<int>(), op->d_dense_df.p,
                                                op->d_dense64.p, op->block_stride(op->dense.B), op->dense.nrows, op->dense.B,
                                                op->w_xss_df.p, op->w_xss.p, op->w_yss.p, s)
                          : launch_bsr_df(op->dense.d_row_ptr.as<int>(), op->dense.d_col.as<int>(), op->d_dense_df.p,
                                          op->block_stride(op->dense.B), op->dense.nrows, op->dense.B, op->w_xss_df.p,
                                          op->w_yss.p, nrhs, 0, s); }),
             "near-field product (double-float)");
  } else {
    BG_CHECK(timed_launch(op->ctx, KC_NEAR, [&] { return launch_bsr_fp64(op->cplx, op->dense.d_row_ptr.as<int>(), op->dense.d_col.as<int>(), op->d_dense64.p,
                        op->block_stride(op->dense.B), op->dense.nrows, op->dense.B, op->w_xss.p, op->w_yss.p, nrhs, 0, s); }),
             "near-field product");
  }
  if (any_far) {
    const long comp_ss = (long)op->ne * op->p2;  // superspace rows per vector component
    const void* xfar = op->w_xss.p;
    void* yfar = op->w_yss.p;
    if (mixed) {
      if (!near32) {
        BG_CHECK(timed_launch(op->ctx, KC_OTHER, [&] { return launch_convert(S64, Sfar, op->w_xss.p, ss_n, op->w_xss32.p, s); }), "x to FP32");
        BG_CHECK(cudaMemsetAsync(op->w_yss32.p, 0, ss_n * sfar, s), "far field");
      }
      xfar = op->w_xss32.p;
      yfar = op->w_yss32.p;
    }
    const int Ll = op->leaf_level;
    const bg_operator::TransformMats& tm = op->tm[mixed ? 1 : 0];
    // Maxwell moment blocks phi, d/ds phi, d/dt phi (np2 x Bq, row-major) for the generic path
    const size_t rsz = mixed ? sizeof(float) : sizeof(double);
    auto mw_mom = [&](int c) -> const void* {
      const char* base = static_cast<const char*>(mixed ? op->d_mom32[c == 2 ? 1 : 0]->p : op->d_mom64[c == 2 ? 1 : 0]->p);
      return base + (c == 0 ? 0 : (size_t)np2 * op->Bq * rsz);
    };
    const char* xc0 = static_cast<const char*>(xfar);
    const char* xc1 = xc0 + comp_ss * nrhs * sfar;
    if (op->maxwell()) {
      // three channels: tangential part of each component, divergence of both
      const size_t chl = (size_t)op->nleaf_cl * np2 * nrhs * sfar;
      char* yl = static_cast<char*>(op->w_y[Ll]->p);
      // tangential channels of both components in one batch: the two components'
      // leaf panels are consecutive in x (component-major) and so are the channels
      const char* xin[3] = {xc0, xc0, xc1};
      char* yout[3] = {yl, yl + 2 * chl, yl + 2 * chl};
      const int blk[3] = {0, 1, 2}, nb[3] = {2 * op->nleaf_cl, op->nleaf_cl, op->nleaf_cl};
      for (int t = 0; t < 3; ++t)
        BG_CHECK(timed_launch(op->ctx, KC_TRANSFORM, [&] {
                   return op->use_tgemm
                              ? launch_tgemm(Sfar, t == 2, tm.a_mw_f[blk[t]], xin[t], op->Bq, yout[t], np2, nb[t], nrhs, s, pl.split_k_batches)
                              : launch_moment_fwd_acc(Sfar, t == 2, mw_mom(blk[t]), np2, op->Bq, nb[t], xin[t],
                                                      yout[t], nrhs, s); }),
                 "forward moments");
      for (int l = Ll - 1; l >= 0; --l) {
        const int nb = 3 * op->nclusters(l);
        BG_CHECK(timed_launch(op->ctx, KC_TRANSFORM, [&] {
                   return op->use_tgemm ? launch_tgemm(Sfar, false, tm.a_tr_f, op->w_y[l + 1]->p, 4L * np2, op->w_y[l]->p, np2, nb, nrhs, s, pl.split_k_batches)
                                        : launch_transfer_fwd(Sfar, mixed ? op->d_tr32.p : op->d_tr64.p, np2, 1, nb,
                                                              op->w_y[l + 1]->p, op->w_y[l]->p, nrhs, s); }),
                 "forward transfer");
      }
    }
    // scalar operators: one fused launch per direction through the
    // tensor-product factors, unless the plan asks for the batched GEMMs
    const bool fused_tr = !op->maxwell() && op->fmm_fused && pl.transforms == 0 &&
                          ((op->cplx ? 2 : 1) * nrhs + 31) / 32 <= op->fmm_cnt_chunks;
    FmmLevelsAny fa{};
    if (fused_tr) {
      const int kk = (op->cplx ? 2 : 1) * nrhs;
      if (mixed) fill_fmm<float>(op, op->d_fmm_fac32.p, kk, xc0, yfar, &fa.f32);
      else fill_fmm<double>(op, op->d_fmm_fac64.p, kk, xc0, yfar, &fa.f64);
      BG_CHECK(timed_launch(op->ctx, KC_TRANSFORM, [&] { return launch_fmm_up(Sfar, fa, op->fmm_hfac.data(), op->nclusters(Ll - 1), s); }),
               "forward transforms (fused)");
    }
    for (int c = 0; c < op->vd && !op->maxwell() && !fused_tr; ++c) {
      const void* mom = mixed ? op->d_mom32[c]->p : op->d_mom64[c]->p;
      const char* xc = c == 0 ? xc0 : xc1;
      char* yl = static_cast<char*>(op->w_y[Ll]->p) + (size_t)c * op->nleaf_cl * op->R * nrhs * sfar;
      BG_CHECK(timed_launch(op->ctx, KC_TRANSFORM, [&] {
                 return op->use_tgemm ? launch_tgemm(Sfar, false, tm.a_mom_f[c], xc, op->Bq, yl, op->R, op->nleaf_cl, nrhs, s, pl.split_k_batches)
                                      : launch_moment_fwd(Sfar, mom, op->R, op->Bq, op->nleaf_cl, xc, yl, nrhs, s); }),
               "forward moments");
      for (int l = Ll - 1; l >= 0; --l) {
        const int ncl = op->nclusters(l);
        const char* ych = static_cast<const char*>(op->w_y[l + 1]->p) + (size_t)c * 4 * ncl * op->R * nrhs * sfar;
        char* ypa = static_cast<char*>(op->w_y[l]->p) + (size_t)c * ncl * op->R * nrhs * sfar;
        BG_CHECK(timed_launch(op->ctx, KC_TRANSFORM, [&] {
                   return op->use_tgemm ? launch_tgemm(Sfar, false, tm.a_tr_f, ych, 4L * op->R, ypa, op->R, ncl, nrhs, s, pl.split_k_batches)
                                        : launch_transfer_fwd(Sfar, mixed ? op->d_tr32.p : op->d_tr64.p, np2, op->nc, ncl,
                                                              ych, ypa, nrhs, s); }),
                 "forward transfer");
      }
    }
    const bool tc = mixed && op->vd == 1 && op->nc == 1 && op->leaf_level < kMaxFarLevels &&
                    far_tc_supported(op->cplx, np2, nrhs);
    const bool tcc = mixed && op->cplx && op->far_tiles && op->leaf_level < kMaxFarLevels;
    const bool tcc_kb = mixed && op->kbatched() && op->kb_nwork > 0;
    if (tcc_kb) {
      // batched wavenumbers: one launch per 16 columns covers every
      // wavenumber's stored tiles (level index q (L + 1) + l), each applied
      // to its own column block of Y
      const int nk = (int)op->kslots.size(), nr = nrhs / nk, nlev = op->leaf_level + 1;
      FarH16Tiles T{};
      for (int q = 0; q < nk; ++q)
        for (int l = 0; l < nlev; ++l) {
          const int v = q * nlev + l;
          T.row_ptr[v] = op->far[l].d_row_ptr.as<int>();
          T.col[v] = op->far[l].d_col.as<int>();
          T.a[v] = static_cast<const unsigned char*>(op->kslots[q].atiles[l]->p);
          T.ainv[v] = op->kslots[q].ainv[l]->as<float>();
          T.b[v] = static_cast<unsigned char*>(op->kb_btiles[v]->p);
          T.binv[v] = op->kb_binv[v]->as<float>();
          T.y[v] = reinterpret_cast<const float*>(static_cast<const char*>(op->w_y[l]->p) + (size_t)q * nr * sfar);
          T.z[v] = reinterpret_cast<float*>(static_cast<char*>(op->w_z[l]->p) + (size_t)q * nr * sfar);
          T.ncl[v] = op->nclusters(l);
        }
      for (int c0 = 0; c0 < nr; c0 += 16) {
        const int nc = std::min(16, nr - c0);
        BG_CHECK(timed_launch(op->ctx, KC_OTHER, [&] { return launch_build_h16c_btiles(T, nk * nlev, np2, nrhs, c0, nc, s); }),
                 "right-hand-side tiles");
        BG_CHECK(timed_launch(op->ctx, KC_FAR_FUSED, [&] { return launch_far_h16c(T, op->kb_work.as<int2>(), op->kb_nwork,
                                                                           np2, nrhs, c0, nc, op->d_err.as<int>(), s); }),
                 "far-field product (batched wavenumbers, stored complex FP16 tiles, tensor cores)");
      }
    } else if (tc && op->far_tiles) {
      // stored FP16 tiles streamed by TMA bulk copies; all levels in one
      // launch, which writes every row of Z
      FarH16Tiles T{};
      for (int l = 0; l <= op->leaf_level; ++l) {
        T.row_ptr[l] = op->far[l].d_row_ptr.as<int>();
        T.col[l] = op->far[l].d_col.as<int>();
        T.a[l] = static_cast<const unsigned char*>(op->d_far_atiles[l]->p);
        T.ainv[l] = op->d_far_ainv[l]->as<float>();
        T.b[l] = static_cast<unsigned char*>(op->w_btiles[l]->p);
        T.binv[l] = op->w_binv[l]->as<float>();
        T.y[l] = static_cast<const float*>(op->w_y[l]->p);
        T.z[l] = static_cast<float*>(op->w_z[l]->p);
        T.ncl[l] = op->nclusters(l);
      }
      BG_CHECK(timed_launch(op->ctx, KC_OTHER, [&] { return launch_build_h16_btiles(T, op->leaf_level + 1, np2, nrhs, s); }),
               "right-hand-side tiles");
      BG_CHECK(timed_launch(op->ctx, KC_FAR_FUSED, [&] { return launch_far_h16(T, op->far_work(pl.far_order), op->n_far_work,
                                                                       np2, nrhs, op->d_err.as<int>(), s, pl.far_ctas,
                                                                       pl.far_tiles == 1); }),
               "far-field product (stored FP16 tiles, tensor cores)");
    } else if (tcc) {
      // complex kernel: stored FP16 tiles of Re K and Im K, 16 complex columns
      // per launch, all levels per launch (every row of Z written). Maxwell
      // applies K to the four kernel columns of every right-hand side.
      FarH16Tiles T{};
      for (int l = 0; l <= op->leaf_level; ++l) {
        T.row_ptr[l] = op->far[l].d_row_ptr.as<int>();
        T.col[l] = op->far[l].d_col.as<int>();
        T.a[l] = static_cast<const unsigned char*>(op->d_far_atiles[l]->p);
        T.ainv[l] = op->d_far_ainv[l]->as<float>();
        T.b[l] = static_cast<unsigned char*>(op->w_btiles[l]->p);
        T.binv[l] = op->w_binv[l]->as<float>();
        T.y[l] = static_cast<const float*>(op->maxwell() ? op->w_yv[l]->p : op->w_y[l]->p);
        T.z[l] = static_cast<float*>(op->maxwell() ? op->w_zv[l]->p : op->w_z[l]->p);
        T.ncl[l] = op->nclusters(l);
      }
      const int nlev = op->leaf_level + 1;
      auto product = [&](int ld, int c0, int nc) -> bg_status {
        BG_CHECK(timed_launch(op->ctx, KC_OTHER, [&] { return launch_build_h16c_btiles(T, nlev, np2, ld, c0, nc, s); }),
                 "right-hand-side tiles");
        BG_CHECK(timed_launch(op->ctx, KC_FAR_FUSED, [&] { return launch_far_h16c(T, op->far_work(pl.far_order), op->n_far_work,
                                                                           np2, ld, c0, nc, op->d_err.as<int>(), s); }),
                 "far-field product (stored complex FP16 tiles, tensor cores)");
        return BG_OK;
      };
      bg_status st;
      if (!op->maxwell()) {
        for (int c0 = 0; c0 < nrhs; c0 += 16)
          if ((st = product(nrhs, c0, std::min(16, nrhs - c0))) != BG_OK) return st;
      } else {
        const std::complex<double> kap(op->kre, op->kim), mk2 = -1.0 / (kap * kap);
        for (int r0 = 0; r0 < nrhs; r0 += bg_operator::kMwRhsChunk) {
          const int nr = std::min((int)bg_operator::kMwRhsChunk, nrhs - r0);
          for (int l = 0; l <= op->leaf_level; ++l)
            BG_CHECK(timed_launch(op->ctx, KC_OTHER, [&] { return launch_mw_far_in(Sfar, op->nclusters(l), np2, op->w_y[l]->p, nrhs,
                                                                            r0, nr, op->d_tan32[l]->p, op->w_yv[l]->p, s); }),
                     "Maxwell far-field columns");
          for (int c0 = 0; c0 < 4 * nr; c0 += 16)
            if ((st = product(4 * nr, c0, std::min(16, 4 * nr - c0))) != BG_OK) return st;
          for (int l = 0; l <= op->leaf_level; ++l)
            BG_CHECK(timed_launch(op->ctx, KC_OTHER, [&] { return launch_mw_far_out(Sfar, op->nclusters(l), np2, op->w_zv[l]->p, nrhs,
                                                                             r0, nr, op->d_tan32[l]->p, mk2.real(),
                                                                             mk2.imag(), op->w_z[l]->p, s); }),
                     "Maxwell far-field columns");
        }
      }
    } else if (tc) {
      // all levels in one tensor-core launch; it writes every row of Z
      FarTcLevels L{};
      for (int l = 0; l <= op->leaf_level; ++l) {
        L.row_ptr[l] = op->far[l].d_row_ptr.as<int>();
        L.col[l] = op->far[l].d_col.as<int>();
        L.pts[l] = op->d_pts32[l]->as<float4>();
        L.cen[l] = op->d_centres[l]->as<d4>();
        L.y[l] = static_cast<const float*>(op->w_y[l]->p);
        L.z[l] = static_cast<float*>(op->w_z[l]->p);
      }
      BG_CHECK(timed_launch(op->ctx, KC_FAR_FUSED, [&] { return launch_far_tc(L, op->far_work(pl.far_order), op->n_far_work, np2, nrhs,
                                                                      op->d_err.as<int>(), s); }),
               "far-field product (tensor cores)");
    }
    // complex FP64 far product of level l on the double-float pipes: z (rows
    // of ld complex entries) = K y, 16 columns per pass, Kr split(y) + Ki split(i y)
    // (columns cb .. cb + ncols - 1 of rows of ld, with the pairs df)
    auto far64_cplx = [&](int l, const DevBuf* df, const void* y, int ld, int cb, int ncols, void* z) -> bg_status {
      const BsrSegment& f = op->far[l];
      const long sdf = ((long)f.B * f.B + 1) / 2 * 2;
      const float2* kr = df->as<float2>();
      const float2* ki = kr + (long)f.col.size() * sdf;
      const long rows = (long)op->nclusters(l) * f.B;
      for (int c0 = cb; c0 < cb + ncols; c0 += 16) {
        const int nc = std::min(16, cb + ncols - c0);
        for (int part = 0; part < 2; ++part) {
          BG_CHECK(timed_launch(op->ctx, KC_OTHER, [&] { return launch_split_df_cols(y, rows, ld, c0, nc, part,
                                                                                  op->w_ydf[l]->p, s); }),
                   "far-field split of Y");
          BG_CHECK(timed_launch(op->ctx, KC_FAR64, [&] { return launch_bsr_df_cols(f.d_row_ptr.as<int>(), f.d_col.as<int>(),
                                                                            part ? ki : kr, sdf, f.nrows, f.B,
                                                                            op->w_ydf[l]->p, z, 2 * nc, 2 * ld,
                                                                            2 * c0, part, s); }),
                   "far-field product (complex double-float)");
        }
      }
      return BG_OK;
    };
    for (int l = 0; l <= op->leaf_level && !tc && !tcc && !tcc_kb; ++l) {
      const BsrSegment& f = op->far[l];
      if (f.col.empty()) {
        BG_CHECK(cudaMemsetAsync(op->w_z[l]->p, 0, (size_t)op->vd * op->nclusters(l) * op->R * nrhs * sfar, s),
                 "far field");
        continue;
      }
      if (op->maxwell()) {
        // tangential and divergence parts through the scalar kernel matrices,
        // kMwRhsChunk right-hand sides (4 kernel columns each) at a time
        if (!mixed && !op->store_far)
          return set_error(op->ctx, BG_UNSUPPORTED, "the FP64 product needs the stored far field");
        const int ncl = op->nclusters(l);
        const void* tan = mixed ? (const void*)op->d_tan32[l]->p : (const void*)op->d_tan64[l]->p;
        const std::complex<double> kap(op->kre, op->kim), mk2 = -1.0 / (kap * kap);
        for (int r0 = 0; r0 < nrhs; r0 += bg_operator::kMwRhsChunk) {
          const int nr = std::min((int)bg_operator::kMwRhsChunk, nrhs - r0);
          BG_CHECK(timed_launch(op->ctx, KC_OTHER, [&] { return launch_mw_far_in(Sfar, ncl, np2, op->w_y[l]->p, nrhs, r0, nr,
                                                                          tan, op->w_yv[l]->p, s); }),
                   "Maxwell far-field columns");
          if (mixed)
            BG_CHECK(timed_launch(op->ctx, KC_FAR_FUSED, [&] { return launch_far_fused(true, op->d_pts32[l]->as<float4>(), op->d_centres[l]->as<d4>(),
                                      f.d_row_ptr.as<int>(), f.d_col.as<int>(), f.nrows, np2, (float)op->kre, (float)op->kim,
                                      op->w_yv[l]->p, op->w_zv[l]->p, 4 * nr, s); }),
                     "far-field product (FP32 fused, Maxwell)");
          else if (op->d_far_df[l]->p) {
            bg_status st = far64_cplx(l, op->d_far_df[l], op->w_yv[l]->p, 4 * nr, 0, 4 * nr, op->w_zv[l]->p);
            if (st != BG_OK) return st;
          } else
            BG_CHECK(timed_launch(op->ctx, KC_FAR64, [&] { return launch_bsr_fp64(true, f.d_row_ptr.as<int>(), f.d_col.as<int>(), op->d_far64[l]->p,
                                  op->block_stride(f.B), f.nrows, f.B, op->w_yv[l]->p, op->w_zv[l]->p, 4 * nr, 0, s); }),
                     "far-field product (Maxwell)");
          BG_CHECK(timed_launch(op->ctx, KC_OTHER, [&] { return launch_mw_far_out(Sfar, ncl, np2, op->w_zv[l]->p, nrhs, r0, nr, tan,
                                                                           mk2.real(), mk2.imag(), op->w_z[l]->p, s); }),
                   "Maxwell far-field columns");
        }
        continue;
      }
      if (mixed) {
        if (op->vd != 1 || op->nc != 1) return set_error(op->ctx, BG_UNSUPPORTED, "mixed far field of vector operators");
        BG_CHECK(timed_launch(op->ctx, KC_FAR_FUSED, [&] { return launch_far_fused(op->cplx, op->d_pts32[l]->as<float4>(), op->d_centres[l]->as<d4>(),
                                  f.d_row_ptr.as<int>(), f.d_col.as<int>(), f.nrows, np2, (float)op->kre, (float)op->kim,
                                  op->w_y[l]->p, op->w_z[l]->p, nrhs, s); }),
                 "far-field product (FP32 fused)");
      } else {
        if (!op->store_far) return set_error(op->ctx, BG_UNSUPPORTED, "the FP64 product needs the stored far field");
        if (op->kbatched()) {
          // batched wavenumbers: wavenumber q's double-float pairs on column block q
          const int nk = (int)op->kslots.size(), nr = nrhs / nk;
          for (int q = 0; q < nk; ++q) {
            bg_status st = far64_cplx(l, op->kslots[q].far_df[l], op->w_y[l]->p, nrhs, q * nr, nr, op->w_z[l]->p);
            if (st != BG_OK) return st;
          }
        } else if (op->cplx && op->d_far_df[l]->p) {
          bg_status st = far64_cplx(l, op->d_far_df[l], op->w_y[l]->p, nrhs, 0, nrhs, op->w_z[l]->p);
          if (st != BG_OK) return st;
        } else if (!op->cplx && op->d_far_df[l]->p) {
          BG_CHECK(timed_launch(op->ctx, KC_OTHER, [&] { return launch_split_df(op->w_y[l]->p, (long)op->nclusters(l) * op->R * nrhs,
                                                                         op->w_ydf[l]->p, s); }),
                   "far-field split of Y");
          BG_CHECK(timed_launch(op->ctx, KC_FAR64, [&] { return launch_bsr_df(f.d_row_ptr.as<int>(), f.d_col.as<int>(), op->d_far_df[l]->p,
                              op->block_stride(f.B), f.nrows, f.B, op->w_ydf[l]->p, op->w_z[l]->p, nrhs, 0, s); }),
                   "far-field product (double-float)");
        }
        else
          BG_CHECK(timed_launch(op->ctx, KC_FAR64, [&] { return launch_bsr_fp64(op->cplx, f.d_row_ptr.as<int>(), f.d_col.as<int>(), op->d_far64[l]->p,
                              op->block_stride(f.B), f.nrows, f.B, op->w_y[l]->p, op->w_z[l]->p, nrhs, 0, s); }),
                   "far-field product");
      }
    }
    if (op->maxwell()) {
      for (int l = 0; l < Ll; ++l) {
        const int nb = 3 * op->nclusters(l);
        BG_CHECK(timed_launch(op->ctx, KC_TRANSFORM, [&] {
                   return op->use_tgemm ? launch_tgemm(Sfar, true, tm.a_tr_b, op->w_z[l]->p, np2, op->w_z[l + 1]->p, 4L * np2, nb, nrhs, s, pl.split_k_batches)
                                        : launch_transfer_bwd(Sfar, mixed ? op->d_tr32.p : op->d_tr64.p, np2, 1, nb,
                                                              op->w_z[l]->p, op->w_z[l + 1]->p, nrhs, s); }),
                 "backward transfer");
      }
      // y_0 += phi^T Zphi_0 + (d/ds phi)^T Zdiv,  y_1 += phi^T Zphi_1 + (d/dt phi)^T Zdiv
      const size_t chl = (size_t)op->nleaf_cl * np2 * nrhs * sfar;
      const char* zl = static_cast<const char*>(op->w_z[Ll]->p);
      char* yc0 = static_cast<char*>(yfar);
      char* yc1 = yc0 + comp_ss * nrhs * sfar;
      const char* zin[3] = {zl, zl + 2 * chl, zl + 2 * chl};
      char* yout[3] = {yc0, yc0, yc1};
      const int blk[3] = {0, 1, 2}, nb[3] = {2 * op->nleaf_cl, op->nleaf_cl, op->nleaf_cl};
      for (int t = 0; t < 3; ++t)
        BG_CHECK(timed_launch(op->ctx, KC_TRANSFORM, [&] {
                   return op->use_tgemm
                              ? launch_tgemm(Sfar, true, tm.a_mw_b[blk[t]], zin[t], np2, yout[t], op->Bq, nb[t], nrhs, s, pl.split_k_batches)
                              : launch_moment_bwd(Sfar, mw_mom(blk[t]), np2, op->Bq, nb[t], zin[t], yout[t], nrhs, s); }),
                 "backward moments");
    }
    if (fused_tr)
      BG_CHECK(timed_launch(op->ctx, KC_TRANSFORM, [&] { return launch_fmm_down(Sfar, fa, op->fmm_hfac.data(), op->nclusters(Ll - 1), s); }),
               "backward transforms (fused)");
    for (int c = 0; c < op->vd && !op->maxwell() && !fused_tr; ++c) {
      for (int l = 0; l < Ll; ++l) {
        const int ncl = op->nclusters(l);
        const char* zpa = static_cast<const char*>(op->w_z[l]->p) + (size_t)c * ncl * op->R * nrhs * sfar;
        char* zch = static_cast<char*>(op->w_z[l + 1]->p) + (size_t)c * 4 * ncl * op->R * nrhs * sfar;
        BG_CHECK(timed_launch(op->ctx, KC_TRANSFORM, [&] {
                   return op->use_tgemm ? launch_tgemm(Sfar, true, tm.a_tr_b, zpa, op->R, zch, 4L * op->R, ncl, nrhs, s, pl.split_k_batches)
                                        : launch_transfer_bwd(Sfar, mixed ? op->d_tr32.p : op->d_tr64.p, np2, op->nc, ncl,
                                                              zpa, zch, nrhs, s); }),
                 "backward transfer");
      }
      const void* mom = mixed ? op->d_mom32[c]->p : op->d_mom64[c]->p;
      const char* zl = static_cast<const char*>(op->w_z[Ll]->p) + (size_t)c * op->nleaf_cl * op->R * nrhs * sfar;
      char* yc = static_cast<char*>(yfar) + c * comp_ss * nrhs * sfar;
      BG_CHECK(timed_launch(op->ctx, KC_TRANSFORM, [&] {
                 return op->use_tgemm ? launch_tgemm(Sfar, true, tm.a_mom_b[c], zl, op->R, yc, op->Bq, op->nleaf_cl, nrhs, s, pl.split_k_batches)
                                      : launch_moment_bwd(Sfar, mom, op->R, op->Bq, op->nleaf_cl, zl, yc, nrhs, s); }),
               "backward moments");
    }
    if (mixed && !near32)
      BG_CHECK(timed_launch(op->ctx, KC_OTHER, [&] { return launch_add_low(op->cplx, op->w_yss32.p, ss_n, op->w_yss.p, s); }), "far field to FP64");
  }
  if (near32)
    BG_CHECK(timed_launch(op->ctx, KC_OTHER, [&] { return launch_convert(Sfar, S64, op->w_yss32.p, ss_n, op->w_yss.p, s); }), "y to FP64");
  return BG_OK;
}

// One H2 product on row-major FP64 work vectors (H2DenseProduct.hpp:33-165).
// Outside profiling runs the middle part is captured once per (nrhs,
// precision) as a CUDA graph and replayed; growing the work vectors or
// re-assembling the operator drops the graphs. A capture that fails falls back
// to direct launches for this operator.
// Batched wavenumbers: column block q of the row-major dof vectors (nrhs /
// nslots columns) goes through slot q's operator.
static bg_status apply_wavenumber_blocks(bg_operator* op, int nrhs, int prec, const void* xdof, void* ydof) {
  const int nk = (int)op->kslots.size();
  if (nrhs % nk) return set_error(op->ctx, BG_INVALID_ARG, "batched wavenumbers: columns must be a multiple of the wavenumbers");
  const int nr = nrhs / nk;
  const size_t usz = op->scalar_bytes(false), blk = (size_t)op->N * nr * usz;
  cudaStream_t s = op->ctx->stream;
  if (op->w_kx.bytes < blk) {
    BG_CHECK(op->w_kx.alloc(blk), "wavenumber column blocks");
    BG_CHECK(op->w_ky.alloc(blk), "wavenumber column blocks");
  }
  bg_status st = BG_OK;
  for (int q = 0; q < nk && st == BG_OK; ++q) {
    const size_t off = (size_t)q * nr * usz, pitch = (size_t)nrhs * usz;
    BG_CHECK(cudaMemcpy2DAsync(op->w_kx.p, nr * usz, static_cast<const char*>(xdof) + off, pitch, nr * usz, op->N,
                               cudaMemcpyDeviceToDevice, s), "wavenumber column block");
    op->activate_slot(q);
    st = apply_operator(op, nr, prec, op->w_kx.p, op->w_ky.p);
    if (st == BG_OK)
      BG_CHECK(cudaMemcpy2DAsync(static_cast<char*>(ydof) + off, pitch, op->w_ky.p, nr * usz, nr * usz, op->N,
                                 cudaMemcpyDeviceToDevice, s), "wavenumber column block");
  }
  op->activate_slot(-1);
  return st;
}

// Whether a product of batched wavenumbers can run as one pass over all of
// them: the FP64 product needs every wavenumber's double-float far field, the
// low-precision ones the tile setup of bg_operator_assemble_wavenumbers.
static bool kbatch_one_pass(const bg_operator* op, int prec) {
  bool any_far = false;
  for (const auto& f : op->far) any_far |= !f.col.empty();
  if (!any_far) return true;
  if (prec != BG_PREC_FP64) return op->kb_nwork > 0;
  for (const auto& k : op->kslots)
    for (int l = 0; l <= op->leaf_level; ++l)
      if (!op->far[l].col.empty() && ((int)k.far_df.size() <= l || !k.far_df[l]->p)) return false;
  return true;
}

bg_status apply_operator(bg_operator* op, int nrhs, int prec, const void* xdof, void* ydof) {
  if (op->kbatched()) {
    if (!kbatch_one_pass(op, prec)) return apply_wavenumber_blocks(op, nrhs, prec, xdof, ydof);
    const int nk = (int)op->kslots.size();
    if (nrhs % nk)
      return set_error(op->ctx, BG_INVALID_ARG, "batched wavenumbers: columns must be a multiple of the wavenumbers");
    const size_t blk = (size_t)op->S * (nrhs / nk) * op->scalar_bytes(false);
    if (op->kb_xs.bytes < blk) {
      op->drop_graphs();  // the column blocks of the near fields move
      BG_CHECK(op->kb_xs.alloc(blk), "near-field column blocks");
      BG_CHECK(op->kb_ys.alloc(blk), "near-field column blocks");
    }
  }
  cudaStream_t s = op->ctx->stream;
  const int S64 = op->stype(false);
  BG_CHECK(timed_launch(op->ctx, KC_TAPPLY, [&] { return launch_csr_apply(S64, op->d_T_ptr.as<int>(), op->d_T_idx.as<int>(), op->d_T_val.as<double>(), op->S, xdof,
                            op->w_xss.p, nrhs, s); }),
           "T x");
  bg_status st = BG_OK;
  bg_context* ctx = op->ctx;
  if (ctx->profiling || !op->use_graphs) {
    st = apply_middle(op, nrhs, prec);
  } else {
    // one graph per shape and wavenumber slot (the slots' fields differ)
    const long key = bg_operator::plan_key(nrhs, prec) + ((long)(op->kslot_active + 1) << 40);
    auto it = op->graphs.find(key);
    if (it == op->graphs.end() && !op->graph_seen.count(key)) {
      // first product of this shape: direct launches (they also raise the
      // kernels' shared-memory limits, which a capture must not do)
      op->graph_seen.insert(key);
      st = apply_middle(op, nrhs, prec);
    } else if (it == op->graphs.end()) {
      // capture: count the launches the graph holds, per kernel class
      const long l0 = ctx->launches;
      long c0[8];
      for (int c = 0; c < 8; ++c) c0[c] = ctx->class_launches[c];
      cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
      bg_status mst = e == cudaSuccess ? apply_middle(op, nrhs, prec) : BG_DEVICE_ERROR;
      cudaGraph_t g = nullptr;
      if (e == cudaSuccess) e = cudaStreamEndCapture(s, &g);
      bg_operator::ProductGraph pg;
      if (e == cudaSuccess && mst == BG_OK && g) e = cudaGraphInstantiate(&pg.exec, g, 0);
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();  // a failed capture leaves no sticky error
      pg.launches = ctx->launches - l0;
      for (int c = 0; c < 8; ++c) pg.class_launches[c] = ctx->class_launches[c] - c0[c];
      ctx->launches = l0;
      for (int c = 0; c < 8; ++c) ctx->class_launches[c] = c0[c];
      if (e != cudaSuccess || mst != BG_OK || !pg.exec) {
        if (pg.exec) cudaGraphExecDestroy(pg.exec);
        op->use_graphs = false;
        st = apply_middle(op, nrhs, prec);
      } else {
        it = op->graphs.emplace(key, pg).first;
      }
    }
    if (op->use_graphs && it != op->graphs.end()) {
      BG_CHECK(cudaGraphLaunch(it->second.exec, s), "H2 product (graph)");
      ctx->launches += it->second.launches;
      for (int c = 0; c < 8; ++c) ctx->class_launches[c] += it->second.class_launches[c];
    }
  }
  if (st != BG_OK) return st;
  BG_CHECK(timed_launch(op->ctx, KC_TAPPLY, [&] { return launch_csr_apply(S64, op->d_Tt_ptr.as<int>(), op->d_Tt_idx.as<int>(), op->d_Tt_val.as<double>(), op->N,
                            op->w_yss.p, ydof, nrhs, s); }),
           "T^T y");
  return BG_OK;
}

// Reads (and clears) the flag a kernel sets when one of its bounded waits ran
// out; call after the stream has been synchronised.
bg_status check_device_flag(bg_operator* op) {
  if (!op->d_err.p) return BG_OK;
  int code = 0;
  BG_CHECK(cudaMemcpy(&code, op->d_err.p, sizeof(int), cudaMemcpyDeviceToHost), "error flag");
  if (code == 0) return BG_OK;
  BG_CHECK(cudaMemset(op->d_err.p, 0, sizeof(int)), "error flag");
  return set_error(op->ctx, BG_TIMEOUT,
                   "a bounded wait of the tensor-core far-field kernel ran out (code " + std::to_string(code) + ")");
}

static bool valid_precision(int p) { return p == BG_PREC_FP64 || p == BG_PREC_MIXED || p == BG_PREC_FP32; }

extern "C" bg_status bg_operator_set_plan(bg_operator* op, int nrhs, int precision, const bg_launch_plan* plan) {
  if (!op || !plan) return BG_INVALID_ARG;
  if (nrhs < 1 || !valid_precision(precision))
    return set_error(op->ctx, BG_INVALID_ARG, "launch plan: nrhs must be positive and the precision a bg_precision");
  if (plan->near_kernel < 0 || plan->near_kernel > 3 || plan->split_k_batches < -1 ||
      plan->split_k_batches > (1 << 24) || plan->far_order < 0 || plan->far_order > 2 || plan->transforms < 0 ||
      plan->transforms > 1 || plan->far_ctas < 0 || plan->far_ctas > 2 || plan->mixed_near < 0 ||
      plan->mixed_near > 2 || plan->far_tiles < 0 || plan->far_tiles > 1)
    return set_error(op->ctx, BG_INVALID_ARG, "launch plan: a field is out of range");
  op->plans[bg_operator::plan_key(nrhs, precision)] = *plan;
  op->drop_graphs();
  return BG_OK;
}

extern "C" bg_status bg_operator_get_plan(const bg_operator* op, int nrhs, int precision, bg_launch_plan* plan) {
  if (!op || !plan || nrhs < 1 || !valid_precision(precision)) return BG_INVALID_ARG;
  *plan = op->plan_for(nrhs, precision);
  return BG_OK;
}

extern "C" bg_status bg_operator_autotune(bg_operator* op, int nrhs, int precision, int reps, bg_tune_report* report) {
  if (!op || !report) return BG_INVALID_ARG;
  bg_context* ctx = op->ctx;
  if (nrhs < 1 || !valid_precision(precision) || reps < 0 || reps > 1000)
    return set_error(ctx, BG_INVALID_ARG, "autotune: nrhs must be positive, reps in [0, 1000]");
  if (ctx->device < 0) return set_error(ctx, BG_UNSUPPORTED, "host-only context: the autotuner needs a GPU");
  if (!op->assembled) return set_error(ctx, BG_INVALID_ARG, "autotune: the operator is not assembled");
  if (op->kbatched()) return set_error(ctx, BG_UNSUPPORTED, "autotune: tune one wavenumber, not a batch");
  if (reps == 0) reps = 5;
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->stream;
  bg_status st = ensure_work(op, nrhs);
  if (st != BG_OK) return st;
  // seeded superspace input in [-1, 1) (a 64-bit linear congruential generator)
  std::vector<double> x((size_t)op->S * nrhs * (op->cplx ? 2 : 1));
  uint64_t z = 0x2545F4914F6CDD1DULL;
  for (double& v : x) {
    z = z * 6364136223846793005ULL + 1442695040888963407ULL;
    v = (double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
  }
  BG_CHECK(cudaMemcpyAsync(op->w_xss.p, x.data(), x.size() * sizeof(double), cudaMemcpyHostToDevice, s),
           "autotune input");
  BG_CHECK(cudaStreamSynchronize(s), "autotune input");
  struct Events {
    cudaEvent_t a = nullptr, b = nullptr;
    ~Events() {
      if (a) cudaEventDestroy(a);
      if (b) cudaEventDestroy(b);
    }
  } ev;
  BG_CHECK(cudaEventCreate(&ev.a), "autotune events");
  BG_CHECK(cudaEventCreate(&ev.b), "autotune events");
  const long key = bg_operator::plan_key(nrhs, precision);
  // the plan in force before tuning, put back if tuning fails
  const auto prev = op->plans.find(key);
  const bool had_plan = prev != op->plans.end();
  const bg_launch_plan saved = had_plan ? prev->second : bg_operator::builtin_plan();
  auto restore = [&] {
    if (had_plan) op->plans[key] = saved;
    else op->plans.erase(key);
  };
  // mean time of one product middle under plan p (after one untimed product,
  // which also raises the kernels' shared-memory limits)
  auto time_plan = [&](const bg_launch_plan& p, double* ms) -> bg_status {
    op->plans[key] = p;
    bg_status r = apply_middle(op, nrhs, precision);
    if (r != BG_OK) return r;
    BG_CHECK(cudaEventRecord(ev.a, s), "autotune events");
    for (int i = 0; i < reps; ++i)
      if ((r = apply_middle(op, nrhs, precision)) != BG_OK) return r;
    BG_CHECK(cudaEventRecord(ev.b, s), "autotune events");
    BG_CHECK(cudaEventSynchronize(ev.b), "autotune events");
    if ((r = check_device_flag(op)) != BG_OK) return r;
    float t = 0.0f;
    BG_CHECK(cudaEventElapsedTime(&t, ev.a, ev.b), "autotune events");
    *ms = (double)t / reps;
    return BG_OK;
  };
  bg_launch_plan cur = bg_operator::builtin_plan();
  double cur_ms = 0.0;
  int count = 1;
  if ((st = time_plan(cur, &cur_ms)) != BG_OK) {
    restore();
    return st;
  }
  const double builtin_ms = cur_ms;
  // one knob at a time; a change is kept when it is at least 2 % faster
  auto sweep = [&](int bg_launch_plan::*field, const std::vector<int>& values) -> bg_status {
    const int start = cur.*field;
    for (int v : values) {
      if (v == start) continue;
      bg_launch_plan p = cur;
      p.*field = v;
      double ms = 0.0;
      bg_status r = time_plan(p, &ms);
      if (r != BG_OK) return r;
      ++count;
      if (ms < 0.98 * cur_ms) {
        cur = p;
        cur_ms = ms;
      }
    }
    return BG_OK;
  };
  const bool mixed = precision != BG_PREC_FP64, near32 = precision == BG_PREC_FP32;
  if (near32) {
    std::vector<int> v = {1, 2};
    if (op->cplx && op->dense.B % 4 == 0) v.push_back(3);
    st = sweep(&bg_launch_plan::near_kernel, v);
  }
  if (st == BG_OK && op->fmm_fused) st = sweep(&bg_launch_plan::transforms, {1});
  if (st == BG_OK && mixed && !op->cplx && op->far_tiles) st = sweep(&bg_launch_plan::far_ctas, {1, 2});
  if (st == BG_OK && mixed && !near32 && !op->cplx && op->d_dense_df.p) st = sweep(&bg_launch_plan::mixed_near, {1, 2});
  if (st == BG_OK && mixed && op->use_tgemm && (!op->fmm_fused || cur.transforms == 1))
    st = sweep(&bg_launch_plan::split_k_batches, {0, 304, 608});
  if (st == BG_OK && mixed && op->d_far_work_alt[0].p) st = sweep(&bg_launch_plan::far_order, {1, 2});
  if (st != BG_OK) {
    restore();
    return st;
  }
  op->plans[key] = cur;
  op->drop_graphs();
  report->candidates = count;
  report->builtin_ms = builtin_ms;
  report->tuned_ms = cur_ms;
  report->plan = cur;
  return BG_OK;
}

static bg_status stage_host(bg_context* ctx, DevBuf* buf, const void* host, long ld, long rows, int ncols, size_t esz,
                            bool to_device) {
  cudaError_t e = buf->alloc((size_t)rows * ncols * esz);
  if (e != cudaSuccess) return cuda_status(ctx, e, "staging buffer");
  if (to_device)
    e = cudaMemcpy2DAsync(buf->p, rows * esz, host, ld * esz, rows * esz, ncols, cudaMemcpyHostToDevice, ctx->stream);
  return cuda_status(ctx, e, "host to device copy");
}

// The product in chunks of at most `chunk` columns.
static bg_status matvec_chunks(bg_operator* op, const void* x, long ldx, void* y, long ldy, int nrhs,
                               const double* alpha, const double* beta, int precision, int on_device, int chunk) {
  cudaStream_t s = op->ctx->stream;
  const size_t usz = op->cplx ? 16 : 8;
  const int uS = op->cplx ? 1 : 0;
  for (int c0 = 0; c0 < nrhs; c0 += chunk) {
    const int k = std::min(chunk, nrhs - c0);
    bg_status st = ensure_work(op, k);
    if (st != BG_OK) return st;
    const char* xp = static_cast<const char*>(x) + (size_t)c0 * ldx * usz;
    char* yp = static_cast<char*>(y) + (size_t)c0 * ldy * usz;
    const void* xd = xp;
    long lx = ldx, ly = ldy;
    void* yd = yp;
    if (!on_device) {
      if ((st = stage_host(op->ctx, &op->ctx->stage_in, xp, ldx, op->N, k, usz, true)) != BG_OK) return st;
      if ((st = stage_host(op->ctx, &op->ctx->stage_out, yp, ldy, op->N, k, usz,
                           beta[0] != 0.0 || beta[1] != 0.0)) != BG_OK)
        return st;
      xd = op->ctx->stage_in.p;
      yd = op->ctx->stage_out.p;
      lx = ly = op->N;
    }
    BG_CHECK(timed_launch(op->ctx, KC_OTHER, [&] { return launch_gather_in(uS, uS, xd, lx, op->N, k, op->w_xdof.p, s); }), "gather x");
    if ((st = apply_operator(op, k, precision, op->w_xdof.p, op->w_ydof.p)) != BG_OK) return st;
    BG_CHECK(timed_launch(op->ctx, KC_OTHER, [&] { return launch_scatter_out(uS, op->w_ydof.p, op->N, k, yd, ly, alpha, beta, s); }), "scatter y");
    if (!on_device)
      BG_CHECK(cudaMemcpy2DAsync(yp, ldy * usz, yd, op->N * usz, op->N * usz, k, cudaMemcpyDeviceToHost, s),
               "device to host copy");
  }
  BG_CHECK(cudaStreamSynchronize(s), "H2 matvec");
  return check_device_flag(op);
}

extern "C" bg_status bg_matvec(bg_operator* op, const void* x, long ldx, void* y, long ldy, int nrhs,
                               const double* alpha, const double* beta, int precision, int on_device) {
  if (!op || nrhs < 0) return BG_INVALID_ARG;
  if (nrhs == 0) return BG_OK;  // no columns: nothing to do (as Eigen's empty product)
  if (!x || !y || ldx < op->N || ldy < op->N) return BG_INVALID_ARG;
  if (op->ctx->device < 0) return set_error(op->ctx, BG_UNSUPPORTED, "host-only context: products need a GPU");
  if (!op->assembled) return set_error(op->ctx, BG_INVALID_ARG, "operator not assembled");
  if (precision != BG_PREC_FP64 && precision != BG_PREC_MIXED && precision != BG_PREC_FP32)
    return set_error(op->ctx, BG_INVALID_ARG, "precision");
  const double one[2] = {1.0, 0.0}, zero2[2] = {0.0, 0.0};
  if (!alpha) alpha = one;
  if (!beta) beta = zero2;
  if (!op->cplx && (alpha[1] != 0.0 || beta[1] != 0.0))
    return set_error(op->ctx, BG_INVALID_ARG, "complex scalars for a real operator");
  cudaSetDevice(op->ctx->device);
  if (op->kbatched()) {
    const int nk = (int)op->kslots.size();
    if (nrhs % nk)
      return set_error(op->ctx, BG_INVALID_ARG, "batched wavenumbers: columns must be a multiple of the wavenumbers");
    const int nr = nrhs / nk;
    if (!kbatch_one_pass(op, precision)) {
      // column block q through wavenumber slot q, one wavenumber at a time
      bg_status st = BG_OK;
      for (int q = 0; q < nk && st == BG_OK; ++q) {
        op->activate_slot(q);
        st = bg_matvec(op, static_cast<const char*>(x) + (size_t)q * nr * ldx * 16, ldx,
                       static_cast<char*>(y) + (size_t)q * nr * ldy * 16, ldy, nr, alpha, beta, precision, on_device);
      }
      op->activate_slot(-1);
      return st;
    }
    // one pass over all wavenumbers per chunk: the columns are permuted on the
    // device so that every chunk holds an equal slice of every block, in
    // block order (what the batched product expects), then permuted back
    cudaStream_t s = op->ctx->stream;
    const int w = std::max(1, std::min(nr, 32 / nk));
    const size_t col = (size_t)op->N * 16;
    const bool by = beta[0] != 0.0 || beta[1] != 0.0;
    DevBuf xp, yp;
    BG_CHECK(xp.alloc(col * nrhs), "product staging");
    BG_CHECK(yp.alloc(col * nrhs), "product staging");
    auto permute = [&](const void* src, long lds, void* dst, long ldd, bool to_slices, cudaMemcpyKind kind) {
      for (int c0 = 0; c0 < nr; c0 += w) {
        const int ws = std::min(w, nr - c0);
        for (int q = 0; q < nk; ++q) {
          const long user = q * nr + c0, perm = (long)c0 * nk + (long)q * ws;
          const long cs = to_slices ? user : perm, cd = to_slices ? perm : user;
          cudaError_t e = cudaMemcpy2DAsync(static_cast<char*>(dst) + (size_t)cd * ldd * 16, ldd * 16,
                                            static_cast<const char*>(src) + (size_t)cs * lds * 16, lds * 16, col, ws,
                                            kind, s);
          if (e != cudaSuccess) return e;
        }
      }
      return cudaSuccess;
    };
    const cudaMemcpyKind in = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    BG_CHECK(permute(x, ldx, xp.p, op->N, true, in), "product staging");
    if (by) BG_CHECK(permute(y, ldy, yp.p, op->N, true, in), "product staging");
    bg_status st = matvec_chunks(op, xp.p, op->N, yp.p, op->N, nrhs, alpha, beta, precision, 1, nk * w);
    if (st != BG_OK) return st;
    BG_CHECK(permute(yp.p, op->N, y, ldy, false, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost),
             "product staging");
    BG_CHECK(cudaStreamSynchronize(s), "H2 matvec");
    return BG_OK;
  }
  return matvec_chunks(op, x, ldx, y, ldy, nrhs, alpha, beta, precision, on_device, 32);
}
