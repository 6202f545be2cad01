/*
 * bembel_gb300 — C ABI of the GB300 (sm_103a) H2 single-layer operator.
 *
 * This is the drop-in boundary for Bembel's
 *   DiscreteOperator<H2Matrix<Scalar>, {Laplace,Helmholtz,Maxwell}SingleLayerOperator>
 * path: geometry -> discrete space -> H2 assembly -> H2 matvec -> Krylov solve.
 * Every entry point names the reference interface it replaces (paths are
 * relative to the Bembel source tree). Plain pointers and sizes only; no
 * exceptions cross this boundary; every call returns a bg_status.
 *
 * Conventions
 *  - Vectors are column-major blocks of nrhs columns with leading dimension
 *    ld >= rows. Complex values are interleaved (re, im) doubles, the layout
 *    of std::complex<double>.
 *  - The row/column space of the operator is the reference's DOF space
 *    (cols of AnsatzSpace::get_transformation_matrix(), AnsatzSpace.hpp:108).
 *  - Helmholtz/Maxwell kernels use the reference sign exp(-i k r)/(4 pi r)
 *    (Helmholtz/SingleLayerOperator.hpp:115-120).
 */
#ifndef BEMBEL_GB300_H_
#define BEMBEL_GB300_H_

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  BG_OK = 0,
  BG_INVALID_ARG = 1,
  BG_OOM = 2,
  BG_UNSUPPORTED = 3,
  BG_DEVICE_ERROR = 4,
  BG_TIMEOUT = 5,
  BG_CANCELLED = 6,
  BG_NOT_CONVERGED = 7
} bg_status;

typedef enum { BG_LAPLACE_SL = 0, BG_HELMHOLTZ_SL = 1, BG_MAXWELL_SL = 2 } bg_op_kind;

/* Arithmetic of a product. BG_PREC_FP64 applies the FP64 H2 matrix (stored
 * near and far field, the reference's H2Matrix). BG_PREC_MIXED keeps the
 * near-field product, T and the vectors in FP64 and evaluates the far field in
 * FP32 on the tensor cores: from couplings split into scaled FP16 high and low
 * parts at assembly (22 bits kept; real operators with the FP64 far field
 * stored), else from couplings generated on the fly; moments and transfers in
 * FP32. BG_PREC_FP32 also applies the near
 * field in FP32 (an FP32 copy of the assembled FP64 blocks); T and the input and
 * output vectors stay FP64. FP32 is meant for the inner operator of the solver,
 * whose outer FP64 iteration removes its rounding. */
typedef enum { BG_PREC_FP64 = 0, BG_PREC_MIXED = 1, BG_PREC_FP32 = 2 } bg_precision;

typedef struct bg_context bg_context;
typedef struct bg_geometry bg_geometry;
typedef struct bg_operator bg_operator;

/* H2 parameters. Defaults (bg_h2_params_default) are the reference's:
 * number_of_points = 9 (H2Matrix.hpp:94-96), eta = 1.6 and
 * min_cluster_level = 1 (BlockClusterTree.hpp:113-118). */
typedef struct {
  int n_p;               /* Chebyshev points per direction */
  double eta;            /* admissibility constant */
  int min_cluster_level; /* leaf clusters hold 4^min_cluster_level elements */
  int store_fp64_far;    /* 1: assemble and store the FP64 far field */
  int keep_fp64_blocks;  /* 1 (default): keep the FP64 coupling blocks after assembly (leaf-block
                            inspection); 0: release them once their double-float pairs and
                            tensor-core tiles are built, which the products use (about a third
                            less device memory; the serving loop does this) */
} bg_h2_params;

/* Solve controls for bg_solve (GMRES with iterative refinement). */
typedef struct {
  double tol;            /* target ||b - A x|| / ||b|| per column */
  int restart;           /* Krylov restart length */
  int max_iter;          /* total inner iterations, all refinement steps */
  int inner_precision;   /* bg_precision of the inner (correction) operator; default BG_PREC_FP32 */
  double inner_tol;      /* relative tolerance of each inner solve; default 2e-3 */
  int max_refinements;   /* outer FP64 residual steps */
} bg_solve_params;

typedef struct {
  int iterations;        /* inner Krylov iterations, summed */
  int refinements;       /* FP64 residual evaluations */
  int fp64_matvecs;
  int low_matvecs;
  double final_relres;   /* max over columns */
} bg_solve_stats;

void bg_h2_params_default(bg_h2_params* p);
void bg_solve_params_default(bg_solve_params* p);

/* Context: one GPU, its streams and scratch. Bembel has no counterpart; it is
 * the owner of everything the reference keeps in process globals. */
bg_status bg_context_create(int device, bg_context** out);
bg_status bg_context_destroy(bg_context* ctx);
const char* bg_last_error_string(bg_context* ctx);
/* The CUDA stream (cudaStream_t) every kernel of this context runs on. */
bg_status bg_context_get_stream(bg_context* ctx, void** stream);
/* Kernel timing: while enabled, every kernel launch is bracketed by CUDA
 * events on the context stream. bg_profile_read synchronises and returns, per
 * kernel class (near-field product, FP64 far-field product, fused FP32 far
 * field, FMM transforms, T application, Krylov vector kernels, other,
 * assembly), the summed device milliseconds and launch counts since the last
 * read, then resets them. */
bg_status bg_profile_enable(bg_context* ctx, int enable);
bg_status bg_profile_read(bg_context* ctx, double* ms8, long* launches8);
/* Kernel classes (bit c for class c, in the order above) that bg_profile_enable
 * brackets with events; default all. Timing only the classes of interest keeps
 * the event overhead out of a measured region. Launch counts cover all. */
bg_status bg_profile_classes(bg_context* ctx, unsigned mask);

/* Geometry(const std::string&) with LoadGeometryFileDAT
 * (Geometry/Geometry.hpp:89-102, Geometry/GeometryIO.hpp:25-122). */
bg_status bg_geometry_load_dat(bg_context* ctx, const char* path, bg_geometry** out);
/* Geometry(const std::string&) with LoadGeometryFileIGS (Geometry/GeometryIGS.hpp:25-151):
 * the rational B-spline surfaces (entity 128) of an IGES file; single-span
 * (Bezier) surfaces only, other entities and interior knots give BG_INVALID_ARG. */
bg_status bg_geometry_load_igs(bg_context* ctx, const char* path, bg_geometry** out);
/* The unit sphere as six analytic patches: patch f is the image x / |x| of
 * one face of the cube [-1, 1]^3, parametrised over [0, 1]^2 with an outward
 * normal (face f on the plane x_{f/2} = +1 for even f, -1 for odd f). No
 * reference counterpart: Bembel's patches are rational B-splines only
 * (Geometry/Patch.hpp:63-104); this kind stands beside them and is accepted
 * wherever a geometry is. bg_geometry_patch_data returns BG_UNSUPPORTED for
 * its patches (they have no control points). */
bg_status bg_geometry_cube_sphere(bg_context* ctx, bg_geometry** out);
bg_status bg_geometry_destroy(bg_geometry* g);
/* Geometry(const PatchVector&) (Geometry/Geometry.hpp:60-63) from Bezier
 * patches already in memory, so an existing Bembel::Geometry can be handed
 * over without a file: patch p has px[p] x py[p] control points (degree + 1 per
 * direction) in the layout of Patch::data_ for a patch without interior knots
 * (Patch.hpp:371): data[4 (px_i py[p] + iy) + k], k = x w, y w, z w, w;
 * the patches are concatenated. */
bg_status bg_geometry_from_bezier(bg_context* ctx, int npatch, const int* px, const int* py, const double* data,
                                  bg_geometry** out);
bg_status bg_geometry_num_patches(const bg_geometry* g, int* n);
/* copy patch p's control data out in the layout above (data may be NULL to
 * query px, py only; else 4 px py doubles) */
bg_status bg_geometry_patch_data(const bg_geometry* g, int patch, int* px, int* py, double* data);
/* Patch::updateSurfacePoint at patch coordinates (Geometry/Patch.hpp:294-365);
 * out12 = [s, t, 1, x(3), dx(3), dy(3)]. Host evaluation. */
bg_status bg_geometry_surface_point(const bg_geometry* g, int patch, double s, double t, double* out12);

/* AnsatzSpace(geometry, M, P) + DiscreteOperator<H2Matrix<S>, Op>(ansatz_space)
 * (AnsatzSpace/AnsatzSpace.hpp:102-111, LinearOperator/DiscreteOperator.hpp:107-145):
 * builds the element tree, block cluster tree, transformation matrix, FMM
 * moments/transfers and uploads the device tables. */
bg_status bg_operator_create(bg_context* ctx, const bg_geometry* g, int M, int P, int op_kind,
                             const bg_h2_params* params, bg_operator** out);
/* HelmholtzSingleLayerOperator::set_wavenumber (Helmholtz/SingleLayerOperator.hpp:124-126). */
bg_status bg_operator_set_wavenumber(bg_operator* op, double re, double im);
/* DiscreteOperator::compute -> H2Matrix::init_H2Matrix (H2Matrix/H2Matrix.hpp:93-250):
 * near-field (DuffyTrick) and far-field (interpolateKernel) assembly on the GPU. */
bg_status bg_operator_assemble(bg_operator* op);
/* No counterpart in the reference, which assembles one wavenumber per
 * DiscreteOperator::compute (Helmholtz/SingleLayerOperator.hpp:124-130,
 * H2Matrix.hpp:93-250). Assembles the near field (the dense leaves) of the
 * Helmholtz operator for the n wavenumbers kre[i] + i kim[i] in one pass:
 * the identical-element rule evaluates every Duffy sample's points, surface
 * measures and basis values once for up to 4 wavenumbers, the common-edge
 * and common-vertex rules run their factorised kernels per wavenumber, and
 * the regular pairs share their per-element quadrature tables. The blocks stay on the device (n near
 * fields, bg_operator_memory counts them); after bg_operator_set_wavenumber
 * to one of them, bg_operator_assemble copies that near field instead of
 * integrating it again and assembles only the far field. A wavenumber
 * prepared twice keeps the later blocks. BG_UNSUPPORTED for other operators. */
bg_status bg_operator_prepare_wavenumbers(bg_operator* op, const double* kre, const double* kim, int n);
/* Near-field quadrature work of a scalar operator, the counts of the
 * reference's rules (LinearOperatorBase.hpp:56-89, DuffyTrick/integrate0-4.hpp):
 * counts8 = [regular pairs, their integrand evaluations (n+1)^4 each,
 * identical pairs, evaluations 8 (n+1)^4 each, common-edge pairs, 6 (n+1)^4
 * each, common-vertex pairs, 4 (n+1)^4 each]. No counterpart in the
 * reference; host only, no device work. */
bg_status bg_operator_quadrature_counts(const bg_operator* op, long* counts8);
/* frees the near fields of bg_operator_prepare_wavenumbers and the
 * wavenumber slots of bg_operator_assemble_wavenumbers (the operator is then
 * unassembled) */
bg_status bg_operator_release_wavenumbers(bg_operator* op);
/* No counterpart in the reference (one wavenumber per
 * DiscreteOperator::compute, Helmholtz/SingleLayerOperator.hpp:124-130).
 * Assembles every wavenumber prepared by bg_operator_prepare_wavenumbers
 * side by side: wavenumber q (in preparation order) gets a slot with its near
 * field (the prepared blocks, which are then freed), its far field and the
 * far field's tensor-core tiles. Afterwards bg_matvec, bg_solve,
 * bg_load_vector and bg_potential take nrhs = n k columns (n wavenumbers,
 * k columns each) and apply wavenumber q to columns q k .. q k + k - 1: one
 * call, and for bg_solve one flexible GMRES over all n k columns, covers
 * every wavenumber. A product makes one pass over all wavenumbers (the
 * tensor-core far field of every wavenumber in one launch per 16 columns)
 * when each has its tiles, else applies them one after another. Other
 * column counts give BG_INVALID_ARG;
 * bg_matvec_noalloc and bg_operator_autotune give BG_UNSUPPORTED.
 * bg_operator_assemble (after bg_operator_set_wavenumber) returns the
 * operator to one wavenumber. Helmholtz single layer only. */
bg_status bg_operator_assemble_wavenumbers(bg_operator* op);
/* the wavenumbers of the slots of bg_operator_assemble_wavenumbers, in
 * column-block order (*n = 0 when the operator holds none); kre, kim may be
 * NULL or hold *n values */
bg_status bg_operator_num_wavenumbers(const bg_operator* op, int* n, double* kre, double* kim);
bg_status bg_operator_destroy(bg_operator* op);
/* info[0..15]: rows (= cols, H2Matrix.hpp:76-77), superspace size, elements,
 * dense leaves, low-rank leaves, vector dimension, FMM components, n_p,
 * is_complex, M, P, dense-leaf levels' cluster size, nnz(T), stored far-field
 * bytes, near-field bytes, element pairs in the near field. */
bg_status bg_operator_info(const bg_operator* op, long* info);
/* seconds of the last bg_operator_assemble: [near field, far field, total] */
bg_status bg_operator_assembly_times(const bg_operator* op, double* t3);

/* H2_time_dense_product_impl::run via generic_product_impl::scaleAndAddTo
 * (H2Matrix/EigenHelper/H2DenseProduct.hpp:33-165, 268-290):
 *   Y = beta * Y + alpha * A X   for nrhs columns.
 * x, y are host pointers when on_device == 0 (staged through pinned buffers),
 * device pointers otherwise. alpha/beta are complex (re, im) pairs; for a real
 * operator their imaginary parts must be 0. precision: bg_precision.
 * nrhs == 0 is an empty product: BG_OK, nothing read or written. */
bg_status bg_matvec(bg_operator* op, const void* x, long ldx, void* y, long ldy, int nrhs,
                    const double* alpha, const double* beta, int precision, int on_device);

/* y = A x for ONE right-hand side without allocating any device memory. This
 * entry point has no counterpart in the reference; it exists for callers that
 * may not call cudaMalloc when they need a product (a host that owns a fixed
 * memory budget and counts every allocation, code inside a pooled allocator it
 * must not disturb, a serving loop that forbids allocation after warm-up
 * because an allocation can stall the device). bg_matvec grows per-operator
 * work vectors on demand and so may allocate.
 * x, y: device pointers to N scalars of the operator's type (double, or
 * interleaved complex double), aligned to that type, not overlapping.
 * precision: BG_PREC_FP64 or BG_PREC_MIXED. The call returns once y is written.
 * Intermediate vectors come from one fixed 16 MiB device array in the library
 * (held on every GPU that loads it until the process exits). An operator whose
 * intermediates do not fit is rejected with BG_INVALID_ARG and a message giving
 * the bytes it would need (sphere, M = 5, P = 2, n_p = 9 needs about 4 MB).
 * Laplace and Helmholtz operators only (Maxwell: BG_UNSUPPORTED).
 * All calls on a device share that array, so calls that overlap on the GPU
 * (other threads, other contexts, other streams) race and give wrong results.
 * The first call on each device looks up the array's device address; make it
 * before any stream capture. */
bg_status bg_matvec_noalloc(bg_operator* op, const void* x, void* y, int precision);

/* DiscreteLinearForm<DirichletTrace<S>, Op>::compute (LinearForm/DiscreteLinearForm.hpp:44-83,
 * LinearForm/DirichletTrace.hpp:38-66) for analytic data (examples/Data.hpp):
 *   kind 0: u(x) = 1/(4 pi |x - x0|), prm = x0 (3 doubles per column)
 *   kind 1: u(x) = exp(-i k |x - x0|)/(4 pi |x - x0|), prm = x0 (3 per column)
 *   kind 2: plane wave u(x) = exp(-i k d.x), prm = d (3 per column)
 * and, for the Maxwell operator only, DiscreteLinearForm<RotatedTangentialTrace<cplx>, Op>
 * (LinearForm/RotatedTangentialTrace.hpp:30-87) of
 *   kind 3: the field of a Hertz dipole (examples/Data.hpp:73-90), prm = position,
 *           moment (6 doubles per column).
 * Output: nrhs load vectors (N x nrhs, column-major, ld = N), host or device.
 * nrhs == 0: BG_OK, nothing written. */
bg_status bg_load_vector(bg_operator* op, int kind, const double* prm, int nrhs, void* out, int on_device);

/* GMRES on the H2 operator with iterative refinement (replaces the Eigen
 * solvers called at examples/LaplaceSingleLayerH2.cpp:78-81 and
 * examples/HelmholtzSingleLayerH2.cpp:82-85). Residuals, the near field and the
 * Krylov basis are FP64; the inner correction operator is params->inner_precision.
 * nrhs == 0: BG_OK with zeroed stats. */
bg_status bg_solve(bg_operator* op, const void* b, void* x, int nrhs, const bg_solve_params* params,
                   bg_solve_stats* stats, int on_device);

/* DiscretePotential<...SingleLayerPotential>::evaluate (Potential/DiscretePotential.hpp:49-107)
 * at npts points (3 doubles each) for nrhs densities rho (N x nrhs), host
 * pointers. Laplace / Helmholtz: out is npts x nrhs (column-major). Maxwell
 * (Maxwell/SingleLayerPotential.hpp:44-95): the field, 3 complex values per
 * point, out[(c * npts + p) * 3 + xyz]. nrhs == 0 or npts == 0: BG_OK, nothing written. */
bg_status bg_potential(bg_operator* op, const void* rho, int nrhs, const double* pts, int npts, void* out);

/* Device memory of an operator: *allocated = bytes it holds now (tables,
 * assembled fields, work vectors, solver workspaces); *estimate = bytes it
 * will hold once assembled and used for solves of up to 32 right-hand sides
 * (computable before bg_operator_assemble; the serving loop admits by it). */
bg_status bg_operator_memory(const bg_operator* op, size_t* allocated, size_t* estimate);

/* Watchdog self-test (no reference counterpart): runs the bounded device wait
 * that the tensor-core kernels use on an mbarrier that nothing completes,
 * limited to limit_cycles SM clock cycles. Returns BG_TIMEOUT (the expected
 * outcome: the wait ran out, the kernel reported it and returned) with the
 * context still usable, BG_OK if the wait completed. */
bg_status bg_watchdog_selftest(bg_context* ctx, long long limit_cycles);

/* ---- launch plans and the autotuner (no reference counterpart) ----
 * A launch plan fixes the kernel variants and schedules of the H2 product for
 * one (number of right-hand sides, precision). Products with no plan set use
 * the built-in choices ({0, -1, 0}). The FP64 product has no choices. */
typedef struct bg_launch_plan {
  /* FP32 near field (BG_PREC_FP32): 0 built-in choice; 1 the pipelined block
   * kernel; 2 register tiles (complex: 2 block rows per thread); 3 complex
   * register tiles of 4 block rows. A variant the block shape does not allow
   * falls back to the built-in choice. */
  int near_kernel;
  /* FP32 transforms: launches of at most this many CTAs (batch items x
   * 32-column panels) use the split-K kernel; -1 built-in (152), 0 never. */
  int split_k_batches;
  /* order of the far-field rows over the persistent CTAs, which take items
   * b, b + G, b + 2G, ...: 0 heaviest first; 1 heaviest first with every
   * second round reversed; 2 heaviest first, each round's items to the CTAs
   * with the least work so far. Results are identical for every order. */
  int far_order;
  /* FMM transforms of scalar operators: 0 built-in (one fused launch per
   * direction through the tensor-product factors of the transfer and moment
   * matrices, where the operator has a transfer level); 1 batched GEMMs with
   * the assembled matrices, level by level. Results agree to rounding. */
  int transforms;
  /* stored-tile far field of real operators (BG_PREC_MIXED, BG_PREC_FP32):
   * 0 built-in (2 when there are at least twice as many far-field rows as
   * SMs, else 1); 1 one persistent CTA of four shared-memory stages per SM;
   * 2 two CTAs of two stages per SM. Results are identical. */
  int far_ctas;
  /* FP64-accurate near field of BG_PREC_MIXED products of real operators:
   * 0 built-in (the tensor-core product on 8 integer digits of 7 bits per
   * operand, exact integer accumulation, where the leaf block size allows
   * it: 4, 16 or 36 rows; else 1); 1 double-float on the FP32 pipes; 2 the
   * double-float product with a quarter of 32 columns on the FP64 pipe
   * (32 columns only, else 1). All agree with the FP64 product to about
   * 1e-14 relative or better. */
  int mixed_near;
  /* couplings of the stored-tile far field of real operators (BG_PREC_MIXED,
   * BG_PREC_FP32): 0 built-in, the FP16 hi and lo tiles (three products per
   * block, about 22 bits of every coupling, product error about 2e-7);
   * 1 the FP16 hi tiles only (two products, half the bytes streamed, about
   * 11 bits, product error about 1e-4): an inner operator for solvers that
   * refine in FP64, which absorb the error in their outer iterations. */
  int far_tiles;
} bg_launch_plan;

typedef struct bg_tune_report {
  int candidates;        /* plans timed */
  double builtin_ms;     /* product between T x and T^T y, built-in plan */
  double tuned_ms;       /* the same with the chosen plan */
  bg_launch_plan plan;   /* the chosen plan (now set on the operator) */
} bg_tune_report;

/* Set / read the plan of products with nrhs right-hand sides at precision.
 * Setting a plan drops the operator's captured CUDA graphs. */
bg_status bg_operator_set_plan(bg_operator* op, int nrhs, int precision, const bg_launch_plan* plan);
bg_status bg_operator_get_plan(const bg_operator* op, int nrhs, int precision, bg_launch_plan* plan);

/* Autotuner: times the product (between T x and T^T y) on seeded inputs with
 * CUDA events, reps products per candidate (0: 5), one knob at a time from
 * the built-in plan, keeps a change only when it is at least 2 % faster, and
 * sets the chosen plan. Needs an assembled operator on a device context. */
bg_status bg_operator_autotune(bg_operator* op, int nrhs, int precision, int reps, bg_tune_report* report);

/* ---- serving loop ----
 * No counterpart in the reference (its examples assemble one operator and
 * solve once). A server owns worker threads on the context's GPU, a queue of
 * solve requests and a cache of assembled operators keyed by (geometry, kind,
 * M, P, wavenumber). Requests for the same operator that are waiting together
 * are solved as one multi-column batch (up to 32 right-hand sides). Admission
 * is by device memory: an operator that is not cached is created only after
 * least-recently-used operators have been evicted until its estimated
 * footprint fits the server's budget; a request whose operator alone exceeds
 * the budget fails with BG_OOM. Load vectors are assembled on the device from
 * analytic data (bg_load_vector kinds), solutions are copied to host memory
 * the caller keeps valid until the request is done. The context must not be
 * used by other threads while a server runs on it. */
typedef struct bg_server bg_server;
typedef struct {
  int geometry;          /* index returned by bg_server_add_geometry */
  int op_kind;           /* bg_op_kind */
  int M, P;
  double kre, kim;       /* wavenumber (Helmholtz, Maxwell) */
  int data_kind;         /* bg_load_vector kind */
  int nrhs;              /* 1 .. 32 */
  const double* data;    /* nrhs x 3 (kind 3: x 6) data parameters, copied at submit */
  double tol;            /* relative residual per column */
  int inner_precision;   /* bg_precision of the inner operator (BG_PREC_FP64: plain FP64 GMRES) */
  void* x;               /* host, N x nrhs column-major (complex interleaved) */
  long x_capacity;       /* scalars available at x */
} bg_request;
typedef struct {
  int status;            /* bg_status of the solve */
  int N;                 /* unknowns of the operator */
  double t_submit, t_start, t_done;  /* seconds since the server started */
  int cache_hit;         /* operator was cached when the request's batch started */
  int batch_nrhs;        /* right-hand sides solved together with this request */
  bg_solve_stats stats;
  char error[160];       /* message of a failed request (empty on success) */
} bg_request_result;
typedef struct {
  long submitted, completed, failed, batches;
  long cache_hits, cache_misses, evictions;
  size_t bytes_in_use, bytes_budget;
  double assembly_s, solve_s;  /* worker time spent assembling / solving */
  int cached_operators;
} bg_server_stats;

/* workers: 1 .. 16 worker threads, each with its own context (stream) on
 * ctx's device; solves on different operators overlap on the GPU. An
 * operator runs on the worker that assembled it (requests for it wait for
 * that worker); a request for an operator no worker holds goes to the first
 * free worker. hbm_budget_bytes is shared by all workers: an operator is
 * admitted once its estimated footprint fits, after evicting the least
 * recently used idle operators of any worker (waiting for busy ones when
 * nothing idle is left); one larger than the whole budget fails with BG_OOM. */
bg_status bg_server_create(bg_context* ctx, size_t hbm_budget_bytes, int workers, bg_server** out);
/* stops the workers after the queue drains and frees every cached operator;
 * no other thread may be inside a bg_server_* call on srv meanwhile */
bg_status bg_server_destroy(bg_server* srv);
bg_status bg_server_add_geometry(bg_server* srv, const bg_geometry* g, int* index);
bg_status bg_server_submit(bg_server* srv, const bg_request* req, long* ticket);
/* blocks until the request is done (timeout_s < 0: no limit; BG_TIMEOUT when
 * it runs out) and collects its result; a ticket that was never issued or was
 * already collected returns BG_INVALID_ARG */
bg_status bg_server_wait(bg_server* srv, long ticket, double timeout_s, bg_request_result* out);
bg_status bg_server_stats_get(bg_server* srv, bg_server_stats* out);

/* ---- inspection entry points used by the parity tests ---- */
/* per element id: patch, vertex ids[4]; and llc[2], ball midpoint[3], radius */
bg_status bg_operator_elements(const bg_operator* op, int* ints5, double* dbl6);
/* per leaf: admissibility (2 dense, 1 low-rank), level, cluster1 id, cluster2 id */
bg_status bg_operator_leaves(const bg_operator* op, int* out4);
/* transformation matrix T (superspace x dofs) in CSR */
bg_status bg_operator_transform(const bg_operator* op, int* ptr, int* idx, double* val);
/* copy one assembled leaf block (row component rc, column component cc) to the
 * host, column-major (complex interleaved); leaf indexes bg_operator_leaves */
bg_status bg_operator_leaf_block(const bg_operator* op, long leaf, int rc, int cc, double* out);

#ifdef __cplusplus
}
#endif
#endif /* BEMBEL_GB300_H_ */
