// Header-style C++ front end of bembel_gb300 (the GB300 H2 single-layer
// operator) over its C ABI, include/bembel_gb300.h.
//
// Three layers, each usable on its own:
//  1. bembel_gb300::{Context, Geometry, Operator<Scalar>}: RAII owners of the C
//     handles; errors become bembel_gb300::Error exceptions (nothing throws
//     across the C ABI itself). Needs only this header and the library.
//  2. Eigen::H2MatrixGPU<Scalar>: a matrix-free operator for Eigen's iterative
//     solvers, with the traits and product glue Bembel's own Eigen::H2Matrix
//     has (H2Matrix/H2Matrix.hpp:26-56, EigenHelper/H2DenseProduct.hpp:268-290):
//     A * X for a vector or a block of columns forwards to bg_matvec, so
//     Eigen::GMRES / ConjugateGradient run on it unchanged. Compiled when
//     <Eigen/Core> is available.
//  3. Bembel::DiscreteOperatorComputer<Eigen::H2MatrixGPU<S>, Op>: the
//     specialisation point of Bembel's DiscreteOperator
//     (LinearOperator/DiscreteOperator.hpp:21-22, 92-102), so that
//       Bembel::DiscreteOperator<Eigen::H2MatrixGPU<double>,
//                                Bembel::LaplaceSingleLayerOperator> op(space);
//       op.compute();
//     assembles on the GPU from the AnsatzSpace's geometry, refinement and
//     degree. Compiled when Bembel's headers are available (include them
//     before this one).
#ifndef BEMBEL_GB300_H2MATRIXGPU_HPP_
#define BEMBEL_GB300_H2MATRIXGPU_HPP_

#include <complex>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "../bembel_gb300.h"

namespace bembel_gb300 {

class Error : public std::runtime_error {
 public:
  Error(bg_status status, const std::string& what) : std::runtime_error(what), status_(status) {}
  bg_status status() const { return status_; }

 private:
  bg_status status_;
};

namespace detail {
inline const char* status_name(bg_status s) {
  switch (s) {
    case BG_OK: return "BG_OK";
    case BG_INVALID_ARG: return "BG_INVALID_ARG";
    case BG_OOM: return "BG_OOM";
    case BG_UNSUPPORTED: return "BG_UNSUPPORTED";
    case BG_DEVICE_ERROR: return "BG_DEVICE_ERROR";
    case BG_TIMEOUT: return "BG_TIMEOUT";
    case BG_CANCELLED: return "BG_CANCELLED";
    case BG_NOT_CONVERGED: return "BG_NOT_CONVERGED";
  }
  return "bg_status";
}
inline void check(bg_status s, bg_context* ctx) {
  if (s == BG_OK) return;
  std::string msg = status_name(s);
  if (ctx) {
    const char* e = bg_last_error_string(ctx);
    if (e && *e) msg += std::string(": ") + e;
  }
  throw Error(s, msg);
}
template <typename S>
struct ScalarKind;
template <>
struct ScalarKind<double> {
  static constexpr bool complex = false;
};
template <>
struct ScalarKind<std::complex<double>> {
  static constexpr bool complex = true;
};
}  // namespace detail

// One GPU (device >= 0) or a host-only context (-1: setup and inspection only).
class Context {
 public:
  explicit Context(int device = 0) {
    bg_context* c = nullptr;
    detail::check(bg_context_create(device, &c), nullptr);
    h_ = std::shared_ptr<bg_context>(c, [](bg_context* p) { bg_context_destroy(p); });
  }
  bg_context* get() const { return h_.get(); }

 private:
  std::shared_ptr<bg_context> h_;
};

// Geometry(filename) (Geometry/Geometry.hpp:89-102) or from Bezier patch data
// in the layout of Bembel's Patch::data_ (see bg_geometry_from_bezier).
class Geometry {
 public:
  static Geometry from_dat(const Context& ctx, const std::string& path) {
    bg_geometry* g = nullptr;
    detail::check(bg_geometry_load_dat(ctx.get(), path.c_str(), &g), ctx.get());
    return Geometry(ctx, g);
  }
  static Geometry from_bezier(const Context& ctx, const std::vector<int>& px, const std::vector<int>& py,
                              const std::vector<double>& data) {
    if (px.size() != py.size()) throw Error(BG_INVALID_ARG, "from_bezier: px and py differ in length");
    bg_geometry* g = nullptr;
    detail::check(bg_geometry_from_bezier(ctx.get(), (int)px.size(), px.data(), py.data(), data.data(), &g),
                  ctx.get());
    return Geometry(ctx, g);
  }
  // the unit sphere as six analytic patches x/|x| of the cube faces (no
  // Bembel counterpart; see bg_geometry_cube_sphere)
  static Geometry cube_sphere(const Context& ctx) {
    bg_geometry* g = nullptr;
    detail::check(bg_geometry_cube_sphere(ctx.get(), &g), ctx.get());
    return Geometry(ctx, g);
  }
  int num_patches() const {
    int n = 0;
    detail::check(bg_geometry_num_patches(h_.get(), &n), ctx_.get());
    return n;
  }
  // patch p's control data: (px, py, 4 px py homogeneous values)
  std::vector<double> patch_data(int p, int* px, int* py) const {
    detail::check(bg_geometry_patch_data(h_.get(), p, px, py, nullptr), ctx_.get());
    std::vector<double> d(4 * (size_t)(*px) * (size_t)(*py));
    detail::check(bg_geometry_patch_data(h_.get(), p, px, py, d.data()), ctx_.get());
    return d;
  }
  bg_geometry* get() const { return h_.get(); }
  const Context& context() const { return ctx_; }

 private:
  Geometry(const Context& ctx, bg_geometry* g)
      : ctx_(ctx), h_(g, [](bg_geometry* p) { bg_geometry_destroy(p); }) {}
  Context ctx_;
  std::shared_ptr<bg_geometry> h_;
};

// The H2 single-layer operator of one discretisation (AnsatzSpace(geometry,
// M, P) + DiscreteOperator<H2Matrix<S>, Op>); Scalar = double (Laplace) or
// std::complex<double> (Helmholtz, Maxwell).
template <typename Scalar>
class Operator {
 public:
  Operator(const Geometry& geo, int refinement_level, int polynomial_degree, int op_kind,
           const bg_h2_params* params = nullptr)
      : geo_(geo) {
    bg_operator* o = nullptr;
    detail::check(bg_operator_create(geo.context().get(), geo.get(), refinement_level, polynomial_degree, op_kind,
                                     params, &o),
                  geo.context().get());
    h_ = std::shared_ptr<bg_operator>(o, [](bg_operator* p) { bg_operator_destroy(p); });
    long info[16];
    detail::check(bg_operator_info(o, info), ctx());
    if ((info[8] != 0) != detail::ScalarKind<Scalar>::complex)
      throw Error(BG_INVALID_ARG, "Operator<Scalar>: scalar type does not match the operator kind");
    n_ = info[0];
  }
  void set_wavenumber(std::complex<double> kappa) {
    detail::check(bg_operator_set_wavenumber(h_.get(), kappa.real(), kappa.imag()), ctx());
  }
  void assemble() { detail::check(bg_operator_assemble(h_.get()), ctx()); }
  long rows() const { return n_; }
  long cols() const { return n_; }
  // Y = beta Y + alpha A X for nrhs columns (column-major, leading dimensions
  // ldx, ldy); host pointers unless on_device
  void matvec(const Scalar* x, long ldx, Scalar* y, long ldy, int nrhs, Scalar alpha = Scalar(1),
              Scalar beta = Scalar(0), int precision = BG_PREC_FP64, bool on_device = false) const {
    const double a[2] = {std::real(alpha), std::imag(alpha)}, b[2] = {std::real(beta), std::imag(beta)};
    detail::check(bg_matvec(h_.get(), x, ldx, y, ldy, nrhs, a, b, precision, on_device ? 1 : 0), ctx());
  }
  // solve A X = B (column-major N x nrhs, ld = N) with the library's solver
  bg_solve_stats solve(const Scalar* b, Scalar* x, int nrhs, const bg_solve_params* params = nullptr,
                       bool on_device = false) const {
    bg_solve_stats st{};
    detail::check(bg_solve(h_.get(), b, x, nrhs, params, &st, on_device ? 1 : 0), ctx());
    return st;
  }
  // launch plan of products with nrhs columns at precision; autotune() times
  // the variants on the GPU and sets the fastest plan
  void set_plan(int nrhs, int precision, const bg_launch_plan& plan) {
    detail::check(bg_operator_set_plan(h_.get(), nrhs, precision, &plan), ctx());
  }
  bg_launch_plan plan(int nrhs, int precision) const {
    bg_launch_plan p{};
    detail::check(bg_operator_get_plan(h_.get(), nrhs, precision, &p), ctx());
    return p;
  }
  bg_tune_report autotune(int nrhs, int precision, int reps = 0) {
    bg_tune_report r{};
    detail::check(bg_operator_autotune(h_.get(), nrhs, precision, reps, &r), ctx());
    return r;
  }
  bg_operator* get() const { return h_.get(); }
  bg_context* ctx() const { return geo_.context().get(); }

 private:
  Geometry geo_;
  std::shared_ptr<bg_operator> h_;
  long n_ = 0;
};

}  // namespace bembel_gb300

#if defined(__has_include)
#if __has_include(<Eigen/Core>) && __has_include(<Eigen/Sparse>)
#include <Eigen/Core>
#include <Eigen/Sparse>

#if defined(BEMBEL_SRC_H2MATRIX_H2MATRIXBASE_HPP_) && defined(BEMBEL_SRC_H2MATRIX_EIGENHELPER_H2DENSEPRODUCT_HPP_)
// Bembel's H2Matrix module is included: H2MatrixGPU joins Bembel's own H2
// storage kind (H2Matrix/EigenHelper/Constants.hpp), so every expression
// Bembel's Eigen glue accepts for H2Matrix works for it too: A * x, and the
// distributive and associative rewrites (H2 + H2, D + H2, H2 - D, a * H2) of
// H2DenseProduct.hpp:179-258, which end in H2_time_dense_product_impl below.
namespace Eigen {
template <typename Scalar_>
class H2MatrixGPU;
namespace internal {
// as traits<H2Matrix<S>> (H2Matrix.hpp:32-45)
template <typename Scalar_>
struct traits<H2MatrixGPU<Scalar_>> {
  typedef Scalar_ Scalar;
  typedef int StorageIndex;
  typedef H2 StorageKind;
  typedef MatrixXpr XprKind;
  enum {
    RowsAtCompileTime = Dynamic,
    ColsAtCompileTime = Dynamic,
    MaxRowsAtCompileTime = Dynamic,
    MaxColsAtCompileTime = Dynamic,
    Flags = NestByRefBit
  };
};
// as is_ref_compatible<H2Matrix<S>> (H2Matrix.hpp:48-54): Eigen's solvers
// must hold the operator by reference, never copy it into a Ref
template <typename Scalar_>
struct is_ref_compatible<H2MatrixGPU<Scalar_>> {
  enum { value = false };
};
template <typename Scalar_>
struct is_ref_compatible<const H2MatrixGPU<Scalar_>> : is_ref_compatible<H2MatrixGPU<Scalar_>> {};
}  // namespace internal

template <typename Scalar_>
class H2MatrixGPU : public H2MatrixBase<H2MatrixGPU<Scalar_>> {
 public:
  typedef Scalar_ Scalar;
  typedef typename NumTraits<Scalar>::Real RealScalar;
  typedef Index StorageIndex;
  enum { ColsAtCompileTime = Dynamic, MaxColsAtCompileTime = Dynamic, IsRowMajor = false, Flags = NestByRefBit };

  H2MatrixGPU() {}
  explicit H2MatrixGPU(std::shared_ptr<bembel_gb300::Operator<Scalar>> op) : op_(std::move(op)) {}
  Index rows() const { return op_ ? op_->rows() : 0; }
  Index cols() const { return op_ ? op_->cols() : 0; }
  template <typename Rhs>
  Product<H2MatrixGPU, Rhs, AliasFreeProduct> operator*(const MatrixBase<Rhs>& x) const {
    return Product<H2MatrixGPU, Rhs, AliasFreeProduct>(*this, x.derived());
  }
  // precision of the products Eigen's solvers request (bg_precision)
  void set_precision(int p) { precision_ = p; }
  int precision() const { return precision_; }
  const std::shared_ptr<bembel_gb300::Operator<Scalar>>& gpu_operator() const { return op_; }
  void set_gpu_operator(std::shared_ptr<bembel_gb300::Operator<Scalar>> op) { op_ = std::move(op); }

 private:
  std::shared_ptr<bembel_gb300::Operator<Scalar>> op_;
  int precision_ = BG_PREC_FP64;
};

namespace internal {
// res += alpha * A * rhs, all columns in one bg_matvec call (the reference
// runs one H2 product per column, H2DenseProduct.hpp:33-165); reached from
// generic_product_impl<Lhs, Rhs, H2, DenseShape, ...>::scaleAndAddTo
// (H2DenseProduct.hpp:260-290) for H2MatrixGPU and every expression of it
template <typename Scalar_, typename DenseRhsType, typename DenseResType, typename AlphaType>
struct H2_time_dense_product_impl<H2MatrixGPU<Scalar_>, DenseRhsType, DenseResType, AlphaType, ColMajor, true> {
  static void run(const H2MatrixGPU<Scalar_>& lhs, const DenseRhsType& rhs, DenseResType& res,
                  const AlphaType& alpha) {
    typedef Matrix<Scalar_, Dynamic, Dynamic> Block;
    const Block x = rhs;  // contiguous, column-major
    Block y = res;
    lhs.gpu_operator()->matvec(x.data(), x.rows(), y.data(), y.rows(), (int)x.cols(), Scalar_(alpha), Scalar_(1),
                               lhs.precision(), false);
    res = y;
  }
};
}  // namespace internal
}  // namespace Eigen

#else
// Eigen alone (no Bembel): a matrix-free operator with SparseMatrix traits
// (the trick H2Matrix.hpp:16-25 describes), enough for Eigen's iterative
// solvers; expressions of several operators need Bembel's H2 storage kind.
namespace Eigen {
template <typename Scalar_>
class H2MatrixGPU;
namespace internal {
template <typename Scalar_>
struct traits<H2MatrixGPU<Scalar_>> : public traits<SparseMatrix<Scalar_>> {};
template <typename Scalar_>
struct is_ref_compatible<H2MatrixGPU<Scalar_>> {
  enum { value = false };
};
template <typename Scalar_>
struct is_ref_compatible<const H2MatrixGPU<Scalar_>> : is_ref_compatible<H2MatrixGPU<Scalar_>> {};
}  // namespace internal

template <typename Scalar_>
class H2MatrixGPU : public EigenBase<H2MatrixGPU<Scalar_>> {
 public:
  typedef Scalar_ Scalar;
  typedef typename NumTraits<Scalar>::Real RealScalar;
  typedef int StorageIndex;
  enum { ColsAtCompileTime = Dynamic, MaxColsAtCompileTime = Dynamic, IsRowMajor = false };

  H2MatrixGPU() {}
  explicit H2MatrixGPU(std::shared_ptr<bembel_gb300::Operator<Scalar>> op) : op_(std::move(op)) {}
  Index rows() const { return op_ ? op_->rows() : 0; }
  Index cols() const { return op_ ? op_->cols() : 0; }
  template <typename Rhs>
  Product<H2MatrixGPU, Rhs, AliasFreeProduct> operator*(const MatrixBase<Rhs>& x) const {
    return Product<H2MatrixGPU, Rhs, AliasFreeProduct>(*this, x.derived());
  }
  void set_precision(int p) { precision_ = p; }
  int precision() const { return precision_; }
  const std::shared_ptr<bembel_gb300::Operator<Scalar>>& gpu_operator() const { return op_; }
  void set_gpu_operator(std::shared_ptr<bembel_gb300::Operator<Scalar>> op) { op_ = std::move(op); }

 private:
  std::shared_ptr<bembel_gb300::Operator<Scalar>> op_;
  int precision_ = BG_PREC_FP64;
};

namespace internal {
// dst += alpha * A * rhs for a vector or a block of columns
// (generic_product_impl::scaleAndAddTo, H2DenseProduct.hpp:268-290)
template <typename Scalar_, typename Rhs>
struct generic_product_impl<H2MatrixGPU<Scalar_>, Rhs, SparseShape, DenseShape, GemvProduct>
    : generic_product_impl_base<H2MatrixGPU<Scalar_>, Rhs,
                                generic_product_impl<H2MatrixGPU<Scalar_>, Rhs>> {
  typedef typename Product<H2MatrixGPU<Scalar_>, Rhs>::Scalar Scalar;
  template <typename Dest>
  static void scaleAndAddTo(Dest& dst, const H2MatrixGPU<Scalar_>& lhs, const Rhs& rhs, const Scalar& alpha) {
    typedef Matrix<Scalar_, Dynamic, Dynamic> Block;
    const Block x = rhs;  // contiguous, column-major
    Block y = dst;
    lhs.gpu_operator()->matvec(x.data(), x.rows(), y.data(), y.rows(), (int)x.cols(), Scalar_(alpha), Scalar_(1),
                               lhs.precision(), false);
    dst = y;
  }
};
}  // namespace internal
}  // namespace Eigen
#endif

#if __has_include(<Bembel/AnsatzSpace>) && defined(BEMBEL_SRC_LINEAROPERATOR_DISCRETEOPERATOR_HPP_)
namespace Bembel {
namespace gb300_detail {
// the wavenumber of the Helmholtz and Maxwell operators; Laplace has none.
// The reference's get_wavenumber() is not const
// (Helmholtz/SingleLayerOperator.hpp:130, Maxwell/SingleLayerOperator.hpp:141),
// so it is read from a copy. Overloads instead of `if constexpr`: Bembel
// builds as C++11 (CMakeLists.txt:74).
template <typename Derived>
inline void set_wavenumber(bembel_gb300::Operator<std::complex<double>>& op, const Derived& lin_op) {
  Derived copy(lin_op);
  op.set_wavenumber(std::complex<double>(copy.get_wavenumber()));
}
template <typename Derived>
inline void set_wavenumber(bembel_gb300::Operator<double>&, const Derived&) {}
template <typename Derived>
inline int op_kind() {
  return std::is_same<Derived, HelmholtzSingleLayerOperator>::value
             ? BG_HELMHOLTZ_SL
             : (std::is_same<Derived, MaxwellSingleLayerOperator>::value ? BG_MAXWELL_SL : BG_LAPLACE_SL);
}
}  // namespace gb300_detail

template <typename Derived>
struct DiscreteOperatorComputer<Eigen::H2MatrixGPU<typename LinearOperatorTraits<Derived>::Scalar>, Derived> {
  typedef typename LinearOperatorTraits<Derived>::Scalar Scalar;
  DiscreteOperatorComputer() {}
  // H2Matrix::init_H2Matrix (H2Matrix.hpp:93-250) on the GPU: the AnsatzSpace's
  // Bezier patches, refinement level and degree define the discretisation;
  // the H2 parameters are the reference's defaults (n_p = 9, eta = 1.6, mcl = 1)
  static void compute(Eigen::H2MatrixGPU<Scalar>* disc_op, const Derived& lin_op,
                      const AnsatzSpace<Derived>& ansatz_space) {
    static bembel_gb300::Context ctx(0);
    const PatchVector& patches = ansatz_space.get_geometry();
    std::vector<int> px, py;
    std::vector<double> data;
    for (const auto& p : patches) {
      if (p.unique_knots_x_.size() != 2 || p.unique_knots_y_.size() != 2)
        throw bembel_gb300::Error(BG_UNSUPPORTED, "patches with interior knots are not supported");
      px.push_back(p.polynomial_degree_x_);
      py.push_back(p.polynomial_degree_y_);
      data.insert(data.end(), p.data_.begin(), p.data_.end());
    }
    auto geo = bembel_gb300::Geometry::from_bezier(ctx, px, py, data);
    auto op = std::make_shared<bembel_gb300::Operator<Scalar>>(geo, ansatz_space.get_refinement_level(),
                                                               ansatz_space.get_polynomial_degree(),
                                                               gb300_detail::op_kind<Derived>());
    gb300_detail::set_wavenumber<Derived>(*op, lin_op);
    op->assemble();
    disc_op->set_gpu_operator(op);
  }
};
}  // namespace Bembel
#endif
#endif
#endif

#endif  // BEMBEL_GB300_H2MATRIXGPU_HPP_
