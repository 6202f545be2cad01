"""bembel_gb300 — GB300-native H2 single-layer boundary element operator.

Python mirror of the reference's user-facing interface for the H2 path
(Geometry, AnsatzSpace, {Laplace,Helmholtz,Maxwell}SingleLayerOperator,
DiscreteOperator<H2Matrix<S>, Op>, H2Matrix * x, DiscreteLinearForm,
DiscretePotential), over the C ABI of include/bembel_gb300.h.

    geo = Geometry("sphere.dat")
    space = AnsatzSpace(geo, refinement_level=5, polynomial_degree=2)
    op = DiscreteOperator(space, LaplaceSingleLayerOperator())
    op.compute()
    A = op.get_discrete_operator()
    y = A @ x                       # FP64 H2 matvec on the GPU
    x, stats = A.solve(b, tol=1e-8) # GMRES with FP64 iterative refinement

Arrays may be numpy arrays (host memory) or CUDA torch tensors (device
memory); blocks of right-hand sides are (N, nrhs).
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import BembelError, H2Params, SolveParams, SolveStats

__all__ = ["Context", "Geometry", "AnsatzSpace", "LaplaceSingleLayerOperator", "HelmholtzSingleLayerOperator",
           "MaxwellSingleLayerOperator", "DiscreteOperator", "H2Matrix", "Server", "BembelError", "default_context"]

_default_ctx = None


class Context:
    """One GPU (device >= 0) or a host-only context (device = -1) that can build
    and inspect discretisations but runs no device work."""

    def __init__(self, device=0):
        L = _lib.load()
        h = ctypes.c_void_p()
        st = L.bg_context_create(device, ctypes.byref(h))
        if st != _lib.BG_OK:
            raise BembelError(st, "cannot create a context on device %d" % device)
        self.h = h
        self.device = device

    def close(self):
        if getattr(self, "h", None):
            _lib.load().bg_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, st):
        _lib.check(st, self.h)


def default_context():
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


class Geometry:
    """Geometry(filename): patches of a .dat or .igs/.iges file (Geometry/Geometry.hpp:89-102)."""

    def __init__(self, filename, context=None):
        self.ctx = context or default_context()
        h = ctypes.c_void_p()
        igs = str(filename).lower().endswith((".igs", ".iges"))
        load = _lib.load().bg_geometry_load_igs if igs else _lib.load().bg_geometry_load_dat
        self.ctx.check(load(self.ctx.h, str(filename).encode(), ctypes.byref(h)))
        self.h = h
        self.filename = str(filename)

    @classmethod
    def cube_sphere(cls, context=None):
        """The unit sphere as six analytic patches, each the image x/|x| of one
        face of the cube [-1, 1]^3 (no control points; the reference's patches
        are rational B-splines only, Patch.hpp:63-104)."""
        self = cls.__new__(cls)
        self.ctx = context or default_context()
        h = ctypes.c_void_p()
        self.ctx.check(_lib.load().bg_geometry_cube_sphere(self.ctx.h, ctypes.byref(h)))
        self.h = h
        self.filename = None
        return self

    def surface_point(self, patch, s, t):
        out = np.zeros(12)
        self.ctx.check(_lib.load().bg_geometry_surface_point(self.h, patch, s, t, _dp(out)))
        return out

    def __del__(self):
        try:
            if getattr(self, "h", None):
                _lib.load().bg_geometry_destroy(self.h)
                self.h = None
        except Exception:
            pass


class AnsatzSpace:
    """AnsatzSpace(geometry, refinement_level, polynomial_degree) (AnsatzSpace.hpp:82-111)."""

    def __init__(self, geometry, refinement_level, polynomial_degree, knot_repetition=1):
        if knot_repetition != 1:
            raise BembelError(_lib.BG_UNSUPPORTED, "knot repetition other than 1")
        self.geometry = geometry
        self.refinement_level = int(refinement_level)
        self.polynomial_degree = int(polynomial_degree)


class _SingleLayer:
    kind = None
    is_complex = False

    def __init__(self):
        self.wavenumber = 0j

    def set_wavenumber(self, k):
        self.wavenumber = complex(k)

    def get_wavenumber(self):
        return self.wavenumber


class LaplaceSingleLayerOperator(_SingleLayer):
    """1/(4 pi |x-y|) (Laplace/SingleLayerOperator.hpp)."""
    kind = _lib.LAPLACE_SL


class HelmholtzSingleLayerOperator(_SingleLayer):
    """exp(-i k |x-y|)/(4 pi |x-y|) (Helmholtz/SingleLayerOperator.hpp)."""
    kind = _lib.HELMHOLTZ_SL
    is_complex = True


class MaxwellSingleLayerOperator(_SingleLayer):
    """Electric field integral operator (Maxwell/SingleLayerOperator.hpp)."""
    kind = _lib.MAXWELL_SL
    is_complex = True


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _is_torch(x):
    return type(x).__module__.startswith("torch")


def _columns(a, n):
    """a (a vector or an n x k block, k = 0 allowed) as n x k."""
    size = a.numel() if _is_torch(a) else a.size
    return a.reshape(n, size // n if n else 0)


def _prec_code(precision):
    if precision not in _lib.PRECISIONS:
        raise BembelError(_lib.BG_INVALID_ARG, "precision must be one of %s" % sorted(_lib.PRECISIONS))
    return _lib.PRECISIONS[precision]


class H2Matrix:
    """Device-resident H2 matrix; rows() == cols() == number of DOFs."""

    def __init__(self, dop):
        self._dop = dop

    @property
    def h(self):
        return self._dop.h

    def rows(self):
        return self._dop.N

    def cols(self):
        return self._dop.N

    @property
    def shape(self):
        return (self._dop.N, self._dop.N)

    @property
    def dtype(self):
        return np.complex128 if self._dop.is_complex else np.float64

    def __matmul__(self, x):
        return self.matvec(x)

    def matvec(self, x, precision="fp64", out=None, alpha=1.0, beta=0.0):
        """out = beta * out + alpha * A x (H2DenseProduct.hpp:268-290).
        precision "fp64": the FP64 H2 matrix; "mixed": FP64 near field, FP32
        on-the-fly far field; "fp32": near and far field in FP32."""
        if precision not in _lib.PRECISIONS:
            raise BembelError(_lib.BG_INVALID_ARG, "precision must be one of %s" % sorted(_lib.PRECISIONS))
        prec = _lib.PRECISIONS[precision]
        N = self._dop.N
        a = np.array([complex(alpha).real, complex(alpha).imag])
        b = np.array([complex(beta).real, complex(beta).imag])
        if _is_torch(x):
            import torch
            squeeze = x.dim() == 1
            X = (_columns(x, N)).t().contiguous()  # (nrhs, N): column-major N x nrhs
            Y = torch.empty_like(X) if out is None else _columns(out, N).t().contiguous()
            on_dev = 1 if X.is_cuda else 0
            if not on_dev:
                raise BembelError(_lib.BG_INVALID_ARG, "pass numpy arrays for host memory")
            self._dop.ctx.check(_lib.load().bg_matvec(self.h, ctypes.c_void_p(X.data_ptr()), N,
                                                      ctypes.c_void_p(Y.data_ptr()), N, X.shape[0], _dp(a), _dp(b),
                                                      prec, on_dev))
            Y = Y.t()
            return Y.reshape(N) if squeeze else Y
        x = np.asarray(x, dtype=self.dtype)
        squeeze = x.ndim == 1
        X = np.asfortranarray(_columns(x, N))
        Y = np.zeros_like(X, order="F") if out is None else np.asfortranarray(_columns(np.asarray(out, self.dtype), N))
        self._dop.ctx.check(_lib.load().bg_matvec(self.h, X.ctypes.data_as(ctypes.c_void_p), N,
                                                  Y.ctypes.data_as(ctypes.c_void_p), N, X.shape[1], _dp(a), _dp(b),
                                                  prec, 0))
        return Y[:, 0].copy() if squeeze else Y

    def solve(self, b, tol=1e-8, restart=200, max_iter=3000, inner="fp32", inner_tol=2e-3, max_refinements=12):
        """GMRES with FP64 iterative refinement; returns (x, stats dict)."""
        p = SolveParams()
        _lib.load().bg_solve_params_default(ctypes.byref(p))
        p.tol, p.restart, p.max_iter = tol, restart, max_iter
        if inner not in _lib.PRECISIONS:
            raise BembelError(_lib.BG_INVALID_ARG, "inner must be one of %s" % sorted(_lib.PRECISIONS))
        p.inner_precision = _lib.PRECISIONS[inner]
        p.inner_tol, p.max_refinements = inner_tol, max_refinements
        st = SolveStats()
        N = self._dop.N
        if _is_torch(b):
            import torch
            squeeze = b.dim() == 1
            B = _columns(b, N).t().contiguous()
            X = torch.empty_like(B) if B.is_cuda else torch.empty(B.shape, dtype=B.dtype, pin_memory=B.is_pinned())
            status = _lib.load().bg_solve(self.h, ctypes.c_void_p(B.data_ptr()), ctypes.c_void_p(X.data_ptr()),
                                          B.shape[0], ctypes.byref(p), ctypes.byref(st), 1 if B.is_cuda else 0)
            x = X.t()
            x = x.reshape(N) if squeeze else x
        else:
            b = np.asarray(b, dtype=self.dtype)
            squeeze = b.ndim == 1
            B = np.asfortranarray(_columns(b, N))
            X = np.zeros_like(B, order="F")
            status = _lib.load().bg_solve(self.h, B.ctypes.data_as(ctypes.c_void_p), X.ctypes.data_as(ctypes.c_void_p),
                                          B.shape[1], ctypes.byref(p), ctypes.byref(st), 0)
            x = X[:, 0].copy() if squeeze else X
        stats = {k: getattr(st, k) for k, _ in SolveStats._fields_}
        if status not in (_lib.BG_OK, _lib.BG_NOT_CONVERGED):
            self._dop.ctx.check(status)
        stats["converged"] = status == _lib.BG_OK
        return x, stats


class DiscreteOperator:
    """DiscreteOperator<H2Matrix<S>, Op>(ansatz_space) (DiscreteOperator.hpp:107-145)."""

    def __init__(self, ansatz_space, linear_operator, n_p=9, eta=1.6, min_cluster_level=1, store_fp64_far=True,
                 keep_fp64_blocks=True):
        self.ansatz_space = ansatz_space
        self.lin_op = linear_operator
        self.ctx = ansatz_space.geometry.ctx
        prm = H2Params()
        _lib.load().bg_h2_params_default(ctypes.byref(prm))
        prm.n_p, prm.eta, prm.min_cluster_level, prm.store_fp64_far = n_p, eta, min_cluster_level, int(store_fp64_far)
        prm.keep_fp64_blocks = int(keep_fp64_blocks)
        h = ctypes.c_void_p()
        self.ctx.check(_lib.load().bg_operator_create(self.ctx.h, ansatz_space.geometry.h,
                                                      ansatz_space.refinement_level, ansatz_space.polynomial_degree,
                                                      linear_operator.kind, ctypes.byref(prm), ctypes.byref(h)))
        self.h = h
        info = self.info()
        self.N = int(info[0])
        self.S = int(info[1])
        self.ne = int(info[2])
        self.n_dense = int(info[3])
        self.n_lowrank = int(info[4])
        self.is_complex = bool(info[8])
        self._matrix = H2Matrix(self)

    def __del__(self):
        try:
            if getattr(self, "h", None):
                _lib.load().bg_operator_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def info(self):
        out = np.zeros(16, dtype=np.int64)
        self.ctx.check(_lib.load().bg_operator_info(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_long))))
        return out

    def get_linear_operator(self):
        return self.lin_op

    def compute(self):
        """Assemble the near and far field on the GPU (H2Matrix::init_H2Matrix)."""
        if self.lin_op.is_complex:
            k = complex(self.lin_op.wavenumber)
            self.ctx.check(_lib.load().bg_operator_set_wavenumber(self.h, k.real, k.imag))
        self.ctx.check(_lib.load().bg_operator_assemble(self.h))

    def prepare_wavenumbers(self, kappas):
        """Near fields of several Helmholtz wavenumbers in one pass
        (bg_operator_prepare_wavenumbers): compute() after set_wavenumber to
        one of them reuses its near field and assembles only the far field."""
        k = np.asarray(kappas, dtype=np.complex128).reshape(-1)
        re_, im_ = np.ascontiguousarray(k.real), np.ascontiguousarray(k.imag)
        self.ctx.check(_lib.load().bg_operator_prepare_wavenumbers(self.h, _dp(re_), _dp(im_), len(k)))

    def quadrature_counts(self):
        """Near-field quadrature work (bg_operator_quadrature_counts): pairs and
        integrand evaluations per rule (regular, identical, edge, vertex)."""
        out = np.zeros(8, dtype=np.int64)
        self.ctx.check(_lib.load().bg_operator_quadrature_counts(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_long))))
        names = ("regular", "identical", "edge", "vertex")
        return {n: {"pairs": int(out[2 * i]), "evaluations": int(out[2 * i + 1])} for i, n in enumerate(names)}

    def release_wavenumbers(self):
        self.ctx.check(_lib.load().bg_operator_release_wavenumbers(self.h))

    def assemble_wavenumbers(self):
        """Assemble every prepared wavenumber side by side
        (bg_operator_assemble_wavenumbers): afterwards products, solves, load
        vectors and potentials take n * k columns, block q (k columns) with
        wavenumber q in preparation order."""
        self.ctx.check(_lib.load().bg_operator_assemble_wavenumbers(self.h))

    def wavenumbers(self):
        """The batched wavenumbers in column-block order (empty when the
        operator holds one)."""
        n = ctypes.c_int()
        self.ctx.check(_lib.load().bg_operator_num_wavenumbers(self.h, ctypes.byref(n), None, None))
        re_, im_ = np.zeros(n.value), np.zeros(n.value)
        if n.value:
            self.ctx.check(_lib.load().bg_operator_num_wavenumbers(self.h, ctypes.byref(n), _dp(re_), _dp(im_)))
        return re_ + 1j * im_

    def assembly_times(self):
        t = np.zeros(3)
        self.ctx.check(_lib.load().bg_operator_assembly_times(self.h, _dp(t)))
        return {"near_s": t[0], "far_s": t[1], "total_s": t[2]}

    def get_discrete_operator(self):
        return self._matrix

    # -- load vectors / potentials (DiscreteLinearForm, DiscretePotential) --
    def load_vector(self, kind, params):
        """Load vectors for analytic data. Dirichlet trace: kind 0 point source
        1/(4 pi r), 1 Helmholtz point source, 2 plane wave; params (nrhs, 3).
        Maxwell (tangential trace): kind 3 Hertz dipole; params (nrhs, 6) =
        position, moment."""
        prm = np.ascontiguousarray(np.asarray(params, dtype=np.float64).reshape(-1, 6 if kind == 3 else 3))
        k = prm.shape[0]
        out = np.zeros((self.N, k), dtype=np.complex128 if self.is_complex else np.float64, order="F")
        self.ctx.check(_lib.load().bg_load_vector(self.h, kind, _dp(prm), k, out.ctypes.data_as(ctypes.c_void_p), 0))
        return out

    def potential(self, rho, points):
        """DiscretePotential::evaluate at points (npts, 3) for densities rho
        (N, nrhs): (npts, nrhs); Maxwell: the field, (npts, 3, nrhs)."""
        rho = np.asfortranarray(_columns(np.asarray(rho, dtype=np.complex128 if self.is_complex else np.float64), self.N))
        pts = np.ascontiguousarray(np.asarray(points, dtype=np.float64).reshape(-1, 3))
        k = rho.shape[1]
        if self.lin_op.kind == _lib.MAXWELL_SL:
            out = np.zeros((k, pts.shape[0], 3), dtype=np.complex128)
        else:
            out = np.zeros((pts.shape[0], k), dtype=rho.dtype, order="F")
        self.ctx.check(_lib.load().bg_potential(self.h, rho.ctypes.data_as(ctypes.c_void_p), k, _dp(pts),
                                                pts.shape[0], out.ctypes.data_as(ctypes.c_void_p)))
        return out.transpose(1, 2, 0) if self.lin_op.kind == _lib.MAXWELL_SL else out

    # -- launch plans and the autotuner --
    def set_plan(self, nrhs, precision="mixed", near_kernel=0, split_k_batches=-1, far_order=0, transforms=0,
                 far_ctas=0, mixed_near=0, far_tiles=0):
        """Kernel variants and schedules of products with nrhs right-hand
        sides at precision (bg_launch_plan; all zeros but split_k_batches = -1
        is the built-in plan)."""
        p = _lib.LaunchPlan(near_kernel, split_k_batches, far_order, transforms, far_ctas, mixed_near, far_tiles)
        self.ctx.check(_lib.load().bg_operator_set_plan(self.h, nrhs, _prec_code(precision), ctypes.byref(p)))

    def get_plan(self, nrhs, precision="mixed"):
        p = _lib.LaunchPlan()
        self.ctx.check(_lib.load().bg_operator_get_plan(self.h, nrhs, _prec_code(precision), ctypes.byref(p)))
        return {"near_kernel": p.near_kernel, "split_k_batches": p.split_k_batches, "far_order": p.far_order,
                "transforms": p.transforms, "far_ctas": p.far_ctas, "mixed_near": p.mixed_near,
                "far_tiles": p.far_tiles}

    def autotune(self, nrhs, precision="mixed", reps=5):
        """Time the product's kernel variants for nrhs right-hand sides at
        precision on the GPU and keep the fastest plan (bg_operator_autotune)."""
        r = _lib.TuneReport()
        self.ctx.check(_lib.load().bg_operator_autotune(self.h, nrhs, _prec_code(precision), reps, ctypes.byref(r)))
        return {"candidates": r.candidates, "builtin_ms": r.builtin_ms, "tuned_ms": r.tuned_ms,
                "plan": {"near_kernel": r.plan.near_kernel, "split_k_batches": r.plan.split_k_batches,
                         "far_order": r.plan.far_order, "transforms": r.plan.transforms,
                         "far_ctas": r.plan.far_ctas, "mixed_near": r.plan.mixed_near,
                         "far_tiles": r.plan.far_tiles}}

    # -- inspection --
    def elements(self):
        ints = np.zeros((self.ne, 5), dtype=np.int32)
        dbl = np.zeros((self.ne, 6))
        self.ctx.check(_lib.load().bg_operator_elements(self.h, ints.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                                        _dp(dbl)))
        return ints, dbl

    def leaves(self):
        # the partition is fixed when the operator is created: read it once
        if getattr(self, "_leaves", None) is None:
            out = np.zeros((self.n_dense + self.n_lowrank, 4), dtype=np.int32)
            self.ctx.check(_lib.load().bg_operator_leaves(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
            self._leaves = out
        return self._leaves.copy()

    def transform_csr(self):
        info = self.info()
        nnz = int(info[12])
        ptr = np.zeros(self.S + 1, dtype=np.int32)
        idx = np.zeros(nnz, dtype=np.int32)
        val = np.zeros(nnz)
        ip = ctypes.POINTER(ctypes.c_int)
        self.ctx.check(_lib.load().bg_operator_transform(self.h, ptr.ctypes.data_as(ip), idx.ctypes.data_as(ip),
                                                         _dp(val)))
        return ptr, idx, val

    def leaf_block(self, leaf, rc=0, cc=0):
        if getattr(self, "_leaves", None) is None:
            self.leaves()
        lv = self._leaves[leaf]
        info = self.info()
        p2 = (int(info[10]) + 1) ** 2
        if lv[0] == 2:
            n = int(info[11]) * p2
        else:
            n = int(info[6]) * int(info[7]) ** 2
        dt = np.complex128 if self.is_complex else np.float64
        buf = np.zeros(n * n, dtype=dt)
        self.ctx.check(_lib.load().bg_operator_leaf_block(self.h, leaf, rc, cc, _dp(buf.view(np.float64))))
        return buf.reshape((n, n), order="F")


class Server:
    """Serving loop of the library (bg_server_*): worker threads, each with
    its own stream on the context's GPU, solve queued requests, batching
    requests for the same operator; assembled operators are cached per
    (geometry, kind, M, P, wavenumber) on the worker that assembled them and
    admitted by device memory against one budget for all workers (least
    recently used idle operators evicted).

        srv = Server(ctx, hbm_budget_bytes=200e9, workers=4)
        g = srv.add_geometry(Geometry("sphere.dat", ctx))
        t = srv.submit(g, "laplace", M=4, P=2, data_kind=0, data=x0)  # x0: (nrhs, 3)
        x, info = srv.wait(t)                                          # x: (N, nrhs)
    """

    KINDS = {"laplace": _lib.LAPLACE_SL, "helmholtz": _lib.HELMHOLTZ_SL, "maxwell": _lib.MAXWELL_SL}

    def __init__(self, ctx, hbm_budget_bytes, workers=1):
        self.ctx = ctx
        h = ctypes.c_void_p()
        ctx.check(_lib.load().bg_server_create(ctx.h, int(hbm_budget_bytes), int(workers), ctypes.byref(h)))
        self.h = h
        self._geos = []
        self._pending = {}

    def add_geometry(self, geometry):
        idx = ctypes.c_int()
        self.ctx.check(_lib.load().bg_server_add_geometry(self.h, geometry.h, ctypes.byref(idx)))
        n = ctypes.c_int()
        self.ctx.check(_lib.load().bg_geometry_num_patches(geometry.h, ctypes.byref(n)))
        self._geos.append((geometry, n.value))
        return idx.value

    def submit(self, geometry, kind, M, P, data_kind, data, kappa=0.0, tol=1e-8, inner="fp32"):
        op_kind = self.KINDS[kind] if isinstance(kind, str) else int(kind)
        data = np.ascontiguousarray(np.asarray(data, dtype=np.float64).reshape(-1, 6 if data_kind == 3 else 3))
        nrhs = data.shape[0]
        vd = 2 if op_kind == _lib.MAXWELL_SL else 1
        bound = vd * self._geos[geometry][1] * (2 ** M + P) ** 2  # dimension before gluing >= N
        cplx = op_kind != _lib.LAPLACE_SL
        x = np.zeros(bound * nrhs, dtype=np.complex128 if cplx else np.float64)
        k = complex(kappa)
        req = _lib.Request(geometry, op_kind, M, P, k.real, k.imag, data_kind, nrhs,
                           data.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), tol, _lib.PRECISIONS[inner],
                           x.ctypes.data_as(ctypes.c_void_p), bound * nrhs)
        t = ctypes.c_long()
        self.ctx.check(_lib.load().bg_server_submit(self.h, ctypes.byref(req), ctypes.byref(t)))
        self._pending[t.value] = (x, nrhs)
        return t.value

    def wait(self, ticket, timeout=-1.0):
        """(x of shape (N, nrhs) or None on failure, result dict)."""
        r = _lib.RequestResult()
        self.ctx.check(_lib.load().bg_server_wait(self.h, ticket, float(timeout), ctypes.byref(r)))
        x, nrhs = self._pending.pop(ticket)
        info = {"status": r.status, "N": r.N, "t_submit": r.t_submit, "t_start": r.t_start, "t_done": r.t_done,
                "cache_hit": bool(r.cache_hit), "batch_nrhs": r.batch_nrhs,
                "stats": {k: getattr(r.stats, k) for k, _ in SolveStats._fields_},
                "error": r.error.decode(errors="replace")}
        ok = r.status in (_lib.BG_OK, _lib.BG_NOT_CONVERGED)
        return (x[:r.N * nrhs].reshape((r.N, nrhs), order="F") if ok else None), info

    def stats(self):
        st = _lib.ServerStats()
        self.ctx.check(_lib.load().bg_server_stats_get(self.h, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in _lib.ServerStats._fields_}

    def close(self):
        if getattr(self, "h", None):
            _lib.load().bg_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
