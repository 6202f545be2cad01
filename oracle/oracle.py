"""ctypes front end of the CPU oracle (test infrastructure only).

The oracle is a CPU restatement of Bembel's H2 single-layer path (geometry,
element tree, block partition, DuffyTrick quadrature, FMM moments/transfers,
H2 assembly and matvec, dense Galerkin matrix, load vectors, potential,
GMRES). It is used by tests/, the smoke check and bench.py's CPU-baseline leg
only; the bembel_gb300 package never imports it.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

LAPLACE, HELMHOLTZ, MAXWELL, DUMMY = 0, 1, 2, 3
# the analytic cube sphere (six x/|x| images of the cube faces) as a geometry name
CUBE_SPHERE = "analytic:cube_sphere"
DENSE, LOWRANK = 2, 1


def build():
    """Compile the oracle with its Makefile (portable flags, x86_64 and aarch64)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        P, I, D, L_ = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_long
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        lp = ctypes.POINTER(ctypes.c_long)
        L.orc_create.restype = P
        L.orc_create.argtypes = [ctypes.c_char_p, I, I, I, D, D, I, D, I, I, I]
        L.orc_destroy.argtypes = [P]
        L.orc_info.argtypes = [P, lp]
        L.orc_assemble_seconds.restype = D
        L.orc_assemble_seconds.argtypes = [P]
        L.orc_transform_csr.argtypes = [P, ip, ip, dp]
        L.orc_elements.argtypes = [P, ip, dp]
        L.orc_leaves.argtypes = [P, ip]
        L.orc_leaf_matrix.argtypes = [P, L_, I, I, dp]
        L.orc_element_pair.argtypes = [P, I, I, dp]
        L.orc_pair_class.argtypes = [P, I, I, ip, dp]
        L.orc_dummy_integrate.restype = D
        L.orc_dummy_integrate.argtypes = [P, I, I, I, I, I, I]
        L.orc_point_integrand.argtypes = [P, I, D, D, D, D, dp]
        L.orc_surface_point.argtypes = [P, I, D, D, dp]
        L.orc_transfer_matrices.argtypes = [I, dp]
        L.orc_moment2d.argtypes = [I, I, I, I, I, I, dp]
        L.orc_moments.argtypes = [P, I, dp]
        L.orc_forward_transform.argtypes = [dp, I, I, dp, I, I, dp, I, dp]
        L.orc_backward_transform.argtypes = [dp, I, I, dp, I, I, dp, I, dp]
        L.orc_matvec.restype = I
        L.orc_matvec.argtypes = [P, dp, dp, I]
        L.orc_matvec_ss.restype = I
        L.orc_matvec_ss.argtypes = [P, dp, dp]
        L.orc_dense_ss.argtypes = [P, dp]
        L.orc_load_vector.argtypes = [P, I, dp, dp]
        L.orc_potential.argtypes = [P, dp, dp, I, dp]
        L.orc_gmres.restype = I
        L.orc_gmres.argtypes = [P, dp, dp, D, I, I]
        L.orc_set_leaf.restype = I
        L.orc_set_leaf.argtypes = [P, L_, I, I, dp]
        L.orc_cg.restype = I
        L.orc_cg.argtypes = [P, dp, dp, D, I, dp]
        L.orc_create_sampled.restype = P
        L.orc_create_sampled.argtypes = [ctypes.c_char_p, I, I, I, D, D, I, D, I, I]
        L.orc_last_product_split.argtypes = [P, dp]
        L.orc_threads.restype = I
        L.orc_projector_csr.argtypes = [P, lp, ip, ip, dp]
        L.orc_bernstein.restype = D
        L.orc_bernstein.argtypes = [I, dp, D, I]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def bernstein(p, coefs, x, der=False):
    """sum_i coefs[i] B_{i,p}(x) (or its derivative) in the Bernstein basis."""
    c = np.ascontiguousarray(np.asarray(coefs, dtype=np.float64)[:p + 1])
    return lib().orc_bernstein(p, _dp(c), float(x), int(der))


def transfer_matrices(np_):
    out = np.zeros((4 * np_ * np_, np_ * np_))  # column-major storage of np2 x 4np2
    lib().orc_transfer_matrices(np_, _dp(out))
    return out.T.copy()


def moment2d(P, cluster_level, cluster_ref, np_, d1=False, d2=False):
    rows = np_ * np_
    cols = (P + 1) ** 2 * 4 ** cluster_ref
    out = np.zeros((cols, rows))
    lib().orc_moment2d(P, cluster_level, cluster_ref, np_, int(d1), int(d2), _dp(out))
    return out.T.copy()


def forward_transform(mom, T, steps, X):
    np_ = int(round(np.sqrt(T.shape[0])))
    mr, mc = mom.shape
    xc = X.shape[1]
    sizes = [mr * (xc // 4 ** i) for i in range(steps + 1)]
    out = np.zeros(sum(sizes))
    lib().orc_forward_transform(_dp(np.asfortranarray(mom)), mr, mc, _dp(np.asfortranarray(T)), np_, steps,
                                _dp(np.asfortranarray(X)), xc, _dp(out))
    res, o = [], 0
    for i in range(steps + 1):
        c = xc // 4 ** i
        res.append(out[o:o + mr * c].reshape((mr, c), order="F"))
        o += mr * c
    return res


def backward_transform(mom, T, steps, Z):
    np_ = int(round(np.sqrt(T.shape[0])))
    mr, mc = mom.shape
    xc = Z[0].shape[1]
    flat = np.concatenate([np.asfortranarray(z).ravel(order="F") for z in Z])
    out = np.zeros(mc * xc)
    lib().orc_backward_transform(_dp(np.asfortranarray(mom)), mr, mc, _dp(np.asfortranarray(T)), np_, steps,
                                 _dp(flat), xc, _dp(out))
    return out


class Problem:
    """Oracle discretisation: geometry file, refinement M, degree P, operator."""

    def __init__(self, geo, M, P, kind=LAPLACE, kappa=0.0, np_=9, eta=1.6, mcl=1, assemble=True,
                 dummy_fun=0, leaf_stride=1):
        kappa = complex(kappa)
        if leaf_stride > 1:
            self.h = lib().orc_create_sampled(geo.encode(), M, P, kind, kappa.real, kappa.imag, np_, eta, mcl,
                                              leaf_stride)
        else:
            self.h = lib().orc_create(geo.encode(), M, P, kind, kappa.real, kappa.imag, np_, eta, mcl,
                                      int(assemble), dummy_fun)
        if not self.h:
            raise RuntimeError("oracle problem creation failed")
        info = np.zeros(12, dtype=np.int64)
        lib().orc_info(self.h, info.ctypes.data_as(ctypes.POINTER(ctypes.c_long)))
        (self.ne, self.S, self.N, self.n_leaves, self.n_dense, self.n_lowrank, self.vd, self.nc, self.np,
         self.nnz, self.M, self.P) = [int(v) for v in info]
        self.kind = kind
        self.kappa = kappa
        self.complex = kind in (HELMHOLTZ, MAXWELL)
        self.dtype = np.complex128 if self.complex else np.float64

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    @property
    def assemble_seconds(self):
        return lib().orc_assemble_seconds(self.h)

    def transform_csr(self):
        ptr = np.zeros(self.S + 1, dtype=np.int32)
        idx = np.zeros(self.nnz, dtype=np.int32)
        val = np.zeros(self.nnz)
        lib().orc_transform_csr(self.h, _ip(ptr), _ip(idx), _dp(val))
        return ptr, idx, val

    def projector_dense(self):
        """The Projector matrix before gluing (Projector.hpp:52-90)."""
        dims = np.zeros(3, dtype=np.int64)
        lp = ctypes.POINTER(ctypes.c_long)
        lib().orc_projector_csr(self.h, dims.ctypes.data_as(lp), None, None, None)
        rows, cols, nnz = (int(v) for v in dims)
        ptr = np.zeros(rows + 1, dtype=np.int32)
        idx = np.zeros(nnz, dtype=np.int32)
        val = np.zeros(nnz)
        lib().orc_projector_csr(self.h, dims.ctypes.data_as(lp), _ip(ptr), _ip(idx), _dp(val))
        T = np.zeros((rows, cols))
        for r in range(rows):
            T[r, idx[ptr[r]:ptr[r + 1]]] += val[ptr[r]:ptr[r + 1]]
        return T

    def transform_dense(self):
        ptr, idx, val = self.transform_csr()
        T = np.zeros((self.S, self.N))
        for r in range(self.S):
            for k in range(ptr[r], ptr[r + 1]):
                T[r, idx[k]] += val[k]
        return T

    def elements(self):
        ints = np.zeros((self.ne, 7), dtype=np.int32)
        dbl = np.zeros((self.ne, 6))
        lib().orc_elements(self.h, _ip(ints), _dp(dbl))
        return ints, dbl

    def leaves(self):
        out = np.zeros((self.n_leaves, 7), dtype=np.int32)
        lib().orc_leaves(self.h, _ip(out))
        return out

    def leaf_matrix(self, leaf, rc=0, cc=0):
        lv = self.leaves()[leaf]
        if lv[0] == DENSE:
            n = lv[6] * (self.P + 1) ** 2
        else:
            n = self.nc * self.np * self.np
        out = np.zeros((n, n), dtype=self.dtype)
        buf = out.T.copy()  # column-major
        if lib().orc_leaf_matrix(self.h, leaf, rc, cc, _dp(buf.view(np.float64))) != 0:
            raise RuntimeError("H2 matrix not assembled")
        return buf.T.copy()

    def set_leaf_matrix(self, leaf, F, rc=0, cc=0):
        """Store leaf matrix F (a problem made with assemble=False)."""
        buf = np.asfortranarray(F, dtype=self.dtype)
        if lib().orc_set_leaf(self.h, leaf, rc, cc, _dp(buf.reshape(-1, order="F").view(np.float64))) != 0:
            raise RuntimeError("leaf index out of range")

    def element_pair(self, id1, id2):
        n = self.vd * (self.P + 1) ** 2
        buf = np.zeros((n, n), dtype=self.dtype)
        lib().orc_element_pair(self.h, id1, id2, _dp(buf.view(np.float64)))
        return buf.T.copy()

    def pair_class(self, id1, id2):
        out = np.zeros(4, dtype=np.int32)
        d = np.zeros(1)
        lib().orc_pair_class(self.h, id1, id2, _ip(out), _dp(d))
        return tuple(int(v) for v in out), float(d[0])

    def dummy_integrate(self, which, id1, id2, qdeg, rot1=0, rot2=0):
        return lib().orc_dummy_integrate(self.h, which, id1, id2, qdeg, rot1, rot2)

    def point_integrand(self, id_, s1, t1, s2, t2):
        n = self.vd * (self.P + 1) ** 2
        buf = np.zeros((n, n), dtype=self.dtype)
        lib().orc_point_integrand(self.h, id_, s1, t1, s2, t2, _dp(buf.view(np.float64)))
        return buf.T.copy()

    def surface_point(self, patch, s, t):
        out = np.zeros(12)
        lib().orc_surface_point(self.h, patch, s, t, _dp(out))
        return out

    def moments(self, comp=0):
        rows = self.nc * self.np * self.np
        cols = 4 * (self.P + 1) ** 2
        out = np.zeros((cols, rows))
        lib().orc_moments(self.h, comp, _dp(out))
        return out.T.copy()

    def matvec(self, x):
        x = np.asarray(x, dtype=self.dtype)
        squeeze = x.ndim == 1
        X = np.asfortranarray(x.reshape(self.N, -1))
        nrhs = X.shape[1]
        xf = X.reshape(-1, order="F")
        yf = np.zeros_like(xf)
        if lib().orc_matvec(self.h, _dp(xf.view(np.float64)), _dp(yf.view(np.float64)), nrhs) != 0:
            raise RuntimeError("H2 matrix not assembled")
        Y = yf.reshape((self.N, nrhs), order="F")
        return Y[:, 0] if squeeze else Y

    def last_product_split(self):
        """(leaf-loop seconds, other seconds, sampled entries, total entries) of the last matvec."""
        out = np.zeros(4)
        lib().orc_last_product_split(self.h, _dp(out))
        return out

    def matvec_ss(self, x):
        x = np.ascontiguousarray(x, dtype=self.dtype)
        y = np.zeros_like(x)
        if lib().orc_matvec_ss(self.h, _dp(x.view(np.float64)), _dp(y.view(np.float64))) != 0:
            raise RuntimeError("H2 matrix not assembled")
        return y

    def dense_ss(self):
        flat = np.zeros(self.S * self.S, dtype=self.dtype)
        lib().orc_dense_ss(self.h, _dp(flat.view(np.float64)))
        return flat.reshape((self.S, self.S), order="F")

    def dense(self):
        D = self.dense_ss()
        T = self.transform_dense()
        return T.T @ D @ T

    def load_vector(self, kind, prm):
        p = np.zeros(8)
        p[:len(prm)] = prm
        out = np.zeros(self.N, dtype=self.dtype)
        lib().orc_load_vector(self.h, kind, _dp(p), _dp(out.view(np.float64)))
        return out

    def potential(self, rho, pts):
        """Single-layer potential at pts (npts, 3); Maxwell: the field, (npts, 3)."""
        rho = np.ascontiguousarray(rho, dtype=self.dtype)
        pts = np.ascontiguousarray(pts, dtype=np.float64)
        out = np.zeros(pts.shape[0] * (3 if self.kind == MAXWELL else 1), dtype=self.dtype)
        lib().orc_potential(self.h, _dp(rho.view(np.float64)), _dp(pts), pts.shape[0], _dp(out.view(np.float64)))
        return out.reshape(-1, 3) if self.kind == MAXWELL else out

    def gmres(self, b, tol=1e-10, restart=100, maxit=1000):
        b = np.ascontiguousarray(b, dtype=self.dtype)
        x = np.zeros_like(b)
        it = lib().orc_gmres(self.h, _dp(b.view(np.float64)), _dp(x.view(np.float64)), tol, restart, maxit)
        return x, it

    def cg(self, b, tol=1e-8, maxit=None):
        """Unpreconditioned CG from x = 0 (the reference's Laplace solver); (x, iterations, relres)."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros_like(b)
        rr = np.zeros(1)
        it = lib().orc_cg(self.h, _dp(b), _dp(x), tol, maxit if maxit else 2 * self.N, _dp(rr))
        if it < 0:
            raise RuntimeError("CG needs a real symmetric operator")
        return x, it, float(rr[0])


def threads():
    return lib().orc_threads()
