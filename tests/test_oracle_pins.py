"""Pin the CPU oracle to the reference's own known-answer tests.

Each test restates one of the reference's unit tests (file named in the
docstring) with the same sizes and tolerance.
"""
import math

import numpy as np
import pytest

from conftest import SPHERE, TORUS

SIGMA = 1e-3


def test_transfer_identity(oracle):
    """tests/test_FMMTransferMatrices.cpp: M2D(level l-1) block k == T_k M2D(level l)."""
    np_, M, cl = 9, 3, 1
    T = oracle.transfer_matrices(np_)
    m1 = oracle.moment2d(0, cl, M - cl, np_)
    m2 = oracle.moment2d(0, cl - 1, M - cl + 1, np_)
    c = m1.shape[1]
    err = sum(np.linalg.norm(m2[:, k * c:(k + 1) * c] - T[:, k * 81:(k + 1) * 81] @ m1) for k in range(4))
    assert err < 1e-12


def test_forward_transformation(oracle):
    """tests/test_FMMForwardTransformation.cpp: forward transform == direct moments, 3 levels."""
    np_, M, cl = 9, 6, 2
    n2 = np_ * np_
    T = oracle.transfer_matrices(np_)
    moms = [oracle.moment2d(0, cl - i, M - cl + i, np_) for i in range(3)]
    moms = [np.vstack([m, m]) for m in moms]  # two FMM components, as the test does
    rng = np.random.default_rng(1)
    v = rng.uniform(-1, 1, moms[2].shape[1])
    X = [v.reshape((m.shape[1], -1), order="F") for m in moms]
    ref = [moms[i] @ X[i] for i in range(3)]
    fwd = oracle.forward_transform(moms[0], T, M - 1 - 1, X[0])
    err = sum(np.linalg.norm(ref[i] - fwd[i]) for i in range(3))
    assert err < 1e-12
    assert fwd[0].shape == (2 * n2, X[0].shape[1])


def test_backward_transformation(oracle):
    """tests/test_FMMBackwardTransformation.cpp: backward transform == M^T v."""
    np_, M, cl = 9, 3, 1
    n2 = np_ * np_
    T = oracle.transfer_matrices(np_)
    m1 = np.vstack([oracle.moment2d(0, cl, M - cl, np_)] * 2)
    m2 = np.vstack([oracle.moment2d(0, cl - 1, M - cl + 1, np_)] * 2)
    rng = np.random.default_rng(2)
    v = rng.uniform(-1, 1, 2 * n2)
    ref = m2.T @ v
    out = oracle.backward_transform(m1, T, 1, [np.zeros((2 * n2, 4)), v.reshape(-1, 1)])
    assert np.linalg.norm(ref - out) < 1e-12


def _axis(ints, dbl, i, j, h):
    a = np.zeros((2, 4))
    a[:, 0] = [dbl[i, 0], dbl[i, 0] + h]
    a[:, 1] = [dbl[i, 1], dbl[i, 1] + h]
    a[:, 2] = [dbl[j, 0], dbl[j, 0] + h]
    a[:, 3] = [dbl[j, 1], dbl[j, 1] + h]
    return a


def _exact_analytic(a):
    # integrate0/1 test function of tests/DuffyTrick/test_testFunctions.hpp
    pi = math.pi
    return ((math.cos(pi * a[0, 0]) - math.cos(pi * a[1, 0])) / pi * 0.5 *
            (math.cos(2 * pi * a[0, 2]) - math.cos(2 * pi * a[1, 2])) / pi *
            (math.exp(-a[0, 1]) - math.exp(-a[1, 1])) * (math.exp(a[1, 3]) - math.exp(a[0, 3])))


def _anti(x0, x1):
    return 0.5 * math.log(SIGMA + (x0 - x1) ** 2) + (x1 - x0) / math.sqrt(SIGMA) * math.atan((x0 - x1) / math.sqrt(SIGMA))


def _exact_nearsingular(a):
    # testFunction4DIntegral: exp(-x0 - 2 y1) / (sigma + (x1 - y0)^2)
    b = a[:, 1:3]
    i2 = _anti(b[1, 0], b[1, 1]) - _anti(b[1, 0], b[0, 1]) - _anti(b[0, 0], b[1, 1]) + _anti(b[0, 0], b[0, 1])
    return ((math.exp(-a[0, 0]) - math.exp(-a[1, 0])) * i2 *
            (0.5 * math.exp(-2 * a[0, 3]) - 0.5 * math.exp(-2 * a[1, 3])))


@pytest.mark.parametrize("which,tol", [(0, 1e-12), (1, 1e-12), (2, 1e-6), (3, 1e-4), (4, 1e-4)])
def test_duffy_trick(oracle, screen_path, which, tol):
    """tests/test_DuffyTrick.cpp: integrate0..4 vs closed-form integrals on the screen, M = 2, degree 16."""
    fun = 0 if which < 2 else 1
    p = oracle.Problem(screen_path, 2, 0, oracle.DUMMY, np_=9, assemble=False, dummy_fun=fun)
    ints, dbl = p.elements()
    h = 0.25
    maxerr, count = 0.0, 0
    for i in range(p.ne):
        for j in range(p.ne):
            if which == 2 and i != j:
                continue
            (cs, r1, r2, _), _ = p.pair_class(i, j)
            if which in (3, 4) and cs != which:
                continue
            v = p.dummy_integrate(which, i, j, 16, r1, r2)
            a = _axis(ints, dbl, i, j, h)
            exact = (_exact_analytic(a) if fun == 0 else _exact_nearsingular(a)) / h ** 2
            maxerr = max(maxerr, abs(exact - v) / abs(exact))
            count += 1
    assert count > 0
    assert maxerr < tol


def test_laplace_helmholtz_integrand(oracle, screen_path):
    """tests/test_Laplace.cpp, tests/test_Helmholtz.cpp: kernel at |x-y| = 1."""
    p = oracle.Problem(screen_path, 0, 0, oracle.LAPLACE, np_=9, assemble=False)
    v = p.point_integrand(0, 0., 0., 0., 1.)
    assert abs(v[0, 0] - 1 / (4 * math.pi)) < 1e-6
    q = oracle.Problem(screen_path, 0, 0, oracle.HELMHOLTZ, kappa=1.0, np_=9, assemble=False)
    v = q.point_integrand(0, 0., 0., 0., 1.)
    assert abs(v[0, 0] - np.exp(-1j) / (4 * math.pi)) < 1e-6


def test_surface_point_update(oracle):
    """tests/test_SurfacePointUpdate.cpp and test_GeometryImportAndEval.cpp on the 6-patch sphere."""
    p = oracle.Problem(SPHERE, 0, 0, oracle.LAPLACE, np_=9, assemble=False)
    eq = np.linspace(0, 1, 11)
    eps = 1e-6
    for patch in range(6):
        for s in eq:
            for t in eq:
                sp = p.surface_point(patch, s, t)
                x = sp[3:6]
                n = np.cross(sp[6:9], sp[9:12])
                assert abs(np.linalg.norm(x) - 1) < 1e-9
                assert np.linalg.norm(x - n / np.linalg.norm(n)) < 1e-9
                # tangent vs central difference of the point map
                s0, s1 = max(s - eps, 0), min(s + eps, 1)
                fd = (p.surface_point(patch, s1, t)[3:6] - p.surface_point(patch, s0, t)[3:6]) / (s1 - s0)
                assert np.linalg.norm(fd - sp[6:9]) < 1e-6 * max(1, np.linalg.norm(sp[6:9]))


def test_torus_geometry(oracle):
    """torus.dat: tube radius 0.5 about R = 2 everywhere."""
    p = oracle.Problem(TORUS, 0, 0, oracle.LAPLACE, np_=9, assemble=False)
    for patch in range(16):
        for s in (0.0, 0.3, 0.77, 1.0):
            for t in (0.0, 0.5, 1.0):
                x = p.surface_point(patch, s, t)[3:6]
                rho = math.hypot(x[0], x[1])
                assert abs(math.hypot(rho - 2.0, x[2]) - 0.5) < 1e-9


@pytest.mark.parametrize("kind,kappa", [(1, 0.0), (1, 2.0), (0, 0.0)])
def test_h2_vs_dense(oracle, kind, kappa):
    """tests/test_LazyEigenSum.cpp: ||H2 a - D a|| < 1e-8, sphere, P = 1, M = 2, n_p = 9."""
    p = oracle.Problem(SPHERE, 2, 1, kind, kappa=kappa, np_=9)
    D = p.dense()
    rng = np.random.default_rng(3)
    a = rng.uniform(-1, 1, p.N)
    if p.complex:
        a = a + 1j * rng.uniform(-1, 1, p.N)
    assert np.linalg.norm(p.matvec(a) - D @ a) < 1e-8


def test_h2_vs_dense_maxwell(oracle):
    """Maxwell single layer: the same H2-vs-dense bound on the sphere, P = 1, M = 1."""
    p = oracle.Problem(SPHERE, 1, 1, oracle.MAXWELL, kappa=1.0, np_=9)
    D = p.dense()
    rng = np.random.default_rng(4)
    a = rng.uniform(-1, 1, p.N) + 1j * rng.uniform(-1, 1, p.N)
    assert np.linalg.norm(p.matvec(a) - D @ a) < 1e-8 * max(1.0, np.linalg.norm(D @ a))


EQ_POINTS = [0.1 * i for i in range(11)]  # tests/Test.hpp:35


def test_bernstein_matches_de_boor(oracle):
    """tests/test_Bernstein.cpp: sum_i c_i B_{i,p}(x) with c_i = (i + 1) / 21
    equals de Boor's evaluation of the spline with the same coefficients on
    the Bezier knot vector, p = 0..20 (derivatives p = 1..20), at the 11
    equispaced points, to 1e-6 (coefficient_accuracy, tests/Test.hpp:39).
    scipy's BSpline is the independent de Boor evaluation."""
    BSpline = pytest.importorskip("scipy.interpolate").BSpline
    maxp = 20
    coefs = [(i + 1) / (maxp + 1) for i in range(maxp + 1)]
    for p in range(maxp + 1):
        spl = BSpline(np.r_[np.zeros(p + 1), np.ones(p + 1)], np.array(coefs[:p + 1]), p)
        der = spl.derivative() if p >= 1 else None
        for x in EQ_POINTS:
            assert abs(oracle.bernstein(p, coefs, x) - float(spl(x))) < 1e-6
            if der is not None:
                assert abs(oracle.bernstein(p, coefs, x, der=True) - float(der(x))) < 1e-6


@pytest.mark.parametrize("p", [1, 2, 3, 4])
@pytest.mark.parametrize("m", [0, 1, 2])
def test_projector_counts_and_partition_of_unity(oracle, screen_path, p, m):
    """tests/test_Projector.cpp on the unit-square screen with knot
    repetition 1: the superspace has (p+1)^2 4^m functions per component; the
    spline space (p + 2^m)^2 (scalar, discontinuous form) or
    2 (p + 2^m)(p - 1 + 2^m) (div-conforming); T maps the all-ones
    coefficients to all ones (partition of unity, 1e-6 there). On a single
    patch the scalar T is this projector; the div-conforming T glues it and,
    on the open screen, drops the functions whose normal component does not
    vanish on the boundary."""
    n = 1 << m
    for kind, kappa, rows, cols in ((oracle.LAPLACE, 0.0, (p + 1) ** 2 * n * n, (p + n) ** 2),
                                    (oracle.MAXWELL, 1.0, 2 * (p + 1) ** 2 * n * n, 2 * (p + n) * (p - 1 + n))):
        pr = oracle.Problem(screen_path, m, p, kind, kappa=kappa, np_=4, assemble=False)
        Pm = pr.projector_dense()
        assert Pm.shape == (rows, cols)
        assert np.max(np.abs(Pm @ np.ones(cols) - 1.0)) < 1e-12
        if kind == oracle.LAPLACE:
            assert np.array_equal(pr.transform_dense(), Pm)
        else:
            # each component loses the 2 (p - 1 + n) functions whose normal
            # component is nonzero on one of its two boundary edges
            assert pr.transform_dense().shape == (rows, cols - 4 * (p - 1 + n))


def test_partition_counts(oracle):
    """Block partition of the sphere, M = 3 (eta = 1.6, min cluster level 1)."""
    p = oracle.Problem(SPHERE, 3, 1, oracle.LAPLACE, np_=6, assemble=False)
    assert (p.n_dense, p.n_lowrank) == (1128, 3768)
    assert p.N == 6 * 9 * 9


def test_laplace_convergence(oracle):
    """examples/LaplaceSingleLayerH2.cpp: potential error of a harmonic Dirichlet problem
    decays at rate >= 0.9 (2P+3); here P = 0, levels 1..3, point-source data."""
    x0 = np.array([0.0, 0.2, 1.8])
    pts = np.array([[0.1, -0.05, 0.2], [0.0, 0.1, -0.2], [-0.15, 0.1, 0.05]])
    ref = 1 / (4 * math.pi * np.linalg.norm(pts - x0, axis=1))
    errs = []
    for M in (1, 2, 3):
        p = oracle.Problem(SPHERE, M, 0, oracle.LAPLACE, np_=9)
        b = p.load_vector(0, x0)
        rho, it = p.gmres(b, tol=1e-12, restart=200, maxit=2000)
        errs.append(np.max(np.abs(p.potential(rho, pts) - ref)))
    rate = math.log2(errs[-2] / errs[-1])
    assert rate >= 0.9 * 3


def _dipole_field(pt, k, pos, mom):
    """examples/Data.hpp:73-90 (Hertz dipole), numpy restatement for the check."""
    c = pt - pos
    r = np.linalg.norm(c, axis=1, keepdims=True)
    n = c / r
    ex = np.exp(-1j * k * r)
    ncl = np.cross(np.cross(n, mom), n)
    hh = n * (3 * (n @ mom))[:, None] - mom
    return k * k * ex / r * ncl + (1 / r ** 3 + 1j * k / r ** 2) * ex * hh


def _sphere_points(radius, m):
    i = np.arange(m) + 0.5
    phi = np.arccos(1 - 2 * i / m)
    th = np.pi * (1 + 5 ** 0.5) * i
    return radius * np.stack([np.cos(th) * np.sin(phi), np.sin(th) * np.sin(phi), np.cos(phi)], 1)


def test_maxwell_field_converges(oracle):
    """examples/MaxwellSingleLayerH2.cpp:30-96: a dipole at (0.2, 0.2, 0.2) with
    moment (0, 0.1, 0.1) inside the sphere, kappa = 2, excitation its tangential
    trace; the single-layer field at 100 points of radius 2 must match the
    dipole field with rate >= 0.9 (2P + 1) over the refinement levels."""
    k, pos, mom = 2.0, np.array([0.2, 0.2, 0.2]), np.array([0.0, 0.1, 0.1])
    grid = _sphere_points(2.0, 100)
    ref = _dipole_field(grid, k, pos, mom)
    errs = []
    for M in (0, 1, 2):
        p = oracle.Problem(SPHERE, M, 1, oracle.MAXWELL, kappa=k, np_=9)
        x, _ = p.gmres(p.load_vector(3, np.r_[pos, mom]), tol=1e-10, restart=500, maxit=5000)
        errs.append(np.max(np.linalg.norm(p.potential(x, grid) - ref, axis=1)))
    rates = np.log2(np.array(errs[:-1]) / np.array(errs[1:]))
    assert np.all(rates >= 0.9 * 3), (errs, rates)


def test_helmholtz_convergence(oracle):
    """examples/HelmholtzSingleLayerH2.cpp:30-98: kappa = 2, the fundamental
    solution with its source at the origin (inside the sphere) as Dirichlet
    data; the potential at 100 points of radius 2 converges at rate
    >= 0.9 (2P + 3), here P = 0 over refinement levels 1..3."""
    k = 2.0
    grid = _sphere_points(2.0, 100)
    r = np.linalg.norm(grid, axis=1)
    ref = np.exp(-1j * k * r) / (4 * math.pi * r)
    errs = []
    for M in (1, 2, 3):
        p = oracle.Problem(SPHERE, M, 0, oracle.HELMHOLTZ, kappa=k, np_=9)
        rho, _ = p.gmres(p.load_vector(1, np.zeros(3)), tol=1e-12, restart=200, maxit=2000)
        errs.append(np.max(np.abs(p.potential(rho, grid) - ref)))
    rates = np.log2(np.array(errs[:-1]) / np.array(errs[1:]))
    assert rates[-1] >= 0.9 * 3, (errs, rates)
