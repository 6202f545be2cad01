"""Full-size checks of the benchmark workloads.

The benchmark workloads, at their full sizes:

- sphere, M = 5, P = 2, n_p = 9, Laplace, 32 point sources;
- torus, M = 4, P = 2, n_p = 10, Helmholtz, kappa = 3, 8 plane waves;
- sphere, M = 4, P = 2, n_p = 9, Maxwell, kappa = 2, 8 Hertz dipoles.

Parity against the oracle on sampled leaves: the oracle assembles every
40th leaf of the same partition (near-field blocks and far-field couplings
alike) and each of those leaves must match the GPU's block to 1e-12
relative, the bound of the small-size leaf tests. Maxwell leaves are compared
in all four component blocks.

Size-independent properties of the whole operator:

- linearity of the FP64 product, to 1e-12 relative;
- the low-precision products against the FP64 product: 1e-5, the tolerance
  of the small-size parity tests. Maxwell uses 1e-3: its FP32 error is up to
  about 1e-5 at M <= 2 (bound 1e-4 there) and grows with 1/(kappa h)^2,
  16 times from M = 2 to M = 4;
- solves with the FP32 inner operator that reach the FP64 residual of 2e-8
  for a tolerance of 1e-8, the residual taken with the FP64 product.

Collected after the other product tests.
"""
import numpy as np
import pytest

from conftest import SPHERE, TORUS

pytestmark = pytest.mark.gpu

LEAF_TOL = 1e-12
LINEAR_TOL = 1e-12
FP32_TOL = 1e-5
MW_FP32_TOL = 1e-3
RES_TOL = 2e-8
LEAF_STRIDE = 40


@pytest.fixture(scope="module")
def ctx():
    import bembel_gb300 as bg
    return bg.Context(0)


def _operator(ctx, geo, M, P, kind, kappa, np_):
    import bembel_gb300 as bg
    lin = {0: bg.LaplaceSingleLayerOperator, 1: bg.HelmholtzSingleLayerOperator, 2: bg.MaxwellSingleLayerOperator}[kind]()
    if kind:
        lin.set_wavenumber(kappa)
    d = bg.DiscreteOperator(bg.AnsatzSpace(bg.Geometry(geo, ctx), M, P), lin, n_p=np_)
    d.compute()
    return d


@pytest.fixture(scope="module")
def laplace_m5(ctx):
    return _operator(ctx, SPHERE, 5, 2, 0, 0.0, 9)


@pytest.fixture(scope="module")
def helmholtz_m4(ctx):
    return _operator(ctx, TORUS, 4, 2, 1, 3.0, 10)


@pytest.fixture(scope="module")
def maxwell_m4(ctx):
    return _operator(ctx, SPHERE, 4, 2, 2, 2.0, 9)


def _rel(a, b):
    return float(np.max(np.linalg.norm(a - b, axis=0) / np.linalg.norm(b, axis=0)))


def _sampled_leaves(d, oracle, geo, M, P, kind, kappa, np_):
    o = oracle.Problem(geo, M, P, kind, kappa=kappa, np_=np_, leaf_stride=LEAF_STRIDE)
    ol, gl = o.leaves(), d.leaves()
    assert len(ol) == len(gl)
    comps = [(0, 0), (0, 1), (1, 0), (1, 1)] if kind == 2 else [(0, 0)]
    worst = {oracle.DENSE: 0.0, oracle.LOWRANK: 0.0}
    count = {oracle.DENSE: 0, oracle.LOWRANK: 0}
    for li in range(0, len(ol), LEAF_STRIDE):
        t = int(ol[li][0])
        count[t] += 1
        for rc, cc in comps:
            a = d.leaf_block(li, rc, cc)
            b = o.leaf_matrix(li, rc, cc)
            nb = np.linalg.norm(b)
            worst[t] = max(worst[t], np.linalg.norm(a - b) / max(nb, 1e-300))
    assert count[oracle.DENSE] > 0 and count[oracle.LOWRANK] > 0, count
    return worst, count


def _check(A, b, x_rand, low_tol):
    y = A.matvec(x_rand)
    h = x_rand.shape[1] // 2
    y1, y2 = A.matvec(x_rand[:, :h]), A.matvec(x_rand[:, h:2 * h])
    comb = A.matvec(2.0 * x_rand[:, :h] - 3.0 * x_rand[:, h:2 * h])
    assert _rel(comb, 2.0 * y1 - 3.0 * y2) < LINEAR_TOL
    for prec in ("mixed", "fp32"):
        assert _rel(A.matvec(x_rand, precision=prec), y) < low_tol, prec
    x, st = A.solve(b, tol=1e-8, inner="fp32")
    assert st["converged"]
    # FP64 residual ||b - A x|| / ||b|| per column
    assert _rel(A.matvec(x), b) < RES_TOL


def test_laplace_sphere_m5_sampled_leaves(laplace_m5, oracle):
    worst, count = _sampled_leaves(laplace_m5, oracle, SPHERE, 5, 2, 0, 0.0, 9)
    assert max(worst.values()) < LEAF_TOL, (worst, count)


def test_helmholtz_torus_m4_sampled_leaves(helmholtz_m4, oracle):
    worst, count = _sampled_leaves(helmholtz_m4, oracle, TORUS, 4, 2, 1, 3.0, 10)
    assert max(worst.values()) < LEAF_TOL, (worst, count)


def test_maxwell_sphere_m4_sampled_leaves(maxwell_m4, oracle):
    worst, count = _sampled_leaves(maxwell_m4, oracle, SPHERE, 4, 2, 2, 2.0, 9)
    assert max(worst.values()) < LEAF_TOL, (worst, count)


def test_laplace_sphere_m5(laplace_m5):
    d = laplace_m5
    rng = np.random.default_rng(3)
    dirs = rng.normal(size=(32, 3))
    src = dirs / np.linalg.norm(dirs, axis=1, keepdims=True) * rng.uniform(1.5, 3.0, (32, 1))
    b = d.load_vector(0, src)
    _check(d.get_discrete_operator(), b, np.random.default_rng(31).uniform(-1, 1, (d.N, 32)), FP32_TOL)


def test_helmholtz_torus_m4(helmholtz_m4):
    d = helmholtz_m4
    rng = np.random.default_rng(5)
    dirs = rng.normal(size=(8, 3))
    b = d.load_vector(2, dirs / np.linalg.norm(dirs, axis=1, keepdims=True))
    xr = rng.uniform(-1, 1, (d.N, 8)) + 1j * rng.uniform(-1, 1, (d.N, 8))
    _check(d.get_discrete_operator(), b, xr, FP32_TOL)


def test_maxwell_sphere_m4(maxwell_m4):
    d = maxwell_m4
    rng = np.random.default_rng(6)
    pos = rng.normal(size=(8, 3))
    pos = 2.5 * pos / np.linalg.norm(pos, axis=1, keepdims=True)
    mom = rng.normal(size=(8, 3))
    b = d.load_vector(3, np.hstack([pos, mom / np.linalg.norm(mom, axis=1, keepdims=True)]))
    xr = rng.uniform(-1, 1, (d.N, 8)) + 1j * rng.uniform(-1, 1, (d.N, 8))
    _check(d.get_discrete_operator(), b, xr, MW_FP32_TOL)
