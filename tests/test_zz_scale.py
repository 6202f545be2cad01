"""Full-size checks through size-independent properties (no oracle at these sizes).

The benchmark workloads, at their full sizes:

- sphere, M = 5, P = 2, n_p = 9, Laplace, 32 point sources;
- torus, M = 4, P = 2, n_p = 10, Helmholtz, kappa = 3, 8 plane waves;
- sphere, M = 4, P = 2, n_p = 9, Maxwell, kappa = 2, 8 Hertz dipoles.

Each is checked for:

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

LINEAR_TOL = 1e-12
FP32_TOL = 1e-5
MW_FP32_TOL = 1e-3
RES_TOL = 2e-8


@pytest.fixture(scope="module")
def ctx():
    import bembel_gb300 as bg
    return bg.Context(0)


def _rel(a, b):
    return float(np.max(np.linalg.norm(a - b, axis=0) / np.linalg.norm(b, axis=0)))


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
    assert _rel(b - A.matvec(x), b) < RES_TOL


def test_laplace_sphere_m5(ctx):
    import bembel_gb300 as bg
    d = bg.DiscreteOperator(bg.AnsatzSpace(bg.Geometry(SPHERE, ctx), 5, 2), bg.LaplaceSingleLayerOperator(), n_p=9)
    d.compute()
    rng = np.random.default_rng(3)
    dirs = rng.normal(size=(32, 3))
    src = dirs / np.linalg.norm(dirs, axis=1, keepdims=True) * rng.uniform(1.5, 3.0, (32, 1))
    b = d.load_vector(0, src)
    _check(d.get_discrete_operator(), b, np.random.default_rng(31).uniform(-1, 1, (d.N, 32)), FP32_TOL)


def test_helmholtz_torus_m4(ctx):
    import bembel_gb300 as bg
    lin = bg.HelmholtzSingleLayerOperator()
    lin.set_wavenumber(3.0)
    d = bg.DiscreteOperator(bg.AnsatzSpace(bg.Geometry(TORUS, ctx), 4, 2), lin, n_p=10)
    d.compute()
    rng = np.random.default_rng(5)
    dirs = rng.normal(size=(8, 3))
    b = d.load_vector(2, dirs / np.linalg.norm(dirs, axis=1, keepdims=True))
    xr = rng.uniform(-1, 1, (d.N, 8)) + 1j * rng.uniform(-1, 1, (d.N, 8))
    _check(d.get_discrete_operator(), b, xr, FP32_TOL)


def test_maxwell_sphere_m4(ctx):
    import bembel_gb300 as bg
    lin = bg.MaxwellSingleLayerOperator()
    lin.set_wavenumber(2.0)
    d = bg.DiscreteOperator(bg.AnsatzSpace(bg.Geometry(SPHERE, ctx), 4, 2), lin, n_p=9)
    d.compute()
    rng = np.random.default_rng(6)
    pos = rng.normal(size=(8, 3))
    pos = 2.5 * pos / np.linalg.norm(pos, axis=1, keepdims=True)
    mom = rng.normal(size=(8, 3))
    b = d.load_vector(3, np.hstack([pos, mom / np.linalg.norm(mom, axis=1, keepdims=True)]))
    xr = rng.uniform(-1, 1, (d.N, 8)) + 1j * rng.uniform(-1, 1, (d.N, 8))
    _check(d.get_discrete_operator(), b, xr, MW_FP32_TOL)
