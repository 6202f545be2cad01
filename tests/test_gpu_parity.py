"""GPU parity against the CPU oracle, through the C ABI.

FP64 path: assembled leaf blocks and the H2 matvec agree with the oracle to
1e-12 relative (Frobenius / 2-norm). FP32 fused far field (with the near
field in FP64 or FP32): 1e-5 relative.
"""
import numpy as np
import pytest

from conftest import SPHERE, TORUS

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
FP32_TOL = 1e-5  # mixed: FP64 near field, FP32 far field


@pytest.fixture(scope="module")
def ctx():
    import bembel_gb300 as bg
    return bg.Context(0)


def _pair(ctx, oracle, geo, M, P, kind, kappa=0.0, np_=6):
    import bembel_gb300 as bg
    ops = {0: bg.LaplaceSingleLayerOperator, 1: bg.HelmholtzSingleLayerOperator, 2: bg.MaxwellSingleLayerOperator}
    lin = ops[kind]()
    if kind in (1, 2):
        lin.set_wavenumber(kappa)
    d = bg.DiscreteOperator(bg.AnsatzSpace(bg.Geometry(geo, ctx), M, P), lin, n_p=np_)
    d.compute()
    o = oracle.Problem(geo, M, P, kind, kappa=kappa, np_=np_)
    return d, o


CASES = [(SPHERE, 2, 1, 0, 0.0, 6), (SPHERE, 2, 2, 0, 0.0, 6), (TORUS, 1, 2, 0, 0.0, 6), (SPHERE, 2, 1, 1, 2.0, 6),
         (SPHERE, 3, 0, 0, 0.0, 9)]


@pytest.mark.parametrize("geo,M,P,kind,kappa,np_", CASES)
def test_leaf_blocks(ctx, oracle, geo, M, P, kind, kappa, np_):
    d, o = _pair(ctx, oracle, geo, M, P, kind, kappa, np_)
    leaves = o.leaves()
    worst = 0.0
    for li in range(len(leaves)):
        a = d.leaf_block(li)
        b = o.leaf_matrix(li)
        worst = max(worst, np.linalg.norm(a - b) / np.linalg.norm(b))
    assert worst < FP64_TOL, worst


@pytest.mark.parametrize("geo,M,P,kind,kappa,np_", CASES)
def test_matvec_fp64_and_mixed(ctx, oracle, geo, M, P, kind, kappa, np_):
    d, o = _pair(ctx, oracle, geo, M, P, kind, kappa, np_)
    rng = np.random.default_rng(7)
    for nrhs in (1, 5):
        x = rng.uniform(-1, 1, (d.N, nrhs))
        if d.is_complex:
            x = x + 1j * rng.uniform(-1, 1, (d.N, nrhs))
        ref = o.matvec(x)
        A = d.get_discrete_operator()
        y64 = A.matvec(x)
        y32 = A.matvec(x, precision="mixed")
        yf = A.matvec(x, precision="fp32")
        assert np.linalg.norm(y64 - ref) / np.linalg.norm(ref) < FP64_TOL
        assert np.linalg.norm(y32 - ref) / np.linalg.norm(ref) < FP32_TOL
        assert np.linalg.norm(yf - ref) / np.linalg.norm(ref) < FP32_TOL


@pytest.mark.parametrize("geo,P", [(SPHERE, 2), (TORUS, 1), (SPHERE, 0)])
def test_mixed_near_field_digits_fp64_accurate(ctx, oracle, geo, P):
    """The tensor-core near field of the mixed product (8 integer digits of 7
    bits per operand, exact integer sums; leaf blocks of 36, 16 and 4 rows)
    against the FP64 product on operators without far field (M = 1), where
    the product is the near field alone: FP64 accuracy, within 5e-14 per
    column of the FP64 product (whose own rounding is of that order, about
    1e-14 measured), for 1, 32 and 45 columns (two passes of 32), with a zero column and
    columns 1e-150 and 1e+150 times the others. The double-float near field
    (launch plan mixed_near = 1, about 1e-13) is held to 1e-12 on the columns
    FP32 pairs can represent."""
    d, o = _pair(ctx, oracle, geo, 1, P, 0)
    assert d.n_lowrank == 0
    A = d.get_discrete_operator()
    rng = np.random.default_rng(23)
    for nrhs in (1, 32, 45):
        x = rng.uniform(-1, 1, (d.N, nrhs))
        if nrhs > 4:
            x[:, 1] = 0.0
            x[:, 2] *= 1e-150
            x[:, 3] *= 1e150
        ref = o.matvec(x)
        y64 = A.matvec(x)
        ymx = A.matvec(x, precision="mixed")
        d.set_plan(nrhs, "mixed", mixed_near=1)
        ydf = A.matvec(x, precision="mixed")
        d.set_plan(nrhs, "mixed")
        for c in range(nrhs):
            n = np.linalg.norm(y64[:, c])
            if n == 0.0:
                assert not ymx[:, c].any() and not ydf[:, c].any()
                continue
            assert np.linalg.norm(ymx[:, c] - y64[:, c]) / n < 5e-14, (nrhs, c)
            if nrhs <= 4 or c > 3:  # FP32 pairs cannot hold 1e+-150
                assert np.linalg.norm(ydf[:, c] - y64[:, c]) / n < 1e-12, (nrhs, c)
        assert np.linalg.norm(y64 - ref) / np.linalg.norm(ref) < FP64_TOL


@pytest.mark.parametrize("mixed_near", [0, 1, 2])
def test_mixed_matvec_32_columns(ctx, oracle, mixed_near):
    """32 columns with far field, every near-field variant of the mixed
    product (tensor-core digits, double-float, double-float with a quarter of
    the columns on the FP64 pipe): every column meets the FP32 bound, and the
    variants differ only by the near field's rounding (the far field is the
    same), far below it."""
    d, o = _pair(ctx, oracle, SPHERE, 2, 2, 0, 0.0, 9)
    x = np.random.default_rng(17).uniform(-1, 1, (d.N, 32))
    ref = o.matvec(x)
    A = d.get_discrete_operator()
    y0 = A.matvec(x, precision="mixed")
    d.set_plan(32, "mixed", mixed_near=mixed_near)
    y = A.matvec(x, precision="mixed")
    d.set_plan(32, "mixed")
    err = np.max(np.linalg.norm(y - ref, axis=0) / np.linalg.norm(ref, axis=0))
    assert err < FP32_TOL, err
    assert np.max(np.linalg.norm(y - y0, axis=0) / np.linalg.norm(ref, axis=0)) < 1e-12


def test_matvec_alpha_beta(ctx, oracle):
    d, o = _pair(ctx, oracle, SPHERE, 2, 1, 0)
    rng = np.random.default_rng(8)
    x = rng.uniform(-1, 1, (d.N, 3))
    y0 = rng.uniform(-1, 1, (d.N, 3))
    ref = 0.5 * y0 - 2.0 * o.matvec(x)
    y = d.get_discrete_operator().matvec(x, out=y0.copy(), alpha=-2.0, beta=0.5)
    assert np.linalg.norm(y - ref) / np.linalg.norm(ref) < FP64_TOL


@pytest.mark.parametrize("kind,kappa,data", [(0, 0.0, 0), (1, 2.0, 1), (1, 2.0, 2)])
def test_load_vector(ctx, oracle, kind, kappa, data):
    d, o = _pair(ctx, oracle, SPHERE, 2, 1, kind, kappa)
    prm = np.array([[0.0, 0.2, 1.8], [0.3, -1.2, 2.0]])
    if data == 2:
        prm = prm / np.linalg.norm(prm, axis=1, keepdims=True)
    got = d.load_vector(data, prm)
    for c in range(prm.shape[0]):
        ref = o.load_vector(data, prm[c])
        assert np.linalg.norm(got[:, c] - ref) / np.linalg.norm(ref) < FP64_TOL


def test_potential(ctx, oracle):
    d, o = _pair(ctx, oracle, SPHERE, 2, 1, 0)
    rng = np.random.default_rng(9)
    rho = rng.uniform(-1, 1, (d.N, 2))
    pts = rng.uniform(-0.25, 0.25, (7, 3))
    got = d.potential(rho, pts)
    for c in range(2):
        ref = o.potential(rho[:, c], pts)
        assert np.linalg.norm(got[:, c] - ref) / np.linalg.norm(ref) < FP64_TOL


@pytest.mark.parametrize("inner", ["fp64", "mixed", "fp32"])
def test_solve_reaches_tolerance(ctx, oracle, inner):
    d, o = _pair(ctx, oracle, SPHERE, 3, 1, 0, 0.0, 6)
    x0 = np.array([[0.0, 0.2, 1.8], [1.0, 1.5, -1.2], [-2.0, 0.3, 0.1]])
    b = d.load_vector(0, x0)
    x, st = d.get_discrete_operator().solve(b, tol=1e-8, inner=inner)
    assert st["converged"]
    for c in range(3):
        r = b[:, c] - o.matvec(x[:, c])
        assert np.linalg.norm(r) / np.linalg.norm(b[:, c]) < 2e-8


@pytest.mark.parametrize("inner", ["fp64", "fp32"])
def test_solve_many_columns(ctx, oracle, inner):
    """300 right-hand sides in one batched solve (more columns than the
    threads of one reduction block): every column reaches the FP64 residual
    1e-8, and the first 8 columns agree with an 8-column solve of the same
    data within what two solutions at that residual may differ by (the
    condition number here is about 8e3)."""
    d, o = _pair(ctx, oracle, SPHERE, 2, 1, 0, 0.0, 6)
    rng = np.random.default_rng(12)
    dirs = rng.normal(size=(300, 3))
    x0 = dirs / np.linalg.norm(dirs, axis=1, keepdims=True) * rng.uniform(1.5, 3.0, (300, 1))
    b = d.load_vector(0, x0)
    A = d.get_discrete_operator()
    x, st = A.solve(b, tol=1e-8, inner=inner)
    assert st["converged"]
    r = b - o.matvec(x)
    res = np.linalg.norm(r, axis=0) / np.linalg.norm(b, axis=0)
    assert res.max() < 2e-8, res.max()
    x8, _ = A.solve(b[:, :8], tol=1e-8, inner=inner)
    assert np.max(np.linalg.norm(x[:, :8] - x8, axis=0) / np.linalg.norm(x8, axis=0)) < 1e-3


# Maxwell single layer (div-conforming vector basis, kappa = 2 as in the EFIE
# workload): all four component blocks of every leaf, the product, the dipole
# excitation and a solve.
MW_CASES = [(SPHERE, 2, 1, 2.0, 6), (SPHERE, 2, 2, 2.0, 6), (TORUS, 1, 2, 1.5, 6)]
MW_FP32_TOL = 1e-4  # the divergence part carries 1/(kappa h)^2: FP32 far field and transforms


@pytest.mark.parametrize("geo,M,P,kappa,np_", MW_CASES)
def test_maxwell_leaf_blocks(ctx, oracle, geo, M, P, kappa, np_):
    d, o = _pair(ctx, oracle, geo, M, P, 2, kappa, np_)
    worst = 0.0
    for li in range(len(o.leaves())):
        for rc in range(2):
            for cc in range(2):
                a = d.leaf_block(li, rc, cc)
                b = o.leaf_matrix(li, rc, cc)
                worst = max(worst, np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
    assert worst < FP64_TOL, worst


@pytest.mark.parametrize("geo,M,P,kappa,np_", MW_CASES)
def test_maxwell_matvec(ctx, oracle, geo, M, P, kappa, np_):
    d, o = _pair(ctx, oracle, geo, M, P, 2, kappa, np_)
    rng = np.random.default_rng(11)
    A = d.get_discrete_operator()
    for nrhs in (1, 3, 11):  # 11 crosses the 8-column chunk of the far field
        x = rng.uniform(-1, 1, (d.N, nrhs)) + 1j * rng.uniform(-1, 1, (d.N, nrhs))
        ref = o.matvec(x)
        y64 = A.matvec(x)
        assert np.linalg.norm(y64 - ref) / np.linalg.norm(ref) < FP64_TOL
        for prec in ("mixed", "fp32"):
            y = A.matvec(x, precision=prec)
            assert np.linalg.norm(y - ref) / np.linalg.norm(ref) < MW_FP32_TOL, prec


def test_maxwell_dipole_load_vector(ctx, oracle):
    d, o = _pair(ctx, oracle, SPHERE, 2, 2, 2, 2.0, 6)
    prm = np.array([[0.0, 0.1, 2.5, 0.3, -0.2, 0.9], [1.5, -1.8, 0.7, 1.0, 0.0, 0.0]])
    got = d.load_vector(3, prm)
    for c in range(prm.shape[0]):
        ref = o.load_vector(3, prm[c])
        assert np.linalg.norm(got[:, c] - ref) / np.linalg.norm(ref) < FP64_TOL


@pytest.mark.parametrize("inner", ["fp64", "fp32"])
def test_maxwell_solve(ctx, oracle, inner):
    d, o = _pair(ctx, oracle, SPHERE, 2, 2, 2, 2.0, 6)
    prm = np.array([[0.0, 0.1, 2.5, 0.3, -0.2, 0.9], [1.5, -1.8, 0.7, 1.0, 0.0, 0.0]])
    b = d.load_vector(3, prm)
    x, st = d.get_discrete_operator().solve(b, tol=1e-8, inner=inner)
    assert st["converged"]
    for c in range(2):
        r = b[:, c] - o.matvec(x[:, c:c + 1])[:, 0]
        assert np.linalg.norm(r) / np.linalg.norm(b[:, c]) < 1e-7


def test_maxwell_potential(ctx, oracle):
    d, o = _pair(ctx, oracle, SPHERE, 2, 2, 2, 2.0, 6)
    rng = np.random.default_rng(13)
    rho = rng.uniform(-1, 1, (d.N, 2)) + 1j * rng.uniform(-1, 1, (d.N, 2))
    pts = np.r_[rng.uniform(-0.3, 0.3, (4, 3)), 2.0 * np.eye(3)]
    got = d.potential(rho, pts)
    for c in range(2):
        ref = o.potential(rho[:, c], pts)
        assert np.linalg.norm(got[:, :, c] - ref) / np.linalg.norm(ref) < FP64_TOL


def test_maxwell_field_converges_on_gpu(ctx):
    """examples/MaxwellSingleLayerH2.cpp:30-96 on the GPU path: dipole inside
    the sphere, field at radius 2, rate >= 0.9 (2P + 1) for P = 1."""
    import bembel_gb300 as bg
    from test_oracle_pins import _dipole_field, _sphere_points
    k, pos, mom = 2.0, np.array([0.2, 0.2, 0.2]), np.array([0.0, 0.1, 0.1])
    grid = _sphere_points(2.0, 100)
    ref = _dipole_field(grid, k, pos, mom)
    errs = []
    for M in (1, 2, 3):
        lin = bg.MaxwellSingleLayerOperator()
        lin.set_wavenumber(k)
        d = bg.DiscreteOperator(bg.AnsatzSpace(bg.Geometry(SPHERE, ctx), M, 1), lin)
        d.compute()
        x, st = d.get_discrete_operator().solve(d.load_vector(3, np.r_[pos, mom]), tol=1e-10)
        assert st["converged"]
        errs.append(np.max(np.linalg.norm(d.potential(x, grid)[:, :, 0] - ref, axis=1)))
    rates = np.log2(np.array(errs[:-1]) / np.array(errs[1:]))
    assert np.all(rates >= 0.9 * 3), (errs, rates)


def test_released_fp64_blocks_keep_products(ctx, oracle):
    """keep_fp64_blocks=False: the products read the double-float pairs and
    tiles, so they still match; only the leaf inspection is refused."""
    import bembel_gb300 as bg
    for kind, k in ((0, 0.0), (1, 2.0)):
        lin = bg.LaplaceSingleLayerOperator() if kind == 0 else bg.HelmholtzSingleLayerOperator()
        if kind:
            lin.set_wavenumber(k)
        d = bg.DiscreteOperator(bg.AnsatzSpace(bg.Geometry(SPHERE, ctx), 2, 1), lin, n_p=6, keep_fp64_blocks=False)
        d.compute()
        o = oracle.Problem(SPHERE, 2, 1, kind, kappa=k, np_=6)
        rng = np.random.default_rng(3)
        x = rng.uniform(-1, 1, (d.N, 3)) + (1j * rng.uniform(-1, 1, (d.N, 3)) if kind else 0)
        ref = o.matvec(x)
        A = d.get_discrete_operator()
        assert np.linalg.norm(A.matvec(x) - ref) / np.linalg.norm(ref) < FP64_TOL
        assert np.linalg.norm(A.matvec(x, precision="fp32") - ref) / np.linalg.norm(ref) < FP32_TOL
        far = [i for i, l in enumerate(d.leaves()) if l[0] == 1][0]
        with pytest.raises(bg.BembelError):
            d.leaf_block(far)


@pytest.mark.parametrize("np_,nrhs", [(10, 3), (6, 20)])
def test_helmholtz_tile_shapes_and_chunks(ctx, oracle, np_, nrhs):
    """Complex tensor-core far field at n_p = 10 (the torus sweep's tile shape)
    and with more right-hand sides than one 16-column pass."""
    d, o = _pair(ctx, oracle, SPHERE, 2, 1, 1, 3.0, np_)
    rng = np.random.default_rng(19)
    x = rng.uniform(-1, 1, (d.N, nrhs)) + 1j * rng.uniform(-1, 1, (d.N, nrhs))
    ref = o.matvec(x)
    A = d.get_discrete_operator()
    assert np.linalg.norm(A.matvec(x) - ref) / np.linalg.norm(ref) < FP64_TOL
    for prec in ("mixed", "fp32"):
        assert np.linalg.norm(A.matvec(x, precision=prec) - ref) / np.linalg.norm(ref) < FP32_TOL, prec


def test_helmholtz_field_converges_on_gpu(ctx):
    """examples/HelmholtzSingleLayerH2.cpp:30-98 on the GPU path: source at the
    origin, kappa = 2, potential at 100 points of radius 2, rate >= 0.9 (2P + 3), P = 0."""
    import math
    import bembel_gb300 as bg
    from test_oracle_pins import _sphere_points
    k = 2.0
    grid = _sphere_points(2.0, 100)
    r = np.linalg.norm(grid, axis=1)
    ref = np.exp(-1j * k * r) / (4 * math.pi * r)
    errs = []
    for M in (1, 2, 3):
        lin = bg.HelmholtzSingleLayerOperator()
        lin.set_wavenumber(k)
        d = bg.DiscreteOperator(bg.AnsatzSpace(bg.Geometry(SPHERE, ctx), M, 0), lin)
        d.compute()
        x, st = d.get_discrete_operator().solve(d.load_vector(1, np.zeros((1, 3))), tol=1e-10)
        assert st["converged"]
        errs.append(np.max(np.abs(d.potential(x, grid)[:, 0] - ref)))
    rates = np.log2(np.array(errs[:-1]) / np.array(errs[1:]))
    assert rates[-1] >= 0.9 * 3, (errs, rates)


def test_watchdog_wait_runs_out_and_context_survives(ctx, oracle):
    """Failure detection without a GPU fault: a bounded wait on an mbarrier
    that nothing completes runs out (about 1 ms), the kernel reports it,
    the call returns BG_TIMEOUT, and the context keeps working."""
    from bembel_gb300 import _lib
    assert _lib.load().bg_watchdog_selftest(ctx.h, 2_000_000) == _lib.BG_TIMEOUT
    assert "ran out" in _lib.load().bg_last_error_string(ctx.h).decode()
    d, o = _pair(ctx, oracle, SPHERE, 2, 1, 0)
    x = np.random.default_rng(4).uniform(-1, 1, (d.N, 2))
    ref = o.matvec(x)
    assert np.linalg.norm(d.get_discrete_operator().matvec(x) - ref) / np.linalg.norm(ref) < FP64_TOL
