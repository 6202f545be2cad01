"""Launch plans and the autotuner (bg_operator_set_plan / bg_operator_autotune).

Every plan must give the product of the built-in plan: the far-field row
orders only permute which persistent CTA computes a row, so the result agrees
to 1e-9 relative (each row is still summed by one CTA in block order); the
near-field kernel variants and the split-K threshold change FP32 summation
orders, so they agree to 1e-5 relative, the tolerance of the other FP32
product tests. The two transform paths (fused launches through the
tensor-product factors, or batched GEMMs with the assembled FMM matrices)
agree to rounding: 1e-12 for the FP64 product, 1e-5 for FP32. The autotuner's chosen plan is then set on the operator and
gives the same product. Collected after the other product tests.
"""
import numpy as np
import pytest

from conftest import SPHERE

pytestmark = pytest.mark.gpu

FP32_TOL = 1e-5
ORDER_TOL = 1e-9


@pytest.fixture(scope="module")
def ctx():
    import bembel_gb300 as bg
    return bg.Context(0)


def _op(ctx, kind, M, P, kappa=1.0):
    import bembel_gb300 as bg
    lin = bg.LaplaceSingleLayerOperator() if kind == "laplace" else bg.HelmholtzSingleLayerOperator()
    if kind != "laplace":
        lin.set_wavenumber(kappa)
    d = bg.DiscreteOperator(bg.AnsatzSpace(bg.Geometry(SPHERE, ctx), M, P), lin)
    d.compute()
    return d


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.fixture(scope="module")
def laplace_m4(ctx):
    # sphere M = 4: 504 far-field rows, more than one round of persistent CTAs
    return _op(ctx, "laplace", 4, 2)


@pytest.mark.parametrize("prec", ["fp32", "mixed"])
def test_every_plan_gives_the_builtin_product(laplace_m4, prec):
    d = laplace_m4
    A = d.get_discrete_operator()
    x = np.random.default_rng(11).uniform(-1, 1, (d.N, 32))
    d.set_plan(32, prec)
    y0 = A.matvec(x, precision=prec)
    for order in (1, 2):
        d.set_plan(32, prec, far_order=order)
        assert _rel(A.matvec(x, precision=prec), y0) < ORDER_TOL
    d.set_plan(32, prec, transforms=1)
    assert _rel(A.matvec(x, precision=prec), y0) < FP32_TOL
    for ctas in (1, 2):
        d.set_plan(32, prec, far_ctas=ctas)
        assert _rel(A.matvec(x, precision=prec), y0) < ORDER_TOL
    for split in (0, 608):
        d.set_plan(32, prec, split_k_batches=split)
        assert _rel(A.matvec(x, precision=prec), y0) < FP32_TOL
    if prec == "fp32":
        for near in (1, 2, 3):
            d.set_plan(32, prec, near_kernel=near)
            assert _rel(A.matvec(x, precision=prec), y0) < FP32_TOL
    d.set_plan(32, prec)


@pytest.mark.parametrize("prec", ["fp32", "mixed", "fp64"])
def test_autotune_sets_a_plan_with_the_same_product(laplace_m4, prec):
    d = laplace_m4
    A = d.get_discrete_operator()
    x = np.random.default_rng(12).uniform(-1, 1, (d.N, 32))
    d.set_plan(32, prec)
    y0 = A.matvec(x, precision=prec)
    r = d.autotune(32, prec, reps=2)
    assert r["candidates"] >= 1 and r["builtin_ms"] > 0 and 0 < r["tuned_ms"] <= r["builtin_ms"]
    assert d.get_plan(32, prec) == r["plan"]
    if prec == "fp64":
        assert r["candidates"] == 2  # the built-in plan and the batched-GEMM transforms
    tol = 1e-12 if prec == "fp64" else FP32_TOL
    assert _rel(A.matvec(x, precision=prec), y0) < tol
    d.set_plan(32, prec)


def test_complex_near_variants(ctx):
    d = _op(ctx, "helmholtz", 3, 2)
    A = d.get_discrete_operator()
    rng = np.random.default_rng(13)
    x = rng.uniform(-1, 1, (d.N, 8)) + 1j * rng.uniform(-1, 1, (d.N, 8))
    y0 = A.matvec(x, precision="fp32")
    for near in (1, 2, 3):
        d.set_plan(8, "fp32", near_kernel=near)
        assert _rel(A.matvec(x, precision="fp32"), y0) < FP32_TOL
    r = d.autotune(8, "fp32", reps=2)
    assert r["candidates"] >= 3
    assert _rel(A.matvec(x, precision="fp32"), y0) < FP32_TOL


def test_fp64_transform_paths_agree(laplace_m4):
    d = laplace_m4
    A = d.get_discrete_operator()
    x = np.random.default_rng(14).uniform(-1, 1, (d.N, 5))
    d.set_plan(5, "fp64")
    y0 = A.matvec(x)
    d.set_plan(5, "fp64", transforms=1)
    assert _rel(A.matvec(x), y0) < 1e-12
    d.set_plan(5, "fp64")


def test_far_hi_tiles_inner_operator(laplace_m4):
    """Launch plan far_tiles = 1 (the FP16 hi coupling tiles only): the mixed
    product stays within 1e-3 of the FP64 product (11 bits per coupling in
    the far field; measured about 1e-4), and the flexible GMRES with that
    inner operator still reaches the FP64 residual 1e-8."""
    d = laplace_m4
    rng = np.random.default_rng(29)
    x = rng.uniform(-1, 1, (d.N, 32))
    A = d.get_discrete_operator()
    y64 = A.matvec(x)
    d.set_plan(32, "mixed", far_tiles=1)
    yhi = A.matvec(x, precision="mixed")
    d.set_plan(32, "mixed")
    ymx = A.matvec(x, precision="mixed")
    err_hi = np.max(np.linalg.norm(yhi - y64, axis=0) / np.linalg.norm(y64, axis=0))
    err_mx = np.max(np.linalg.norm(ymx - y64, axis=0) / np.linalg.norm(y64, axis=0))
    assert err_hi < 1e-3 and err_mx < 1e-5, (err_hi, err_mx)
    b = d.load_vector(0, 3.0 * rng.normal(size=(32, 3)) / np.sqrt(3))
    d.set_plan(32, "mixed", far_tiles=1)
    xs, st = A.solve(b, tol=1e-8, inner="mixed")
    d.set_plan(32, "mixed")
    assert st["converged"]
    res = np.linalg.norm(b - A.matvec(xs), axis=0) / np.linalg.norm(b, axis=0)
    assert res.max() < 2e-8, res.max()
