"""Near fields of several Helmholtz wavenumbers in one pass
(bg_operator_prepare_wavenumbers).

Five wavenumbers are prepared together (one launch of 4 and one of 1 per
Duffy rule). For two of them the operator is then assembled with the
prepared near field, and its leaf blocks and products are compared with an
operator assembled for that wavenumber alone: the batched kernels evaluate
the same samples, in the same order for regular and identical pairs and in
another (the single-wavenumber kernels factorise the common-edge and
common-vertex rules' inner sums), so the blocks agree to 1e-13 relative.
One wavenumber is also checked against the oracle (1e-12, the bound of the
other leaf-block tests).
"""
import numpy as np
import pytest

from conftest import SPHERE, TORUS

pytestmark = pytest.mark.gpu

KAPPAS = [0.7, 2.0, 3.5, 5.1, 6.0]
SAME_TOL = 1e-13
FP64_TOL = 1e-12


@pytest.fixture(scope="module")
def ctx():
    import bembel_gb300 as bg
    return bg.Context(0)


def _op(ctx, geo, M, P, kappa, np_=6):
    import bembel_gb300 as bg
    lin = bg.HelmholtzSingleLayerOperator()
    lin.set_wavenumber(kappa)
    return bg.DiscreteOperator(bg.AnsatzSpace(bg.Geometry(geo, ctx), M, P), lin, n_p=np_), lin


@pytest.mark.parametrize("geo,M,P", [(SPHERE, 2, 2), (TORUS, 1, 1)])
def test_prepared_near_fields_match_single_assembly(ctx, geo, M, P):
    d, lin = _op(ctx, geo, M, P, KAPPAS[0])
    d.prepare_wavenumbers(KAPPAS)
    rng = np.random.default_rng(21)
    x = rng.uniform(-1, 1, (d.N, 3)) + 1j * rng.uniform(-1, 1, (d.N, 3))
    dense = [i for i, lv in enumerate(d.leaves()) if lv[0] == 2]
    for kappa in (KAPPAS[1], KAPPAS[4]):
        lin.set_wavenumber(kappa)
        d.compute()
        ref, _ = _op(ctx, geo, M, P, kappa)
        ref.compute()
        worst = max(np.linalg.norm(d.leaf_block(i) - ref.leaf_block(i)) / np.linalg.norm(ref.leaf_block(i))
                    for i in dense)
        assert worst < SAME_TOL, (kappa, worst)
        y, yr = d.get_discrete_operator().matvec(x), ref.get_discrete_operator().matvec(x)
        assert np.linalg.norm(y - yr) / np.linalg.norm(yr) < SAME_TOL
    d.release_wavenumbers()


def test_prepared_near_field_against_oracle(ctx, oracle):
    d, lin = _op(ctx, SPHERE, 2, 1, KAPPAS[0])
    d.prepare_wavenumbers(KAPPAS)
    lin.set_wavenumber(KAPPAS[3])
    d.compute()
    o = oracle.Problem(SPHERE, 2, 1, oracle.HELMHOLTZ, kappa=KAPPAS[3], np_=6)
    worst = 0.0
    for li in range(len(o.leaves())):
        a, b = d.leaf_block(li), o.leaf_matrix(li)
        worst = max(worst, np.linalg.norm(a - b) / np.linalg.norm(b))
    assert worst < FP64_TOL, worst


def test_batched_wavenumbers(ctx):
    """Three wavenumbers assembled side by side
    (bg_operator_assemble_wavenumbers): one call of the product, the load
    vector, the potential and the solve covers all three, column block q with
    wavenumber q, and each block equals the single-wavenumber operator's
    result (products 1e-13 as above; the mixed and FP32 products to 1e-12).
    The products run as one pass over all wavenumbers (one tensor-core
    far-field launch per 16 columns of every block), also with 3 x 40 columns,
    which the product takes in slices of 10 columns of every block.
    The batched solve is one flexible GMRES over the 3 x 4 columns; every
    block meets the FP64 residual 2e-8 of its own wavenumber's operator, also
    with 3 x 90 columns, which the solver takes in two slices of every
    block."""
    import bembel_gb300 as bg
    ks = [0.7, 2.0, 3.5]
    nr = 4
    d, lin = _op(ctx, SPHERE, 2, 1, ks[0])
    d.prepare_wavenumbers(ks)
    d.assemble_wavenumbers()
    assert np.allclose(d.wavenumbers(), ks)
    refs = []
    for k in ks:
        r, _ = _op(ctx, SPHERE, 2, 1, k)
        r.compute()
        refs.append(r)
    rng = np.random.default_rng(41)
    x = rng.uniform(-1, 1, (d.N, 3 * nr)) + 1j * rng.uniform(-1, 1, (d.N, 3 * nr))
    A = d.get_discrete_operator()
    for prec, tol in (("fp64", 1e-13), ("mixed", 1e-12), ("fp32", 1e-12)):
        y = A.matvec(x, precision=prec)
        for q in range(3):
            yr = refs[q].get_discrete_operator().matvec(x[:, q * nr:(q + 1) * nr], precision=prec)
            assert np.linalg.norm(y[:, q * nr:(q + 1) * nr] - yr) / np.linalg.norm(yr) < tol, (prec, q)
    dirs = rng.normal(size=(3 * nr, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    b = d.load_vector(2, dirs)
    for q in range(3):
        br = refs[q].load_vector(2, dirs[q * nr:(q + 1) * nr])
        assert np.linalg.norm(b[:, q * nr:(q + 1) * nr] - br) / np.linalg.norm(br) < 1e-14
    xs, st = A.solve(b, tol=1e-8, inner="fp32")
    assert st["converged"]
    pts = rng.uniform(-0.3, 0.3, (5, 3))
    pot = d.potential(xs, pts)
    for q in range(3):
        Aq = refs[q].get_discrete_operator()
        bq, xq = b[:, q * nr:(q + 1) * nr], xs[:, q * nr:(q + 1) * nr]
        res = np.linalg.norm(bq - Aq.matvec(xq), axis=0) / np.linalg.norm(bq, axis=0)
        assert res.max() < 2e-8, (q, res)
        pr = refs[q].potential(xq, pts)
        assert np.linalg.norm(pot[:, q * nr:(q + 1) * nr] - pr) / np.linalg.norm(pr) < 1e-14
    # 40 columns per wavenumber: four slices of 10 columns of every block
    xw = rng.uniform(-1, 1, (d.N, 3 * 40)) + 1j * rng.uniform(-1, 1, (d.N, 3 * 40))
    for prec, tol in (("fp64", 1e-13), ("mixed", 1e-12)):
        y = A.matvec(xw, precision=prec)
        for q in range(3):
            yr = refs[q].get_discrete_operator().matvec(xw[:, q * 40:(q + 1) * 40], precision=prec)
            assert np.linalg.norm(y[:, q * 40:(q + 1) * 40] - yr) / np.linalg.norm(yr) < tol, (prec, q)
    with pytest.raises(bg.BembelError):
        A.matvec(x[:, :5])
    with pytest.raises(bg.BembelError):
        d.leaf_block(0)
    # 90 columns per wavenumber: the solve runs in slices of 85 and 5 columns
    # of every block (two batches); each block still solves its own system
    big = 90
    dirs = rng.normal(size=(big, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    bb = d.load_vector(2, np.tile(dirs, (3, 1)))
    xb, st = A.solve(bb, tol=1e-8, inner="fp32")
    assert st["converged"]
    for q in range(3):
        Aq = refs[q].get_discrete_operator()
        bq, xq = bb[:, q * big:(q + 1) * big], xb[:, q * big:(q + 1) * big]
        res = np.linalg.norm(bq - Aq.matvec(xq), axis=0) / np.linalg.norm(bq, axis=0)
        assert res.max() < 2e-8, (q, res.max())
    d.release_wavenumbers()
    lin.set_wavenumber(ks[1])
    d.compute()
    y = d.get_discrete_operator().matvec(x[:, :nr])
    yr = refs[1].get_discrete_operator().matvec(x[:, :nr])
    assert np.linalg.norm(y - yr) / np.linalg.norm(yr) < 1e-12
