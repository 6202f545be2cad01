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
