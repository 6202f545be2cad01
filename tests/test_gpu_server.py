"""Serving loop (bg_server_*): requests on different operators, batching,
eviction under a small memory budget and admission failure, checked by the
FP64 residual of every served solution."""
import ctypes

import numpy as np
import pytest

from conftest import SPHERE, TORUS

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import bembel_gb300 as bg
    return bg.Context(0)


def _residual(ctx, geo, kind, M, P, kappa, data_kind, data, x):
    import bembel_gb300 as bg
    lin = {"laplace": bg.LaplaceSingleLayerOperator, "helmholtz": bg.HelmholtzSingleLayerOperator}[kind]()
    if kind != "laplace":
        lin.set_wavenumber(kappa)
    d = bg.DiscreteOperator(bg.AnsatzSpace(bg.Geometry(geo, ctx), M, P), lin)
    d.compute()
    b = d.load_vector(data_kind, data)
    r = b - d.get_discrete_operator().matvec(x)
    return np.max(np.linalg.norm(r, axis=0) / np.linalg.norm(b, axis=0))


def _cases():
    rng = np.random.default_rng(21)
    pts = lambda n: rng.normal(size=(n, 3)) / 0.4  # point sources outside the surfaces (|x| ~ 2.5 and more)
    dirs = lambda n: (lambda d: d / np.linalg.norm(d, axis=1, keepdims=True))(rng.normal(size=(n, 3)))
    far = lambda n: (lambda d: 3.5 * d)(dirs(n))
    return [
        (0, SPHERE, "laplace", 2, 1, 0.0, 0, far(3)),
        (0, SPHERE, "laplace", 2, 1, 0.0, 0, far(2)),
        (0, SPHERE, "helmholtz", 2, 1, 2.0, 2, dirs(4)),
        (1, TORUS, "laplace", 1, 2, 0.0, 0, 1.5 * far(2)),
        (0, SPHERE, "laplace", 2, 1, 0.0, 0, far(5)),
    ]


def test_server_solves_and_batches(ctx):
    import bembel_gb300 as bg
    srv = bg.Server(ctx, 50e9, workers=2)
    gs = [srv.add_geometry(bg.Geometry(SPHERE, ctx)), srv.add_geometry(bg.Geometry(TORUS, ctx))]
    cases = _cases()
    tickets = [srv.submit(gs[g], kind, M, P, dk, data, kappa=k) for g, _, kind, M, P, k, dk, data in cases]
    out = [srv.wait(t, timeout=300) for t in tickets]
    st = srv.stats()
    # collected and never-issued tickets are refused instead of waiting forever
    from bembel_gb300 import _lib
    for t in (tickets[0], max(tickets) + 1000):
        r = _lib.RequestResult()
        assert _lib.load().bg_server_wait(srv.h, t, -1.0, ctypes.byref(r)) == _lib.BG_INVALID_ARG
    srv.close()
    assert st["completed"] == len(cases) and st["failed"] == 0, [(i["status"], i["error"]) for _, i in out]
    assert st["cache_misses"] == 3  # three distinct operators
    assert st["batches"] <= len(cases)
    for (g, geo, kind, M, P, k, dk, data), (x, info) in zip(cases, out):
        assert info["status"] == 0 and x is not None
        assert info["t_submit"] <= info["t_start"] <= info["t_done"]
        assert info["batch_nrhs"] >= data.shape[0]
        assert _residual(ctx, geo, kind, M, P, k, dk, data, x) < 1e-7


def test_server_evicts_under_budget(ctx):
    import bembel_gb300 as bg
    from bembel_gb300 import _lib
    # budget: room for the larger of two operators, not for both
    sizes = []
    for M in (2, 3):
        d = bg.DiscreteOperator(bg.AnsatzSpace(bg.Geometry(SPHERE, ctx), M, 1), bg.LaplaceSingleLayerOperator(),
                                keep_fp64_blocks=False)  # as the server caches them
        import ctypes
        a, e = ctypes.c_size_t(), ctypes.c_size_t()
        ctx.check(_lib.load().bg_operator_memory(d.h, ctypes.byref(a), ctypes.byref(e)))
        sizes.append(e.value)
    srv = bg.Server(ctx, int(max(sizes) + min(sizes) // 2))
    g = srv.add_geometry(bg.Geometry(SPHERE, ctx))
    data = 3.0 * np.array([[0.0, 0.6, 0.8], [1.0, 0.0, 0.0]])
    seq = [2, 3, 2, 3]
    res = []
    for M in seq:  # one at a time, so each request needs the other operator evicted
        x, info = srv.wait(srv.submit(g, "laplace", M, 1, 0, data), timeout=300)
        res.append((M, x, info))
    st = srv.stats()
    srv.close()
    assert st["evictions"] >= 3 and st["failed"] == 0
    assert st["bytes_in_use"] <= st["bytes_budget"]
    for M, x, info in res:
        assert not info["cache_hit"]
        assert _residual(ctx, SPHERE, "laplace", M, 1, 0.0, 0, data, x) < 1e-7


def test_server_budget_is_shared_by_workers(ctx):
    """Two workers, a budget with room for the larger of two operators but
    not for both, and less than twice it: the larger operator is admitted
    (the budget is not split between the workers), and alternating requests
    evict each other's operators across workers."""
    import ctypes
    import bembel_gb300 as bg
    from bembel_gb300 import _lib
    sizes = []
    for M in (2, 3):
        d = bg.DiscreteOperator(bg.AnsatzSpace(bg.Geometry(SPHERE, ctx), M, 1), bg.LaplaceSingleLayerOperator(),
                                keep_fp64_blocks=False)
        a, e = ctypes.c_size_t(), ctypes.c_size_t()
        ctx.check(_lib.load().bg_operator_memory(d.h, ctypes.byref(a), ctypes.byref(e)))
        sizes.append(e.value)
    budget = int(max(sizes) + min(sizes) // 2)
    assert budget < 2 * max(sizes)
    srv = bg.Server(ctx, budget, workers=2)
    g = srv.add_geometry(bg.Geometry(SPHERE, ctx))
    data = 3.0 * np.array([[0.0, 0.6, 0.8], [1.0, 0.0, 0.0]])
    res = []
    for M in (3, 2, 3, 2):
        x, info = srv.wait(srv.submit(g, "laplace", M, 1, 0, data), timeout=300)
        res.append((M, x, info))
    st = srv.stats()
    srv.close()
    assert st["failed"] == 0 and st["evictions"] >= 3, st
    assert st["bytes_in_use"] <= st["bytes_budget"]
    for M, x, info in res:
        assert info["status"] == 0
        assert _residual(ctx, SPHERE, "laplace", M, 1, 0.0, 0, data, x) < 1e-7


def test_server_rejects_operator_above_budget(ctx):
    import bembel_gb300 as bg
    from bembel_gb300 import _lib
    srv = bg.Server(ctx, 1 << 20)
    g = srv.add_geometry(bg.Geometry(SPHERE, ctx))
    x, info = srv.wait(srv.submit(g, "laplace", 3, 2, 0, [[0.0, 0.0, 3.0]]), timeout=60)
    st = srv.stats()
    srv.close()
    assert x is None and info["status"] == _lib.BG_OOM
    assert st["failed"] == 1 and st["cached_operators"] == 0


def test_server_results_alone_and_in_the_mix(ctx):
    """Each request's solution is the same whether it is served alone or
    together with the others (batched with same-operator requests, overlapped
    with other operators' solves on other worker streams), within the solve
    tolerance: both meet the 1e-8 residual and agree to 1e-5 relative."""
    import bembel_gb300 as bg
    cases = _cases()
    srv = bg.Server(ctx, 50e9, workers=2)
    gs = [srv.add_geometry(bg.Geometry(SPHERE, ctx)), srv.add_geometry(bg.Geometry(TORUS, ctx))]
    alone = [srv.wait(srv.submit(gs[g], kind, M, P, dk, data, kappa=k), timeout=300)
             for g, _, kind, M, P, k, dk, data in cases]
    tickets = [srv.submit(gs[g], kind, M, P, dk, data, kappa=k) for g, _, kind, M, P, k, dk, data in cases]
    mix = [srv.wait(t, timeout=300) for t in tickets]
    srv.close()
    for (x1, i1), (x2, i2) in zip(alone, mix):
        assert i1["status"] == 0 and i2["status"] == 0
        assert i1["stats"]["final_relres"] <= 1e-8 and i2["stats"]["final_relres"] <= 1e-8
        assert np.linalg.norm(x2 - x1) / np.linalg.norm(x1) < 1e-5
