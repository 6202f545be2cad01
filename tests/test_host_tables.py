"""Host-side setup of the product (host-only context, no GPU) against the oracle:
element tree, vertex topology, enclosing balls, block partition and the
transformation matrix T."""
import re

import numpy as np
import pytest

from conftest import CUBE, ROOT, SPHERE, TORUS, geometry


@pytest.fixture(scope="module")
def bg_host():
    import bembel_gb300 as bg
    return bg, bg.Context(-1)


def test_library_exports_every_declared_symbol():
    import ctypes
    from bembel_gb300 import _lib
    header = open(ROOT + "/include/bembel_gb300.h").read()
    names = set(re.findall(r"\b(bg_[a-z0-9_]+)\s*\(", header))
    assert len(names) >= 20
    L = ctypes.CDLL(_lib.LIB_PATH) if _lib._lib is None else _lib._lib
    _lib.load()
    missing = [n for n in sorted(names) if not hasattr(_lib.load(), n)]
    assert not missing


@pytest.mark.parametrize("geo,M,P", [(SPHERE, 3, 1), (SPHERE, 2, 2), (TORUS, 2, 2), (SPHERE, 1, 0), (SPHERE, 0, 1),
                                     (CUBE, 3, 1), (CUBE, 2, 2)])
def test_tables_match_oracle(bg_host, oracle, geo, M, P):
    bg, ctx = bg_host
    g = geometry(bg, geo, ctx)
    d = bg.DiscreteOperator(bg.AnsatzSpace(g, M, P), bg.LaplaceSingleLayerOperator(), n_p=6)
    o = oracle.Problem(geo, M, P, oracle.LAPLACE, np_=6, assemble=False)
    assert (d.N, d.S, d.n_dense, d.n_lowrank) == (o.N, o.S, o.n_dense, o.n_lowrank)
    pi, pd = d.elements()
    oi, od = o.elements()
    assert np.array_equal(pi[:, 0], oi[:, 0])
    # vertex numbering differs, the identification must be the same bijection
    mp = {}
    for e in range(d.ne):
        for k in range(4):
            assert mp.setdefault(int(pi[e, 1 + k]), int(oi[e, 3 + k])) == int(oi[e, 3 + k])
    assert len(set(mp.values())) == len(mp)
    assert np.array_equal(pd[:, :2], od[:, :2])
    assert np.array_equal(pd[:, 2:], od[:, 2:])  # enclosing balls bit-identical
    ps = set(map(tuple, d.leaves().tolist()))
    os_ = set(map(tuple, o.leaves()[:, :4].tolist()))
    assert ps == os_
    a, b = d.transform_csr(), o.transform_csr()
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert np.abs(a[2] - b[2]).max() < 1e-13


@pytest.mark.parametrize("geo,M,P", [(SPHERE, 1, 1), (SPHERE, 2, 2), (TORUS, 1, 3), ("screen", 1, 2), ("screen", 2, 1),
                                     (CUBE, 2, 2)])
def test_divconforming_transform_matches_oracle(bg_host, oracle, screen_path, geo, M, P):
    """Maxwell's T = Projector * Glue (div-conforming gluing across patch
    edges, boundary functions of an open surface dropped), against the oracle."""
    bg, ctx = bg_host
    geo = screen_path if geo == "screen" else geo
    lin = bg.MaxwellSingleLayerOperator()
    lin.set_wavenumber(1.0)
    d = bg.DiscreteOperator(bg.AnsatzSpace(geometry(bg, geo, ctx), M, P), lin, n_p=4)
    o = oracle.Problem(geo, M, P, oracle.MAXWELL, kappa=1.0, np_=4, assemble=False)
    assert (d.N, d.S) == (o.N, o.S)
    a, b = d.transform_csr(), o.transform_csr()
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert np.abs(a[2] - b[2]).max() < 1e-13


def test_surface_point_matches_oracle(bg_host, oracle):
    bg, ctx = bg_host
    g = bg.Geometry(SPHERE, ctx)
    o = oracle.Problem(SPHERE, 0, 0, oracle.LAPLACE, np_=6, assemble=False)
    rng = np.random.default_rng(5)
    for _ in range(50):
        p, s, t = int(rng.integers(6)), rng.uniform(), rng.uniform()
        assert np.abs(g.surface_point(p, s, t)[3:] - o.surface_point(p, s, t)[3:]).max() < 1e-14


def test_host_only_context_refuses_device_work(bg_host):
    bg, ctx = bg_host
    g = bg.Geometry(SPHERE, ctx)
    d = bg.DiscreteOperator(bg.AnsatzSpace(g, 1, 1), bg.LaplaceSingleLayerOperator(), n_p=6)
    with pytest.raises(bg.BembelError) as ei:
        d.compute()
    assert "host-only" in str(ei.value)


def test_invalid_arguments(bg_host):
    bg, ctx = bg_host
    with pytest.raises(bg.BembelError):
        bg.Geometry("/nonexistent/file.dat", ctx)
    g = bg.Geometry(SPHERE, ctx)
    with pytest.raises(bg.BembelError):
        bg.DiscreteOperator(bg.AnsatzSpace(g, 1, 7), bg.LaplaceSingleLayerOperator())
    with pytest.raises(bg.BembelError):
        bg.DiscreteOperator(bg.AnsatzSpace(g, 1, 1), bg.LaplaceSingleLayerOperator(), n_p=1)


def test_memory_estimate_before_assembly(bg_host):
    """The serving loop admits operators by this estimate; it is available
    before assembly and covers the stored fields."""
    import ctypes
    from bembel_gb300 import _lib
    bg, ctx = bg_host
    g = bg.Geometry(SPHERE, ctx)
    prev = 0
    for M in (1, 2, 3):
        d = bg.DiscreteOperator(bg.AnsatzSpace(g, M, 2), bg.LaplaceSingleLayerOperator())
        a, e = ctypes.c_size_t(), ctypes.c_size_t()
        ctx.check(_lib.load().bg_operator_memory(d.h, ctypes.byref(a), ctypes.byref(e)))
        info = d.info()
        assert a.value == 0  # nothing on a device
        assert e.value >= int(info[13]) + int(info[14]) and e.value > prev
        prev = e.value


def test_host_only_context_refuses_server(bg_host):
    import ctypes
    from bembel_gb300 import _lib
    bg, ctx = bg_host
    h = ctypes.c_void_p()
    assert _lib.load().bg_server_create(ctx.h, 1 << 30, 1, ctypes.byref(h)) == _lib.BG_UNSUPPORTED
    assert _lib.load().bg_server_create(ctx.h, 0, 1, ctypes.byref(h)) == _lib.BG_INVALID_ARG
    assert _lib.load().bg_server_create(ctx.h, 1 << 30, 0, ctypes.byref(h)) == _lib.BG_INVALID_ARG


def test_igs_geometry_matches_dat(bg_host, tmp_path):
    """LoadGeometryFileIGS (Geometry/GeometryIGS.hpp:25-151): the sphere written
    as IGES entity 128 evaluates like the .dat sphere; other entities and
    interior knots are refused."""
    import sys
    sys.path.insert(0, ROOT + "/tests/golden")
    from igs_writer import read_dat, write_igs
    bg, ctx = bg_host
    patches = read_dat(SPHERE)
    igs = str(tmp_path / "sphere.igs")
    write_igs(patches, igs)
    a, b = bg.Geometry(SPHERE, ctx), bg.Geometry(igs, ctx)
    rng = np.random.default_rng(17)
    for _ in range(60):
        p, s, t = int(rng.integers(len(patches))), rng.uniform(), rng.uniform()
        assert np.abs(a.surface_point(p, s, t)[3:] - b.surface_point(p, s, t)[3:]).max() < 1e-13
    d1 = bg.DiscreteOperator(bg.AnsatzSpace(a, 2, 2), bg.LaplaceSingleLayerOperator())
    d2 = bg.DiscreteOperator(bg.AnsatzSpace(b, 2, 2), bg.LaplaceSingleLayerOperator())
    assert d1.N == d2.N and d1.n_lowrank == d2.n_lowrank
    bad = str(tmp_path / "bad.igs")
    write_igs(patches[:1], bad, entity=126)
    with pytest.raises(bg.BembelError):
        bg.Geometry(bad, ctx)
    px, py = patches[0][0], patches[0][1]
    write_igs(patches[:1], bad, knots=[([0.0] * px + [0.5] + [1.0] * px, [0.0] * py + [1.0] * py)])
    with pytest.raises(bg.BembelError) as ei:
        bg.Geometry(bad, ctx)
    assert "interior knots" in str(ei.value)
    # a control point with a negative weight is refused, as in the .dat reader
    px, py, X, Y, Z, W = patches[0]
    W = [-W[0]] + list(W[1:])
    X, Y, Z = ([-v[0]] + list(v[1:]) for v in (X, Y, Z))
    write_igs([(px, py, X, Y, Z, W)], bad)
    with pytest.raises(bg.BembelError) as ei:
        bg.Geometry(bad, ctx)
    assert "weight" in str(ei.value)


def test_watchdog_selftest_needs_a_gpu(bg_host):
    from bembel_gb300 import _lib
    bg, ctx = bg_host
    assert _lib.load().bg_watchdog_selftest(ctx.h, 1000) == _lib.BG_UNSUPPORTED
    assert _lib.load().bg_watchdog_selftest(ctx.h, 0) == _lib.BG_INVALID_ARG


def test_launch_plans_round_trip_and_validation(bg_host):
    """Launch plans are operator state keyed by (nrhs, precision): unset keys
    read as the built-in plan, out-of-range fields are refused, and the
    autotuner itself needs a device."""
    from bembel_gb300 import BembelError, _lib
    bg, ctx = bg_host
    d = bg.DiscreteOperator(bg.AnsatzSpace(bg.Geometry(SPHERE, ctx), 2, 2), bg.LaplaceSingleLayerOperator())
    builtin = {"near_kernel": 0, "split_k_batches": -1, "far_order": 0, "transforms": 0, "far_ctas": 0,
               "mixed_near": 0, "far_tiles": 0}
    assert d.get_plan(32, "mixed") == builtin
    d.set_plan(32, "fp32", near_kernel=2, split_k_batches=608, far_order=2, transforms=1, far_ctas=2, mixed_near=2,
               far_tiles=1)
    assert d.get_plan(32, "fp32") == {"near_kernel": 2, "split_k_batches": 608, "far_order": 2, "transforms": 1,
                                      "far_ctas": 2, "mixed_near": 2, "far_tiles": 1}
    assert d.get_plan(32, "mixed") == builtin and d.get_plan(16, "fp32") == builtin
    for bad in ({"near_kernel": 4}, {"near_kernel": -1}, {"split_k_batches": -2}, {"far_order": 3}, {"transforms": 2},
                {"transforms": -1}, {"far_ctas": 3}, {"far_ctas": -1}, {"mixed_near": 3}, {"mixed_near": -1},
                {"far_tiles": 2}, {"far_tiles": -1}):
        with pytest.raises(BembelError):
            d.set_plan(8, "mixed", **bad)
    with pytest.raises(BembelError):
        d.set_plan(0, "mixed")
    with pytest.raises(BembelError):
        d.get_plan(8, "fp16")
    assert d.get_plan(8, "mixed") == builtin
    with pytest.raises(BembelError) as e:
        d.autotune(32, "mixed")
    assert e.value.status == _lib.BG_UNSUPPORTED


def test_empty_inputs_are_no_ops(bg_host):
    """Zero right-hand sides or zero points: empty results and no error,
    before any device work (Eigen's products with empty operands are no-ops)."""
    bg, ctx = bg_host
    d = bg.DiscreteOperator(bg.AnsatzSpace(bg.Geometry(SPHERE, ctx), 1, 1), bg.LaplaceSingleLayerOperator())
    A = d.get_discrete_operator()
    assert A.matvec(np.zeros((d.N, 0))).shape == (d.N, 0)
    x, st = A.solve(np.zeros((d.N, 0)))
    assert x.shape == (d.N, 0) and st["converged"] and st["iterations"] == 0
    assert d.load_vector(0, np.zeros((0, 3))).shape == (d.N, 0)
    assert d.potential(np.zeros((d.N, 0)), np.ones((4, 3))).shape == (4, 0)
    assert d.potential(np.zeros((d.N, 2)), np.zeros((0, 3))).shape == (0, 2)
    with pytest.raises(bg.BembelError):  # one column still needs a device
        A.matvec(np.zeros(d.N))


def test_dat_loader_refuses_incomplete_patches(bg_host, tmp_path):
    """A .dat file cut inside its last patch, or with a zero weight, is an
    error instead of a geometry that evaluates to inf / nan."""
    bg, ctx = bg_host
    lines = open(SPHERE).read().splitlines()
    for cut in (len(lines) - 1, len(lines) - 3, len(lines) - 7):
        p = tmp_path / ("cut%d.dat" % cut)
        p.write_text("\n".join(lines[:cut]) + "\n")
        with pytest.raises(bg.BembelError):
            bg.Geometry(str(p), ctx)
    w = list(lines)
    w[-1] = " ".join(["0.0"] + w[-1].split()[1:])  # first weight of the last patch
    p = tmp_path / "zero_weight.dat"
    p.write_text("\n".join(w) + "\n")
    with pytest.raises(bg.BembelError) as ei:
        bg.Geometry(str(p), ctx)
    assert "weight" in str(ei.value)


def test_abi_entry_points_refuse_null_arguments(bg_host):
    """Every entry point declared in the header returns a status (no crash)
    when called with null pointers and zero sizes: first with null handles,
    then with valid host-only handles and everything else null or zero. Zero
    right-hand sides are an empty call (BG_OK); everything else is refused."""
    import ctypes
    from bembel_gb300 import _lib
    bg, ctx = bg_host
    hdr = re.sub(r"/\*.*?\*/", "", open(ROOT + "/include/bembel_gb300.h").read(), flags=re.S)
    decls = {name: [p.strip().replace(" ", "") for p in params.split(",")]
             for name, params in re.findall(r"\b(bg_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", hdr)}
    assert len(decls) >= 40
    g = bg.Geometry(SPHERE, ctx)
    d = bg.DiscreteOperator(bg.AnsatzSpace(g, 2, 1), bg.LaplaceSingleLayerOperator())
    handles = {"bg_context*": ctx.h, "bg_operator*": d.h, "constbg_operator*": d.h, "bg_geometry*": g.h,
               "constbg_geometry*": g.h}
    L = _lib.load()
    statuses = set(range(len(_lib.STATUS_NAMES)))
    for name, params in sorted(decls.items()):
        if name.endswith("_destroy") or name.endswith("_default") or name == "bg_last_error_string":
            continue
        for with_handles in (False, True):
            args, types = [], []
            for i, p in enumerate(params):
                ptype = p.rsplit("*", 1)[0] + "*" if "*" in p else p
                if i == 0 and with_handles and ptype in handles:
                    args.append(ctypes.c_void_p(handles[ptype].value if hasattr(handles[ptype], "value")
                                                else handles[ptype]))
                    types.append(ctypes.c_void_p)
                elif "*" in p:
                    args.append(None)
                    types.append(ctypes.c_void_p)
                elif p.startswith("double"):
                    args.append(0.0)
                    types.append(ctypes.c_double)
                else:
                    args.append(0)
                    types.append(ctypes.c_long if p.startswith(("long", "size_t")) else ctypes.c_int)
            f = getattr(L, name)
            saved = (f.argtypes, f.restype)
            f.argtypes, f.restype = types, ctypes.c_int
            try:
                st = f(*args)
            finally:
                f.argtypes, f.restype = saved
            assert st in statuses, (name, with_handles, st)
            if not with_handles:
                assert st == _lib.BG_INVALID_ARG, name


def test_quadrature_counts(bg_host):
    """Near-field quadrature work on the host: every element pair of the dense
    leaves is counted once, evaluations follow the reference's rules."""
    bg, ctx = bg_host
    d = bg.DiscreteOperator(bg.AnsatzSpace(bg.Geometry(SPHERE, ctx), 2, 1), bg.LaplaceSingleLayerOperator())
    info = d.info()
    c = d.quadrature_counts()
    pairs = sum(v["pairs"] for v in c.values())
    assert pairs == int(info[3]) * int(info[11]) ** 2
    assert c["identical"]["pairs"] == d.ne
    for name, per in (("identical", 8), ("edge", 6), ("vertex", 4)):
        if c[name]["pairs"]:
            q4 = c[name]["evaluations"] // (per * c[name]["pairs"])
            assert q4 * per * c[name]["pairs"] == c[name]["evaluations"] and round(q4 ** 0.25) ** 4 == q4


def test_cube_sphere_patches(bg_host, oracle):
    """The analytic cube sphere: points on the unit sphere, derivatives equal
    to central differences, outward normals, surface area 4 pi by Gauss
    quadrature, faces meeting along the cube edges, and the same frames as the
    oracle's restatement."""
    bg, ctx = bg_host
    g = bg.Geometry.cube_sphere(ctx)
    o = oracle.Problem(CUBE, 0, 0, oracle.LAPLACE, np_=6, assemble=False)
    rng = np.random.default_rng(11)
    h = 1e-6
    for _ in range(60):
        p, s, t = int(rng.integers(6)), rng.uniform(0.01, 0.99), rng.uniform(0.01, 0.99)
        f = g.surface_point(p, s, t)
        x, dx, dy = f[3:6], f[6:9], f[9:12]
        assert abs(np.linalg.norm(x) - 1.0) < 1e-15
        fd_s = (g.surface_point(p, s + h, t)[3:6] - g.surface_point(p, s - h, t)[3:6]) / (2 * h)
        fd_t = (g.surface_point(p, s, t + h)[3:6] - g.surface_point(p, s, t - h)[3:6]) / (2 * h)
        assert np.abs(fd_s - dx).max() < 1e-8 and np.abs(fd_t - dy).max() < 1e-8
        assert np.dot(np.cross(dx, dy), x) > 0
        assert np.abs(f[3:] - o.surface_point(p, s, t)[3:]).max() < 1e-15
    xg, wg = np.polynomial.legendre.leggauss(24)
    xg, wg = (xg + 1) / 2, wg / 2
    area = 0.0
    for p in range(6):
        for s, ws in zip(xg, wg):
            for t, wt in zip(xg, wg):
                f = g.surface_point(p, s, t)
                area += ws * wt * np.linalg.norm(np.cross(f[6:9], f[9:12]))
    assert abs(area - 4 * np.pi) < 1e-9
    # every patch corner is a cube corner direction, shared by three faces
    corners = {}
    for p in range(6):
        for s, t in ((0, 0), (1, 0), (1, 1), (0, 1)):
            key = tuple(np.round(g.surface_point(p, s, t)[3:6] * np.sqrt(3), 12))
            corners[key] = corners.get(key, 0) + 1
    assert len(corners) == 8 and set(corners.values()) == {3}
    # analytic patches have no control points to hand out
    import ctypes
    px, py = ctypes.c_int(), ctypes.c_int()
    st = bg._lib.load().bg_geometry_patch_data(g.h, 0, ctypes.byref(px), ctypes.byref(py), None)
    assert st == bg._lib.BG_UNSUPPORTED


def test_batched_wavenumbers_host_only(bg_host):
    """On a host-only context the batched-wavenumber entry points refuse to
    assemble (no device), and an operator holds no wavenumber slots."""
    from bembel_gb300 import BembelError
    bg, ctx = bg_host
    lin = bg.HelmholtzSingleLayerOperator()
    lin.set_wavenumber(1.0)
    d = bg.DiscreteOperator(bg.AnsatzSpace(bg.Geometry(SPHERE, ctx), 1, 1), lin, n_p=4)
    assert len(d.wavenumbers()) == 0
    with pytest.raises(BembelError):
        d.assemble_wavenumbers()
    d.release_wavenumbers()  # nothing to release: a no-op
    assert len(d.wavenumbers()) == 0
