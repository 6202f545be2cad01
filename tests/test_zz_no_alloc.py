"""bg_matvec_noalloc: the single-right-hand-side H2 product that allocates no
device memory, for callers that may not call cudaMalloc when they need a
product (fixed memory budgets, pooled allocators, serving loops that forbid
allocation after warm-up).

Checked through the C ABI against bg_matvec (the existing entry point) on two
calls in a row with different inputs, FP64 to 1e-12 and mixed precision to
1e-5 relative (the tolerances of the other product tests). Device free memory
must not change across calls once the first call on the device has looked up
the fixed scratch array. An operator whose intermediate vectors exceed the
16 MiB array is rejected with BG_INVALID_ARG and a message naming the size.

This file is collected after the other product tests on purpose; it must
also pass alone.
"""
import ctypes

import numpy as np
import pytest

from conftest import SPHERE

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
FP32_TOL = 1e-5


def _entry():
    from bembel_gb300 import _lib
    f = _lib.load().bg_matvec_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    return f


@pytest.fixture(scope="module")
def ctx():
    import bembel_gb300 as bg
    return bg.Context(0)


def _operator(ctx, M, P, kind, kappa=0.0, np_=9, assemble=True, keep_fp64_blocks=True):
    import bembel_gb300 as bg
    lin = bg.LaplaceSingleLayerOperator() if kind == 0 else bg.HelmholtzSingleLayerOperator()
    if kind == 1:
        lin.set_wavenumber(kappa)
    d = bg.DiscreteOperator(bg.AnsatzSpace(bg.Geometry(SPHERE, ctx), M, P), lin, n_p=np_,
                            keep_fp64_blocks=keep_fp64_blocks)
    if assemble:
        d.compute()
    return d


def _noalloc(ctx, d, x_dev, y_dev, precision):
    import torch
    from bembel_gb300 import _lib
    torch.cuda.synchronize()  # x was written on torch's stream; the library uses its own
    st = _entry()(d.h, ctypes.c_void_p(x_dev.data_ptr()), ctypes.c_void_p(y_dev.data_ptr()), precision)
    ctx.check(st)
    assert st == _lib.BG_OK
    return y_dev.cpu().numpy()


@pytest.mark.parametrize("M,P,kind,kappa", [(3, 2, 0, 0.0), (2, 1, 1, 2.0)])
def test_noalloc_matches_matvec_twice(ctx, M, P, kind, kappa):
    import torch
    from bembel_gb300 import _lib
    d = _operator(ctx, M, P, kind, kappa)
    A = d.get_discrete_operator()
    rng = np.random.default_rng(11)
    dtype = torch.complex128 if d.is_complex else torch.float64
    for precision, name, tol in ((_lib.PREC_FP64, "fp64", FP64_TOL), (_lib.PREC_MIXED, "mixed", FP32_TOL)):
        y_dev = torch.empty(d.N, dtype=dtype, device="cuda:0")
        for call in range(2):
            x = rng.uniform(-1, 1, d.N)
            if d.is_complex:
                x = x + 1j * rng.uniform(-1, 1, d.N)
            x_dev = torch.from_numpy(x).to("cuda:0")
            torch.cuda.synchronize()
            free_before = torch.cuda.mem_get_info(0)[0]
            y = _noalloc(ctx, d, x_dev, y_dev, precision)
            free_after = torch.cuda.mem_get_info(0)[0]
            if call == 1:
                # the scratch address is looked up on the first call of the
                # process; from then on a call takes no device memory at all
                assert free_after == free_before, (free_before, free_after)
            ref = A.matvec(x.reshape(-1, 1), precision=name).reshape(-1)
            err = np.linalg.norm(y - ref) / np.linalg.norm(ref)
            assert err < tol, (name, call, err)


def test_noalloc_rejects_operators_beyond_scratch(ctx):
    import torch
    from bembel_gb300 import _lib
    # sphere, M = 7, P = 1: about 48 MB of intermediate vectors, above 16 MiB.
    # The size check comes before any device work, so the operator is not assembled.
    d = _operator(ctx, 7, 1, 0, assemble=False)
    x_dev = torch.zeros(d.N, dtype=torch.float64, device="cuda:0")
    y_dev = torch.zeros(d.N, dtype=torch.float64, device="cuda:0")
    st = _entry()(d.h, ctypes.c_void_p(x_dev.data_ptr()), ctypes.c_void_p(y_dev.data_ptr()), _lib.PREC_FP64)
    assert st == _lib.BG_INVALID_ARG
    msg = _lib.load().bg_last_error_string(ctx.h).decode()
    assert "scratch" in msg and "16 MiB" in msg, msg


@pytest.mark.parametrize("kind,kappa", [(0, 0.0), (1, 2.0)])
def test_noalloc_fp64_without_fp64_blocks(ctx, kind, kappa):
    """An operator assembled with keep_fp64_blocks=False (as the serving cache
    builds them) has released its FP64 coupling blocks; the FP64 product then
    runs on their double-float copies, as bg_matvec does."""
    import torch
    from bembel_gb300 import _lib
    d = _operator(ctx, 3, 2, kind, kappa, keep_fp64_blocks=False)
    A = d.get_discrete_operator()
    rng = np.random.default_rng(12)
    dtype = torch.complex128 if d.is_complex else torch.float64
    y_dev = torch.empty(d.N, dtype=dtype, device="cuda:0")
    for call in range(2):
        x = rng.uniform(-1, 1, d.N)
        if d.is_complex:
            x = x + 1j * rng.uniform(-1, 1, d.N)
        y = _noalloc(ctx, d, torch.from_numpy(x).to("cuda:0"), y_dev, _lib.PREC_FP64)
        ref = A.matvec(x.reshape(-1, 1), precision="fp64").reshape(-1)
        err = np.linalg.norm(y - ref) / np.linalg.norm(ref)
        assert err < FP64_TOL, (call, err)

