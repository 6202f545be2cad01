"""Benchmark: batched H2 single-layer solves on one GB300.

Workload (one "step"): the Laplace single-layer Galerkin system on the
6-patch NURBS sphere (sphere.dat), refinement M = 5 (6144 elements), B-spline
degree P = 2 (6936 DOFs), interpolation n_p = 9, eta = 1.6, with 32 right-hand
sides from seeded point sources |x0| ~ U[1.5, 3] (uniform directions): one
batched solve of all 32 systems to rel. residual 1e-8. The operator is
assembled once before the timed region (as DiscreteOperator::compute in the
reference) and reused by every solve.

value:  solves/s = right-hand sides solved to 1e-8 per second: FP64 flexible
        GMRES over the FP64 H2 matrix, preconditioned by an inner GMRES (tol
        2e-3) on the mixed operator: near field at FP64 accuracy, far field
        on the tensor cores from FP16 hi/lo splits with FP32 accumulation
        (--inner mixed, the default; --inner fp32 also puts the near field in
        FP32, which goes beyond the mixed form of the workload definition).
        Operands in HBM. Every solve meets 1e-8 in the FP64 relative residual
        ||b - A x|| / ||b|| of every column.
e2e:    the same through the public C ABI with host (pinned) buffers, the
        host->device copy of b and device->host copy of x inside each step.
Also reported: the plain FP64 GPU solve, H2 matvec/s (FP64 and mixed),
p50/p99 step latency, assembly time, accuracy vs FP64 and vs the analytic
point-source potential, the roofline of the dominant kernel and the CPU
baseline (the CPU oracle, which restates the reference algorithm).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
GEO = os.path.join(ROOT, "tests", "golden", "geo", "sphere.dat")
M, P, NP, NRHS = 5, 2, 9, 32
TOL = 1e-8
INNER_TOL = 2e-3  # relative tolerance of each inner (preconditioning) solve; the library default
METRIC = "solves/s (32-RHS batched Laplace SL H2 solves to rel.err 1e-8, mixed precision)"
# FP32 FMA throughput of one GB300 measured with an FMA-chain probe (TFLOP/s)
FP32_FMA_TFLOPS = 75.0
# DRAM bytes (read + write) per low-rank block of k_far_h16, from one ncu
# capture of the same kernel on the M=4 sphere (512.2 MB read + 7.2 MB
# written for 17 616 blocks: 29 484 bytes per block against 28 496 bytes of
# stored tiles and edge couplings; the rest is right-hand-side tiles missing
# L2 and the output)
FAR_TILE_DRAM_BYTES_PER_BLOCK = (512.184e6 + 7.199e6) / 17616
INNER_DESC = {"mixed": "inner GMRES(near field FP64-accurate (tensor cores, 8 integer digits per operand, exact "
                       "integer sums), far field FP16 hi/lo tensor cores, FP32 accumulation)",
              "fp32": "inner GMRES(near field FP32, far field FP16 hi/lo tensor cores, FP32 accumulation)"}


def workload_config(extra=None):
    cfg = {"workload": "laplace_sl_h2_sphere_M5_P2_np9_32rhs", "geometry": "sphere.dat (6 NURBS patches)",
           "elements": 6144, "dofs": 6936, "refinement": M, "degree": P, "n_p": NP, "eta": 1.6, "nrhs": NRHS,
           "tol": TOL, "rhs": "point sources |x0|~U[1.5,3], seed 3",
           "l2": "flush: 256 MiB buffer written between timed steps; operator data (near field 175 MB) > L2",
           "solver": "FGMRES(FP64 H2) preconditioned by an inner GMRES(2e-3) on a low-precision operator"}
    if extra:
        cfg.update(extra)
    return cfg


def rhs_points():
    rng = np.random.default_rng(3)
    d = rng.normal(size=(NRHS, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rho = rng.uniform(1.5, 3.0, (NRHS, 1))
    return d * rho


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                vals = [v.strip() for v in out.stdout.strip().split(",")]
                if len(vals) == 6:
                    self.samples.append(vals)
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no nvidia-smi samples"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[2 + i].strip() == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


# ---------------------------------------------------------------------------
# CG iterations of one 1-RHS solve of this workload to 1e-8 (right-hand side
# 0), measured by the reference arm's complete solve on the GB300 host
CG_ITERS_C2 = 335
CG_SAMPLE_ITERS = 16  # CG iterations per timed CPU step


def cpu_sample(op, seconds=15.0):
    """CPU baseline of the GPU line, on a bounded sample of the workload.

    The oracle (the reference's OpenMP H2 product and CG solver, restated)
    gets the GPU-assembled operator's leaf matrices (equal to the oracle's own
    assembly to 1e-12; the CPU assembly alone takes over a minute, and the
    metric excludes assembly). Then steps of CG_SAMPLE_ITERS CG iterations of
    a 1-RHS solve run for about `seconds`; solves/s = 1 / (CG_ITERS_C2 x the
    measured time per iteration)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    t0 = time.time()
    p = oracle.Problem(GEO, M, P, oracle.LAPLACE, np_=NP, assemble=False)
    for li in range(p.n_leaves):
        p.set_leaf_matrix(li, op.leaf_block(li))
    t_load = time.time() - t0
    b = p.load_vector(0, rhs_points()[0])
    p.matvec(b)  # warm-up
    times = []
    t1 = time.time()
    while len(times) < 3 or time.time() - t1 < seconds:
        t2 = time.perf_counter()
        p.cg(b, tol=0.0, maxit=CG_SAMPLE_ITERS)
        times.append(time.perf_counter() - t2)
    t_iter = float(np.sum(times)) / (len(times) * CG_SAMPLE_ITERS)
    return {"value": 1.0 / (CG_ITERS_C2 * t_iter), "unit": "solves/s", "cores": oracle.threads(), "kind": "port",
            "sample": ("CPU oracle (restates the reference OpenMP H2 product and its CG solver) on the GPU-assembled "
                       "leaves (copied in %.1f s): %d x %d CG iterations timed, %.2f ms per iteration; solve = %d "
                       "iterations (measured by the reference arm's complete solve); bench.py --impl reference "
                       "measures the same with the CPU's own assembly"
                       % (t_load, len(times), CG_SAMPLE_ITERS, 1e3 * t_iter, CG_ITERS_C2))}


def cpu_reference_setup():
    """The CPU path of the reference on this workload, restated by the oracle:
    full H2 assembly (DiscreteOperator<H2Matrix<double>, LaplaceSingleLayerOperator>::compute,
    OpenMP over leaves) and the load vectors of the 32 point sources."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    t0 = time.time()
    p = oracle.Problem(GEO, M, P, oracle.LAPLACE, np_=NP)
    t_asm = time.time() - t0
    x0 = rhs_points()
    b = [p.load_vector(0, x0[c]) for c in range(NRHS)]
    return oracle, p, b, t_asm


def run_reference(args):
    """Reference arm: the reference's CPU solve of this workload, timed.

    Setup (untimed, reported): the full H2 assembly on all host cores, then
    one complete 1-RHS solve to 1e-8 with the reference's solver for the
    Laplace single layer, conjugate gradients without preconditioner
    (examples/LaplaceSingleLayerH2.cpp:77-80), which measures the iterations
    per solve I and the full solve time. Each iteration is one 1-RHS H2 product
    with the reference's OpenMP structure (H2DenseProduct.hpp:33-165) plus the
    CG vector updates. Warm-up steps are single untimed H2 products. Each timed
    step runs CG_SAMPLE_ITERS iterations of a fresh 1-RHS solve (right-hand
    side k + 1 mod 32), so K steps fit in minutes although one solve takes
    about 20 s. value = 1 / (I x measured time per iteration): right-hand
    sides solved per second, the unit of the GPU arm; both factors are measured
    in this run, the full solve beside them as a check."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    t0 = time.time()
    oracle, p, b, t_asm = cpu_reference_setup()
    t1 = time.perf_counter()
    _, iters, relres = p.cg(b[0], tol=TOL)
    full_s = time.perf_counter() - t1
    for _ in range(max(0, args.warmup)):
        p.matvec(b[0])
    steps = max(1, args.steps)
    times = []
    for k in range(steps):
        t1 = time.perf_counter()
        p.cg(b[(k + 1) % NRHS], tol=0.0, maxit=CG_SAMPLE_ITERS)
        times.append(time.perf_counter() - t1)
    total = float(np.sum(times))
    t_iter = total / (steps * CG_SAMPLE_ITERS)
    value = 1.0 / (iters * t_iter)
    cores = oracle.threads()
    sample = ("measured: CPU oracle (restates the reference OpenMP H2 path and its CG solver), full assembly %.1f s "
              "(untimed setup); %d timed steps of %d CG iterations on the assembled operator, %.2f ms per "
              "iteration; iterations per 1-RHS solve to 1e-8 measured by a complete solve in the same run: %d "
              "(%.2f s, final rel. residual %.1e)"
              % (t_asm, steps, CG_SAMPLE_ITERS, 1e3 * t_iter, iters, full_s, relres))
    line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": args.gpus,
            "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / steps,
            "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded point sources on sphere.dat)",
            "impl": "reference", "config": workload_config({"parallelism": "cpu openmp",
                                                            "solver": "CG, no preconditioner (reference example)",
                                                            "step": "%d CG iterations of a 1-RHS solve"
                                                                    % CG_SAMPLE_ITERS}),
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "setup_s": {"assembly": t_asm, "full_solve": full_s},
            "full_solve": {"iterations": iters, "seconds": full_s, "solves_per_s": 1.0 / full_s,
                           "final_relres": relres},
            "note": "the reference needs Eigen, absent here and on the GPU box; the CPU oracle port stands in",
            "wall_s": time.time() - t0}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def aggregate_replicas(total_ms, dist=None, device="cuda"):
    """Whole-job time of N independent replicas: the maximum over the ranks of
    their timed totals (the job is as slow as its slowest replica)."""
    if dist is None or dist.get_world_size() <= 1:
        return total_ms
    import torch
    t = torch.tensor([total_ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def col_rel_err(a, ref):
    """Largest column-wise relative error ||a_c - ref_c|| / ||ref_c|| (numpy arrays, N x k)."""
    a, ref = np.asarray(a).reshape(ref.shape[0], -1), np.asarray(ref).reshape(ref.shape[0], -1)
    return float(np.max(np.linalg.norm(a - ref, axis=0) / np.linalg.norm(ref, axis=0)))


def replica_value(nrhs, steps, world, total_ms):
    """solves/s of the whole job: every replica solves nrhs right-hand sides per step."""
    return world * nrhs * steps / (total_ms * 1e-3)


def run_gpu(args):
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import bembel_gb300 as bg
    from bembel_gb300 import _lib
    L = _lib.load()
    ctx = bg.Context(local)
    sp = ctypes_void_p()
    L.bg_context_get_stream(ctx.h, ctypes_byref(sp))
    stream = torch.cuda.ExternalStream(sp.value, device=torch.device("cuda", local))

    t0 = time.time()
    op = bg.DiscreteOperator(bg.AnsatzSpace(bg.Geometry(GEO, ctx), M, P), bg.LaplaceSingleLayerOperator(), n_p=NP)
    op.compute()
    asm = op.assembly_times()
    asm["wall_s"] = time.time() - t0
    quad = op.quadrature_counts()
    # launch plans of the 32-column products: built-in, or timed by the
    # library's autotuner (outside the timed region)
    plans = {"launch_plans": "built-in"}
    if args.autotune:
        plans = {"launch_plans": {p: op.autotune(NRHS, p) for p in ("fp32", "mixed")}}
    A = op.get_discrete_operator()
    N = op.N
    x0 = rhs_points()
    b_host = op.load_vector(0, x0)                      # (N, 32) float64, Fortran order
    b_dev = torch.from_numpy(np.ascontiguousarray(b_host.T)).cuda()  # (32, N) = column-major N x 32
    b_dev_t = b_dev.t()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def solve(inner, b):
        return A.solve(b, tol=TOL, inner=inner, inner_tol=INNER_TOL, restart=200, max_refinements=12)

    # FP64 GPU path (reference solution for the accuracy report), outside the timed region
    x64, st64 = solve("fp64", b_dev_t)
    ev = lambda: torch.cuda.Event(enable_timing=True)

    def timed_steps(inner, b, steps, warmup, profile=False):
        for _ in range(warmup):
            solve(inner, b)
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        times, stats = [], None
        if profile:
            # inside the timed region only the dominant kernel class is bracketed
            # with events (one pair per product); launches are counted for all
            L.bg_profile_classes(ctx.h, 1 << CLASSES.index("far_fused_fp32"))
            L.bg_profile_enable(ctx.h, 1)
            _read_profile(L, ctx)  # reset counters
        for _ in range(steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            e0, e1 = ev(), ev()
            e0.record(stream)
            x, stats = solve(inner, b)
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        torch.cuda.synchronize()
        prof = _read_profile(L, ctx) if profile else None
        if profile:
            L.bg_profile_enable(ctx.h, 0)
        if dist:
            dist.barrier()
        return np.array(times), x, stats, prof

    def class_breakdown(inner, b):
        """Device time per kernel class of one untimed solve, every class bracketed."""
        L.bg_profile_classes(ctx.h, 0xFF)
        L.bg_profile_enable(ctx.h, 1)
        _read_profile(L, ctx)
        solve(inner, b)
        prof = _read_profile(L, ctx)
        L.bg_profile_enable(ctx.h, 0)
        return prof

    inner = args.inner
    other = "mixed" if inner == "fp32" else "fp32"
    clocks = ClockSampler(local)
    with clocks:
        t_mixed, xm, stm, prof = timed_steps(inner, b_dev_t, args.steps, args.warmup, profile=True)
    breakdown = class_breakdown(inner, b_dev_t)
    t_fp64, _, _, _ = timed_steps("fp64", b_dev_t, max(1, min(2, args.steps)), 1)
    t_other, _, st_other, _ = timed_steps(other, b_dev_t, max(1, min(2, args.steps)), 1)
    # the mixed form with the far field from the FP16 hi coupling tiles only
    # (launch plan far_tiles = 1: half the bytes, about 11 bits per coupling)
    op.set_plan(NRHS, "mixed", far_tiles=1)
    t_hi, x_hi, st_hi, _ = timed_steps("mixed", b_dev_t, max(1, min(2, args.steps)), 1)
    op.set_plan(NRHS, "mixed")
    # end to end: host pinned b, host x, copies inside the step
    b_pin = torch.from_numpy(np.ascontiguousarray(b_host.T)).pin_memory()
    t_e2e, xe, _, _ = timed_steps(inner, b_pin.t(), args.steps, 1)

    # matvec throughput (32 RHS per product)
    def mv_rate(prec, reps=5):
        x = torch.randn(N, NRHS, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        for _ in range(2):
            A.matvec(x, precision=prec)
        torch.cuda.synchronize()
        e0, e1 = ev(), ev()
        e0.record(stream)
        for _ in range(reps):
            A.matvec(x, precision=prec)
        e1.record(stream)
        e1.synchronize()
        return reps / (e0.elapsed_time(e1) * 1e-3)
    mv64, mvmx, mv32 = mv_rate("fp64"), mv_rate("mixed"), mv_rate("fp32")
    # product error of the low-precision operators against the FP64 product
    xr = torch.randn(N, NRHS, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()  # the library reads xr on its own (non-blocking) stream
    y_ref = A.matvec(xr, precision="fp64").cpu().numpy()
    mv_err = {p: col_rel_err(A.matvec(xr, precision=p).cpu().numpy(), y_ref) for p in ("mixed", "fp32")}

    total_ms = aggregate_replicas(float(t_mixed.sum()), dist)
    value = replica_value(NRHS, args.steps, world, total_ms)
    fp64_value = NRHS / (float(np.mean(t_fp64)) * 1e-3)
    e2e_value = NRHS / (float(np.mean(t_e2e)) * 1e-3)

    # both solvers driven to 1e-12: what remains of the solution difference
    # once the stopping tolerance no longer dominates it
    x64_12, st64_12 = A.solve(b_dev_t, tol=1e-12, inner="fp64", restart=200, max_refinements=12)
    xm_12, stm_12 = A.solve(b_dev_t, tol=1e-12, inner=inner, inner_tol=INNER_TOL, restart=200, max_refinements=20)
    diff_12 = col_rel_err(xm_12.cpu().numpy(), x64_12.cpu().numpy())

    # accuracy: mixed vs FP64 solution, and potential error vs the analytic point source
    xm_np = xm.cpu().numpy() if hasattr(xm, "cpu") else xm
    x64_np = x64.cpu().numpy() if hasattr(x64, "cpu") else x64
    rel_vs_fp64 = col_rel_err(xm_np, x64_np)
    rng = np.random.default_rng(2)
    pts = rng.normal(size=(100, 3))
    pts = pts / np.linalg.norm(pts, axis=1, keepdims=True) * (0.25 * rng.uniform(0, 1, (100, 1)) ** (1 / 3))
    pot = op.potential(xm_np, pts)
    ref = 1.0 / (4 * np.pi * np.linalg.norm(pts[:, None, :] - x0[None, :, :], axis=2))
    pot_err = float(np.max(np.abs(pot - ref)) / np.max(np.abs(ref)))
    pot64_err = float(np.max(np.abs(op.potential(x64_np, pts) - ref)) / np.max(np.abs(ref)))

    if rank != 0:
        return
    roof = _roofline(op, prof, stm, args.steps)
    line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32",
            "data": "synthetic (seeded point sources, sphere.dat geometry)",
            "config": workload_config({"parallelism": "replicas x%d" % world if world > 1 else "single gpu",
                                       "inner_operator": INNER_DESC[inner], **plans}),
            "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": int(N * NRHS * 8),
                    "d2h_bytes_per_step": int(N * NRHS * 8)},
            "gpu_launches": int(prof["launches_total"]) if prof else None,
            "roofline": roof, "clocks": clocks.summary(),
            "latency_ms": {"p50": float(np.percentile(t_mixed, 50)), "p99": float(np.percentile(t_mixed, 99))},
            "fp64_path": {"solves_per_s": fp64_value, "ms_per_step": float(np.mean(t_fp64)),
                          "iterations": st64["iterations"]},
            "mixed_over_fp64": value / world / fp64_value,
            "arms": {
                inner: {"solves_per_s": value / world, "over_fp64": value / world / fp64_value,
                        "operator": INNER_DESC[inner], "within_workload_mixed_form": inner == "mixed",
                        "iterations": stm["iterations"], "refinements": stm["refinements"]},
                other: {"solves_per_s": NRHS / (float(np.mean(t_other)) * 1e-3),
                        "over_fp64": NRHS / (float(np.mean(t_other)) * 1e-3) / fp64_value,
                        "operator": INNER_DESC[other], "within_workload_mixed_form": other == "mixed",
                        "iterations": st_other["iterations"], "refinements": st_other["refinements"]},
                "mixed_far_hi": {"solves_per_s": NRHS / (float(np.mean(t_hi)) * 1e-3),
                                 "over_fp64": NRHS / (float(np.mean(t_hi)) * 1e-3) / fp64_value,
                                 "operator": "inner GMRES(near field as in mixed, far field from the FP16 hi "
                                             "coupling tiles only (launch plan far_tiles = 1), FP32 accumulation)",
                                 "within_workload_mixed_form": True,
                                 "iterations": st_hi["iterations"], "refinements": st_hi["refinements"],
                                 "final_relres": st_hi["final_relres"],
                                 "solution_vs_fp64": col_rel_err(x_hi.cpu().numpy(), x64.cpu().numpy())}},
            "solver": {k: stm[k] for k in ("iterations", "refinements", "fp64_matvecs", "low_matvecs",
                                            "final_relres")},
            "accuracy": {"criterion": "every column stops at FP64 relative residual ||b - A x|| / ||b|| <= 1e-8 "
                                      "(A the FP64 H2 matrix); solution errors are reported beside it",
                         "mixed_final_relres": stm["final_relres"],
                         "mixed_vs_fp64_solution": rel_vs_fp64,
                         "mixed_vs_fp64_solution_both_at_1e-12": diff_12,
                         "relres_at_1e-12": {"fp64": st64_12["final_relres"], "mixed": stm_12["final_relres"]},
                         "potential_vs_analytic": pot_err,
                         "fp64_potential_vs_analytic": pot64_err, "fp64_final_relres": st64["final_relres"],
                         "mixed_matvec_vs_fp64": mv_err["mixed"], "fp32_matvec_vs_fp64": mv_err["fp32"]},
            "matvec": {"fp64_products_per_s_32rhs": mv64, "mixed_products_per_s_32rhs": mvmx,
                       "fp32_products_per_s_32rhs": mv32, "fp64_matvec_per_s": mv64 * NRHS,
                       "mixed_matvec_per_s": mvmx * NRHS, "fp32_matvec_per_s": mv32 * NRHS},
            "assembly_s": asm,
            "assembly_roofline": assembly_roofline(quad, asm["near_s"], P, fp64_peak_tflops()),
            "kernel_ms_per_solve": {k: round(v, 3) for k, v in breakdown["ms"].items()},
            "kernel_launches_per_solve": breakdown["launches"]}
    if world == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_sample(op)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def class_breakdown(L, ctx, fn):
    """Device time and launches per kernel class of fn(), every class bracketed."""
    L.bg_profile_classes(ctx.h, 0xFF)
    L.bg_profile_enable(ctx.h, 1)
    _read_profile(L, ctx)
    fn()
    prof = _read_profile(L, ctx)
    L.bg_profile_enable(ctx.h, 0)
    return {"ms": {k: round(v, 3) for k, v in prof["ms"].items() if v},
            "launches": {k: v for k, v in prof["launches"].items() if v}}


CLASSES = ["near_fp64", "far_fp64", "far_fused_fp32", "transforms", "t_apply", "krylov", "other", "assembly"]


def _read_profile(L, ctx):
    import ctypes
    ms = (ctypes.c_double * 8)()
    ln = (ctypes.c_long * 8)()
    L.bg_profile_read(ctx.h, ms, ln)
    return {"ms": {CLASSES[i]: ms[i] for i in range(8)}, "launches": {CLASSES[i]: ln[i] for i in range(8)},
            "launches_total": sum(ln[i] for i in range(8))}


def near_flops_per_evaluation(P):
    """FP64 flops of one near-field integrand evaluation of a real scalar
    kernel (Laplace), the minimal work of the reference's evaluateIntegrand
    (Laplace/SingleLayerOperator.hpp:44-85 and its basis interaction,
    AnsatzSpace/SuperSpace.hpp:173-178): the kernel value 1/(4 pi r) times the two
    weights (3 differences, r^2 by one multiply and two FMAs, reciprocal
    square root and scaling: 14 flops) and the rank-one update of the
    (P+1)^2 x (P+1)^2 element-pair block, one multiply and one FMA per
    entry (3 (P+1)^4 flops). Surface points, measures and basis values are
    not counted: they can be shared between samples (the kernels share
    most of them)."""
    return 3 * (P + 1) ** 4 + 14


def fp64_peak_tflops():
    """Measured FP64 rate of this GPU: cuBLAS DGEMM (torch.matmul, 4096^3,
    best of 5, CUDA events)."""
    import torch
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    best = None
    for _ in range(6):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        best = ms if best is None else min(best, ms)
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


def assembly_roofline(quad, near_s, P, peak):
    """Near-field assembly against the FP64 pipe: integrand evaluations of the
    reference's rules (bg_operator_quadrature_counts: regular pairs
    integrate0/1, identical integrate2, common edge integrate3, common vertex
    integrate4) x near_flops_per_evaluation(P), over the near-field assembly
    time (all rules, one launch sequence)."""
    evals = sum(v["evaluations"] for v in quad.values())
    fpe = near_flops_per_evaluation(P)
    tf = evals * fpe / near_s / 1e12
    return {"bound": "fp64", "evaluations": {k: v["evaluations"] for k, v in quad.items()},
            "pairs": {k: v["pairs"] for k, v in quad.items()}, "near_s": near_s,
            "evaluations_per_s": evals / near_s, "fp64_flops_per_evaluation": fpe,
            "achieved": tf, "peak": peak, "unit": "TFLOP/s", "frac": tf / peak,
            "peak_source": "cuBLAS DGEMM 4096^3 on this GPU (torch.matmul float64, best of 5)"}


def far_tile_bytes(np2):
    """Bytes of one low-rank block as stored for the tensor-core far field:
    FP16 hi + lo tiles of row groups of 8 targets x K sources (K = n_p^2
    rounded down to 16 when n_p^2 >= 16, else up to 8), then the remaining
    source columns as FP32 couplings (rounded up to 16 bytes)."""
    mg = (np2 + 7) // 8
    if np2 >= 16:
        km = np2 // 16 * 16
        edge = ((np2 - km) * np2 * 4 + 15) // 16 * 16
    else:
        km, edge = (np2 + 7) // 8 * 8, 0
    return 2 * mg * 8 * km * 2 + edge


def far_algorithmic_bytes(np2):
    """Algorithmic bytes of one low-rank block in the tensor-core product:
    (n_p^2)^2 couplings x 4 bytes (FP16 hi + lo), no padding."""
    return np2 * np2 * 4


def _roofline(op, prof, stats, steps):
    """Roofline of the dominant kernel class of the timed solves.

    achieved = algorithmic bytes (or flops) of the class over the timed region
    / its summed CUDA-event time on the library stream (= per launch figure /
    average launch time)."""
    import json as _j
    if not prof:
        return None
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peaks = _j.load(open(peaks_path)) if os.path.exists(peaks_path) else {}
    hbm = peaks.get("hbm_gbs", 6800.0)
    src = "measured (MEASURED_PEAKS.json)" if peaks else "fallback"
    cls = max(prof["ms"], key=lambda k: prof["ms"][k])
    n = max(1, prof["launches"][cls])
    ms = prof["ms"][cls]
    t = ms * 1e-3 / n  # seconds per launch
    info = op.info()
    nlow = float(info[4])
    block_entries = float(info[7]) ** 4  # (n_p^2)^2 couplings per low-rank block
    base = {"kernel_class": cls, "launches": n, "avg_launch_ms": t * 1e3, "class_ms": ms}
    if cls == "near_fp64":
        algo = float(info[14])  # stored FP64 near-field blocks, streamed once per launch
        ach = algo / t / 1e9
        base.update({"kernel": "k_bsr_pipe (near-field block-sparse product, 32 RHS)", "bound": "hbm",
                     "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm, "traffic": None,
                     "peak_source": src, "algorithmic_bytes_per_launch": algo})
        return base
    if cls == "far_fused_fp32":
        # k_far_h16: one launch per product streams the split operand
        # tiles of every low-rank block once (TMA bulk copies) into tcgen05.mma
        np2 = int(info[7]) ** 2
        tile = far_tile_bytes(np2)
        algo = nlow * far_algorithmic_bytes(np2)
        ach = algo / t / 1e9
        traffic = nlow * FAR_TILE_DRAM_BYTES_PER_BLOCK
        base.update({"kernel": "k_far_h16 (stored scaled FP16 hi/lo tiles, TMA bulk copy -> tcgen05.mma, 32 RHS)",
                     "bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                     "traffic": traffic, "peak_source": src,
                     "algorithmic_bytes_per_launch": algo,
                     "algorithmic_bytes_rule": "low-rank blocks x (n_p^2)^2 couplings x 4 B (FP16 hi + lo), unpadded",
                     "stored_bytes_per_block": tile, "traffic_over_algorithmic": traffic / algo,
                     "stored_tiles_gbs": nlow * tile / t / 1e9,
                     "contraction_tflops": 2.0 * nlow * block_entries * NRHS / t / 1e12})
        return base
    base.update({"bound": None, "achieved": None, "peak": None, "unit": None, "frac": None, "traffic": None})
    return base


def run_maxwell(args):
    """Side workload (not the headline line): the Maxwell single layer (EFIE)
    on the sphere, M = 4, P = 2, n_p = 9, kappa = 2, with 8 right-hand sides
    from Hertz dipoles at distance 2.5 with seeded random orientations (seed 6),
    excitation = tangential trace. Reports batched solves/s to 1e-8 with the
    FP32 inner operator and with the plain FP64 path, H2 products/s, the
    assembly time and the mixed-vs-FP64 solution difference."""
    import torch
    import bembel_gb300 as bg
    from bembel_gb300 import _lib
    L = _lib.load()
    ctx = bg.Context(0)
    sp = ctypes_void_p()
    L.bg_context_get_stream(ctx.h, ctypes_byref(sp))
    stream = torch.cuda.ExternalStream(sp.value, device=torch.device("cuda", 0))
    m, p, n_p, k, nrhs = 4, 2, 9, 2.0, 8
    t0 = time.time()
    lin = bg.MaxwellSingleLayerOperator()
    lin.set_wavenumber(k)
    op = bg.DiscreteOperator(bg.AnsatzSpace(bg.Geometry(GEO, ctx), m, p), lin, n_p=n_p)
    op.compute()
    asm = op.assembly_times()
    asm["wall_s"] = time.time() - t0
    A = op.get_discrete_operator()
    rng = np.random.default_rng(6)
    pos = rng.normal(size=(nrhs, 3))
    pos = 2.5 * pos / np.linalg.norm(pos, axis=1, keepdims=True)
    mom = rng.normal(size=(nrhs, 3))
    mom = mom / np.linalg.norm(mom, axis=1, keepdims=True)
    b_host = op.load_vector(3, np.hstack([pos, mom]))
    b = torch.from_numpy(np.ascontiguousarray(b_host.T)).cuda().t()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    ev = lambda: torch.cuda.Event(enable_timing=True)

    def timed(inner, steps, warmup):
        for _ in range(warmup):
            A.solve(b, tol=TOL, inner=inner, inner_tol=INNER_TOL, restart=200, max_refinements=12)
        ts, x, st = [], None, None
        for _ in range(steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            e0, e1 = ev(), ev()
            e0.record(stream)
            x, st = A.solve(b, tol=TOL, inner=inner, inner_tol=INNER_TOL, restart=200, max_refinements=12)
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        return np.array(ts), x, st

    clocks = ClockSampler(0)
    with clocks:
        t_mx, xm, stm = timed("fp32", args.steps, args.warmup)
    t_64, x64, st64 = timed("fp64", max(1, min(2, args.steps)), 1)

    def mv_rate(prec, reps=5):
        x = torch.randn(op.N, nrhs, dtype=torch.complex128, device="cuda")
        for _ in range(2):
            A.matvec(x, precision=prec)
        torch.cuda.synchronize()
        e0, e1 = ev(), ev()
        e0.record(stream)
        for _ in range(reps):
            A.matvec(x, precision=prec)
        e1.record(stream)
        e1.synchronize()
        return reps / (e0.elapsed_time(e1) * 1e-3)

    def breakdown(fn):
        L.bg_profile_classes(ctx.h, 0xFF)
        L.bg_profile_enable(ctx.h, 1)
        _read_profile(L, ctx)
        fn()
        prof = _read_profile(L, ctx)
        L.bg_profile_enable(ctx.h, 0)
        return {"ms": {kk: round(v, 3) for kk, v in prof["ms"].items() if v}, "launches":
                {kk: v for kk, v in prof["launches"].items() if v}}

    xq = torch.randn(op.N, nrhs, dtype=torch.complex128, device="cuda")
    per_product = {prec: breakdown(lambda: A.matvec(xq, precision=prec)) for prec in ("fp64", "fp32")}
    per_solve = breakdown(lambda: A.solve(b, tol=TOL, inner="fp32", inner_tol=INNER_TOL, restart=200,
                                          max_refinements=12))
    xm_np, x64_np = xm.cpu().numpy(), x64.cpu().numpy()
    torch.cuda.synchronize()  # xq (torch's stream) is read on the library's stream
    y_ref = A.matvec(xq, precision="fp64").cpu().numpy()
    mv_err = {pr: col_rel_err(A.matvec(xq, precision=pr).cpu().numpy(), y_ref) for pr in ("mixed", "fp32")}
    info = op.info()
    line = {"workload": "maxwell_sl_h2_sphere_M4_P2_np9_kappa2_8rhs", "metric": "solves/s (8-RHS batched Maxwell "
            "SL H2 solves to rel.err 1e-8)", "unit": "solves/s", "value": nrhs / (float(np.mean(t_mx)) * 1e-3),
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.mean(t_mx)),
            "dtype": "c128+c64", "data": "synthetic (seeded Hertz dipoles at distance 2.5, sphere.dat)",
            "config": {"elements": int(info[2]), "dofs": op.N, "refinement": m, "degree": p, "n_p": n_p,
                       "kappa": k, "nrhs": nrhs, "tol": TOL, "dense_leaves": int(info[3]),
                       "lowrank_leaves": int(info[4]), "far_field_bytes": int(info[13]),
                       "near_field_bytes": int(info[14]),
                       "l2": "flush: 256 MiB buffer written between timed steps"},
            "fp64_path": {"solves_per_s": nrhs / (float(np.mean(t_64)) * 1e-3), "ms_per_step": float(np.mean(t_64)),
                          "iterations": st64["iterations"]},
            "solver": {kk: stm[kk] for kk in ("iterations", "refinements", "fp64_matvecs", "low_matvecs",
                                             "final_relres")},
            "accuracy": {"mixed_vs_fp64_solution": col_rel_err(xm_np, x64_np),
                         "fp64_final_relres": st64["final_relres"],
                         "mixed_matvec_vs_fp64": mv_err["mixed"], "fp32_matvec_vs_fp64": mv_err["fp32"]},
            "matvec": {"fp64_products_per_s_8rhs": mv_rate("fp64"), "fp32_products_per_s_8rhs": mv_rate("fp32")},
            "assembly_s": asm, "clocks": clocks.summary(),
            "kernel_ms_per_product": per_product, "kernel_ms_per_solve": per_solve}
    print(json.dumps(line), flush=True)


def run_cube(args):
    """Side workload (not the headline line): the Laplace single layer on the
    analytic cube sphere (six patches x/|x| of the cube faces), P = 1, 2^3
    refinement (384 elements), n_p = 6, eta = 1.6; Dirichlet data of a point
    source at (0, 0.2, 1.8) jittered by U(-0.05, 0.05) per coordinate (seed
    2024), one right-hand side, plain FP64 GMRES to 1e-8; the potential at 100
    seeded interior points of radius <= 0.25 against the analytic one. Timed:
    --steps solves after --warmup; cpu_baseline: the oracle's assembly and
    GMRES of the same problem on the host cores."""
    import torch
    import bembel_gb300 as bg
    ctx = bg.Context(0)
    m, p, n_p = 3, 1, 6
    rng = np.random.default_rng(2024)
    x0 = np.array([0.0, 0.2, 1.8]) + rng.uniform(-0.05, 0.05, 3)
    dd = rng.normal(size=(100, 3))
    dd /= np.linalg.norm(dd, axis=1, keepdims=True)
    pts = dd * (0.25 * rng.uniform(0, 1, 100) ** (1 / 3))[:, None]
    u = 1.0 / (4 * np.pi * np.linalg.norm(pts - x0, axis=1))
    t0 = time.time()
    op = bg.DiscreteOperator(bg.AnsatzSpace(bg.Geometry.cube_sphere(ctx), m, p), bg.LaplaceSingleLayerOperator(),
                             n_p=n_p, eta=1.6)
    op.compute()
    torch.cuda.synchronize()
    t_asm = time.time() - t0
    A = op.get_discrete_operator()
    b = op.load_vector(0, x0[None, :])
    for _ in range(max(1, args.warmup)):
        x, st = A.solve(b, tol=TOL, inner="fp64")
    torch.cuda.synchronize()
    t0 = time.time()
    for _ in range(args.steps):
        x, st = A.solve(b, tol=TOL, inner="fp64")
    torch.cuda.synchronize()
    t_solve = (time.time() - t0) / args.steps
    pot = op.potential(x, pts)[:, 0]
    err = float(np.max(np.abs(pot - u)) / np.max(np.abs(u)))
    # CPU baseline: the oracle (restatement of the reference's CPU path), same problem
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    t0 = time.time()
    o = oracle.Problem(oracle.CUBE_SPHERE, m, p, oracle.LAPLACE, np_=n_p, eta=1.6)
    xo = o.gmres(o.load_vector(0, x0), tol=TOL)
    xo = xo[0] if isinstance(xo, tuple) else xo
    t_cpu = time.time() - t0
    err_cpu = float(np.max(np.abs(o.potential(xo, pts) - u)) / np.max(np.abs(u)))
    line = {"workload": "laplace_sl_h2_cube_sphere_M3_P1_np6_1rhs",
            "metric": "solves/s (1-RHS Laplace SL H2 solve to rel.err 1e-8, FP64)", "unit": "solves/s",
            "value": 1.0 / t_solve, "ms_per_solve": t_solve * 1e3, "steps": args.steps, "iterations": st["iterations"],
            "final_relres": st["final_relres"], "assembly_s": t_asm, "potential_vs_analytic": err,
            "dtype": "f64", "data": "synthetic (seeded jittered point source and interior points, analytic cube sphere)",
            "config": {"geometry": "analytic cube sphere (6 patches x/|x|)", "elements": 384, "dofs": op.N,
                       "refinement": m, "degree": p, "n_p": n_p, "eta": 1.6, "tol": TOL},
            "cpu_baseline": {"assembly_plus_solve_s": t_cpu, "potential_vs_analytic": err_cpu, "kind": "port",
                             "cores": os.cpu_count(),
                             "sample": "measured: the oracle's full H2 assembly and GMRES of the same problem"}}
    print(json.dumps(line), flush=True)


def run_helmholtz(args):
    """Side workload (not the headline line): the Helmholtz single layer on the
    16-patch torus (R = 2, r = 0.5), M = 4, P = 2, n_p = 10, swept over seeded
    wavenumbers kappa ~ U[0.5, 6] (seed 4) with 64 plane-wave right-hand sides
    exp(-i kappa d.x), d uniform on the sphere (seed 5). The near fields of all
    wavenumbers are assembled first in one pass (bg_operator_prepare_wavenumbers:
    shared Duffy samples, 4 wavenumbers per launch); per wavenumber the
    operator then assembles only its far field (couplings, tensor-core tiles)
    and the 64 systems are solved to 1e-8 with the FP32 inner operator; the
    first wavenumber is also solved on the plain FP64 path. --kappas bounds
    how many of the 16 wavenumbers run."""
    import torch
    import bembel_gb300 as bg
    from bembel_gb300 import _lib
    L = _lib.load()
    ctx = bg.Context(0)
    sp = ctypes_void_p()
    L.bg_context_get_stream(ctx.h, ctypes_byref(sp))
    stream = torch.cuda.ExternalStream(sp.value, device=torch.device("cuda", 0))
    geo = os.path.join(ROOT, "tests", "golden", "geo", "torus.dat")
    m, p, n_p, nrhs = 4, 2, 10, 64
    kappas = np.random.default_rng(4).uniform(0.5, 6.0, 16)[:max(1, min(16, args.kappas))]
    d = np.random.default_rng(5).normal(size=(nrhs, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    lin = bg.HelmholtzSingleLayerOperator()
    op = bg.DiscreteOperator(bg.AnsatzSpace(bg.Geometry(geo, ctx), m, p), lin, n_p=n_p)
    A = op.get_discrete_operator()
    ev = lambda: torch.cuda.Event(enable_timing=True)

    def timed(fn):
        torch.cuda.synchronize()
        e0, e1 = ev(), ev()
        e0.record(stream)
        out = fn()
        e1.record(stream)
        e1.synchronize()
        return out, e0.elapsed_time(e1) * 1e-3

    if args.kappa_batch > 0:
        return run_helmholtz_batched(args, op, lin, A, kappas, d, timed, ctx)
    per = []
    clocks = ClockSampler(0)
    t_all = time.time()
    with clocks:
        t0 = time.time()
        op.prepare_wavenumbers(kappas)
        torch.cuda.synchronize()
        t_prep = time.time() - t0
        for i, k in enumerate(kappas):
            lin.set_wavenumber(float(k))
            t0 = time.time()
            op.compute()
            torch.cuda.synchronize()
            t_asm = time.time() - t0
            b = torch.from_numpy(np.ascontiguousarray(op.load_vector(2, d).T)).cuda().t()
            (x, st), t_solve = timed(lambda: A.solve(b, tol=TOL, inner="fp32", inner_tol=INNER_TOL, restart=200,
                                                     max_refinements=12))
            rec = {"kappa": float(k), "assembly_s": t_asm, "solve_s": t_solve, "iterations": st["iterations"],
                   "fp64_matvecs": st["fp64_matvecs"], "final_relres": st["final_relres"]}
            if i == 0:
                if not args.no_fp64:
                    (x64, st64), t64 = timed(lambda: A.solve(b, tol=TOL, inner="fp64", restart=200,
                                                             max_refinements=12))
                    rec.update({"fp64_solve_s": t64, "fp64_iterations": st64["iterations"],
                                "mixed_vs_fp64_solution": float(np.max(
                                    np.linalg.norm((x - x64).cpu().numpy(), axis=0) /
                                    np.linalg.norm(x64.cpu().numpy(), axis=0)))})
                xq = torch.randn(op.N, nrhs, dtype=torch.complex128, device="cuda")
                for prec in ("fp64", "fp32"):  # warm-up
                    A.matvec(xq, precision=prec)
                _, tm64 = timed(lambda: A.matvec(xq, precision="fp64"))
                _, tm32 = timed(lambda: A.matvec(xq, precision="fp32"))
                torch.cuda.synchronize()
                y_ref = A.matvec(xq, precision="fp64").cpu().numpy()
                rec["fp32_matvec_vs_fp64"] = col_rel_err(A.matvec(xq, precision="fp32").cpu().numpy(), y_ref)
                rec.update({"fp64_product_ms_64rhs": tm64 * 1e3, "fp32_product_ms_64rhs": tm32 * 1e3,
                            "kernel_ms_per_product": {prec: class_breakdown(L, ctx, lambda: A.matvec(xq, precision=prec))
                                                      for prec in ("fp64", "fp32")}})
            per.append(rec)
    wall = time.time() - t_all
    solve_s = sum(r["solve_s"] for r in per)
    asm_s = sum(r["assembly_s"] for r in per)
    info = op.info()
    line = {"workload": "helmholtz_sl_h2_torus_M4_P2_np10_64rhs_kappa_sweep",
            "metric": "solves/s (64 plane waves per wavenumber, Helmholtz SL H2 solves to rel.err 1e-8)",
            "unit": "solves/s", "value": nrhs * len(per) / solve_s,
            "value_with_assembly": nrhs * len(per) / (solve_s + asm_s + t_prep), "kappas": len(per), "wall_s": wall,
            "near_fields_batched_s": t_prep,
            "assembly_note": "near fields of all wavenumbers in one pass (near_fields_batched_s); per wavenumber "
                             "assembly_s is the far field plus the copy of its prepared near field",
            "fp64_path": ({"solves_per_s": nrhs / per[0]["fp64_solve_s"], "iterations": per[0]["fp64_iterations"]}
                          if "fp64_solve_s" in per[0] else None),
            "dtype": "c128+c64", "data": "synthetic (seeded wavenumbers and plane-wave directions, torus.dat)",
            "config": {"elements": int(info[2]), "dofs": op.N, "refinement": m, "degree": p, "n_p": n_p, "nrhs": nrhs,
                       "tol": TOL, "dense_leaves": int(info[3]), "lowrank_leaves": int(info[4]),
                       "far_field_bytes": int(info[13]), "near_field_bytes": int(info[14])},
            "per_kappa": per, "clocks": clocks.summary()}
    print(json.dumps(line), flush=True)


def run_helmholtz_batched(args, op0, lin, A0, kappas, d, timed, ctx):
    """The same sweep with --kappa-batch B wavenumbers at a time assembled side
    by side (bg_operator_assemble_wavenumbers) and solved together: one
    flexible GMRES over B x 64 columns, whose products apply wavenumber q to
    column block q. The wavenumbers are taken in ascending order, so that a
    batch holds wavenumbers of similar iteration counts. The FP64 coupling
    blocks are released after assembly (the FP64 products use their
    double-float copies), which keeps B = 4 at this size within HBM."""
    import ctypes
    import torch
    import bembel_gb300 as bg
    geo = os.path.join(ROOT, "tests", "golden", "geo", "torus.dat")
    m, p, n_p, nrhs = 4, 2, 10, 64
    B = args.kappa_batch
    op = bg.DiscreteOperator(bg.AnsatzSpace(bg.Geometry(geo, ctx), m, p), lin, n_p=n_p, keep_fp64_blocks=False)
    A = op.get_discrete_operator()
    ks = np.sort(kappas)
    per = []
    clocks = ClockSampler(0)
    t_all = time.time()
    with clocks:
        for b0 in range(0, len(ks), B):
            kb = ks[b0:b0 + B]
            lin.set_wavenumber(float(kb[0]))
            t0 = time.time()
            op.prepare_wavenumbers(kb)
            op.assemble_wavenumbers()
            torch.cuda.synchronize()
            t_asm = time.time() - t0
            dirs = np.tile(d, (len(kb), 1))
            b = torch.from_numpy(np.ascontiguousarray(op.load_vector(2, dirs).T)).cuda().t()
            (x, st), t_solve = timed(lambda: A.solve(b, tol=TOL, inner="fp32", inner_tol=INNER_TOL, restart=200,
                                                     max_refinements=12))
            used = bg._lib.load()
            alloc, est = ctypes.c_size_t(), ctypes.c_size_t()
            used.bg_operator_memory(op.h, ctypes.byref(alloc), ctypes.byref(est))
            per.append({"kappas": [float(k) for k in kb], "assembly_s": t_asm, "solve_s": t_solve,
                        "iterations": st["iterations"], "fp64_matvecs": st["fp64_matvecs"],
                        "final_relres": st["final_relres"], "device_bytes": int(alloc.value)})
            op.release_wavenumbers()
    wall = time.time() - t_all
    solve_s = sum(r["solve_s"] for r in per)
    asm_s = sum(r["assembly_s"] for r in per)
    info = op.info()
    line = {"workload": "helmholtz_sl_h2_torus_M4_P2_np10_64rhs_kappa_sweep_batched",
            "metric": "solves/s (64 plane waves per wavenumber, Helmholtz SL H2 solves to rel.err 1e-8)",
            "unit": "solves/s", "value": nrhs * len(ks) / solve_s,
            "value_with_assembly": nrhs * len(ks) / (solve_s + asm_s), "kappas": len(ks), "kappa_batch": B,
            "wall_s": wall,
            "assembly_note": "per batch: near fields of its wavenumbers in one pass, then every wavenumber's far "
                             "field and tiles side by side",
            "dtype": "c128+c64", "data": "synthetic (seeded wavenumbers and plane-wave directions, torus.dat)",
            "config": {"elements": int(info[2]), "dofs": op.N, "refinement": m, "degree": p, "n_p": n_p, "nrhs": nrhs,
                       "tol": TOL, "solver": "one FGMRES(FP64 H2) over kappa_batch x 64 columns, inner GMRES(2e-3) "
                                             "on the FP32 operator"},
            "per_batch": per, "clocks": clocks.summary()}
    print(json.dumps(line), flush=True)


def serving_stream(n, max_level, seed=7):
    """Seeded request stream: Poisson arrivals (mean 200/s), sphere or torus,
    refinement 2^M with M uniform in {2..max_level}, P in {1, 2}, Laplace or
    Helmholtz with kappa ~ U[0.5, 8] snapped to 8 bucket centres, 1-32
    right-hand sides (point sources outside the surface, or plane waves)."""
    rng = np.random.default_rng(seed)
    centres = 0.5 + 7.5 * (np.arange(8) + 0.5) / 8
    t, out = 0.0, []
    for _ in range(n):
        t += rng.exponential(1.0 / 200.0)
        geo = int(rng.integers(2))
        m = int(rng.integers(2, max_level + 1))
        p = int(rng.integers(1, 3))
        helm = bool(rng.integers(2))
        k = float(centres[np.argmin(np.abs(centres - rng.uniform(0.5, 8.0)))]) if helm else 0.0
        nrhs = int(rng.integers(1, 33))
        d = rng.normal(size=(nrhs, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        if helm:
            data, dk = d, 2
        else:
            r = rng.uniform(1.5, 3.0, (nrhs, 1)) if geo == 0 else rng.uniform(3.0, 4.5, (nrhs, 1))
            data, dk = d * r, 0
        out.append({"t": t, "geo": geo, "M": m, "P": p, "kind": "helmholtz" if helm else "laplace", "kappa": k,
                    "data_kind": dk, "data": data})
    return out


def run_serving(args):
    """Side workload (not the headline line): the serving loop (bg_server) on a
    seeded Poisson stream of Laplace / Helmholtz solve requests. Pass 1 starts
    with an empty operator cache, pass 2 replays the stream with the cache as
    pass 1 left it (mixed inner operator), pass 3 replays the first requests on
    the plain FP64 path. Latency = completion - submission; throughput = solved
    right-hand sides per second of the pass."""
    import torch
    import bembel_gb300 as bg
    ctx = bg.Context(0)
    free, total = torch.cuda.mem_get_info()
    budget = int(min(200e9, 0.8 * free))
    srv = bg.Server(ctx, budget, workers=args.workers)
    geos = [srv.add_geometry(bg.Geometry(GEO, ctx)),
            srv.add_geometry(bg.Geometry(os.path.join(ROOT, "tests", "golden", "geo", "torus.dat"), ctx))]
    stream = serving_stream(args.requests, args.max_level)

    def one_pass(reqs, inner):
        t0 = time.time()
        tickets = []
        for r in reqs:
            dt = r["t"] - (time.time() - t0)
            if dt > 0:
                time.sleep(dt)
            tickets.append(srv.submit(geos[r["geo"]], r["kind"], r["M"], r["P"], r["data_kind"], r["data"],
                                      kappa=r["kappa"], tol=TOL, inner=inner))
        res = [srv.wait(t)[1] for t in tickets]
        lat = np.array([x["t_done"] - x["t_submit"] for x in res])
        span = max(x["t_done"] for x in res) - min(x["t_submit"] for x in res)
        nr = sum(r["data"].shape[0] for r in reqs)
        ok = sum(1 for x in res if x["status"] in (0, 7))
        return {"requests": len(reqs), "ok": ok, "rhs": nr, "span_s": span, "solves_per_s": nr / span,
                "requests_per_s": len(reqs) / span, "p50_ms": 1e3 * float(np.percentile(lat, 50)),
                "p99_ms": 1e3 * float(np.percentile(lat, 99)), "cache_hits": sum(x["cache_hit"] for x in res),
                "max_final_relres": max(x["stats"]["final_relres"] for x in res)}

    clocks = ClockSampler(0)
    with clocks:
        cold = one_pass(stream, "fp32")
        s1 = srv.stats()
        warm = one_pass(stream, "fp32")
        k = min(len(stream), args.fp64_requests)
        warm_k = one_pass(stream[:k], "fp32")
        fp64 = one_pass(stream[:k], "fp64")
    st = srv.stats()
    srv.close()
    keys = {(r["geo"], r["kind"], r["M"], r["P"], r["kappa"]) for r in stream}
    line = {"workload": "serving_poisson200_laplace_helmholtz_sphere_torus",
            "metric": "served solves/s and p50/p99 latency (rel.err 1e-8)", "unit": "solves/s",
            "value": warm["solves_per_s"], "offered_requests_per_s": 200.0,
            "config": {"requests": len(stream), "distinct_operators": len(keys), "levels": [2, args.max_level],
                       "workers": args.workers,
                       "degrees": [1, 2], "kappa_buckets": 8, "nrhs": [1, 32], "hbm_budget_bytes": budget,
                       "note": "requests for one operator that wait together are solved as one batch"},
            "cold_cache": cold, "warm_cache": warm,
            "mixed_vs_fp64_same_requests": {"mixed": warm_k, "fp64": fp64},
            "server": {"after_cold": s1, "final": st}, "clocks": clocks.summary()}
    print(json.dumps(line), flush=True)


def ctypes_void_p():
    import ctypes
    return ctypes.c_void_p()


def ctypes_byref(x):
    import ctypes
    return ctypes.byref(x)


def run_profile_case(args):
    """Small fixed cases for ncu (not a bench line): 'matvec' assembles the
    workload's operator (refinement --profile-m) and applies five 32-column
    products at --precision; 'solve' runs one batched solve with the chosen
    inner operator."""
    import torch
    import bembel_gb300 as bg
    ctx = bg.Context(0)
    store = True  # the tensor-core far field streams tiles built from the stored FP64 blocks
    m = args.profile_m if args.profile_m is not None else M
    if args.workload == "maxwell":
        # EFIE on the sphere, P = 2, n_p = 9, kappa = 2, 8 right-hand sides
        lin = bg.MaxwellSingleLayerOperator()
        lin.set_wavenumber(2.0)
        op = bg.DiscreteOperator(bg.AnsatzSpace(bg.Geometry(GEO, ctx), m, P), lin, n_p=NP)
        op.compute()
        A = op.get_discrete_operator()
        x = torch.randn(op.N, 8, dtype=torch.complex128, device="cuda")
        for _ in range(5):
            A.matvec(x, precision=args.precision)
        torch.cuda.synchronize()
        print(json.dumps({"profile": "matvec", "workload": "maxwell", "precision": args.precision, "M": m, "N": op.N,
                          "products": 5}))
        return
    if args.profile == "batched":
        # Helmholtz on the torus (M = --profile-m, default 3), 4 wavenumbers
        # assembled side by side, three mixed products of 4 x 16 columns
        lin = bg.HelmholtzSingleLayerOperator()
        lin.set_wavenumber(1.0)
        mb = args.profile_m if args.profile_m is not None else 3
        op = bg.DiscreteOperator(bg.AnsatzSpace(bg.Geometry(os.path.join(ROOT, "tests", "golden", "geo", "torus.dat"),
                                                            ctx), mb, P), lin, n_p=10)
        ks = [1.0, 2.0, 3.0, 4.0]
        op.prepare_wavenumbers(ks)
        op.assemble_wavenumbers()
        A = op.get_discrete_operator()
        x = torch.randn(op.N, 4 * 16, dtype=torch.complex128, device="cuda")
        for _ in range(3):
            A.matvec(x, precision="mixed")
        torch.cuda.synchronize()
        print(json.dumps({"profile": "batched", "M": mb, "N": op.N, "kappas": ks, "columns": 64, "products": 3}))
        return
    op = bg.DiscreteOperator(bg.AnsatzSpace(bg.Geometry(GEO, ctx), m, P), bg.LaplaceSingleLayerOperator(), n_p=NP,
                             store_fp64_far=store)
    op.compute()
    A = op.get_discrete_operator()
    if args.profile == "matvec":
        x = torch.randn(op.N, NRHS, dtype=torch.float64, device="cuda")
        for _ in range(5):
            A.matvec(x, precision=args.precision)
        torch.cuda.synchronize()
        print(json.dumps({"profile": "matvec", "precision": args.precision, "M": m, "N": op.N, "products": 5}))
    else:
        b = op.load_vector(0, rhs_points())
        _, st = A.solve(b, tol=TOL, inner=args.inner, inner_tol=INNER_TOL, restart=200, max_refinements=12)
        print(json.dumps({"profile": "solve", "inner": args.inner, "N": op.N, "stats": st}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--inner", default="mixed", choices=["mixed", "fp32"],
                    help="precision of the inner (preconditioning) operator: mixed (near field FP64-accurate, the "
                         "workload's mixed form) or fp32 (near field FP32 as well)")
    ap.add_argument("--profile", choices=["matvec", "solve", "batched"], default=None,
                    help="run a small fixed case for ncu instead of the benchmark")
    ap.add_argument("--precision", default="fp32", choices=["fp64", "mixed", "fp32"],
                    help="product precision of --profile matvec")
    ap.add_argument("--profile-m", type=int, default=None, help="refinement level of --profile cases (default 5)")
    ap.add_argument("--workload", default="laplace", choices=["laplace", "maxwell", "helmholtz", "serving", "cube"],
                    help="laplace: the headline line; maxwell / helmholtz: side workloads")
    ap.add_argument("--kappas", type=int, default=4, help="wavenumbers of the helmholtz sweep (of 16)")
    ap.add_argument("--kappa-batch", type=int, default=0,
                    help="helmholtz: wavenumbers assembled side by side and solved together (0: one at a time)")
    ap.add_argument("--no-fp64", action="store_true", help="helmholtz: skip the plain FP64 solve")
    ap.add_argument("--requests", type=int, default=100, help="serving: requests in the stream")
    ap.add_argument("--max-level", type=int, default=4, help="serving: largest refinement level (2..6)")
    ap.add_argument("--fp64-requests", type=int, default=30, help="serving: requests replayed on the FP64 path")
    ap.add_argument("--workers", type=int, default=4, help="serving: worker streams of the server")
    ap.add_argument("--autotune", action="store_true",
                    help="laplace: set the 32-column products' launch plans with the autotuner first")
    args = ap.parse_args()
    if args.workload == "cube" and args.impl == "gb300" and not args.profile:
        run_cube(args)
    elif args.workload == "maxwell" and args.impl == "gb300" and not args.profile:
        run_maxwell(args)
    elif args.workload == "helmholtz" and args.impl == "gb300" and not args.profile:
        run_helmholtz(args)
    elif args.workload == "serving" and args.impl == "gb300" and not args.profile:
        run_serving(args)
    elif args.profile:
        run_profile_case(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
