#!/usr/bin/env python
"""Benchmark: stochastic-Galerkin CG solve time to a 1e-8 FP64 relative
residual on one GB300, mixed precision vs FP64, plus the operator-apply
bandwidth.

Workload (one "step"): the SG Poisson problem on the unit square with P2
elements on a 256 x 256 mesh (263 169 dofs), affine cosine KLE coefficient
a = 1 + sum_{m<=20} 0.547 m^-2 cos(pi b1 x) cos(pi b2 y) y_m, orthonormal
Legendre basis, the 150 multi-indices of largest weight (M = 20); one
mean-preconditioned PCG solve from x0 = 0 to ||b - A x|| <= 1e-8 ||b||
(FP64 true residual), mixed precision (FP32 inner PCG, FP64 refinement).
Inputs are synthetic (the reference publishes no dataset): the operator is
assembled on the host and resident in HBM before timing; the operator and
vectors (~0.8 GB) exceed the 129 MB L2, so no flush is needed.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the reference algorithm on the host cores, complete
solves only: the LU factorisation of the mean preconditioner once (SciPy
SuperLU, outside the steps, reported as factor_s), then per step one whole
solve_primal! (solvers_poisson_primal.jl:130-169): left-preconditioned GMRES
without restarts to a true relative residual of 1e-8, with the plain-C mul!
(:86-124) and the per-mode LU solves of ldiv! (:47-78) on all host threads.
A step takes tens of seconds, so the arm times as many complete solves as fit
in SGFEM_REF_BUDGET_S seconds (default 150, at least one) and prints the count
it timed.  The config-1 problem (P1 32x32, M=5, P=21) is timed the same way
and reported under "config1".
N > 1 runs independent replicas (the path has no data-path exchange).
"""
import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SG CG solve time to 1e-8 rel. residual, mixed vs FP64 on 1 GB300; apply GB/s"
WORKLOAD = "P2 256x256 (263169 dofs), M=20, P=150 top-weight Legendre set, affine cosine KLE, mean-preconditioned PCG to 1e-8"
# wall-clock budget of the reference arm's timed solves (seconds)
REF_BUDGET_S = float(os.environ.get("SGFEM_REF_BUDGET_S", "150"))


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return None


def setup_workload(pkg, N=256):
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=150)
    M, P = 20, 150
    mis = pkg.top_weight_multiindices(M, P, C.decay_factors)
    V = pkg.H1Pk(pkg.unit_square_mesh(N), 2)
    TB = pkg.TensorizedBasis(pkg.LegendrePolynomials, M, max(max(m) for m in mis),
                             max(max(m) for m in mis) + 4, multi_indices=mis)
    sol = pkg.SGFEVector(V, TB)
    Ks, b0 = pkg.assemble(pkg.PoissonProblemPrimal, sol, C, rhs=lambda x, y: np.ones_like(x))
    return V, TB, Ks, b0


def algorithmic_bytes(n, P, nnz, M1, es):
    """Bytes one apply must move at least once: X read, Y written, M+1 values
    and one column index per nonzero, the row pointers."""
    return 2 * n * P * es + nnz * M1 * es + nnz * 4 + (n + 1) * 4


def algorithmic_flops(n, P, nnz, Qn, nnzG):
    return 2.0 * nnz * Qn + 2.0 * n * nnzG


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.p = None
        self.path = os.path.join("/tmp", f"sgfem_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(n_gpus):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    return rank, world, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def allmax(pg, v):
    if pg is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def reference_solver(Ks, TB, V):
    """The reference's solve_primal! on the host cores (oracle/refsolve.py): the
    LU factorisation of the mean preconditioner happens here, once."""
    from oracle import refsolve
    return refsolve.ReferenceSolver(Ks, TB.G.toarray(), V.bdofs, TB.nmodes)


def time_reference_solves(rs, b0, warmup, steps, budget_s):
    """Complete reference solves to a 1e-8 true relative residual: `warmup`
    untimed ones (at most three), then timed ones until `steps` are done or the
    budget is spent (at least one).  Returns ([ms per solve], last stats)."""
    for _ in range(min(warmup, 3)):
        rs.solve(b0, rtol=1e-8)
    out, st = [], None
    t0 = time.perf_counter()
    while len(out) < max(1, steps):
        _, st = rs.solve(b0, rtol=1e-8)
        out.append(st["time_s"] * 1e3)
        if time.perf_counter() - t0 + st["time_s"] > budget_s:
            break
    return out, st


def reference_config1():
    """Config 1 (P1 32x32, M=5, total degree 2, P=21) through the reference's
    solve_primal! on the host: ms per complete solve to 1e-8."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    C, V, TB, sol, Ks, b0 = config1_problem(pkg)
    rs = reference_solver(Ks, TB, V)
    ts, st = time_reference_solves(rs, b0, 1, 20, 20.0)
    return {"workload": "config1: P1 32x32 (1089 dofs), M=5, P=21, GMRES + LU to 1e-8", "ms": statistics.median(ts),
            "solves_timed": len(ts), "iterations": st["iterations"], "relres": st["relres"],
            "factor_s": rs.t_factor, "threads": rs.nthreads}


def run_reference(args, rank, world, pg):
    import __graft_entry__ as ge
    if rank != 0:
        return
    pkg = ge.load_package()
    ge_build_oracle()
    V, TB, Ks, b0 = setup_workload(pkg)
    rs = reference_solver(Ks, TB, V)
    ts, st = time_reference_solves(rs, b0, args.warmup, args.steps, REF_BUDGET_S)
    v = statistics.median(ts)
    c1 = reference_config1()
    sample = (f"{len(ts)} complete solves (GMRES + per-mode LU solves, {st['iterations']} iterations to a true "
              f"relative residual of {st['relres']:.2e}) on {rs.nthreads} threads; SuperLU factorisation of K_0 "
              f"once before the steps ({rs.t_factor:.1f} s)")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "ms", "n_gpus": world, "steps": len(ts),
            "steps_requested": args.steps, "warmup": min(args.warmup, 3), "ms_per_step": v,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "parallelism": "replicas"},
            "cpu_baseline": {"value": v, "unit": "ms", "cores": rs.nthreads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "iterations": st["iterations"], "relres": st["relres"], "factor_s": rs.t_factor,
            "time_split_s": st["split_s"], "solve_ms_all": ts, "config1": c1}
    print(json.dumps(line), flush=True)


def ge_build_oracle():
    from oracle import cbuild
    cbuild.build()


def run_ours(args, rank, world, local, pg):
    import __graft_entry__ as ge
    import torch
    pkg = ge.load_package()
    device = local if world > 1 else 0
    torch.cuda.set_device(device)
    V, TB, Ks, b0 = setup_workload(pkg)
    op = pkg.SGOperator(V, TB, Ks, device=device)
    ctx = op.ctx
    n, ld = ctx.device_layout()
    P = TB.nmodes
    opts = ctx.default_options(precision=pkg.MIXED, rtol=1e-8, inner_rtol=1e-4)
    opts64 = ctx.default_options(precision=pkg.FP64, rtol=1e-8)
    x = torch.zeros(n * ld, dtype=torch.float64, device=f"cuda:{device}")

    def solve_once(o):
        x.zero_()
        torch.cuda.synchronize()
        return ctx.solve_device(b0, x.data_ptr(), o)

    for _ in range(args.warmup):
        solve_once(opts)
    clocks = ClockSampler(device)
    barrier(pg)
    torch.cuda.synchronize()
    clocks.start()
    t0 = time.perf_counter()
    dev_ms = []
    launches = 0
    relres = []
    iters = []
    for _ in range(args.steps):
        st = solve_once(opts)
        dev_ms.append(st.time_ms)
        launches += st.kernel_launches
        relres.append(st.relres)
        iters.append(st.iterations)
    torch.cuda.synchronize()
    wall = (time.perf_counter() - t0) * 1e3 / args.steps
    barrier(pg)
    clk = clocks.stop()
    ms = allmax(pg, statistics.mean(dev_ms))

    # FP64 solve (the comparison arm of the metric)
    st64 = solve_once(opts64)
    fp64_ms = allmax(pg, st64.time_ms)

    # e2e through the public C ABI with host buffers (pinned), x0 -> GPU, x -> host
    xh = torch.zeros(n * P, dtype=torch.float64, pin_memory=True).numpy()
    # five calls after one warm-up; the median is reported (a host-side stall of a single
    # call, with the device part unchanged, otherwise moves a short mean by several ms);
    # Python's collector is paused around the calls
    e2e, e2e_dev = [], []
    gc.collect()
    gc.disable()
    try:
        for k in range(6):
            xh[:] = 0.0
            t = time.perf_counter()
            st_e = ctx.solve(b0, xh, opts)
            if k > 0:
                e2e.append((time.perf_counter() - t) * 1e3)
                e2e_dev.append(st_e.time_ms)  # the device part of the same call (CUDA events)
    finally:
        gc.enable()
    e2e_ms = allmax(pg, statistics.median(e2e))

    # dominant kernel: the FP32 apply of the inner PCG (and the FP64 apply)
    nnz = Ks[0].nnz
    M1 = len(Ks)
    B32 = algorithmic_bytes(n, P, nnz, M1, 4)
    B64 = algorithmic_bytes(n, P, nnz, M1, 8)
    t32 = ctx.time_apply(pkg.FP32, 20)
    t64 = ctx.time_apply(pkg.FP64, 10)
    pk = peaks()
    peak_gbs = pk["hbm_gbs"] if pk else 6800.0
    ach = B32 / (t32 * 1e-3) / 1e9
    traffic = None
    tp = os.path.join(ROOT, "profiles", "roofline_traffic.json")
    if os.path.exists(tp):
        try:
            traffic = json.load(open(tp)).get("apply_fp32_bytes_per_launch")
        except Exception:
            traffic = None
    line = {
        "metric": METRIC, "value": ms, "unit": "ms", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "precision": "mixed (FP32 PCG with FP64 solution accumulation, double-FP32 refinement residual, FP64 result)",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "l2": "inputs larger than L2 (operator + vectors ~0.8 GB)"},
        "fp64_solve_ms": fp64_ms, "mixed_speedup_vs_fp64": fp64_ms / ms,
        "iterations": statistics.median(iters), "relres": max(relres), "wall_ms_per_step": wall,
        "e2e": {"value": e2e_ms, "unit": "ms", "h2d_bytes_per_step": int(n * P * 8 + n * 8),
                "d2h_bytes_per_step": int(n * P * 8), "statistic": "median of 5 calls",
                "samples_ms": [round(v, 3) for v in e2e],
                "device_ms_of_samples": [round(v, 3) for v in e2e_dev]},
        "gpu_launches": int(launches),
        "apply_variant": ctx.apply_variant[1],
        "roofline": {"bound": "hbm",
                     "kernel": ("sg_apply_jit (SG operator apply, FP32, specialised by NVRTC)"
                                if ctx.apply_variant[0] == 1 else "k_apply<float> (SG operator apply, FP32)"),
                     "achieved": ach, "peak": peak_gbs, "unit": "GB/s", "frac": ach / peak_gbs,
                     "traffic": traffic, "algorithmic_bytes": B32, "ms_per_launch": t32,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs" if pk else "fallback 6.8 TB/s"},
        "precondition_ms": {"fp32": ctx.time_precondition(pkg.FP32, 10), "fp64": ctx.time_precondition(pkg.FP64, 5)},
        "apply_fp64": {"ms_per_launch": t64, "GB/s": B64 / (t64 * 1e-3) / 1e9,
                       "GFLOP/s": algorithmic_flops(n, P, nnz, ctx_qn(op), TB.G.nnz) / (t64 * 1e-3) / 1e9},
        "refinement_residual": dict(zip(("ms", "arithmetic"), ctx.time_residual(5))),
        "solve_structure": {"fp32_iterations": statistics.median(iters), "refinement_steps": st.outer_iterations,
                            "fp64_applies": st.fp64_applies, "lattice_preconditioner": ctx.lattice_log},
        "clocks": clk,
    }
    op.close()
    if rank == 0 and not args.no_cpu_baseline:
        ge_build_oracle()
        rs = reference_solver(Ks, TB, V)
        ts, st = time_reference_solves(rs, b0, 0, 1, 0.0)
        line["cpu_baseline"] = {"value": ts[0], "unit": "ms", "cores": rs.nthreads, "kind": "port",
                                "sample": f"one complete solve of this workload by the reference algorithm (GMRES "
                                          f"+ per-mode LU solves, {st['iterations']} iterations to a true relative "
                                          f"residual of {st['relres']:.2e}); SuperLU factorisation before it "
                                          f"({rs.t_factor:.1f} s, not counted)"}
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_profile(args):
    """Small, bounded launches for ncu: `apply32` / `apply64` launch the apply 1+3
    times; `precond32` / `precond64` apply the lattice preconditioner 1+2 times
    (three pass kernels each); `residual` evaluates the mixed refinement residual
    1+2 times; `solve` runs one mixed solve."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    V, TB, Ks, b0 = setup_workload(pkg, N=args.mesh)
    op = pkg.SGOperator(V, TB, Ks, device=0)
    if args.profile in ("apply32", "apply64"):
        prec = pkg.FP32 if args.profile == "apply32" else pkg.FP64
        ms = op.ctx.time_apply(prec, 3)
        print(json.dumps({"profile": args.profile, "ms_per_apply": ms}))
    elif args.profile == "residual":
        ms, kind = op.ctx.time_residual(2)
        print(json.dumps({"profile": "residual", "ms_per_residual": ms, "kind": kind}))
    elif args.profile in ("precond32", "precond64"):
        prec = pkg.FP32 if args.profile == "precond32" else pkg.FP64
        ms = op.ctx.time_precondition(prec, 2)
        print(json.dumps({"profile": args.profile, "ms_per_application": ms, "form": op.ctx.lattice_log}))
    else:
        x = np.zeros(V.ndofs * TB.nmodes)
        st = op.solve_primal(b0, x, rtol=1e-8, precision=pkg.MIXED)
        print(json.dumps({"profile": "solve", **st}))
    op.close()


# ---------------------------------------------------------------- other workloads
def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _timed(fn):
    import torch
    torch.cuda.synchronize()
    t = time.perf_counter()
    r = fn()
    torch.cuda.synchronize()
    return r, (time.perf_counter() - t) * 1e3


def config1_problem(pkg, N=32, M=5, deg=2):
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=150)
    V = pkg.H1Pk(pkg.unit_square_mesh(N), 1)
    mis = pkg.total_degree_multiindices(M, deg)
    TB = pkg.TensorizedBasis(pkg.LegendrePolynomials, M, deg, deg + 4, multi_indices=mis)
    sol = pkg.SGFEVector(V, TB)
    Ks, b0 = pkg.assemble(pkg.PoissonProblemPrimal, sol, C, rhs=lambda x, y: np.ones_like(x))
    return C, V, TB, sol, Ks, b0


def run_config1(args):
    """Config 1 (P1 32x32, M=5, total degree 2, P=21): FP64 PCG and mixed PCG to
    --rtol (default 1e-10; 1e-8 is the mixed-vs-FP64 target) and one estimator
    pass; config 3's mixed-precision errors against FP64 (solution, energy norm,
    estimator)."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    C, V, TB, sol, Ks, b0 = config1_problem(pkg)
    f = lambda x, y: np.ones_like(x)
    op = pkg.SGOperator(V, TB, Ks, device=0)
    n, P = V.ndofs, TB.nmodes
    res = {}
    for name, prec in (("fp64", pkg.FP64), ("mixed", pkg.MIXED)):
        ts = []
        for k in range(args.warmup + args.steps):
            x = np.zeros(n * P)
            st = op.solve_primal(b0, x, rtol=args.rtol, precision=prec)
            if k >= args.warmup:
                ts.append(st["time_ms"])
        res[name] = (x, st, statistics.median(ts))
    x64, xm = res["fp64"][0], res["mixed"][0]
    e64 = float(np.sqrt(x64 @ op.mul(x64)))
    em = float(np.sqrt(xm @ op.mul(xm)))
    sol.entries[:] = x64
    pkg.estimate(pkg.PoissonProblemPrimal, sol, C, rhs=f, bonus_quadorder=2, tail_extension=(10, 2), op=op)
    tes = []
    for _ in range(max(1, args.steps)):
        (eta64, ec64, ext), t = _timed(lambda: pkg.estimate(pkg.PoissonProblemPrimal, sol, C, rhs=f, bonus_quadorder=2,
                                                            tail_extension=(10, 2), op=op))
        tes.append(t)
    sol.entries[:] = xm
    etam, ecm, _ = pkg.estimate(pkg.PoissonProblemPrimal, sol, C, rhs=f, bonus_quadorder=2, tail_extension=(10, 2),
                                op=op)
    line = {"workload": f"config1: P1 32x32 (1089 dofs), M=5, total degree 2 (P=21), PCG to {args.rtol:g} + estimator",
            "fp64_solve_ms": res["fp64"][2], "fp64_iterations": res["fp64"][1]["iterations"],
            "mixed_speedup_vs_fp64": res["fp64"][2] / res["mixed"][2],
            "mixed_solve_ms": res["mixed"][2], "mixed_iterations": res["mixed"][1]["iterations"],
            "mixed_outer": res["mixed"][1]["outer_iterations"],
            "estimate_ms_wall": statistics.median(tes), "P_ext": len(ext),
            "mixed_vs_fp64": {"solution_rel_2norm": _rel(xm, x64), "energy_norm_rel": abs(em - e64) / e64,
                              "eta4modes_rel": _rel(etam, eta64), "eta4cell_rel_max":
                                  float(np.max(np.abs(ecm - ec64)) / np.max(np.abs(ec64)))},
            "relres": {"fp64": res["fp64"][1]["relres"], "mixed": res["mixed"][1]["relres"]},
            "note": "estimate_ms_wall includes the host-side extension of the multi-index set and argument setup"}
    op.close()
    print(json.dumps(line), flush=True)


def run_estimate(args):
    """Config 2's estimator pass: estimate(PoissonProblemPrimal) of the mixed
    solution of the headline workload (P2 256x256, M=20, P=150), default
    bonus_quadorder = 1 and tail_extension = (10, 2); wall time of the whole call
    (host extension of the multi-index set, argument setup, kernels)."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=150)
    V, TB, Ks, b0 = setup_workload(pkg, N=args.mesh)
    op = pkg.SGOperator(V, TB, Ks, device=0)
    sol = pkg.SGFEVector(V, TB)
    st = op.solve_primal(b0, sol.entries, rtol=1e-8, precision=pkg.MIXED)
    f = lambda x, y: np.ones_like(x)
    pkg.estimate(pkg.PoissonProblemPrimal, sol, C, rhs=f, op=op)
    ts = []
    for _ in range(max(1, args.steps)):
        (em, ec, ext), t = _timed(lambda: pkg.estimate(pkg.PoissonProblemPrimal, sol, C, rhs=f, op=op))
        ts.append(t)
    op.close()
    line = {"workload": f"config 2 estimator pass: P2 {args.mesh}x{args.mesh} ({V.ndofs} dofs), M=20, P=150, "
                        f"bonus_quadorder 1, tail_extension (10, 2)",
            "estimate_ms_wall": statistics.median(ts), "P_ext": len(ext), "M_ext": len(ext[0]),
            "ncells": V.mesh.ncells, "solve_relres": st["relres"],
            "eta_total": float(np.sqrt(np.sum(em ** 2)))}
    print(json.dumps(line), flush=True)


def run_equilibration(args):
    """Equilibration estimator (sgfem_estimate_equilibration) on the config 1 basis
    (M=5, total degree 2, P=21) for P1 meshes of 32x32 and 128x128 and a P2 64x64
    mesh, on the solved SG system; the oracle (pure Python, one thread) on the P1
    8x8 mesh is the CPU rate, compared per (cell, extended mode)."""
    import __graft_entry__ as ge
    from oracle import basis as ob
    from oracle import coefficient as oc
    from oracle import equilibration as oq
    from oracle import fem as of
    pkg = ge.load_package()
    f = lambda x, y: np.ones_like(x)
    cases = []
    for N, order in ((32, 1), (128, 1), (64, 2)):
        C, V, TB, sol, Ks, b0 = config1_problem(pkg, N=N)
        if order == 2:
            V = pkg.H1Pk(pkg.unit_square_mesh(N), 2)
            sol = pkg.SGFEVector(V, TB)
            Ks, b0 = pkg.assemble(pkg.PoissonProblemPrimal, sol, C, rhs=f)
        op = pkg.SGOperator(V, TB, Ks, device=0)
        op.solve_primal(b0, sol.entries, rtol=1e-10, precision=pkg.FP64)
        pkg.estimate_equilibration(pkg.PoissonProblemPrimal, sol, C, rhs=f, op=op)
        ts = []
        for _ in range(max(1, args.steps)):
            (em, ec, ext), t = _timed(lambda: pkg.estimate_equilibration(pkg.PoissonProblemPrimal, sol, C, rhs=f,
                                                                         op=op))
            ts.append(t)
        op.close()
        cases.append({"mesh": f"P{order} {N}x{N}", "ncells": V.mesh.ncells, "P_ext": len(ext),
                      "gpu_ms_wall": statistics.median(ts),
                      "us_per_cell_mode": statistics.median(ts) * 1e3 / (V.mesh.ncells * len(ext))})
    C, V, TB, sol, Ks, b0 = config1_problem(pkg, N=8)
    Vo = of.LagrangeSpace(of.StructuredMesh(8), 1)
    Co = oc.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=150)
    U = np.random.default_rng(3).standard_normal(V.ndofs * TB.nmodes)
    t = time.perf_counter()
    _, oec, oext = oq.estimate_equilibration(Vo, U, TB.multi_indices, ob.LEGENDRE, Co, lambda x, y: 1.0 + 0 * x)
    t_cpu = (time.perf_counter() - t) * 1e3
    cpu_rate = t_cpu * 1e3 / (Vo.mesh.ncells * len(oext))
    line = {"workload": "equilibration estimator: config 1 basis (M=5, total degree 2, P=21), RT_k patch problems on "
                        "every node, div penalty 1e5",
            "cases": cases,
            "cpu_baseline": {"kind": "port", "cores": 1, "sample": "oracle on P1 8x8 (128 cells)",
                             "ms": t_cpu, "us_per_cell_mode": cpu_rate},
            "speedup_per_cell_mode_vs_cpu": cpu_rate / cases[1]["us_per_cell_mode"]}
    print(json.dumps(line), flush=True)


def run_lognormal(args):
    """Config 3 lognormal variant: LogTransformedPoissonProblemPrimal, Hermite,
    P1 128x128 (16641 dofs), M=10, 80 top-weight multi-indices, mean 0, tau=0.9;
    device GMRES(20) to 1e-8, FP64 against mixed precision."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=0.0, maxm=150)
    M, P = 10, 80
    mis = pkg.top_weight_multiindices(M, P, C.decay_factors)
    deg = max(max(m) for m in mis)
    V = pkg.H1Pk(pkg.unit_square_mesh(128), 1)
    TB = pkg.TensorizedBasis(pkg.HermitePolynomials, M, deg, deg + 4, multi_indices=mis)
    sol = pkg.SGFEVector(V, TB)
    (Ks, b), t_asm = _timed(lambda: pkg.assemble(pkg.LogTransformedPoissonProblemPrimal, sol, C,
                                                 rhs=lambda x, y: np.ones_like(x)))
    op = pkg.SGOperator(V, TB, Ks, device=0)
    out = {}
    restart = args.restart
    for name, prec in (("fp64", pkg.FP64), ("mixed", pkg.MIXED)):
        ts = []
        for k in range(args.warmup + args.steps):
            x = np.zeros(V.ndofs * P)
            st = op.solve_logpoisson(b, x, rtol=1e-8, precision=prec, restart=restart, maxit=3000, allow_maxit=True)
            if k >= args.warmup:
                ts.append(st["time_ms"])
        out[name] = (x, st, statistics.median(ts))
    x64, xm = out["fp64"][0], out["mixed"][0]
    line = {"workload": f"lognormal: P1 128x128 (16641 dofs), Hermite, M=10, P=80, GMRES({restart}) to 1e-8",
            "fp64_solve_ms": out["fp64"][2], "fp64_iterations": out["fp64"][1]["iterations"],
            "mixed_solve_ms": out["mixed"][2], "mixed_iterations": out["mixed"][1]["iterations"],
            "mixed_outer": out["mixed"][1]["outer_iterations"],
            "mixed_speedup_vs_fp64": out["fp64"][2] / out["mixed"][2],
            "mixed_vs_fp64_solution_rel_2norm": _rel(xm, x64),
            "relres": {"fp64": out["fp64"][1]["relres"], "mixed": out["mixed"][1]["relres"]},
            "host_assembly_ms": t_asm, "apply_fp64_ms": op.ctx.time_apply(pkg.FP64, 10),
            "apply_fp32_ms": op.ctx.time_apply(pkg.FP32, 10)}
    op.close()
    print(json.dumps(line), flush=True)


def run_sampling(args):
    """Config 4 sampling: 1e5 samples y ~ U[-1,1]^20 (NumPy PCG64, seed 123) on the
    config-1 mesh: per batch of 512, the P2 deterministic problems solved on the
    device (mixed PCG to 1e-10) and the errors of the config-1 SG solution for the
    truncations m = 0..5 (sampling-error kernel)."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    C, V, TB, sol, Ks, b0 = config1_problem(pkg)
    op = pkg.SGOperator(V, TB, Ks, device=0)
    op.solve_primal(b0, sol.entries, rtol=1e-12, precision=pkg.FP64)
    op.close()
    S_total = args.samples
    Ms, B = 20, 512
    rng = np.random.default_rng(123)
    Y = rng.uniform(-1.0, 1.0, size=(Ms, S_total))
    w = np.full(S_total, 0.5 ** Ms)
    f = lambda x, y: np.ones_like(x)
    (res, per), t_all = _timed(lambda: pkg.calculate_sampling_error(
        sol, C, order=2, rhs=f, Msamples=Ms, samples=Y, weights=w, batch=B, rtol=1e-10, precision=pkg.MIXED,
        return_per_sample=True))
    # phase split on one batch
    Vd = pkg.H1Pk(V.mesh, 2)
    Kd = pkg.assemble_stiffness(Vd, C, list(range(Ms + 1)), 12)
    bd = pkg.assemble_rhs(Vd, f, 2)
    sp_ = pkg.SampleProblems(Vd, Kd, Y[:, :B])
    sp_.solve(bd, rtol=1e-10, keep_on_device=True)
    _, t_solve = _timed(lambda: sp_.solve(bd, rtol=1e-10, keep_on_device=True))
    st = sp_.stats
    _, t_err = _timed(lambda: sp_.sampling_error(sol, 4))
    sp_.close()
    line = {"workload": f"sampling: {S_total} samples U[-1,1]^20, config-1 SG solution (P1, P=21) vs P2 "
                        f"deterministic solves on the 32x32 mesh (4225 dofs), batches of {B}, m=0..5",
            "samples_per_s": S_total / (t_all * 1e-3), "total_s": t_all * 1e-3,
            "batch_solve_ms": t_solve, "batch_solve_device_ms": st["time_ms"], "batch_iterations": st["iterations"],
            "batch_error_ms": t_err, "stress_uniform": [float(v) for v in res[2]],
            "u_uniform": [float(v) for v in res[3]]}
    if not args.no_cpu_baseline:
        from oracle import sampling as osm
        from oracle import basis as ob
        from oracle import fem as of
        from oracle import coefficient as oc
        mesh = of.StructuredMesh(32)
        Vo_sg, Vo_det = of.LagrangeSpace(mesh, 1), of.LagrangeSpace(mesh, 2)
        Co = oc.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=150)
        Kdo = [K.tocsr() for K in Kd]
        TBo = ob.TensorizedBasis(ob.LEGENDRE, 5, 2, 6, multi_indices=TB.multi_indices)
        osm.calculate_sampling_error(sol.entries, TBo, Vo_sg, Vo_det, Kdo, bd, Y[:, :1], w[:1], order=2)
        ns = 40
        t = time.perf_counter()
        osm.calculate_sampling_error(sol.entries, TBo, Vo_sg, Vo_det, Kdo, bd, Y[:, :ns], w[:ns], order=2)
        per_sample = (time.perf_counter() - t) / ns
        line["cpu_baseline"] = {"value": 1.0 / per_sample, "unit": "samples/s", "cores": 1, "kind": "port",
                                "sample": f"{ns} samples through the oracle (SuperLU solve of the P2 problem + "
                                          f"vectorised error integrals for m=0..5), single thread"}
    print(json.dumps(line), flush=True)


def run_adjoint(args):
    """Config 5: J = int_[0.25,0.75]^2 E[u] dx, gradient with respect to the KLE
    block factors theta_m and the nodal P1 mean field alpha by one adjoint solve;
    central finite differences (h = 1e-6) on random directions."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    N, M = args.mesh, 20 if args.mesh >= 128 else 5
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=150)
    V = pkg.H1Pk(pkg.unit_square_mesh(N), 1)
    mis = pkg.total_degree_multiindices(M, 2) if M <= 5 else pkg.top_weight_multiindices(M, 150, C.decay_factors)
    deg = max(max(m) for m in mis)
    TB = pkg.TensorizedBasis(pkg.LegendrePolynomials, M, deg, deg + 4, multi_indices=mis)
    Q = pkg.MeanQoI(V, TB, C, rhs=lambda x, y: np.ones_like(x))
    theta, alpha = np.ones(M), np.ones(V.mesh.nnodes)
    # FP64 PCG floor: 1e-12 is attainable on the small mesh only; the finite-difference
    # step grows with the solve tolerance there (error ~ rtol / h + h^2)
    small = N <= 64
    rtol, rtol_fd, h = (1e-12, 2e-13, 1e-6) if small else (1e-10, 1e-10, 1e-4)
    Q.value_and_gradient(theta, alpha, rtol=rtol)
    (r, t_grad) = _timed(lambda: Q.value_and_gradient(theta, alpha, rtol=rtol))
    J, gt, ga, st = r
    (_, t_fwd) = _timed(lambda: Q.value(theta, alpha, rtol=rtol))
    rng = np.random.default_rng(5)
    errs = []
    for _ in range(args.directions):
        dt = rng.standard_normal(M)
        da = rng.standard_normal(V.mesh.nnodes)
        fd = (Q.value(theta + h * dt, alpha + h * da, rtol=rtol_fd) - Q.value(theta - h * dt, alpha - h * da,
                                                                                rtol=rtol_fd)) / (2 * h)
        an = gt @ dt + ga @ da
        errs.append(abs(fd - an) / abs(an))
    line = {"workload": f"adjoint: P1 {N}x{N} ({V.ndofs} nodes), M={M}, P={TB.nmodes}, FP64 PCG to {rtol:g}",
            "fd_step": h, "fd_solve_rtol": rtol_fd,
            "J": J, "gradient_ms_wall": t_grad, "forward_ms_wall": t_fwd, "gradient_cost_vs_forward": t_grad / t_fwd,
            "forward_device_ms": st["forward"]["time_ms"], "adjoint_device_ms": st["adjoint"]["time_ms"],
            "fd_directions": len(errs), "fd_rel_err_max": max(errs) if errs else None,
            "fd_rel_err_median": statistics.median(errs) if errs else None,
            "note": "wall times include host assembly of K_0(alpha) and the context setup in both arms"}
    print(json.dumps(line), flush=True)


def run_batch(args):
    """Config 4 batching: the SG problems of the SplitMix64 stream (seed = problem
    index; n x n P1 mesh with n = 16 + r % 113, M = 4 + r % 13, total degree
    1 + r % 3), all solved together to 1e-8 by the batched PCG with the mean-based
    preconditioner (sine transforms on the unit-square lattice)."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=150)
    shapes = pkg.config4_problems(args.problems)
    B = pkg.SGBatch(0)
    t0 = time.perf_counter()
    unknowns = 0
    bytes32 = 0
    for N, M, d in shapes:
        mis = pkg.total_degree_multiindices(M, d)
        TB = pkg.TensorizedBasis(pkg.LegendrePolynomials, M, d, d + 4, multi_indices=mis)
        V = pkg.H1Pk(pkg.unit_square_mesh(N), 1)
        sol = pkg.SGFEVector(V, TB)
        Ks, b0 = pkg.assemble(pkg.PoissonProblemPrimal, sol, C, rhs=lambda x, y: np.ones_like(x), device=0)
        B.add(V, TB, Ks, b0)
        unknowns += V.ndofs * TB.nmodes
        bytes32 += algorithmic_bytes(V.ndofs, TB.nmodes, Ks[0].nnz, len(Ks), 4)
    t_setup = time.perf_counter() - t0
    t0 = time.perf_counter()
    B.finalize()
    t_fin = time.perf_counter() - t0
    _, st = B.solve(rtol=1e-8, maxit=20000, check_every=16, want_solutions=False)
    line = {"workload": f"batch: {len(shapes)} SG problems (SplitMix64 shapes), {unknowns} unknowns in total, "
                        f"PCG (mean-based sine-transform preconditioner) to 1e-8, one launch per phase",
            "solve_ms": st["time_ms"], "problems_per_s": len(shapes) / (st["time_ms"] * 1e-3),
            "iterations_max": st["iterations_max"], "converged": st["converged"], "relres_max": st["relres_max"],
            "graph_replays": st["graph_replays"], "kernel_launches": st["kernel_launches"],
            "host_setup_s": t_setup, "finalize_s": t_fin, "tuning": B.tuning}
    # the FP32 apply of the chosen form: the fastest timed candidate of the finalize sweep
    import re
    f32 = B.tuning.split("FP32 ", 1)[-1] if "FP32 " in B.tuning else ""
    t32 = [float(v) for v in re.findall(r":([0-9.]+)ms", f32)]
    if t32:
        pk = peaks()
        peak_gbs = pk["hbm_gbs"] if pk else 6800.0
        ach = bytes32 / (min(t32) * 1e-3) / 1e9
        line["apply_fp32"] = {"ms": min(t32), "algorithmic_bytes": bytes32, "GB/s": ach, "frac_hbm": ach / peak_gbs,
                              "peak_source": "MEASURED_PEAKS.json hbm_gbs" if pk else "fallback 6.8 TB/s"}
    B.close()
    print(json.dumps(line), flush=True)


def ctx_qn(op):
    # pair count P + sum_m nzcols(G_m), from the coupling matrix
    G = op.TB.G.tocsr()
    P = op.P
    M = op.M
    q = P
    for m in range(M):
        q += int(np.count_nonzero(np.asarray(np.abs(G[m * P:(m + 1) * P]).sum(axis=0)).ravel()))
    return q


def run_assembly(args):
    """K_0..K_20 of the headline workload (P2 256x256, cosine coefficient, order-4
    cell rule): host assembly (the caller-side restatement) vs sgfem_assemble_stiffness
    (wall time including the pattern and gather lists built on the host)."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=150)
    V = pkg.H1Pk(pkg.unit_square_mesh(args.mesh), 2)
    ms = list(range(21))
    pkg.assemble_stiffness_gpu(V, C, [0], 4)  # context and library warm-up
    t = time.perf_counter()
    Kg = pkg.assemble_stiffness_gpu(V, C, ms, 4)
    t_gpu = (time.perf_counter() - t) * 1e3
    t = time.perf_counter()
    Kh = pkg.assemble_stiffness(V, C, ms, 4)
    t_host = (time.perf_counter() - t) * 1e3
    err = max(float(np.abs(a.data - b.data).max() / np.abs(a.data).max()) for a, b in zip(Kh, Kg))
    line = {"workload": f"assembly: K_0..K_20 of P2 {args.mesh}x{args.mesh} ({V.ndofs} dofs, {Kg[0].nnz} nonzeros), "
                        f"cosine coefficient, order-4 cell rule",
            "gpu_ms_wall": t_gpu, "host_ms_wall": t_host, "speedup": t_host / t_gpu, "max_rel_diff": err}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile", choices=["apply32", "apply64", "precond32", "precond64", "residual", "solve"], default=None,
                    help="profiling target for ncu: set up the workload, run the kernel(s) a few times, exit")
    ap.add_argument("--mesh", type=int, default=256, help="mesh size for --profile / --workload adjoint")
    ap.add_argument("--workload", choices=["config2", "config1", "lognormal", "sampling", "adjoint", "batch",
                                           "assembly", "equilibration", "estimate"],
                    default="config2", help="config2 is the headline bench line; the others print their own line")
    ap.add_argument("--samples", type=int, default=100000, help="--workload sampling: number of samples")
    ap.add_argument("--directions", type=int, default=20, help="--workload adjoint: finite-difference directions")
    ap.add_argument("--restart", type=int, default=100, help="--workload lognormal: GMRES restart length")
    ap.add_argument("--problems", type=int, default=256, help="--workload batch: number of problems")
    ap.add_argument("--rtol", type=float, default=1e-10, help="--workload config1: solve tolerance")
    args = ap.parse_args()
    if args.profile:
        return run_profile(args)
    if args.workload != "config2":
        return {"config1": run_config1, "lognormal": run_lognormal, "sampling": run_sampling,
                "adjoint": run_adjoint, "batch": run_batch, "assembly": run_assembly,
                "equilibration": run_equilibration, "estimate": run_estimate}[args.workload](args)
    rank, world, local, pg = dist_setup(args.gpus)
    if args.impl == "reference":
        run_reference(args, rank, world, pg)
    else:
        import __graft_entry__ as ge
        ge.load_package()
        run_ours(args, rank, world, local, pg)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
