"""Benchmark: DoFs/s of the GMG-preconditioned CG solve to 1e-10 relative
residual (UG4/ugcore FV1 assemble-and-solve path) on one GB300.

Workload (default): 3D Poisson on the unit cube, 2x2x2 hexahedra refined 6
times (129^3 = 2,146,689 DoFs, 57,066,625 nonzeros), FV1, zero Dirichlet
boundary, seeded source f ~ U[-1,1], GMG V(2,2) damped Jacobi (0.6),
StdTransfer, LU base, CG to ||r||/||r0|| < 1e-10 from x0 = 0, FP64.
One "step" = one complete solve on device-resident data.  The matrix
(0.69 GB CRS) is larger than L2 (129 MB), so no L2 flush is needed between
steps.  The mixed-precision (FP32 GMG inside FP64 CG) solve and the assembly
are measured as extra fields.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun with N > 1 every rank solves its own replica on its own GPU
("replicas only": the path has no data exchange at one GPU per problem);
value = N * DoFs / max-over-ranks time per step.  --impl reference times the
CPU oracle port of the reference algebra (oracle/; serial like ugcore's hot
path) on the same workload, one independent replica per host core, rank 0
only.  The `roofline` object gives the top-level FP64 smoother's fraction of
the measured HBM copy bandwidth and, in `roofline.fp64`, of the FP64 rate
measured with cuBLAS DGEMM, the bound that holds for it on GB300.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DoFs/s for GMG-PCG solve to 1e-10 rel (FP64 vs mixed) + adjoint grad time"
# DRAM bytes (read + write) per launch of the top-level FP64 smoothing kernel,
# mean of the two launches captured by
#   ncu --set full --clock-control none -k regex:k_smooth -c 2 -o prof \
#       python bench.py --steps 2 --warmup 3 --no-extras --no-cpu
# (summary in profiles/k_smooth_fp64_poisson129.md); the FP64 pipe was 82 % busy.
NCU_TRAFFIC_TOP_SMOOTH = 512.1e6
NCU_FP64_PIPE_TOP_SMOOTH = 0.82
UNIT = "DoFs/s"
WORKLOAD = "c1: 3D Poisson FP64, unit cube 2x2x2 hex refined 6x (129^3 = 2,146,689 DoFs), GMG V(2,2) Jacobi(0.6)-PCG to 1e-10"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p["hbm_gbs"], "measured"
    except Exception:
        return 6800.0, "fallback"


def fp64_peak_tflops():
    """FP64 throughput measured here: cuBLAS DGEMM 4096^3 (torch.matmul,
    best of 3, CUDA events) -- the denominator of the FP64-pipe fraction of
    the FP64 kernels, which GB300's FP64 rate bounds before HBM"""
    import torch
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    best = None
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        best = ms if best is None else min(best, ms)
    del a, b
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.remove(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for i, nm in enumerate(names):
                if r[5 + i].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


# ----------------------------------------------------- byte accounting ----
def level_sizes(p):
    """(N, nnz, nslices, nnz_P, nnz_R) per level, from the device matrices."""
    import ugcore_gb300 as ug
    out = []
    for l in range(p.hier.num_levels):
        A = ug.GPUSparseMatrix(p.ctx)
        p.disc.assemble_jacobian(A, l)
        n, _, nnz = A.info()
        nP = nR = 0
        if l > p.cfg["base"]:
            nP = len(p.gmg.transfer(l, 0)[1])
            nR = len(p.gmg.transfer(l, 1)[1])
        out.append(dict(N=n, nnz=nnz, ns=(n + 31) // 32, nP=nP, nR=nR))
    return out


def op_bytes(sz, sv):
    """algorithmic bytes of one sweep over a level operator.  Structured levels
    use the constant-offset layout, which needs no column indices: nnz*sv."""
    return sz["nnz"] * sv


def smooth_bytes(sz, sv, top):
    """algorithmic bytes of the 4 fused Jacobi launches of one V(2,2) visit of a level:
    operator values once per launch; vectors once per launch."""
    N, M = sz["N"], op_bytes(sz, sv)
    din = 8 if top else sv                      # top pre-step reads the FP64 defect r
    pre1 = M + N * (din + sv + sv + sv)         # x=d_in, dinv, sc w, d_out w
    pre2 = M + N * (sv + sv + 2 * sv + sv)      # x=d, dinv, sc r/w, d_out w
    post1 = M + N * (sv + sv + sv + 2 * sv + sv)  # w, d_base, dinv, sc r/w, d_out w
    post2 = M + N * (sv + sv + 2 * sv + (8 if top else 0))  # d, dinv, sc r/w, (r for rho)
    return pre1 + pre2 + post1 + post2


def iteration_bytes(sizes, sv):
    """algorithmic bytes of one PCG iteration (V(2,2) cycle + CG kernels).
    The transfers of the structured hierarchy are applied from grid indices
    (no stored P or R): vectors only."""
    L = len(sizes) - 1
    tot = 0
    for l in range(1, L + 1):
        s, c = sizes[l], sizes[l - 1]
        tot += smooth_bytes(s, sv, l == L)
        tot += s["N"] * sv + c["N"] * sv                       # restrict: d read, coarse d written
        tot += c["N"] * sv + s["N"] * (2 * sv + sv + sv)       # prolong: coarse sc, sc r/w, dfac, w
    b = sizes[0]["N"]
    tot += b * b * 8 + 2 * b * sv                                  # dense base solve
    top = sizes[L]
    tot += op_bytes(top, 8) + top["N"] * (sv + 16 + 16)          # q = A z + beta q, p update, (q,p)
    tot += top["N"] * 48                                            # x, r updates + norm
    return tot


def assembly_bytes(p, sz):
    """bytes a top-level assembly must move: the operator's values and the
    rhs written once (8 nnz + 8 N) and, unless one coefficient serves every
    element, the element coefficients read once (8 E); on structured levels
    the geometry is per element class (a few KB) and the pattern is known"""
    N, E = sz["N"], p.hier.num_elements()
    coef = 0 if p.cfg["coef"] == "const" else 8 * E
    return 8 * sz["nnz"] + 8 * N + coef


def profile_summary(prof, top=14):
    """largest per-kernel totals of one profiled solve: tag|kernel -> [launches, ms]"""
    items = sorted(prof.items(), key=lambda kv: -kv[1][1])[:top]
    return {k.replace("decltype(mv)", "MV"): [v[0], round(v[1], 4)] for k, v in items}


def max_over_ranks(v, world):
    """max of a per-rank float over all ranks (NCCL on GPUs, gloo on CPU)."""
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(ms_local, n, world):
    """whole-job DoFs/s of `world` independent replicas of an n-DoF solve:
    world * n / (max over ranks of ms per step)."""
    ms = max_over_ranks(ms_local, world)
    return world * n / (ms * 1e-3), ms


# ------------------------------------------------------------ our arm -----
def run_ours(args, rank, world, local_rank):
    import torch
    import ugcore_gb300 as ug
    from ugcore_gb300 import problems

    jobs = None
    if rank == 0 and world == 1 and not args.no_cpu:
        jobs = OracleJobs(["c1"] + ([] if args.no_extras else ["c2", "c3grad"]))
    torch.cuda.set_device(local_rank)
    ctx = ug.Context(local_rank)
    stream = torch.cuda.ExternalStream(ctx.stream)
    cfg = problems.config("c1", precision="fp64")
    t0 = time.perf_counter()
    p = problems.Problem(ctx, cfg)
    ctx.synchronize()
    setup_s = time.perf_counter() - t0
    n = p.n

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    def timed(fn, steps):
        barrier()
        torch.cuda.synchronize()
        ctx.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        e1.synchronize()
        torch.cuda.synchronize()
        barrier()
        return e0.elapsed_time(e1) / steps

    for _ in range(args.warmup):
        st = p.solve()
    clk = ClockSampler(local_rank)
    clk.start()
    k0 = ctx.kernel_launches()
    ms = timed(p.solve, args.steps)
    launches = ctx.kernel_launches() - k0
    clocks = clk.stop()
    st = p.solve()
    value, ms_max = replica_value(ms, n, world)

    # ---- e2e: C ABI with host buffers (H2D of b, D2H of x inside the region)
    b_host = torch.empty(n, dtype=torch.float64).pin_memory()
    x_host = torch.empty(n, dtype=torch.float64).pin_memory()
    p.b.copy_to(b_host.numpy())
    p.solver.solve_host(b_host, x_host)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        p.solver.solve_host(b_host, x_host)
    e2e_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    e2e_ms = max_over_ranks(e2e_ms, world)

    # ---- live per-kernel timing (CUDA events on the library stream)
    sizes = level_sizes(p)
    ctx.profile_begin()
    p.solve()
    prof = ctx.profile_end()
    iters = st["steps"]
    top = len(sizes) - 1
    hbm, peak_kind = peaks()
    fp64_peak = fp64_peak_tflops()
    smooth = [(k, v) for k, v in prof.items() if k.startswith("L%d|" % top) and "k_smooth" in k]
    s_cnt = sum(v[0] for _, v in smooth)
    s_ms = sum(v[1] for _, v in smooth)
    visits = s_cnt / 4.0
    s_bytes = smooth_bytes(sizes[top], 8, True) * visits
    achieved = s_bytes / (s_ms * 1e-3) / 1e9
    total_prof_ms = sum(v[1] for v in prof.values())
    it_bytes = iteration_bytes(sizes, 8)
    solve_gbs = it_bytes * iters / (ms * 1e-3) / 1e9

    # ---- mixed precision variant of the same workload
    mixed = None
    if not args.no_extras:
        pm = problems.Problem(ctx, problems.config("c1", precision="mixed"))
        for _ in range(args.warmup):
            pm.solve()
        ms_m = max_over_ranks(timed(pm.solve, args.steps), world)
        ctx.profile_begin()
        pm.solve()
        prof_m = ctx.profile_end()
        stm = pm.solve()
        xm, x64 = pm.x.numpy(), p.x.numpy()
        xo = jobs.solution("c1") if jobs else None
        mixed = {"value": world * n / (ms_m * 1e-3), "ms_per_step": ms_m, "steps_pcg": stm["steps"],
                 "speedup_vs_fp64": ms_max / ms_m,
                 "rel_residual": stm["defect"] / stm["initial_defect"],
                 "max_rel_diff_vs_fp64_solution": float(abs(xm - x64).max() / abs(x64).max()),
                 "max_rel_err_vs_fp64_oracle": None if xo is None else float(abs(xm - xo).max() / abs(xo).max()),
                 "hbm_gbs_solve": iteration_bytes(sizes, 4) * stm["steps"] / (ms_m * 1e-3) / 1e9,
                 "kernel_profile": profile_summary(prof_m)}
        del pm

    target = adj = conv = rap = unstr = smoothers = None
    if not args.no_extras:
        target = run_target(args, ctx, timed, world, hbm, jobs)
        adj = run_adjoint_grad(args, ctx, timed)
        conv = run_convection_adjoint(args, ctx, timed, world, hbm)
        rap = run_galerkin(args, ctx, timed, world)
        unstr = run_unstructured(args, ctx, timed, world, hbm)
        smoothers = run_smoothers(args, ctx, timed, world)

    # ---- assembly throughput (top level, FP64 FV1 + CRS values + rhs)
    asm = None
    if not args.no_extras:
        A2 = ug.GPUSparseMatrix(ctx)
        b2 = ug.GPUVector(ctx, n)
        p.disc.assemble_linear(A2, b2)   # pattern build (first call)
        ms_a = timed(lambda: p.disc.assemble_linear(A2, b2), 3)
        asm = {"ms": ms_a, "dofs_per_s": n / (ms_a * 1e-3),
               "gbs": assembly_bytes(p, sizes[top]) / (ms_a * 1e-3) / 1e9, "setup_s_all_levels": setup_s}

    cpu = cpu_c2 = cpu_c3 = None
    if jobs:
        cpu = cpu_baseline_from(jobs, "c1", "c1")
        if not args.no_extras:
            cpu_c2 = cpu_baseline_from(jobs, "c2", "c2 (FP64)")
            r = jobs.results().get("c3grad", {})
            cpu_c3 = r if "error" in r or not r else {
                "value": r["ms"], "unit": "ms per gradient", "cores": 1, "kind": "port",
                "sample": "best of 3 full gradients dJ/dm of the 257^2 problem (%d DoFs, %d elements): "
                          "assembly and multigrid set-up, forward CG, transposed set-up and CG, element "
                          "gradient" % (r["n"], r["elements"])}
        jobs.close()

    if rank != 0:
        return None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded splitmix64 source, structured grid)",
        "config": {"workload": WORKLOAD, "dofs": n, "nnz": sizes[top]["nnz"], "pcg_steps": iters,
                   "rel_residual": st["defect"] / st["initial_defect"], "levels": len(sizes),
                   "l2": "inputs larger than L2 (matrix %.2f GB > 129 MB), no flush" % (sizes[top]["nnz"] * 12e-9),
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "e2e": {"value": world * n / (e2e_ms * 1e-3), "unit": UNIT, "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": 8 * n, "d2h_bytes_per_step": 8 * n,
                "api": "ug4gb_solver_solve_host (C ABI, pinned host b in, x out)"},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": "k_smooth (fused damped-Jacobi SpMV, top level, 4 launches/cycle)",
                     "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "peak_kind": peak_kind, "traffic": NCU_TRAFFIC_TOP_SMOOTH,
                     "limiter": "FP64 FMA pipe (%.0f%% busy in ncu): 27 FP64 FMAs per row" % (100 * NCU_FP64_PIPE_TOP_SMOOTH),
                     "bytes_per_launch": s_bytes / max(s_cnt, 1), "avg_launch_ms": s_ms / max(s_cnt, 1),
                     "share_of_solve": s_ms / total_prof_ms if total_prof_ms else None,
                     # the bound that holds: 28 FP64 FMAs per row (27 diagonals + the Jacobi update)
                     "fp64": {"achieved_tflops": 56.0 * n / (s_ms / max(s_cnt, 1) * 1e-3) / 1e12,
                              "peak_tflops": fp64_peak, "peak_kind": "measured (cuBLAS DGEMM 4096^3)",
                              "frac": 56.0 * n / (s_ms / max(s_cnt, 1) * 1e-3) / 1e12 / fp64_peak}},
        "solve_roofline": {"achieved": solve_gbs, "peak": hbm, "unit": "GB/s", "frac": solve_gbs / hbm,
                           "bytes_per_iteration": it_bytes},
        "kernel_profile": profile_summary(prof),
        "mixed": mixed,
        "variable_coefficient_tets": target,
        "adjoint_gradient": adj,
        "convection_adjoint": conv,
        "galerkin_coarse_operators": rap,
        "unstructured_tets": unstr,
        "smoothers_convection": smoothers,
        "assembly": asm,
        "clocks": clocks,
        "cpu_baseline": cpu,
    }
    if not args.no_extras:
        line["headline"] = headline_summary(mixed, target, adj, conv, asm, cpu, cpu_c2, cpu_c3)
    return line


def _r(x, nd=4):
    return None if x is None else float("%.*g" % (nd, x))


def headline_summary(mixed, target, adj, conv, asm, cpu_c1, cpu_c2, cpu_c3):
    """the numbers the target of this path is stated in, in one compact
    object at the end of the line: the 3D variable-coefficient problem with
    the FP32 multigrid (time, HBM fraction of the whole solve, speed-up over
    FP64, error against the FP64 oracle), the adjoint-gradient times, the
    mixed-precision error of every configuration, and the CPU baselines"""
    tf, tm = target["fp64"], target["mixed"]
    out = {
        "c2_mixed_ms": _r(tm["ms_per_step"]), "c2_fp64_ms": _r(tf["ms_per_step"]),
        "c2_mixed_speedup_vs_fp64": _r(target["mixed_speedup_vs_fp64"]),
        "c2_mixed_solve_hbm_frac": _r(tm["solve_frac_of_measured_hbm"]),
        "c2_mixed_pcg_steps": tm["pcg_steps"], "c2_fp64_pcg_steps": tf["pcg_steps"],
        "c2_mixed_max_rel_err_vs_fp64_oracle": _r(target.get("max_rel_err_mixed_vs_fp64_oracle")),
        "c1_mixed_ms": _r(mixed["ms_per_step"]), "c1_mixed_speedup_vs_fp64": _r(mixed["speedup_vs_fp64"]),
        "c1_mixed_max_rel_err_vs_fp64_oracle": _r(mixed.get("max_rel_err_vs_fp64_oracle")),
        "c3_grad_ms_fp64": _r(adj["fp64_ms"]), "c3_grad_ms_mixed": _r(adj["mixed_ms"]),
        "c4_mixed_ms": _r(conv["mixed"]["ms_per_solve"]), "c4_fp64_ms": _r(conv["fp64"]["ms_per_solve"]),
        "c4_mixed_adjoint_ms": _r(conv["mixed"].get("adjoint_ms")),
        "c4_mixed_max_rel_diff_vs_gpu_fp64": _r(conv.get("max_rel_diff_mixed_vs_fp64")),
        "c1_assembly_ms": _r(asm["ms"]) if asm else None,
        "cpu_1core_c1_fp64_dofs_per_s": _r(cpu_c1.get("value")) if cpu_c1 else None,
        "cpu_1core_c2_fp64_dofs_per_s": _r(cpu_c2.get("value")) if cpu_c2 else None,
        "cpu_1core_c3_grad_ms": _r(cpu_c3.get("value")) if cpu_c3 else None,
    }
    if cpu_c2 and cpu_c2.get("value"):
        out["c2_mixed_vs_cpu_1core"] = _r(tm["dofs_per_s"] / cpu_c2["value"])
    if cpu_c3 and cpu_c3.get("value"):
        out["c3_grad_fp64_vs_cpu_1core"] = _r(cpu_c3["value"] / adj["fp64_ms"])
    return out


def run_target(args, ctx, timed, world, hbm, jobs=None):
    """3D variable-coefficient diffusion on Kuhn tetrahedra (4^3 hexes x 6 tets,
    refined 5 times, K = exp(2 g), g a 64-mode Gaussian field): FP64 GMG-PCG
    against FP32-GMG-in-FP64-CG, both to 1e-10."""
    from ugcore_gb300 import problems
    out = {"workload": "3D variable-coefficient diffusion, tets (4^3 hexes x 6, refined 5x), K=exp(2g), "
                       "GMG V(2,2) Jacobi(0.6)-PCG to 1e-10"}
    xs, res = {}, {}
    for prec in ("fp64", "mixed"):
        p = problems.Problem(ctx, problems.config("c2", precision=prec))
        for _ in range(args.warmup):
            p.solve()
        ms = max_over_ranks(timed(p.solve, args.steps), world)
        st = p.solve()
        sizes = level_sizes(p)
        sv = 8 if prec == "fp64" else 4
        gbs = iteration_bytes(sizes, sv) * st["steps"] / (ms * 1e-3) / 1e9
        xs[prec] = p.x.numpy()
        res[prec] = {"ms_per_step": ms, "dofs_per_s": world * p.n / (ms * 1e-3), "pcg_steps": st["steps"],
                     "rel_residual": st["defect"] / st["initial_defect"],
                     "solve_gbs": gbs, "solve_frac_of_measured_hbm": gbs / hbm}
        out["dofs"], out["nnz"] = p.n, sizes[-1]["nnz"]
        del p
    out.update(res)
    out["mixed_speedup_vs_fp64"] = res["fp64"]["ms_per_step"] / res["mixed"]["ms_per_step"]
    out["max_rel_diff_mixed_vs_fp64"] = float(abs(xs["mixed"] - xs["fp64"]).max() / abs(xs["fp64"]).max())
    xo = jobs.solution("c2") if jobs else None
    if xo is not None:
        out["max_rel_err_mixed_vs_fp64_oracle"] = float(abs(xs["mixed"] - xo).max() / abs(xo).max())
        out["max_rel_err_fp64_vs_fp64_oracle"] = float(abs(xs["fp64"] - xo).max() / abs(xo).max())
    return out


def run_adjoint_grad(args, ctx, timed):
    """time of one full gradient dJ/dm (forward assemble + solve, transposed
    GMG-PCG solve, element adjoint kernel) through the autograd Function, on
    the 257x257 quadrilateral inverse problem, FP64 and mixed."""
    import numpy as np
    import torch
    from ugcore_gb300 import adjoint, problems
    out = {"workload": "2D inverse problem 257x257 quads, J = 0.5||u(m) - u_obs||^2, dJ/dm per element"}
    for prec in ("fp64", "mixed"):
        cfg = problems.config("c3", precision=prec)
        prob = adjoint.DifferentiableProblem(ctx, cfg)
        m = torch.tensor(prob.m_top, dtype=torch.float64, device="cuda")
        f = torch.ones(prob.n, dtype=torch.float64, device="cuda")
        u_obs = torch.zeros(prob.n, dtype=torch.float64, device="cuda")

        def grad():
            mm = m.clone().requires_grad_(True)
            u = adjoint.fv1_solve(mm, f, prob)
            (0.5 * ((u - u_obs) ** 2).sum()).backward()
            return mm.grad

        for _ in range(args.warmup):
            grad()
        # each gradient timed on its own (it ends with a host wait for the
        # adjoint solve's statistics anyway); the median is reported, so that
        # a host hiccup in one step does not move the number
        times = []
        for _ in range(args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            grad()
            torch.cuda.synchronize()
            times.append((time.perf_counter() - t0) * 1e3)
        out[prec + "_ms"] = float(np.median(times))
        out[prec + "_ms_mean"] = float(np.mean(times))
        out["dofs"], out["elements"] = prob.n, prob.num_elements
        del prob
    return out


def run_convection_adjoint(args, ctx, timed, world, hbm):
    """3D convection-diffusion, 3^3 hexes refined 6 times (193^3 = 7,189,057
    DoFs), D = 1e-2, v = curl of a 16-mode potential at cell Peclet 10, full
    upwind: GMG-preconditioned BiCGStab to 1e-10 in FP64 and with the FP32
    multigrid; then the adjoint of J = sum of u^2 over a seeded 10% vertex
    subset: one transposed BiCGStab solve with the transposed multigrid plus
    the source-gradient kernel (dJ/df per vertex).  Bytes per BiCGStab half
    step are counted as one V-cycle plus one FP64 operator pass and six
    vector passes."""
    import numpy as np
    import ugcore_gb300 as ug
    from ugcore_gb300 import problems
    out = {"workload": "3D convection-diffusion 193^3 hexes (7.19M DoFs), D=1e-2, cell Peclet 10, full upwind, "
                       "GMG V(2,2) Jacobi(0.6)-BiCGStab to 1e-10; adjoint dJ/df for J = sum_S u^2"}
    xs = {}
    for prec in ("fp64", "mixed"):
        p = problems.Problem(ctx, problems.config("c4", precision=prec))
        for _ in range(min(args.warmup, 2)):
            p.solve()
        steps = max(2, args.steps // 3)
        ms = max_over_ranks(timed(p.solve, steps), world)
        st = p.solve()
        sizes = level_sizes(p)
        sv = 8 if prec == "fp64" else 4
        gbs = iteration_bytes(sizes, sv) * st["steps"] / (ms * 1e-3) / 1e9
        res = {"ms_per_solve": ms, "dofs_per_s": world * p.n / (ms * 1e-3), "bicgstab_half_steps": st["steps"],
               "rel_residual": st["defect"] / st["initial_defect"], "solve_gbs": gbs,
               "solve_frac_of_measured_hbm": gbs / hbm}
        if prec == "mixed":
            # adjoint: rhs = dJ/du on a seeded 10% subset, Dirichlet entries zero
            u = p.x.numpy()
            S = np.random.default_rng(p.cfg["seed"]).random(p.n) < 0.1
            p.adjoint_solve(np.where(S, 2.0 * u, 0.0))      # builds A^T, the transposed multigrid, fills rhs
            gf = ug.GPUVector(ctx, p.n)

            def adjoint_step():
                p.lam.set(0.0)
                p.solverT.apply(p.lam, p.rhs)
                p.disc.grad_source(p.lam, out=gf)
            adjoint_step()
            ms_a = max_over_ranks(timed(adjoint_step, steps), world)
            sta = p.solverT.stats()
            res["adjoint_ms"] = ms_a
            res["adjoint_half_steps"] = sta["steps"]
            res["adjoint_rel_residual"] = sta["defect"] / sta["initial_defect"]
        out[prec] = res
        out["dofs"], out["nnz"] = p.n, sizes[-1]["nnz"]
        xs[prec] = p.x.numpy()
        del p
    out["mixed_speedup_vs_fp64"] = out["fp64"]["ms_per_solve"] / out["mixed"]["ms_per_solve"]
    # the GPU FP64 solution of this problem matches the FP64 oracle to 1e-8
    # (tests/test_gpu_full_size.py); the oracle itself needs minutes here
    out["max_rel_diff_mixed_vs_fp64"] = float(abs(xs["mixed"] - xs["fp64"]).max() / abs(xs["fp64"]).max())
    return out


def run_smoothers(args, ctx, timed, world):
    """the smoothers on the 193^3 convection-diffusion problem (mixed
    precision, BiCGStab to 1e-10): damped Jacobi, multicolour Gauss-Seidel,
    its symmetric variant and multicolour ILU(0), time per solve and half
    steps"""
    from ugcore_gb300 import problems
    out = {"workload": "3D convection-diffusion 193^3 hexes (7.19M DoFs), GMG V(2,2) mixed precision, "
                       "BiCGStab to 1e-10, by smoother"}
    for sm, damp in (("jacobi", 0.6), ("mcgs", 1.0), ("mcsgs", 1.0), ("ilu", 1.0)):
        p = problems.Problem(ctx, problems.config("c4", precision="mixed", smoother=sm, damp=damp))
        for _ in range(min(args.warmup, 2)):
            p.solve()
        ms = max_over_ranks(timed(p.solve, max(2, args.steps // 3)), world)
        st = p.solve()
        out[sm] = {"ms_per_solve": ms, "bicgstab_half_steps": st["steps"],
                   "rel_residual": st["defect"] / st["initial_defect"]}
        del p
    return out


def run_galerkin(args, ctx, timed, world):
    """set_rap(true): coarse operators R A P (GPU sparse triple product)
    against re-assembly, on the 129^3 hex Poisson (FP64) and lognormal tet
    (mixed) problems: multigrid set-up time (host clock around init, which
    ends with a synchronisation) and the solve."""
    from ugcore_gb300 import problems
    out = {}
    for name, prec in (("c1", "fp64"), ("c2", "mixed")):
        res = {}
        for rap in (False, True):
            p = problems.Problem(ctx, problems.config(name, precision=prec, rap=rap))
            t0 = time.perf_counter()
            p.gmg.init(p.A)
            p.solver.init(p.A)
            init_s = time.perf_counter() - t0
            for _ in range(min(args.warmup, 2)):
                p.solve()
            ms = max_over_ranks(timed(p.solve, max(2, args.steps // 3)), world)
            st = p.solve()
            res["rap" if rap else "reassembly"] = {"gmg_init_s": init_s, "ms_per_solve": ms,
                                                   "pcg_steps": st["steps"],
                                                   "rel_residual": st["defect"] / st["initial_defect"]}
            del p
        out["%s_%s" % (name, prec)] = res
    return out


def sell_iteration_bytes(sizes, sv):
    """algorithmic bytes of one PCG iteration on an unstructured hierarchy:
    SELL-32 operators (values + 32-bit column indices per stored entry) and
    stored P / R, otherwise as iteration_bytes"""
    L = len(sizes) - 1
    tot = 0
    for l in range(1, L + 1):
        s, c = sizes[l], sizes[l - 1]
        M = s["nnz"] * (sv + 4)
        tot += smooth_bytes(dict(s, nnz=0), sv, l == L) + 4 * M
        tot += s["nR"] * (sv + 4) + s["N"] * sv + c["N"] * sv          # R d
        tot += s["nP"] * (sv + 4) + c["N"] * sv + s["N"] * (4 * sv)    # sc += dfac * (P sc_c)
    b = sizes[0]["N"]
    tot += b * b * 8 + 2 * b * sv
    top = sizes[L]
    tot += top["nnz"] * 12 + top["N"] * (sv + 16 + 16) + top["N"] * 48
    return tot


def run_unstructured(args, ctx, timed, world, hbm):
    """Unstructured tetrahedral hierarchy: the 12-tetrahedron unit-cube UGX
    grid (tests/golden/grids/cube_tets.ugx) refined 7 times regularly
    (25.2M tets, 4.26M DoFs), K = exp(2 g), Dirichlet subset "Bottom";
    GMG V(2,2) Jacobi(0.6) on assembled P/R and SELL-32 operators, PCG to
    1e-10, FP64 and mixed precision."""
    import ctypes as C
    import ugcore_gb300 as ug
    from ugcore_gb300 import _lib, fields
    nref = 7
    t0 = time.perf_counter()
    hier = ug.UnstructuredHierarchy.from_ugx(ctx, os.path.join(ROOT, "tests", "golden", "grids", "cube_tets.ugx"),
                                             nref, "Bottom")
    grid_s = time.perf_counter() - t0
    n = hier.num_vertices()
    disc = ug.DomainDiscretization(hier)
    disc.set_diffusion_field(fields.ScalarField(3, 64, 8.0, 1 ^ fields.COEF_SEED_XOR), factor=2.0)
    disc.set_source_uniform(1)
    A = ug.GPUSparseMatrix(ctx)
    b = ug.GPUVector(ctx, n)
    disc.assemble_linear(A, b)
    ms_asm = timed(lambda: disc.assemble_linear(A, b), 3)
    out = {"workload": "unstructured tets: 12-tet unit cube (UGX) refined 7x regularly, K=exp(2g), "
                       "GMG V(2,2) Jacobi(0.6)-PCG to 1e-10, SELL-32 operators, stored P/R",
           "dofs": n, "elements": hier.num_elements(), "hierarchy_setup_s": grid_s,
           "assembly_ms": ms_asm, "assembly_dofs_per_s": n / (ms_asm * 1e-3)}
    for prec in ("fp64", "mixed"):
        gmg = ug.GeometricMultiGrid(disc)
        gmg.set_smoother(ug.Jacobi(0.6))
        gmg.set_precision(prec)
        t0 = time.perf_counter()
        gmg.init(A)
        init_s = time.perf_counter() - t0
        solver = ug.CG(ctx)
        solver.set_preconditioner(gmg)
        solver.set_convergence_check(ug.StdConvCheck(200, 1e-300, 1e-10))
        solver.init(A)
        x = ug.GPUVector(ctx, n)

        def solve():
            x.set(0.0)
            solver.apply(x, b)
        for _ in range(min(args.warmup, 3)):
            solve()
        ms = max_over_ranks(timed(solve, max(2, args.steps // 3)), world)
        st = solver.stats()
        sizes = []
        for l in range(hier.num_levels):
            r, nnz = C.c_int(), C.c_int64()
            _lib.check(_lib.lib().ug4gb_gmg_level_info(gmg.h, l, C.byref(r), C.byref(nnz)))
            nP = nR = 0
            if l > 0:
                rr, cc, z = C.c_int(), C.c_int(), C.c_int64()
                _lib.check(_lib.lib().ug4gb_gmg_transfer_info(gmg.h, l, 0, C.byref(rr), C.byref(cc), C.byref(z)))
                nP = z.value
                _lib.check(_lib.lib().ug4gb_gmg_transfer_info(gmg.h, l, 1, C.byref(rr), C.byref(cc), C.byref(z)))
                nR = z.value
            sizes.append(dict(N=r.value, nnz=nnz.value, nP=nP, nR=nR))
        gbs = sell_iteration_bytes(sizes, 8 if prec == "fp64" else 4) * st["steps"] / (ms * 1e-3) / 1e9
        out[prec] = {"ms_per_solve": ms, "dofs_per_s": world * n / (ms * 1e-3), "pcg_steps": st["steps"],
                     "rel_residual": st["defect"] / st["initial_defect"], "gmg_init_s": init_s,
                     "solve_gbs": gbs, "solve_frac_of_measured_hbm": gbs / hbm}
        out["nnz"] = sizes[-1]["nnz"]
        del solver, gmg
    out["mixed_speedup_vs_fp64"] = out["fp64"]["ms_per_solve"] / out["mixed"]["ms_per_solve"]
    return out


def _oracle_params(name):
    """oracle parameters of a benchmark configuration (FP64, as ugcore runs it)"""
    from oracle import oracle as orc
    from ugcore_gb300 import problems
    c = problems.config(name, precision="fp64")
    et = {"quad": orc.ORC_QUAD, "hex": orc.ORC_HEX, "tet": orc.ORC_TET}[c["elem"]]
    ck = {"const": 0 if c["diffusion"] == 1.0 else 3, "lognormal": 1, "logk": 2}[c["coef"]]
    return orc.make_params(elem_type=et, mx=c["mx"], my=c["my"], mz=c["mz"], nref=c["nref"], seed=c["seed"],
                           coef_kind=ck, coef_modes=c["coef_modes"], coef_kmax=c["coef_kmax"],
                           vel_kind=1 if c["vel"] else 0, vel_modes=c["vel_modes"], vel_kmax=c["vel_kmax"],
                           diffusion=c["diffusion"], peclet=c["peclet"], solver=0 if c["solver"] == "cg" else 1,
                           damp=c["damp"], nu1=c["nu1"], nu2=c["nu2"], maxit=c["maxit"], rel_red=c["rel_red"])


def _oracle_job(name, out_dir, q):
    """CPU baseline legs (run in a spawned process, one core each): the
    oracle port of the reference path on a benchmark configuration.
    "c1"/"c2": assembly + multigrid set-up, then one full FP64 solve (timed;
    the solution is kept to state the mixed-precision error against it).
    "c3grad": one full adjoint gradient dJ/dm of the 257^2 inverse problem
    as the GPU leg computes it (f = 1, J = 0.5 |u|^2): set-up, forward solve,
    transposed set-up and solve, element gradient."""
    import numpy as np
    from oracle import oracle as orc
    from ugcore_gb300 import fields, problems
    try:
        if name in ("c1", "c2"):
            t0 = time.perf_counter()
            P = orc.Problem(_oracle_params(name))
            t1 = time.perf_counter()
            s = P.solve()
            t2 = time.perf_counter()
            path = os.path.join(out_dir, name + ".npy")
            np.save(path, s["x"])
            q.put((name, {"setup_s": t1 - t0, "solve_s": t2 - t1, "steps": s["steps"], "n": P.nv(), "x": path}))
        elif name == "c3grad":
            c = problems.config("c3", precision="fp64")
            par = _oracle_params("c3")
            par.coef_kind = 0
            coords, elems, _ = orc.Problem(par).level_geometry()
            m = fields.ScalarField(2, c["coef_modes"], c["coef_kmax"], c["seed"] ^ fields.COEF_SEED_XOR)(
                coords[elems].mean(axis=1))
            f = np.ones(len(coords))
            times = []
            for _ in range(3):
                t0 = time.perf_counter()
                P = orc.Problem(_oracle_params("c3"), m_top=m, f_top=f)
                u = P.solve()["x"]
                lam = P.adjoint(u)["lam"]
                P.grad_logk(u, lam)
                times.append(time.perf_counter() - t0)
                del P
            q.put((name, {"ms": 1e3 * min(times), "n": len(coords), "elements": len(elems)}))
    except Exception as ex:  # reported, never fatal for the GPU legs
        q.put((name, {"error": repr(ex)}))


class OracleJobs:
    """the CPU baseline legs, started in spawned processes before the GPU
    work so that they run beside it (a forked child of a CUDA process is not
    safe; spawn is)"""

    def __init__(self, names):
        import multiprocessing as mp
        from oracle import oracle as orc
        orc.build()
        self.dir = tempfile.mkdtemp(prefix="ug4gb_bench_")
        ctx = mp.get_context("spawn")
        self.q = ctx.Queue()
        self.procs = [ctx.Process(target=_oracle_job, args=(nm, self.dir, self.q)) for nm in names]
        for pr in self.procs:
            pr.start()
        self.res = {}

    def results(self, timeout=600.0):
        t_end = time.time() + timeout
        while len(self.res) < len(self.procs) and time.time() < t_end:
            try:
                name, r = self.q.get(timeout=max(0.1, t_end - time.time()))
                self.res[name] = r
            except Exception:
                break
        for pr in self.procs:
            pr.join(timeout=1.0)
        return self.res

    def solution(self, name):
        import numpy as np
        r = self.results().get(name, {})
        return np.load(r["x"]) if "x" in r else None

    def close(self):
        import shutil
        for pr in self.procs:
            if pr.is_alive():
                pr.terminate()
        shutil.rmtree(self.dir, ignore_errors=True)


def cpu_baseline_from(jobs, name, label):
    """cpu_baseline object of one oracle solve leg"""
    r = jobs.results().get(name)
    if not r or "error" in r:
        return {"error": (r or {}).get("error", "not finished")}
    return {"value": r["n"] / r["solve_s"], "unit": UNIT, "cores": 1, "kind": "port",
            "sample": "one full %s solve (%d DoFs, %d steps, %.2f s) after %.1f s of assembly/set-up; "
                      "single thread like ugcore's hot path" % (label, r["n"], r["steps"], r["solve_s"], r["setup_s"])}


# ------------------------------------------------------ reference arm -----
def _reference_worker(steps, warmup, barrier, out):
    """one replica of the reference arm: the oracle port solving the c1
    workload (its own process, one core)"""
    from oracle import oracle as orc
    P = orc.Problem(orc.make_params(elem_type=orc.ORC_HEX, mx=2, my=2, mz=2, nref=6, seed=1))
    for _ in range(warmup):
        P.solve()
    barrier.wait()
    t0 = time.perf_counter()
    s = None
    for _ in range(steps):
        s = P.solve()
    t1 = time.perf_counter()
    out.put((t0, t1, s["steps"], P.nv()))


def run_reference(args, rank, world):
    """The reference's CPU path on all host cores: the serial oracle port (the
    reference hot path is single-threaded, OpenMP off, ugcore
    cmake/ug_includes.cmake:188) run as one independent replica per core, each
    solving the c1 workload; value = replicas x DoFs / wall time per step."""
    if rank != 0:
        return None
    import multiprocessing as mp
    from oracle import oracle as orc
    orc.build()
    nw = int(os.environ.get("UG4GB_REFERENCE_WORKERS", "0")) or (os.cpu_count() or 1)
    warm = args.warmup
    ctx = mp.get_context("spawn")
    barrier = ctx.Barrier(nw)
    out = ctx.Queue()
    procs = [ctx.Process(target=_reference_worker, args=(args.steps, warm, barrier, out)) for _ in range(nw)]
    for pr in procs:
        pr.start()
    res = [out.get() for _ in range(nw)]
    for pr in procs:
        pr.join()
    wall = max(r[1] for r in res) - min(r[0] for r in res)
    ms = 1e3 * wall / args.steps
    n = res[0][3]
    value = nw * n / (ms * 1e-3)
    return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": warm, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded splitmix64 source, structured grid)",
            "impl": "reference",
            "config": {"workload": WORKLOAD, "dofs": n, "pcg_steps": res[0][2]},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nw, "kind": "port",
                             "sample": "%d concurrent replicas (one process per host core) of the full c1 solve; "
                                       "each step = one solve per replica" % nw},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1 and args.impl == "ours":
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    if args.impl == "reference":
        line = run_reference(args, rank, world)
    else:
        line = run_ours(args, rank, world, local_rank)
    if line is not None:
        print(json.dumps(line))
    if world > 1 and args.impl == "ours":
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
