"""Solve one named configuration on cuda:0 a few times and print the solver
statistics as JSON, e.g. to profile one precision or layout in isolation:

    python -m ugcore_gb300.run_case --config c2 --precision mixed --solves 2
    python -m ugcore_gb300.run_case --config c1 --nref 5 --format sell
    python -m ugcore_gb300.run_case --config c2 --precision mixed --direct --sweep-fusion 1

--assemblies N re-assembles the top-level operator and rhs N times after
the set-up and reports the time per assembly (--row-assembly 0 selects the
element kernel instead of the row-wise one on structured levels, 1 the
row-wise kernel also with a constant coefficient, 2 the default):

    python -m ugcore_gb300.run_case --config c1 --solves 0 --assemblies 3

--coarse-levels K cycles the base and K levels above it in one launch (-1
the default choice, 0 none):

    python -m ugcore_gb300.run_case --config c3 --direct --coarse-levels 3

--gradients N times N adjoint gradients dJ/dm of J = 0.5 |u(m)|^2 through
torch.autograd (forward assembly and solve, transposed solve, element
gradient) on the configuration's problem with a per-element log coefficient:

    python -m ugcore_gb300.run_case --config c3 --solves 0 --gradients 5

--ugx FILE runs an unstructured hierarchy instead (the UGX coarse grid refined
--nref times, Dirichlet subsets --dirichlet, lognormal K, CG, Jacobi V(2,2)):

    python -m ugcore_gb300.run_case --ugx tests/golden/grids/cube_tets.ugx --nref 7 --dirichlet Bottom

--direct runs the solves with the library profiler on: every kernel is
launched directly instead of being replayed from the solve's CUDA graph
(profilers cannot attribute kernels inside graphs with conditional nodes),
and the per-kernel CUDA-event totals are printed with the statistics.

Configurations: c0 2D Poisson 129^2 quads, c1 3D Poisson 129^3 hexes,
c2 3D lognormal diffusion on Kuhn tets (129^3 vertices), c3 2D log-K field
257^2 quads, c4 3D convection-diffusion 193^3 hexes (BiCGStab).
"""
import argparse
import json
import time


class _UgxProblem:
    """the solve of one unstructured hierarchy, with Problem's solve()"""

    def __init__(self, ctx, args):
        import ugcore_gb300 as ug
        from ugcore_gb300 import fields
        self.hier = ug.UnstructuredHierarchy.from_ugx(ctx, args.ugx, 3 if args.nref is None else args.nref,
                                                      args.dirichlet)
        self.n = self.hier.num_vertices()
        self.disc = ug.DomainDiscretization(self.hier)
        self.disc.set_diffusion_field(fields.ScalarField(self.hier.dim, 64, 8.0, 1 ^ fields.COEF_SEED_XOR),
                                      factor=2.0)
        self.disc.set_source_uniform(1)
        self.A = ug.GPUSparseMatrix(ctx)
        self.b = ug.GPUVector(ctx, self.n)
        self.disc.assemble_linear(self.A, self.b)
        self.gmg = ug.GeometricMultiGrid(self.disc)
        self.gmg.set_smoother({None: lambda: ug.Jacobi(0.6), "jacobi": lambda: ug.Jacobi(0.6),
                               "mcgs": lambda: ug.GaussSeidel(1.0), "mcsgs": lambda: ug.SymmetricGaussSeidel(1.0),
                               "ilu": lambda: ug.ILU(1.0)}[args.smoother]())
        self.gmg.set_precision(args.precision or "fp64")
        self.gmg.init(self.A)
        self.solver = ug.CG(ctx)
        self.solver.set_preconditioner(self.gmg)
        self.solver.set_convergence_check(ug.StdConvCheck(200, 1e-300, 1e-10))
        self.solver.init(self.A)
        self.x = ug.GPUVector(ctx, self.n)

    def solve(self):
        self.x.set(0.0)
        self.solver.apply(self.x, self.b)
        return self.solver.stats()


def ugx_problem(ctx, args):
    return _UgxProblem(ctx, args)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="c1")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default=None)
    ap.add_argument("--nref", type=int, default=None)
    ap.add_argument("--smoother", choices=["jacobi", "mcgs", "mcsgs", "ilu"], default=None)
    ap.add_argument("--format", choices=["auto", "sell"], default="auto")
    ap.add_argument("--solves", type=int, default=1)
    ap.add_argument("--direct", action="store_true")
    ap.add_argument("--sweep-fusion", type=int, default=None)
    ap.add_argument("--sweep-planes", type=int, default=None)
    ap.add_argument("--ugx", default=None)
    ap.add_argument("--dirichlet", default=None)
    ap.add_argument("--assemblies", type=int, default=0)
    ap.add_argument("--row-assembly", type=int, default=None)
    ap.add_argument("--coarse-levels", type=int, default=None)
    ap.add_argument("--gradients", type=int, default=0)
    args = ap.parse_args()

    import ugcore_gb300 as ug
    from ugcore_gb300 import problems
    over = {}
    if args.precision:
        over["precision"] = args.precision
    if args.nref is not None:
        over["nref"] = args.nref
    if args.smoother:
        over["smoother"] = args.smoother
        over["damp"] = 0.6 if args.smoother == "jacobi" else 1.0
    ctx = ug.Context(0)
    ctx.set_operator_format(args.format)
    ctx.set_tuning(sweep_fusion=args.sweep_fusion, sweep_planes=args.sweep_planes,
                   row_assembly=args.row_assembly, coarse_levels=args.coarse_levels)
    t0 = time.perf_counter()
    p = ugx_problem(ctx, args) if args.ugx else problems.Problem(ctx, problems.config(args.config, **over))
    ctx.synchronize()
    setup = time.perf_counter() - t0
    out = []
    if args.direct:
        ctx.profile_begin()
    for _ in range(args.solves):
        t0 = time.perf_counter()
        st = p.solve()
        ctx.synchronize()
        out.append({"ms": (time.perf_counter() - t0) * 1e3, "steps": st["steps"],
                    "rel_residual": st["defect"] / st["initial_defect"]})
    res = {"config": args.ugx or args.config, "dofs": p.n, "setup_s": setup, "solves": out}
    if args.assemblies:
        ctx.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.assemblies):
            p.disc.assemble_linear(p.A, p.b)
        ctx.synchronize()
        res["assembly_ms"] = (time.perf_counter() - t0) * 1e3 / args.assemblies
    if args.gradients:
        import torch
        from ugcore_gb300 import adjoint
        prob = adjoint.DifferentiableProblem(ctx, problems.config(args.config, **over))
        m0 = torch.tensor(prob.m_top, device="cuda")
        f = torch.ones(prob.n, dtype=torch.float64, device="cuda")
        times = []
        for r in range(args.gradients):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            mm = (m0 * (1.0 + 0.01 * r)).clone().requires_grad_(True)
            u = adjoint.fv1_solve(mm, f, prob)
            (0.5 * (u ** 2).sum()).backward()
            torch.cuda.synchronize()
            times.append((time.perf_counter() - t0) * 1e3)
        res["gradient_ms"] = times
    if args.direct:
        prof = ctx.profile_end()
        res["kernels"] = {k: [v[0], round(v[1], 4)] for k, v in sorted(prof.items(), key=lambda kv: -kv[1][1])[:12]}
    print(json.dumps(res))


if __name__ == "__main__":
    main()
