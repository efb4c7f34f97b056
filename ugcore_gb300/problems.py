"""The benchmark problems (seeded synthetic inputs) and a one-object setup of
assemble + GMG + Krylov on the GPU.

Configurations (unit square / cube, zero Dirichlet boundary, FV1):
  c0  2D Poisson FP64: 2x2 quads refined 6x (129^2 = 16,641 DoFs), K = 1,
      f ~ U[-1,1] per vertex, GMG V(2,2) Jacobi(0.6), LU base, CG to 1e-10.
  c1  3D Poisson: 2x2x2 hexes refined 6x (129^3 = 2,146,689 DoFs), as c0;
      FP64 or mixed, multicolour Gauss-Seidel as an opt-in smoother.
  c2  3D variable coefficient, mixed: 4^3 hexes x 6 Kuhn tets refined 5x
      (129^3 vertices), K = exp(2 g), g a unit-variance 64-mode field with
      |kappa| <= 8 (contrast ~1e4-1e5), CG with an FP32 GMG.
  c3  2D adjoint: 2x2 quads refined 7x (257^2 = 66,049 DoFs), K = exp(m),
      m = 32-mode field at element centroids.
  c4  3D convection-diffusion adjoint: 3^3 hexes refined 6x (193^3 =
      7,189,057 DoFs), D = 1e-2, v = curl of a 16-mode vector potential scaled
      to cell Peclet 10, full upwind, BiCGStab with an FP32 GMG.
Every field is drawn from splitmix64 streams (fields.py), identical to the
oracle's generator, so the GPU and CPU paths solve the same problem.
"""
import copy

import numpy as np

from . import fields
from .algebra import (BackwardGaussSeidel, BaseSmoothing, BiCGStab, CG, DomainDiscretization, GaussSeidel, GeometricMultiGrid,
                      GPUSparseMatrix,
                      GPUVector, ILU, Jacobi, StdConvCheck, StdTransfer, StructuredHierarchy, SymmetricGaussSeidel,
                      ThetaTimeStep)

BASE = dict(elem="quad", mx=2, my=2, mz=1, nref=6, seed=1, coef="const", diffusion=1.0, coef_modes=64,
            coef_kmax=8.0, vel=None, vel_modes=16, vel_kmax=2.0, peclet=10.0, solver="cg", smoother="jacobi",
            damp=0.6, nu1=2, nu2=2, cycle=1, base=0, precision="fp64", maxit=200, rel_red=1e-10,
            min_defect=1e-300, rap=False, bicg_restart=0, bicg_min_ortho=0.0, damp_prol=1.0, damp_res=1.0,
            adjoint_memory="store")

CONFIGS = {
    "c0": dict(elem="quad", mx=2, my=2, nref=6),
    "c1": dict(elem="hex", mx=2, my=2, mz=2, nref=6),
    "c2": dict(elem="tet", mx=4, my=4, mz=4, nref=5, coef="lognormal", precision="mixed"),
    "c3": dict(elem="quad", mx=2, my=2, nref=7, coef="logk", coef_modes=32),
    "c4": dict(elem="hex", mx=3, my=3, mz=3, nref=6, coef="const", diffusion=1e-2, vel="curl", solver="bicgstab",
               precision="mixed"),
}


def config(name, **over):
    cfg = copy.deepcopy(BASE)
    cfg.update(CONFIGS[name] if name in CONFIGS else {})
    cfg.update(over)
    return cfg


def logk_field(cfg, hier):
    """m per top-level element: the 32-mode field at element centroids."""
    coords, elems, _ = hier.export()
    cent = coords[elems].mean(axis=1)
    g = fields.ScalarField(hier.dim, cfg["coef_modes"], cfg["coef_kmax"], cfg["seed"] ^ fields.COEF_SEED_XOR)
    return g(cent)


class Problem:
    """Assemble-and-solve setup of one configuration on one GPU."""

    def __init__(self, ctx, cfg, m_top=None, f_top=None):
        self.ctx, self.cfg = ctx, cfg
        c = cfg
        self.hier = StructuredHierarchy(ctx, c["elem"], c["mx"], c["my"], c["mz"], c["nref"])
        self.n = self.hier.num_vertices()
        self.disc = DomainDiscretization(self.hier)
        if c["coef"] == "const":
            self.disc.set_diffusion(c["diffusion"])
        elif c["coef"] == "lognormal":
            g = fields.ScalarField(self.hier.dim, c["coef_modes"], c["coef_kmax"], c["seed"] ^ fields.COEF_SEED_XOR)
            self.disc.set_diffusion_field(g, factor=2.0)
        elif c["coef"] == "logk":
            self.m_top = logk_field(c, self.hier) if m_top is None else m_top
            self.disc.set_log_diffusion(self.m_top)
        else:
            raise ValueError(c["coef"])
        if c["vel"] == "curl":
            vf = fields.CurlField(c["vel_modes"], c["vel_kmax"], c["seed"] ^ fields.VEL_SEED_XOR)
            nx = c["mx"] * (1 << c["nref"]) + 1
            self.disc.set_velocity_field(vf, c["peclet"] * 2.0 * c["diffusion"] * (nx - 1))
            self.disc.set_upwind("full")
        if f_top is not None:
            self.disc.set_source(f_top)
        else:
            self.disc.set_source_uniform(c["seed"])
        self.A = GPUSparseMatrix(ctx)
        self.b = GPUVector(ctx, self.n)
        self.disc.assemble_linear(self.A, self.b)
        self.gmg = self._make_gmg(transposed=False)
        self.gmg.init(self.A)
        self.solver = self._make_solver()
        self.solver.set_preconditioner(self.gmg)
        self.solver.set_convergence_check(StdConvCheck(c["maxit"], c["min_defect"], c["rel_red"]))
        self.solver.init(self.A)
        self.x = GPUVector(ctx, self.n)
        self.rhs = GPUVector(ctx, self.n)

    def _make_solver(self):
        c = self.cfg
        s = (CG if c["solver"] == "cg" else BiCGStab)(self.ctx)
        if c["solver"] != "cg":
            s.set_restart(c.get("bicg_restart", 0))
            s.set_min_orthogonality(c.get("bicg_min_ortho", 0.0))
        return s

    def _make_gmg(self, transposed):
        c = self.cfg
        g = GeometricMultiGrid(self.disc)
        kinds = {"jacobi": Jacobi, "mcgs": GaussSeidel, "mcsgs": SymmetricGaussSeidel, "ilu": ILU,
                 "mcbgs": BackwardGaussSeidel}
        g.set_smoother(kinds[c["smoother"]](c["damp"]))
        if c.get("post_smoother"):
            # a post-smoother of its own (set_postsmoother)
            g.set_postsmoother(kinds[c["post_smoother"]](c.get("post_damp", 1.0)))
        g.set_cycle_type(c["cycle"])
        g.set_num_presmooth(c["nu1"])
        g.set_num_postsmooth(c["nu2"])
        g.set_base_level(c["base"])
        if c.get("base_solver", "lu") == "smoother":
            g.set_base_solver(BaseSmoothing(c.get("base_steps", 10)))
        g.set_precision(c["precision"])
        g.set_transposed(transposed)
        g.set_rap(c["rap"])
        if c.get("damp_prol", 1.0) != 1.0 or c.get("damp_res", 1.0) != 1.0:
            t = StdTransfer()
            t.set_prolongation_damping(c.get("damp_prol", 1.0))
            t.set_restriction_damping(c.get("damp_res", 1.0))
            g.set_transfer(t)
        return g

    def forward_ready(self):
        """the operator, multigrid and solver hold the forward problem again
        after an adjoint solve that reused them (adjoint_memory
        "recompute"): re-assembly and a value refresh of the multigrid"""
        if getattr(self, "_fwd_valid", True):
            return
        self.disc.assemble_linear(self.A, self.b)
        self.gmg.set_transposed(False)
        self.gmg.init(self.A)
        self.solver.init(self.A)
        self._fwd_valid = True
        # the operator no longer holds the transposed problem
        self._adj_ready = False

    def solve(self, raise_on_failure=True):
        """x = A^{-1} b from x0 = 0; b is kept."""
        self.forward_ready()
        self.x.set(0.0)
        ok = self.solver.apply(self.x, self.b, raise_on_failure=raise_on_failure)
        st = self.solver.stats()
        st["ok"] = ok
        return st

    # ---- time stepping --------------------------------------------------
    def theta_steps(self, theta, dt, nsteps, u0, t0=0.0):
        """nsteps steps of the theta scheme du/dt + A u = f from u0, as
        ugcore's SolveLinearTimeProblem (scripts/util/time_step_util.lua:
        643-870) for a constant step: the step's matrix, the multigrid (coarse
        levels: the time-discrete jacobians M + theta dt A) and the solver are
        set up once; every step prepares the time discretisation with the
        previous solution, assembles its right-hand side and applies the
        solver from the previous solution.  Returns (u as numpy, iterations per
        step)."""
        c = self.cfg
        td = ThetaTimeStep(self.disc, theta)
        u = GPUVector(self.ctx, self.n).copy_from(u0)
        A = GPUSparseMatrix(self.ctx)
        b = GPUVector(self.ctx, self.n)
        gmg = self._make_gmg(transposed=False)
        gmg.set_discretization(td)
        solver = self._make_solver()
        solver.set_preconditioner(gmg)
        solver.set_convergence_check(StdConvCheck(c["maxit"], c["min_defect"], c["rel_red"]))
        steps, t = [], t0
        for s in range(nsteps):
            td.prepare_step(u, t, dt)
            td.assemble_linear(A, b)
            if s == 0:
                gmg.init(A)
                solver.init(A)
            solver.apply(u, b)
            steps.append(solver.stats()["steps"])
            t = td.future_time()
        return u.numpy(), steps

    # ---- adjoint --------------------------------------------------------
    def adjoint_setup(self):
        """A^T, the transposed multigrid and its solver for the current
        operator; the objects are kept across operator updates and only
        re-initialised (invalidate_adjoint).

        adjoint_memory "store" (default): a second operator, multigrid and
        solver hold the transposed problem beside the forward one.
        "recompute": the forward operator and multigrid are transposed in
        place (level by level, through the transposition permutation of their
        symmetric patterns) and serve the adjoint solve; the next forward
        solve re-assembles them.  The adjoint then needs no memory beyond the
        forward solve's (the levels are recomputed instead of stored)."""
        if getattr(self, "_adj_ready", False):
            return
        if self.cfg.get("adjoint_memory", "store") == "recompute":
            if getattr(self, "lam", None) is None:
                self.lam = GPUVector(self.ctx, self.n)
            self.forward_ready()
            # the transposed multigrid is built from the forward operator
            # (it transposes its own copy of the top level), then the
            # operator itself is transposed for the solver
            self.gmg.set_transposed(True)
            self.gmg.init(self.A)
            self.disc.adjoint_operator(self.A, self.A)
            self.solver.init(self.A)
            self.AT, self.gmgT, self.solverT = self.A, self.gmg, self.solver
            self._fwd_valid = False
            self._adj_ready = True
            return
        if getattr(self, "gmgT", None) is None:
            self.AT = GPUSparseMatrix(self.ctx)
            self.gmgT = self._make_gmg(transposed=True)
            self.solverT = self._make_solver()
            self.solverT.set_preconditioner(self.gmgT)
            self.solverT.set_convergence_check(StdConvCheck(self.cfg["maxit"], self.cfg["min_defect"],
                                                            self.cfg["rel_red"]))
            self.lam = GPUVector(self.ctx, self.n)
        self.disc.adjoint_operator(self.A, self.AT)
        self.gmgT.init(self.A)
        self.solverT.init(self.AT)
        self._adj_ready = True

    def invalidate_adjoint(self):
        """the operator changed: the next adjoint solve re-initialises"""
        self._adj_ready = False

    def adjoint_solve(self, g):
        """lambda = A^{-T} g (g = dJ/du, Dirichlet entries ignored)."""
        self.adjoint_setup()
        _, _, bnd = self.hier.export()
        gg = np.array(g, dtype=np.float64, copy=True)
        gg[bnd.astype(bool)] = 0.0
        self.rhs.copy_from(gg)
        self.lam.set(0.0)
        self.solverT.apply(self.lam, self.rhs)
        return self.solverT.stats()
