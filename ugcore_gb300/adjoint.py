"""Differentiable FV1 solve: u = A(exp(m))^{-1} b(f) as a torch.autograd.Function.

No ugcore counterpart (ugcore has no adjoint).  The forward pass assembles the
operator for the element log-coefficients m and the vertex source f on the
GPU, re-initialises the multigrid (coarse levels get the children's mean m)
and solves with GMG-preconditioned CG/BiCGStab.  The backward pass solves the
transposed system A^T lambda = dJ/du with the same multigrid built on the
transposed level operators (Dirichlet rows reset to identity) and forms
    dJ/dm_e = -K_e * sum_{i not Dirichlet} lambda_i (A1_e u_e)_i
    dJ/df_i = lambda_i * |SCV_i|
with element-local kernels.  The forward pass keeps only u (one vector) for
the backward pass.  The transposed multigrid either sits beside the forward
one (adjoint_memory "store": one extra hierarchy of device memory) or is the
forward multigrid transposed in place, level by level, and re-assembled for
the next forward pass (adjoint_memory "recompute": no memory beyond the
forward solve's).
"""
import torch

from . import problems
from .algebra import GPUVector


def _library_waits_for_torch(ctx):
    """the library's stream waits (on the device, through an event) for the
    work queued so far on torch's current stream"""
    torch.cuda.ExternalStream(ctx.stream).wait_stream(torch.cuda.current_stream())


def _torch_waits_for_library(ctx):
    torch.cuda.current_stream().wait_stream(torch.cuda.ExternalStream(ctx.stream))


class DifferentiableProblem(problems.Problem):
    """A Problem whose coefficient and source come from torch tensors.  The
    solution lives in a torch tensor the library writes directly; the two
    streams are ordered by events, not by host synchronisation."""

    def __init__(self, ctx, cfg, m=None, f=None):
        cfg = dict(cfg)
        cfg["coef"] = "logk"
        super().__init__(ctx, cfg, m_top=None if m is None else m.detach().cpu().numpy(),
                         f_top=None if f is None else f.detach().cpu().numpy())
        self.num_elements = self.hier.num_elements()
        self._x_t = torch.zeros(self.n, dtype=torch.float64, device="cuda")
        self.x = GPUVector(self.ctx, wrap=self._x_t)
        self._inputs = None

    def update(self, m, f):
        """re-assemble for new (m, f) (CUDA float64 tensors) and re-initialise
        (on an unchanged hierarchy the multigrid and the solvers refresh their
        values in place and keep their captured graphs)."""
        _library_waits_for_torch(self.ctx)
        # kept alive until the library has read them (the uploads synchronise)
        self._inputs = (m.detach().contiguous(), f.detach().contiguous())
        self.disc.set_log_diffusion(self._inputs[0])
        self.disc.set_source(self._inputs[1])
        self.disc.assemble_linear(self.A, self.b)
        self.gmg.set_transposed(False)
        self.gmg.init(self.A)
        self.solver.init(self.A)
        self._fwd_valid = True
        self.invalidate_adjoint()

    def solve_u(self):
        """solve; returns u as a new CUDA tensor (a copy on torch's stream)"""
        self.solve()
        _torch_waits_for_library(self.ctx)
        return self._x_t.clone()

    def backward(self, u_tensor, grad_u):
        self.adjoint_setup()
        if getattr(self, "_interior", None) is None:
            _, _, bnd = self.hier.export()
            self._interior = torch.tensor(1.0 - bnd.astype("float64"), device=u_tensor.device)
        # rhs = dJ/du without its Dirichlet entries
        rhs_t = (grad_u.detach() * self._interior).contiguous()
        u_t = u_tensor.detach().contiguous()
        gm = torch.empty(self.num_elements, dtype=torch.float64, device=u_tensor.device)
        gf = torch.empty(self.n, dtype=torch.float64, device=u_tensor.device)
        _library_waits_for_torch(self.ctx)
        rhs = GPUVector(self.ctx, wrap=rhs_t)
        u = GPUVector(self.ctx, wrap=u_t)
        self.lam.set(0.0)
        self.solverT.apply(self.lam, rhs)
        self.disc.grad_logk(u, self.lam, out=gm)
        self.disc.grad_source(self.lam, out=gf)
        _torch_waits_for_library(self.ctx)
        self.last_adjoint_stats = self.solverT.stats()
        return gm, gf


class FV1Solve(torch.autograd.Function):
    """u = FV1Solve.apply(m, f, problem): differentiable in m and f."""

    @staticmethod
    def forward(ctx, m, f, problem):
        problem.update(m, f)
        u = problem.solve_u()
        ctx.problem = problem
        ctx.save_for_backward(u)
        return u

    @staticmethod
    def backward(ctx, grad_u):
        (u,) = ctx.saved_tensors
        gm, gf = ctx.problem.backward(u, grad_u)
        return gm, gf, None


def fv1_solve(m, f, problem):
    return FV1Solve.apply(m, f, problem)
