"""The compliance path as a differentiable torch function.

`ComplianceObjective(domain, bc, f, ...)(x)` returns the compliance c(x) = f . u(x) of the structured-grid
problem FilterConv -> SIMP -> K(x) -> K u = f as a 0-d FP64 CUDA tensor that torch autograd differentiates:
the forward pass is the response of the GPU modules (pymoto_gb300.modules, the same objects a pyMOTO Network
runs), the backward pass their hand-written adjoint kernels -- the LDA-projected adjoint solve, the sensitivity
contraction -p x^(p-1) u_e^T K0 u_e (pmg_sens_contract / pmg_sens_contract_mixed), the SIMP derivative and
the filter transpose (pmg_conv_filter_adjoint) -- wrapped in one torch.autograd.Function.  It mirrors what
pyMOTO's Network.sensitivity() computes for the same modules (pymoto/core_objects.py:750-829).
"""
import numpy as np
import torch

from .modules import EinSum, FilterConv, LinSolve, SIMP, AssembleStiffness
from .core import Network, Signal


class ComplianceObjective:
    """c(x) = f . u with K(x) u = f, x the design field (FP64 CUDA tensor, one value per element).

    domain, bc (constrained dof indices), f (load vector): the problem.  radius (FilterConv, relative units),
    penal / xmin (SIMP), solver (a pymoto_gb300 LinearSolver; None: LinSolve's default, CG with an FP64
    multigrid hierarchy to 1e-10) configure the path.  Building the object evaluates the network once at x = 0.5
    (modules run when they are connected, as in pyMOTO).  Calling it with a tensor that requires grad gives a
    tensor whose backward() fills x.grad through the adjoint kernels."""

    def __init__(self, domain, bc, f, radius=2.5, penal=3.0, xmin=1e-9, solver=None, sensitivity_precision="fp64"):
        self.domain = domain
        self.f = f if isinstance(f, torch.Tensor) else torch.as_tensor(np.asarray(f, dtype=np.float64))
        self.f = self.f.to(device="cuda", dtype=torch.float64)
        self.sx = Signal("x", torch.full((domain.nel,), 0.5, dtype=torch.float64, device="cuda"))
        with Network() as fn:
            xf = FilterConv(domain, radius=radius)(self.sx)
            xs = SIMP(xmin=xmin, penal=penal)(xf)
            K = AssembleStiffness(domain, bc=bc, sensitivity_precision=sensitivity_precision)(xs)
            u = LinSolve(hermitian=True, symmetric=True, solver=solver)(K, self.f)   # None: CG + FP64 multigrid
            self.sc = EinSum("i,i->")(u, self.f)
        self.network = fn

    def __call__(self, x):
        return _Compliance.apply(x, self)

    def _forward(self, x):
        self.sx.state = x.detach().contiguous()
        self.network.response()
        c = self.sc.state
        return c.reshape(()) if isinstance(c, torch.Tensor) else torch.tensor(float(c), dtype=torch.float64,
                                                                                 device=x.device)

    def _backward(self, gc):
        self.network.reset()
        self.sc.sensitivity = gc
        self.network.sensitivity()
        dx = self.sx.sensitivity
        self.network.reset()
        return dx if isinstance(dx, torch.Tensor) else torch.as_tensor(dx, device="cuda")


class _Compliance(torch.autograd.Function):
    """Forward: the GPU modules' response; backward: their adjoint kernels (no autograd tape inside)."""

    @staticmethod
    def forward(ctx, x, objective):
        ctx.objective = objective
        return objective._forward(x)

    @staticmethod
    def backward(ctx, gc):
        dx = ctx.objective._backward(float(gc))
        return dx * 1.0, None
