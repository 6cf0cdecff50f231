"""Gradients through the DNS: hand-written adjoint of the RK4 step behind
torch.autograd.

The reference differentiates its JAX step (spectral_solver.py:50-80) with jax.grad.
Here the forward trajectory runs on the CUDA step kernels, storing one checkpoint per
step; the backward sweep recomputes each step's inner RK4 stages from its checkpoint
and applies the step's vector-Jacobian product (``l3es_adjoint_step``). Gradients of
complex half spectra follow PyTorch's convention (dL/dRe + i dL/dIm).

    plan = make_plan(128, 5e-3, 3, 2e-3, "const_power", kf=2, eps_inj=0.1)
    ip = coarse_plan(3, 128, 32)
    u_hat0.requires_grad_(True)
    loss = coarse_mse(integrate(u_hat0, plan, 20), target, ip)
    loss.backward()                       # u_hat0.grad

``loss_and_grad`` gives the same numbers without autograd bookkeeping. Supported
forcings: none, const_power and ekin_tot (its kinetic-energy rescaling after each step
is differentiated too). ``interp`` differentiates the particle velocities of the
combined loop (coarsening + NUFFT or exact DFT interpolation at fixed positions), so a
loss on particle velocities reaches the initial spectrum through ``integrate``.
"""

from __future__ import annotations

from . import _native
from .spectral_solver import _torch

FORCING = {"none": "none", "const_power": "const_power", "ekin_tot": "ekin_tot"}


def make_plan(N, nu, dim, dt, forcing_type="none", kf=0, eps_inj=0.0, drag=0.0, batch=1, e_kin_init=0.0):
    """A step plan whose adjoint is available (forcing none, const_power or ekin_tot;
    the explicit viscous scheme)."""
    if forcing_type not in FORCING:
        raise ValueError("differentiable forcings: 'none', 'const_power', 'ekin_tot'")
    p = _native.Plan(dim=dim, n=N, nu=nu, dt=dt, forcing=forcing_type, kf=kf or 0, eps_inj=eps_inj,
                     drag=drag, batch=batch, e_kin_init=e_kin_init)
    p.adjoint_prepare()
    return p


def coarse_plan(dim, N, c):
    """Coarsening plan for the loss (spectral_filtering from N to c)."""
    return _native.InterpPlan(dim=dim, ckp_n=c, n_fine=N, np_max=1)


def _fn_classes():
    torch = _torch()

    class Trajectory(torch.autograd.Function):
        """u_hat0 -> u_hat after nsteps RK4 steps; one checkpoint per step."""

        @staticmethod
        def forward(ctx, u_hat0, plan, nsteps):
            uh = u_hat0.detach().clone()
            ck = []
            for _ in range(int(nsteps)):
                ck.append(uh.clone())
                plan.step(uh, 1)
            ctx.plan, ctx.ck = plan, ck
            return uh

        @staticmethod
        def backward(ctx, grad):
            lam = grad.detach().contiguous().clone()
            for u0 in reversed(ctx.ck):
                ctx.plan.adjoint_step(u0, lam)
            ctx.ck = None
            return lam, None, None

    class CoarseMSE(torch.autograd.Function):
        """u_hat -> mean((spectral_filtering(irfftn(u_hat), c) - target)^2)."""

        @staticmethod
        def forward(ctx, u_hat, target, iplan):
            loss = torch.zeros(1, dtype=torch.float64, device=u_hat.device)
            g = torch.empty_like(u_hat)
            iplan.coarse_mse(u_hat.detach().contiguous(), target.contiguous(), loss, g)
            ctx.save_for_backward(g)
            return loss[0]

        @staticmethod
        def backward(ctx, grad_loss):
            (g,) = ctx.saved_tensors
            return g * grad_loss.to(g.real.dtype), None, None

    class Interp(torch.autograd.Function):
        """u_hat (fine half spectrum) -> particle velocities u_r at fixed positions r
        (spectral_filtering to the plan's coarse grid, then NUFFT or exact DFT
        interpolation, integrator.py:36-91); the backward pass is l3es_interp_vjp."""

        @staticmethod
        def forward(ctx, u_hat, r, iplan, backend):
            u_r = torch.empty(r.shape, dtype=torch.float64, device=r.device)
            iplan.set_spectrum(u_hat.detach().contiguous())
            iplan.interp(r, u_r, backend=backend)
            ctx.iplan, ctx.backend, ctx.shape = iplan, backend, u_hat.shape
            ctx.save_for_backward(r)
            return u_r

        @staticmethod
        def backward(ctx, grad_u_r):
            (r,) = ctx.saved_tensors
            g = torch.empty(ctx.shape, dtype=torch.complex64, device=r.device)
            ctx.iplan.interp_vjp(r, grad_u_r.detach().to(torch.float64).contiguous(), g, backend=ctx.backend)
            return g, None, None, None

    return Trajectory, CoarseMSE, Interp


_CLASSES = None


def _classes():
    global _CLASSES
    if _CLASSES is None:
        _CLASSES = _fn_classes()
    return _CLASSES


def integrate(u_hat0, plan, nsteps):
    """Differentiable nsteps RK4 steps (torch.autograd)."""
    return _classes()[0].apply(u_hat0, plan, nsteps)


def coarse_mse(u_hat, target, iplan):
    """Differentiable coarse-grid MSE loss (0-d float64 tensor)."""
    return _classes()[1].apply(u_hat, target, iplan)


def particle_plan(dim, N, c, np_max, width=6):
    """Interpolation plan for particle losses (coarsening from N to c, np_max particles)."""
    return _native.InterpPlan(dim=dim, ckp_n=c, n_fine=N, width=width, np_max=np_max)


def interp(u_hat, r, iplan, backend="nufft"):
    """Differentiable particle velocities (np, dim) float64 at fixed positions r from the
    fine half spectrum u_hat (torch.autograd; positions get no gradient)."""
    return _classes()[2].apply(u_hat, r, iplan, backend)


def loss_and_grad(u_hat0, plan, nsteps, target, iplan, checkpoints=None):
    """(loss, dloss/du_hat0) of coarse_mse(integrate(u_hat0)) by one forward sweep with
    per-step checkpoints and one adjoint sweep. ``checkpoints``: optional list of
    nsteps preallocated tensors shaped like u_hat0."""
    torch = _torch()
    uh = u_hat0.detach().clone()
    ck = checkpoints if checkpoints is not None else [torch.empty_like(uh) for _ in range(int(nsteps))]
    for i in range(int(nsteps)):
        ck[i].copy_(uh)
        plan.step(uh, 1)
    loss = torch.zeros(1, dtype=torch.float64, device=uh.device)
    lam = torch.empty_like(uh)
    iplan.coarse_mse(uh, target.contiguous(), loss, lam)
    for i in range(int(nsteps) - 1, -1, -1):
        plan.adjoint_step(ck[i], lam)
    return loss[0], lam


def rhs_vjp(plan, u_hat, g):
    """(d rhs / d u_hat)^T g for one right-hand-side evaluation."""
    out = _torch().empty_like(u_hat)
    plan.rhs_vjp(u_hat.contiguous(), g.contiguous(), out)
    return out
