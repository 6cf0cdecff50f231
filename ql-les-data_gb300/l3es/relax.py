"""SPH particle relaxation: drop-in for l3es/relax.py (relax_wrapper).

The reference builds a JAX-SPH neighbour list, quintic kernel and Tait EoS and returns
two jitted functions (relax.py:16-178). Here both run as CUDA kernels behind
``l3es_sph_*`` (cell list rebuilt per call, one thread per particle in cell order).
Positions and velocities are float64 (np, dim) torch CUDA tensors (numpy arrays are
accepted and copied to the device).
"""

from __future__ import annotations

import numpy as np

from . import _native
from .spectral_solver import _torch


def _pos(x):
    torch = _torch()
    return torch.as_tensor(x, dtype=torch.float64, device="cuda").contiguous()


class _SphPlans:
    """One SphPlan per (dim, N, L), grown when more particles arrive."""

    def __init__(self, N, dim, L):
        self.N, self.dim, self.L = int(N), int(dim), float(L)
        self.plan = None

    def get(self, npart):
        if self.plan is None or self.plan.np_max < npart:
            self.plan = _native.SphPlan(self.dim, self.N, self.L, max(npart, self.N**self.dim))
        return self.plan


def relax_wrapper(N, dim=3, L=2 * np.pi, is_physical=False, u_ref=None):
    """relax.py:16-178. Returns (loop_body, sph_body):

    loop_body(r) -> acceleration (np, dim): pressure plus half the transport-velocity
    term, in physical units (``is_physical`` only chose the reference's internal units
    and does not change the result);
    sph_body(r, u) -> {"acc_p", "acc_visc", "acc_tvf"} (requires is_physical, as the
    reference asserts).
    """
    if u_ref is None:
        raise ValueError("relax_wrapper needs u_ref (the EoS reference velocity)")
    plans = _SphPlans(N, dim, L)
    torch = _torch()

    def loop_body(r):
        r = _pos(r)
        acc = torch.empty_like(r)
        plans.get(r.shape[0]).relax_acceleration(r, acc, u_ref)
        return acc

    def sph_body(r, u):
        assert is_physical, "sph is only implemented for physical units."
        r, u = _pos(r), _pos(u)
        out = {k: torch.empty_like(r) for k in ("acc_p", "acc_visc", "acc_tvf")}
        plans.get(r.shape[0]).forces(r, u, out["acc_p"], out["acc_visc"], out["acc_tvf"], u_ref)
        return out

    return loop_body, sph_body


def relax_velocity_wrapper(N, dim, L, u_ref, relax_dt_factor):
    """The combined loop's relaxation (combined.py:132-142) as one fused call:
    fn(r0, u_r, dt, r_out=None) -> u_relaxed, with r_out = shift(r0, dt u_relaxed)
    written when given."""
    plans = _SphPlans(N, dim, L)
    torch = _torch()

    def fn(r0, u_r, dt, r_out=None):
        r0, u_r = _pos(r0), _pos(u_r)
        u_out = torch.empty_like(r0)
        plans.get(r0.shape[0]).relax_velocity(r0, u_r, u_out, dt, relax_dt_factor, u_ref, r_out=r_out)
        return u_out

    return fn
