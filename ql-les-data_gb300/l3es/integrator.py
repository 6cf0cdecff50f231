"""Particle interpolation and advection: drop-in for the hot-path part of
l3es/integrator.py (``shift_fn``, ``spectral_interpolator_wrapper``,
``set_up_integrator``). Positions and velocities are float64 (np, dim) torch CUDA
tensors, as the reference keeps them in FP64. ``set_up_integrator`` also returns the
SPH density and relaxation functions (l3es.utils.rho_computer, l3es.relax.relax_wrapper).
"""

from __future__ import annotations

import numpy as np

from . import _native
from .spectral_solver import _torch


def shift_fn(r, dr, box_size=2 * np.pi):
    """(r + dr) mod box_size (integrator.py:21-23)."""
    torch = _torch()
    r = torch.as_tensor(r, dtype=torch.float64, device="cuda").contiguous()
    dr = torch.as_tensor(dr, dtype=torch.float64, device="cuda").contiguous()
    return _native.shift(r, dr, 1.0, box_size)


def spectral_interpolator_wrapper(N, fft_axes=(1, 2, 3), splits=128, backend="nufft"):
    """integrator.py:26-93: returns fn(u, r) -> u_r (np, dim), u the coarse grid field
    (3, N, N, N) or (2, N, N). backend 'nufft' is the type-2 NUFFT (ES kernel, width 6,
    upsampling 2); 'dft' the exact sum. ``splits`` only shaped the reference's JAX
    batching and has no effect here."""
    assert splits & (splits - 1) == 0, "Splits must be a power of 2"
    assert backend in ["dft", "nufft"]
    dim = len(fft_axes)
    plans = {}

    def interpolate(u, r):
        torch = _torch()
        r = torch.as_tensor(r, dtype=torch.float64, device="cuda").contiguous()
        npart = r.shape[0]
        p = plans.get("p")
        if p is None or p.np_max < npart:
            p = _native.InterpPlan(dim=dim, ckp_n=N, n_fine=0, width=6, np_max=npart)
            plans["p"] = p
        t = torch.as_tensor(u, dtype=torch.float32, device="cuda")
        if dim == 2:
            f = torch.zeros(3, N, N, 1, dtype=torch.float32, device="cuda")
            f[: t.shape[0], :, :, 0] = t.reshape(t.shape[0], N, N)
        else:
            f = t.contiguous()
        p.set_field(f)
        out = torch.empty_like(r)
        p.interp(r, out, backend=backend)
        return out

    return interpolate


def pos_init_cartesian(L, n, dim):
    """Cell-centred lattice of n^dim particles in [0, L)^dim, C order (the layout of
    jax_sph's pos_init_cartesian_2d/3d used at integrator.py:103-106)."""
    dx = L / n
    ax = (np.arange(n) + 0.5) * dx
    g = np.meshgrid(*([ax] * dim), indexing="ij")
    return np.stack([a.ravel() for a in g], axis=1)


def set_up_integrator(state_0_path, dim, N, dft_splits, u_ref, interp_backend):
    """integrator.py:96-114. Returns the reference's 7-tuple
    (r, comp_rho, interpolator, relax_fn, sph_fn, L, fft_axes). state_0_path may name a
    .npy/.npz file holding the initial positions (the reference reads an h5 written by
    JAX-SPH)."""
    from .relax import relax_wrapper
    from .utils import rho_computer

    torch = _torch()
    L = 2 * np.pi
    fft_axes = (1, 2, 3) if dim == 3 else (1, 2)
    if state_0_path is not None:
        data = np.load(state_0_path)
        r = data["r"] if hasattr(data, "files") else data
    else:
        r = pos_init_cartesian(L, N, dim)
    r = torch.as_tensor(np.asarray(r, dtype=np.float64), device="cuda")
    interpolator = spectral_interpolator_wrapper(N, fft_axes, splits=dft_splits or 1, backend=interp_backend)
    comp_rho = rho_computer(N, dim=dim, L=L)
    relax_fn, sph_fn = relax_wrapper(N, dim, L, is_physical=True, u_ref=u_ref)
    return r, comp_rho, interpolator, relax_fn, sph_fn, L, fft_axes
