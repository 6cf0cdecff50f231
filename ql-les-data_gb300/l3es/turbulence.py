"""Particle -> grid analysis: drop-in for the DFT path of l3es/turbulence.py.

``ur_to_u_dft_wrapper`` and ``u_and_spectrum_from_ur(..., interp_backend="dft")``
with the reference's arguments; the exact sum runs on the GPU
(``l3es_interp_particles_to_grid``). The reference's default moving-least-squares
backend (KD-tree neighbours, turbulence.py:145-253) is not part of this package.
"""

from __future__ import annotations

import numpy as np

from . import _native
from .spectral_solver import _torch
from .utils import energy_spectrum

_PLANS: dict = {}


def _plan(n, dim, npart):
    key = (_torch().cuda.current_device(), n, dim)
    p = _PLANS.get(key)
    if p is None or p.np_max < npart:
        p = _native.InterpPlan(dim=dim, ckp_n=n, n_fine=0, np_max=max(npart, 1))
        _PLANS[key] = p
    return p


def ur_to_u_dft_wrapper(N, L, dim=3, fft_axes=(1, 2, 3)):
    """turbulence.py:299-339: body(r, u_r) -> u_grid of shape (N^dim, dim), the real
    part of the inverse FFT of sum_j u_r[j] exp(-i k.r_j)."""
    assert abs(L - 2 * np.pi) < 1e-12, "the wavenumbers assume a 2 pi box"

    def body(r, u_r):
        torch = _torch()
        r = torch.as_tensor(np.asarray(r.cpu() if hasattr(r, "cpu") else r), dtype=torch.float64).cuda()
        u = torch.as_tensor(np.asarray(u_r.cpu() if hasattr(u_r, "cpu") else u_r), dtype=torch.float64).cuda()
        p = _plan(N, dim, r.shape[0])
        out = torch.empty((3,) + (N,) * dim, dtype=torch.float32, device="cuda")
        p.particles_to_grid(r.contiguous(), u.contiguous(), out)
        return out[:dim].reshape(dim, -1).T

    return body


def u_and_spectrum_from_ur(ckp_N, L, dim=3, interp_backend="mls", fft_axes=(1, 2, 3)):
    """turbulence.py:342-377 for interp_backend='dft': body(r, u_r) -> (u_grid, ek),
    u_grid (dim, N, N, N) in 3D or (dim, N, N, 1) in 2D."""
    if interp_backend != "dft":
        raise NotImplementedError("only the 'dft' particle-to-grid backend is available")
    interpolate = ur_to_u_dft_wrapper(ckp_N, L, dim, fft_axes)

    def body(r, u_r):
        u_grid = interpolate(r, u_r)
        shape = (dim,) + (ckp_N,) * dim if dim == 3 else (dim, ckp_N, ckp_N, 1)
        u_grid = u_grid.T.reshape(shape)
        ek = energy_spectrum(u_grid, dim=dim) if dim == 3 else energy_spectrum(
            _torch().cat([u_grid, _torch().zeros_like(u_grid[:1])]), dim=2)
        return u_grid, ek

    return body
