"""Spectral utilities: drop-in for the hot-path part of l3es/utils.py.

``spectral_filtering``, ``energy_spectrum``, ``comp_dissipation_rate``,
``get_real_wavenumber_grid``, ``write_u`` and the SPH density ``rho_computer`` with the
reference's arguments. Fields are torch CUDA tensors (NumPy arrays are accepted and
moved to the GPU); the work runs in the CUDA library. Finite-difference
vorticity/divergence and the incompressible projections of the reference module are
outside this package.
"""

from __future__ import annotations

import os

import numpy as np

from . import _native
from .spectral_solver import _any_plan, _as_phys, _as_spec, _torch

EPS = float(np.finfo(np.float64).eps)

_INTERP: dict = {}


def _interp_plan(dim, n_fine, c, np_max=0, width=6):
    torch = _torch()
    key = (torch.cuda.current_device(), dim, int(n_fine), int(c), int(width))
    p = _INTERP.get(key)
    if p is None or p.np_max < np_max:
        p = _native.InterpPlan(dim=dim, ckp_n=c, n_fine=n_fine, width=width, np_max=max(np_max, 1))
        _INTERP[key] = p
    return p


def get_real_wavenumber_grid(n, dim):
    """utils.py:18-32: integer wavenumbers with the half axis first (Nyquist positive)."""
    Nf = n // 2 + 1
    k = np.fft.fftfreq(n, 1.0 / n)
    kx = k[:Nf].copy()
    kx[-1] *= -1
    if dim == 2:
        k_field = np.array(np.meshgrid(kx, k, indexing="ij"), dtype=int)
    else:
        k_field = np.array(np.meshgrid(kx, k, k, indexing="ij"), dtype=int)
    return k_field, np.arange(n)


def _spectrum_of(u):
    """(u_hat, dim, n) of a physical field (3, n, n, n), (3, n, n, 1) or (2, n, n)."""
    torch = _torch()
    t = u if isinstance(u, torch.Tensor) else torch.from_numpy(np.asarray(u))
    t = t.to(device="cuda", dtype=torch.float32)
    if t.ndim == 4 and t.shape[-1] != 1:
        dim, n = 3, t.shape[1]
        phys = t.contiguous()
    else:
        dim, n = 2, t.shape[1]
        t2 = t.reshape(t.shape[0], n, n)
        phys = torch.zeros(3, n, n, 1, dtype=torch.float32, device="cuda")
        phys[: t2.shape[0], :, :, 0] = t2
    p = _any_plan(dim, n)
    uh = torch.empty(p.spec_shape, dtype=torch.complex64, device="cuda")
    p.rfftn(phys, uh)
    return uh, dim, n


def spectral_filtering(u, ckp_N):
    """utils.py:100-138: keep the modes k in [-c/2, c/2-1] of each axis, inverse
    transform on the c grid and divide by (N/c)^dim. u: (3, N, N, N) or (2, N, N);
    returns (3, c, c, c) or (2, c, c), float32 on the GPU."""
    uh, dim, n = _spectrum_of(u)
    ncomp = u.shape[0]
    if ckp_N == n:
        return _torch().as_tensor(u, device="cuda", dtype=_torch().float32)
    return filter_spectrum(uh, n, ckp_N, dim)[:ncomp]


def filter_spectrum(u_hat, N, ckp_N, dim=3):
    """spectral_filtering straight from the half spectrum of the fine field (no
    fine-grid FFT): (3, c, c, c) for dim 3, (3, c, c) for dim 2."""
    torch = _torch()
    p = _interp_plan(dim, N, ckp_N)
    p.set_spectrum(_as_spec(u_hat, N, dim))
    out = torch.empty(p.coarse_shape, dtype=torch.float32, device="cuda")
    p.coarse_field(out)
    return out if dim == 3 else out[..., 0]


def energy_spectrum(vel, mul_fac: float = 1.0, is_scalar_field: bool = False, dim=3):
    """utils.py:35-97 (shells int(|k| + 0.5), 4 pi k^2 / samples); float64 (n,) on the GPU."""
    torch = _torch()
    if dim == 2:
        v = vel[:2, :, :, 0] if vel.ndim == 4 else vel[:2]
    else:
        v = vel
    uh, d, n = _spectrum_of(v)
    p = _any_plan(d, n)
    ek = torch.empty(n, dtype=torch.float64, device="cuda")
    p.energy_spectrum(uh, ek, mul_fac)
    return ek


def comp_dissipation_rate(u_hat, nu):
    """utils.py:300-315: nu <|curl u|^2>, 3D (0-d float64 tensor on the GPU)."""
    torch = _torch()
    n = u_hat.shape[1]
    p = _any_plan(3, n)
    out = torch.empty(1, dtype=torch.float64, device="cuda")
    p.dissipation(_as_spec(u_hat, n, 3), nu, out)
    return out[0]


def write_u(u, tstep, dst_path, ckp_N, suffix=""):
    """utils.py:141-166: save the (filtered) field as u_{ckp_N}_{tstep:05d}{suffix}.npy;
    2D fields (3, N, N, 1) are written as (2, c, c)."""
    N_u = u.shape[1]
    dim = 2 if u.shape[-1] == 1 else 3
    uu = u if dim == 3 else u[:2, :, :, 0]
    assert ckp_N <= N_u, "ckp_N must be less than or equal to N."
    assert ckp_N % 2 == 0 and N_u % 2 == 0, "Only tested for even N and ckp_N."
    y = uu if ckp_N == N_u else spectral_filtering(uu, ckp_N)
    os.makedirs(dst_path, exist_ok=True)
    arr = y.detach().cpu().numpy() if hasattr(y, "detach") else np.asarray(y)
    np.save(os.path.join(dst_path, f"u_{ckp_N}_{tstep:05d}{suffix}.npy"), arr)


def rho_computer(N, dim=3, L=2 * np.pi):
    """utils.py:169-218: returns comp_rho(r) -> SPH density (np,) float64 of the
    particles at r (quintic kernel, h = L/N, cutoff 3h, mass (L/N)^dim, the particle
    itself included)."""
    from .relax import _SphPlans, _pos

    plans = _SphPlans(N, dim, L)
    torch = _torch()

    def comp_rho(r):
        r = _pos(r)
        rho = torch.empty(r.shape[0], dtype=torch.float64, device="cuda")
        plans.get(r.shape[0]).density(r, rho)
        return rho

    return comp_rho
