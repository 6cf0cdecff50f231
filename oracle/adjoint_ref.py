"""FP64 NumPy adjoint (vector-Jacobian products) of the l3es RK4 step and of the
coarse-grid MSE loss.

TEST INFRASTRUCTURE ONLY (oracle); never on the product path.

The reference differentiates its JAX step with jax.grad (no hand-written adjoint in
the repository; the step is spectral_solver.py:50-80). This module is the FP64
restatement of the same derivative, derived operator by operator and pinned by
central finite differences of oracle.numpy_ref in the tests (jax is not available
here, so there is no jax.grad output to compare with).

Conventions. Arrays are half spectra (rfftn layout). For a real loss L the gradient
with respect to a complex array z is dL/dRe z + i dL/dIm z, so that
dL = Re sum(conj(grad) * dz) over the stored entries (PyTorch's convention). With
w = 1 on the half-axis planes 0 and N/2 and 2 elsewhere (the multiplicity of a stored
mode in the full spectrum):
  irfftn u = C(u_hat)   has adjoint  C^T v = w rfftn(v) / N^d
  rfftn  U = F(u)       has adjoint  F^T G = N^d irfftn(G / w)
  curl i k x            is self-adjoint (i [k]x is Hermitian), P and the dealias
                        mask are real symmetric.
For du = P D F(u x w) - nu k^2 u_hat - drag u_hat + f(u_hat), u = C(u_hat),
w = C(i k x u_hat), and a cotangent g of du:
  m = irfftn(D P g / w)                              (= F^T(D P g) / N^d)
  vjp = w [rfftn(w x m) + i k x rfftn(m x u)] - (nu k^2 + drag) g + f'(u_hat)^T g
with, for the constant-power band force f = s u_hat on 0 < |k|^2 <= kf^2,
s = eps / (2 E_f + tiny), E_f = sum_band w |u_hat|^2 / (2 N^(2d)):
  f'^T g = s g + c w u_hat on the band,  c = -2 eps beta / ((2 E_f + tiny)^2 N^(2d)),
  beta = Re sum_band conj(g) u_hat.
"""

from __future__ import annotations

import numpy as np

from oracle import numpy_ref as R


def _w(N, dim):
    """Half-axis multiplicities; broadcast along the last (half) axis in 2D and 3D."""
    return R.half_weights(N, dim)


def rhs_vjp_wrapper(N, nu, fft_axes=(1, 2, 3), drag=0.0, const_power=None):
    """vjp(u_hat, g) of rhs_wrapper(N, nu, fft_axes, drag, const_power=...)."""
    dim = len(fft_axes)
    kkk, kkk2, kko, dealias = R.wavenumbers(N, dim)
    ikkk = 1j * kkk
    w = _w(N, dim)

    def vjp(u_hat, g):
        pg = (g - np.sum(g * kko, axis=0) * kkk) * dealias
        m = R._irfftn(pg / w, axes=fft_axes)
        u = R._irfftn(u_hat, axes=fft_axes)
        om = R._irfftn(np.cross(ikkk, u_hat, axis=0), axes=fft_axes)
        a = R._rfftn(np.cross(om, m, axis=0), axes=fft_axes)
        b = R._rfftn(np.cross(m, u, axis=0), axes=fft_axes)
        r = w * (a + np.cross(ikkk, b, axis=0))
        r -= (nu * kkk2 + drag) * g
        if const_power is not None:
            eps_inj, mask = const_power
            e_f = R.band_energy(u_hat, mask, N, dim)
            den = 2.0 * e_f + R.EPS
            beta = float(np.sum((np.conj(g) * u_hat * mask).real))
            c = -2.0 * eps_inj * beta / (den * den * float(N) ** (2 * dim))
            r += (eps_inj / den) * g * mask + c * w * u_hat * mask
        return r

    return vjp


def rk4_step(u_hat, dt, rhs_fn):
    """One RK4 step of spectral_solver.py:65-80 with u = irfftn(u_hat) at every stage
    and no ekin_tot rescaling."""
    a = [1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0]
    b = [0.5, 0.5, 1.0]
    u0, acc, us = u_hat, u_hat.copy(), u_hat
    for rk in range(4):
        du = rhs_fn(None, us, 1)
        if rk < 3:
            us = u0 + b[rk] * dt * du
        acc = acc + a[rk] * dt * du
    return acc


def rk4_step_vjp(u_hat0, lam1, dt, rhs_fn, vjp_fn):
    """Cotangent of u_hat at the start of one RK4 step (spectral_solver.py:65-80, no
    ekin_tot rescaling) from the cotangent lam1 of the state after it. The stage
    states are recomputed from the checkpoint u_hat0."""
    k1 = rhs_fn(None, u_hat0, 1)
    ua = u_hat0 + 0.5 * dt * k1
    k2 = rhs_fn(None, ua, 1)
    ub = u_hat0 + 0.5 * dt * k2
    k3 = rhs_fn(None, ub, 1)
    uc = u_hat0 + dt * k3
    lam = lam1.copy()
    r = vjp_fn(uc, dt / 6.0 * lam1)
    lam += r
    r = vjp_fn(ub, dt / 3.0 * lam1 + dt * r)
    lam += r
    r = vjp_fn(ua, dt / 3.0 * lam1 + 0.5 * dt * r)
    lam += r
    r = vjp_fn(u_hat0, dt / 6.0 * lam1 + 0.5 * dt * r)
    lam += r
    return lam


def coarse_mse(u_hat, target, c, fft_axes=(1, 2, 3)):
    """mean((spectral_filtering(irfftn(u_hat), c) - target)^2) over the dim velocity
    components (utils.py:100-138 for the coarsening)."""
    dim = len(fft_axes)
    u = R._irfftn(u_hat, axes=fft_axes)[:dim]
    uc = R.spectral_filtering(u, c)
    return float(np.mean((uc - target) ** 2))


def _box_count(N, c, dim):
    """n(k) = [k in box] + [-k in box] per stored mode, box = [-c/2, c/2 - 1]^dim,
    frequencies taken in [-N/2, N/2 - 1]."""
    idx_full = np.arange(N)
    sgn = np.where(idx_full < N // 2, idx_full, idx_full - N)
    neg = np.where((-idx_full) % N < N // 2, (-idx_full) % N, (-idx_full) % N - N)
    H = N // 2 + 1
    inb = (sgn >= -c // 2) & (sgn <= c // 2 - 1)
    inb_neg = (neg >= -c // 2) & (neg <= c // 2 - 1)
    if dim == 3:
        a = inb[:, None, None] & inb[None, :, None] & inb[None, None, :H]
        b = inb_neg[:, None, None] & inb_neg[None, :, None] & inb_neg[None, None, :H]
    else:
        a = inb[:, None] & inb[None, :H]
        b = inb_neg[:, None] & inb_neg[None, :H]
    return a.astype(np.float64) + b.astype(np.float64)


def coarse_mse_grad(u_hat, target, c, fft_axes=(1, 2, 3)):
    """Gradient of coarse_mse with respect to the fine half spectrum u_hat:
    G = (w / (2 N^d)) n(k) V(k), V = rfftn_c(2 (u_c - target) / size) read at
    (kx mod c, ky mod c, kz); components beyond dim are zero."""
    dim = len(fft_axes)
    N = u_hat.shape[1]
    u = R._irfftn(u_hat, axes=fft_axes)[:dim]
    uc = R.spectral_filtering(u, c)
    v = 2.0 * (uc - target) / uc.size
    V = np.fft.rfftn(v, axes=fft_axes)
    H = N // 2 + 1
    ix = np.arange(N) % c
    kz = np.minimum(np.arange(H), c // 2)
    if dim == 3:
        Vf = V[:, ix][:, :, ix][:, :, :, kz]
    else:
        Vf = V[:, ix][:, :, kz]
    n = _box_count(N, c, dim)
    G = np.zeros(u_hat.shape, dtype=np.complex128)
    G[:dim] = (_w(N, dim) / (2.0 * float(N) ** dim)) * n * Vf
    return G


def trajectory_loss_and_grad(u_hat0, nsteps, dt, rhs_fn, vjp_fn, target, c, fft_axes=(1, 2, 3)):
    """Loss after nsteps RK4 steps from u_hat0 and its gradient with respect to u_hat0
    (checkpoint per step, stages recomputed in the backward sweep)."""
    ck = [u_hat0]
    uh = u_hat0
    for _ in range(nsteps):
        uh = rk4_step(uh, dt, rhs_fn)
        ck.append(uh)
    loss = coarse_mse(uh, target, c, fft_axes)
    lam = coarse_mse_grad(uh, target, c, fft_axes)
    for n in range(nsteps - 1, -1, -1):
        lam = rk4_step_vjp(ck[n], lam, dt, rhs_fn, vjp_fn)
    return loss, lam
