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


def ekin_tot_forward(u_rk, mask, e0, N, dim):
    """The ekin_tot rescaling after the RK4 update (spectral_solver.py:82-112) in the
    Parseval form: E = sum w |u_hat|^2 / (2 N^(2d)) over the stored modes, E_low over the
    band (mask), alpha = sqrt(max(0, (E0 - (E - E_low)) / (E_low + eps)));
    u_new = u_rk (alpha mask + 1 - mask). Returns (u_new, alpha, E_high, E_low)."""
    w = _w(N, dim)
    nd = float(N) ** (2 * dim)
    e_all = np.sum(w * np.sum(np.abs(u_rk) ** 2, axis=0)) / (2.0 * nd)
    e_low = np.sum(w * np.sum(np.abs(u_rk * mask) ** 2, axis=0)) / (2.0 * nd)
    e_high = e_all - e_low
    alpha = np.sqrt(max(0.0, (e0 - e_high) / (e_low + R.EPS)))
    return u_rk * (alpha * mask + (1 - mask)), alpha, e_high, e_low


def ekin_tot_vjp(u_rk, lam, mask, e0, N, dim):
    """Adjoint of ekin_tot_forward at u_rk for the cotangent lam of u_new:
    with beta = Re sum_band conj(lam) u_rk and d alpha = (1 / (2 alpha)) (-dE_high / (E_low + eps)
    - (E0 - E_high) dE_low / (E_low + eps)^2), dE = Re sum w conj(u_rk) du / N^(2d):
        lam_rk = (1 - mask) (lam - c_h w u_rk) + mask (alpha lam - c_l w u_rk),
        c_h = beta / (2 alpha (E_low + eps) N^(2d)),  c_l = beta alpha / (2 (E_low + eps) N^(2d))
    (alpha = 0, where the rescaling saturates, contributes no alpha term)."""
    w = _w(N, dim)
    nd = float(N) ** (2 * dim)
    _, alpha, e_high, e_low = ekin_tot_forward(u_rk, mask, e0, N, dim)
    beta = float(np.real(np.sum(np.conj(lam) * u_rk * mask)))
    if alpha > 0.0:
        c_h = beta / (2.0 * alpha * (e_low + R.EPS) * nd)
        c_l = beta * alpha / (2.0 * (e_low + R.EPS) * nd)
    else:
        c_h = c_l = 0.0
    return (1 - mask) * (lam - c_h * w * u_rk) + mask * (alpha * lam - c_l * w * u_rk)


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


def coarse_field_vjp(v, N, c, fft_axes=(1, 2, 3), ncomp=3):
    """Adjoint of u_hat -> spectral_filtering(irfftn(u_hat), c) (utils.py:100-138): the
    gradient with respect to the fine half spectrum of L = sum(v * u_c) for a real
    coarse-grid cotangent v (dim, c, ...):
    G = (w / (2 N^d)) n(k) V(k), V = rfftn_c(v) read at (kx mod c, ky mod c, kz);
    components beyond dim are zero."""
    dim = len(fft_axes)
    V = np.fft.rfftn(v, axes=fft_axes)
    H = N // 2 + 1
    ix = np.arange(N) % c
    kz = np.minimum(np.arange(H), c // 2)
    if dim == 3:
        Vf = V[:, ix][:, :, ix][:, :, :, kz]
    else:
        Vf = V[:, ix][:, :, kz]
    n = _box_count(N, c, dim)
    shape = (ncomp, N, N, H) if dim == 3 else (ncomp, N, H)
    G = np.zeros(shape, dtype=np.complex128)
    G[:dim] = (_w(N, dim) / (2.0 * float(N) ** dim)) * n * Vf
    return G


def coarse_mse_grad(u_hat, target, c, fft_axes=(1, 2, 3)):
    """Gradient of coarse_mse with respect to the fine half spectrum u_hat (the
    coarse-field adjoint of the residual 2 (u_c - target) / size)."""
    dim = len(fft_axes)
    N = u_hat.shape[1]
    u = R._irfftn(u_hat, axes=fft_axes)[:dim]
    uc = R.spectral_filtering(u, c)
    v = 2.0 * (uc - target) / uc.size
    return coarse_field_vjp(v, N, c, fft_axes, ncomp=u_hat.shape[0])


def interp_vjp(lam, r, N, c, fft_axes=(1, 2, 3)):
    """Gradient with respect to the fine half spectrum of L = sum(lam * u_r), u_r the
    particle velocities of the combined loop (spectral_filtering to c, then the exact
    spectral interpolation of integrator.py:62-91 at r; interpolate_from_uhat_dft).
    lam, r: (Np, dim). The interpolation u_r = Re sum_k U(k) exp(i k.r) / c^d over the
    c^d modes of U = fftn(u_c) has the coarse-grid adjoint
        v(x) = Re sum_k Ubar(k) exp(i k.x),  Ubar(k) = sum_j lam_j exp(-i k.r_j) / c^d,
    which then goes through coarse_field_vjp."""
    dim = len(fft_axes)
    k = np.fft.fftfreq(c, 1.0 / c)
    ph = [np.exp(-1j * r[:, d, None] * k[None, :]) for d in range(dim)]  # (Np, c) per axis
    if dim == 3:
        ub = np.einsum("jc,ja,jb,jz->cabz", lam, ph[0], ph[1], ph[2])
    else:
        ub = np.einsum("jc,ja,jb->cab", lam, ph[0], ph[1])
    ub /= float(c) ** dim
    v = np.real(np.fft.ifftn(ub, axes=fft_axes)) * float(c) ** dim
    return coarse_field_vjp(v, N, c, fft_axes)


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
