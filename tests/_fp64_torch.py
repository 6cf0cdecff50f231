"""FP64 torch restatement (on the GPU) of the 3D RK4 step, its vector-Jacobian
product and the coarse-grid MSE loss with its gradient.

TEST INFRASTRUCTURE ONLY: finite-difference and gradient references for the 128^3
differentiation workload, where the NumPy oracle would take minutes. Same math as
oracle/numpy_ref.py (rhs_wrapper with const_power, rk4) and oracle/adjoint_ref.py
(rhs_vjp_wrapper, rk4_step_vjp, coarse_mse, coarse_mse_grad); tests/test_adjoint_gpu.py
checks it against them at 32^3.
"""

from __future__ import annotations

import torch


class Fp64Model:
    def __init__(self, n, nu, dt, kf=0, eps_inj=0.0, drag=0.0, device="cuda"):
        f64 = torch.float64
        self.n, self.nu, self.dt, self.kf, self.eps, self.drag = n, nu, dt, kf, eps_inj, drag
        kx = torch.fft.fftfreq(n, 1.0 / n, dtype=f64, device=device)
        kz = kx[: n // 2 + 1].clone()
        kz[-1] *= -1
        self.k = torch.stack(torch.meshgrid(kx, kx, kz, indexing="ij"))
        self.k2 = (self.k * self.k).sum(0)
        self.kok2 = self.k / torch.where(self.k2 == 0, torch.ones_like(self.k2), self.k2)
        kmax = 2.0 / 3.0 * (n // 2 + 1)
        self.dealias = (self.k.abs() < kmax).all(0).to(f64)
        self.band = ((self.k2 > 0) & (self.k2 <= kf * kf)).to(f64) if kf else None
        w = torch.full((n // 2 + 1,), 2.0, dtype=f64, device=device)
        w[0] = w[-1] = 1.0
        self.w = w
        self.s = (n, n, n)
        self.ax = (1, 2, 3)

    def _irfft(self, a):
        return torch.fft.irfftn(a, s=self.s, dim=self.ax)

    def _rfft(self, a):
        return torch.fft.rfftn(a, dim=self.ax)

    def _curl(self, a):
        return 1j * torch.linalg.cross(self.k.to(a.dtype), a, dim=0)

    def _band_energy(self, uh):
        return 0.5 * float((self.w * ((uh * self.band).abs() ** 2).sum(0)).sum()) / float(self.n) ** 6

    def rhs(self, uh):
        u = self._irfft(uh)
        om = self._irfft(self._curl(uh))
        du = self._rfft(torch.linalg.cross(u, om, dim=0)) * self.dealias
        du = du - (du * self.kok2).sum(0) * self.k
        du = du - (self.nu * self.k2 + self.drag) * uh
        if self.band is not None:
            du = du + (self.eps / (2.0 * self._band_energy(uh) + 2.220446049250313e-16)) * uh * self.band
        return du

    def vjp(self, uh, g):
        pg = (g - (g * self.kok2).sum(0) * self.k) * self.dealias
        m = self._irfft(pg / self.w)
        u = self._irfft(uh)
        om = self._irfft(self._curl(uh))
        r = self.w * (self._rfft(torch.linalg.cross(om, m, dim=0)) + self._curl(self._rfft(torch.linalg.cross(m, u, dim=0))))
        r = r - (self.nu * self.k2 + self.drag) * g
        if self.band is not None:
            den = 2.0 * self._band_energy(uh) + 2.220446049250313e-16
            beta = float((torch.conj(g) * uh * self.band).real.sum())
            c = -2.0 * self.eps * beta / (den * den * float(self.n) ** 6)
            r = r + (self.eps / den) * g * self.band + c * self.w * uh * self.band
        return r

    def step(self, uh):
        a = [1 / 6, 1 / 3, 1 / 3, 1 / 6]
        b = [0.5, 0.5, 1.0]
        acc, us = uh.clone(), uh
        for rk in range(4):
            du = self.rhs(us)
            if rk < 3:
                us = uh + b[rk] * self.dt * du
            acc = acc + a[rk] * self.dt * du
        return acc

    def step_vjp(self, u0, lam1):
        dt = self.dt
        ua = u0 + 0.5 * dt * self.rhs(u0)
        ub = u0 + 0.5 * dt * self.rhs(ua)
        uc = u0 + dt * self.rhs(ub)
        lam = lam1.clone()
        r = self.vjp(uc, dt / 6 * lam1)
        lam = lam + r
        r = self.vjp(ub, dt / 3 * lam1 + dt * r)
        lam = lam + r
        r = self.vjp(ua, dt / 3 * lam1 + 0.5 * dt * r)
        lam = lam + r
        r = self.vjp(u0, dt / 6 * lam1 + 0.5 * dt * r)
        return lam + r

    def coarse(self, uh, c):
        n = self.n
        y = torch.fft.fftshift(torch.fft.fftn(self._irfft(uh), dim=self.ax), dim=self.ax)
        sl = slice(n // 2 - c // 2, n // 2 + c // 2)
        y = torch.fft.ifftshift(y[:, sl, sl, sl], dim=self.ax)
        return (torch.fft.ifftn(y, dim=self.ax) / (n / c) ** 3).real

    def coarse_mse(self, uh, target):
        c = target.shape[1]
        return float(((self.coarse(uh, c) - target) ** 2).mean())

    def coarse_mse_grad(self, uh, target):
        n, c = self.n, target.shape[1]
        v = 2.0 * (self.coarse(uh, c) - target) / target.numel()
        V = torch.fft.rfftn(v, dim=self.ax)
        dev = uh.device
        idx = torch.arange(n, device=dev)
        sgn = torch.where(idx < n // 2, idx, idx - n)
        ng = (-idx) % n
        neg = torch.where(ng < n // 2, ng, ng - n)
        H = n // 2 + 1
        inb = (sgn >= -(c // 2)) & (sgn <= c // 2 - 1)
        inn = (neg >= -(c // 2)) & (neg <= c // 2 - 1)
        cnt = ((inb[:, None, None] & inb[None, :, None] & inb[None, None, :H]).double()
               + (inn[:, None, None] & inn[None, :, None] & inn[None, None, :H]).double())
        ix = idx % c
        kz = torch.clamp(torch.arange(H, device=dev), max=c // 2)
        Vf = V[:, ix][:, :, ix][:, :, :, kz]
        return (self.w / (2.0 * float(n) ** 3)) * cnt * Vf

    def loss_and_grad(self, uh0, nsteps, target):
        ck, uh = [], uh0
        for _ in range(nsteps):
            ck.append(uh)
            uh = self.step(uh)
        loss = self.coarse_mse(uh, target)
        lam = self.coarse_mse_grad(uh, target)
        for u0 in reversed(ck):
            lam = self.step_vjp(u0, lam)
        return loss, lam

    def loss_after(self, uh0, nsteps, target):
        uh = uh0
        for _ in range(nsteps):
            uh = self.step(uh)
        return self.coarse_mse(uh, target)
