"""Spectral DNS solver: drop-in for l3es/spectral_solver.py on a GB300.

Same functions, arguments and return tuples as the reference
(``rhs_wrapper``, ``rk4_wrapper``, ``comp_dt``, ``custom_jit_integrate``,
``set_up_solver``, ``simulate``). Fields are torch CUDA tensors: ``u`` float32
(3, N, N, N) or (3, N, N, 1), ``u_hat`` complex64 (3, N, N, N//2+1) or
(3, N, N//2+1) — the reference's layouts. The arithmetic runs in the CUDA library
(FP32 fields, FP64 reductions); there is no CPU fallback.
"""

from __future__ import annotations

import csv
import os
from time import time

import numpy as np

from . import _native
from .init_fields import init_forcing_mask_hit, init_u_hit, init_u_kolm, init_u_random2d, init_u_tgv, init_u_tgv2d

EPS = float(np.finfo(np.float64).eps)  # jnp.finfo(float).eps under x64

_PLANS: dict = {}


def _torch():
    import torch

    return torch


def _plan(dim, n, nu, dt, forcing="none", kf=0, e0=0.0, **ext):
    """Plan cache keyed like the reference's executable cache (spectral_solver.py:221-225):
    one plan per (dim, N, nu, dt, forcing) on the current device."""
    torch = _torch()
    key = (torch.cuda.current_device(), dim, n, float(nu), float(dt), forcing, int(kf or 0),
           tuple(sorted(ext.items())))
    p = _PLANS.get(key)
    if p is None:
        p = _native.Plan(dim=dim, n=n, nu=nu, dt=dt, forcing=forcing, kf=kf or 0, e_kin_init=e0, **ext)
        _PLANS[key] = p
    if forcing == "ekin_tot" and getattr(p, "_e0", None) != float(e0):
        p.set_e0(e0)
        p._e0 = float(e0)
    return p


def _any_plan(dim, n):
    """A cached plan of this grid (for transforms and diagnostics, which do not depend
    on nu, dt or forcing); creates an unforced one if there is none yet."""
    torch = _torch()
    dev = torch.cuda.current_device()
    for key, p in _PLANS.items():
        if key[0] == dev and key[1] == dim and key[2] == n:
            return p
    return _plan(dim, n, 0.0, 1.0)


def _as_spec(u_hat, n, dim):
    torch = _torch()
    t = u_hat if isinstance(u_hat, torch.Tensor) else torch.from_numpy(np.asarray(u_hat))
    t = t.to(device="cuda", dtype=torch.complex64).contiguous()
    shape = (3, n, n, n // 2 + 1) if dim == 3 else (3, n, n // 2 + 1)
    return t.reshape(shape)


def _as_phys(u, n, dim):
    torch = _torch()
    t = u if isinstance(u, torch.Tensor) else torch.from_numpy(np.asarray(u))
    t = t.to(device="cuda", dtype=torch.float32).contiguous()
    return t.reshape((3, n, n, n) if dim == 3 else (3, n, n, 1))


class RhsFn:
    """rhs_fn(u, u_hat, rk) of rhs_wrapper (spectral_solver.py:50-60).

    The velocity is always evaluated from u_hat (at rk = 0 the reference uses the
    caller's u, which equals irfftn(u_hat) up to rounding in every driver)."""

    def __init__(self, N, nu, fft_axes, **ext):
        self.N, self.nu, self.fft_axes, self.ext = int(N), float(nu), tuple(fft_axes), ext
        self.dim = len(self.fft_axes)

    def __call__(self, u, u_hat, rk=0):
        torch = _torch()
        ext = dict(self.ext)
        forcing, kf = ext.pop("forcing", "none"), ext.pop("kf", 0)
        p = _plan(self.dim, self.N, self.nu, 1.0, forcing, kf, **ext)
        uh = _as_spec(u_hat, self.N, self.dim)
        du = torch.empty_like(uh)
        p.rhs(uh, du)
        return du


def rhs_wrapper(N, nu, fft_axes=(1, 2, 3)):
    """Spectral Navier-Stokes right-hand side (spectral_solver.py:27-62)."""
    return RhsFn(N, nu, fft_axes)


def _infer_kf(mask, N):
    mask = np.asarray(mask.cpu() if hasattr(mask, "cpu") else mask).astype(bool)
    for kf in range(1, N // 4 + 1):
        ref = init_forcing_mask_hit(N, kf)
        if ref.shape == mask.shape and np.array_equal(ref, mask):
            return kf
    raise ValueError("forcing_mask must be init_forcing_mask_hit(N, kf) for an integer kf <= N/4")


class StepFn:
    """step_fn(u, u_hat) -> (u, u_hat, e_inj) of rk4_wrapper (spectral_solver.py:73-118).

    Functional like the reference: inputs are not modified. e_inj is a 0-d float64
    device tensor (0 without ekin_tot forcing)."""

    def __init__(self, dt, rhs_fn, forcing_mask, e_kin_init, forcing_type, fft_axes):
        self.dt = float(dt)
        self.N, self.nu, self.dim = rhs_fn.N, rhs_fn.nu, len(tuple(fft_axes))
        self.forcing = "ekin_tot" if (forcing_mask is not None and forcing_type == "ekin_tot") else "none"
        self.kf = _infer_kf(forcing_mask, self.N) if self.forcing == "ekin_tot" else 0
        self.e0 = float(e_kin_init or 0.0)
        self.ext = dict(rhs_fn.ext)

    @property
    def plan(self):
        return _plan(self.dim, self.N, self.nu, self.dt, self.forcing, self.kf, self.e0, **self.ext)

    def __call__(self, u, u_hat):
        torch = _torch()
        p = self.plan
        uh = _as_spec(u_hat, self.N, self.dim).clone()
        u_new = torch.empty(p.phys_shape, dtype=torch.float32, device="cuda")
        e_inj = torch.zeros(1, dtype=torch.float64, device="cuda")
        p.step(uh, 1, u_out=u_new, e_inj=e_inj)
        return u_new, uh, e_inj[0]

    def advance(self, u_hat, nsteps, u_out=None, e_inj=None):
        """In-place variant: nsteps steps on u_hat (no copies)."""
        self.plan.step(u_hat, nsteps, u_out=u_out, e_inj=e_inj)


def rk4_wrapper(dt, rhs_fn, forcing_mask, e_kin_init, forcing_type, fft_axes=(1, 2, 3)):
    """Runge-Kutta 4 integrator (spectral_solver.py:65-120)."""
    return StepFn(dt, rhs_fn, forcing_mask, e_kin_init, forcing_type, fft_axes)


def _field_stats(u, dim):
    torch = _torch()
    n = u.shape[1]
    p = _any_plan(dim, n)
    out = torch.empty(4, dtype=torch.float64, device="cuda")
    p.field_stats(_as_phys(u, n, dim), out)
    return out


def comp_dt(u, dx, nu, cfl=1.0):
    """cfl / min_c(max|u_c| / dx + nu / dx^2) (spectral_solver.py:123-127)."""
    dim = 3 if u.shape[-1] != 1 else 2
    umax = _field_stats(u, dim)[:3].cpu().numpy()
    return float(cfl / (umax / dx + nu / dx**2).min())


def custom_jit_integrate(path_pref, rejit, integrate_fn, u, u_hat):
    """The reference compiles and caches an XLA executable here (spectral_solver.py:130-153).
    The CUDA kernels are compiled ahead of time and plans are cached per configuration,
    so the step function is returned as it is."""
    return integrate_fn


def _initial_field(case, N, dim, seed, ext):
    L = 2 * np.pi
    if case == "TGV3D":
        g = np.arange(N) * L / N
        x, y, z = np.meshgrid(g, g, g, indexing="ij")
        return init_u_tgv(x, y, z)
    if case == "TGV2D":
        return init_u_tgv2d(N, target_dim=3, rescale=L)
    if case == "HIT":
        return init_u_hit(N, seed, ext.get("spectrum", "k-5/3"), ext.get("kp", 4.0))
    if case == "Kolm":
        # init_fields.py:191-212 (spectral_solver.py:195-196); init="random2d" selects the
        # band-limited random-phase field (|k| <= init_kmax, KE init_energy) instead
        if ext.get("init", "kolm") == "random2d":
            return init_u_random2d(N, seed, ext.get("init_kmax", 8.0), ext.get("init_energy", 0.5))
        return init_u_kolm(N, seed=seed, target_dim=3, grid_n=ext.get("kolm_grid", 2048))
    raise ValueError(f"unknown case {case!r}")


def set_up_solver(N, nu, dim, case, dt, seed, ckp_N, kf, e_kin_target=None, forcing_type="ekin_tot",
                  rejit=True, **ext):
    """spectral_solver.py:156-230: grids, initial field, KE rescale, rfftn, E0, step
    function and one warm-up step. Returns the reference's 9-tuple
    (u, u_hat, xyz_vis, dx, integrate_fn, L, fft_axes, e_kin_init, e_inj).

    Extension keywords (no reference counterpart): spectrum='k4exp', kp (HIT init),
    drag, kolm_k, kolm_amp (2D Kolmogorov forcing), eps_inj (constant-power forcing on
    0 < |k| <= kf, selected with forcing_type='const_power'), scheme='integrating_factor'
    (the viscous term integrated exactly by exp(-nu k^2 t) instead of the reference's
    explicit term; default 'explicit')."""
    torch = _torch()
    L = 2 * np.pi
    dx = L / N
    fft_axes = (1, 2, 3) if dim == 3 else (1, 2)
    len_z_vis = ckp_N if dim == 3 else 1
    x = np.arange(ckp_N)
    xyz_vis = np.array(np.meshgrid(x, x, np.arange(len_z_vis), indexing="ij")) * L / ckp_N
    if dim == 2:
        xyz_vis = (xyz_vis.T + np.array([0, 0, L - dx])).T
    init_ext = {k: ext[k] for k in ("spectrum", "kp", "init", "init_kmax", "init_energy", "kolm_grid") if k in ext}
    plan_ext = {k: ext[k] for k in ("drag", "kolm_k", "kolm_amp", "eps_inj", "scheme") if k in ext}
    u = _initial_field(case, N, dim, seed, init_ext)
    e_kin_init = 0.5 * np.mean(np.sum(u * u, axis=0))
    if forcing_type != "none":
        u = u * np.sqrt(e_kin_target / (e_kin_init + EPS))
    e_kin_init = float(0.5 * np.mean(np.sum(u * u, axis=0)))
    u_t = _as_phys(u, N, dim)
    p0 = _any_plan(dim, N)
    u_hat = torch.empty(p0.spec_shape, dtype=torch.complex64, device="cuda")
    p0.rfftn(u_t, u_hat)
    if case == "HIT" and forcing_type == "ekin_tot":
        mask = init_forcing_mask_hit(N, kf)
        rhs = RhsFn(N, nu, fft_axes, **plan_ext)
        integrate_fn = StepFn(dt, rhs, mask, e_kin_init, "ekin_tot", fft_axes)
    elif forcing_type == "const_power":
        rhs = RhsFn(N, nu, fft_axes, forcing="const_power", kf=kf, **plan_ext)
        integrate_fn = _ConstPowerStep(dt, rhs, fft_axes)
    else:
        rhs = RhsFn(N, nu, fft_axes, **plan_ext)
        integrate_fn = StepFn(dt, rhs, None, e_kin_init, "none", fft_axes)
    path_pref = f".cache/spectral_gpu_{N}_{dim}" + (f"_{kf}_{forcing_type}" if forcing_type != "none" else "")
    integrate_fn = custom_jit_integrate(path_pref, rejit, integrate_fn, u_t, u_hat)
    t0 = time()
    u_t, u_hat, e_inj = integrate_fn(u_t, u_hat)
    torch.cuda.synchronize()
    print(f"[l3es_gb300] warm-up step {time() - t0:.3f} s")
    return u_t, u_hat, xyz_vis, dx, integrate_fn, L, fft_axes, e_kin_init, e_inj


class _ConstPowerStep(StepFn):
    """Extension: RK4 with the constant-power band forcing inside the right-hand side."""

    def __init__(self, dt, rhs_fn, fft_axes):
        ext = dict(rhs_fn.ext)
        self.band_kf = int(ext.pop("kf"))
        ext.pop("forcing")
        rhs_fn.ext = ext
        super().__init__(dt, rhs_fn, None, 0.0, "none", fft_axes)

    @property
    def plan(self):
        return _plan(self.dim, self.N, self.nu, self.dt, "const_power", self.band_kf, 0.0, **self.ext)


def simulate(case="TGV3D", N=64, dim=3, nu=0.000625, t_final=0.1, t_burnin=0.0, dt=0.01, u_ref=1.0,
             ckp_N=32, seed=42, rejit=True, forcing_type="none", e_kin_target=None, kf=None, log_freq=20,
             vis_freq=10**8, ckp_freq=1, dst_path=None):
    """Simulation driver (spectral_solver.py:233-367): same loop order, burn-in forcing
    switch, diagnostics.csv columns, write_u checkpoints and TGV validation. Plots
    (vis_freq) are not produced: they are matplotlib output outside the hot path."""
    from .utils import write_u

    torch = _torch()
    u, u_hat, xyz_vis, dx, integrate_fn, L, _, e_kin_init, e_inj = set_up_solver(
        N, nu, dim, case, dt, seed, ckp_N, kf, e_kin_target, forcing_type, rejit)
    dst_path = dst_path or "results"
    dst_ckp = os.path.join(dst_path, "sim")
    os.makedirs(dst_path, exist_ok=True)
    diagnostics_path = os.path.join(dst_path, "diagnostics.csv")
    with open(diagnostics_path, "w", newline="") as f:
        csv.writer(f).writerow(["step", "time", "umax", "ekin", "dt_est", "e_inj"])
    e_inj_acc = torch.zeros((), dtype=torch.float64, device="cuda")
    print(f"[l3es_gb300] {case} dim={dim} N={N} nu={nu} dt={dt} t_final={t_final} KE0={e_kin_init:.4f}")
    t_sim, t0 = 0.0, time()
    tstep_max = round(t_final / dt)
    burnin_steps = round(t_burnin / dt) if t_burnin > 0 else 0
    e_kin = None
    i = 0
    for i in range(tstep_max + 1):
        if i == burnin_steps and case == "HIT":
            _, _, _, _, integrate_fn, _, _, _, _ = set_up_solver(
                N, nu, dim, case, dt, seed, ckp_N, kf, e_kin_target, "none", rejit)
        t_temp = time()
        u, u_hat, e_inj = integrate_fn(u, u_hat)
        torch.cuda.synchronize()
        t_sim += time() - t_temp
        _check_blowup(integrate_fn, i)
        e_inj_acc += e_inj
        if i % log_freq == 0:
            st = _field_stats(u, dim).cpu().numpy()
            umax, e_kin = float(st[:3].max()), float(st[3])
            dt_est = float(dt_from_stats(st, dx, nu))
            with open(diagnostics_path, "a", newline="") as f:
                csv.writer(f).writerow([i, float(i * dt), umax, e_kin, dt_est, float(e_inj)])
            print(f"[{i:>7d}/{tstep_max}] umax {umax:.4f}  KE {e_kin:.4f}  dt_cfl {dt_est:.5f}  "
                  f"e_inj {float(e_inj):.4f}")
        if i == burnin_steps:
            write_u(u, i, dst_path, N, suffix="_burnin")
        if i % ckp_freq == 0 and i >= burnin_steps:
            write_u(u, i, dst_ckp, ckp_N)
    if case == "HIT" and forcing_type != "none" and i > 0:
        avg = float(e_inj_acc) / i
        if avg > 0:
            tau = 1.0 / (avg * kf**2) ** (1 / 3)
            kmax = np.sqrt(2) * N / 3
            eta = (nu**3 / avg) ** 0.25
            re_l = f", Re_lambda {np.sqrt(20 * e_kin**2 / (3 * nu * avg)):.2f}" if e_kin is not None else ""
            print(f"[l3es_gb300] forced HIT: mean injection {avg:.4f}, large-eddy time {tau:.3f} "
                  f"({t_final / tau:.2f} of them simulated), Kolmogorov scale {eta:.4f}, "
                  f"kmax*eta {kmax * eta:.3f}{re_l}")
    print(f"[l3es_gb300] wall {time() - t0:.2f} s, of which stepping {t_sim:.2f} s")
    if t_final == 0.1 and case == "TGV3D":
        e_kin = float(_field_stats(u, dim)[3])
        assert round(e_kin - 0.124953117517, 2) == 0, f"e_kin = {e_kin}"
        print("[l3es_gb300] TGV3D kinetic energy matches the spectralDNS value")
    return u, u_hat


def _check_blowup(integrate_fn, step):
    """Raises NonFiniteError naming the step if the last step of the driver's step
    function wrote NaN or infinite values (the plan's device flag, set by the final
    RK update; the reference shows a blow-up only in its umax / dt_est log columns,
    spectral_solver.py:318-324). The drivers synchronise every step anyway."""
    p = getattr(integrate_fn, "plan", None)
    if p is None:
        return
    try:
        p.check()
    except _native.NonFiniteError as e:
        raise _native.NonFiniteError(f"step {step}: {e}") from None


def dt_from_stats(stats, dx, nu, cfl=1.0):
    """comp_dt from the per-component maxima returned by the field statistics kernel."""
    umax = np.asarray(stats[:3], dtype=np.float64)
    return cfl / (umax / dx + nu / dx**2).min()
