"""DNS + Lagrangian particles driver: drop-in for l3es/combined.py.

Same keyword set and loop order as the reference (combined.py:18-219): at every step
the DNS advances, the field is coarsened to ckp_N, the particle velocity is
interpolated from it at the positions from before the step's advection, and the
particles move by an explicit Euler shift. On the GPU the coarsening is taken
directly from the fine spectrum and the interpolation and shift are fused
(l3es_interp_set_spectrum + l3es_interp with r_out).

With relax_dt_factor > 0 the interpolated velocity is relaxed by one SPH step at the
predicted positions (combined.py:132-142) in one fused call (l3es_sph_relax_velocity,
which also advects the particles with the relaxed velocity). The SPH density maximum
is logged on log/checkpoint steps as in the reference. Outside this package: plots.
Particle checkpoints go to step_XXXXX.npz files with the reference's keys r and u (the
unrelaxed interpolated velocity, as the reference writes; the reference writes h5
through JAX-SPH), and the run's settings to config.json (sim / com sections).
"""

from __future__ import annotations

import csv
import json
import os
from time import time

import numpy as np

from .integrator import set_up_integrator
from .relax import relax_velocity_wrapper
from .spectral_solver import _check_blowup, _field_stats, dt_from_stats, set_up_solver, _torch
from .utils import _interp_plan, write_u


def combined(case, N=256, dim=3, nu=0.000625, t_final=0.1, t_burnin=0, dt=0.01, u_ref=4.0, ckp_N=64,
             state_0_path=None, interp_backend="dft", relax_dt_factor=0.0, dft_splits=8, seed=42, rejit=True,
             forcing_type="none", e_kin_target=None, kf=None, log_freq=100, vis_freq=100, ckp_freq=100,
             dst_path=None, **ext):
    """Integrate particles along the DNS velocity (combined.py:18-219). Returns the final
    (u, u_hat, r).

    Extension keyword (besides set_up_solver's): advection='rk4' moves the particles by
    one classical RK4 step through the step's coarse field held fixed
    (l3es_interp_advect_rk4) instead of the reference's Euler shift; it cannot be
    combined with relax_dt_factor > 0, whose relaxation step does its own shift."""
    torch = _torch()
    advection = ext.pop("advection", "euler")
    if advection not in ("euler", "rk4"):
        raise ValueError(f"advection must be 'euler' or 'rk4', got {advection!r}")
    if advection == "rk4" and (relax_dt_factor or 0.0) > 0.0:
        raise ValueError("advection='rk4' and SPH relaxation (relax_dt_factor > 0) exclude each other")
    dst_path = dst_path or "results"
    int_path = os.path.join(dst_path, "com")
    os.makedirs(int_path, exist_ok=True)
    # the run's settings in the reference's config layout (main.py:72-73 saves the merged
    # config.yaml beside the trajectory); gen_dataset reads it for the dataset metadata
    with open(os.path.join(dst_path, "config.json"), "w") as f:
        json.dump({"mode": "combined", "seed": seed,
                   "sim": {"case": case, "N": N, "dim": dim, "nu": nu, "t_final": t_final, "t_burnin": t_burnin,
                           "dt": dt, "u_ref": u_ref, "ckp_N": ckp_N, "forcing_type": forcing_type,
                           "e_kin_target": e_kin_target, "kf": kf},
                   "com": {"state_0_path": state_0_path, "interp_backend": interp_backend,
                           "relax_dt_factor": relax_dt_factor, "dft_splits": dft_splits, "log_freq": log_freq,
                           "vis_freq": vis_freq, "ckp_freq": ckp_freq, "dst_path": dst_path}}, f, indent=1)
    diagnostics_path = os.path.join(dst_path, "diagnostics.csv")
    with open(diagnostics_path, "w", newline="") as f:
        csv.writer(f).writerow(["step", "time", "umax", "ekin", "dt_est", "e_inj", "rho_max"])

    u, u_hat, xyz_vis, dx_dns, integrate_fn, L, fft_axes, ek_ini, e_inj = set_up_solver(
        N, nu, dim, case, dt, seed, ckp_N, kf, e_kin_target, forcing_type, rejit, **ext)
    print(f"[l3es_gb300] {case} + particles dim={dim} N={N} nu={nu} dt={dt} t_final={t_final} KE0={ek_ini:.4f}")
    r, comp_rho, _, _, _, _, _ = set_up_integrator(state_0_path, dim, ckp_N, dft_splits, u_ref, interp_backend)
    npart = r.shape[0]
    ip = _interp_plan(dim, N, ckp_N, np_max=npart)
    relax = relax_velocity_wrapper(ckp_N, dim, L, u_ref, relax_dt_factor) if (relax_dt_factor or 0.0) > 0.0 else None
    u_r = torch.empty_like(r)
    r_next = torch.empty_like(r)
    e_acc = torch.zeros((), dtype=torch.float64, device="cuda")

    t_sim, t_int, t0 = 0.0, 0.0, time()
    tstep_max = round(t_final / dt)
    burnin_steps = round(t_burnin / dt) if t_burnin > 0 else 0
    for i in range(tstep_max + 1):
        if i == burnin_steps:
            write_u(u, i, dst_path, N, suffix="_burnin")
        if i == burnin_steps and case == "HIT":
            _, _, _, _, integrate_fn, _, _, _, _ = set_up_solver(
                N, nu, dim, case, dt, seed, ckp_N, kf, e_kin_target, "none", rejit, **ext)
        t_temp = time()
        u, u_hat, e_inj = integrate_fn(u, u_hat)
        torch.cuda.synchronize()
        t_sim += time() - t_temp
        _check_blowup(integrate_fn, i)
        e_acc += e_inj

        t_temp = time()
        # u_lres = spectral_filtering(u_hres, ckp_N); u_r = interpolator(u_lres, r);
        # r_next = shift_fn(r, dt * u_r)   (combined.py:122-130, :199)
        ip.set_spectrum(u_hat)
        if advection == "rk4":
            ip.advect_rk4(r, u_r, dt, r_next, backend=interp_backend)
        elif relax is None:
            ip.interp(r, u_r, backend=interp_backend, dt=dt, r_out=r_next)
        else:
            # u_r_0 kept for the checkpoint; particles advance with the relaxed velocity
            ip.interp(r, u_r, backend=interp_backend)
            relax(r, u_r, dt, r_out=r_next)
        torch.cuda.synchronize()
        t_int += time() - t_temp

        is_ckp = (i % ckp_freq == 0) and (i >= burnin_steps)
        rho_max = ""
        if i % log_freq == 0 or is_ckp or i % vis_freq == 0:
            rho_max = float(comp_rho(r).max())
        if i % log_freq == 0:
            st = _field_stats(u, dim).cpu().numpy()
            umax, e_kin = float(st[:3].max()), float(st[3])
            dt_est = float(dt_from_stats(st, dx_dns, nu))
            with open(diagnostics_path, "a", newline="") as f:
                csv.writer(f).writerow([i, float(i * dt), umax, e_kin, dt_est, float(e_inj), rho_max])
            print(f"[{i:>7d}/{tstep_max}] umax {umax:.4f}  KE {e_kin:.4f}  dt_cfl {dt_est:.5f}  "
                  f"e_inj {float(e_inj):.4f}  rho_max {rho_max:.4f}")
        if is_ckp:
            np.savez(os.path.join(int_path, f"step_{i:05d}.npz"), r=r.cpu().numpy(), u=u_r.cpu().numpy())
        r, r_next = r_next, r

    if case == "HIT" and forcing_type != "none" and tstep_max > 0:
        avg = float(e_acc) / tstep_max
        if avg > 0:
            tau = 1.0 / (avg * kf**2) ** (1 / 3)
            print(f"[l3es_gb300] forced HIT: mean injection {avg:.4f}, large-eddy time {tau:.3f} "
                  f"({t_final / tau:.2f} of them simulated)")
    print(f"[l3es_gb300] wall {time() - t0:.2f} s: stepping {t_sim:.2f} s, particles {t_int:.2f} s")
    return u, u_hat, r
