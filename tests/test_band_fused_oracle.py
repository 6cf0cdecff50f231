"""The band-fused RK4 step form, restated in FP64 NumPy on the CPU, equals the reference's
RK4 step (oracle rk4_wrapper, following spectral_solver.py:65-80) to FP64 rounding.

The restatement follows the kernels' data flow (csrc/dns_kernels.cuh: XLin, BandRk):
the band B = {|kx| <= kd, |ky| <= kd, kz < kt} is updated in place in the state, with
the step's initial band values kept aside (P) and the accumulator over B only (C); every
other mode keeps u0 in the state during the step, enters each stage's right-hand side
scaled by its closed-form stage polynomial, and is written once, at the last stage, as
P4(z) u0. A wrong stage polynomial, band or accumulator rebuild shows up here at the
1e-6 level against the 1e-12 this test allows.
"""

import numpy as np
import pytest

from oracle import numpy_ref as R

A_RK4 = (1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0)
B_RK4 = (0.5, 0.5, 1.0)


def _lin_stage_factor(rk, z):
    """Field written by stage rk of a mode with du = -z/dt u, over u0 (rk 3: new state)."""
    return (1 - z / 2,
            1 - z / 2 + z * z / 4,
            1 - z + z * z / 2 - z ** 3 / 4,
            1 - z + z * z / 2 - z ** 3 / 6 + z ** 4 / 24)[rk]


def _dealias_kd(n):
    kd = 0
    while kd + 1 < 2.0 / 3.0 * (n // 2 + 1):
        kd += 1
    return kd


def band_fused_step(uh, rhs, dt, nu, drag, n, kt, dim=3):
    """One RK4 step in the band-fused form (FP64). rhs(u_hat) is the full right-hand side.
    2D: the band is |kx| <= kd, khalf < kt (the half axis is the second one)."""
    kkk, kkk2, _, _ = R.wavenumbers(n, dim)
    kd = _dealias_kd(n)
    if dim == 3:
        band = (np.abs(kkk[0]) <= kd) & (np.abs(kkk[1]) <= kd) & (np.arange(n // 2 + 1)[None, None, :] < kt)
    else:
        band = (np.abs(kkk[0]) <= kd) & (np.arange(n // 2 + 1)[None, :] < kt)
    z = (nu * kkk2 + drag) * dt
    S = uh.copy()
    P = None
    C = None
    for rk in range(4):
        # the x inverse's view of the stage input: S on the band, the stage polynomial of
        # the previous stage times u0 (still in S) elsewhere
        us = S if rk == 0 else np.where(band, S, _lin_stage_factor(rk - 1, z) * S)
        du = rhs(us)
        if rk == 0:  # P <- u0 on the band; no accumulator yet
            P = np.where(band, S, 0)
            S = np.where(band, S + B_RK4[0] * dt * du, S)
        elif rk == 1:  # accumulator rebuilt from the stage-0 field: a0 dt k1 = (a0/b0)(us - u0)
            C = np.where(band, P + (A_RK4[0] / B_RK4[0]) * (us - P) + A_RK4[1] * dt * du, 0)
            S = np.where(band, P + B_RK4[1] * dt * du, S)
        elif rk == 2:
            C = np.where(band, C + A_RK4[2] * dt * du, 0)
            S = np.where(band, P + B_RK4[2] * dt * du, S)
        else:  # the band from the accumulator, every other mode by its closed form
            S = np.where(band, C + A_RK4[3] * dt * du, _lin_stage_factor(3, z) * S)
    return S


@pytest.mark.parametrize("forced,drag", [(False, 0.0), (True, 0.0), (False, 0.07)])
def test_band_fused_step_is_the_reference_rk4_step(forced, drag):
    n, nu, dt = 16, 2e-2, 5e-3
    kt = 8  # the kernels' stored half-axis columns at n = 16 (kd + 1 = 6, rounded up to 8)
    u = R.init_u_hit(n, 9, spectrum="k4exp", kp=3.0)
    u *= np.sqrt(0.5 / R.kinetic_energy(u))
    uh = np.fft.rfftn(u, axes=(1, 2, 3))
    cp = None
    if forced:
        _, kkk2, _, _ = R.wavenumbers(n, 3)
        cp = (0.1, ((kkk2 > 0) & (kkk2 <= 4)).astype(float))
    rhs_fn = R.rhs_wrapper(n, nu, drag=drag, const_power=cp)
    step = R.rk4_wrapper(dt, rhs_fn, None, 0.0, "none")
    ref_u, ref_uh = u, uh
    got = uh
    for _ in range(3):
        ref_u, ref_uh, _ = step(ref_u, ref_uh)
        got = band_fused_step(got, lambda x: rhs_fn(None, x, 1), dt, nu, drag, n, kt)
    err = np.abs(got - ref_uh).max() / np.abs(ref_uh).max()
    assert err < 1e-12, err


def test_band_fused_step_is_the_reference_rk4_step_in_2d():
    """2D Kolmogorov flow (drag, sin 4y forcing) at 32^2: the forcing mode (0, 4) lies in
    the band (kt = 16), so the band-fused form applies."""
    n, nu, dt, steps = 32, 1e-3, 1e-3, 3
    kt = 16  # kd + 1 = 12, rounded up to a multiple of 8
    u = R.init_u_random2d(n, 11)
    uh = np.fft.rfftn(u, axes=(1, 2)).squeeze()
    rhs_fn = R.rhs_wrapper(n, nu, (1, 2), drag=0.1, force_hat=R.kolmogorov_forcing_hat(n, 1.0, 4))
    step = R.rk4_wrapper(dt, rhs_fn, None, 0.0, "none", (1, 2))
    ref_u, ref_uh, got = u, uh, uh
    for _ in range(steps):
        ref_u, ref_uh, _ = step(ref_u, ref_uh)
        got = band_fused_step(got, lambda x: rhs_fn(None, x, 1), dt, nu, 0.1, n, kt, dim=2)
    err = np.abs(got - ref_uh).max() / np.abs(ref_uh).max()
    assert err < 1e-12, err
