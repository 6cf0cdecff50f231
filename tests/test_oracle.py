"""The FP64 oracle against the reference's own golden vectors (CPU only)."""

import os

import numpy as np
import pytest

from oracle import numpy_ref as R
from oracle import nufft_ref as NU

from conftest import GOLDEN


def _rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


def test_tgv3d_rk4_matches_reference(gold):
    g = gold("tgv3d_n16")
    N = int(g["N"])
    step = R.rk4_wrapper(float(g["dt"]), R.rhs_wrapper(N, float(g["nu"])), None, 0.0, "none")
    u, uh = g["u0"], g["u_hat0"]
    for _ in range(int(g["steps"])):
        u, uh, _ = step(u, uh)
    assert _rel(uh, g["u_hat"]) < 1e-12
    assert _rel(u, g["u"]) < 1e-12
    # the reference's two implementations agree with each other too
    assert _rel(g["u_hat_spectraldns"], g["u_hat"]) < 1e-12


def test_random3d_rhs_and_steps(gold):
    g = gold("rand3d_n16")
    N, nu, dt = int(g["N"]), float(g["nu"]), float(g["dt"])
    rhs = R.rhs_wrapper(N, nu)
    assert _rel(rhs(g["u0"], g["u_hat0"], 0), g["rhs_rk0"]) < 1e-12
    assert _rel(rhs(g["u0"], g["u_hat0"], 1), g["rhs_rk1"]) < 1e-12
    step = R.rk4_wrapper(dt, rhs, None, 0.0, "none")
    u, uh = g["u0"], g["u_hat0"]
    for _ in range(int(g["steps"])):
        u, uh, _ = step(u, uh)
    assert _rel(uh, g["u_hat"]) < 1e-12


def test_hit_init_and_ekin_forcing(gold):
    g = gold("hit3d_n16_ekin")
    N = int(g["N"])
    assert _rel(R.init_u_hit(N, int(g["seed"])), g["u_init"]) < 1e-13
    assert np.array_equal(R.init_forcing_mask_hit(N, int(g["kf"])), g["forcing_mask"])
    u, uh, dx, fn, L, axes, e0, e_inj = R.set_up_solver(
        N, float(g["nu"]), 3, "HIT", float(g["dt"]), int(g["seed"]), 8, int(g["kf"]),
        float(g["e_kin_target"]), "ekin_tot")
    assert abs(e0 - float(g["e_kin_init"])) < 1e-13
    hist = [e_inj]
    for _ in range(int(g["steps_after_setup"])):
        u, uh, e = fn(u, uh)
        hist.append(e)
    assert _rel(uh, g["u_hat"]) < 1e-11
    assert np.allclose(hist, g["e_inj"], rtol=1e-9, atol=1e-12)
    # ekin_tot pins the kinetic energy to its initial value
    assert abs(R.kinetic_energy(u) - e0) < 1e-10


def test_tgv2d_setup_and_steps(gold):
    g = gold("tgv2d_n32")
    N = int(g["N"])
    assert _rel(R.init_u_tgv2d(N, 3, 2 * np.pi), g["u_init"]) < 1e-14
    u, uh, dx, fn, *_ = R.set_up_solver(N, float(g["nu"]), 2, "TGV2D", float(g["dt"]),
                                        42, 8, None, None, "none")
    for _ in range(int(g["steps_after_setup"])):
        u, uh, _ = fn(u, uh)
    assert uh.shape == g["u_hat"].shape and u.shape == g["u"].shape
    assert _rel(uh, g["u_hat"]) < 1e-12


def test_random2d_three_components(gold):
    g = gold("rand2d_n32")
    N = int(g["N"])
    step = R.rk4_wrapper(float(g["dt"]), R.rhs_wrapper(N, float(g["nu"]), (1, 2)),
                         None, 0.0, "none", (1, 2))
    u, uh = g["u0"], g["u_hat0"]
    for _ in range(int(g["steps"])):
        u, uh, _ = step(u, uh)
    assert _rel(uh, g["u_hat"]) < 1e-12


def test_utils(gold):
    g = gold("utils")
    assert _rel(R.spectral_filtering(g["f3"], 8), g["filt3_8"]) < 1e-13
    assert _rel(R.spectral_filtering(g["f2"], 8), g["filt2_8"]) < 1e-13
    assert _rel(R.spectral_filtering(g["f3"], 16), g["filt3_16"]) < 1e-13
    assert _rel(R.energy_spectrum(g["f3"]), g["ek3"]) < 1e-12
    v2 = np.concatenate([g["f2"], 0 * g["f2"][:1]])[..., None]
    assert _rel(R.energy_spectrum(v2, dim=2), g["ek2"]) < 1e-12
    uh3 = np.fft.rfftn(g["f3"], axes=(1, 2, 3))
    assert abs(R.comp_dissipation_rate(uh3, 0.01) - float(g["diss3"])) < 1e-12 * abs(float(g["diss3"]))
    assert abs(R.comp_dt(g["f3"], 2 * np.pi / 16, 0.01, 0.5) - float(g["dt3"])) < 1e-15


def test_interp_dft_and_shift(gold):
    g = gold("interp")
    assert _rel(R.interpolate_dft(g["g3"], g["r3"]), g["ur3"]) < 1e-12
    assert _rel(R.interpolate_dft(g["g2"], g["r2"]), g["ur2"]) < 1e-12
    assert _rel(R.shift_fn(g["r3"], g["dr"]), g["shifted"]) < 1e-15


def test_nufft_restatement_accuracy(gold):
    g = gold("interp")
    for w, tol in ((6, 1e-4), (8, 1e-6)):
        a = NU.interpolate_nufft(g["g3"], g["r3"], w=w)
        assert _rel(a, g["ur3"]) < tol
        b = NU.interpolate_nufft(g["g2"], g["r2"], w=w)
        assert _rel(b, g["ur2"]) < tol


@pytest.mark.slow
def test_tgv64_known_answer():
    """from_spectralDNS/main_numpy.py:134-137: KE after 10 steps, 7 decimals."""
    N = 64
    xyz = np.mgrid[:N, :N, :N].astype(float) * 2 * np.pi / N
    u = R.init_u_tgv(*xyz)
    uh = np.fft.rfftn(u, axes=(1, 2, 3))
    step = R.rk4_wrapper(0.01, R.rhs_wrapper(N, 0.000625), None, 0.0, "none")
    for _ in range(10):
        u, uh, _ = step(u, uh)
    ke = R.kinetic_energy(u)
    assert round(ke - 0.124953117517, 7) == 0
    ref = float(open(os.path.join(GOLDEN, "tgv64_ke.txt")).read().splitlines()[-1])
    assert abs(ke - ref) < 1e-14


def test_particles_to_grid_dft(gold):
    g = gold("p2g")
    c3, c2 = int(g["c3"]), int(g["c2"])
    u3 = R.particles_to_grid_dft(g["r3"], g["u3"], c3)
    assert _rel(u3.reshape(3, -1).T, g["grid3"]) < 1e-12
    assert _rel(u3, g["ugrid3"]) < 1e-12
    u2 = R.particles_to_grid_dft(g["r2"], g["u2"], c2)
    assert _rel(u2.reshape(2, -1).T, g["grid2"]) < 1e-12
    assert _rel(R.energy_spectrum(u3), g["ek3"]) < 1e-12


def _lattice(n, dim, jitter=0.0, seed=0):
    L = 2 * np.pi
    r = R.pos_init_cartesian(L, n, dim)
    if jitter:
        r = np.mod(r + jitter * (L / n) * np.random.default_rng(seed).uniform(-1, 1, r.shape), L)
    return r


def test_sph_quintic_normalisation():
    """The restated quintic constants: the 2D kernel integrates to 1; the 3D constant
    3/(359 pi) of the published kernel integrates to 360/359."""
    from scipy.integrate import quad

    from oracle import sph_ref as S

    h = 0.37
    i2 = quad(lambda r: 2 * np.pi * r * S.quintic_w(r, h, 2), 0, 3 * h, points=[h, 2 * h])[0]
    i3 = quad(lambda r: 4 * np.pi * r * r * S.quintic_w(r, h, 3), 0, 3 * h, points=[h, 2 * h])[0]
    assert abs(i2 - 1.0) < 1e-12 and abs(i3 - 360 / 359) < 1e-12
    q = np.linspace(0.01, 2.99, 50)
    num = (S.quintic_w(q + 1e-6, 1.0, 3) - S.quintic_w(q - 1e-6, 1.0, 3)) / 2e-6
    assert np.abs(num - S.quintic_grad_w(q, 1.0, 3)).max() < 1e-6 * np.abs(num).max()


@pytest.mark.parametrize("n,dim", [(8, 3), (12, 2)])
def test_sph_tree_search_matches_bruteforce(n, dim):
    from oracle import sph_ref as S

    r = _lattice(n, dim, jitter=0.4, seed=1)
    L, cut = 2 * np.pi, 3 * 2 * np.pi / n
    i, j, d = S._pairs(r, L, cut)
    bi, bj, bd = S.pairs_bruteforce(r, L, cut)
    a = sorted(zip(i.tolist(), j.tolist()))
    assert a == sorted(zip(bi.tolist(), bj.tolist()))
    key = {(x, y): k for k, (x, y) in enumerate(zip(bi.tolist(), bj.tolist()))}
    order = [key[(x, y)] for x, y in zip(i.tolist(), j.tolist())]
    assert np.abs(d - bd[order]).max() < 1e-12


@pytest.mark.parametrize("n,dim", [(16, 3), (32, 2)])
def test_sph_lattice_and_momentum(n, dim):
    """A lattice has uniform density and no net acceleration; the pair forces of a
    jittered set are antisymmetric, so they sum to zero."""
    from oracle import sph_ref as S

    rho = S.density(_lattice(n, dim), n, dim)
    assert np.ptp(rho) < 1e-12 and abs(rho.mean() - (1.0027654191593 if dim == 3 else 1.0000632245946)) < 1e-9
    assert np.abs(S.relax_acceleration(_lattice(n, dim), n, dim, 4.0)).max() < 1e-9
    r = _lattice(n, dim, jitter=0.3, seed=2)
    a = S.relax_acceleration(r, n, dim, 4.0)
    assert np.abs(a.sum(0)).max() < 1e-9 * np.abs(a).max() * len(r)
    u = np.random.default_rng(3).standard_normal(r.shape)
    f = S.sph_forces(r, u, n, dim, 4.0)
    np.testing.assert_allclose(f["acc_p"] + 0.5 * f["acc_tvf"], a, rtol=0, atol=1e-9 * np.abs(a).max())
    assert np.abs(f["acc_visc"].sum(0)).max() < 1e-9 * np.abs(f["acc_visc"]).max() * len(r)


def test_integrating_factor_oracle_decays_a_shear_mode_exactly():
    """Extension oracle term: for u = (sin y, 0, 0) the nonlinear term u x curl u is a
    gradient and the projection removes it, so the exact solution decays as exp(-nu t).
    The integrating-factor RK4 reproduces that to rounding; the explicit RK4 step
    carries its truncation error (exp(-x) minus its 4th-order Taylor polynomial)."""
    import numpy as np

    n, nu, dt, steps = 16, 0.1, 0.1, 4  # nu k^2 dt <= 1.92 on the grid: explicit RK4 stable
    y = np.arange(n) * 2 * np.pi / n
    u = np.zeros((3, n, n, n))
    u[0] = np.sin(y)[None, :, None]
    uh = np.fft.rfftn(u, axes=(1, 2, 3))
    step_if = R.rk4_if_wrapper(dt, R.rhs_wrapper(n, 0.0), nu, n)
    step_ex = R.rk4_wrapper(dt, R.rhs_wrapper(n, nu), None, 0.0, "none")
    a, ah, b, bh = u, uh, u, uh
    for _ in range(steps):
        a, ah, _ = step_if(a, ah)
        b, bh, _ = step_ex(b, bh)
    exact = np.exp(-nu * dt * steps) * u
    assert np.abs(a - exact).max() < 1e-14
    x = nu * dt
    rk4_factor = (1 - x + x**2 / 2 - x**3 / 6 + x**4 / 24) ** steps
    assert abs(np.abs(b - rk4_factor * u).max()) < 1e-14
    assert np.abs(b - exact).max() > 1e-13


def test_integrating_factor_oracle_matches_explicit_as_dt_shrinks():
    """Both forms are 4th-order accurate: on a random 3D field their one-step results
    differ by O(dt^5), so halving dt cuts the difference about 32-fold."""
    import numpy as np

    n, nu = 16, 0.05
    rng = np.random.default_rng(3)
    u = rng.standard_normal((3, n, n, n))
    uh = np.fft.rfftn(u, axes=(1, 2, 3))
    uh[:, :, :, 6:] = 0
    uh[:, 6:-5] = 0
    uh[:, :, 6:-5] = 0
    u = np.fft.irfftn(uh, axes=(1, 2, 3))
    diffs = []
    for dt in (0.02, 0.01):
        _, a, _ = R.rk4_if_wrapper(dt, R.rhs_wrapper(n, 0.0), nu, n)(u, uh)
        _, b, _ = R.rk4_wrapper(dt, R.rhs_wrapper(n, nu), None, 0.0, "none")(u, uh)
        diffs.append(np.abs(a - b).max())
    assert 16 < diffs[0] / diffs[1] < 64


def test_particle_rk4_oracle_is_fourth_order_on_a_frozen_cellular_flow():
    """Extension oracle term: RK4 advection through the exact spectral interpolant of a
    steady 2D cellular flow u = (sin x cos y, -cos x sin y): the error after a fixed
    time falls ~16x when dt halves (Euler: ~2x); reference solution by RK4 at dt/16."""
    import numpy as np

    c = 16
    g = np.arange(c) * 2 * np.pi / c
    x, y = np.meshgrid(g, g, indexing="ij")
    u = np.stack([np.sin(x) * np.cos(y), -np.cos(x) * np.sin(y)])
    rng = np.random.default_rng(4)
    r0 = rng.uniform(0, 2 * np.pi, (50, 2))

    def interp(r):
        return R.interpolate_dft(u, r)

    def run(dt, steps, rk4=True):
        r = r0.copy()
        for _ in range(steps):
            if rk4:
                _, r = R.advect_rk4(interp, r, dt)
            else:
                r = R.shift_fn(r, dt * interp(r))
        return r

    t_end = 0.8
    ref = run(t_end / 128, 128)

    def err(r):
        d = np.mod(r - ref + np.pi, 2 * np.pi) - np.pi
        return np.abs(d).max()

    e1, e2 = err(run(t_end / 8, 8)), err(run(t_end / 16, 16))
    assert 12 < e1 / e2 < 20
    f1, f2 = err(run(t_end / 8, 8, False)), err(run(t_end / 16, 16, False))
    assert 1.6 < f1 / f2 < 2.5
    assert e2 < 1e-2 * f2
