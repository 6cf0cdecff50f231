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
