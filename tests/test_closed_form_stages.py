"""The closed-form RK4 stages that the step forms 1 and 2 apply to modes outside the band.

A mode whose right-hand side is exactly -(nu k^2 + drag) u (no nonlinear or forcing
term) goes through the reference's RK4 stage sequence (oracle rk4_wrapper, following
spectral_solver.py:74-80) as polynomials in z = (nu k^2 + drag) dt times the step's
initial value u0. The kernels evaluate these polynomials (lin_stage_factor in
csrc/dns_kernels.cuh); this test checks the same polynomials against the oracle's stage
inputs, in FP64, on the CPU.
"""

import numpy as np

from oracle import numpy_ref as R


def _stage_factors(z):
    """Stage inputs of rk 1, 2, 3 and the new state, over u0."""
    return (1 - z / 2,
            1 - z / 2 + z * z / 4,
            1 - z + z * z / 2 - z ** 3 / 4,
            1 - z + z * z / 2 - z ** 3 / 6 + z ** 4 / 24)


def test_linear_decay_stages_are_the_closed_form_polynomials():
    rng = np.random.default_rng(3)
    lam = np.array([0.0, 1e-3, 0.7, 5.0, 37.0, 410.0])  # nu k^2 + drag for six modes
    dt = 2e-3
    u0 = rng.standard_normal(lam.size) + 1j * rng.standard_normal(lam.size)
    seen = {}

    def rhs(u, u_hat, rk):
        seen[rk] = u_hat.copy()
        return -lam * u_hat

    step = R.rk4_wrapper(dt, rhs, None, 0.0, "none", fft_axes=(0,))
    _, u_new, _ = step(None, u0.copy())  # the stage inputs are recorded by rhs
    z = lam * dt
    f1, f2, f3, f4 = _stage_factors(z)
    np.testing.assert_allclose(seen[0], u0, rtol=0, atol=0)
    np.testing.assert_allclose(seen[1], f1 * u0, rtol=1e-14, atol=1e-15)
    np.testing.assert_allclose(seen[2], f2 * u0, rtol=1e-14, atol=1e-15)
    np.testing.assert_allclose(seen[3], f3 * u0, rtol=1e-14, atol=1e-15)
    np.testing.assert_allclose(u_new, f4 * u0, rtol=1e-14, atol=1e-15)


def test_closed_form_matches_the_oracle_step_on_a_single_mode_outside_the_band():
    """One divergence-free Fourier mode (k = (7, -6, 5) at 16^3, outside the dealiased
    band): u x curl u of a single mode is parallel to k at +-2k, which the Leray
    projection removes, so the oracle step is the mode's linear decay, the closed form."""
    n, nu, dt = 16, 0.05, 1e-2
    _, kkk2, _, _ = R.wavenumbers(n, 3)
    kx, ky, kz = 7, -6, 5
    kvec = np.array([kx, ky, kz], float)
    a = np.array([1.0, 0.5, -0.25])
    a -= kvec * (a @ kvec) / (kvec @ kvec)  # divergence free
    uh = np.zeros((3, n, n, n // 2 + 1), complex)
    uh[:, kx % n, ky % n, kz] = (a + 0.3j * a[::-1] - 0.3j * kvec * (a[::-1] @ kvec) / (kvec @ kvec)) * n ** 3
    u = np.fft.irfftn(uh, s=(n, n, n), axes=(1, 2, 3))
    step = R.rk4_wrapper(dt, R.rhs_wrapper(n, nu), None, 0.0, "none")
    _, uh1, _ = step(u, uh)
    _, _, _, f4 = _stage_factors(nu * kkk2 * dt)
    assert np.abs(uh1 - f4 * uh).max() <= 1e-12 * np.abs(uh).max()
