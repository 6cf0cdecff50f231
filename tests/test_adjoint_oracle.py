"""The FP64 adjoint oracle (oracle/adjoint_ref.py) against central finite differences
of the FP64 forward oracle: RHS vector-Jacobian products (with drag and the
constant-power band force), the coarse-grid MSE loss gradient (filtered and
unfiltered), and a 3-step trajectory gradient, in 2D and 3D."""

import numpy as np
import pytest

from oracle import adjoint_ref as A
from oracle import numpy_ref as R

N = 16


def _setup(dim, seed):
    rng = np.random.default_rng(seed)
    axes = (1, 2, 3) if dim == 3 else (1, 2)
    u = rng.standard_normal((3,) + (N,) * dim)
    if dim == 2:
        u[2] = 0.0
    uh = 0.05 * np.fft.rfftn(u, axes=axes)
    _, kkk2, _, _ = R.wavenumbers(N, dim)
    mask = ((kkk2 > 0) & (kkk2 <= 4)).astype(float)

    def crand():
        z = rng.standard_normal(uh.shape) + 1j * rng.standard_normal(uh.shape)
        if dim == 2:
            z[2] = 0.0
        return z

    return rng, axes, uh, mask, crand


@pytest.mark.parametrize("dim", [3, 2])
@pytest.mark.parametrize("forced", [False, True])
def test_rhs_vjp_matches_finite_differences(dim, forced):
    rng, axes, uh, mask, crand = _setup(dim, 1)
    cp = (0.1, mask) if forced else None
    rhs = R.rhs_wrapper(N, 0.01, axes, drag=0.05, const_power=cp)
    vjp = A.rhs_vjp_wrapper(N, 0.01, axes, drag=0.05, const_power=cp)
    g, d, h = crand(), crand(), 1e-5
    fd = np.sum((np.conj(g) * (rhs(None, uh + h * d, 1) - rhs(None, uh - h * d, 1))).real) / (2 * h)
    an = np.sum((np.conj(vjp(uh, g)) * d).real)
    assert abs(fd - an) < 1e-8 * abs(an)


@pytest.mark.parametrize("dim", [3, 2])
@pytest.mark.parametrize("c", [8, 16])
def test_coarse_mse_grad_matches_finite_differences(dim, c):
    rng, axes, uh, mask, crand = _setup(dim, 2)
    tgt = rng.standard_normal((dim,) + (c,) * dim)
    d, h = crand(), 1e-5
    fd = (A.coarse_mse(uh + h * d, tgt, c, axes) - A.coarse_mse(uh - h * d, tgt, c, axes)) / (2 * h)
    an = np.sum((np.conj(A.coarse_mse_grad(uh, tgt, c, axes)) * d).real)
    assert abs(fd - an) < 1e-7 * abs(an)


@pytest.mark.parametrize("dim", [3, 2])
def test_trajectory_gradient_matches_finite_differences(dim):
    rng, axes, uh, mask, crand = _setup(dim, 3)
    rhs = R.rhs_wrapper(N, 0.01, axes, const_power=(0.1, mask))
    vjp = A.rhs_vjp_wrapper(N, 0.01, axes, const_power=(0.1, mask))
    tgt = 0.01 * rng.standard_normal((dim,) + (8,) * dim)
    _, G = A.trajectory_loss_and_grad(uh, 3, 0.01, rhs, vjp, tgt, 8, axes)
    d, h = crand(), 1e-5
    lp, _ = A.trajectory_loss_and_grad(uh + h * d, 3, 0.01, rhs, vjp, tgt, 8, axes)
    lm, _ = A.trajectory_loss_and_grad(uh - h * d, 3, 0.01, rhs, vjp, tgt, 8, axes)
    an = np.sum((np.conj(G) * d).real)
    assert abs((lp - lm) / (2 * h) - an) < 1e-6 * abs(an)


def test_fp64_torch_restatement_equals_numpy_oracle():
    """tests/_fp64_torch.py (the 128^3 finite-difference reference) is the same math."""
    torch = pytest.importorskip("torch")
    from _fp64_torch import Fp64Model

    rng, axes, uh, mask, crand = _setup(3, 4)
    rhs = R.rhs_wrapper(N, 5e-3, axes, drag=0.02, const_power=(0.1, mask))
    vjp = A.rhs_vjp_wrapper(N, 5e-3, axes, drag=0.02, const_power=(0.1, mask))
    M = Fp64Model(N, 5e-3, 2e-3, kf=2, eps_inj=0.1, drag=0.02, device="cpu")
    t, g = torch.from_numpy(uh), crand()
    tgt = rng.standard_normal((3, 8, 8, 8))

    def rel(a, b):
        return float(np.abs(a.numpy() - b).max() / np.abs(b).max())

    assert rel(M.rhs(t), rhs(None, uh, 1)) < 1e-13
    assert rel(M.vjp(t, torch.from_numpy(g)), vjp(uh, g)) < 1e-13
    assert rel(M.step_vjp(t, torch.from_numpy(g)), A.rk4_step_vjp(uh, g, 2e-3, rhs, vjp)) < 1e-13
    l1, g1 = M.loss_and_grad(t, 2, torch.from_numpy(tgt))
    l2, g2 = A.trajectory_loss_and_grad(uh, 2, 2e-3, rhs, vjp, tgt, 8)
    assert abs(l1 - l2) < 1e-13 * l2 and rel(g1, g2) < 1e-12


@pytest.mark.parametrize("dim", [3, 2])
def test_interp_vjp_matches_finite_differences(dim):
    """The FP64 adjoint of the particle interpolation (coarsening to c, then the exact
    spectral interpolation at fixed positions) against central differences of the
    forward oracle (interpolate_from_uhat_dft) along random directions."""
    rng, axes, uh, mask, crand = _setup(dim, 21)
    c, npart = 8, 40
    r = rng.uniform(0, 2 * np.pi, (npart, dim))
    lam = rng.standard_normal((npart, dim))

    def loss(u_hat):
        return float(np.sum(lam * R.interpolate_from_uhat_dft(u_hat, N, c, r, dim)))

    g = A.interp_vjp(lam, r, N, c, axes)
    assert g.shape == uh.shape
    h = 1e-4
    for _ in range(4):
        d = crand()
        fd = (loss(uh + h * d) - loss(uh - h * d)) / (2 * h)
        ad = float(np.real(np.sum(np.conj(g) * d)))
        assert abs(ad - fd) <= 1e-8 * max(1.0, abs(fd)), (ad, fd)


@pytest.mark.parametrize("dim", [3, 2])
def test_ekin_tot_vjp_matches_finite_differences(dim):
    """The FP64 adjoint of the ekin_tot rescaling (spectral_solver.py:82-112) against
    central differences of its Parseval form, and the whole forced RK4 step
    (rk4_step_vjp after ekin_tot_vjp) against the reference restatement's step
    (rk4_wrapper with forcing_type 'ekin_tot'), along spectra of real fields."""
    rng, axes, uh, mask, crand = _setup(dim, 31)
    e0 = 0.8 * A.ekin_tot_forward(uh, mask, 0.0, N, dim)[2] + 0.5 * A.ekin_tot_forward(uh, mask, 0.0, N, dim)[3]
    lam = crand()
    g = A.ekin_tot_vjp(uh, lam, mask, e0, N, dim)

    def real_dir(seed):
        x = np.random.default_rng(seed).standard_normal((3,) + (N,) * dim)
        if dim == 2:
            x[2] = 0.0
        return np.fft.rfftn(x, axes=axes) * np.abs(uh).max() / N**dim

    h = 1e-4
    for k in range(3):
        d = real_dir(k)
        lp = float(np.real(np.sum(np.conj(lam) * A.ekin_tot_forward(uh + h * d, mask, e0, N, dim)[0])))
        lm = float(np.real(np.sum(np.conj(lam) * A.ekin_tot_forward(uh - h * d, mask, e0, N, dim)[0])))
        fd = (lp - lm) / (2 * h)
        ad = float(np.real(np.sum(np.conj(g) * d)))
        assert abs(ad - fd) <= 1e-7 * max(1.0, abs(fd)), (ad, fd)
    # the forced step: the reference restatement's rk4_wrapper(..., "ekin_tot")
    nu, dt = 0.01, 0.01
    rhs = R.rhs_wrapper(N, nu, axes)
    vjp = A.rhs_vjp_wrapper(N, nu, axes)
    step = R.rk4_wrapper(dt, rhs, mask, e0, "ekin_tot", axes)
    def phys(x):  # the step's first stage reads the caller's u = irfftn(u_hat)
        x = np.fft.irfftn(x, axes=axes)
        return x[..., None] if dim == 2 else x

    u_rk = A.rk4_step(uh, dt, rhs)
    gs = A.rk4_step_vjp(uh, A.ekin_tot_vjp(u_rk, lam, mask, e0, N, dim), dt, rhs, vjp)
    for k in range(2):
        d = real_dir(10 + k)
        up, um = step(phys(uh + h * d), uh + h * d)[1], step(phys(uh - h * d), uh - h * d)[1]
        fd = float(np.real(np.sum(np.conj(lam) * (up - um)))) / (2 * h)
        ad = float(np.real(np.sum(np.conj(gs) * d)))
        assert abs(ad - fd) <= 1e-6 * max(1.0, abs(fd)), (ad, fd)
