"""Hand-written adjoint on the GPU vs the FP64 adjoint oracle (oracle/adjoint_ref.py,
itself pinned by finite differences) and vs central finite differences of the GPU
forward (the 128^3 differentiation workload: 20 RK4 steps, 16 seeded directions).

FP32 transforms put the vector-Jacobian products within ~1e-5 of the FP64 values
(relative to their largest entry); the tolerances below are written per check.
"""

import numpy as np
import pytest

from oracle import adjoint_ref as A
from oracle import numpy_ref as R

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _c64(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.complex64)).cuda()


def _rel(a, b):
    a = a.cpu().numpy() if hasattr(a, "cpu") else a
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _state(dim, n, seed, kp=3.0):
    if dim == 3:
        u = R.init_u_hit(n, seed, "k4exp", kp)
        u *= np.sqrt(0.5 / R.kinetic_energy(u))
        return np.fft.rfftn(u, axes=(1, 2, 3))
    u = R.init_u_random2d(n, seed)
    return np.fft.rfftn(u[..., 0] if u.ndim == 4 else u, axes=(1, 2))


def _crand(shape, seed, dim, scale=1.0):
    rng = np.random.default_rng(seed)
    z = scale * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
    if dim == 2:
        z[2] = 0.0
    return z


def _oracle_fns(dim, n, nu, drag, forced):
    axes = (1, 2, 3) if dim == 3 else (1, 2)
    cp = None
    if forced:
        _, kkk2, _, _ = R.wavenumbers(n, dim)
        cp = (0.1, ((kkk2 > 0) & (kkk2 <= 4)).astype(float))
    return (axes, R.rhs_wrapper(n, nu, axes, drag=drag, const_power=cp),
            A.rhs_vjp_wrapper(n, nu, axes, drag=drag, const_power=cp))


CASES = [(3, 32, 5e-3, 0.0, True), (3, 32, 1e-2, 0.05, False), (2, 64, 1e-3, 0.1, False), (2, 64, 2e-3, 0.0, True)]


@pytest.mark.parametrize("dim,n,nu,drag,forced", CASES)
def test_rhs_vjp_matches_oracle(dim, n, nu, drag, forced):
    from l3es import adjoint as AD

    uh = _state(dim, n, 3)
    axes, rhs, vjp = _oracle_fns(dim, n, nu, drag, forced)
    g = _crand(uh.shape, 4, dim, np.abs(uh).max())
    plan = AD.make_plan(n, nu, dim, 1e-3, "const_power" if forced else "none", kf=2, eps_inj=0.1, drag=drag)
    got = AD.rhs_vjp(plan, _c64(uh), _c64(g))
    assert _rel(got, vjp(uh, g)) < 3e-5


@pytest.mark.parametrize("dim,n,c", [(3, 64, 16), (3, 32, 32), (2, 64, 32), (2, 32, 8)])
def test_coarse_mse_matches_oracle(dim, n, c):
    from l3es import adjoint as AD

    axes = (1, 2, 3) if dim == 3 else (1, 2)
    uh = _state(dim, n, 5)
    tgt = np.random.default_rng(6).standard_normal((dim,) + (c,) * dim).astype(np.float32)
    ip = AD.coarse_plan(dim, n, c)
    loss = torch.zeros(1, dtype=torch.float64, device="cuda")
    grad = torch.empty(uh.shape, dtype=torch.complex64, device="cuda")
    ip.coarse_mse(_c64(uh), torch.from_numpy(tgt).cuda(), loss, grad)
    assert abs(float(loss) - A.coarse_mse(uh, tgt, c, axes)) < 1e-6 * A.coarse_mse(uh, tgt, c, axes)
    assert _rel(grad, A.coarse_mse_grad(uh, tgt, c, axes)) < 1e-5


@pytest.mark.parametrize("dim,n,nu,drag,forced", CASES)
def test_adjoint_step_matches_oracle(dim, n, nu, drag, forced):
    from l3es import adjoint as AD

    dt = 2e-3
    uh = _state(dim, n, 7)
    axes, rhs, vjp = _oracle_fns(dim, n, nu, drag, forced)
    lam = _crand(uh.shape, 8, dim)
    plan = AD.make_plan(n, nu, dim, dt, "const_power" if forced else "none", kf=2, eps_inj=0.1, drag=drag)
    u0 = _c64(uh)
    keep = u0.clone()
    got = _c64(lam)
    plan.adjoint_step(u0, got)
    assert torch.equal(u0, keep)  # the checkpoint is not modified
    assert _rel(got, A.rk4_step_vjp(uh, lam, dt, rhs, vjp)) < 3e-5


def test_trajectory_gradient_matches_oracle():
    from l3es import adjoint as AD

    dim, n, c, nu, dt, steps = 3, 32, 16, 5e-3, 2e-3, 5
    uh = _state(dim, n, 9)
    axes, rhs, vjp = _oracle_fns(dim, n, nu, 0.0, True)
    tgt = 0.5 * np.random.default_rng(10).standard_normal((3, c, c, c)).astype(np.float32)
    loss_ref, g_ref = A.trajectory_loss_and_grad(uh, steps, dt, rhs, vjp, tgt.astype(np.float64), c, axes)
    plan = AD.make_plan(n, nu, dim, dt, "const_power", kf=2, eps_inj=0.1)
    loss, g = AD.loss_and_grad(_c64(uh), plan, steps, torch.from_numpy(tgt).cuda(), AD.coarse_plan(3, n, c))
    assert abs(float(loss) - loss_ref) < 1e-5 * loss_ref
    assert _rel(g, g_ref) < 1e-4


def test_autograd_matches_direct_sweep():
    from l3es import adjoint as AD

    n, c, steps = 32, 16, 3
    uh = _c64(_state(3, n, 11))
    tgt = torch.from_numpy(np.random.default_rng(12).standard_normal((3, c, c, c)).astype(np.float32)).cuda()
    plan = AD.make_plan(n, 5e-3, 3, 2e-3, "const_power", kf=2, eps_inj=0.1)
    ip = AD.coarse_plan(3, n, c)
    x = uh.clone().requires_grad_(True)
    loss = AD.coarse_mse(AD.integrate(x, plan, steps), tgt, ip)
    loss.backward()
    l2, g2 = AD.loss_and_grad(uh, plan, steps, tgt, ip)
    assert float(loss.detach()) == float(l2)
    assert torch.equal(x.grad, g2)


@pytest.mark.parametrize("dim,n,kf", [(3, 32, 2), (2, 64, 3)])
def test_ekin_tot_adjoint_step_matches_oracle(dim, n, kf):
    """The adjoint of the step with ekin_tot forcing (the RK4 reverse sweep after the
    adjoint of the kinetic-energy rescaling, spectral_solver.py:82-112) vs the FP64
    oracle (ekin_tot_vjp, then rk4_step_vjp), with E0 below the current energy so the
    rescaling is active."""
    from l3es import _native

    nu, dt = 5e-3, 2e-3
    uh = _state(dim, n, 17)
    axes, rhs, vjp = _oracle_fns(dim, n, nu, 0.0, False)
    _, kkk2, _, _ = R.wavenumbers(n, dim)
    mask = ((kkk2 > 0) & (kkk2 <= kf * kf)).astype(float)
    e_all = A.ekin_tot_forward(uh, mask, 0.0, n, dim)
    e0 = 0.95 * (e_all[2] + e_all[3])
    u_rk = A.rk4_step(uh, dt, rhs)
    lam = _crand(uh.shape, 18, dim)
    ref = A.rk4_step_vjp(uh, A.ekin_tot_vjp(u_rk, lam, mask, e0, n, dim), dt, rhs, vjp)
    plan = _native.Plan(dim=dim, n=n, nu=nu, dt=dt, forcing="ekin_tot", kf=kf, e_kin_init=e0)
    plan.adjoint_prepare()
    u0 = _c64(uh)
    got = _c64(lam)
    plan.adjoint_step(u0, got)
    assert _rel(got, ref) < 3e-5
    # the forward step agrees with the oracle's rescaled step too (same e0, same state)
    fw = _c64(uh)
    plan.step(fw, 1)
    assert _rel(fw, A.ekin_tot_forward(u_rk, mask, e0, n, dim)[0]) < 2e-5


def test_integrating_factor_plans_have_no_adjoint():
    from l3es import _native

    p = _native.Plan(dim=3, n=16, nu=1e-2, dt=1e-3, scheme="integrating_factor")
    with pytest.raises(RuntimeError, match="explicit"):
        p.adjoint_prepare()


def _workload128():
    """128^3 HIT (k_p = 3, constant power 0.1 on |k| <= 2, nu 5e-3), 20 RK4 steps at
    dt 2e-3, loss = MSE of the 32^3 coarsened velocity against a seeded target
    (the coarsened HIT field of another seed)."""
    n, c = 128, 32
    uh = _state(3, n, 13)
    tgt = R.spectral_filtering(np.fft.irfftn(_state(3, n, 14), axes=(1, 2, 3)), c)
    return n, c, 20, 2e-3, uh, np.ascontiguousarray(tgt, dtype=np.float32)


def test_differentiation_workload_gradient_vs_fp64():
    """The FP32 adjoint gradient against the FP64 gradient of the same loss
    (tests/_fp64_torch.py, the oracle's math in FP64 on the GPU)."""
    from _fp64_torch import Fp64Model

    from l3es import adjoint as AD

    n, c, steps, dt, uh, tgt = _workload128()
    plan = AD.make_plan(n, 5e-3, 3, dt, "const_power", kf=2, eps_inj=0.1)
    loss, g = AD.loss_and_grad(_c64(uh), plan, steps, torch.from_numpy(tgt).cuda(), AD.coarse_plan(3, n, c))
    M = Fp64Model(n, 5e-3, dt, kf=2, eps_inj=0.1)
    loss64, g64 = M.loss_and_grad(torch.from_numpy(uh).cuda(), steps, torch.from_numpy(tgt.astype(np.float64)).cuda())
    assert abs(float(loss) - loss64) < 1e-5 * loss64
    assert _rel(g, g64.cpu().numpy()) < 1e-4


def test_differentiation_workload_finite_differences():
    """Directional derivatives of the FP32 adjoint gradient against FP64 central
    differences (step 1e-3) on 16 seeded directions: random HIT fields (k_p = 3
    spectrum) scaled to the norm of u_hat0. Agreement to 1e-4 of the largest
    directional derivative."""
    from _fp64_torch import Fp64Model

    from l3es import adjoint as AD

    n, c, steps, dt, uh, tgt = _workload128()
    plan = AD.make_plan(n, 5e-3, 3, dt, "const_power", kf=2, eps_inj=0.1)
    _, g = AD.loss_and_grad(_c64(uh), plan, steps, torch.from_numpy(tgt).cuda(), AD.coarse_plan(3, n, c))
    g = g.to(torch.complex128)
    M = Fp64Model(n, 5e-3, dt, kf=2, eps_inj=0.1)
    u64 = torch.from_numpy(uh).cuda()
    t64 = torch.from_numpy(tgt.astype(np.float64)).cuda()
    norm = float(torch.linalg.vector_norm(u64))
    h = 1e-3
    ad, fd = [], []
    for k in range(16):
        d = torch.from_numpy(_state(3, n, 100 + k)).cuda()
        d *= norm / float(torch.linalg.vector_norm(d))
        fd.append((M.loss_after(u64 + h * d, steps, t64) - M.loss_after(u64 - h * d, steps, t64)) / (2 * h))
        ad.append(float((torch.conj(g) * d).real.sum()))
    ad, fd = np.array(ad), np.array(fd)
    assert np.abs(ad - fd).max() < 1e-4 * np.abs(ad).max()


def test_batched_adjoint_matches_single_plans():
    """A batch-2 plan (per-trajectory viscosity, constant power) takes each
    trajectory's adjoint step as its own single plan does."""
    from l3es import adjoint as AD

    n, dt, nus = 32, 2e-3, [4e-3, 9e-3]
    states = [_state(3, n, 20 + b) for b in range(2)]
    lams = [_crand(states[0].shape, 30 + b, 3) for b in range(2)]
    singles = []
    for b in range(2):
        p = AD.make_plan(n, nus[b], 3, dt, "const_power", kf=2, eps_inj=0.1)
        lam = _c64(lams[b])
        p.adjoint_step(_c64(states[b]), lam)
        singles.append(lam.cpu().numpy())
    pb = AD.make_plan(n, 0.0, 3, dt, "const_power", kf=2, eps_inj=0.1, batch=2)
    pb.set_nu(nus)
    lam_b = torch.stack([_c64(l) for l in lams]).contiguous()
    pb.adjoint_step(torch.stack([_c64(s) for s in states]).contiguous(), lam_b)
    got = lam_b.cpu().numpy()
    for b in range(2):
        assert np.abs(got[b] - singles[b]).max() <= 1e-6 * np.abs(singles[b]).max()


@pytest.mark.parametrize("dim,n,c,np_", [(3, 32, 16, 600), (2, 64, 32, 900)])
def test_interp_vjp_matches_oracle_and_finite_differences(dim, n, c, np_):
    """Adjoint of the particle interpolation (coarsening + NUFFT / exact DFT at fixed
    positions) vs the FP64 oracle VJP of interpolate_dft, and its directional
    derivatives vs central differences of the FP64 forward oracle (1e-4)."""
    from l3es import adjoint as AD

    axes = (1, 2, 3) if dim == 3 else (1, 2)
    uh = _state(dim, n, 3)
    if dim == 2:
        uh = uh.reshape(3, n, n // 2 + 1)
    rng = np.random.default_rng(9)
    r = rng.uniform(0, 2 * np.pi, (np_, dim))
    lam = rng.standard_normal((np_, dim))
    ref = A.interp_vjp(lam, r, n, c, axes)
    ip = AD.particle_plan(dim, n, c, np_)
    rt = torch.from_numpy(r).cuda()
    lt = torch.from_numpy(lam).cuda()

    from oracle import nufft_ref as NU

    def loss64(u_hat, backend):
        # FP64 forward of the same backend: the exact DFT (integrator.py:62-91) or the
        # restated type-2 NUFFT (ES kernel w = 6, sigma = 2), after spectral_filtering
        if backend == "dft":
            return float(np.sum(lam * R.interpolate_from_uhat_dft(u_hat, n, c, r, dim)))
        u = np.fft.irfftn(u_hat, s=(n,) * dim, axes=axes)[:dim]
        return float(np.sum(lam * NU.interpolate_nufft(R.spectral_filtering(u, c), r, w=6)))

    for backend, tol in (("dft", 2e-5), ("nufft", 1e-4)):
        g = torch.empty(uh.shape, dtype=torch.complex64, device="cuda")
        ip.interp_vjp(rt, lt, g, backend=backend)
        torch.cuda.synchronize()
        assert _rel(g, ref) < tol, backend
        gn = g.cpu().numpy().astype(np.complex128)
        h = 1e-3
        for k in range(3):
            x = np.random.default_rng(100 + k).standard_normal((3,) + (n,) * dim)
            if dim == 2:
                x[2] = 0.0
            d = np.fft.rfftn(x, axes=axes) * (np.abs(uh).max() / n**dim)
            fd = (loss64(uh + h * d, backend) - loss64(uh - h * d, backend)) / (2 * h)
            ad = float(np.real(np.sum(np.conj(gn) * d)))
            assert abs(ad - fd) <= 1e-4 * max(abs(fd), 1e-12), (backend, ad, fd)
    # autograd through the interpolation gives the same gradient
    u = _c64(uh).requires_grad_(True)
    ur = AD.interp(u, rt, ip, backend="nufft")
    (ur * lt).sum().backward()
    assert _rel(u.grad, ref) < 1e-4


def test_particle_loss_gradient_through_the_step():
    """A loss on particle velocities after 3 RK4 steps differentiates back to the
    initial half spectrum (adjoint steps + interpolation adjoint, autograd), vs central
    differences of the FP64 oracle trajectory (1e-4)."""
    from l3es import adjoint as AD

    n, c, np_, nu, dt, steps = 32, 16, 500, 0.01, 5e-3, 3
    uh = _state(3, n, 4)
    rng = np.random.default_rng(10)
    r = rng.uniform(0, 2 * np.pi, (np_, 3))
    lam = rng.standard_normal((np_, 3))
    plan = AD.make_plan(n, nu, 3, dt)
    ip = AD.particle_plan(3, n, c, np_)
    u = _c64(uh).requires_grad_(True)
    ur = AD.interp(AD.integrate(u, plan, steps), torch.from_numpy(r).cuda(), ip, backend="dft")
    (ur * torch.from_numpy(lam).cuda()).sum().backward()
    g = u.grad.cpu().numpy().astype(np.complex128)
    rhs = R.rhs_wrapper(n, nu)

    def loss64(u_hat):
        for _ in range(steps):
            u_hat = A.rk4_step(u_hat, dt, rhs)
        return float(np.sum(lam * R.interpolate_from_uhat_dft(u_hat, n, c, r)))

    h = 1e-3
    for k in range(3):
        x = np.random.default_rng(200 + k).standard_normal((3, n, n, n))
        d = np.fft.rfftn(x, axes=(1, 2, 3)) * (np.abs(uh).max() / n**3)
        fd = (loss64(uh + h * d) - loss64(uh - h * d)) / (2 * h)
        ad = float(np.real(np.sum(np.conj(g) * d)))
        assert abs(ad - fd) <= 1e-4 * max(abs(fd), 1e-12), (ad, fd)
