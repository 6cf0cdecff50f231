"""CUDA DNS step vs the FP64 oracle and the reference's golden vectors (GPU).

Tolerance: the CUDA path computes in FP32 (FP64 reductions); fields are compared by
max |a - b| / max |b|, which stays below 2e-5 for the few-step cases here (FP32
unit roundoff 6e-8 times the FFT depth and step count).
"""

import numpy as np
import pytest

from oracle import numpy_ref as R

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

RTOL = 2e-5


def _rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _plan(**kw):
    from l3es import _native

    return _native.Plan(**kw)


def _c64(a):
    return torch.from_numpy(np.ascontiguousarray(a).astype(np.complex64)).cuda()


def _f32(a):
    return torch.from_numpy(np.ascontiguousarray(a).astype(np.float32)).cuda()


@pytest.mark.parametrize("dim,n", [(3, 16), (3, 32), (3, 64), (3, 128), (2, 16), (2, 64), (2, 256), (2, 512)])
def test_rfftn_irfftn_match_numpy(dim, n):
    rng = np.random.default_rng(n + dim)
    shape = (3, n, n, n) if dim == 3 else (3, n, n, 1)
    axes = (1, 2, 3) if dim == 3 else (1, 2)
    u = rng.standard_normal(shape)
    p = _plan(dim=dim, n=n, nu=0.01, dt=0.01)
    uh = torch.empty(p.spec_shape, dtype=torch.complex64, device="cuda")
    p.rfftn(_f32(u), uh)
    ref = np.fft.rfftn(u, axes=axes).reshape(p.spec_shape)
    assert _rel(uh.cpu().numpy(), ref) < RTOL
    # irfftn of a non-Hermitian-consistent spectrum: numpy semantics (imag of DC/Nyquist dropped)
    spec = ref + 0.1 * (rng.standard_normal(ref.shape) + 1j * rng.standard_normal(ref.shape)) * np.abs(ref).max()
    out = torch.empty(p.phys_shape, dtype=torch.float32, device="cuda")
    p.irfftn(_c64(spec), out)
    ref_u = np.fft.irfftn(spec.reshape((3, n, n, n // 2 + 1) if dim == 3 else (3, n, n // 2 + 1)), axes=axes)
    assert _rel(out.cpu().numpy().reshape(ref_u.shape), ref_u) < RTOL


def test_rhs_matches_reference_golden(gold):
    g = gold("rand3d_n16")
    p = _plan(dim=3, n=16, nu=float(g["nu"]), dt=float(g["dt"]))
    du = torch.empty(p.spec_shape, dtype=torch.complex64, device="cuda")
    p.rhs(_c64(g["u_hat0"]), du)
    assert _rel(du.cpu().numpy(), g["rhs_rk0"]) < RTOL


@pytest.mark.parametrize("case", ["tgv3d_n16", "rand3d_n16"])
def test_step3d_matches_reference_golden(gold, case):
    g = gold(case)
    n = int(g["N"])
    p = _plan(dim=3, n=n, nu=float(g["nu"]), dt=float(g["dt"]))
    uh = _c64(g["u_hat0"])
    u = torch.empty(p.phys_shape, dtype=torch.float32, device="cuda")
    p.step(uh, int(g["steps"]), u_out=u)
    assert _rel(uh.cpu().numpy(), g["u_hat"]) < RTOL
    assert _rel(u.cpu().numpy(), g["u"]) < RTOL


def test_step2d_three_components_golden(gold):
    g = gold("rand2d_n32")
    p = _plan(dim=2, n=32, nu=float(g["nu"]), dt=float(g["dt"]))
    uh = _c64(g["u_hat0"])
    u = torch.empty(p.phys_shape, dtype=torch.float32, device="cuda")
    p.step(uh, int(g["steps"]), u_out=u)
    assert _rel(uh.cpu().numpy(), g["u_hat"]) < RTOL
    assert _rel(u.cpu().numpy(), g["u"]) < RTOL


def test_tgv2d_golden(gold):
    g = gold("tgv2d_n32")
    n = int(g["N"])
    u0, uh0, *_ = R.set_up_solver(n, float(g["nu"]), 2, "TGV2D", float(g["dt"]), 42, 8,
                                  None, None, "none", warmup=False)
    p = _plan(dim=2, n=n, nu=float(g["nu"]), dt=float(g["dt"]))
    uh = _c64(uh0)
    p.step(uh, 1 + int(g["steps_after_setup"]))  # set_up_solver's warm-up step + 3
    assert _rel(uh.cpu().numpy(), g["u_hat"]) < RTOL


def test_hit_ekin_forcing_golden(gold):
    g = gold("hit3d_n16_ekin")
    n, dt = int(g["N"]), float(g["dt"])
    _, uh0, _, _, _, _, e0, _ = R.set_up_solver(n, float(g["nu"]), 3, "HIT", dt, int(g["seed"]), 8,
                                                int(g["kf"]), float(g["e_kin_target"]), "ekin_tot",
                                                warmup=False)
    assert abs(e0 - float(g["e_kin_init"])) < 1e-12
    p = _plan(dim=3, n=n, nu=float(g["nu"]), dt=dt, forcing="ekin_tot", kf=int(g["kf"]),
              e_kin_init=e0)
    uh = _c64(uh0)
    steps = 1 + int(g["steps_after_setup"])
    einj = torch.zeros(steps, dtype=torch.float64, device="cuda")
    p.step(uh, steps, e_inj=einj)
    assert _rel(uh.cpu().numpy(), g["u_hat"]) < RTOL
    np.testing.assert_allclose(einj.cpu().numpy(), g["e_inj"], rtol=1e-3, atol=1e-6)
    ke = torch.zeros(1, dtype=torch.float64, device="cuda")
    p.kinetic_energy(uh, ke)
    assert abs(float(ke) - e0) < 1e-6 * e0  # ekin_tot pins KE to E0


def test_tgv64_known_answer():
    """from_spectralDNS/main_numpy.py:136: KE after 10 steps = 0.124953117517."""
    n = 64
    xyz = np.mgrid[:n, :n, :n].astype(float) * 2 * np.pi / n
    u0 = R.init_u_tgv(*xyz)
    p = _plan(dim=3, n=n, nu=0.000625, dt=0.01)
    uh = torch.empty(p.spec_shape, dtype=torch.complex64, device="cuda")
    p.rfftn(_f32(u0), uh)
    u = torch.empty(p.phys_shape, dtype=torch.float32, device="cuda")
    p.step(uh, 10, u_out=u)
    ke_phys = 0.5 * float((u.double() ** 2).sum(0).mean())
    ke = torch.zeros(1, dtype=torch.float64, device="cuda")
    p.kinetic_energy(uh, ke)
    assert abs(ke_phys - 0.124953117517) < 2e-7
    assert abs(float(ke) - 0.124953117517) < 2e-7


@pytest.mark.parametrize("n", [128, 256])
def test_step3d_large_vs_oracle(n):
    """One RK4 step on a band-limited random field at production sizes."""
    rng = np.random.default_rng(7)
    u0 = R.init_u_hit(n, 3, spectrum="k4exp", kp=4.0)
    u0 *= np.sqrt(0.5 / R.kinetic_energy(u0))
    R.set_workers(None)
    try:
        uh0 = np.fft.rfftn(u0, axes=(1, 2, 3))
        step = R.rk4_wrapper(2e-3, R.rhs_wrapper(n, 5e-3), None, 0.0, "none")
        _, uh_ref, _ = step(u0, uh0)
    finally:
        R.set_workers(1)
    p = _plan(dim=3, n=n, nu=5e-3, dt=2e-3)
    uh = _c64(uh0)
    p.step(uh, 1)
    p.check()
    assert _rel(uh.cpu().numpy(), uh_ref) < RTOL
    del rng


@pytest.mark.parametrize("dim,n", [(2, 32), (2, 64), (3, 32)])
def test_rhs_outside_dealias_band_is_viscous_only(dim, n):
    """Modes outside the 2/3 cube only feel -nu k^2 u_hat (spectral_solver.py:56-59):
    with nu = 0 the right-hand side there is exactly zero, for every component."""
    rng = np.random.default_rng(n + dim)
    shape = (3, n, n, n) if dim == 3 else (3, n, n, 1)
    axes = (1, 2, 3) if dim == 3 else (1, 2)
    u = rng.standard_normal(shape)
    uh = np.fft.rfftn(u, axes=axes).reshape((3, n, n, n // 2 + 1) if dim == 3 else (3, n, n // 2 + 1))
    p = _plan(dim=dim, n=n, nu=0.0, dt=1e-3)
    du = torch.full(p.spec_shape, float("nan"), dtype=torch.complex64, device="cuda")
    p.rhs(_c64(uh), du)
    d = du.cpu().numpy()
    kd = max(k for k in range(n) if k < 2.0 / 3.0 * (n // 2 + 1))
    kx = np.fft.fftfreq(n, 1.0 / n)
    out_x = np.abs(kx) > kd
    assert not np.isnan(d).any()
    assert np.abs(d[:, out_x]).max() == 0.0
    ref = R.rhs_wrapper(n, 0.0, axes)(u, uh, 1)
    assert _rel(d, ref) < RTOL


@pytest.mark.parametrize("k", [(1, 2, 3), (1, 1, 26), (2, 30, 1), (3, -25, 28), (-5, 0, 23)])
def test_single_mode_decays_by_the_rk4_polynomial(k):
    """One transverse Fourier mode has u x curl u parallel to k (a gradient the projection
    removes), so each RK4 step multiplies it by R(-z) = 1 - z + z^2/2 - z^3/6 + z^4/24,
    z = nu |k|^2 dt. At 64^3 (kd = 21, kt = 24) the cases lie in the dealiasing cube,
    outside it along kz (kz = 23, 26, 28: still in the rows the RK update treats in full)
    and outside the rows |ky| <= kd, where the update takes the closed form; the step
    must give the same factor on every path. Outside the dealiasing cube the mode's 2k product aliases onto
    another wavenumber, so the amplitude is kept at 1e-9: that quadratic residue stays
    below FP32 rounding of the mode itself."""
    n, nu, dt, steps = 64, 5e-4, 0.4, 5
    kx, ky, kz = k
    kvec = np.array([kx, ky, kz], dtype=np.float64)
    a = np.cross(kvec, [0.3, -0.7, 0.5]) + 1j * np.cross(kvec, [0.2, 0.4, -0.1])  # a . k = 0
    a *= 1e-9 / np.abs(a).max()
    uh0 = np.zeros((3, n, n, n // 2 + 1), dtype=np.complex128)
    uh0[:, kx % n, ky % n, kz] = a * n**3
    z = nu * float(kvec @ kvec) * dt
    rz = 1 - z + z**2 / 2 - z**3 / 6 + z**4 / 24
    p = _plan(dim=3, n=n, nu=nu, dt=dt)
    g = _c64(uh0)
    p.step(g, steps)
    p.check()
    got = g.cpu().numpy()
    want = uh0 * rz**steps
    assert _rel(got, want) < 2e-6, (k, z)


def test_step3d_512_vs_fp64():
    """The largest compiled grid, 512^3: two RK4 steps with constant-power forcing
    against the FP64 torch restatement of the same step (tests/_fp64_torch.py, equal
    to the NumPy oracle to 1e-13 on small grids), and the KE reduction against FP64."""
    from _fp64_torch import Fp64Model

    n, nu, dt = 512, 2e-3, 1e-3
    u0 = R.init_u_hit(n, 5, spectrum="k4exp", kp=4.0)
    u0 *= np.sqrt(0.5 / R.kinetic_energy(u0))
    uh0 = np.fft.rfftn(u0, axes=(1, 2, 3))
    del u0
    M = Fp64Model(n, nu, dt, kf=2, eps_inj=0.1)
    ref = torch.from_numpy(uh0).cuda()
    for _ in range(2):
        ref = M.step(ref)
    p = _plan(dim=3, n=n, nu=nu, dt=dt, forcing="const_power", kf=2, eps_inj=0.1)
    uh = _c64(uh0)
    del uh0
    p.step(uh, 2)
    p.check()
    err = float((uh.to(torch.complex128) - ref).abs().max() / ref.abs().max())
    assert err < RTOL
    ke = torch.zeros(1, dtype=torch.float64, device="cuda")
    p.kinetic_energy(uh, ke)
    w = M.w
    ke64 = 0.5 * float((w * (ref.abs() ** 2).sum(0)).sum()) / float(n) ** 6
    assert abs(float(ke) - ke64) < 1e-6 * ke64


def test_step3d_256_fifty_steps_vs_fp64():
    """The headline workload's step at full size (256^3, Rogallo k^4 exp init at KE 0.5,
    constant-power forcing eps = 0.1 on |k| <= 2, nu = 5e-3, dt = 4.87e-3, every kernel
    the bench times) over 50 steps against the FP64 torch restatement: the whole field,
    the kinetic energy and the shell spectrum."""
    from _fp64_torch import Fp64Model

    n, nu, dt, steps = 256, 5e-3, 4.87e-3, 50
    u0 = R.init_u_hit(n, 0, spectrum="k4exp", kp=4.0)
    u0 *= np.sqrt(0.5 / R.kinetic_energy(u0))
    uh0 = np.fft.rfftn(u0, axes=(1, 2, 3))
    del u0
    M = Fp64Model(n, nu, dt, kf=2, eps_inj=0.1)
    ref = torch.from_numpy(uh0).cuda()
    for _ in range(steps):
        ref = M.step(ref)
    p = _plan(dim=3, n=n, nu=nu, dt=dt, forcing="const_power", kf=2, eps_inj=0.1)
    uh = _c64(uh0)
    del uh0
    p.step(uh, steps)
    p.check()
    d = uh.to(torch.complex128) - ref
    assert float(d.abs().max() / ref.abs().max()) < RTOL
    assert float(torch.linalg.vector_norm(d) / torch.linalg.vector_norm(ref)) < 1e-5
    w = M.w
    e32 = (w * (uh.to(torch.complex128).abs() ** 2).sum(0)).sum()
    e64 = (w * (ref.abs() ** 2).sum(0)).sum()
    assert abs(float(e32 / e64) - 1.0) < 1e-6
    # shell spectrum, shells 1..85 (the dealiased range)
    kx = torch.fft.fftfreq(n, 1.0 / n, dtype=torch.float64, device="cuda")
    kz = torch.arange(n // 2 + 1, dtype=torch.float64, device="cuda")
    kk = torch.sqrt(kx[:, None, None] ** 2 + kx[None, :, None] ** 2 + kz[None, None, :] ** 2)
    shell = (kk + 0.5).long().clamp(max=n)
    e_a = torch.zeros(n + 1, dtype=torch.float64, device="cuda").index_add_(
        0, shell.flatten(), (w * (uh.to(torch.complex128).abs() ** 2).sum(0)).flatten())
    e_b = torch.zeros(n + 1, dtype=torch.float64, device="cuda").index_add_(
        0, shell.flatten(), (w * (ref.abs() ** 2).sum(0)).flatten())
    assert float(((e_a - e_b).abs() / e_b)[1:86].max()) < 1e-5


@pytest.mark.parametrize("forcing", ["none", "const_power", "ekin_tot"])
def test_step_energy_equals_kinetic_energy(forcing):
    """l3es_step_energy's KE (after ekin_tot rescaling: e_high + alpha^2 e_low) equals
    l3es_kinetic_energy of the final state; batch of 2."""
    n = 32
    us = []
    for b in range(2):
        u = R.init_u_hit(n, 40 + b, spectrum="k4exp", kp=3.0)
        us.append(np.fft.rfftn(u * np.sqrt(0.5 / R.kinetic_energy(u)), axes=(1, 2, 3)))
    p = _plan(dim=3, n=n, nu=5e-3, dt=2e-3, batch=2, forcing=forcing, kf=2, eps_inj=0.1, e_kin_init=0.5)
    uh = torch.stack([_c64(x) for x in us]).contiguous()
    ke = torch.zeros(2, dtype=torch.float64, device="cuda")
    p.step(uh, 3, ke=ke)
    ref = torch.zeros(2, dtype=torch.float64, device="cuda")
    p.kinetic_energy(uh, ref)
    # ekin_tot reports e_high + alpha^2 e_low of the rescaling, the recount sees the
    # rescaled FP32 state; otherwise only the FP32 rounding of the mode energies differs
    np.testing.assert_allclose(ke.cpu().numpy(), ref.cpu().numpy(), rtol=1e-6 if forcing == "ekin_tot" else 1e-7)
    if forcing == "ekin_tot":
        np.testing.assert_allclose(ke.cpu().numpy(), 0.5, rtol=1e-6)


@pytest.mark.parametrize("n", [64, 256])
def test_batched_3d_step_equals_single_plans(n):
    """A batch of 3 trajectories in one plan (the x pass loads each trajectory's three
    components as one bulk tensor block) equals three single-trajectory plans, bit for bit."""
    us = []
    for b in range(3):
        u = R.init_u_hit(n, 11 + b, spectrum="k4exp", kp=3.0)
        us.append(np.fft.rfftn(u * np.sqrt(0.5 / R.kinetic_energy(u)), axes=(1, 2, 3)))
    pb = _plan(dim=3, n=n, nu=5e-3, dt=2e-3, batch=3, forcing="const_power", kf=2, eps_inj=0.1)
    uhb = torch.stack([_c64(x) for x in us]).contiguous()
    pb.step(uhb, 2)
    pb.check()
    for b in range(3):
        p1 = _plan(dim=3, n=n, nu=5e-3, dt=2e-3, forcing="const_power", kf=2, eps_inj=0.1)
        uh1 = _c64(us[b])
        p1.step(uh1, 2)
        p1.check()
        assert torch.equal(uh1, uhb[b])



def test_bounded_wait_gives_up_and_context_stays_usable():
    """The mbarrier wait of the bulk-copy kernels is bounded: a wait that nothing
    completes returns L3ES_ETIMEOUT, and the context still runs a step afterwards."""
    from l3es import _native

    lib = _native.load()
    assert lib.l3es_selftest_bounded_wait(None) == -5
    assert b"ran out" in lib.l3es_last_error()
    n = 64
    u0 = R.init_u_hit(n, 2, spectrum="k4exp", kp=3.0)
    p = _plan(dim=3, n=n, nu=5e-3, dt=2e-3)
    uh = _c64(np.fft.rfftn(u0, axes=(1, 2, 3)))
    p.step(uh, 1)
    p.check()
    assert torch.isfinite(torch.view_as_real(uh)).all()


def test_misaligned_spectrum_is_refused_not_faulted():
    """A spectrum that starts 8 bytes off a 16-byte boundary (a view one mode into a
    buffer) is refused with L3ES_EINVAL before any launch (the elementwise kernels read
    two modes at a time); the Python binding refuses it too."""
    import ctypes

    from l3es import _native

    n = 16
    p = _plan(dim=3, n=n, nu=5e-3, dt=2e-3)
    numel = int(np.prod(p.spec_shape))
    buf = torch.zeros(numel + 1, dtype=torch.complex64, device="cuda")
    bad = buf[1:].view(p.spec_shape)
    assert bad.data_ptr() % 16 == 8
    with pytest.raises(ValueError):
        p.step(bad, 1)
    lib = _native.load()
    assert lib.l3es_step(p._h, ctypes.c_void_p(bad.data_ptr()), None, 1, None, None) == -1
    assert b"aligned" in lib.l3es_last_error()
    ke = torch.zeros(1, dtype=torch.float64, device="cuda")
    assert lib.l3es_kinetic_energy(p._h, ctypes.c_void_p(bad.data_ptr()), ctypes.c_void_p(ke.data_ptr()), None) == -1
    good = buf[:numel].view(p.spec_shape)
    p.step(good, 1)
    p.check()


@pytest.mark.parametrize("dim,n", [(3, 32), (2, 64)])
def test_nonfinite_state_is_reported_and_cleared(dim, n):
    """Blow-up detection: a NaN written into u_hat on the host before the call spreads
    through the step; the final RK update flags it and l3es_plan_check reports
    L3ES_ENONFINITE (NonFiniteError), once. A finite state then steps cleanly. (A NaN
    in the data neither traps nor hangs the GPU: the kernels only add and multiply it.)"""
    from l3es import _native

    rng = np.random.default_rng(7)
    shape = (3, n, n, n) if dim == 3 else (3, n, n, 1)
    axes = (1, 2, 3) if dim == 3 else (1, 2)
    u = 0.1 * rng.standard_normal(shape)
    p = _plan(dim=dim, n=n, nu=5e-3, dt=1e-3)
    spec = np.fft.rfftn(u, axes=axes).reshape(p.spec_shape)
    bad = spec.copy()
    bad[(0,) * len(p.spec_shape[:-1]) + (1,)] = np.nan
    uh = _c64(bad)
    p.step(uh, 1)
    with pytest.raises(_native.NonFiniteError, match="non-finite"):
        p.check()
    p.check()  # the flag was cleared by the report
    lib = _native.load()
    uh = _c64(spec)
    p.step(uh, 2)
    assert lib.l3es_plan_check(p._h) == 0
    assert torch.isfinite(torch.view_as_real(uh)).all()


def _band_limited(dim, n, seed, kmax=6):
    rng = np.random.default_rng(seed)
    shape = (3, n, n, n) if dim == 3 else (3, n, n, 1)
    axes = (1, 2, 3) if dim == 3 else (1, 2)
    u = rng.standard_normal(shape)
    if dim == 2:
        u[2] = 0.0
    uh = np.fft.rfftn(u, axes=axes)
    k = np.fft.fftfreq(n, 1.0 / n)
    kh = np.arange(n // 2 + 1)
    if dim == 3:
        kk = np.sqrt(k[:, None, None] ** 2 + k[None, :, None] ** 2 + kh[None, None, :] ** 2)
    else:
        kk = np.sqrt(k[:, None, None] ** 2 + kh[None, :, None] ** 2)
    uh = np.where(kk <= kmax, uh, 0.0)
    u = np.fft.irfftn(uh, s=(n,) * dim, axes=axes)
    if dim == 2:
        u = u.reshape(3, n, n, 1)
    return u / np.abs(u).max()


@pytest.mark.parametrize("dim,n", [(3, 32), (2, 64)])
def test_integrating_factor_step_matches_oracle(dim, n):
    """Extension: RK4 with the viscous term by the integrating factor exp(-nu k^2 t)
    vs the oracle's Lawson RK4 (rk4_if_wrapper), a few steps (2D with drag and
    Kolmogorov forcing)."""
    nu, dt, steps = 0.02, 5e-3, 3
    u = _band_limited(dim, n, 11)
    axes = (1, 2, 3) if dim == 3 else (1, 2)
    uh0 = np.fft.rfftn(u, axes=axes)
    kw, okw = {}, {}
    if dim == 2:
        uh0 = uh0.squeeze(-1)
        kw = dict(drag=0.1, kolm_k=4, kolm_amp=1.0)
        okw = dict(drag=0.1, force_hat=R.kolmogorov_forcing_hat(n, 1.0, 4))
    step = R.rk4_if_wrapper(dt, R.rhs_wrapper(n, 0.0, axes, **okw), nu, n, axes)
    uu, uh = u, uh0
    for _ in range(steps):
        uu, uh, _ = step(uu, uh)
    p = _plan(dim=dim, n=n, nu=nu, dt=dt, scheme="integrating_factor", **kw)
    g = _c64(uh0)
    p.step(g, steps)
    p.check()
    assert _rel(g.cpu().numpy(), uh) < RTOL
    # and it differs from the explicit form by the (small) truncation difference only
    q = _plan(dim=dim, n=n, nu=nu, dt=dt, **kw)
    ge = _c64(uh0)
    q.step(ge, steps)
    assert _rel(ge.cpu().numpy(), uh) < 1e-3


def test_integrating_factor_is_stable_where_explicit_rk4_blows_up():
    """nu k^2 dt far above explicit RK4's stability limit (~2.8) for the high modes:
    the explicit step produces non-finite values (reported as NonFiniteError), the
    integrating-factor step stays finite and matches the oracle."""
    from l3es import _native

    n, nu, dt, steps = 32, 0.2, 0.05, 40  # nu k^2 dt up to 0.2 * 0.05 * 768 = 7.7 on the grid
    u = _band_limited(3, n, 12, kmax=4)
    uh0 = np.fft.rfftn(u, axes=(1, 2, 3))
    pe = _plan(dim=3, n=n, nu=nu, dt=dt)
    rng = np.random.default_rng(0)
    noise = 1e-6 * (rng.standard_normal(uh0.shape) + 1j * rng.standard_normal(uh0.shape))
    ge = _c64(uh0 + noise)  # round-off-sized content in the stiff modes
    for _ in range(20):
        pe.step(ge, steps)
        try:
            pe.check()
        except _native.NonFiniteError:
            break
    else:
        pytest.fail("the explicit step stayed finite where it should be unstable")
    step = R.rk4_if_wrapper(dt, R.rhs_wrapper(n, 0.0), nu, n)
    uu, uh = u, uh0 + noise
    for _ in range(steps):
        uu, uh, _ = step(uu, uh)
    pi = _plan(dim=3, n=n, nu=nu, dt=dt, scheme="integrating_factor")
    gi = _c64(uh0 + noise)
    pi.step(gi, steps)
    pi.check()
    assert _rel(gi.cpu().numpy(), uh) < 1e-4


def test_integrating_factor_decays_a_shear_mode_exactly():
    """u = (sin y, 0, 0): the nonlinear term is a pure gradient, so the exact solution
    is exp(-nu t) u; the integrating-factor step reproduces it to FP32 rounding."""
    n, nu, dt, steps = 32, 0.5, 0.1, 10
    y = np.arange(n) * 2 * np.pi / n
    u = np.zeros((3, n, n, n))
    u[0] = np.sin(y)[None, :, None]
    p = _plan(dim=3, n=n, nu=nu, dt=dt, scheme="integrating_factor")
    g = _c64(np.fft.rfftn(u, axes=(1, 2, 3)))
    p.step(g, steps)
    out = torch.empty(p.phys_shape, dtype=torch.float32, device="cuda")
    p.irfftn(g, out)
    assert np.abs(out.cpu().numpy() - np.exp(-nu * dt * steps) * u).max() < 1e-6


@pytest.mark.parametrize("n", [64, 128, 256])
def test_every_kernel_schedule_gives_the_same_step(n):
    """The kernel schedules (x pass, y-pass radix, line pass, band pass variants; at 256
    also the radix-16 line passes) compute the same RK4 step to FP32 rounding
    (against the default schedule)."""
    import itertools

    u0 = R.init_u_hit(n, 3, spectrum="k4exp", kp=3.0)
    uh0 = np.fft.rfftn(u0, axes=(1, 2, 3))
    p = _plan(dim=3, n=n, nu=5e-3, dt=2e-3, forcing="const_power", kf=2, eps_inj=0.1)
    ref = _c64(uh0)
    p.step(ref, 2)
    ref = ref.cpu().numpy()
    keys = p.SCHEDULE_KEYS
    line_vals = (0, 1, 2, 3) if n == 256 else (0, 1)
    for combo in itertools.product((0, 1), (0, 1), line_vals, (0, 1)):
        p.set_schedule(dict(zip(keys, combo)))
        g = _c64(uh0)
        p.step(g, 2)
        p.check()
        assert _rel(g.cpu().numpy(), ref) < 2e-6, combo


@pytest.mark.parametrize("case", ["3d64_const_power", "3d128_none", "3d64_const_power_batch3_x_plain",
                                  "2d256_kolmogorov", "3d256_const_power", "3d64_drag_nu_batch2",
                                  "3d32_ekin_tot"])
def test_rk_step_forms_agree(case):
    """The three forms of the explicit RK4 step (one elementwise update of the whole
    spectrum; the closed form of the linear decay outside the dealiased rows; the stage
    combination fused into the band pass with every other mode scaled inside the next
    x inverse) compute the same steps to FP32 rounding, with the one-tile and the
    persistent x and band passes, single and batched plans."""
    steps = 3
    if case.startswith("2d"):
        n = 256
        u = R.init_u_random2d(n, 11)
        uh0 = np.fft.rfftn(u, axes=(1, 2)).squeeze()[None]
        kw = dict(dim=2, n=n, nu=1e-3, dt=1e-3, drag=0.1, kolm_k=4, kolm_amp=1.0)
        batch = 1
    else:
        n = int(case[2:case.index("_")])
        batch = 3 if "batch3" in case else 1
        uh0 = []
        for b in range(batch):
            u = R.init_u_hit(n, 3 + b, spectrum="k4exp", kp=3.0)
            uh0.append(np.fft.rfftn(u * np.sqrt(0.5 / R.kinetic_energy(u)), axes=(1, 2, 3)))
        uh0 = np.stack(uh0)
        kw = dict(dim=3, n=n, nu=5e-3, dt=2e-3)
        if "const_power" in case:
            kw.update(forcing="const_power", kf=2, eps_inj=0.1)
        if "drag" in case:
            kw.update(drag=0.05)
        if "ekin_tot" in case:
            kw.update(forcing="ekin_tot", kf=2, e_kin_init=0.5)
    if "batch2" in case:  # the drag case also runs two trajectories of different viscosity
        batch = 2
        uh0 = np.stack([uh0[0], 0.5 * uh0[0]])
    p = _plan(batch=batch, **kw)
    if "nu" in case.split("_"):
        p.set_nu([5e-3, 2e-2])
    assert p.step_form == (2 if kw["dim"] == 3 else 1)
    if "x_plain" in case:
        p.set_schedule({"x_bulk": 0, "band_bulk": 0})
    outs = {}
    for form in (0, 1, 2):
        p.step_form = form
        g = _c64(uh0 if batch > 1 else uh0[0])
        p.step(g, steps)
        p.check()
        outs[form] = g.cpu().numpy()
    assert _rel(outs[1], outs[0]) < 2e-6
    assert _rel(outs[2], outs[0]) < 2e-6
    with pytest.raises(Exception, match="form"):
        p.step_form = 3


@pytest.mark.parametrize("n,batch", [(256, 1), (128, 3), (512, 1)])
def test_2d_x_tile_widths_agree(n, batch):
    """2D x passes in 2-column tiles (schedule entry 0, the default in 2D) and in
    8-column tiles give the same Kolmogorov steps in both 2D step forms, single and
    batched, and match the FP64 oracle."""
    nu, dt, steps = 1e-3, 1e-3, 3
    us = [R.init_u_random2d(n, 11 + b) for b in range(batch)]
    uh0 = np.stack([np.fft.rfftn(u, axes=(1, 2)).squeeze() for u in us])
    p = _plan(dim=2, n=n, nu=nu, dt=dt, drag=0.1, kolm_k=4, kolm_amp=1.0, batch=batch)
    assert p.schedule["x_bulk"] == 1
    outs = {}
    for xb in (1, 0):
        for form in (1, 2):
            p.set_schedule({"x_bulk": xb})
            p.step_form = form
            g = _c64(uh0 if batch > 1 else uh0[0])
            p.step(g, steps)
            p.check()
            outs[(xb, form)] = g.cpu().numpy().reshape(uh0.shape)
    for key, v in outs.items():
        assert _rel(v, outs[(1, 1)]) < 2e-6, key
    rhs = R.rhs_wrapper(n, nu, (1, 2), drag=0.1, force_hat=R.kolmogorov_forcing_hat(n, 1.0, 4))
    step = R.rk4_wrapper(dt, rhs, None, 0.0, "none", (1, 2))
    for b in range(batch):
        uu, uh = us[b], uh0[b]
        for _ in range(steps):
            uu, uh, _ = step(uu, uh)
        assert _rel(outs[(1, 1)][b], uh) < 2e-5


def test_forcing_outside_the_band_takes_the_whole_spectrum_form():
    """A Kolmogorov forcing wavenumber beyond the stored band (kolm_k = 26 >= kt = 24 at
    64^2) puts a forcing term on a mode the band pass does not own: every requested step
    form then runs the whole-spectrum update, and the steps match the FP64 oracle.
    (Constant-power forcing cannot reach beyond the band: plans take kf <= N/4 < kd.)"""
    n, nu, dt, kk, steps = 64, 1e-3, 1e-3, 26, 3
    u = R.init_u_random2d(n, 11)
    uh0 = np.fft.rfftn(u, axes=(1, 2)).squeeze()
    rhs = R.rhs_wrapper(n, nu, (1, 2), drag=0.1, force_hat=R.kolmogorov_forcing_hat(n, 1.0, kk))
    step = R.rk4_wrapper(dt, rhs, None, 0.0, "none", (1, 2))
    uu, uh = u, uh0
    for _ in range(steps):
        uu, uh, _ = step(uu, uh)
    p = _plan(dim=2, n=n, nu=nu, dt=dt, drag=0.1, kolm_k=kk, kolm_amp=1.0)
    for form in (2, 1, 0):
        p.step_form = form
        g = _c64(uh0)
        p.step(g, steps)
        p.check()
        assert _rel(g.cpu().numpy(), uh) < RTOL, form


def test_line_pass_variants_agree_in_2d_at_256():
    """2D Kolmogorov flow at 256^2 (drag, sin 4y forcing): every line pass variant gives
    the same steps, and the radix-16 forms against the FP64 oracle."""
    n, nu, dt, steps = 256, 1e-3, 1e-3, 3
    u = R.init_u_random2d(n, 11)  # |k| <= 8, KE 0.5
    uh0 = np.fft.rfftn(u, axes=(1, 2)).squeeze()
    p = _plan(dim=2, n=n, nu=nu, dt=dt, drag=0.1, kolm_k=4, kolm_amp=1.0)
    outs = {}
    for lp in (0, 1, 2, 3):
        p.set_schedule({"line_pair": lp})
        g = _c64(uh0)
        p.step(g, steps)
        p.check()
        outs[lp] = g.cpu().numpy()
    for lp in (0, 2, 3):
        assert _rel(outs[lp], outs[1]) < 2e-6, lp
    rhs = R.rhs_wrapper(n, nu, (1, 2), drag=0.1, force_hat=R.kolmogorov_forcing_hat(n, 1.0, 4))
    step = R.rk4_wrapper(dt, rhs, None, 0.0, "none", (1, 2))
    uu, uh = u, uh0
    for _ in range(steps):
        uu, uh, _ = step(uu, uh)
    assert _rel(outs[2], uh) < 2e-5 and _rel(outs[3], uh) < 2e-5


def test_autotune_picks_a_schedule_and_caches_it(tmp_path):
    from l3es import _native

    cache = str(tmp_path / "sched.txt")
    p = _plan(dim=3, n=128, nu=5e-3, dt=2e-3)
    s1 = p.autotune(cache)
    assert set(s1) == set(_native.Plan.SCHEDULE_KEYS) and all(v in (0, 1) for v in s1.values())
    lines = open(cache).read().splitlines()
    assert len(lines) == 1 and "|d3|n128|b1" in lines[0]
    q = _plan(dim=3, n=128, nu=1e-2, dt=1e-3)
    q.set_schedule({k: 1 - v for k, v in s1.items()})
    assert q.autotune(cache) == s1  # read from the cache, not re-timed
    assert len(open(cache).read().splitlines()) == 1
    # the tuner times whole steps on zeroed scratch, where a constant-power coefficient
    # can overflow: nothing of that reaches the plan's error word
    r = _plan(dim=2, n=64, nu=1e-3, dt=1e-3, forcing="const_power", kf=2, eps_inj=0.1, kolm_k=4, kolm_amp=1.0)
    r.autotune("")
    r.check()
