"""Coarsening, NUFFT / DFT interpolation and advection on the GPU vs the oracle."""

import numpy as np
import pytest

from oracle import numpy_ref as R
from oracle import nufft_ref as NU

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


def _plan(**kw):
    from l3es import _native

    return _native.InterpPlan(**kw)


def _t(a, dt):
    return torch.from_numpy(np.ascontiguousarray(a).astype(dt)).cuda()


@pytest.mark.parametrize("dim,n,c", [(3, 32, 16), (3, 64, 32), (3, 256, 32), (2, 64, 16), (2, 256, 64)])
def test_filter_from_spectrum_matches_spectral_filtering(dim, n, c):
    """spectral_filtering(irfftn(u_hat), c) from the fine spectrum (utils.py:100-138)."""
    rng = np.random.default_rng(dim * 1000 + n)
    shape = (3, n, n, n) if dim == 3 else (3, n, n)
    axes = (1, 2, 3) if dim == 3 else (1, 2)
    u = rng.standard_normal(shape)
    uh = np.fft.rfftn(u, axes=axes)
    # the reference infers dim from len(u): 2D fields go in as (2, N, N) (combined.py:122)
    ref = R.spectral_filtering(u if dim == 3 else u[:2], c)
    p = _plan(dim=dim, ckp_n=c, n_fine=n)
    p.set_spectrum(_t(uh, np.complex64))
    out = torch.empty(p.coarse_shape, dtype=torch.float32, device="cuda")
    p.coarse_field(out)
    got = out.cpu().numpy().reshape((3,) + (c,) * dim)
    assert _rel(got[: len(ref)], ref) < 2e-5


@pytest.mark.parametrize("dim,c,np_", [(3, 16, 500), (3, 32, 32768), (2, 64, 4096)])
def test_nufft_and_dft_interp_match_oracle(dim, c, np_):
    rng = np.random.default_rng(c + dim)
    shape = (3,) + (c,) * dim
    g = rng.standard_normal(shape)
    # keep the exact sum cheap for the oracle: a band-limited coarse field
    axes = tuple(range(1, dim + 1))
    gh = np.fft.fftn(g, axes=axes)
    k = np.fft.fftfreq(c, 1.0 / c)
    kk = np.sqrt(sum(np.meshgrid(*([k ** 2] * dim), indexing="ij")))
    g = np.real(np.fft.ifftn(gh * (kk <= c / 2 - 1), axes=axes))
    r = rng.uniform(0, 2 * np.pi, (np_, dim))
    sub = slice(0, min(np_, 2000))
    comp = g[:dim] if dim == 2 else g
    ref = R.interpolate_dft(comp, r[sub])
    p = _plan(dim=dim, ckp_n=c, np_max=np_)
    field = g if dim == 3 else g[..., None]
    p.set_field(_t(field, np.float32))
    rt = _t(r, np.float64)
    for backend, tol in (("nufft", 5e-5), ("dft", 2e-5)):
        ur = torch.empty_like(rt)
        p.interp(rt, ur, backend=backend)
        assert _rel(ur.cpu().numpy()[sub], ref) < tol, backend
    # the NUFFT restatement of finufft agrees with the CUDA NUFFT closely too
    ur = torch.empty_like(rt)
    p.interp(rt, ur, backend="nufft")
    ref_nu = NU.interpolate_nufft(comp, r[sub], w=6)
    assert _rel(ur.cpu().numpy()[sub], ref_nu) < 1e-5


def test_dft_interp_reference_golden(gold):
    g = gold("interp")
    c = int(g["c"])
    for dim, field, r, ref in ((3, g["g3"], g["r3"], g["ur3"]), (2, g["g2"], g["r2"], g["ur2"])):
        p = _plan(dim=dim, ckp_n=16 if c < 16 else c, np_max=len(r)) if c >= 16 else None
        if p is None:
            # c = 8 fixture: embed in a 16-point grid by spectral zero padding
            cc = 16
            axes = tuple(range(1, dim + 1))
            fh = np.fft.fftshift(np.fft.fftn(field, axes=axes), axes=axes)
            big = np.zeros((field.shape[0],) + (cc,) * dim, dtype=complex)
            sl = tuple([slice(None)] + [slice(cc // 2 - c // 2, cc // 2 + c // 2)] * dim)
            big[sl] = fh
            field = np.real(np.fft.ifftn(np.fft.ifftshift(big, axes=axes), axes=axes)) * (cc / c) ** dim
            p = _plan(dim=dim, ckp_n=cc, np_max=len(r))
        f3 = np.concatenate([field, np.zeros_like(field[:1])]) if dim == 2 else field
        p.set_field(_t(f3 if dim == 3 else f3[..., None], np.float32))
        rt = _t(r, np.float64)
        ur = torch.empty_like(rt)
        p.interp(rt, ur, backend="dft")
        assert _rel(ur.cpu().numpy(), ref) < 2e-5


def test_fused_filter_interp_advect_matches_combined_loop():
    """combined.py:122-130 and :199 from the fine spectrum, vs the oracle (dft)."""
    n, c, dt = 64, 32, 0.01
    rng = np.random.default_rng(3)
    u = R.init_u_hit(n, 5, "k4exp", 4.0)
    uh = np.fft.rfftn(u, axes=(1, 2, 3))
    r = rng.uniform(0, 2 * np.pi, (1500, 3))
    u_r_ref = R.interpolate_from_uhat_dft(uh, n, c, r)
    r_ref = R.shift_fn(r, dt * u_r_ref)
    p = _plan(dim=3, ckp_n=c, n_fine=n, np_max=len(r))
    p.set_spectrum(_t(uh, np.complex64))
    rt = _t(r, np.float64)
    ur = torch.empty_like(rt)
    r_new = torch.empty_like(rt)
    p.interp(rt, ur, backend="nufft", dt=dt, r_out=r_new)
    assert _rel(ur.cpu().numpy(), u_r_ref) < 5e-5
    # positions move by dt * u_r: the NUFFT's ~1e-5 relative error times dt
    assert np.abs(r_new.cpu().numpy() - r_ref).max() < 1e-5


def test_shift_matches_reference_golden(gold):
    from l3es import _native

    g = gold("interp")
    out = _native.shift(_t(g["r3"], np.float64), _t(g["dr"], np.float64))
    assert np.abs(out.cpu().numpy() - g["shifted"]).max() < 1e-14


def _band_field(dim, c, seed):
    rng = np.random.default_rng(seed)
    g = rng.standard_normal((3,) + (c,) * dim)
    axes = tuple(range(1, dim + 1))
    gh = np.fft.fftn(g, axes=axes)
    k = np.fft.fftfreq(c, 1.0 / c)
    kk = np.sqrt(sum(np.meshgrid(*([k ** 2] * dim), indexing="ij")))
    g = np.real(np.fft.ifftn(gh * (kk <= c / 4), axes=axes))
    return g / np.abs(g).max()


@pytest.mark.parametrize("dim,c,np_", [(3, 16, 700), (2, 32, 1024)])
def test_rk4_advection_matches_oracle(dim, c, np_):
    """Extension: RK4 particle advection through the coarse field held fixed, both
    backends, vs the oracle's advect_rk4 over the exact DFT interpolant."""
    g = _band_field(dim, c, 40 + dim)
    comp = g[:dim] if dim == 2 else g
    rng = np.random.default_rng(5)
    r = rng.uniform(0, 2 * np.pi, (np_, dim))
    dt = 0.2
    u_ref, r_ref = R.advect_rk4(lambda x: R.interpolate_dft(comp, x), r, dt)
    p = _plan(dim=dim, ckp_n=c, np_max=np_)
    p.set_field(_t(g if dim == 3 else g[..., None], np.float32))
    rt = _t(r, np.float64)
    for backend, tol in (("dft", 2e-5), ("nufft", 5e-5)):
        ur = torch.empty_like(rt)
        rn = torch.empty_like(rt)
        p.advect_rk4(rt, ur, dt, rn, backend=backend)
        assert _rel(ur.cpu().numpy(), u_ref) < tol, backend
        d = np.mod(rn.cpu().numpy() - r_ref + np.pi, 2 * np.pi) - np.pi
        assert np.abs(d).max() < tol * dt * np.abs(u_ref).max(), backend
        assert (rn.cpu().numpy() >= 0).all() and (rn.cpu().numpy() < 2 * np.pi).all()
    # the Euler step of l3es_interp differs from RK4 at second order in dt
    ur = torch.empty_like(rt)
    re = torch.empty_like(rt)
    p.interp(rt, ur, backend="dft", dt=dt, r_out=re)
    de = np.mod(re.cpu().numpy() - r_ref + np.pi, 2 * np.pi) - np.pi
    assert np.abs(de).max() > 100 * 2e-5 * dt * np.abs(u_ref).max()


def test_rk4_advection_rejects_aliased_outputs():
    p = _plan(dim=3, ckp_n=16, np_max=64)
    r = torch.zeros(64, 3, dtype=torch.float64, device="cuda")
    u = torch.empty_like(r)
    with pytest.raises(RuntimeError, match="separate"):
        p.advect_rk4(r, u, 0.1, r)


@pytest.mark.parametrize("dim,n,c,b,np_", [(2, 128, 32, 3, 1024), (3, 64, 16, 2, 600)])
def test_batched_interp_plan_equals_single_plans(dim, n, c, b, np_):
    """One batched interpolator (l3es_interp_plan_create_batch) over the [b][3] spectra of
    a batched step plan gives the same velocities and advected positions, bit for bit,
    as one interpolator per trajectory; its single-trajectory calls are refused."""
    from l3es import _native

    rng = np.random.default_rng(dim * 10 + b)
    shape = (b, 3, n, n, n // 2 + 1) if dim == 3 else (b, 3, n, n // 2 + 1)
    uh = torch.from_numpy((rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)).cuda()
    r = torch.from_numpy(rng.uniform(0, 2 * np.pi, (b, np_, dim))).cuda()
    dt = 1e-3
    pb = _native.InterpPlan(dim=dim, ckp_n=c, n_fine=n, np_max=np_, batch=b)
    pb.set_spectrum(uh)
    ur_b = torch.empty_like(r)
    rn_b = torch.empty_like(r)
    pb.interp(r, ur_b, dt=dt, r_out=rn_b)
    for t in range(b):
        ps = _native.InterpPlan(dim=dim, ckp_n=c, n_fine=n, np_max=np_)
        ps.set_spectrum(uh[t].contiguous())
        ur = torch.empty(np_, dim, dtype=torch.float64, device="cuda")
        rn = torch.empty_like(ur)
        ps.interp(r[t].contiguous(), ur, dt=dt, r_out=rn)
        assert torch.equal(ur, ur_b[t]) and torch.equal(rn, rn_b[t]), t
    with pytest.raises(RuntimeError, match="NUFFT only"):
        pb.interp(r, ur_b, backend="dft")
    with pytest.raises(ValueError):
        pb.interp(r[0].contiguous(), ur_b[0].contiguous())
