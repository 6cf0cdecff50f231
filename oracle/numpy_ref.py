"""FP64 NumPy restatement of the l3es pseudo-spectral DNS hot path.

TEST INFRASTRUCTURE ONLY. This module is the oracle that the CUDA path is checked
against. Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` may import it; the product path (``l3es`` package, C-ABI library) never
does, and fails loudly when its CUDA library is missing.

Every function follows a named reference function op for op (file:line within the
tumaer/ql-les-data project). Parity is pinned by the reference's own golden value
(``from_spectralDNS/main_numpy.py:136``: TGV 64^3 KE after 10 RK4 steps =
0.124953117517) and by fixtures generated from the reference's own runnable NumPy
solver (``tests/golden/make_golden.py``).

Terms that the benchmark workloads need but the reference does not have
(linear drag, Kolmogorov forcing, constant-power band forcing, the
k^4 exp(-2(k/kp)^2) Rogallo spectrum, band-limited random 2D init) are opt-in
arguments that default to the reference behaviour.
"""

from __future__ import annotations

import os

import numpy as np

try:  # scipy's pocketfft takes a worker count; numpy's does not
    import scipy.fft as _sfft
except Exception:  # pragma: no cover
    _sfft = None

# jnp.finfo(float).eps with x64 (l3es/spectral_solver.py:23, init_fields.py:9)
EPS = float(np.finfo(np.float64).eps)

_WORKERS = 1


def set_workers(n: int | None) -> None:
    """Number of host threads the FFTs use (1 = plain numpy.fft)."""
    global _WORKERS
    _WORKERS = max(1, int(n if n is not None else (os.cpu_count() or 1)))


def _rfftn(a, axes):
    if _WORKERS > 1 and _sfft is not None:
        return _sfft.rfftn(a, axes=axes, workers=_WORKERS)
    return np.fft.rfftn(a, axes=axes)


def _irfftn(a, axes, s=None, norm=None):
    if _WORKERS > 1 and _sfft is not None:
        return _sfft.irfftn(a, s=s, axes=axes, norm=norm, workers=_WORKERS)
    return np.fft.irfftn(a, s=s, axes=axes, norm=norm)


def _fftn(a, axes):
    if _WORKERS > 1 and _sfft is not None:
        return _sfft.fftn(a, axes=axes, workers=_WORKERS)
    return np.fft.fftn(a, axes=axes)


def _ifftn(a, axes):
    if _WORKERS > 1 and _sfft is not None:
        return _sfft.ifftn(a, axes=axes, workers=_WORKERS)
    return np.fft.ifftn(a, axes=axes)


# ---------------------------------------------------------------------------------
# wavenumber tables (l3es/spectral_solver.py:27-48)
# ---------------------------------------------------------------------------------
def wavenumbers(N: int, dim: int = 3):
    """kkk, kkk2, kkk/kkk2 and the cube dealias mask of ``rhs_wrapper``.

    spectral_solver.py:32-48: ``fftfreq`` integer wavenumbers, the half (last) axis
    truncated to N//2+1 with its Nyquist entry made positive; in 2D a zero third
    component is appended; dealias keeps |k_i| < 2/3 (N//2+1) on every axis.
    """
    kx = np.fft.fftfreq(N, 1.0 / N)
    kz = kx[: N // 2 + 1].copy()
    kz[-1] *= -1
    if dim == 3:
        kkk = np.array(np.meshgrid(kx, kx, kz, indexing="ij"), dtype=np.int64)
    else:
        kk = np.array(np.meshgrid(kx, kz, indexing="ij"), dtype=np.int64)
        kkk = np.concatenate([kk, np.zeros((1, N, N // 2 + 1), dtype=np.int64)], 0)
    kkk2 = np.sum(kkk * kkk, 0, dtype=np.int64)
    kkk_over_kkk2 = kkk.astype(np.float64) / np.where(kkk2 == 0, 1, kkk2).astype(
        np.float64
    )
    kmax_dealias = 2.0 / 3.0 * (N // 2 + 1)
    dealias = (
        (np.abs(kkk[0]) < kmax_dealias)
        & (np.abs(kkk[1]) < kmax_dealias)
        & (np.abs(kkk[2]) < kmax_dealias)
    )
    return kkk, kkk2, kkk_over_kkk2, dealias


def kolmogorov_forcing_hat(N: int, amp: float = 1.0, kf: int = 4):
    """Half-spectrum of f = (amp sin(kf y), 0, 0) on an N x N grid (extension).

    Not in the reference (its Kolm case is unforced; spectral_solver.py:50-60).
    ``rfftn(sin(kf y))`` over (x, y) is -i N^2/2 at (kx=0, ky=kf).
    """
    f = np.zeros((3, N, N // 2 + 1), dtype=np.complex128)
    f[0, 0, kf] = -0.5j * amp * N * N
    return f


# ---------------------------------------------------------------------------------
# RHS and RK4 (l3es/spectral_solver.py:27-120)
# ---------------------------------------------------------------------------------
def rhs_wrapper(N, nu, fft_axes=(1, 2, 3), drag=0.0, force_hat=None,
                const_power=None):
    """rhs_fn(u, u_hat, rk) of spectral_solver.py:50-60.

    du = P[dealias * rfftn(u x curl u)] - nu k^2 u_hat  (P: Leray projection applied
    as du -= (sum du.k/k^2) k). Extension terms (all off by default):
      drag        du -= drag * u_hat
      force_hat   du += force_hat            (e.g. Kolmogorov sin(4y))
      const_power (eps, mask): du += eps/(2 E_f) * u_hat * mask, with E_f the
                  kinetic energy of the masked modes (constant power injection).
    """
    dim = len(fft_axes)
    kkk, kkk2, kkk_over_kkk2, dealias = wavenumbers(N, dim)
    ikkk = 1j * kkk

    def rhs_fn(u, u_hat, rk):
        if rk > 0:
            u = _irfftn(u_hat, axes=fft_axes)
        curl = _irfftn(np.cross(ikkk, u_hat, axis=0), axes=fft_axes)
        du = _rfftn(np.cross(u.squeeze(), curl, axis=0), axes=fft_axes)
        du *= dealias
        p_hat = np.sum(du * kkk_over_kkk2, axis=0)
        du -= p_hat * kkk
        du -= nu * kkk2 * u_hat
        if drag:
            du -= drag * u_hat
        if force_hat is not None:
            du += force_hat
        if const_power is not None:
            eps_inj, mask = const_power
            e_f = band_energy(u_hat, mask, N, dim)
            du += (eps_inj / (2.0 * e_f + EPS)) * u_hat * mask
        return du

    return rhs_fn


def half_weights(N: int, dim: int):
    """Multiplicity of each half-spectrum mode in the full spectrum (Parseval)."""
    w = np.full(N // 2 + 1, 2.0)
    w[0] = 1.0
    w[-1] = 1.0
    return w


def band_energy(u_hat, mask, N, dim):
    """0.5 mean(|irfftn(u_hat * mask)|^2) via Parseval (FP64)."""
    w = half_weights(N, dim)
    e = np.sum(w * np.sum(np.abs(u_hat * mask) ** 2, axis=0))
    return 0.5 * e / float(N) ** (2 * dim)


def rk4_wrapper(dt, rhs_fn, forcing_mask, e_kin_init, forcing_type,
                fft_axes=(1, 2, 3)):
    """step_fn(u, u_hat) -> (u, u_hat, e_inj) of spectral_solver.py:65-120."""
    a_rk4 = [1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0]
    b_rk4 = [0.5, 0.5, 1.0]

    def step_fn(u, u_hat):
        u_temp1, u_temp2 = u_hat.copy(), u_hat.copy()
        for rk in range(4):
            du = rhs_fn(u, u_hat, rk)
            if rk < 3:
                u_hat = u_temp1 + b_rk4[rk] * dt * du
            u_temp2 += a_rk4[rk] * dt * du
        u_hat = u_temp2

        e_inj = 0.0
        if forcing_mask is not None and forcing_type == "ekin_tot":
            # spectral_solver.py:82-112 (Lamorgese et al. 2005 KE rescaling)
            u_new = _irfftn(u_hat, axes=fft_axes)
            e_kin_new = 0.5 * np.mean(np.sum(u_new * u_new, axis=0))
            u_lower = _irfftn(u_hat * forcing_mask, axes=fft_axes)
            e_kin_lower = 0.5 * np.mean(np.sum(u_lower * u_lower, axis=0))
            e_kin_high = e_kin_new - e_kin_lower
            alpha = np.sqrt(max(0.0, (e_kin_init - e_kin_high) / (e_kin_lower + EPS)))
            e_inj = max(0.0, (e_kin_init - e_kin_new) / dt)
            u_hat = u_hat * (alpha * forcing_mask + (1 - forcing_mask))

        u = _irfftn(u_hat, axes=fft_axes)
        if len(fft_axes) == 2:
            u = np.expand_dims(u, -1)
        return u, u_hat, e_inj

    return step_fn


def rk4_if_wrapper(dt, rhs_fn_inviscid, nu, N, fft_axes=(1, 2, 3)):
    """Extension (no reference counterpart): the classical RK4 step with the viscous term
    integrated exactly by an integrating factor (Lawson's RK4 on v = exp(nu k^2 t) u_hat).
    rhs_fn_inviscid is rhs_wrapper(N, 0.0, ...) (the right-hand side without viscosity);
    with E(s) = exp(-nu k^2 s):
        k1 = R(u0);  a = E(h/2) (u0 + h/2 k1)
        k2 = R(a);   b = E(h/2) u0 + h/2 k2
        k3 = R(b);   c = E(h) u0 + h E(h/2) k3
        k4 = R(c);   u1 = E(h) u0 + h/6 (E(h) k1 + 2 E(h/2) (k2 + k3) + k4)
    Returns step_fn(u, u_hat) -> (u, u_hat, 0.0) like rk4_wrapper."""
    dim = len(fft_axes)
    _, kkk2, _, _ = wavenumbers(N, dim)
    eh = np.exp(-nu * kkk2 * 0.5 * dt)
    e1 = eh * eh
    h = dt

    def step_fn(u, u_hat):
        u0 = u_hat
        k1 = rhs_fn_inviscid(u, u0, 0)
        a = eh * (u0 + 0.5 * h * k1)
        k2 = rhs_fn_inviscid(None, a, 1)
        b = eh * u0 + 0.5 * h * k2
        k3 = rhs_fn_inviscid(None, b, 2)
        c = e1 * u0 + h * eh * k3
        k4 = rhs_fn_inviscid(None, c, 3)
        u1 = e1 * u0 + h / 6.0 * (e1 * k1 + 2.0 * eh * (k2 + k3) + k4)
        u_new = _irfftn(u1, axes=fft_axes)
        if dim == 2:
            u_new = np.expand_dims(u_new, -1)
        return u_new, u1, 0.0

    return step_fn


def comp_dt(u, dx, nu, cfl=1.0):
    """spectral_solver.py:123-127 (Hickel et al. 2006, eq. 61)."""
    umax = np.max(np.abs(u), axis=(1, 2, 3))
    return cfl / (umax / dx + nu / dx**2).min()


# ---------------------------------------------------------------------------------
# initial fields (l3es/init_fields.py)
# ---------------------------------------------------------------------------------
def init_u_tgv(x, y, z):
    """init_fields.py:12-16."""
    return np.array(
        [np.sin(x) * np.cos(y) * np.cos(z), -np.cos(x) * np.sin(y) * np.cos(z), x * 0]
    )


def init_u_tgv2d(Nx, target_dim=2, rescale=1.0):
    """init_fields.py:19-30 (cell-centred grid, meshgrid 'xy' ordering)."""
    L = rescale
    dx = L / Nx
    x_axis = np.linspace(dx / 2, L - dx / 2, Nx)
    x, y = np.meshgrid(x_axis, x_axis)
    u = np.array([-np.cos(x) * np.sin(y), np.sin(x) * np.cos(y)])
    if target_dim == 3:
        u = u[..., None]
        u = np.concatenate([u, np.zeros((1, Nx, Nx, 1))], axis=0)
    return u * rescale


def rogallo_spectrum(nmax: int, spectrum: str = "k-5/3", kp: float = 4.0):
    """E_k table of init_u_hit (init_fields.py:38-41).

    'k-5/3' is the reference's k^(-5/3)/(4 pi k^2); 'k4exp' (extension) is
    k^4 exp(-2 (k/kp)^2) / (4 pi k^2).
    """
    E_k = np.zeros(nmax + 1) + EPS
    k_arr = np.arange(1, nmax + 1, dtype=np.float64)
    if spectrum == "k-5/3":
        E_k[1:] = k_arr ** (-5 / 3) / (4 * np.pi * k_arr**2)
    elif spectrum == "k4exp":
        E_k[1:] = k_arr**4 * np.exp(-2.0 * (k_arr / kp) ** 2) / (4 * np.pi * k_arr**2)
    else:
        raise ValueError(f"unknown spectrum {spectrum!r}")
    return E_k


def init_u_hit(N, seed=42, spectrum="k-5/3", kp=4.0):
    """Rogallo random-phase solenoidal field, init_fields.py:33-106.

    Same legacy ``np.random.seed`` stream and draw shape (N//2+1, N, N, 3) as the
    reference, so the phases are bit-identical.
    """
    rs = np.random.RandomState(seed)
    nmax = round(np.sqrt(3 * N**2) / 2)
    E_k = rogallo_spectrum(nmax, spectrum, kp)

    k1_loop = np.arange(N // 2 + 1)
    k2_loop = np.arange(-N // 2, N // 2)
    k3_loop = np.arange(-N // 2, N // 2)
    K1, K2, K3 = np.meshgrid(k1_loop, k2_loop, k3_loop, indexing="ij")
    WK = np.sqrt(K1**2 + K2**2 + K3**2)
    WK12 = np.sqrt(K1**2 + K2**2)
    NK = np.clip(np.round(WK).astype(int), 0, nmax)
    AMP = np.sqrt(E_k[NK])

    phis = 2 * np.pi * rs.random_sample((N // 2 + 1, N, N, 3))
    phi1, phi2, phi3 = phis[..., 0], phis[..., 1], phis[..., 2]
    ai = AMP * np.exp(1j * phi1) * np.cos(phi3)
    bi = AMP * np.exp(1j * phi2) * np.sin(phi3)
    del phis, phi1, phi2, phi3

    WK_safe = np.where(WK == 0, 1.0, WK)
    WK12_safe = np.where(WK12 == 0, 1.0, WK12)
    u_loop = np.zeros((N // 2 + 1, N, N, 3), dtype=np.complex128)
    u_loop[..., 0] = (ai * WK * K2 + bi * K1 * K3) / (WK_safe * WK12_safe)
    u_loop[..., 1] = (bi * K2 * K3 - ai * WK * K1) / (WK_safe * WK12_safe)
    u_loop[..., 2] = -bi * WK12 / WK_safe
    m12 = WK12 == 0
    u_loop[..., 0] = np.where(m12, ai, u_loop[..., 0])
    u_loop[..., 1] = np.where(m12, bi, u_loop[..., 1])
    m0 = WK == 0
    for c in range(3):
        u_loop[..., c] = np.where(m0, 0.0, u_loop[..., c])

    j_idx = (N + k2_loop) % N
    k_idx = (N + k3_loop) % N
    j_inv = np.argsort(j_idx)
    k_inv = np.argsort(k_idx)
    u = u_loop[:, j_inv, :][:, :, k_inv]

    Nf_ = N // 2
    u[0, -Nf_ + 1 :, -Nf_ + 1 :, :] = np.flip(np.conj(u[0, 1:Nf_, 1:Nf_, :]), axis=(0, 1))
    u[0, 1:Nf_, -Nf_ + 1 :, :] = np.flip(np.conj(u[0, -Nf_ + 1 :, 1:Nf_, :]), axis=(0, 1))
    u[0, 0, -Nf_ + 1 :, :] = np.flip(np.conj(u[0, 0, 1:Nf_, :]), axis=0)
    u[0, -Nf_ + 1 :, 0, :] = np.flip(np.conj(u[0, 1:Nf_, 0, :]), axis=0)

    return _irfftn(u.transpose(3, 0, 1, 2), axes=(-1, -2, -3), norm="forward")


def init_forcing_mask_hit(N, kf=3):
    """init_fields.py:167-188: 0 < |k|^2 <= kf^2 on the rfftn half spectrum."""
    k1 = np.fft.fftfreq(N, 1.0 / N)
    k3 = k1[: N // 2 + 1].copy()
    k3[-1] *= -1
    k1k2k3 = np.asarray(np.meshgrid(k1, k1, k3, indexing="ij"))
    k_mag = np.sum(k1k2k3**2, axis=0)
    return (k_mag <= kf**2) & (k_mag > 0)


def init_u_random2d(N, seed=0, kmax=8.0, energy=0.5, target_dim=3):
    """Band-limited random-phase 2D field (extension; no reference counterpart).

    Stream function psi_hat with unit amplitude and uniform random phase on
    0 < |k| <= kmax, u = d psi/dy, v = -d psi/dx, rescaled to 0.5 mean |u|^2 = energy.
    Layout (3, N, N, 1) like init_u_tgv2d(target_dim=3).
    """
    rng = np.random.default_rng(seed)
    kx = np.fft.fftfreq(N, 1.0 / N)
    ky = np.arange(N // 2 + 1, dtype=np.float64)
    KX, KY = np.meshgrid(kx, ky, indexing="ij")
    kk = np.sqrt(KX**2 + KY**2)
    band = (kk > 0) & (kk <= kmax)
    phase = rng.uniform(0.0, 2 * np.pi, size=KX.shape)
    psi_hat = np.where(band, np.exp(1j * phase), 0.0)
    u = _irfftn(1j * KY * psi_hat, axes=(0, 1), s=(N, N))
    v = _irfftn(-1j * KX * psi_hat, axes=(0, 1), s=(N, N))
    uv = np.array([u, v])
    e = 0.5 * np.mean(np.sum(uv * uv, axis=0))
    uv *= np.sqrt(energy / e)
    if target_dim == 3:
        uv = np.concatenate([uv[..., None], np.zeros((1, N, N, 1))], axis=0)
    return uv


# ---------------------------------------------------------------------------------
# solver set-up (l3es/spectral_solver.py:156-230)
# ---------------------------------------------------------------------------------
def init_u_kolm(N, L=2 * np.pi, max_velocity=4.2, seed=42, target_dim=3, iter=4,
                grid_n=2048, peak_wavenumber=4.0):
    """Kolmogorov initial field (init_fields.py:191-212), restating JAX-CFD's
    filtered_velocity_field on a grid_n^2 grid of side L: seeded white noise
    (np.random.default_rng(seed), 2 components), radial log-normal filter
    exp(-(ln k - ln k_p)^2 / 2) / k with k in cycles per unit length (Nyquist row and
    column zeroed), then `iter` x (Leray projection, scale max |u| to max_velocity),
    then spectral_filtering to N^2. Full complex FFTs here. PARITY UNPINNED: JAX's
    generator and JAX-CFD are unavailable, so this only checks the drop-in's own
    restatement of the same construction."""
    G = grid_n
    rng = np.random.default_rng(seed)
    noise = rng.standard_normal((2, G, G))
    k1 = np.fft.fftfreq(G, L / G)
    KX, KY = np.meshgrid(k1, k1, indexing="ij")
    kk = np.hypot(KX, KY)
    with np.errstate(divide="ignore", invalid="ignore"):
        filt = np.where(kk > 0, np.exp(-0.5 * (np.log(kk) - np.log(peak_wavenumber)) ** 2) / kk, 0.0)
    filt[G // 2, :] = 0.0
    filt[:, G // 2] = 0.0
    vh = _fftn(noise, axes=(1, 2)) * filt
    k2 = np.where(kk > 0, kk * kk, 1.0)
    for _ in range(max(1, iter)):
        kv = (KX * vh[0] + KY * vh[1]) / k2
        vh = np.array([vh[0] - KX * kv, vh[1] - KY * kv])
        v = _ifftn(vh, axes=(1, 2)).real
        vh = vh * (max_velocity / np.max(np.sqrt(np.sum(v * v, axis=0))))
    u = spectral_filtering(_ifftn(vh, axes=(1, 2)).real, N)[..., None]
    if target_dim == 3:
        u = np.concatenate([u, np.zeros((1, N, N, 1))], axis=0)
    return u


def set_up_solver(N, nu, dim, case, dt, seed, ckp_N, kf, e_kin_target=None,
                  forcing_type="ekin_tot", warmup=True, **ext):
    """Host restatement of spectral_solver.py:156-230 (no executable cache).

    Returns (u, u_hat, dx, step_fn, L, fft_axes, e_kin_init, e_inj). Like the
    reference, one step is taken before returning (``warmup``).
    """
    L = 2 * np.pi
    dx = L / N
    len_z = N if dim == 3 else 1
    fft_axes = (1, 2, 3) if dim == 3 else (1, 2)
    xyz = np.array(np.meshgrid(np.arange(N), np.arange(N), np.arange(len_z),
                               indexing="ij")) * L / N
    forcing_mask = init_forcing_mask_hit(N, kf) if (
        case == "HIT" and forcing_type != "none") else None
    if case == "TGV3D":
        u = init_u_tgv(xyz[0], xyz[1], xyz[2])
    elif case == "TGV2D":
        u = init_u_tgv2d(N, target_dim=3, rescale=L)
    elif case == "HIT":
        u = init_u_hit(N, seed, ext.get("spectrum", "k-5/3"), ext.get("kp", 4.0))
    elif case == "Kolm" and ext.get("init", "kolm") == "random2d":
        u = init_u_random2d(N, seed, ext.get("init_kmax", 8.0),
                            ext.get("init_energy", 0.5))
    elif case == "Kolm":
        u = init_u_kolm(N, seed=seed, target_dim=3, grid_n=ext.get("kolm_grid", 2048))
    else:
        raise ValueError(case)
    e_kin_init = 0.5 * np.mean(np.sum(u * u, axis=0))
    if forcing_type != "none":
        u = u * np.sqrt(e_kin_target / (e_kin_init + EPS))
    u_hat = _rfftn(u, axes=fft_axes).squeeze()
    e_kin_init = 0.5 * np.mean(np.sum(u * u, axis=0))
    rhs = rhs_wrapper(N, nu, fft_axes, **{k: v for k, v in ext.items()
                                          if k in ("drag", "force_hat", "const_power")})
    step_fn = rk4_wrapper(dt, rhs, forcing_mask, e_kin_init, forcing_type, fft_axes)
    e_inj = 0.0
    if warmup:
        u, u_hat, e_inj = step_fn(u, u_hat)
    return u, u_hat, dx, step_fn, L, fft_axes, e_kin_init, e_inj


# ---------------------------------------------------------------------------------
# spectral utilities (l3es/utils.py)
# ---------------------------------------------------------------------------------
def spectral_filtering(u, ckp_N):
    """utils.py:100-138: keep k in [-c/2, c/2-1] per axis, ifftn / (N/c)^d, real."""
    N_u = u.shape[1]
    dim = len(u)
    fft_axes = (1, 2, 3) if dim == 3 else (1, 2)
    y_fft = _fftn(u, axes=fft_axes)
    sl = slice(N_u // 2 - ckp_N // 2, N_u // 2 + ckp_N // 2)
    slices = tuple([slice(None)] + [sl] * dim)
    y_sub = np.fft.ifftshift(np.fft.fftshift(y_fft, axes=fft_axes)[slices],
                             axes=fft_axes)
    return (_ifftn(y_sub, axes=fft_axes) / (N_u / ckp_N) ** dim).real


def energy_spectrum(vel, mul_fac=1.0, is_scalar_field=False, dim=3):
    """utils.py:35-97 (rfftn over reversed axes; shells int(|k|+0.5))."""
    if dim == 2:
        vel = vel[:2, :, :, 0]
    ns = vel.shape[1:]
    assert all(n == ns[0] for n in ns)
    n = ns[0]
    if dim == 2:
        vel_hat = _rfftn(vel, axes=(2, 1))
    else:
        vel_hat = _rfftn(vel, axes=(3, 2, 1))
    Nf = n // 2 + 1
    k = np.fft.fftfreq(n, 1.0 / n)
    kx = k[:Nf].copy()
    kx[-1] *= -1
    if dim == 2:
        k_field = np.array(np.meshgrid(kx, k, indexing="ij"), dtype=int)
    else:
        k_field = np.array(np.meshgrid(kx, k, k, indexing="ij"), dtype=int)
    fact = (2 * (k_field[0] > 0) * (k_field[0] < n // 2)
            + 1 * (k_field[0] == 0) + 1 * (k_field[0] == n // 2))
    k_norm = np.linalg.norm(k_field, axis=0, ord=2)
    shell = (k_norm + 0.5).astype(int).flatten()
    vel_hat = vel_hat / n**dim
    abs_energy = np.sum(np.abs(vel_hat**2), axis=0) * fact * mul_fac
    n_samples = np.zeros(n)
    np.add.at(n_samples, shell, fact.flatten())
    ek = np.zeros(n)
    np.add.at(ek, shell, abs_energy.flatten())
    ek *= 4 * np.pi * np.arange(n) ** 2 / (n_samples + EPS)
    return ek


def comp_dissipation_rate(u_hat, nu):
    """utils.py:300-315: nu <|curl u|^2> from the spectral curl."""
    n = u_hat.shape[1]
    kkk, _, _, _ = wavenumbers(n, 3)
    curl = _irfftn(np.cross(1j * kkk, u_hat, axis=0), axes=(1, 2, 3))
    return nu * np.mean(np.sum(curl**2, axis=0))


def kinetic_energy(u):
    """0.5 mean(sum u^2) as logged at spectral_solver.py:318."""
    return 0.5 * float(np.mean(np.sum(u * u, axis=0)))


# ---------------------------------------------------------------------------------
# particles (l3es/integrator.py)
# ---------------------------------------------------------------------------------
def shift_fn(r, dr, box_size=2 * np.pi):
    """integrator.py:21-23 (Python modulo: result in [0, box))."""
    return np.mod(r + dr, box_size)


def interpolate_dft(u, r, chunk=2048):
    """Exact spectral interpolation of integrator.py:62-91.

    u: (3, c, c, c) or (2, c, c) real grid field; r: (Np, dim) positions.
    u_r[j] = real(mean_k(fftshift(fftn(u))(k) exp(i k.x_j))).
    """
    dim = u.shape[0] if u.ndim == 4 else 2
    dim = 3 if u.ndim == 4 else 2
    fft_axes = (1, 2, 3) if dim == 3 else (1, 2)
    c = u.shape[1]
    u_hat = np.fft.fftshift(_fftn(u, axes=fft_axes), axes=fft_axes)
    k = np.fft.fftshift(np.fft.fftfreq(c, 1.0 / c))
    ncomp = u.shape[0]
    out = np.empty((len(r), ncomp))
    # separable evaluation: exp(i k.x) = prod_d exp(i k_d x_d)
    for s in range(0, len(r), chunk):
        rr = r[s : s + chunk]
        ex = np.exp(1j * rr[:, 0, None] * k[None, :])
        ey = np.exp(1j * rr[:, 1, None] * k[None, :])
        if dim == 3:
            ez = np.exp(1j * rr[:, 2, None] * k[None, :])
            t = np.einsum("cabz,pz->cpab", u_hat, ez)
            t = np.einsum("cpab,pb->cpa", t, ey)
            val = np.einsum("cpa,pa->cp", t, ex)
        else:
            t = np.einsum("cab,pb->cpa", u_hat, ey)
            val = np.einsum("cpa,pa->cp", t, ex)
        out[s : s + chunk] = (val.real / c**dim).T
    return out


def advect_rk4(interp, r, dt, box_size=2 * np.pi):
    """Extension (no reference counterpart; the reference advances particles by one
    explicit Euler step with the post-step velocity, integrator.py:21-23 and
    combined.py:199): classical RK4 for dr/dt = u(r) with the velocity field held fixed
    at the post-step field. interp(r) -> velocities (Np, dim). Returns (u(r), r_new):
        v1 = u(r),  v2 = u(r + dt/2 v1),  v3 = u(r + dt/2 v2),  v4 = u(r + dt v3),
        r_new = (r + dt/6 (v1 + 2 v2 + 2 v3 + v4)) mod box
    (stage positions wrapped into the box as well)."""
    v1 = interp(r)
    v2 = interp(np.mod(r + 0.5 * dt * v1, box_size))
    v3 = interp(np.mod(r + 0.5 * dt * v2, box_size))
    v4 = interp(np.mod(r + dt * v3, box_size))
    return v1, np.mod(r + dt / 6.0 * (v1 + 2.0 * v2 + 2.0 * v3 + v4), box_size)


def interpolate_from_uhat_dft(u_hat, N, ckp_N, r, dim=3):
    """Combined-loop particle velocity (combined.py:122-130, dft backend)."""
    fft_axes = (1, 2, 3) if dim == 3 else (1, 2)
    u = _irfftn(u_hat, axes=fft_axes)
    if dim == 2:
        u = u[:2]
    u_lres = u if ckp_N == N else spectral_filtering(u, ckp_N)
    return interpolate_dft(u_lres, r)


def pos_init_cartesian(L, c, dim, jitter=0.0, seed=0):
    """Cell-centred particle lattice (stand-in for jax_sph pos_init_cartesian_*).

    One particle per cell of a c^dim lattice on [0, L)^dim, optionally jittered by
    ``jitter`` cell widths (uniform), wrapped into the box.
    """
    dx = L / c
    ax = (np.arange(c) + 0.5) * dx
    grids = np.meshgrid(*([ax] * dim), indexing="ij")
    r = np.stack([g.ravel() for g in grids], axis=1)
    if jitter:
        rng = np.random.default_rng(seed)
        r = r + rng.uniform(-jitter, jitter, size=r.shape) * dx
    return np.mod(r, L)


# ---------------------------------------------------------------------------------
# particle -> grid analysis (l3es/turbulence.py:299-339)
# ---------------------------------------------------------------------------------
def particles_to_grid_dft(r, u_r, n):
    """ur_to_u_dft_wrapper(N, L, dim): S(k) = sum_j u_r[j] exp(-i k.r_j) for k on the
    full n^dim grid (fftfreq order), u_grid = real(ifftn(S)); returns (dim, n, ..., n)."""
    dim = r.shape[1]
    k = np.fft.fftfreq(n, 1.0 / n)
    K = np.array(np.meshgrid(*([k] * dim), indexing="ij")).reshape(dim, -1)
    S = np.zeros((u_r.shape[1], K.shape[1]), dtype=np.complex128)
    for s in range(0, len(r), 4096):
        ph = np.exp(-1j * (r[s : s + 4096] @ K))  # (chunk, modes)
        S += u_r[s : s + 4096].T @ ph
    S = S.reshape((u_r.shape[1],) + (n,) * dim)
    return np.real(np.fft.ifftn(S, axes=tuple(range(1, dim + 1))))
