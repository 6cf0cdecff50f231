"""Initial velocity fields and the HIT forcing band (drop-in for l3es/init_fields.py).

Initial conditions are host-side set-up, computed in FP64 NumPy as in the reference
(the random phases must come from NumPy's legacy generator to be bit-identical);
the solver moves them to the GPU once. Returned arrays are NumPy float64.
"""

from __future__ import annotations

import numpy as np

EPS = float(np.finfo(np.float64).eps)


def init_u_tgv(x, y, z):
    """Taylor-Green vortex u = (sin x cos y cos z, -cos x sin y cos z, 0)
    (init_fields.py:12-16)."""
    x, y, z = (np.asarray(a) for a in (x, y, z))
    cz = np.cos(z)
    return np.stack([np.sin(x) * np.cos(y) * cz, -np.cos(x) * np.sin(y) * cz, 0.0 * x])


def init_u_tgv2d(Nx, target_dim=2, rescale=1.0):
    """Cell-centred 2D TGV (init_fields.py:19-30): u = -cos X sin Y, v = sin X cos Y on
    a meshgrid in 'xy' order (X varies along the second axis), times `rescale`."""
    L = float(rescale)
    c = (np.arange(Nx) + 0.5) * (L / Nx)
    X, Y = np.meshgrid(c, c)
    u = np.stack([-np.cos(X) * np.sin(Y), np.sin(X) * np.cos(Y)])
    if target_dim == 3:
        u = np.concatenate([u[..., None], np.zeros((1, Nx, Nx, 1))], axis=0)
    return u * L


def _spectrum_table(nmax, spectrum, kp):
    k = np.arange(nmax + 1, dtype=np.float64)
    e = np.full(nmax + 1, EPS)
    kk = k[1:]
    if spectrum == "k-5/3":
        e[1:] = kk ** (-5.0 / 3.0) / (4.0 * np.pi * kk**2)
    elif spectrum == "k4exp":
        e[1:] = kk**2 * np.exp(-2.0 * (kk / kp) ** 2) / (4.0 * np.pi)
    else:
        raise ValueError(f"spectrum must be 'k-5/3' or 'k4exp', got {spectrum!r}")
    return e


def hit_spectrum(N, seed=42, spectrum="k-5/3", kp=4.0):
    """Rogallo random-phase solenoidal half spectrum, shape (3, N//2+1, N, N).

    Same construction as init_fields.py:33-106: amplitude sqrt(E(round|k|)), phases
    2 pi * np.random.random((N//2+1, N, N, 3)) after np.random.seed(seed), drawn in
    the loop order k1 = 0..N/2, k2 = -N/2..N/2-1, k3 = -N/2..N/2-1; the k1 = 0 plane
    made conjugate-symmetric for |k2|, |k3| != N/2. Axis 1 is the half axis.
    ``spectrum='k4exp'`` replaces E(k) = k^-5/3 / (4 pi k^2) with k^4 exp(-2 (k/kp)^2)
    / (4 pi k^2) (extension, same phases).
    """
    rs = np.random.RandomState(seed)
    h = N // 2 + 1
    nmax = int(round(np.sqrt(3.0 * N * N) / 2.0))
    table = _spectrum_table(nmax, spectrum, kp)
    phase = 2.0 * np.pi * rs.random_sample((h, N, N, 3))
    # loop order -> FFT order on the two full axes: loop index j holds k = j - N/2,
    # whose FFT index is (j - N/2) mod N, i.e. a roll by N/2
    phase = np.roll(phase, -(N // 2), axis=(1, 2))
    k1 = np.arange(h, dtype=np.float64)[:, None, None]
    kf = np.fft.fftfreq(N, 1.0 / N)
    k2 = kf[None, :, None]
    k3 = kf[None, None, :]
    kmag = np.sqrt(k1 * k1 + k2 * k2 + k3 * k3)
    k12 = np.sqrt(k1 * k1 + k2 * k2)
    amp = np.sqrt(table[np.clip(np.round(kmag).astype(np.int64), 0, nmax)])
    a = amp * np.exp(1j * phase[..., 0]) * np.cos(phase[..., 2])
    b = amp * np.exp(1j * phase[..., 1]) * np.sin(phase[..., 2])
    del phase
    denom = np.where(kmag == 0, 1.0, kmag) * np.where(k12 == 0, 1.0, k12)
    on_axis = k12 == 0
    ux = np.where(on_axis, a, (a * kmag * k2 + b * k1 * k3) / denom)
    uy = np.where(on_axis, b, (b * k2 * k3 - a * kmag * k1) / denom)
    uz = -b * k12 / np.where(kmag == 0, 1.0, kmag)
    spec = np.stack([ux, uy, uz])
    spec[:, 0, 0, 0] = 0.0
    # Hermitian symmetry on the k1 = 0 plane: S(j, k) = conj S(-j, -k) for the
    # targets k in (N/2, N) (j != N/2) and (j in (N/2, N), k = 0)
    p = spec[:, 0]
    jj = np.arange(N)
    neg = (N - jj) % N
    hi = jj > N // 2
    mid = jj != N // 2
    tgt = (mid[:, None] & hi[None, :]) | (hi[:, None] & (jj == 0)[None, :])
    src = np.conj(p[:, neg][:, :, neg])
    p[:, tgt] = src[:, tgt]
    return spec


def init_u_hit(N, seed=42, spectrum="k-5/3", kp=4.0):
    """Real HIT field (3, N, N, N) in FP64 (init_fields.py:33-106): the unnormalised
    inverse real FFT (norm='forward') of :func:`hit_spectrum`, half axis first."""
    spec = hit_spectrum(N, seed, spectrum, kp)
    return np.fft.irfftn(spec, s=(N, N, N), axes=(2, 3, 1), norm="forward")


def init_forcing_mask_hit(N, kf=3):
    """Forcing band 0 < |k|^2 <= kf^2 on the rfftn half spectrum (init_fields.py:167-188),
    with the half-axis Nyquist wavenumber counted as +N/2."""
    k = np.fft.fftfreq(N, 1.0 / N)
    kh = np.abs(k[: N // 2 + 1])
    k2 = k[:, None, None] ** 2 + k[None, :, None] ** 2 + kh[None, None, :] ** 2
    return (k2 > 0) & (k2 <= kf * kf)


def init_u_random2d(N, seed=0, kmax=8.0, energy=0.5, target_dim=3):
    """Band-limited random-phase 2D initial field (extension, no reference counterpart).

    Stream function with unit amplitude and uniform random phase
    (``np.random.default_rng(seed)``) on 0 < |k| <= kmax; u = d psi / dy,
    v = -d psi / dx; rescaled to kinetic energy `energy`. Layout (3, N, N, 1).
    """
    rng = np.random.default_rng(seed)
    kx = np.fft.fftfreq(N, 1.0 / N)[:, None]
    ky = np.arange(N // 2 + 1, dtype=np.float64)[None, :]
    kk = np.sqrt(kx * kx + ky * ky)
    phase = rng.uniform(0.0, 2.0 * np.pi, size=kk.shape)
    psi = np.where((kk > 0) & (kk <= kmax), np.exp(1j * phase), 0.0)
    uv = np.stack([np.fft.irfftn(1j * ky * psi, s=(N, N), axes=(0, 1)),
                   np.fft.irfftn(-1j * kx * psi, s=(N, N), axes=(0, 1))])
    uv *= np.sqrt(energy / (0.5 * np.mean(np.sum(uv * uv, axis=0))))
    if target_dim == 3:
        uv = np.concatenate([uv[..., None], np.zeros((1, N, N, 1))], axis=0)
    return uv


def _spectral_filter_np(u, c):
    """spectral_filtering (utils.py:100-138) of (ncomp, G, G) in FP64: full FFT, keep the
    shifted modes [G/2 - c/2, G/2 + c/2) of each axis (k in [-c/2, c/2-1]), inverse FFT
    on the c grid divided by (G/c)^2, real part."""
    G = u.shape[-1]
    uh = np.fft.fftshift(np.fft.fftn(u, axes=(1, 2)), axes=(1, 2))
    sl = slice(G // 2 - c // 2, G // 2 + c // 2)
    uh = np.fft.ifftshift(uh[:, sl, sl], axes=(1, 2))
    return np.fft.ifftn(uh, axes=(1, 2)).real / (G / c) ** 2


def _lognormal_density(k, peak):
    """Log-normal radial spectral filter exp(-(ln k - ln peak)^2 / 2) / k (the 1/k spreads
    the 2D shell area so the shell energy, not the mode amplitude, is log-normal); 0 at k=0."""
    with np.errstate(divide="ignore", invalid="ignore"):
        d = np.exp(-0.5 * (np.log(k) - np.log(peak)) ** 2) / k
    return np.where(k > 0, d, 0.0)


def init_u_kolm(N, L=2 * np.pi, max_velocity=4.2, seed=42, target_dim=3, iter=4, grid_n=2048,
                peak_wavenumber=4.0):
    """Kolmogorov-flow initial field (drop-in for init_fields.py:191-212).

    The reference builds it with JAX-CFD's filtered_velocity_field on a 2048^2 grid of
    side L and coarsens it to N x N with spectral_filtering. Restated here in FP64 NumPy
    (JAX-CFD and JAX's random generator are not available, so values are seeded by
    ``np.random.default_rng(seed)`` instead and do not match the reference bit for bit):
      1. white Gaussian noise for each of the 2 velocity components on grid_n^2 points;
      2. radial spectral filter with a log-normal density peaked at `peak_wavenumber`
         (wavenumbers in cycles per unit length, the grid's fftfreq(grid_n, L/grid_n));
      3. `iter` times: divergence-free (Leray) projection, then scaling so that the
         largest pointwise speed equals `max_velocity`;
      4. keep the modes k in [-N/2, N/2-1] of each axis and transform back on the N^2
         grid, i.e. spectral_filtering (utils.py:100-138), values unchanged in scale.
    Returns (2, N, N, 1), or (3, N, N, 1) with a zero third component for target_dim 3.
    """
    G = int(grid_n)
    if G % N:
        raise ValueError(f"grid_n={G} must be a multiple of N={N}")
    rng = np.random.default_rng(seed)
    noise = rng.standard_normal((2, G, G))
    f = np.fft.fftfreq(G, L / G)                      # cycles per unit length
    fh = np.fft.rfftfreq(G, L / G)
    kabs = np.sqrt(f[:, None] ** 2 + fh[None, :] ** 2)
    dens = _lognormal_density(kabs, peak_wavenumber)
    dens[G // 2, :] = 0.0  # Nyquist row and column: no consistent projection there
    dens[:, G // 2] = 0.0
    vh = np.fft.rfftn(noise, axes=(1, 2)) * dens
    kx = f[:, None] + 0.0 * fh[None, :]
    ky = 0.0 * f[:, None] + fh[None, :]
    k2 = kabs * kabs
    inv_k2 = np.where(k2 > 0, 1.0 / np.where(k2 > 0, k2, 1.0), 0.0)
    for _ in range(max(1, int(iter))):
        div = kx * vh[0] + ky * vh[1]                 # projection: v - k (k . v) / |k|^2
        vh = np.stack([vh[0] - kx * div * inv_k2, vh[1] - ky * div * inv_k2])
        v = np.fft.irfftn(vh, s=(G, G), axes=(1, 2))
        vh *= max_velocity / np.sqrt((v * v).sum(0)).max()
    v0 = _spectral_filter_np(np.fft.irfftn(vh, s=(G, G), axes=(1, 2)), N)[..., None]
    if target_dim == 3:
        v0 = np.concatenate([v0, np.zeros((1, N, N, 1))], axis=0)
    return v0

