"""FP64 NumPy restatement of the type-2 NUFFT used by the l3es particle layer.

TEST INFRASTRUCTURE ONLY (the oracle and the CPU baseline); never on the product path.

The reference calls ``finufft.nufft3d2`` / ``nufft2d2`` (finufft 2.5.0, pinned at
poetry.lock:502; call sites l3es/integrator.py:53 and :55, isign=+1, default
tolerance). finufft is not vendored and not installed here, so its published
algorithm (Barnett, Magland, af Klinteberg, SIAM J. Sci. Comput. 41 (2019)) is
restated: exponential-of-semicircle (ES) kernel
    phi(z) = exp(beta (sqrt(1 - z^2) - 1)),  |z| <= 1,  beta = 2.30 w,
upsampling sigma = 2 (fine grid n = 2c), deconvolution by the kernel's Fourier
transform (Gauss-Legendre quadrature), inverse FFT on the fine grid, and a
w-point tensor-product gather per target. The exact sum it approximates is the
in-repo DFT backend (integrator.py:62-91), which is the parity anchor.
"""

from __future__ import annotations

import numpy as np


def es_beta(w: int) -> float:
    return 2.30 * w


def es_kernel(z, w: int):
    """phi(z) on |z| <= 1 (0 outside)."""
    beta = es_beta(w)
    z = np.asarray(z, dtype=np.float64)
    out = np.zeros_like(z)
    m = np.abs(z) <= 1.0
    out[m] = np.exp(beta * (np.sqrt(1.0 - z[m] ** 2) - 1.0))
    return out


def es_fourier(k, w: int, n: int, nquad: int = 100):
    """psi_hat_k = (1/2pi) int psi(x) e^{-ikx} dx for psi(x) = phi(x / (w h / 2)),

    h = 2 pi / n; equals (w / (2 n)) int_{-1}^{1} phi(z) cos(pi k z w / n) dz.
    """
    zq, wq = np.polynomial.legendre.leggauss(nquad)
    phi = es_kernel(zq, w)
    k = np.asarray(k, dtype=np.float64)
    return (w / (2.0 * n)) * np.sum(
        wq[None, :] * phi[None, :] * np.cos(np.pi * k[:, None] * zq[None, :] * w / n),
        axis=1,
    )


def nufft2(coeff_shifted, r, w: int = 6, sigma: int = 2, isign: int = 1):
    """Type-2 NUFFT: f_j = sum_k F_k exp(isign i k.x_j) for fftshift-ordered F.

    coeff_shifted: (ncomp, c, ..., c) complex, axis order (x, y[, z]), modes
    k = -c/2 .. c/2-1 along each axis; r: (Np, dim) in [0, 2 pi).
    Returns complex (ncomp, Np).
    """
    ncomp = coeff_shifted.shape[0]
    dim = coeff_shifted.ndim - 1
    c = coeff_shifted.shape[1]
    n = sigma * c
    k1 = np.arange(-c // 2, c // 2)
    psi = es_fourier(k1, w, n)
    # deconvolve and zero-pad onto the fine grid (modes at k mod n)
    G = np.zeros((ncomp,) + (n,) * dim, dtype=np.complex128)
    dec = coeff_shifted.astype(np.complex128)
    for d in range(dim):
        shape = [1] * (dim + 1)
        shape[d + 1] = c
        dec = dec / psi.reshape(shape)
    idx = np.mod(k1, n)
    G[np.ix_(range(ncomp), *([idx] * dim))] = dec
    # g_l = sum_k G_k exp(isign i 2 pi k l / n): unnormalised inverse (isign=+1)
    axes = tuple(range(1, dim + 1))
    if isign > 0:
        g = np.fft.ifftn(G, axes=axes) * float(n) ** dim
    else:
        g = np.fft.fftn(G, axes=axes)
    h = 2 * np.pi / n
    Np = r.shape[0]
    # per-dimension kernel weights and wrapped indices
    ws, ids = [], []
    for d in range(dim):
        x = r[:, d] / h
        l0 = np.ceil(x - w / 2.0).astype(np.int64)
        ll = l0[:, None] + np.arange(w)[None, :]
        z = (x[:, None] - ll) / (w / 2.0)
        ws.append(es_kernel(z, w))
        ids.append(np.mod(ll, n))
    out = np.zeros((ncomp, Np), dtype=np.complex128)
    if dim == 3:
        for a in range(w):
            for b in range(w):
                wab = ws[0][:, a] * ws[1][:, b]
                ia, ib = ids[0][:, a], ids[1][:, b]
                for cc in range(w):
                    out += g[:, ia, ib, ids[2][:, cc]] * (wab * ws[2][:, cc])[None, :]
    else:
        for a in range(w):
            for b in range(w):
                out += g[:, ids[0][:, a], ids[1][:, b]] * (ws[0][:, a] * ws[1][:, b])[None, :]
    return out / float(n) ** dim


def interpolate_nufft(u, r, w: int = 6):
    """integrator.py:36-60 with the finufft call replaced by :func:`nufft2`."""
    dim = 3 if u.ndim == 4 else 2
    axes = (1, 2, 3) if dim == 3 else (1, 2)
    c = u.shape[1]
    u_hat = np.fft.fftshift(np.fft.fftn(u, axes=axes), axes=axes)
    vals = nufft2(u_hat, r, w=w, isign=1)
    return np.real(vals).T / float(c) ** dim
