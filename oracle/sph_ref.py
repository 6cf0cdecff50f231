"""FP64 NumPy restatement of the l3es SPH particle relaxation and density.

TEST INFRASTRUCTURE ONLY (oracle); never on the product path.

Follows l3es/relax.py:16-111 (relax_wrapper.loop_body), l3es/utils.py:169-218
(rho_computer) and the relaxation block of the combined loop (combined.py:132-142).
Those call jax_sph 0.1.0 (poetry.lock:832), which is neither vendored nor installed;
its pieces are restated from their published definitions:
  - QuinticKernel(h, dim): Morris et al. (1997) quintic spline with cutoff 3h,
    W(q) = sigma (max(0,3-q)^5 - 6 max(0,2-q)^5 + 15 max(0,1-q)^5), q = r/h,
    sigma = 1/(120 h), 7/(478 pi h^2), 3/(359 pi h^3) in 1, 2, 3 dimensions;
  - TaitEoS(p_ref, rho_ref, p_background, gamma): p = p_ref ((rho/rho_ref)^gamma - 1)
    + p_background;
  - neighbor_list(..., mask_self=False): every pair with distance below the cutoff,
    the particle itself included, periodic minimum-image displacements.
Parity: pinned to the reference's own relax.py and utils.rho_computer, run with a
stand-in for jax_sph whose kernel and EoS are the definitions above
(tests/golden/make_golden_sph.py; matched to 1e-12 by tests/test_sph_oracle.py).
jax_sph's own constants remain a restatement, checked for internal consistency
(symmetry, constant density on a lattice, momentum conservation).
"""

from __future__ import annotations

import numpy as np

EPS = float(np.finfo(np.float64).eps)

SIGMA = {1: lambda h: 1.0 / (120.0 * h), 2: lambda h: 7.0 / (478.0 * np.pi * h * h),
         3: lambda h: 3.0 / (359.0 * np.pi * h**3)}


def quintic_w(r, h, dim):
    q = r / h
    q1, q2, q3 = (np.maximum(0.0, a - q) for a in (1.0, 2.0, 3.0))
    return SIGMA[dim](h) * (q3**5 - 6.0 * q2**5 + 15.0 * q1**5)


def quintic_grad_w(r, h, dim):
    """dW/dr."""
    q = r / h
    q1, q2, q3 = (np.maximum(0.0, a - q) for a in (1.0, 2.0, 3.0))
    return SIGMA[dim](h) / h * (-5.0 * q3**4 + 30.0 * q2**4 - 75.0 * q1**4)


def _pairs(r, L, cutoff):
    """All (i, j, r_i - r_j wrapped) with |r_i - r_j| < cutoff, self pairs included."""
    from scipy.spatial import cKDTree

    tree = cKDTree(np.mod(r, L), boxsize=L)
    pairs = tree.query_pairs(cutoff, output_type="ndarray")
    n = len(r)
    i = np.concatenate([pairs[:, 0], pairs[:, 1], np.arange(n)])
    j = np.concatenate([pairs[:, 1], pairs[:, 0], np.arange(n)])
    d = periodic_displacement(r[i], r[j], L)
    return i, j, d


def density(r, N, dim, L=2 * np.pi):
    """rho_computer(N, dim, L)(r) (utils.py:169-218): mass sum_j W(|r_ij|)."""
    dx = L / N
    i, j, d = _pairs(r, L, 3.0 * dx)
    dist = np.sqrt(np.sum(d * d, axis=1))
    rho = np.zeros(len(r))
    np.add.at(rho, i, quintic_w(dist, dx, dim))
    return dx**dim * rho


def relax_acceleration(r, N, dim, u_ref, L=2 * np.pi):
    """relax_wrapper(N, dim, L, is_physical=True, u_ref).loop_body (relax.py:73-111):
    pressure (Tait, gamma 1, c = 10 u_ref) plus the transport-velocity term."""
    dx = L / N
    mass = dx**dim
    p_eos = (10.0 * u_ref) ** 2
    i, j, d = _pairs(r, L, 3.0 * dx)
    dist = np.sqrt(np.sum(d * d, axis=1))
    rho = np.zeros(len(r))
    np.add.at(rho, i, mass * quintic_w(dist, dx, dim))
    p = p_eos * (rho - 1.0)
    e = d / (dist[:, None] + EPS)
    grad = quintic_grad_w(dist, dx, dim)[:, None] * e
    ri, rj, pi, pj = rho[i], rho[j], p[i], p[j]
    p_ij = (rj * pi + ri * pj) / (ri + rj)
    pref = mass * ((1.0 / ri) ** 2 + (1.0 / rj) ** 2)
    acc = (-pref * p_ij)[:, None] * grad + (0.5 * pref * (-p_eos))[:, None] * grad
    out = np.zeros_like(r)
    np.add.at(out, i, acc)
    return out


def sph_forces(r, u, N, dim, u_ref, L=2 * np.pi):
    """relax_wrapper(...).sph_body(r, u) (relax.py:122-176): pressure, viscous (eta 1)
    and transport-velocity accelerations."""
    dx = L / N
    mass = dx**dim
    p_eos = (10.0 * u_ref) ** 2
    i, j, d = _pairs(r, L, 3.0 * dx)
    dist = np.sqrt(np.sum(d * d, axis=1))
    rho = np.zeros(len(r))
    np.add.at(rho, i, mass * quintic_w(dist, dx, dim))
    p = p_eos * (rho - 1.0)
    dw = quintic_grad_w(dist, dx, dim)
    grad = dw[:, None] * d / (dist[:, None] + EPS)
    ri, rj, pi, pj = rho[i], rho[j], p[i], p[j]
    p_ij = (rj * pi + ri * pj) / (ri + rj)
    pref = mass * ((1.0 / ri) ** 2 + (1.0 / rj) ** 2)
    out = {k: np.zeros_like(r) for k in ("acc_p", "acc_visc", "acc_tvf")}
    np.add.at(out["acc_p"], i, (-pref * p_ij)[:, None] * grad)
    np.add.at(out["acc_visc"], i, (pref / (dist + EPS) * dw)[:, None] * (u[i] - u[j]))
    np.add.at(out["acc_tvf"], i, (pref * (-p_eos))[:, None] * grad)
    return out


def periodic_displacement(a, b, L):
    """jax_md space.periodic displacement: mod(a - b + L/2, L) - L/2."""
    return np.mod(a - b + 0.5 * L, L) - 0.5 * L


def relax_velocity(r0, u_r, dt, relax_dt_factor, N, dim, u_ref, L=2 * np.pi):
    """combined.py:132-142: move to the next positions, one relaxation kick, and the
    velocity that reaches the relaxed positions in one step (minimum image)."""
    r_temp = np.mod(r0 + dt * u_r, L)
    a = relax_acceleration(r_temp, N, dim, u_ref, L)
    r_temp = np.mod(r_temp + (relax_dt_factor * dt) ** 2 * a, L)
    return periodic_displacement(r_temp, r0, L) / dt


def pairs_bruteforce(r, L, cutoff):
    """Every ordered pair (self included) within the cutoff by an O(n^2) minimum-image
    scan; an independent check of the tree search above on small inputs."""
    d = r[:, None, :] - r[None, :, :]
    d -= L * np.round(d / L)
    dist = np.sqrt(np.sum(d * d, axis=2))
    i, j = np.nonzero(dist < cutoff)
    return i, j, d[i, j]
