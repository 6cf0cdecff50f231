"""Stand-in for the pieces of jax_sph 0.1.0 that l3es/relax.py and l3es/utils.py call.

TEST INFRASTRUCTURE ONLY: used by ``make_golden_sph.py`` to run the reference's own
relax.py (relax_wrapper: loop_body, sph_body) and utils.py (rho_computer) where jax_sph
(poetry.lock:832) is not installed. The kernel and equation of state come from the
oracle's restatement of their published definitions (oracle/sph_ref.py: the Morris et
al. quintic spline with cutoff 3h, the Tait EoS); the neighbour list is an O(n^2)
minimum-image scan that, like jax_sph's list with mask_self=False, includes every
particle itself. The golden vectors it yields pin the reference's own code on these
paths (pair forces, transport-velocity term, density sum, unit handling); the kernel
and EoS constants stay a restatement.
"""

from __future__ import annotations

import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", ".."))
from oracle import sph_ref as S  # noqa: E402


class QuinticKernel:
    def __init__(self, h, dim=3):
        self.h, self.dim = float(h), int(dim)
        self.cutoff = 3.0 * self.h

    def w(self, r):
        return S.quintic_w(np.asarray(r, dtype=np.float64), self.h, self.dim)

    def grad_w(self, r):
        return S.quintic_grad_w(np.asarray(r, dtype=np.float64), self.h, self.dim)


class TaitEoS:
    def __init__(self, p_ref, rho_ref, p_background, gamma):
        self.p_ref, self.rho_ref, self.p_bg, self.gamma = p_ref, rho_ref, p_background, gamma

    def p_fn(self, rho):
        return self.p_ref * ((rho / self.rho_ref) ** self.gamma - 1.0) + self.p_bg


class _Space:
    """jax_md.space subset: periodic displacement (minimum image) and distance."""

    @staticmethod
    def periodic(side):
        side = np.asarray(side, dtype=np.float64)

        def displacement(ra, rb):
            return np.mod(ra - rb + 0.5 * side, side) - 0.5 * side

        def shift(r, dr):
            return np.mod(r + dr, side)

        return displacement, shift

    @staticmethod
    def distance(dr):
        return np.sqrt(np.sum(np.asarray(dr) ** 2, axis=-1))


space = _Space()


class _Neighbors:
    def __init__(self, box, cutoff, mask_self, idx=None):
        self.box, self.cutoff, self.mask_self = np.asarray(box, dtype=np.float64), cutoff, mask_self
        self.idx = idx
        self.cell_list_capacity = 0

    def update(self, r, num_particles=None):
        r = np.asarray(r, dtype=np.float64)
        d = r[:, None, :] - r[None, :, :]
        d = np.mod(d + 0.5 * self.box, self.box) - 0.5 * self.box
        i, j = np.nonzero(np.sqrt(np.sum(d * d, axis=2)) < self.cutoff)
        if self.mask_self:
            keep = i != j
            i, j = i[keep], j[keep]
        return _Neighbors(self.box, self.cutoff, self.mask_self, (i, j))


def neighbor_list(displacement_fn, box_size, backend=None, r_cutoff=None, capacity_multiplier=None,
                  mask_self=True, num_particles_max=None, pbc=None):
    class _Fn:
        def allocate(self, r, num_particles=None):
            return _Neighbors(box_size, r_cutoff, mask_self).update(r)

        def update(self, r, nbrs, **kw):
            return nbrs.update(r)

    return _Fn()


def _lattice(box_size, dx, dim):
    n = [int(round(b / dx)) for b in np.asarray(box_size)[:dim]]
    axes = [(np.arange(k) + 0.5) * dx for k in n]
    return np.stack([g.ravel() for g in np.meshgrid(*axes, indexing="ij")], axis=1)


def pos_init_cartesian_2d(box_size, dx):
    return _lattice(box_size, dx, 2)


def pos_init_cartesian_3d(box_size, dx):
    return _lattice(box_size, dx, 3)


def install() -> None:
    """Replace the import stubs of jax_numpy_shim with this stand-in."""
    sys.modules["jax_sph.kernel"].QuinticKernel = QuinticKernel
    sys.modules["jax_sph.eos"].TaitEoS = TaitEoS
    sys.modules["jax_sph.jax_md"].space = space
    sys.modules["jax_sph.partition"].neighbor_list = neighbor_list
    sys.modules["jax_sph.utils"].pos_init_cartesian_2d = pos_init_cartesian_2d
    sys.modules["jax_sph.utils"].pos_init_cartesian_3d = pos_init_cartesian_3d
