"""Golden vectors of the SPH relaxation and density from the reference's own source.

Run here (not on the GPU machine, where the reference is absent):
    python tests/golden/make_golden_sph.py <path of the reference checkout>

Runs l3es/relax.py (relax_wrapper(N, dim, L, is_physical=True, u_ref): loop_body and
sph_body, as l3es/integrator.py:112 builds them) and l3es/utils.py (rho_computer) as
written, on NumPy through ``jax_numpy_shim`` with ``jax_sph_standin`` in place of the
absent jax_sph (kernel and EoS from the oracle's restatement of their published
definitions). Inputs: jittered lattices, 2D 16^2 and 3D 8^3 (u_ref 4), seeded.
Output: ``tests/golden/sph.npz``.
"""

from __future__ import annotations

import importlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _jittered(n, dim, seed, jitter=0.35, L=2 * np.pi):
    rng = np.random.default_rng(seed)
    dx = L / n
    axes = [(np.arange(n) + 0.5) * dx] * dim
    r = np.stack([g.ravel() for g in np.meshgrid(*axes, indexing="ij")], axis=1)
    return np.mod(r + rng.uniform(-jitter, jitter, r.shape) * dx, L)


def main(ref_root: str) -> None:
    sys.path.insert(0, HERE)
    import jax_numpy_shim
    import jax_sph_standin

    jax_numpy_shim.install()
    jax_sph_standin.install()
    sys.path.insert(0, ref_root)
    rx = importlib.import_module("l3es.relax")
    ut = importlib.import_module("l3es.utils")
    out = {}
    for n, dim, seed in ((16, 2, 3), (8, 3, 4)):
        u_ref = 4.0
        r = _jittered(n, dim, seed)
        u = np.random.default_rng(seed + 100).standard_normal(r.shape)
        loop_body, sph_body = rx.relax_wrapper(n, dim, 2 * np.pi, is_physical=True, u_ref=u_ref)
        rho = np.asarray(ut.rho_computer(n, dim, 2 * np.pi)(r))
        acc = np.asarray(loop_body(r))
        f = sph_body(r, u)
        out[f"d{dim}_n{n}"] = dict(n=n, dim=dim, u_ref=u_ref, r=r, u=u, rho=rho, acc_relax=acc,
                                   acc_p=np.asarray(f["acc_p"]), acc_visc=np.asarray(f["acc_visc"]),
                                   acc_tvf=np.asarray(f["acc_tvf"]))
        print(f"{dim}D n={n}: rho [{rho.min():.4f}, {rho.max():.4f}], |acc| max {np.abs(acc).max():.3e}")
    flat = {f"{case}/{k}": np.asarray(v) for case, d in out.items() for k, v in d.items()}
    np.savez_compressed(os.path.join(HERE, "sph.npz"), **flat)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden_sph.py <path of the reference checkout>")
    main(sys.argv[1])
