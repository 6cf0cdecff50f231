"""The SPH oracle (oracle/sph_ref.py) against golden vectors made by running the
reference's own relax.py (relax_wrapper: loop_body, sph_body) and utils.py
(rho_computer) with a stand-in for the absent jax_sph (tests/golden/make_golden_sph.py).
CPU only."""

import numpy as np
import pytest

from oracle import sph_ref as S

CASES = ["d2_n16", "d3_n8"]


def _case(gold, name):
    g = gold("sph")
    return {k.split("/", 1)[1]: v for k, v in g.items() if k.startswith(name + "/")}


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("name", CASES)
def test_density_matches_reference(gold, name):
    c = _case(gold, name)
    n, dim = int(c["n"]), int(c["dim"])
    assert _rel(S.density(c["r"], n, dim), c["rho"]) < 1e-13


@pytest.mark.parametrize("name", CASES)
def test_relax_acceleration_matches_reference(gold, name):
    c = _case(gold, name)
    n, dim, u_ref = int(c["n"]), int(c["dim"]), float(c["u_ref"])
    assert _rel(S.relax_acceleration(c["r"], n, dim, u_ref), c["acc_relax"]) < 1e-12


@pytest.mark.parametrize("name", CASES)
def test_sph_forces_match_reference(gold, name):
    c = _case(gold, name)
    n, dim, u_ref = int(c["n"]), int(c["dim"]), float(c["u_ref"])
    f = S.sph_forces(c["r"], c["u"], n, dim, u_ref)
    for k in ("acc_p", "acc_visc", "acc_tvf"):
        assert _rel(f[k], c[k]) < 1e-12, k
