"""SPH density and relaxation on the GPU vs the FP64 oracle (oracle/sph_ref.py).

Pair geometry runs in FP32 from cell-local coordinates and the neighbour sums in FP64,
so densities agree to 1e-6 and accelerations to 1e-4 of their largest magnitude.
Cases cover the one-cell minimum-image search (n < 9), the smallest cell grid (n = 9:
three cells per axis, every stencil cell distinct), 2D and 3D.
"""

import numpy as np
import pytest

from oracle import numpy_ref as R
from oracle import sph_ref as S

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

L = 2 * np.pi
RHO_TOL = 1e-6
ACC_TOL = 1e-4
CASES = [(16, 3), (9, 3), (8, 3), (32, 2), (6, 2)]


def _r(n, dim, jitter=0.35, seed=0):
    return R.pos_init_cartesian(L, n, dim, jitter=jitter, seed=seed)


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def _rel(a, b):
    a = a.cpu().numpy() if hasattr(a, "cpu") else a
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("n,dim", CASES)
def test_density_matches_oracle(n, dim):
    from l3es import _native

    r = _r(n, dim)
    p = _native.SphPlan(dim, n)
    rho = torch.empty(r.shape[0], dtype=torch.float64, device="cuda")
    p.density(_dev(r), rho)
    ref = S.density(r, n, dim)
    assert np.abs(rho.cpu().numpy() - ref).max() < RHO_TOL


@pytest.mark.parametrize("n,dim", CASES)
def test_relax_acceleration_matches_oracle(n, dim):
    from l3es import _native

    r = _r(n, dim, seed=1)
    p = _native.SphPlan(dim, n)
    acc = torch.empty(r.shape, dtype=torch.float64, device="cuda")
    p.relax_acceleration(_dev(r), acc, 4.0)
    assert _rel(acc, S.relax_acceleration(r, n, dim, 4.0)) < ACC_TOL


@pytest.mark.parametrize("n,dim", [(16, 3), (32, 2)])
def test_sph_forces_match_oracle(n, dim):
    from l3es.relax import relax_wrapper

    r = _r(n, dim, seed=2)
    u = 4.0 * np.random.default_rng(5).standard_normal(r.shape)
    loop_body, sph_body = relax_wrapper(n, dim, L, is_physical=True, u_ref=4.0)
    got = sph_body(r, u)
    ref = S.sph_forces(r, u, n, dim, 4.0)
    for k in ("acc_p", "acc_visc", "acc_tvf"):
        assert _rel(got[k], ref[k]) < ACC_TOL, k
    # the non-dimensional mode returns the same physical acceleration
    nd, _ = relax_wrapper(n, dim, L, is_physical=False, u_ref=4.0)
    assert _rel(nd(r), S.relax_acceleration(r, n, dim, 4.0)) < ACC_TOL


@pytest.mark.parametrize("n,dim", [(32, 3), (64, 2), (8, 3)])
def test_relax_velocity_matches_oracle(n, dim):
    """combined.py:132-142 with the hit32 settings (u_ref 4, dt 2e-3, factor 2)."""
    from l3es import _native

    dt, f, u_ref = 2e-3, 2.0, 4.0
    r0 = _r(n, dim, jitter=0.25, seed=3)
    u_r = u_ref * np.random.default_rng(4).standard_normal(r0.shape)
    p = _native.SphPlan(dim, n)
    u_out = torch.empty(r0.shape, dtype=torch.float64, device="cuda")
    r_out = torch.empty_like(u_out)
    p.relax_velocity(_dev(r0), _dev(u_r), u_out, dt, f, u_ref, r_out=r_out)
    ref = S.relax_velocity(r0, u_r, dt, f, n, dim, u_ref)
    got = u_out.cpu().numpy()
    # the relaxation kick itself, (f dt)^2 a / dt, to 1e-4 of its largest value
    assert np.abs((got - u_r) - (ref - u_r)).max() < ACC_TOL * np.abs(ref - u_r).max()
    assert np.abs(r_out.cpu().numpy() - np.mod(r0 + dt * got, L)).max() < 1e-13


def test_results_do_not_depend_on_launch_or_order():
    from l3es import _native

    n, dim = 16, 3
    r = _r(n, dim, seed=6)
    p = _native.SphPlan(dim, n)
    a1 = torch.empty(r.shape, dtype=torch.float64, device="cuda")
    a2 = torch.empty_like(a1)
    p.relax_acceleration(_dev(r), a1, 4.0)
    p.relax_acceleration(_dev(r), a2, 4.0)
    assert torch.equal(a1, a2)
    perm = np.random.default_rng(7).permutation(r.shape[0])
    a3 = torch.empty_like(a1)
    p.relax_acceleration(_dev(r[perm]), a3, 4.0)
    assert _rel(a3, a1.cpu().numpy()[perm]) < 1e-5
    # positions outside the box are wrapped first
    a4 = torch.empty_like(a1)
    p.relax_acceleration(_dev(r + L * np.array([1.0, -2.0, 3.0])), a4, 4.0)
    assert _rel(a4, a1.cpu().numpy()) < 1e-5


def test_argument_checks():
    from l3es import _native

    p = _native.SphPlan(2, 8)
    r = _dev(_r(8, 2))
    big = _dev(np.zeros((65, 2)))
    with pytest.raises(RuntimeError, match="np_max"):
        p.density(big, torch.empty(65, dtype=torch.float64, device="cuda"))
    with pytest.raises(RuntimeError, match="alias"):
        p.relax_velocity(r, r.clone(), r, 1e-3, 2.0, 1.0)
    empty = torch.empty((0, 2), dtype=torch.float64, device="cuda")
    p.relax_acceleration(empty, torch.empty_like(empty), 1.0)


def test_rho_computer_and_set_up_integrator():
    from l3es import integrator as I
    from l3es.utils import rho_computer

    r, comp_rho, interp, relax_fn, sph_fn, Lb, axes = I.set_up_integrator(None, 2, 16, 4, 1.0, "dft")
    assert callable(comp_rho) and callable(relax_fn) and callable(sph_fn)
    rho = comp_rho(r)
    np.testing.assert_allclose(rho.cpu().numpy(), S.density(r.cpu().numpy(), 16, 2), atol=RHO_TOL)
    # lattice: no net force (the pair terms are ~1e2 here and cancel to FP32 rounding)
    assert np.abs(relax_fn(r).cpu().numpy()).max() < 1e-3
    rr = _r(12, 3, seed=8)
    np.testing.assert_allclose(rho_computer(12, 3)(rr).cpu().numpy(), S.density(rr, 12, 3), atol=RHO_TOL)


def test_combined_with_relaxation_matches_oracle_loop(tmp_path):
    """combined() with relax_dt_factor 2 on a 2D case (64^2 DNS, 16^2 particles, dft)
    vs the oracle loop: step, coarsen, interpolate, relax at the predicted positions,
    advect with the relaxed velocity; checkpoints hold the unrelaxed velocity."""
    from l3es import combined as C

    n, c, dt, nu, steps, u_ref, f = 64, 16, 1e-3, 1e-3, 3, 1.0, 2.0
    u, uh, r = C.combined("Kolm", N=n, dim=2, nu=nu, t_final=steps * dt, dt=dt, ckp_N=c, interp_backend="dft",
                          relax_dt_factor=f, u_ref=u_ref, log_freq=1, ckp_freq=1, dst_path=str(tmp_path), seed=3)
    u_o, uh_o, dx, fn, *_ = R.set_up_solver(n, nu, 2, "Kolm", dt, 3, c, None, None, "none")
    r_o = R.pos_init_cartesian(L, c, 2)
    rows = open(tmp_path / "diagnostics.csv").read().splitlines()
    for i in range(steps + 1):
        u_o, uh_o, _ = fn(u_o, uh_o)
        ur = R.interpolate_dft(R.spectral_filtering(u_o[:2, :, :, 0], c), r_o)
        last = np.load(tmp_path / "com" / f"step_{i:05d}.npz")
        assert _rel(last["u"], ur) < 5e-5
        assert np.abs(last["r"] - r_o).max() < 1e-6
        rho_max = float(rows[1 + i].split(",")[-1])
        assert abs(rho_max - S.density(r_o, c, 2).max()) < 1e-6
        u_rel = S.relax_velocity(r_o, ur, dt, f, c, 2, u_ref)
        r_o = R.shift_fn(r_o, dt * u_rel)
    assert np.abs(r.cpu().numpy() - r_o).max() < 1e-6


@pytest.mark.parametrize("name", ["d2_n16", "d3_n8"])
def test_sph_matches_reference_golden(gold, name):
    """Density, relaxation acceleration and the three sph_body terms against the
    reference's own relax.py / utils.py run with a jax_sph stand-in
    (tests/golden/make_golden_sph.py)."""
    from l3es import _native
    from l3es.relax import relax_wrapper

    c = {k.split("/", 1)[1]: v for k, v in gold("sph").items() if k.startswith(name + "/")}
    n, dim, u_ref = int(c["n"]), int(c["dim"]), float(c["u_ref"])
    r, u = c["r"], c["u"]
    p = _native.SphPlan(dim, n)
    rho = torch.empty(r.shape[0], dtype=torch.float64, device="cuda")
    p.density(_dev(r), rho)
    assert np.abs(rho.cpu().numpy() - c["rho"]).max() < RHO_TOL
    acc = torch.empty(r.shape, dtype=torch.float64, device="cuda")
    p.relax_acceleration(_dev(r), acc, u_ref)
    assert _rel(acc, c["acc_relax"]) < ACC_TOL
    _, sph_body = relax_wrapper(n, dim, L, is_physical=True, u_ref=u_ref)
    got = sph_body(r, u)
    for k in ("acc_p", "acc_visc", "acc_tvf"):
        assert _rel(got[k], c[k]) < ACC_TOL, k
