"""Batched trajectories and CUDA-graph replay on the GPU.

A plan with batch > 1 steps several same-size trajectories in one launch per kernel
(per-trajectory viscosity and ekin_tot target); it must give each trajectory the
result of its own single plan. A graph recorded from library calls must replay to
the same bits as the calls run directly.
"""

import numpy as np
import pytest

from oracle import numpy_ref as R

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _fields(dim, n, count, seed):
    out = []
    for b in range(count):
        if dim == 3:
            u = R.init_u_hit(n, seed + b, "k4exp", 3.0)
            u *= np.sqrt(0.5 / R.kinetic_energy(u))
        else:
            u = R.init_u_random2d(n, seed + b)
        out.append(u)
    return out


def _spec(plan_cls, dim, n, u):
    p = plan_cls(dim=dim, n=n, nu=0.01, dt=1e-3)
    uh = torch.empty(p.spec_shape, dtype=torch.complex64, device="cuda")
    p.rfftn(torch.from_numpy(np.ascontiguousarray(u, dtype=np.float32)).cuda(), uh)
    return uh


@pytest.mark.parametrize("dim,n,forcing,line", [(3, 32, "ekin_tot", None), (3, 32, "const_power", None),
                                                 (2, 64, "none", None), (2, 256, "none", 2), (2, 256, "none", 3)])
def test_batched_plan_matches_single_plans(dim, n, forcing, line):
    """A batched plan equals one plan per trajectory; at 256 also with the radix-16 line
    passes (line 2, and 3 fed by bulk copies: the trajectory index enters its copy
    addresses)."""
    from l3es import _native

    count, dt, steps = 3, 2e-3, 3
    nus = [4e-3, 8e-3, 1.2e-2]
    us = _fields(dim, n, count, 11)
    e0s = [R.kinetic_energy(u) for u in us]
    kw = dict(forcing=forcing, kf=2 if forcing != "none" else 0, eps_inj=0.1)
    singles = []
    for b in range(count):
        p = _native.Plan(dim=dim, n=n, nu=nus[b], dt=dt, e_kin_init=e0s[b], **kw)
        if line is not None:
            p.set_schedule({"line_pair": line})
        uh = _spec(_native.Plan, dim, n, us[b])
        p.step(uh, steps)
        singles.append(uh.cpu().numpy())
    pb = _native.Plan(dim=dim, n=n, nu=0.0, dt=dt, batch=count, **kw)
    if line is not None:
        pb.set_schedule({"line_pair": line})
    pb.set_nu(nus)
    pb.set_e0(e0s)
    uhb = torch.stack([_spec(_native.Plan, dim, n, u) for u in us]).contiguous()
    einj = torch.zeros(steps * count, dtype=torch.float64, device="cuda")
    pb.step(uhb, steps, e_inj=einj)
    got = uhb.cpu().numpy()
    for b in range(count):
        assert np.array_equal(got[b], singles[b]) or \
            np.abs(got[b] - singles[b]).max() <= 1e-6 * np.abs(singles[b]).max()
    if forcing == "ekin_tot":
        ke = torch.zeros(count, dtype=torch.float64, device="cuda")
        pb.kinetic_energy(uhb, ke)
        np.testing.assert_allclose(ke.cpu().numpy(), e0s, rtol=1e-6)


def test_graph_replay_equals_direct_calls():
    from l3es import _native

    n, steps = 32, 5
    u = _fields(3, n, 1, 5)[0]
    p = _native.Plan(dim=3, n=n, nu=5e-3, dt=2e-3, forcing="const_power", kf=2, eps_inj=0.1)
    ip = _native.InterpPlan(dim=3, ckp_n=16, n_fine=n, np_max=500)
    rng = np.random.default_rng(0)
    r0 = torch.from_numpy(rng.uniform(0, 2 * np.pi, (500, 3))).cuda()

    # direct
    uh_d = _spec(_native.Plan, 3, n, u)
    r_d = [r0.clone(), torch.empty_like(r0)]
    ur_d = torch.empty_like(r0)
    for _ in range(steps):
        p.step(uh_d, 1)
        ip.set_spectrum(uh_d)
        ip.interp(r_d[0], ur_d, dt=2e-3, r_out=r_d[1])
        r_d.reverse()
    # recorded once (two steps with the ping-pong positions), replayed
    uh_g = _spec(_native.Plan, 3, n, u)
    r_a, r_b = r0.clone(), torch.empty_like(r0)
    ur_g = torch.empty_like(r0)
    cap = _native.Graph.begin()
    for src, dst in ((r_a, r_b), (r_b, r_a)):
        p.step(uh_g, 1, stream=cap)
        ip.set_spectrum(uh_g, stream=cap)
        ip.interp(src, ur_g, dt=2e-3, r_out=dst, stream=cap)
    g = _native.Graph.end(cap)
    for _ in range(steps // 2):
        g.launch()
    # one more step directly to reach 5
    p.step(uh_g, 1)
    ip.set_spectrum(uh_g)
    ip.interp(r_a, ur_g, dt=2e-3, r_out=r_b)
    torch.cuda.synchronize()
    assert torch.equal(uh_g, uh_d)
    assert torch.equal(ur_g, ur_d)
    assert torch.equal(r_b, r_d[0])


def test_graph_of_two_grid_sizes():
    from l3es import _native

    pa = _native.Plan(dim=2, n=64, nu=1e-3, dt=1e-3, kolm_k=4, kolm_amp=1.0, drag=0.1)
    pb = _native.Plan(dim=3, n=32, nu=5e-3, dt=2e-3)
    ua, ub = _fields(2, 64, 1, 1)[0], _fields(3, 32, 1, 2)[0]
    ref_a, ref_b = _spec(_native.Plan, 2, 64, ua), _spec(_native.Plan, 3, 32, ub)
    pa.step(ref_a, 4)
    pb.step(ref_b, 4)
    ga, gb = _spec(_native.Plan, 2, 64, ua), _spec(_native.Plan, 3, 32, ub)
    cap = _native.Graph.begin()
    pa.step(ga, 1, stream=cap)
    pb.step(gb, 1, stream=cap)
    g = _native.Graph.end(cap)
    for _ in range(4):
        g.launch()
    torch.cuda.synchronize()
    assert torch.equal(ga, ref_a) and torch.equal(gb, ref_b)


def test_kolmogorov_drag_extension_matches_oracle():
    """2D extension terms (f_x = sin(4y), drag 0.1) vs the oracle's opt-in terms."""
    from l3es import _native

    n, nu, dt, steps = 64, 1e-3, 1e-3, 3
    u = _fields(2, n, 1, 7)[0]
    uh0 = np.fft.rfftn(u, axes=(1, 2)).squeeze()
    rhs = R.rhs_wrapper(n, nu, (1, 2), drag=0.1, force_hat=R.kolmogorov_forcing_hat(n, 1.0, 4))
    step = R.rk4_wrapper(dt, rhs, None, 0.0, "none", (1, 2))
    uu, uh = u, uh0
    for _ in range(steps):
        uu, uh, _ = step(uu, uh)
    p = _native.Plan(dim=2, n=n, nu=nu, dt=dt, kolm_k=4, kolm_amp=1.0, drag=0.1)
    g = torch.from_numpy(np.ascontiguousarray(uh0, dtype=np.complex64)).cuda()
    p.step(g, steps)
    assert np.abs(g.cpu().numpy() - uh).max() < 2e-5 * np.abs(uh).max()


def test_kolmogorov_256_with_particles_matches_oracle_loop():
    """The 2D Kolmogorov configuration end to end: 256^2, f_x = sin(4y), nu = 1e-3,
    drag 0.1, random-phase initial field with |k| <= 8 and kinetic energy 0.5, dt = 1e-3;
    4096 particles on a jittered 64^2 lattice interpolated by NUFFT (sigma 2, width 6)
    from the 64^2 coarsening and advected (Euler) every step, 20 steps (the combined
    loop's order: DNS step, coarsen, interpolate at the old positions, shift), against
    the FP64 oracle loop with the exact spectral interpolation."""
    from l3es import _native

    n, nu, dt, c, steps = 256, 1e-3, 1e-3, 64, 20
    u = R.init_u_random2d(n, 0, 8.0, 0.5)
    uh64 = np.fft.rfftn(u[..., 0], axes=(1, 2))
    r64 = R.pos_init_cartesian(2 * np.pi, c, 2, jitter=0.25, seed=0)
    rhs = R.rhs_wrapper(n, nu, (1, 2), drag=0.1, force_hat=R.kolmogorov_forcing_hat(n, 1.0, 4))
    step = R.rk4_wrapper(dt, rhs, None, 0.0, "none", (1, 2))
    plan = _native.Plan(dim=2, n=n, nu=nu, dt=dt, kolm_k=4, kolm_amp=1.0, drag=0.1)
    ip = _native.InterpPlan(dim=2, ckp_n=c, n_fine=n, width=6, np_max=len(r64))
    g = torch.from_numpy(np.ascontiguousarray(uh64, dtype=np.complex64)).cuda()
    r = [torch.from_numpy(r64.copy()).cuda(), torch.empty(len(r64), 2, dtype=torch.float64, device="cuda")]
    ur = torch.empty(len(r64), 2, dtype=torch.float64, device="cuda")
    uu, uh = u, uh64
    for _ in range(steps):
        uu, uh, _ = step(uu, uh)
        v = R.interpolate_from_uhat_dft(uh, n, c, r64, dim=2)
        r64 = R.shift_fn(r64, dt * v)
        plan.step(g, 1)
        ip.set_spectrum(g)
        ip.interp(r[0], ur, backend="nufft", dt=dt, r_out=r[1])
        r.reverse()
    plan.check()
    assert np.abs(g.cpu().numpy() - uh).max() < 2e-5 * np.abs(uh).max()
    assert np.abs(ur.cpu().numpy() - v).max() < 5e-5 * np.abs(v).max()
    d = np.mod(r[0].cpu().numpy() - r64 + np.pi, 2 * np.pi) - np.pi
    assert np.abs(d).max() < 5e-5 * steps * dt * np.abs(v).max()


def test_graph_branches_equal_direct_calls():
    """Two grid sizes and a particle update recorded on separate branches of one graph
    (l3es_graph_fork / _join) give bit-identical results to the same calls made
    directly, over several replays."""
    from l3es import _native

    pa = _native.Plan(dim=2, n=64, nu=1e-3, dt=1e-3, kolm_k=4, kolm_amp=1.0, drag=0.1)
    pb = _native.Plan(dim=3, n=32, nu=5e-3, dt=2e-3)
    ua, ub = _fields(2, 64, 1, 3)[0], _fields(3, 32, 1, 4)[0]
    ip = _native.InterpPlan(dim=2, ckp_n=16, n_fine=64, np_max=100)
    r0 = torch.from_numpy(np.random.default_rng(5).uniform(0, 2 * np.pi, (100, 2))).cuda()
    ref_a, ref_b = _spec(_native.Plan, 2, 64, ua), _spec(_native.Plan, 3, 32, ub)
    ref_r, ur = r0.clone(), torch.empty_like(r0)
    rn = torch.empty_like(r0)
    for _ in range(3):
        pa.step(ref_a, 1)
        ip.set_spectrum(ref_a)
        ip.interp(ref_r, ur, dt=1e-3, r_out=rn)
        ref_r.copy_(rn)
        pb.step(ref_b, 1)
    ga, gb = _spec(_native.Plan, 2, 64, ua), _spec(_native.Plan, 3, 32, ub)
    r, ur2, rn2 = r0.clone(), torch.empty_like(r0), torch.empty_like(r0)
    cap = _native.Graph.begin()
    b1 = _native.Graph.fork(cap)
    pa.step(ga, 1, stream=b1)
    b11 = _native.Graph.fork(b1)
    ip.set_spectrum(ga, stream=b11)
    ip.interp(r, ur2, dt=1e-3, r_out=rn2, stream=b11)
    _native.Graph.join(b1, b11)
    b2 = _native.Graph.fork(cap)
    pb.step(gb, 1, stream=b2)
    _native.Graph.join(cap, b1)
    _native.Graph.join(cap, b2)
    g = _native.Graph.end(cap)
    for _ in range(3):
        g.launch()
        r.copy_(rn2)
    torch.cuda.synchronize()
    assert torch.equal(ga, ref_a) and torch.equal(gb, ref_b)
    assert torch.equal(r, ref_r)
