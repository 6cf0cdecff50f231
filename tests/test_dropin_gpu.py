"""The l3es drop-in call surface on the GPU vs the reference's own golden vectors.

Functions are called with the reference's names and arguments
(spectral_solver.set_up_solver / rk4_wrapper / simulate, utils.*, integrator.*,
combined.combined). FP32 results are compared with the FP64 fixtures at 2e-5
(relative to the field maximum), like the kernel tests.
"""

import numpy as np
import pytest

from oracle import numpy_ref as R
from oracle import nufft_ref as NU

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

RTOL = 2e-5


def _rel(a, b):
    a = a.detach().cpu().numpy() if hasattr(a, "detach") else np.asarray(a)
    b = np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def test_set_up_solver_hit_ekin_golden(gold):
    from l3es import spectral_solver as S

    g = gold("hit3d_n16_ekin")
    out = S.set_up_solver(16, float(g["nu"]), 3, "HIT", float(g["dt"]), 42, 8, int(g["kf"]),
                          float(g["e_kin_target"]), "ekin_tot", True)
    u, uh, xyz_vis, dx, fn, L, axes, e0, e_inj = out
    assert len(out) == 9 and axes == (1, 2, 3) and abs(L - 2 * np.pi) < 1e-15
    assert abs(e0 - float(g["e_kin_init"])) < 1e-12
    inj = [float(e_inj)]
    for _ in range(int(g["steps_after_setup"])):
        u, uh, e = fn(u, uh)
        inj.append(float(e))
    assert _rel(uh, g["u_hat"]) < RTOL
    assert _rel(u, g["u"]) < RTOL
    np.testing.assert_allclose(inj, g["e_inj"], rtol=1e-3, atol=1e-6)


def test_set_up_solver_tgv2d_golden(gold):
    from l3es import spectral_solver as S

    g = gold("tgv2d_n32")
    u, uh, *_rest = S.set_up_solver(32, float(g["nu"]), 2, "TGV2D", float(g["dt"]), 42, 8, None, None, "none")
    fn = _rest[2]
    for _ in range(int(g["steps_after_setup"])):
        u, uh, _ = fn(u, uh)
    assert tuple(u.shape) == (3, 32, 32, 1) and tuple(uh.shape) == (3, 32, 17)
    assert _rel(uh, g["u_hat"]) < RTOL


def test_rk4_wrapper_is_functional(gold):
    from l3es import spectral_solver as S

    g = gold("rand3d_n16")
    step = S.rk4_wrapper(float(g["dt"]), S.rhs_wrapper(16, float(g["nu"])), None, 0.0, "none")
    uh0 = torch.from_numpy(np.ascontiguousarray(g["u_hat0"], dtype=np.complex64)).cuda()
    keep = uh0.clone()
    u, uh = None, uh0
    for _ in range(int(g["steps"])):
        u, uh, _ = step(u, uh)
    assert torch.equal(uh0, keep)  # inputs are not modified
    assert _rel(uh, g["u_hat"]) < RTOL
    du = S.rhs_wrapper(16, float(g["nu"]))(None, uh0, 0)
    assert _rel(du, g["rhs_rk0"]) < RTOL


def test_simulate_tgv_validation(tmp_path):
    """simulate() runs the reference's TGV3D validation (12 steps, spectral_solver.py:363-367)."""
    from l3es import spectral_solver as S

    u, uh = S.simulate(case="TGV3D", N=64, dim=3, nu=0.000625, t_final=0.1, dt=0.01, ckp_N=32,
                       log_freq=5, ckp_freq=5, dst_path=str(tmp_path))
    ke = 0.5 * float((u.double() ** 2).sum(0).mean())
    assert abs(ke - 0.12494373453629146) < 2e-7  # the oracle's 12-step value
    rows = open(tmp_path / "diagnostics.csv").read().splitlines()
    assert rows[0] == "step,time,umax,ekin,dt_est,e_inj" and len(rows) == 4
    assert (tmp_path / "sim" / "u_32_00010.npy").exists()
    assert (tmp_path / "u_64_00000_burnin.npy").exists()


def test_utils_golden(gold):
    from l3es import spectral_solver as S
    from l3es import utils as U

    g = gold("utils")
    assert _rel(U.spectral_filtering(g["f3"], 8), g["filt3_8"]) < RTOL
    assert _rel(U.spectral_filtering(g["f2"], 8), g["filt2_8"]) < RTOL
    assert _rel(U.spectral_filtering(g["f3"], 16), g["filt3_16"]) < RTOL
    assert _rel(U.energy_spectrum(torch.from_numpy(g["f3"]).float()), g["ek3"]) < RTOL
    v2 = np.concatenate([g["f2"], 0 * g["f2"][:1]])[..., None]
    assert _rel(U.energy_spectrum(v2, dim=2), g["ek2"]) < RTOL
    uh3 = np.fft.rfftn(g["f3"], axes=(1, 2, 3))
    assert abs(float(U.comp_dissipation_rate(torch.from_numpy(uh3.astype(np.complex64)).cuda(), 0.01))
               - float(g["diss3"])) < 1e-5 * float(g["diss3"])
    dt = S.comp_dt(torch.from_numpy(g["f3"]).float().cuda(), 2 * np.pi / 16, 0.01, 0.5)
    assert abs(dt - float(g["dt3"])) < 1e-6 * float(g["dt3"])


def test_integrator_golden(gold):
    from l3es import integrator as I

    g = gold("interp")
    c = int(g["c"])
    for axes, field, r, ref in (((1, 2, 3), g["g3"], g["r3"], g["ur3"]), ((1, 2), g["g2"], g["r2"], g["ur2"])):
        dft = I.spectral_interpolator_wrapper(c, axes, splits=4, backend="dft")
        assert _rel(dft(field, r), ref) < RTOL
        nufft = I.spectral_interpolator_wrapper(c, axes, splits=4, backend="nufft")
        assert _rel(nufft(field, r), ref) < 1e-4
        assert _rel(nufft(field, r), NU.interpolate_nufft(field, r, w=6)) < 1e-5
    assert _rel(I.shift_fn(g["r3"], g["dr"]), g["shifted"]) < 1e-15


def test_combined_kolmogorov_matches_oracle_loop(tmp_path):
    """combined() on a 2D case (64^2 DNS, 16^2 particles, dft backend) vs the oracle's
    loop with the same order: step, coarsen, interpolate at old positions, shift."""
    from l3es import combined as C

    n, c, dt, nu, steps = 64, 16, 1e-3, 1e-3, 3
    u, uh, r = C.combined("Kolm", N=n, dim=2, nu=nu, t_final=steps * dt, dt=dt, ckp_N=c, interp_backend="dft",
                          log_freq=1, ckp_freq=1, dst_path=str(tmp_path), seed=3)
    # oracle: set_up_solver (with its warm-up step) then steps + 1 loop iterations
    u_o, uh_o, dx, fn, *_ = R.set_up_solver(n, nu, 2, "Kolm", dt, 3, c, None, None, "none")
    ax = (np.arange(c) + 0.5) * 2 * np.pi / c
    gx, gy = np.meshgrid(ax, ax, indexing="ij")
    r_o = np.stack([gx.ravel(), gy.ravel()], axis=1)
    for i in range(steps + 1):
        u_o, uh_o, _ = fn(u_o, uh_o)
        ur = R.interpolate_dft(R.spectral_filtering(u_o[:2, :, :, 0], c), r_o)
        last = np.load(tmp_path / "com" / f"step_{i:05d}.npz")
        assert _rel(last["u"], ur) < 5e-5
        r_o = R.shift_fn(r_o, dt * ur)
    assert np.abs(r.cpu().numpy() - r_o).max() < 1e-6
    assert _rel(uh, uh_o) < RTOL


def test_particles_to_grid_golden(gold):
    from l3es import turbulence as T

    g = gold("p2g")
    c3, c2 = int(g["c3"]), int(g["c2"])
    assert _rel(T.ur_to_u_dft_wrapper(c3, 2 * np.pi, 3)(g["r3"], g["u3"]), g["grid3"]) < RTOL
    assert _rel(T.ur_to_u_dft_wrapper(c2, 2 * np.pi, 2, (1, 2))(g["r2"], g["u2"]), g["grid2"]) < RTOL
    ug, ek = T.u_and_spectrum_from_ur(c3, 2 * np.pi, 3, "dft")(g["r3"], g["u3"])
    assert _rel(ug, g["ugrid3"]) < RTOL
    assert _rel(ek, g["ek3"]) < RTOL


def test_particles_to_grid_large_vs_oracle():
    """32^3 particles to a 32^3 grid (the combined loop's analysis size)."""
    from l3es import turbulence as T

    rng = np.random.default_rng(9)
    c = 32
    r = rng.uniform(0, 2 * np.pi, (c**3, 3))
    u = rng.standard_normal((c**3, 3))
    got = T.ur_to_u_dft_wrapper(c, 2 * np.pi, 3)(r, u)
    sub = R.particles_to_grid_dft(r[:4096], u[:4096], c)  # linear in the particles
    got_sub = T.ur_to_u_dft_wrapper(c, 2 * np.pi, 3)(r[:4096], u[:4096])
    assert _rel(got_sub, sub.reshape(3, -1).T) < 5e-5
    assert got.shape == (c**3, 3)


def test_combined_trajectories_to_dataset(tmp_path):
    """combined() runs (Kolm init on a 256^2 fine grid) write config.json and particle
    checkpoints that gen_dataset assembles into train/valid/test + metadata."""
    import json

    from l3es import combined as C
    from l3es import gen_dataset as GD

    raw = tmp_path / "raw"
    for seed in (3, 0, 2, 1):
        C.combined("Kolm", N=32, dim=2, nu=1e-3, t_final=4e-3, dt=1e-3, ckp_N=8, interp_backend="dft",
                   log_freq=1, ckp_freq=1, dst_path=str(raw / f"traj_{seed}"), seed=seed, kolm_grid=256)
    cfg = json.loads((raw / "traj_0" / "config.json").read_text())
    assert cfg["sim"]["case"] == "Kolm" and cfg["sim"]["ckp_N"] == 8 and cfg["com"]["ckp_freq"] == 1
    dst = tmp_path / "ds"
    GD.main(["--src_dir", str(raw), "--dst_dir", str(dst), "--split", "2_1_1"])
    meta = json.loads((dst / "metadata_every1.json").read_text())
    assert meta["case"] == "KOLM" and meta["dim"] == 2 and meta["num_particles_max"] == 64
    assert meta["sequence_length_train"] == 5 and meta["num_trajs_train"] == 2
    ext = ".h5" if GD.h5py is not None else ".npz"
    (pt, pos, u), = list(GD._read_split(str(dst / f"test{ext}")))
    last = np.load(raw / "traj_3" / "com" / "step_00004.npz")
    assert pos.shape == (5, 64, 2)
    np.testing.assert_array_equal(pos[-1], last["r"].astype(np.float32))
    np.testing.assert_array_equal(u[-1], last["u"].astype(np.float32))
    assert all(np.isfinite(meta[k]).all() for k in ("vel_std", "acc_std", "u_std", "au_std"))
