"""Generate golden input/output vectors from the reference's own source files.

Run here (not on the GPU machine, where the reference is absent):
    python tests/golden/make_golden.py <path of the reference checkout>

The reference (tumaer/ql-les-data, package ``l3es``) needs jax 0.4.29, which is not
installed, so ``jax_numpy_shim`` supplies a NumPy-backed ``jax.numpy`` (FP64, the
precision the reference forces at l3es/spectral_solver.py:24). The reference's
``custom_jit_integrate`` (XLA compile + serialise, spectral_solver.py:130-153) is
replaced by the identity; everything else runs as written. The NumPy port
``from_spectralDNS/main_numpy.py`` runs unmodified (with a stub matplotlib).

Output: ``tests/golden/*.npz``, small (N <= 32) so the CPU test-suite stays fast.
"""

from __future__ import annotations

import importlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref_root: str) -> None:
    sys.path.insert(0, HERE)
    import jax_numpy_shim

    jax_numpy_shim.install()
    sys.path.insert(0, ref_root)
    sys.path.insert(0, os.path.join(ref_root, "from_spectralDNS"))
    ss = importlib.import_module("l3es.spectral_solver")
    ut = importlib.import_module("l3es.utils")
    inf = importlib.import_module("l3es.init_fields")
    itg = importlib.import_module("l3es.integrator")
    mn = importlib.import_module("main_numpy")
    ss.custom_jit_integrate = lambda path_pref, rejit, fn, u, u_hat: fn

    A = np.asarray
    out = {}

    # --- 1. TGV3D, 16^3, 3 steps: l3es rk4 and the spectralDNS NumPy port -------
    N, nu, dt = 16, 1.0 / 1600, 0.01
    xyz = np.mgrid[:N, :N, :N].astype(float) * 2 * np.pi / N
    u0 = A(inf.init_u_tgv(xyz[0], xyz[1], xyz[2]))
    uh0 = np.fft.rfftn(u0, axes=(1, 2, 3))
    step = ss.rk4_wrapper(dt, ss.rhs_wrapper(N, nu), None, 0.0, "none")
    u, uh = u0, uh0
    for _ in range(3):
        u, uh, _e = step(u, uh)
    mn.nu = nu  # main_numpy.rhs_fn reads a module-global nu (main_numpy.py:85, :111)
    step_np = mn.rk4_wrapper(dt, mn.rhs_wrapper(N))
    u2, uh2 = u0, uh0
    for _ in range(3):
        u2, uh2 = step_np(u2, uh2)
    out["tgv3d_n16"] = dict(N=N, nu=nu, dt=dt, steps=3, u0=u0, u_hat0=uh0,
                           u_hat=A(uh), u=A(u), u_hat_spectraldns=uh2)

    # --- 2. random full-spectrum 3D field, 16^3, 2 steps (Nyquist content) -------
    rng = np.random.default_rng(1234)
    N, nu, dt = 16, 0.02, 0.004
    u0 = rng.standard_normal((3, N, N, N))
    uh0 = np.fft.rfftn(u0, axes=(1, 2, 3))
    step = ss.rk4_wrapper(dt, ss.rhs_wrapper(N, nu), None, 0.0, "none")
    u, uh = u0, uh0
    rhs0 = A(ss.rhs_wrapper(N, nu)(u0, uh0, 0))
    rhs1 = A(ss.rhs_wrapper(N, nu)(u0, uh0, 1))
    for _ in range(2):
        u, uh, _e = step(u, uh)
    out["rand3d_n16"] = dict(N=N, nu=nu, dt=dt, steps=2, u0=u0, u_hat0=uh0,
                            rhs_rk0=rhs0, rhs_rk1=rhs1, u_hat=A(uh), u=A(u))

    # --- 3. forced HIT via set_up_solver (includes the warm-up step) -------------
    N, nu, dt, kf, ek = 16, 0.01, 0.005, 2, 1.25
    r = ss.set_up_solver(N, nu, 3, "HIT", dt, 42, 8, kf, ek, "ekin_tot", True)
    u, uh, _, dx, fn, L, axes, e_kin_init, e_inj0 = r
    hist = [float(e_inj0)]
    for _ in range(2):
        u, uh, e = fn(u, uh)
        hist.append(float(e))
    out["hit3d_n16_ekin"] = dict(N=N, nu=nu, dt=dt, kf=kf, e_kin_target=ek, seed=42,
                                steps_after_setup=2, e_kin_init=float(e_kin_init),
                                e_inj=np.array(hist), u_hat=A(uh), u=A(u),
                                u_init=A(inf.init_u_hit(N, 42)),
                                forcing_mask=A(inf.init_forcing_mask_hit(N, kf)))

    # --- 4. TGV2D via set_up_solver, 32^2, 3 more steps ---------------------------
    N, nu, dt = 32, 0.06283, 0.001
    r = ss.set_up_solver(N, nu, 2, "TGV2D", dt, 42, 8, None, None, "none", True)
    u, uh = r[0], r[1]
    for _ in range(3):
        u, uh, _e = r[4](u, uh)
    out["tgv2d_n32"] = dict(N=N, nu=nu, dt=dt, steps_after_setup=3,
                           u_init=A(inf.init_u_tgv2d(N, target_dim=3, rescale=2 * np.pi)),
                           u_hat=A(uh), u=A(u))

    # --- 5. random 2D field with a nonzero third component, 32^2, 2 steps --------
    N, nu, dt = 32, 0.01, 0.002
    u0 = rng.standard_normal((3, N, N, 1))
    uh0 = np.fft.rfftn(u0, axes=(1, 2)).squeeze()
    step = ss.rk4_wrapper(dt, ss.rhs_wrapper(N, nu, (1, 2)), None, 0.0, "none", (1, 2))
    u, uh = u0, uh0
    for _ in range(2):
        u, uh, _e = step(u, uh)
    out["rand2d_n32"] = dict(N=N, nu=nu, dt=dt, steps=2, u0=u0, u_hat0=uh0,
                            u_hat=A(uh), u=A(u))

    # --- 6. spectral filtering, energy spectrum, dissipation, comp_dt ------------
    f3 = rng.standard_normal((3, 16, 16, 16))
    f2 = rng.standard_normal((2, 32, 32))
    uh3 = np.fft.rfftn(f3, axes=(1, 2, 3))
    out["utils"] = dict(
        f3=f3, f2=f2,
        filt3_8=A(ut.spectral_filtering(f3, 8)),
        filt2_8=A(ut.spectral_filtering(f2, 8)),
        filt3_16=A(ut.spectral_filtering(f3, 16)),
        ek3=A(ut.energy_spectrum(f3, 1.0, False, 3)),
        ek2=A(ut.energy_spectrum(np.concatenate([f2, 0 * f2[:1]])[..., None], 1.0,
                                 False, 2)),
        diss3=float(ut.comp_dissipation_rate(uh3, 0.01)),
        dt3=float(ss.comp_dt(f3, 2 * np.pi / 16, 0.01, 0.5)),
    )

    # --- 7. exact DFT interpolation and the periodic shift ----------------------
    c = 8
    g3 = rng.standard_normal((3, c, c, c))
    g2 = rng.standard_normal((2, c, c))
    r3 = rng.uniform(0, 2 * np.pi, (40, 3))
    r2 = rng.uniform(0, 2 * np.pi, (40, 2))
    i3 = itg.spectral_interpolator_wrapper(c, (1, 2, 3), splits=4, backend="dft")
    i2 = itg.spectral_interpolator_wrapper(c, (1, 2), splits=4, backend="dft")
    dr = rng.uniform(-1.0, 1.0, (40, 3))
    out["interp"] = dict(c=c, g3=g3, g2=g2, r3=r3, r2=r2,
                         ur3=A(i3(g3, r3)), ur2=A(i2(g2, r2)),
                         dr=dr, shifted=A(itg.shift_fn(r3, dr)))

    # --- 8. particle -> grid exact DFT and its spectrum (turbulence.py:299-377) ----
    tb = importlib.import_module("l3es.turbulence")
    c3, c2 = 8, 16
    rp3 = rng.uniform(0, 2 * np.pi, (c3**3, 3))
    up3 = rng.standard_normal((c3**3, 3))
    rp2 = rng.uniform(0, 2 * np.pi, (c2**2, 2))
    up2 = rng.standard_normal((c2**2, 2))
    g3 = A(tb.ur_to_u_dft_wrapper(c3, 2 * np.pi, 3, (1, 2, 3))(rp3, up3))
    g2 = A(tb.ur_to_u_dft_wrapper(c2, 2 * np.pi, 2, (1, 2))(rp2, up2))
    ug3, ek3 = tb.u_and_spectrum_from_ur(c3, 2 * np.pi, 3, "dft", (1, 2, 3))(rp3, up3)
    out["p2g"] = dict(c3=c3, c2=c2, r3=rp3, u3=up3, r2=rp2, u2=up2, grid3=g3, grid2=g2,
                      ugrid3=A(ug3), ek3=A(ek3))

    for name, d in out.items():
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **{k: np.asarray(v) for k, v in d.items()})
        print(f"wrote {path} ({os.path.getsize(path) // 1024} KB)")

    # --- 8. the reference's own known answer, 64^3 TGV after 10 steps ------------
    N, nu, dt = 64, 0.000625, 0.01
    xyz = np.mgrid[:N, :N, :N].astype(float) * 2 * np.pi / N
    u = mn.init_u_tgv(xyz[0], xyz[1], xyz[2])
    uh = np.fft.rfftn(u, axes=(1, 2, 3))
    mn.nu = nu
    step_np = mn.rk4_wrapper(dt, mn.rhs_wrapper(N))
    for _ in range(10):
        u, uh = step_np(u, uh)
    ke = 0.5 * np.mean(np.sum(u * u, axis=0))
    assert round(ke - 0.124953117517, 7) == 0  # main_numpy.py:136
    with open(os.path.join(HERE, "tgv64_ke.txt"), "w") as f:
        f.write(f"# TGV3D 64^3 nu=1/1600 dt=0.01, KE after 10 RK4 steps\n")
        f.write(f"# reference assert (from_spectralDNS/main_numpy.py:136): 0.124953117517\n")
        f.write(f"{float(ke)!r}\n")
    print("tgv64 KE", ke)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the reference checkout>")
    main(sys.argv[1])
