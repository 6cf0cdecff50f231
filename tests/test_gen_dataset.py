"""Dataset assembly (gen_dataset.py:24-239) and the Kolmogorov initial field
(init_fields.py:191-212): host-side, CPU only."""

import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [os.path.join(HERE, "..", "ql-les-data_gb300"), os.path.join(HERE, "..")]

from l3es import gen_dataset as GD  # noqa: E402
from l3es import init_fields as F  # noqa: E402
from oracle import numpy_ref as R  # noqa: E402

L = 2 * np.pi


def _make_trajs(root, seeds, frames=6, npart=16 * 16, dim=2, ckp_N=16, ckp_freq=3):
    rng = np.random.default_rng(0)
    data = {}
    for s in seeds:
        com = root / f"traj_{s}" / "com"
        com.mkdir(parents=True)
        r = rng.uniform(0, L, size=(npart, dim))
        rs, us = [], []
        for i in range(frames):
            u = rng.normal(size=(npart, dim))
            rs.append(r.copy())
            us.append(u)
            np.savez(com / f"step_{i * ckp_freq:05d}.npz", r=r, u=u)
            r = np.mod(r + 0.05 * u, L)  # crosses the periodic boundary now and then
        data[s] = (np.stack(rs), np.stack(us))
        cfg = {"seed": s, "sim": {"case": "Kolm", "dim": dim, "ckp_N": ckp_N, "dt": 1e-3, "t_final": 0.1,
                                  "nu": 1e-3, "u_ref": 6.0},
               "com": {"ckp_freq": ckp_freq}}
        (root / f"traj_{s}" / "config.json").write_text(json.dumps(cfg))
    return data


def _stats_oracle(trajs, every):
    """Independent restatement of gen_dataset.py:138-239 on float32 arrays."""
    side = np.float32(L)
    vels, us = [], []
    for pos, u in trajs:
        r = pos.astype(np.float32)[::every]
        d = r[1:] - r[:-1]
        vels.append(d - side * np.floor(d / side + 0.5))
        us.append(u.astype(np.float32)[::every])
    out = {}
    for name, arrs in (("vel", vels), ("u", us)):
        m = np.mean([a.mean((0, 1)) for a in arrs], axis=0)
        am = np.mean([(a[1:] - a[:-1]).mean((0, 1)) for a in arrs], axis=0)
        # the reference's velocity / acceleration spreads are about 0 (gen_dataset.py:157)
        c, ac = (m, am) if name == "u" else (0.0, 0.0)
        sd = np.mean([np.square(a - c).mean((0, 1)) for a in arrs], axis=0) ** 0.5
        asd = np.mean([np.square(a[1:] - a[:-1] - ac).mean((0, 1)) for a in arrs], axis=0) ** 0.5
        out[name] = (m, sd, am, asd)
    return out


def test_dataset_splits_metadata_and_stats(tmp_path):
    src, dst = tmp_path / "raw", tmp_path / "ds"
    seeds = [10, 2, 0, 7]                       # ordered by seed value: 0, 2, 7, 10
    data = _make_trajs(src, seeds)
    GD.main(["--src_dir", str(src), "--dst_dir", str(dst), "--split", "2_1_1"])
    ext = ".h5" if GD.h5py is not None else ".npz"
    order = sorted(seeds)
    expect = {"train": order[:2], "valid": order[2:3], "test": order[3:]}
    for split, ss in expect.items():
        got = list(GD._read_split(str(dst / f"{split}{ext}")))
        assert len(got) == len(ss)
        for (ptype, pos, u), s in zip(got, ss):
            assert pos.dtype == np.float32 and pos.shape == (6, 256, 2)
            np.testing.assert_array_equal(ptype, np.zeros(256))
            np.testing.assert_array_equal(pos, data[s][0].astype(np.float32))
            np.testing.assert_array_equal(u, data[s][1].astype(np.float32))
    meta = json.loads((dst / "metadata.json").read_text())
    assert meta["case"] == "KOLM" and meta["dim"] == 2 and meta["write_every"] == 3
    assert meta["num_trajs_train"] == 2 and meta["num_trajs_test"] == 1
    assert meta["sequence_length_train"] == meta["sequence_length_test"] == 6
    assert meta["num_particles_max"] == 256 and meta["bounds"] == [[0, L]] * 2
    assert meta["default_connectivity_radius"] == 0.59   # 1.5 * 2 pi / 16 = 0.589...
    stats = json.loads((dst / "metadata_every1.json").read_text())
    ref = _stats_oracle([data[s] for s in expect["train"]], 1)
    for name, keys in (("vel", ("vel_mean", "vel_std", "acc_mean", "acc_std")),
                       ("u", ("u_mean", "u_std", "au_mean", "au_std"))):
        for k, v in zip(keys, ref[name]):
            np.testing.assert_allclose(stats[k], v, rtol=1e-4, atol=1e-6)


def test_dataset_frame_slicing_and_sliced_stats(tmp_path):
    src, dst = tmp_path / "raw", tmp_path / "ds"
    data = _make_trajs(src, [0, 1, 2, 3, 4], frames=7)
    GD.main(["--src_dir", str(src), "--dst_dir", str(dst), "--split", "3_1_1",
             "--skip_first_n_frames", "1", "--slice_every_nth_frame", "2"])
    meta = json.loads((dst / "metadata.json").read_text())
    assert meta["sequence_length_train"] == 3 and meta["write_every"] == 6   # frames 1, 3, 5
    assert meta["num_trajs_train"] == 3 and meta["num_trajs_test"] == 1
    ext = ".h5" if GD.h5py is not None else ".npz"
    (_, pos, _), = list(GD._read_split(str(dst / f"test{ext}")))
    np.testing.assert_array_equal(pos, data[4][0][1::2].astype(np.float32))
    # sliced dataset + sliced stats is refused, as in the reference
    with pytest.raises(ValueError):
        GD.main(["--src_dir", str(src), "--dst_dir", str(dst), "--only_stats", "--stats_every_nth", "2",
                 "--slice_every_nth_frame", "2"])
    # frames written every step: unsliced dataset, stats on every 2nd frame
    src1, dst1 = tmp_path / "raw1", tmp_path / "ds1"
    data1 = _make_trajs(src1, [0, 1, 2, 3, 4], frames=7, ckp_freq=1)
    GD.main(["--src_dir", str(src1), "--dst_dir", str(dst1), "--split", "3_1_1"])
    with pytest.raises(ValueError):   # write_every 3 with sliced stats is refused too
        GD.main(["--src_dir", str(src), "--dst_dir", str(dst), "--only_stats", "--stats_every_nth", "2"])
    GD.main(["--src_dir", str(src1), "--dst_dir", str(dst1), "--only_stats", "--stats_every_nth", "2"])
    stats = json.loads((dst1 / "metadata_every2.json").read_text())
    assert stats["write_every"] == 2
    ref = _stats_oracle([data1[s] for s in (0, 1, 2)], 2)
    np.testing.assert_allclose(stats["vel_std"], ref["vel"][1], rtol=1e-4)
    np.testing.assert_allclose(stats["au_mean"], ref["u"][2], rtol=1e-4, atol=1e-6)


def test_periodic_displacement_minimum_image():
    side = np.float32(L)
    a = np.array([[0.1, 6.2]], np.float32)
    b = np.array([[6.2, 0.1]], np.float32)
    d = GD.periodic_displacement(a, b, side)
    assert np.all(np.abs(d) < np.pi) and np.allclose(d, [[0.1 + L - 6.2, 6.2 - L - 0.1]], atol=1e-5)


@pytest.mark.parametrize("N,G", [(32, 128), (64, 256)])
def test_kolm_init_matches_oracle_and_is_solenoidal(N, G):
    u = F.init_u_kolm(N, seed=5, grid_n=G)
    assert u.shape == (3, N, N, 1) and not u[2].any()
    np.testing.assert_allclose(u, R.init_u_kolm(N, seed=5, grid_n=G), atol=1e-12)
    vh = np.fft.fft2(u[:2, :, :, 0])
    k = np.fft.fftfreq(N, 1.0 / N)
    div = k[:, None] * vh[0] + k[None, :] * vh[1]
    inner = (np.abs(k)[:, None] < N // 2) & (np.abs(k)[None, :] < N // 2)
    assert np.abs(div[inner]).max() < 1e-10 * np.abs(vh).max()
    # on its own grid the field reaches the prescribed maximum speed
    full = F.init_u_kolm(G, seed=5, grid_n=G, target_dim=2)
    assert full.shape == (2, G, G, 1)
    assert abs(np.sqrt((full[..., 0] ** 2).sum(0)).max() - 4.2) < 1e-12
    assert not np.array_equal(u, F.init_u_kolm(N, seed=6, grid_n=G))


@pytest.mark.parametrize("case", ["plain", "sliced", "statsliced"])
def test_dataset_matches_reference_golden(tmp_path, case):
    """The same trajectories through the reference's own gen_dataset.py (run with
    stand-ins for h5py, omegaconf and jax_sph's io and periodic space; see
    tests/golden/make_golden_dataset.py) and through l3es.gen_dataset: identical split
    contents, metadata and statistics."""
    z = np.load(os.path.join(HERE, "golden", "gen_dataset.npz"))
    g = {k.split(":", 1)[1]: z[k] for k in z.files if k.startswith(case + ":")}
    cfg = json.loads(str(g["config"]))
    src, dst = tmp_path / "raw", tmp_path / "ds"
    for s in g["seeds"]:
        com = src / f"traj_{s}" / "com"
        com.mkdir(parents=True)
        r, u = g[f"in_r_{s}"], g[f"in_u_{s}"]
        for k in range(r.shape[0]):
            np.savez(com / f"step_{k * cfg['com']['ckp_freq']:05d}.npz", r=r[k], u=u[k])
        (src / f"traj_{s}" / "config.json").write_text(json.dumps(cfg))
    GD.main(["--src_dir", str(src), "--dst_dir", str(dst), "--split", str(g["split"]),
             "--skip_first_n_frames", str(int(g["skip"])), "--slice_every_nth_frame", str(int(g["slice"])),
             "--stats_every_nth", str(int(g["stats"]))])
    ext = ".h5" if GD.h5py is not None else ".npz"
    for split in ("train", "valid", "test"):
        got = list(GD._read_split(str(dst / f"{split}{ext}")))
        keys = sorted({k.split("/")[1] for k in g if k.startswith(f"out_{split}/")})
        assert len(got) == len(keys)
        for (ptype, pos, u), key in zip(got, keys):
            np.testing.assert_array_equal(ptype, g[f"out_{split}/{key}/particle_type"])
            np.testing.assert_array_equal(pos, g[f"out_{split}/{key}/position"])
            np.testing.assert_array_equal(u, g[f"out_{split}/{key}/u"])
    meta = json.loads((dst / "metadata.json").read_text())
    ref_meta = json.loads(str(g["metadata"]))
    assert meta == ref_meta
    n = int(g["stats"])
    stats = json.loads((dst / f"metadata_every{n}.json").read_text())
    ref_stats = json.loads(str(g["metadata_stats"]))
    assert stats.keys() == ref_stats.keys()
    for k, v in ref_stats.items():
        if k.endswith(("_mean", "_std")):
            np.testing.assert_allclose(stats[k], v, rtol=2e-6, atol=1e-7)
        else:
            assert stats[k] == v, k
