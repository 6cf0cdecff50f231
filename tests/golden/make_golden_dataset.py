"""Golden vectors for the dataset assembly (f4), from the reference's own
gen_dataset/gen_dataset.py run here.

    python tests/golden/make_golden_dataset.py <path of the reference checkout>

The script needs h5py, omegaconf, jax (vmap), jax_sph.io_state (read_h5 / write_h5)
and jax_sph.jax_md.space, none of which is installed. Stand-ins:
  - jax.vmap: jax_numpy_shim's loop over the mapped axis;
  - h5py.File: an in-memory store of named arrays (create_dataset / items / get /
    indexing), enough for what the script writes and then reads back;
  - jax_sph.io_state.read_h5: returns the frame arrays registered for a path (the
    frame files exist on disk, empty, because the script lists directories);
  - jax_sph.jax_md.space.periodic: jax_md's published periodic displacement,
    mod(Ra - Rb + side/2, side) - side/2 (its shift function is not used);
  - omegaconf.OmegaConf.load: reads the trajectory's config.yaml, written as JSON (a
    subset of YAML), into attribute access.
Everything the script computes (split rule, frame slicing, metadata, statistics) runs
as written. Output: tests/golden/gen_dataset.npz with the inputs and outputs of three
cases (plain, sliced frames, sliced statistics).
"""

from __future__ import annotations

import importlib.util
import json
import os
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


class _Store:
    files: dict = {}   # h5 path -> {dataset name: array}
    frames: dict = {}  # frame path -> {"r": ..., "u": ...}


class _Group:
    def __init__(self, d, prefix):
        self._d, self._p = d, prefix

    def get(self, name):
        return self._d[f"{self._p}/{name}"]

    def __getitem__(self, name):
        return self._d[f"{self._p}/{name}"]


class _H5File:
    def __init__(self, path, mode="r"):
        self.path = path
        if mode == "w":
            _Store.files[path] = {}
        self.d = _Store.files[path]

    def create_dataset(self, name, data, dtype=None, compression=None, chunks=None):
        self.d[name] = np.array(data, dtype=dtype) if dtype is not None else np.array(data)

    def items(self):
        keys = sorted({k.split("/")[0] for k in self.d})
        return [(k, _Group(self.d, k)) for k in keys]

    def close(self):
        pass


def _periodic(side):
    side = np.asarray(side, dtype=np.float64)

    def displacement(ra, rb, **_):
        return np.mod(ra - rb + 0.5 * side, side) - 0.5 * side

    return displacement, None


def _ns(x):
    if isinstance(x, dict):
        return types.SimpleNamespace(**{k: _ns(v) for k, v in x.items()})
    return x


def install_stubs():
    sys.path.insert(0, HERE)
    import jax_numpy_shim

    jax_numpy_shim.install()
    h5 = types.ModuleType("h5py")
    h5.File = _H5File
    sys.modules["h5py"] = h5
    sys.modules["jax_sph.io_state"].read_h5 = lambda path, array_type="numpy": dict(_Store.frames[path])
    sys.modules["jax_sph.io_state"].write_h5 = lambda d, path: None
    sys.modules["jax_sph.jax_md"].space = types.SimpleNamespace(periodic=_periodic)
    om = types.ModuleType("omegaconf")
    om.OmegaConf = types.SimpleNamespace(load=lambda path: _ns(json.load(open(path))))
    sys.modules["omegaconf"] = om


def make_trajs(root, seeds, frames, npart, dim, cfg, rng):
    """traj_<seed>/com/step_XXXXX.h5 frames (registered with the store) and config.yaml."""
    data = {}
    for s in seeds:
        com = os.path.join(root, f"traj_{s}", "com")
        os.makedirs(com)
        r0 = rng.uniform(0, 2 * np.pi, (npart, dim))
        v = 0.3 * rng.standard_normal((npart, dim))
        rs, us = [], []
        for k in range(frames):
            r = np.mod(r0 + 0.7 * k * v + 0.05 * rng.standard_normal((npart, dim)), 2 * np.pi)
            u = v + 0.1 * rng.standard_normal((npart, dim))
            step = k * cfg["com"]["ckp_freq"]
            path = os.path.join(com, f"step_{step:05d}.h5")
            open(path, "w").close()
            _Store.frames[path] = {"r": r, "u": u}
            rs.append(r)
            us.append(u)
        with open(os.path.join(root, f"traj_{s}", "config.yaml"), "w") as f:
            json.dump(cfg, f)
        data[s] = (np.stack(rs), np.stack(us))
    return data


def main(ref_root: str) -> None:
    install_stubs()
    spec = importlib.util.spec_from_file_location("ref_gen_dataset", os.path.join(ref_root, "gen_dataset",
                                                                                   "gen_dataset.py"))
    gd = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gd)
    rng = np.random.default_rng(2024)
    out = {}
    # the reference asserts write_every == 1 when the statistics are sliced
    cases = [("plain", dict(split="2_1_1", skip=0, slice_=1, stats=1, ckp_freq=3)),
             ("sliced", dict(split="3_1_1", skip=1, slice_=2, stats=1, ckp_freq=3)),
             ("statsliced", dict(split="2_1_1", skip=0, slice_=1, stats=2, ckp_freq=1))]
    for name, cs in cases:
        cfg = {"sim": {"case": "kolm", "dim": 2, "ckp_N": 8, "dt": 0.001, "t_final": 0.5, "nu": 0.001,
                       "u_ref": 6.0},
               "com": {"ckp_freq": cs["ckp_freq"]}}
        seeds = [3, 11, 5, 7, 2, 13]
        with tempfile.TemporaryDirectory() as tmp:
            src, dst = os.path.join(tmp, "src"), os.path.join(tmp, "dst")
            data = make_trajs(src, seeds, frames=7, npart=64, dim=2, cfg=cfg, rng=rng)
            args = types.SimpleNamespace(src_dir=src, dst_dir=dst, split=cs["split"],
                                         skip_first_n_frames=cs["skip"], slice_every_nth_frame=cs["slice_"],
                                         is_visualize=False, stats_every_nth=cs["stats"], only_stats=False)
            gd.single_h5_files_to_h5_dataset(args)
            gd.compute_statistics_h5(args)
            meta = json.load(open(os.path.join(dst, "metadata.json")))
            meta_s = json.load(open(os.path.join(dst, f"metadata_every{cs['stats']}.json")))
            d = {"seeds": np.array(seeds), "split": cs["split"], "skip": cs["skip"], "slice": cs["slice_"],
                 "stats": cs["stats"], "config": json.dumps(cfg), "metadata": json.dumps(meta),
                 "metadata_stats": json.dumps(meta_s)}
            for s, (r, u) in data.items():
                d[f"in_r_{s}"] = r
                d[f"in_u_{s}"] = u
            for split in ("train", "valid", "test"):
                for key, arr in _Store.files[os.path.join(dst, f"{split}.h5")].items():
                    d[f"out_{split}/{key}"] = arr
        for k, v in d.items():
            out[f"{name}:{k}"] = np.asarray(v)
    path = os.path.join(HERE, "gen_dataset.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({os.path.getsize(path) // 1024} KB)")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden_dataset.py <path of the reference checkout>")
    main(sys.argv[1])
