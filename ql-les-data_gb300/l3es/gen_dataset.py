"""ML dataset assembly from combined() trajectories (drop-in for gen_dataset/gen_dataset.py).

Input: a source directory with one traj_<seed> directory per trajectory, each holding
com/step_XXXXX.npz particle checkpoints (keys r, u; written by combined) and the run's
config.json (or the reference's config.yaml, when PyYAML is installed). Output, in the
LagrangeBench layout the reference writes (gen_dataset.py:24-135):
  train / valid / test split files with one group per trajectory, "00000/position",
  "00000/u" (float32, (frames, particles, dim)) and "00000/particle_type" (zeros);
  metadata.json with the same keys; metadata_every<n>.json with the velocity and
  acceleration statistics (gen_dataset.py:138-239).
Split files are HDF5 (<split>.h5) when h5py is installed, otherwise .npz archives with
the same group/dataset keys. Host-side NumPy, like the reference (which forces JAX onto
the CPU for this script).
"""

from __future__ import annotations

import argparse
import json
import os

import numpy as np

try:  # optional: the reference's storage format
    import h5py  # type: ignore
except ImportError:  # pragma: no cover - depends on the install
    h5py = None


def _frame_number(name: str) -> int:
    """step_00012.npz / xxx_12.h5 -> 12 (gen_dataset.py:69: int(x.split("_")[1][:-3]))."""
    return int(name.split("_")[1].split(".")[0])


def _read_frame(path: str):
    if path.endswith(".npz"):
        with np.load(path) as z:
            return z["r"], z["u"]
    if h5py is None:
        raise ValueError(f"{path}: reading .h5 frames needs h5py")
    with h5py.File(path, "r") as f:
        return f["r"][...], f["u"][...]


def _load_config(traj_dir: str) -> dict:
    path = os.path.join(traj_dir, "config.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f)
    path = os.path.join(traj_dir, "config.yaml")
    try:
        import yaml  # type: ignore
    except ImportError as e:
        raise ValueError(f"{traj_dir}: no config.json, and reading config.yaml needs PyYAML") from e
    with open(path) as f:
        return yaml.safe_load(f)


def _split_path(dst_dir: str, split: str) -> str:
    return os.path.join(dst_dir, f"{split}.h5" if h5py is not None else f"{split}.npz")


def _write_split(path: str, groups: dict) -> None:
    if h5py is not None:
        with h5py.File(path, "w") as hf:
            for key, (ptype, vel, pos) in groups.items():
                hf.create_dataset(f"{key}/particle_type", data=ptype)
                chunks = (1, pos.shape[1], pos.shape[2])
                hf.create_dataset(f"{key}/u", data=vel, dtype=np.float32, compression="gzip", chunks=chunks)
                hf.create_dataset(f"{key}/position", data=pos, dtype=np.float32, compression="gzip", chunks=chunks)
        return
    arrays = {}
    for key, (ptype, vel, pos) in groups.items():
        arrays[f"{key}/particle_type"] = ptype
        arrays[f"{key}/u"] = vel.astype(np.float32)
        arrays[f"{key}/position"] = pos.astype(np.float32)
    np.savez_compressed(path, **arrays)


def _read_split(path: str):
    """Yields (particle_type, position, u) per trajectory, in key order."""
    if path.endswith(".h5"):
        with h5py.File(path, "r") as hf:
            for _, g in hf.items():
                yield g["particle_type"][:], g["position"][...], g["u"][...]
        return
    with np.load(path) as z:
        keys = sorted({k.split("/")[0] for k in z.files})
        for k in keys:
            yield z[f"{k}/particle_type"], z[f"{k}/position"], z[f"{k}/u"]


def periodic_displacement(ra, rb, side):
    """Minimum-image displacement ra - rb in a periodic box (JAX-MD space.periodic,
    used by gen_dataset.py:146-150): mod(ra - rb + side/2, side) - side/2."""
    return np.mod(ra - rb + 0.5 * side, side) - 0.5 * side


def single_h5_files_to_h5_dataset(args) -> None:
    """gen_dataset.py:24-135: trajectories ordered by seed, split by the relative ratio
    args.split ("train_valid_test"; valid and test get ceil(valid / sum * n) each),
    frames from skip_first_n_frames every slice_every_nth_frame, metadata.json."""
    os.makedirs(args.dst_dir, exist_ok=True)
    dirs = [d for d in os.listdir(args.src_dir) if os.path.isdir(os.path.join(args.src_dir, d))]
    dirs = sorted([d for d in dirs if d.startswith("traj_")], key=lambda x: int(x.split("_")[-1]))
    if not dirs:
        raise ValueError(f"no traj_* directories in {args.src_dir}")
    splits = np.array([int(s) for s in args.split.split("_")])
    num_eval = int(np.ceil(splits[1] / splits.sum() * len(dirs)))
    bounds = np.cumsum([0, len(dirs) - 2 * num_eval, num_eval, num_eval])
    num_trajs_train, num_trajs_test = len(dirs) - 2 * num_eval, num_eval
    files_per_traj = len(os.listdir(os.path.join(args.src_dir, dirs[0], "com")))
    seq_len = int(np.ceil((files_per_traj - args.skip_first_n_frames) / args.slice_every_nth_frame))
    for i, split in enumerate(["train", "valid", "test"]):
        groups = {}
        for j, d in enumerate(dirs[bounds[i]:bounds[i + 1]]):
            com = os.path.join(args.src_dir, d, "com")
            files = sorted([f for f in os.listdir(com) if f.endswith((".npz", ".h5"))], key=_frame_number)
            files = files[args.skip_first_n_frames::args.slice_every_nth_frame]
            frames = [_read_frame(os.path.join(com, f)) for f in files]
            if args.is_visualize:  # per-frame copies for viewers (gen_dataset.py:17-21)
                for f, (r, u) in zip(files, frames):
                    np.savez(os.path.join(com, f.rsplit(".", 1)[0] + "_vis.npz"), r=r, u=u)
            pos = np.stack([r for r, _ in frames])          # (frames, particles, dim)
            vel = np.stack([u for _, u in frames])
            groups[str(j).zfill(5)] = (np.zeros(pos.shape[1]), vel, pos)
        _write_split(_split_path(args.dst_dir, split), groups)
        print(f"Finished {args.src_dir} {split} with {len(groups)} entries!")
    cfg = _load_config(os.path.join(args.src_dir, dirs[-1]))
    sim, com = cfg["sim"], cfg["com"]
    dx = 2 * np.pi / sim["ckp_N"]
    metadata = {
        "case": str(sim["case"]).upper(),
        "dim": sim["dim"],
        "dx": dx,
        "dt": sim["dt"],
        "t_end": sim["t_final"],
        "viscosity": sim["nu"],
        "u_ref": sim["u_ref"],
        "write_every": com["ckp_freq"] * args.slice_every_nth_frame,
        "sequence_length_train": seq_len,
        "num_trajs_train": int(num_trajs_train),
        "sequence_length_test": seq_len,
        "num_trajs_test": int(num_trajs_test),
        "num_particles_max": sim["ckp_N"] ** sim["dim"],
        "periodic_boundary_conditions": [True] * 3,
        "bounds": [[0, 2 * np.pi]] * sim["dim"],
    }
    # 1.5 dx to two significant digits, as the reference formats it
    metadata["default_connectivity_radius"] = float(
        np.format_float_positional(1.5 * dx, precision=2, unique=False, fractional=False, trim="k"))
    with open(os.path.join(args.dst_dir, "metadata.json"), "w") as f:
        json.dump(metadata, f)


def compute_statistics_h5(args) -> dict:
    """gen_dataset.py:138-239: means and standard deviations over the train split of the
    position-difference velocity (minimum image), its frame difference, the particle
    velocity u and its frame difference, every stats_every_nth frame; stds below 1e-7
    become 1. Writes metadata_every<n>.json and returns the updated metadata."""
    with open(os.path.join(args.dst_dir, "metadata.json")) as f:
        metadata = json.load(f)
    periodic = np.array(metadata["periodic_boundary_conditions"]).any()
    box = np.array(metadata["bounds"], dtype=np.float64)
    side = (box[:, 1] - box[:, 0]).astype(np.float32)
    path = _split_path(args.dst_dir, "train")
    n = args.stats_every_nth
    # checked before the statistics (the reference asserts it after computing them)
    if not (metadata["write_every"] == 1 or n == 1):
        raise ValueError("Either keep the dataset without slicing and have sliced stats files, "
                         "or slice the dataset and have unsliced stats.")

    def fields():
        for ptype, pos, u in _read_split(path):
            fluid = ptype == 0
            r = pos[::n][:, fluid]
            uu = u[::n][:, fluid]
            vel = periodic_displacement(r[1:], r[:-1], side) if periodic else r[1:] - r[:-1]
            yield vel, uu

    vs, avs, us, aus = [], [], [], []
    for vel, uu in fields():
        vs.append(vel.mean((0, 1)))
        avs.append((vel[1:] - vel[:-1]).mean((0, 1)))
        us.append(uu.mean((0, 1)))
        aus.append((uu[1:] - uu[:-1]).mean((0, 1)))
    vel_mean, acc_mean = np.stack(vs).mean(0), np.stack(avs).mean(0)
    u_mean, au_mean = np.stack(us).mean(0), np.stack(aus).mean(0)
    # As the reference computes them: its velocity and acceleration spreads are taken
    # about 0, because the centring values it subtracts (v_mean, av_mean) are set to 0.0
    # and never updated (gen_dataset.py:157, :180-183); u and au are centred on their means.
    v_sq, av_sq, u_sq, au_sq = [], [], [], []
    for vel, uu in fields():
        v_sq.append(np.square(vel).mean((0, 1)))
        av_sq.append(np.square(vel[1:] - vel[:-1]).mean((0, 1)))
        u_sq.append(np.square(uu - u_mean).mean((0, 1)))
        au_sq.append(np.square(uu[1:] - uu[:-1] - au_mean).mean((0, 1)))
    stds = [np.stack(a).mean(0) ** 0.5 for a in (v_sq, av_sq, u_sq, au_sq)]
    vel_std, acc_std, u_std, au_std = (np.where(s < 1e-7, 1, s) for s in stds)
    metadata.update({"vel_mean": vel_mean.tolist(), "vel_std": vel_std.tolist(),
                     "acc_mean": acc_mean.tolist(), "acc_std": acc_std.tolist(),
                     "u_mean": u_mean.tolist(), "u_std": u_std.tolist(),
                     "au_mean": au_mean.tolist(), "au_std": au_std.tolist()})
    metadata["write_every"] = metadata["write_every"] * n
    with open(os.path.join(args.dst_dir, f"metadata_every{n}.json"), "w") as f:
        json.dump(metadata, f)
    return metadata


def parse_args(argv=None):
    p = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    p.add_argument("--src_dir", type=str)
    p.add_argument("--dst_dir", type=str)
    p.add_argument("--split", default="2_1_1", type=str, help="Relative ratio.")
    p.add_argument("--skip_first_n_frames", type=int, default=0)
    p.add_argument("--slice_every_nth_frame", type=int, default=1)
    p.add_argument("--is_visualize", action="store_true")
    p.add_argument("--stats_every_nth", type=int, default=1)
    p.add_argument("--only_stats", action="store_true")
    args = p.parse_args(argv)
    if not (args.slice_every_nth_frame == 1 or args.stats_every_nth == 1):
        raise ValueError("Either keep the dataset without slicing and have sliced stats files, "
                         "or slice the dataset and have unsliced stats.")
    return args


def main(argv=None) -> None:
    args = parse_args(argv)
    if not args.only_stats:
        single_h5_files_to_h5_dataset(args)
    compute_statistics_h5(args)


if __name__ == "__main__":
    main()
