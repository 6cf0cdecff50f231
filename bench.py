"""Throughput of the l3es pseudo-spectral DNS step on GB300 (one JSON line).

Workload (the metric's configuration): 3D forced homogeneous isotropic turbulence on
[0, 2 pi)^3 at 256^3, FP32 bulk with FP64 reductions; Rogallo initial field with
E(k) ~ k^4 exp(-2 (k/4)^2), seeded phases, KE 0.5; constant-power forcing eps = 0.1
on 0 < |k| <= 2; nu = 5e-3; dt from CFL 0.5 (fixed); 32^3 particles uniform in the
box, interpolated from the 32^3 spectral coarsening by type-2 NUFFT (sigma 2,
width 6) and advected every step. A step = one RK4 step + coarsening + NUFFT +
advection. Data are synthetic and seeded.

    python bench.py [--gpus N --steps K --warmup W] [--impl reference]

N > 1 (under torchrun) runs independent replicas, one per GPU (the path does not
shard); value = all ranks' steps / max-over-ranks time.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [ROOT, os.path.join(ROOT, "ql-les-data_gb300")]

METRIC = "RK4 steps/s at 256^3 HIT: FP32 form vs FP64 plain, same GB300, <=1e-5 rel KE err"
N_GRID = 256
NU = 5e-3
EPS_INJ = 0.1
KF = 2
KP = 4.0
KE0 = 0.5
CFL = 0.5
SEED = 0
CKP_N = 32
WITH_PARTICLES = True  # coarsening + NUFFT + advection inside the step


TRAFFIC_JSON = os.path.join(ROOT, "profiles", "dram_traffic_hit256.json")
# kernel kinds of the library's timer -> name prefixes of their 256^3 launches in ncu
TRAFFIC_KERNELS = {"line_cross": ("line_cross<256", "line_cross2<256", "line_cross3<256"),
                   "ky_pass_inv": ("ky_inv_rhs<256",),
                   "kx_inv_curl": ("kx_inv_tma<256, 1, 1", "kx_inv_tma<256, true, true",
                                   "kx_inv<256, 3, 1, 1", "kx_inv<256, 3, true, true"),
                   "rk_update": ("k_rk_update<256", "k_rk_update_lin<256"),
                   "kx_fwd_band": ("kx_fwd_band<256", "kx_fwd_band_tma<256"),
                   "ky_pass_fwd": ("ky_pass<256, (int)-1", "ky_pass<256, -1")}


def sources_sha256():
    """Hash of the kernel sources (csrc/*.cu, *.cuh, *.h and the public header): a DRAM
    traffic record applies only to the kernels it was measured on."""
    import glob
    import hashlib

    h = hashlib.sha256()
    files = []
    for pat in ("ql-les-data_gb300/csrc/*.cu", "ql-les-data_gb300/csrc/*.cuh", "ql-les-data_gb300/csrc/*.h",
                "include/*.h"):
        files += glob.glob(os.path.join(ROOT, pat))
    for f in sorted(files, key=lambda p: os.path.relpath(p, ROOT)):
        h.update(os.path.relpath(f, ROOT).encode())
        h.update(open(f, "rb").read())
    return h.hexdigest()


def record_traffic(csv_path, out_path, command):
    """Turns an ncu launch list (`ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum,
    gpu__time_duration.sum --print-units base --csv --log-file CSV ...`) into a JSON
    record of DRAM bytes per launch per kernel kind, tagged with the hash of the sources
    it was measured on."""
    import csv as _csv

    scale = {"byte": 1.0, "Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9, "nsecond": 1e-9, "usecond": 1e-6,
             "msecond": 1e-3, "second": 1.0, "ns": 1e-9, "us": 1e-6, "ms": 1e-3, "s": 1.0}
    rows = [r for r in _csv.reader(open(csv_path)) if r]
    head = next(i for i, r in enumerate(rows) if "Kernel Name" in r and "Metric Name" in r)
    cols = rows[head]
    ki, mi, ui, vi, ii = (cols.index(c) for c in ("Kernel Name", "Metric Name", "Metric Unit", "Metric Value", "ID"))
    launches = {}
    for r in rows[head + 1:]:
        if len(r) <= vi:
            continue
        val = float(r[vi].replace(",", "")) * scale.get(r[ui], 1.0)
        launches.setdefault((r[ii], r[ki]), {})[r[mi]] = val
    def short(full):
        # "void l3es::line_cross2<256>(const float2 *, ...)" -> "line_cross2<256>"
        name = full[5:] if full.startswith("void ") else full
        # template arguments may hold parentheses ("ky_pass<256, (int)-1, 0>")
        name = name[:name.index(">(") + 1] if ">(" in name else name.split("(")[0]
        return name.replace("l3es::", "")

    def kind_of(name):
        return next((k for k, pres in TRAFFIC_KERNELS.items() if name.startswith(pres)), None)

    # the autotuner times every variant first; per kind, keep the variant of the last
    # launch (the schedule the run settled on)
    chosen = {}
    for (lid, full) in sorted(launches, key=lambda key: int(key[0]) if key[0].isdigit() else 0):
        k = kind_of(short(full))
        if k is not None:
            chosen[k] = short(full)
    kinds = {}
    for (_, full), m in launches.items():
        name = short(full)
        kind = kind_of(name)
        if kind is None or chosen.get(kind) != name:
            continue
        d = kinds.setdefault(kind, {"kernel": name, "launches": 0, "dram_read_bytes": 0.0, "dram_write_bytes": 0.0,
                                    "seconds": 0.0})
        d["launches"] += 1
        d["dram_read_bytes"] += m.get("dram__bytes_read.sum", 0.0)
        d["dram_write_bytes"] += m.get("dram__bytes_write.sum", 0.0)
        d["seconds"] += m.get("gpu__time_duration.sum", 0.0)
    for d in kinds.values():
        n = d["launches"]
        d["traffic_per_launch"] = (d["dram_read_bytes"] + d["dram_write_bytes"]) / n
        d["us_per_launch_serialised"] = 1e6 * d["seconds"] / n
    rec = {"sources_sha256": sources_sha256(), "command": command, "kernels": kinds}
    with open(out_path, "w") as f:
        json.dump(rec, f, indent=1)
    return rec


def _ncu_traffic(kernel: str):
    """(DRAM bytes read + written per launch of `kernel`, note) from the ncu record
    profiles/dram_traffic_hit256.json, or (None, why) when there is none for these
    kernel sources."""
    if not os.path.exists(TRAFFIC_JSON):
        return None, "no ncu traffic record"
    rec = json.load(open(TRAFFIC_JSON))
    if rec.get("sources_sha256") != sources_sha256():
        return None, "the ncu traffic record was measured on other kernel sources"
    d = rec.get("kernels", {}).get(kernel)
    if not d:
        return None, f"no {kernel} launches in the ncu traffic record"
    return float(d["traffic_per_launch"]), "ncu dram__bytes_read.sum + dram__bytes_write.sum per launch"


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region (median SM clock, throttle reasons)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.p is not None:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()

    def summary(self):
        try:
            rows = [r.split(",") for r in open(self.f.name).read().strip().splitlines() if r.strip()]
        except Exception:
            rows = []
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4)
                          if len(r) > 5 + i and r[5 + i].strip().lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def replica_throughput(ms_local, world, dist=None, device="cpu"):
    """Replicas (one independent trajectory per rank): the job time is the slowest
    rank's, throughput = world / job time. Returns (max ms per step, steps/s)."""
    ms = float(ms_local)
    if dist is not None and world > 1:
        import torch

        t = torch.tensor([ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t)
    return ms, world * 1e3 / ms


def initial_field(n):
    """Host FP64 initial field of the workload (product init, l3es.init_fields)."""
    from l3es import init_fields as F

    u = F.init_u_hit(n, SEED, spectrum="k4exp", kp=KP)
    u *= np.sqrt(KE0 / (0.5 * np.mean(np.sum(u * u, axis=0))))
    dx = 2 * np.pi / n
    umax = np.abs(u).max(axis=(1, 2, 3))
    dt = CFL / (umax / dx + NU / dx**2).min()  # comp_dt (spectral_solver.py:123-127)
    return u, float(dt)


def initial_field_oracle(n):
    """The same initial field from the FP64 oracle's restatement of init_fields.py
    (used by the CPU arms, which import nothing from the product)."""
    from oracle import numpy_ref as R

    u = R.init_u_hit(n, SEED, spectrum="k4exp", kp=KP)
    u *= np.sqrt(KE0 / (0.5 * np.mean(np.sum(u * u, axis=0))))
    dx = 2 * np.pi / n
    dt = CFL / (np.abs(u).max(axis=(1, 2, 3)) / dx + NU / dx**2).min()
    return u, float(dt)


def particles(c, seed=SEED):
    rng = np.random.default_rng(seed + 1)
    return rng.uniform(0.0, 2 * np.pi, size=(c**3, 3))


# ---------------------------------------------------------------------------------
# reference arm / CPU baseline: the FP64 NumPy restatement on the host cores
# ---------------------------------------------------------------------------------
def cpu_step_rate(n, steps, warmup, u0=None, dt=None):
    from oracle import numpy_ref as R
    from oracle import nufft_ref as NU_

    cores = os.cpu_count() or 1
    R.set_workers(cores)
    if u0 is None:
        u0, dt = initial_field_oracle(n)
    uh = R._rfftn(u0, axes=(1, 2, 3))
    mask = R.init_forcing_mask_hit(n, KF)
    step = R.rk4_wrapper(dt, R.rhs_wrapper(n, NU, const_power=(EPS_INJ, mask)), None, 0.0, "none")
    r = particles(CKP_N)
    u = u0

    def one(u, uh, r):
        u, uh, _ = step(u, uh)
        if not WITH_PARTICLES:
            return u, uh, r
        u_l = R.spectral_filtering(u, CKP_N)
        ur = NU_.interpolate_nufft(u_l, r, w=6)
        return u, uh, R.shift_fn(r, dt * ur)

    for _ in range(warmup):
        u, uh, r = one(u, uh, r)
    t0 = time.perf_counter()
    for _ in range(steps):
        u, uh, r = one(u, uh, r)
    el = time.perf_counter() - t0
    R.set_workers(1)
    return steps / el, cores


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    steps, warmup = max(1, min(args.steps, 2)), min(args.warmup, 1)
    rate, cores = cpu_step_rate(args.n, steps, warmup)
    sample = f"{steps} timed + {warmup} warm-up steps of the {args.n}^3 workload, FP64 NumPy/SciPy"
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": "steps/s", "n_gpus": args.gpus,
        "steps": steps, "warmup": warmup, "ms_per_step": 1e3 / rate, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"hit3d_{args.n}_forced_const_power_particles{CKP_N}^3", "n": args.n},
        "cpu_baseline": {"value": rate, "unit": "steps/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": rate, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------------
# FP64 plain form on the same GPU: the reference algorithm restated with torch.fft
# (cuFFT) in complex128, op for op (spectral_solver.py:27-120). Comparator only.
# ---------------------------------------------------------------------------------
def fp64_model(n, dt, nu=NU, kf=KF, eps_inj=EPS_INJ):
    """(rhs, step, weights) of the FP64 plain form at n^3 with constant-power forcing."""
    import torch

    dev = "cuda"
    kx = torch.fft.fftfreq(n, 1.0 / n, dtype=torch.float64, device=dev)
    kz = kx[: n // 2 + 1].clone()
    kz[-1] *= -1
    kkk = torch.stack(torch.meshgrid(kx, kx, kz, indexing="ij"))
    kkk2 = (kkk * kkk).sum(0)
    kok2 = kkk / torch.where(kkk2 == 0, torch.ones_like(kkk2), kkk2)
    kmax = 2.0 / 3.0 * (n // 2 + 1)
    dealias = ((kkk.abs() < kmax).all(0)).to(torch.float64)
    band = ((kkk2 > 0) & (kkk2 <= kf * kf)).to(torch.float64)
    wts = torch.full((n // 2 + 1,), 2.0, dtype=torch.float64, device=dev)
    wts[0] = wts[-1] = 1.0
    axes = (1, 2, 3)

    def rhs(u_hat):
        u = torch.fft.irfftn(u_hat, s=(n, n, n), dim=axes)
        curl = torch.fft.irfftn(1j * torch.linalg.cross(kkk.to(u_hat.dtype), u_hat, dim=0), s=(n, n, n), dim=axes)
        du = torch.fft.rfftn(torch.linalg.cross(u, curl, dim=0), dim=axes)
        du = du * dealias
        du = du - (du * kok2).sum(0) * kkk
        du = du - nu * kkk2 * u_hat
        ef = 0.5 * float((wts * ((u_hat * band).abs() ** 2).sum(0)).sum()) / float(n) ** 6
        return du + (eps_inj / (2 * ef + 1e-300)) * u_hat * band

    a = [1 / 6, 1 / 3, 1 / 3, 1 / 6]
    b = [0.5, 0.5, 1.0]

    def step(u_hat):
        u0_ = u_hat.clone()
        acc = u_hat.clone()
        uh = u_hat
        for rk in range(4):
            du = rhs(uh)
            if rk < 3:
                uh = u0_ + b[rk] * dt * du
            acc += a[rk] * dt * du
        return acc

    return rhs, step, wts


def _spectral_stats(uh, n, nu=NU):
    """FP64 statistics of a (3, n, n, n/2+1) half spectrum (either precision, promoted):
    kinetic energy, shell energies E(s) over s = int(|k| + 0.5) (utils.py:35-97 up to its
    constant factor, which cancels in a relative error) and the dissipation
    nu <|curl u|^2> = nu sum w k^2 |u_hat|^2 / N^6 (utils.py:300-315), by Parseval."""
    import torch

    u = uh.to(torch.complex128)
    dev = u.device
    kx = torch.fft.fftfreq(n, 1.0 / n, dtype=torch.float64, device=dev)
    kz = torch.arange(n // 2 + 1, dtype=torch.float64, device=dev)
    k2 = kx[:, None, None] ** 2 + kx[None, :, None] ** 2 + kz[None, None, :] ** 2
    w = torch.full((n // 2 + 1,), 2.0, dtype=torch.float64, device=dev)
    w[0] = w[-1] = 1.0
    e = (u.abs() ** 2).sum(0) * w / float(n) ** 6  # 2 x energy density per stored mode
    shell = (k2.sqrt() + 0.5).long().flatten()
    spec = torch.zeros(int(shell.max()) + 1, dtype=torch.float64, device=dev).index_add_(0, shell, e.flatten())
    return {"ke": 0.5 * float(e.sum()), "spectrum": 0.5 * spec, "diss": nu * float((e * k2).sum())}


def accuracy_check(plan, uh0, u0, dt, n, steps, marks=(100,)):
    """The metric's accuracy clause and more: the FP32 step (this library) and the FP64
    plain form (complex128 cuFFT, same GPU) from the same initial field, compared after
    each of `marks` steps and after `steps`: relative kinetic-energy error (the criterion,
    1e-5), shell-spectrum errors (maximum over the shells 1 <= s <= kd of
    |E32 - E64| / E64, and the relative L2 error over those shells), the relative
    dissipation error and the relative L2 error of the whole half spectrum. Also times
    the FP64 comparator (CUDA events over its step loops only)."""
    import torch

    _, step64, _ = fp64_model(n, dt)
    kd = int(np.floor(2.0 / 3.0 * (n // 2 + 1) - 1e-12))
    uh32 = uh0.clone()
    uh64 = torch.fft.rfftn(torch.from_numpy(u0).to("cuda"), dim=(1, 2, 3))
    step64(uh64.clone())  # creates the cuFFT plans outside the timed loops (result discarded)
    torch.cuda.synchronize()
    ms64, done, out = 0.0, 0, []
    for m in sorted(set([k for k in marks if 0 < k < steps] + [steps])):
        plan.step(uh32, m - done)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(m - done):
            uh64 = step64(uh64)
        e1.record()
        torch.cuda.synchronize()
        ms64 += e0.elapsed_time(e1)
        done = m
        a, b = _spectral_stats(uh32, n), _spectral_stats(uh64, n)
        sa, sb = a["spectrum"][1 : kd + 1], b["spectrum"][1 : kd + 1]
        w = torch.full((n // 2 + 1,), 2.0, dtype=torch.float64, device="cuda")
        w[0] = w[-1] = 1.0
        d2 = float(((uh32.to(torch.complex128) - uh64).abs() ** 2 * w).sum())
        out.append({"steps": m, "ke_fp32": a["ke"], "ke_fp64": b["ke"], "rel_err": abs(a["ke"] - b["ke"]) / b["ke"],
                    "spectrum_max_rel_err": float(((sa - sb).abs() / sb).max()),
                    "spectrum_l2_rel_err": float(torch.linalg.vector_norm(sa - sb) / torch.linalg.vector_norm(sb)),
                    "dissipation_rel_err": abs(a["diss"] - b["diss"]) / b["diss"],
                    "field_l2_rel_err": (d2 / float((uh64.abs() ** 2 * w).sum())) ** 0.5})
    last = dict(out[-1])
    last["criterion"] = 1e-5
    last["shells"] = f"1..{kd}"
    last["earlier"] = out[:-1]
    del uh32, uh64
    return last, 1e3 * steps / ms64


def fp64_plain_rate(u0, dt, n, steps, warmup):
    import torch

    _, step, wts = fp64_model(n, dt)
    uh = torch.fft.rfftn(torch.from_numpy(u0).to("cuda"), dim=(1, 2, 3))
    step(uh.clone())  # creates the cuFFT plans outside the timed region (result discarded)
    for _ in range(warmup):
        uh = step(uh)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        uh = step(uh)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    # kinetic energy by Parseval on the half spectrum, FP64
    ke = 0.5 * float((wts * (uh.abs() ** 2).sum(0)).sum()) / float(n) ** 6
    return 1e3 / ms, ke


# ---------------------------------------------------------------------------------
# Differentiation workload: 128^3 HIT (Rogallo k4exp, k_p = 3, KE 0.5, constant power
# 0.1 on |k| <= 2, nu 5e-3), 20 RK4 steps at dt 2e-3, loss = MSE of the 32^3 spectral
# coarsening of the final velocity against a seeded target (the coarsened field of
# another seed). Gradient w.r.t. the initial half spectrum by the hand-written adjoint
# (per-step checkpoints, stages recomputed). Checks: FP64 central differences (step
# 1e-3 of a direction with the norm of u_hat0) on seeded random HIT directions, and
# the FP64 loss. Cost: adjoint step / forward step, CUDA events.
# ---------------------------------------------------------------------------------
def adjoint_cost(n, dt, reps=10):
    """Milliseconds of one forward step and of one adjoint step (l3es_adjoint_step: the
    three stages recomputed + four VJPs) of the headline HIT workload at n^3."""
    import torch

    from l3es import _native

    u0, _ = initial_field(n)
    plan = _native.Plan(dim=3, n=n, nu=NU, dt=dt, forcing="const_power", kf=KF, eps_inj=EPS_INJ)
    plan.autotune("")
    uh = torch.empty(plan.spec_shape, dtype=torch.complex64, device="cuda")
    plan.rfftn(torch.from_numpy(u0.astype(np.float32)).cuda(), uh)
    x, lam = uh.clone(), uh.clone()
    for _ in range(3):
        plan.step(x, 1)
        plan.adjoint_step(uh, lam)
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    ev[0].record()
    for _ in range(reps):
        plan.step(x, 1)
    ev[1].record()
    for _ in range(reps):
        plan.adjoint_step(uh, lam)
    ev[2].record()
    torch.cuda.synchronize()
    plan.check()
    fwd, adj = ev[0].elapsed_time(ev[1]) / reps, ev[1].elapsed_time(ev[2]) / reps
    return {"n": n, "fwd_ms_per_step": fwd, "adj_ms_per_step": adj, "adjoint_over_forward": adj / fwd}


def adjoint_check(dirs=16, n=128, c=32, steps=20, dt=2e-3, h=1e-3):
    import torch

    from l3es import adjoint as AD
    from l3es import init_fields as F
    from l3es import utils as U

    def hit(seed):
        u = F.init_u_hit(n, seed, spectrum="k4exp", kp=3.0)
        return u * np.sqrt(KE0 / (0.5 * np.mean(np.sum(u * u, axis=0))))

    plan = AD.make_plan(n, NU, 3, dt, "const_power", kf=KF, eps_inj=EPS_INJ)
    ip = AD.coarse_plan(3, n, c)

    def spec(u):
        out = torch.empty(plan.spec_shape, dtype=torch.complex64, device="cuda")
        plan.rfftn(torch.from_numpy(u.astype(np.float32)).cuda(), out)
        return out

    uh = spec(hit(SEED))
    target = U.spectral_filtering(torch.from_numpy(hit(SEED + 1).astype(np.float32)).cuda(), c).float().contiguous()
    loss, g = AD.loss_and_grad(uh, plan, steps, target, ip)
    # cost: one forward step vs one adjoint step (warm, CUDA events)
    x, lam = uh.clone(), g.clone()
    for _ in range(3):
        plan.step(x, 1)
        plan.adjoint_step(uh, lam)
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    reps = 20
    ev[0].record()
    for _ in range(reps):
        plan.step(x, 1)
    ev[1].record()
    for _ in range(reps):
        plan.adjoint_step(uh, lam)
    ev[2].record()
    torch.cuda.synchronize()
    fwd_ms, adj_ms = ev[0].elapsed_time(ev[1]) / reps, ev[1].elapsed_time(ev[2]) / reps
    # FP64 references: the plain form's step and the same coarse MSE in complex128
    _, step64, _ = fp64_model(n, dt)
    t64 = target.double()

    def loss64(u_hat):
        for _ in range(steps):
            u_hat = step64(u_hat)
        y = torch.fft.fftshift(torch.fft.fftn(torch.fft.irfftn(u_hat, s=(n, n, n), dim=(1, 2, 3)), dim=(1, 2, 3)),
                               dim=(1, 2, 3))
        sl = slice(n // 2 - c // 2, n // 2 + c // 2)
        y = torch.fft.ifftshift(y[:, sl, sl, sl], dim=(1, 2, 3))
        uc = (torch.fft.ifftn(y, dim=(1, 2, 3)) / (n / c) ** 3).real
        return float(((uc - t64) ** 2).mean())

    u64 = uh.to(torch.complex128)
    l64 = loss64(u64)
    g64 = g.to(torch.complex128)
    norm = float(torch.linalg.vector_norm(u64))
    ad, fd = [], []
    for k in range(dirs):
        d = spec(hit(100 + k)).to(torch.complex128)
        d *= norm / float(torch.linalg.vector_norm(d))
        fd.append((loss64(u64 + h * d) - loss64(u64 - h * d)) / (2 * h))
        ad.append(float((torch.conj(g64) * d).real.sum()))
    ad, fd = np.array(ad), np.array(fd)
    fd_check = None
    if dirs > 0:
        fd_check = {"directions": dirs, "step": h,
                    "reference": "FP64 plain form (complex128 cuFFT), central differences",
                    "max_abs_err_over_max_abs_dd": float(np.abs(ad - fd).max() / np.abs(ad).max()),
                    "max_rel_err_per_direction": float(np.max(np.abs(ad - fd) / np.abs(fd))), "criterion": 1e-4}
    # the combined step with particles: loss = sum(lam * u_r) of the 32^3 particles'
    # NUFFT velocities after the 20 steps; gradient = adjoint steps + interpolation adjoint
    from l3es import adjoint as AD_

    npart = c**3
    rng = np.random.default_rng(SEED + 7)
    r = torch.from_numpy(rng.uniform(0.0, 2 * np.pi, (npart, 3))).cuda()
    lam_r = torch.from_numpy(rng.standard_normal((npart, 3))).cuda()
    ipp = AD_.particle_plan(3, n, c, npart)
    u_r = torch.empty(npart, 3, dtype=torch.float64, device="cuda")
    x = uh.clone()
    ck = [torch.empty_like(uh) for _ in range(steps)]
    for i in range(steps):
        ck[i].copy_(x)
        plan.step(x, 1)
    gp = torch.empty_like(uh)
    ipp.interp_vjp(r, lam_r, gp, backend="nufft")
    for i in range(steps - 1, -1, -1):
        plan.adjoint_step(ck[i], gp)
    # cost: forward combined step (DNS step, coarsening, NUFFT) vs its adjoint
    for _ in range(3):
        plan.step(x, 1)
        ipp.set_spectrum(x)
        ipp.interp(r, u_r, backend="nufft")
        plan.adjoint_step(uh, lam)
        ipp.interp_vjp(r, lam_r, lam, backend="nufft")
    torch.cuda.synchronize()
    ev[0].record()
    for _ in range(reps):
        plan.step(x, 1)
        ipp.set_spectrum(x)
        ipp.interp(r, u_r, backend="nufft")
    ev[1].record()
    for _ in range(reps):
        ipp.interp_vjp(r, lam_r, lam, backend="nufft")
        plan.adjoint_step(uh, lam)
    ev[2].record()
    torch.cuda.synchronize()
    cf_ms, ca_ms = ev[0].elapsed_time(ev[1]) / reps, ev[1].elapsed_time(ev[2]) / reps
    # FP64 reference: the plain form's trajectory and the exact spectral interpolation
    # (separable sums over the 32^3 coarse modes, chunks of particles)
    rr = r.double()
    kc = torch.fft.fftfreq(c, 1.0 / c, dtype=torch.float64, device="cuda")

    def ploss64(u_hat):
        for _ in range(steps):
            u_hat = step64(u_hat)
        y = torch.fft.fftshift(torch.fft.fftn(torch.fft.irfftn(u_hat, s=(n, n, n), dim=(1, 2, 3)), dim=(1, 2, 3)),
                               dim=(1, 2, 3))
        sl = slice(n // 2 - c // 2, n // 2 + c // 2)
        y = torch.fft.ifftshift(y[:, sl, sl, sl], dim=(1, 2, 3))
        U = torch.fft.fftn((torch.fft.ifftn(y, dim=(1, 2, 3)) / (n / c) ** 3).real, dim=(1, 2, 3))
        tot = 0.0
        for s0 in range(0, npart, 4096):
            p = rr[s0 : s0 + 4096]
            ex, ey, ez = (torch.exp(1j * p[:, d, None] * kc[None, :]) for d in range(3))
            t = torch.einsum("cabz,pz->cpab", U, ez)
            t = torch.einsum("cpab,pb->cpa", t, ey)
            v = torch.einsum("cpa,pa->cp", t, ex).real / c**3
            tot += float((v.T * lam_r[s0 : s0 + 4096]).sum())
        return tot

    pdirs = min(dirs, 4)
    gp64 = gp.to(torch.complex128)
    pad, pfd = [], []
    for k in range(pdirs):
        d = spec(hit(200 + k)).to(torch.complex128)
        d *= norm / float(torch.linalg.vector_norm(d))
        pfd.append((ploss64(u64 + h * d) - ploss64(u64 - h * d)) / (2 * h))
        pad.append(float((torch.conj(gp64) * d).real.sum()))
    pad, pfd = np.array(pad), np.array(pfd)
    particles = {
        "loss": f"sum(lam * u_r) of {npart} particles (NUFFT w=6 from the {c}^3 coarsening) after {steps} steps",
        "fwd_ms_per_step": cf_ms, "adj_ms_per_step": ca_ms, "adjoint_over_forward": ca_ms / cf_ms,
        "note": "forward: DNS step + coarsening + NUFFT interpolation; adjoint: step VJP (stages recomputed) + "
                "interpolation VJP (type-1 spread, forward FFT, deconvolution, coarse-to-fine adjoint)",
        "fd": None if pdirs == 0 else {
            "directions": pdirs, "step": h,
            "reference": "FP64 plain form + exact spectral interpolation (complex128), central differences",
            "max_rel_err_per_direction": float(np.max(np.abs(pad - pfd) / np.abs(pfd))), "criterion": 1e-4},
    }
    return {
        "workload": f"hit3d_{n} k_p=3 const_power, {steps} RK4 steps dt={dt}, loss = MSE of the {c}^3 coarsening vs "
                    "a seeded target",
        "fwd_ms_per_step": fwd_ms, "adj_ms_per_step": adj_ms, "adjoint_over_forward": adj_ms / fwd_ms,
        "target_ratio": 3.0,
        "loss_fp32": float(loss), "loss_fp64": l64, "loss_rel_err": abs(float(loss) - l64) / l64,
        "fd": fd_check,
        "particle_loss": particles,
    }


def run_adjoint(args):
    """The differentiation workload alone (one JSON line): time per adjoint step of the
    128^3, 20-step loss gradient relative to a forward step, and its checks."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import torch

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    res = adjoint_check(dirs=args.adjoint_dirs)
    line = {"metric": "adjoint RK4 step cost / forward step at 128^3 (differentiation workload)",
            "value": res["adjoint_over_forward"], "unit": "ratio", "higher_is_better": False, "n_gpus": 1,
            "dtype": "f32 (fp64 reductions)", "data": "synthetic", "config": {"workload": res["workload"]},
            "adjoint": res}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------------
# further single-trajectory configurations (keys of the headline line)
# ---------------------------------------------------------------------------------
def jittered_lattice(c, dim, seed, jitter=0.25):
    """c^dim particles on the cell centres of a c^dim lattice in [0, 2 pi)^dim, moved by
    up to +-jitter cells (seeded), wrapped into the box."""
    rng = np.random.default_rng(seed)
    h = 2 * np.pi / c
    ax = (np.arange(c) + 0.5) * h
    g = np.stack([a.ravel() for a in np.meshgrid(*([ax] * dim), indexing="ij")], 1)
    return np.mod(g + rng.uniform(-jitter, jitter, g.shape) * h, 2 * np.pi)


def _graph_rate(record, steps, warmup):
    """Steps/s of a step recorded as two ping-pong graphs (record(parity) -> Graph),
    CUDA events on the current stream."""
    import torch

    graphs = [record(0), record(1)]
    for i in range(max(warmup, 2)):
        graphs[i & 1].launch()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for i in range(steps):
        graphs[i & 1].launch()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    return 1e3 / ms, ms


def hit_ekin_tot_rate(steps, warmup, n=N_GRID):
    """The reference's own HIT configuration (configs/hit32_1.yaml: 256^3, nu = 2e-3,
    dt = 2e-3, ekin_tot forcing on 0 < |k| <= 3 holding the kinetic energy at 1.25,
    32^3 particles interpolated by NUFFT from the 32^3 coarsening and relaxed by SPH
    with relax_dt_factor 2 and u_ref 4 every step, as combined.py:122-142, :199 runs
    them). Initial field: init_u_hit's k^-5/3 spectrum, seed 42; particles: a jittered
    lattice (the reference reads a relaxed particle file, which is not shipped)."""
    import torch

    from l3es import _native
    from l3es import init_fields as F

    nu, dt, kf, e0, c, u_ref, factor = 2e-3, 2e-3, 3, 1.25, 32, 4.0, 2.0
    u = F.init_u_hit(n, 42)
    u *= np.sqrt(e0 / (0.5 * np.mean(np.sum(u * u, axis=0))))
    plan = _native.Plan(dim=3, n=n, nu=nu, dt=dt, forcing="ekin_tot", kf=kf, e_kin_init=e0)
    uh = torch.empty(plan.spec_shape, dtype=torch.complex64, device="cuda")
    plan.rfftn(torch.from_numpy(u.astype(np.float32)).cuda(), uh)
    npart = c**3
    ip = _native.InterpPlan(dim=3, ckp_n=c, n_fine=n, width=6, np_max=npart)
    sph = _native.SphPlan(3, c, 2 * np.pi, npart)
    r = [torch.from_numpy(jittered_lattice(c, 3, 42)).cuda(), torch.empty(npart, 3, dtype=torch.float64, device="cuda")]
    u_r, u_rel = (torch.empty(npart, 3, dtype=torch.float64, device="cuda") for _ in range(2))
    einj = torch.zeros(1, dtype=torch.float64, device="cuda")

    def record(parity):
        src, dst = (r[0], r[1]) if parity == 0 else (r[1], r[0])
        cap = _native.Graph.begin()
        plan.step(uh, 1, e_inj=einj, stream=cap)
        ip.set_spectrum(uh, stream=cap)
        ip.interp(src, u_r, backend="nufft", stream=cap)
        sph.relax_velocity(src, u_r, u_rel, dt, factor, u_ref, r_out=dst, stream=cap)
        return _native.Graph.end(cap)

    rate, ms = _graph_rate(record, steps, warmup)
    plan.check()
    ke = torch.zeros(1, dtype=torch.float64, device="cuda")
    plan.kinetic_energy(uh, ke)
    return {"value": rate, "unit": "steps/s", "ms_per_step": ms, "steps": steps, "ke_after": float(ke),
            "config": "reference configs/hit32_1.yaml: 256^3, nu 2e-3, dt 2e-3, ekin_tot kf=3 KE 1.25, "
                      "32^3 particles (jittered lattice) by NUFFT w=6 + SPH relaxation (factor 2, u_ref 4), "
                      "one graph launch per step"}


def kolm2d_rate(steps, warmup, n=256):
    """BASELINE's 2D Kolmogorov configuration: 256^2, f_x = sin(4 y), nu = 1e-3, linear
    drag 0.1, random-phase initial field band-limited to |k| <= 8 with kinetic energy
    0.5 (seed 0), dt = 1e-3; 64^2 particles on a jittered lattice interpolated by NUFFT
    (sigma 2, width 6) from the 64^2 spectral coarsening and advected (Euler) every step."""
    import torch

    from l3es import _native
    from l3es import init_fields as F

    nu, dt, c = 1e-3, 1e-3, 64
    u = F.init_u_random2d(n, 0, 8.0, 0.5)
    plan = _native.Plan(dim=2, n=n, nu=nu, dt=dt, kolm_k=4, kolm_amp=1.0, drag=0.1)
    uh = torch.empty(plan.spec_shape, dtype=torch.complex64, device="cuda")
    plan.rfftn(torch.from_numpy(u.astype(np.float32)).cuda(), uh)
    npart = c * c
    ip = _native.InterpPlan(dim=2, ckp_n=c, n_fine=n, width=6, np_max=npart)
    r = [torch.from_numpy(jittered_lattice(c, 2, 0)).cuda(), torch.empty(npart, 2, dtype=torch.float64, device="cuda")]
    u_r = torch.empty(npart, 2, dtype=torch.float64, device="cuda")

    def record(parity):
        src, dst = (r[0], r[1]) if parity == 0 else (r[1], r[0])
        cap = _native.Graph.begin()
        plan.step(uh, 1, stream=cap)
        ip.set_spectrum(uh, stream=cap)
        ip.interp(src, u_r, backend="nufft", dt=dt, r_out=dst, stream=cap)
        return _native.Graph.end(cap)

    k = max(steps, 1000)
    rate, ms = _graph_rate(record, k, warmup)
    plan.check()
    return {"value": rate, "unit": "steps/s", "ms_per_step": ms, "steps": k,
            "config": "2D Kolmogorov 256^2, sin(4y) forcing, nu 1e-3, drag 0.1, random2d |k|<=8 KE 0.5, dt 1e-3, "
                      "64^2 jittered particles by NUFFT w=6 from the 64^2 coarsening, Euler; one graph launch per step"}


# ---------------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------------
def run_ours(args):
    import torch

    from l3es import _native

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    n = args.n
    u0, dt = initial_field(n)
    plan = _native.Plan(dim=3, n=n, nu=NU, dt=dt, forcing="const_power", kf=KF, eps_inj=EPS_INJ)
    if args.schedule is not None:
        plan.set_schedule(dict(zip(plan.SCHEDULE_KEYS, args.schedule)))
        schedule = plan.schedule
    else:
        schedule = plan.autotune("")  # the library's autotuner, timed fresh (no cache file)
    uh = torch.empty(plan.spec_shape, dtype=torch.complex64, device="cuda")
    u_dev = torch.from_numpy(u0.astype(np.float32)).cuda()
    plan.rfftn(u_dev, uh)
    del u_dev
    uh0 = uh.clone()
    stream = torch.cuda.current_stream()
    r_host = particles(CKP_N)
    npart = r_host.shape[0]
    ip = _native.InterpPlan(dim=3, ckp_n=CKP_N, n_fine=n, width=6, np_max=npart)
    r_buf = [torch.from_numpy(r_host).cuda(), torch.empty(npart, 3, dtype=torch.float64, device="cuda")]
    u_r = torch.empty(npart, 3, dtype=torch.float64, device="cuda")

    def step():
        plan.step(uh, 1)
        if WITH_PARTICLES:
            # combined.py:97-130, :199: velocity from the post-step field at the old
            # positions, then the Euler shift
            ip.set_spectrum(uh)
            ip.interp(r_buf[0], u_r, backend="nufft", dt=dt, r_out=r_buf[1])
            r_buf.reverse()

    for _ in range(args.warmup):
        step()
    # the whole step recorded once per particle-buffer parity through the library's
    # graph API (l3es_graph_*): one launch per step instead of ~30
    graphs = []
    for src, dst in ((r_buf[0], r_buf[1]), (r_buf[1], r_buf[0])):
        cap = _native.Graph.begin()
        plan.step(uh, 1, stream=cap)
        if WITH_PARTICLES:
            ip.set_spectrum(uh, stream=cap)
            ip.interp(src, u_r, backend="nufft", dt=dt, r_out=dst, stream=cap)
        graphs.append(_native.Graph.end(cap))
    for i in range(2):  # graph warm-up (first launch uploads the graph)
        graphs[i].launch(stream)
    barrier()
    with Clocks(local) as clk:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for i in range(args.steps):
            graphs[i & 1].launch(stream)
        e1.record(stream)
        barrier()
    ms = e0.elapsed_time(e1) / args.steps
    clocks = clk.summary()
    ms, value = replica_throughput(ms, world, dist, device="cuda")

    # instrumented pass: per-kernel CUDA events for the roofline numerator/denominator
    plan.timing(True)
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    stats = plan.kernel_stats()
    plan.timing(False)
    plan.check()  # no kernel gave up a bounded wait during the timed or instrumented steps
    # launches of the particle layer per step (crop, prep, 3 grid passes, memset-free
    # binning: count + scan + scatter, gather)
    part_launches = 8 * args.steps if WITH_PARTICLES else 0
    launches = sum(v[0] for v in stats.values()) + part_launches
    top = max(stats.items(), key=lambda kv: kv[1][1])
    name, (nl, tms, tb) = top
    peak, peak_kind = _peaks()
    achieved = tb / (tms * 1e-3) / 1e9
    kernels = {k: {"launches": v[0], "ms_per_launch": v[1] / v[0], "share": v[1] / sum(x[1] for x in stats.values()),
                   "gbs": v[2] / (v[1] * 1e-3) / 1e9 if v[1] > 0 else None} for k, v in stats.items()}

    # the same step also returning the physical N^3 velocity each step, as the reference's
    # step_fn does (spectral_solver.py:114-118); the workload itself needs only the
    # coarsened field, which the step takes straight from u_hat
    with_u_out = None
    if not args.skip_baselines:
        u_phys = torch.empty(plan.phys_shape, dtype=torch.float32, device="cuda")
        graphs_u = []
        for src, dst in ((r_buf[0], r_buf[1]), (r_buf[1], r_buf[0])):
            cap = _native.Graph.begin()
            plan.step(uh, 1, u_out=u_phys, stream=cap)
            if WITH_PARTICLES:
                ip.set_spectrum(uh, stream=cap)
                ip.interp(src, u_r, backend="nufft", dt=dt, r_out=dst, stream=cap)
            graphs_u.append(_native.Graph.end(cap))
        for i in range(4):
            graphs_u[i & 1].launch(stream)
        ku = max(10, min(args.steps, 50))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for i in range(ku):
            graphs_u[i & 1].launch(stream)
        e1.record(stream)
        torch.cuda.synchronize()
        mu = e0.elapsed_time(e1) / ku
        with_u_out = {"value": 1000.0 / mu, "unit": "steps/s", "ms_per_step": mu, "steps": ku,
                      "note": "the timed step plus the irfftn of the new state into a physical N^3 FP32 "
                              "velocity every step (what the reference's step_fn returns); not part of value"}
        del graphs_u, u_phys

    # end to end through the public API with host buffers: per step the state stays
    # resident (as in the reference), the step's scalar result (KE) comes back to host
    if args.skip_baselines:
        e2e_ms = float("nan")
    # end to end through the public API with host buffers, as the reference's combined
    # loop holds them: particle positions on the host go in, velocities, new positions
    # and the kinetic energy come back every step (the field state stays resident)
    ke_dev = torch.zeros(1, dtype=torch.float64, device="cuda")
    ke_host = torch.zeros(1, dtype=torch.float64).pin_memory()
    r_pin = torch.from_numpy(r_host).pin_memory()
    ur_pin = torch.empty(npart, 3, dtype=torch.float64).pin_memory()
    r_dev = torch.empty(npart, 3, dtype=torch.float64, device="cuda")
    r_new = torch.empty_like(r_dev)
    # device part of the step (DNS step, coarsening, NUFFT + advection, KE) as one graph;
    # the host copies run around each launch on the same stream
    cap = _native.Graph.begin()
    plan.step(uh, 1, ke=ke_dev, stream=cap)  # the step and the KE of the new state
    ip.set_spectrum(uh, stream=cap)
    ip.interp(r_dev, u_r, backend="nufft", dt=dt, r_out=r_new, stream=cap)
    g_e2e = _native.Graph.end(cap)
    nsteps_e2e = 0 if args.skip_baselines else args.steps
    # (a) host waits for every step before issuing the next
    barrier()
    t0 = time.perf_counter()
    for _ in range(nsteps_e2e):
        r_dev.copy_(r_pin, non_blocking=True)
        g_e2e.launch(stream)
        ur_pin.copy_(u_r, non_blocking=True)
        r_pin.copy_(r_new, non_blocking=True)
        ke_host.copy_(ke_dev, non_blocking=True)
        stream.synchronize()
    e2e_sync_ms = (time.perf_counter() - t0) * 1e3 / max(nsteps_e2e, 1)
    # (b) pipelined on two streams: the DNS step (with its KE) on the main stream, the
    # particle part on a second one: H2D of the positions, coarsening once the step's
    # field exists, interpolation + advection, D2H of u_r and the new positions. The next
    # DNS step waits only until the coarsening has read the field, so the interpolation
    # and the copies of step i run under the DNS of step i+1; the positions still travel
    # device -> pinned host -> device every step, and the host reads step i's results
    # (double-buffered pinned outputs, one event wait per step) while step i+1 runs.
    cap = _native.Graph.begin()
    plan.step(uh, 1, ke=ke_dev, stream=cap)
    g_dns = _native.Graph.end(cap)
    cap = _native.Graph.begin()
    ip.set_spectrum(uh, stream=cap)
    g_crop = _native.Graph.end(cap)
    cap = _native.Graph.begin()
    ip.interp(r_dev, u_r, backend="nufft", dt=dt, r_out=r_new, stream=cap)
    g_part = _native.Graph.end(cap)
    side = torch.cuda.Stream()
    ev_dns, ev_crop = torch.cuda.Event(), torch.cuda.Event()
    ur_pins = [ur_pin, torch.empty_like(ur_pin).pin_memory()]
    ke_hosts = [ke_host, torch.zeros(1, dtype=torch.float64).pin_memory()]
    evs = [torch.cuda.Event(), torch.cuda.Event()]
    ke_seen = []
    barrier()
    t0 = time.perf_counter()
    for i in range(nsteps_e2e):
        b = i & 1
        if i > 0:
            stream.wait_event(ev_crop)  # the previous coarsening has read the field
        g_dns.launch(stream)
        ke_hosts[b].copy_(ke_dev, non_blocking=True)
        ev_dns.record(stream)
        with torch.cuda.stream(side):
            r_dev.copy_(r_pin, non_blocking=True)  # after the previous step's D2H (same stream)
            side.wait_event(ev_dns)
            g_crop.launch(side)
            ev_crop.record(side)
            g_part.launch(side)
            ur_pins[b].copy_(u_r, non_blocking=True)
            r_pin.copy_(r_new, non_blocking=True)
            evs[b].record(side)  # also after the KE copy: the side stream waited on ev_dns
        if i > 0:
            evs[b ^ 1].synchronize()
            ke_seen.append(float(ke_hosts[b ^ 1][0]))
    if nsteps_e2e:
        evs[(nsteps_e2e - 1) & 1].synchronize()
        ke_seen.append(float(ke_hosts[(nsteps_e2e - 1) & 1][0]))
        e2e_ms = (time.perf_counter() - t0) * 1e3 / nsteps_e2e
        assert len(ke_seen) == nsteps_e2e and all(np.isfinite(ke_seen))
    h2d = npart * 3 * 8
    d2h = 2 * npart * 3 * 8 + 8

    # accuracy clause of the metric: kinetic energy of the FP32 step after K steps vs
    # the FP64 plain form from the same initial field (which also times the comparator)
    ke_check = None
    fp64_rate = None
    if rank == 0 and not args.skip_baselines and args.ke_steps > 0:
        ke_check, fp64_rate = accuracy_check(plan, uh0, u0, dt, n, args.ke_steps, marks=(100,))
        plan.check()  # no blow-up and no bounded wait gave up over the K steps

    adjoint = None
    if rank == 0 and not args.skip_baselines and args.adjoint_dirs > 0:
        adjoint = adjoint_check(dirs=args.adjoint_dirs)
        # the same cost ratio on the headline 256^3 workload (no gradient check there)
        adjoint["at_headline_size"] = adjoint_cost(n, dt)
    extra = {}
    if rank == 0 and not args.skip_baselines:
        extra["hit_ekin_tot"] = hit_ekin_tot_rate(args.steps, args.warmup)
        extra["kolm2d_256"] = kolm2d_rate(args.steps, args.warmup)
        b = run_batch24(args, emit=False)
        extra["batch24"] = {k: b[k] for k in ("value", "unit", "ms_per_step", "steps", "speedup_vs_sequential",
                                              "sequential", "schedules")}
        extra["batch24"]["workload"] = b["config"]["workload"]
        extra["batch24"]["batched"] = b["config"]["batched"]

    line = None
    if rank == 0 and args.skip_baselines:
        line = {"metric": METRIC, "value": value, "unit": "steps/s", "ms_per_step": ms, "kernels": kernels,
                "note": "--skip-baselines (profiling run): no comparator, CPU or e2e legs"}
    elif rank == 0:
        # FP64 plain comparator (timed by the KE check, else a few steps) and the CPU sample
        if fp64_rate is None:
            fp64_rate, _ = fp64_plain_rate(u0, dt, n, steps=max(2, min(args.steps, 5)), warmup=1)
        cpu_rate, cores = cpu_step_rate(n, 1, 0, u0=u0, dt=dt)
        traffic, traffic_note = _ncu_traffic(name)
        line = {
            "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (fp64 reductions)", "data": "synthetic",
            "config": {"workload": f"hit3d_{n}_forced_const_power_particles{CKP_N}^3", "n": n, "nu": NU, "dt": dt,
                       "particles": f"{npart} uniform, NUFFT sigma=2 w=6 from the {CKP_N}^3 coarsening, Euler",
                       "forcing": f"const_power eps={EPS_INJ} 0<|k|<={KF}", "init": f"rogallo k4exp kp={KP} KE={KE0}",
                       "parallelism": "replicas" if world > 1 else "1 gpu", "schedule": schedule,
                       "l2": "working set (~1.3 GB) larger than L2, no flush"},
            "roofline": {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                         "traffic_source": traffic_note, "algo_bytes_per_launch": tb / nl,
                         "ms_per_launch": tms / nl},
            "kernels": kernels,
            "fp64_plain": {"value": fp64_rate, "unit": "steps/s", "speedup": value / world / fp64_rate,
                           "note": "reference algorithm restated with torch.fft (cuFFT) in complex128, same GPU"},
            "ke_check": ke_check,
            "adjoint": adjoint,
            "cpu_baseline": {"value": cpu_rate, "unit": "steps/s", "cores": cores, "kind": "port",
                             "sample": f"1 step at {n}^3 (RK4 + filter + NUFFT + advection), FP64 NumPy/SciPy"},
            "e2e": {"value": 1e3 / e2e_ms, "unit": "steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "synced_each_step": 1e3 / e2e_sync_ms,
                    "note": "host-timed through the public API: every step copies the pinned host positions in "
                            "and the velocities, new positions and KE out; value: the DNS step and the particle "
                            "part (positions in, coarsening, interpolation + advection, results out) as library "
                            "graphs on two streams, the particle part and copies of step i under the DNS of step "
                            "i+1, the host reading step i's results while step i+1 runs; synced_each_step: one "
                            "graph per step and the host waits for every step before the next"},
            "with_u_out": with_u_out,
            **extra,
            "gpu_launches": launches,
            "clocks": clocks,
            "workspace_gb": plan.workspace_bytes / 1e9,
        }
    del uh0
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    if line is not None:
        print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------------
# 24 mixed trajectories: 16 2D Kolmogorov runs (8 at 128^2, 6 at 256^2, 2 at 512^2,
# nu in [5e-4, 2e-3], 32^2 particles each) and 8 3D HIT runs (6 at 64^3, 2 at 128^3,
# Rogallo k4exp kp=4), seeds 0-23. Batched: one plan per size with per-trajectory
# viscosity, the whole step (DNS + particles) recorded as one CUDA graph. Sequential:
# one plan per trajectory, launched one after another.
# ---------------------------------------------------------------------------------
BATCH_GROUPS = [(2, 128, 8), (2, 256, 6), (2, 512, 2), (3, 64, 6), (3, 128, 2)]


def _batch_runs():
    from l3es import init_fields as F

    runs, seed = [], 0
    nus2d = np.linspace(5e-4, 2e-3, 16)
    i2 = 0
    for dim, n, count in BATCH_GROUPS:
        for _ in range(count):
            if dim == 2:
                u = F.init_u_random2d(n, seed)
                nu = float(nus2d[i2])
                i2 += 1
                dt = 1e-3
            else:
                u = F.init_u_hit(n, seed, spectrum="k4exp", kp=4.0)
                u *= np.sqrt(0.5 / (0.5 * np.mean(np.sum(u * u, axis=0))))
                nu = 5e-3
                dx = 2 * np.pi / n
                dt = float(CFL / (np.abs(u).max(axis=(1, 2, 3)) / dx + nu / dx**2).min())
            runs.append(dict(dim=dim, n=n, nu=nu, dt=dt, u=u, seed=seed))
            seed += 1
    return runs


def run_batch24(args, emit=True):
    """Times the 24-trajectory workload; prints its JSON line (emit) or returns it."""
    import torch

    from l3es import _native

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    runs = _batch_runs()
    points = sum(r["n"] ** r["dim"] for r in runs)
    kw2 = dict(kolm_k=4, kolm_amp=1.0, drag=0.1)

    def spec(plan, u, dim, n):
        uh = torch.empty((3, n, n, n // 2 + 1) if dim == 3 else (3, n, n // 2 + 1), dtype=torch.complex64,
                         device="cuda")
        tmp = _native.Plan(dim=dim, n=n, nu=0.0, dt=1.0)
        tmp.rfftn(torch.from_numpy(u.astype(np.float32)).cuda(), uh)
        return uh

    def particles2d(seed):
        rng = np.random.default_rng(100 + seed)
        ax = (np.arange(32) + 0.5) * 2 * np.pi / 32
        gx, gy = np.meshgrid(ax, ax, indexing="ij")
        r = np.stack([gx.ravel(), gy.ravel()], 1) + rng.uniform(-0.25, 0.25, (1024, 2)) * 2 * np.pi / 32
        return torch.from_numpy(np.mod(r, 2 * np.pi)).cuda()

    # batched: one plan per size (autotuned), one graph per step
    groups, pos, schedules = [], 0, {}
    for dim, n, count in BATCH_GROUPS:
        rs = runs[pos : pos + count]
        pos += count
        dt = min(r["dt"] for r in rs)
        pl = _native.Plan(dim=dim, n=n, nu=0.0, dt=dt, batch=count, **(kw2 if dim == 2 else {}))
        pl.set_nu([r["nu"] for r in rs])
        schedules[f"{dim}d_{n}x{count}"] = pl.autotune("")
        uh = torch.stack([spec(pl, r["u"], dim, n) for r in rs]).contiguous()
        part = None
        if dim == 2:
            # one batched interpolator per size: each particle kernel launches once for the
            # group's trajectories ([count][1024][2] positions)
            ip = _native.InterpPlan(dim=2, ckp_n=32, n_fine=n, np_max=1024, batch=count)
            rr = [torch.stack([particles2d(r["seed"]) for r in rs]).contiguous(),
                  torch.empty(count, 1024, 2, dtype=torch.float64, device="cuda")]
            part = (ip, rr, torch.empty(count, 1024, 2, dtype=torch.float64, device="cuda"), dt)
        groups.append((pl, uh, part))

    def record(graph_pingpong):
        # one graph branch per grid size: its batched DNS step, then its batched particle
        # update; the sizes run side by side
        cap = _native.Graph.begin()
        for pl, uh, part in groups:
            br = _native.Graph.fork(cap)
            pl.step(uh, 1, stream=br)
            if part is not None:
                ip, rr, ur, dt = part
                ip.set_spectrum(uh, stream=br)
                src, dst = (rr[0], rr[1]) if graph_pingpong == 0 else (rr[1], rr[0])
                ip.interp(src, ur, dt=dt, r_out=dst, stream=br)
            _native.Graph.join(cap, br)
        return _native.Graph.end(cap)

    graphs = [record(0), record(1)]
    steps = args.batch_steps
    for i in range(args.warmup):
        graphs[i % 2].launch()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        e0.record()
        for i in range(steps):
            graphs[i % 2].launch()
        e1.record()
        torch.cuda.synchronize()
    t_batched = e0.elapsed_time(e1) / 1e3
    batched_rate = points * steps / t_batched

    # sequential per-run launches (no batching, no graph)
    singles = []
    for r in runs:
        pl = _native.Plan(dim=r["dim"], n=r["n"], nu=r["nu"], dt=r["dt"], **(kw2 if r["dim"] == 2 else {}))
        uh = spec(pl, r["u"], r["dim"], r["n"])
        part = None
        if r["dim"] == 2:
            ip = _native.InterpPlan(dim=2, ckp_n=32, n_fine=r["n"], np_max=1024)
            part = (ip, [particles2d(r["seed"]), torch.empty(1024, 2, dtype=torch.float64, device="cuda")],
                    torch.empty(1024, 2, dtype=torch.float64, device="cuda"))
        singles.append((pl, uh, part, r["dt"]))
    seq_steps = max(10, steps // 5)

    def seq_step():
        for pl, uh, part, dt in singles:
            pl.step(uh, 1)
            if part is not None:
                ip, rr, ur = part
                ip.set_spectrum(uh)
                ip.interp(rr[0], ur, dt=dt, r_out=rr[1])
                rr.reverse()

    for _ in range(args.warmup):
        seq_step()
    torch.cuda.synchronize()
    e0.record()
    for _ in range(seq_steps):
        seq_step()
    e1.record()
    torch.cuda.synchronize()
    t_seq = e0.elapsed_time(e1) / 1e3
    seq_rate = points * seq_steps / t_seq
    line = {
        "metric": "grid-point updates/s, 24 mixed 2D/3D trajectories (DNS + particles)", "value": batched_rate,
        "unit": "grid-point updates/s", "n_gpus": 1, "steps": steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * t_batched / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (fp64 reductions)", "data": "synthetic",
        "config": {"workload": "batch24: 2D Kolmogorov 8x128^2 + 6x256^2 + 2x512^2 (32^2 particles each), "
                               "3D HIT 6x64^3 + 2x128^3", "grid_points_per_step": points,
                   "batched": "5 step plans (one per size, per-trajectory nu) + 3 batched particle plans (one per 2D "
                              "size), one CUDA graph per step with one branch per size (concurrent)"},
        "sequential": {"value": seq_rate, "steps": seq_steps, "ms_per_step": 1e3 * t_seq / seq_steps,
                       "note": "24 single-trajectory plans launched one after another"},
        "speedup_vs_sequential": batched_rate / seq_rate,
        "schedules": schedules,
        "clocks": clk.summary(),
    }
    if not emit:
        return line
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_GRID)
    ap.add_argument("--workload", default="hit256", choices=["hit256", "batch24", "adjoint", "kolm2d"],
                    help="hit256: the metric's 256^3 step; batch24: 24 mixed trajectories; "
                         "adjoint: the 128^3 differentiation workload alone; kolm2d: the 2D Kolmogorov "
                         "256^2 configuration alone (its --steps steps, at least 1000)")
    ap.add_argument("--batch-steps", type=int, default=500)
    ap.add_argument("--ke-steps", type=int, default=1000,
                    help="steps of the FP32-vs-FP64 accuracy check: kinetic energy (the metric's clause), "
                         "spectrum, dissipation and field errors (0 = skip)")
    ap.add_argument("--adjoint-dirs", type=int, default=16,
                    help="directions of the 128^3 adjoint finite-difference check (0 = skip the adjoint leg)")
    ap.add_argument("--skip-baselines", action="store_true",
                    help="profiling runs: time our step only (no FP64 plain, CPU or e2e legs)")
    ap.add_argument("--record-traffic", metavar="NCU_CSV", default=None,
                    help="no benchmark: turn an ncu DRAM launch list of the 256^3 step into the JSON traffic record "
                         "(--traffic-out) that the headline's roofline.traffic reads")
    ap.add_argument("--traffic-out", default=TRAFFIC_JSON)
    ap.add_argument("--traffic-command", default="", help="the ncu command that made NCU_CSV (stored in the record)")
    ap.add_argument("--schedule", default=None, metavar="X,Y,LINE,BAND",
                    help="set the 256^3 plan's kernel schedule (x_bulk,y_radix8,line_pair,band_bulk) instead of "
                         "autotuning it: profiling runs under ncu, whose serialised launches would steer the "
                         "autotuner elsewhere, use the schedule the plain run chose")
    args = ap.parse_args()
    if args.schedule is not None:
        vals = [int(v) for v in args.schedule.split(",")]
        if len(vals) != 4:
            ap.error("--schedule takes four comma-separated integers")
        args.schedule = vals
    if args.record_traffic:
        rec = record_traffic(args.record_traffic, args.traffic_out, args.traffic_command)
        print(json.dumps({k: v["traffic_per_launch"] for k, v in rec["kernels"].items()}))
        return 0
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "adjoint":
        return run_adjoint(args)
    if args.workload == "kolm2d":
        print(json.dumps(kolm2d_rate(args.steps, args.warmup)), flush=True)
        return 0
    return run_batch24(args) if args.workload == "batch24" else run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
