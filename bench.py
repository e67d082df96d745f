"""Benchmark of the particle step: particle-steps/s on one GB300 (or N replicas).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload box512_corrected] [--form fp32mlp|fp32|fp64]

The default line is the corrected step: the FP32 form with the learned
correction fused into its advance (the committed network, BF16 tcgen05
inference per particle and stage) on 512^3 cells x 2^27 particles with
d_p/dx 0.5 and mass loading 1.0; the plain FP32 step and the FP64 drop-in run
beside it on the same inputs (fp32_plain, fp64_dropin).

A step is one RK4 step (4 stages + the per-step reorder) of every particle:
interpolation, advance, wrap, and the concentration, momentum and energy
deposits. Inputs are seeded synthetic fields and particles of the workload's
shapes (first_repo_gb300/csrc/pstep_gen.c); no dataset is involved.

value  : particle-steps/s with everything resident in HBM (CUDA events around
         K steps on the library's stream), summed over ranks.
e2e    : the same metric through the C ABI with host buffers: per step the
         particle state and gas fields are copied in from pinned host memory and
         the particle state and the deposited fields copied back.
roofline: the dominant kernel phase, algorithmic bytes per launch / its mean
         launch time (CUDA events around the phase during the timed region).
cpu_baseline: the oracle (C restatement of the reference step, single thread as
         the reference runs per rank) on a bounded sample of the workload.
--impl reference: the reference's CPU step (the oracle port; the reference's own
         build needs its sources, which exist only where it was compiled) on
         all host cores, one independent single-rank instance per core.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from first_repo_gb300 import config, gen  # noqa: E402

# Algorithmic (compulsory) bytes, FP64 drop-in form, per particle per stage of
# each phase, and per ghosted cell per launch. Keep in step with the kernels.
#   advance  k=0 reads base(7) + RHS_T + x_int record (3 frac + key) = 92 B,
#            writes new(7) + np1(7) + new record(3 frac + key) + RHS_T + RHS_u(3) + leave code = 173 B;
#            k=1..3 also read *_int(7) and *_np1(7) = +112 B;  fields U(3) and T read once per launch.
FP64_ADVANCE_BYTES = {0: 92 + 173, 1: 92 + 173 + 112, 2: 92 + 173 + 112, 3: 92 + 173 + 112}
FP64_ADVANCE_CELL_BYTES = 4 * 8
# FP32 form: a particle set is 32 B (cell + 3 offsets + u,v,w,T).
#   k=0 reads base + RHS_T = 36 B; writes *_new + *_np1 + RHS_u(3) + RHS_T = 80 B
#   k=1..3 read base, *_int, *_np1 + RHS_T = 100 B; write 80 B.  fp32 fields U(3), T once per launch.
FP32_ADVANCE_BYTES = {0: 36 + 80, 1: 100 + 80, 2: 100 + 80, 3: 100 + 80}
FP32_ADVANCE_CELL_BYTES = 4 * 4
# with the learned correction the advance also reads and writes the drive state
# (slip 3 + temperature difference, bf16 x 4) and reads the kept network output (bf16 x 4):
# +24 B per particle and stage.
FP32MLP_ADVANCE_EXTRA = 24
# The network kernel (once per step): x_int cell + offsets + u,v,w (28 B), the drive state
# (8 B), the network output written (8 B) = 44 B per particle; the velocity field (3 fp32)
# once per launch; the weights (13 KB) once per CTA.
FP32MLP_NETWORK_BYTES = (44.0, 12.0)
# Deposits, per particle and per cell of one launch:
#   FP32 (one fused walk): *_int cell+offsets (16) + RHS_u (12) + *_new cell+offsets (16) + RHS_T (4) = 48 B;
#        per cell: cell_start (4) + five fp64 fields written (40) = 44 B.
#   FP64 int deposit: x_int record (3 frac + key = 28) + RHS_u (24) = 52 B; per cell: cell_start (4) +
#        four fp64 fields written (32) = 36 B.   FP64 temperature deposit: x_new record (28) + RHS_T (8) = 36 B;
#        per cell: cell_start (4) + one field (8) = 12 B.
#   FP64 counting sort: key read twice + index written (12 B); per cell: counts/scan/cursor (~20 B).
PHASE_BYTES = {
    ("fp32", "advance"): (sum(FP32_ADVANCE_BYTES.values()) / 4.0, FP32_ADVANCE_CELL_BYTES),
    ("fp32", "deposit_int"): (48.0, 44.0),
    ("fp32mlp", "advance"): (sum(FP32_ADVANCE_BYTES.values()) / 4.0 + FP32MLP_ADVANCE_EXTRA, FP32_ADVANCE_CELL_BYTES),
    ("fp32mlp", "deposit_int"): (48.0, 44.0),
    ("fp32mlp", "network"): FP32MLP_NETWORK_BYTES,
    ("fp64", "advance"): (sum(FP64_ADVANCE_BYTES.values()) / 4.0, FP64_ADVANCE_CELL_BYTES),
    ("fp64", "deposit_int"): (52.0, 36.0),
    ("fp64", "deposit_temp"): (36.0, 12.0),
    ("fp64", "sort"): (12.0, 20.0),
}

MEASURED_PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM = 6800.0


def rank_info():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")),
            int(os.environ.get("WORLD_SIZE", "1")))


def max_over_ranks(x: float, dist, device: str) -> float:
    """The largest value over the ranks (the timed region's time is the slowest rank's)."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(world: int, n_per_rank: int, ms_per_step: float) -> float:
    """Whole-job particle-steps/s: every rank steps its own replica of n particles."""
    return world * n_per_rank / (ms_per_step / 1e3)


class Clocks:
    """nvidia-smi sampled every 200 ms while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.rows = []
        self.proc = None
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.t:
            self.t.join(timeout=2)

    def summary(self):
        sm = [float(r[1]) for r in self.rows if len(r) > 8 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 8 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            if len(r) > 8:
                for nm, v in zip(names, r[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def peaks():
    try:
        with open(MEASURED_PEAKS) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM, "fallback"


def make_inputs(wl):
    t0 = time.time()
    case = gen.make_case(wl.n, wl.n_particles, wl.seed, wl.clustered, nblobs=wl.nblobs)
    bp = config.box_params(wl.n, wl.n_particles, dp_over_dx=wl.dp_over_dx, mass_loading=wl.mass_loading)
    fields = [gen.ghost(case[k]) for k in ("ux", "uy", "uz", "T")]
    return case, bp, fields, time.time() - t0


_PINNED = []  # keeps the pinned host allocations alive


def pinned_like(a: np.ndarray) -> np.ndarray:
    import torch
    t = torch.empty(a.shape, dtype=torch.float64 if a.dtype == np.float64 else torch.int32, pin_memory=True)
    _PINNED.append(t)
    out = t.numpy()
    out[...] = a
    return out


def fp32_error_report(g32, g64, L: float, n_cells: int) -> dict:
    """The FP32 form's error against the FP64 step run on the same inputs for the same
    number of steps, matched by particle id and computed on the device.

    Per particle, `*_max` is the largest error and `*_bulk` the largest over all but a
    fraction 1e-6 of the particles: the reference's face-normal interpolation
    (particle.cpp:340-360) is piecewise constant across the other two axes, so a particle
    whose stage position lies within the fp32 resolution of a cell face (about 1e-7 cells)
    can take the neighbouring cell's transverse velocity in one form and not the other, an
    O(dx |grad u|) difference for that particle; `*_count` counts particles beyond 1e-5.
      position_cells            |x32 - x64| (periodic) in cell units
      velocity_rel              |u32 - u64| / |u64| (velocity vectors)
      temperature_rel           |T32 - T64| / |T64|
      rhs_t_rel_to_max          |RHS_T32 - RHS_T64| / max |RHS_T64|
      fields                    per deposited field max |f32 - f64| / max |f64| (C: interior)
      fields_l2                 per deposited field ||f32 - f64|| / ||f64|| over the interior
      energy_mean_rel           |mean32 - mean64| / |mean64|
      momentum_rel_to_abs       per component |sum32 - sum64| / sum |RHS_RU64| over the interior
    """
    import torch
    dev = "cuda"
    n = g32.np
    if g64.np != n:
        raise ValueError("populations differ in size")
    k_out = max(1, int(1e-6 * n))

    def arr(g, name, dtype=torch.float64):
        t = torch.empty(n, dtype=dtype, device=dev)
        g.array(name, out=t)
        return t

    def stats(name, e, rep):
        rep[name + "_max"] = float(e.max())
        rep[name + "_bulk"] = float(torch.topk(e, k_out + 1).values[-1])
        rep[name + "_count"] = int((e > 1e-5).sum())

    i32 = torch.argsort(arr(g32, "flag", torch.int32))
    i64 = torch.argsort(arr(g64, "flag", torch.int32))
    if not torch.equal(arr(g32, "flag", torch.int32)[i32], arr(g64, "flag", torch.int32)[i64]):
        raise ValueError("particle ids differ")
    rep = {"particles": n, "bulk_excludes": k_out}
    dx = L / n_cells
    pos = torch.zeros(n, dtype=torch.float64, device=dev)
    for k in ("x", "y", "z"):
        d = arr(g32, k)[i32] - arr(g64, k)[i64]
        d = torch.remainder(d + L / 2, L) - L / 2
        pos = torch.maximum(pos, d.abs() / dx)
    stats("position_cells", pos, rep)
    del pos
    du = torch.zeros(n, dtype=torch.float64, device=dev)
    sp = torch.zeros(n, dtype=torch.float64, device=dev)
    for k in ("u", "v", "w"):
        a, b = arr(g32, k)[i32], arr(g64, k)[i64]
        du += (a - b) ** 2
        sp += b ** 2
        del a, b
    stats("velocity_rel", torch.sqrt(du) / torch.sqrt(sp).clamp_min(1e-300), rep)
    del du, sp
    a, b = arr(g32, "T")[i32], arr(g64, "T")[i64]
    stats("temperature_rel", (a - b).abs() / b.abs().clamp_min(1e-300), rep)
    a, b = arr(g32, "RHS_T")[i32], arr(g64, "RHS_T")[i64]
    stats("rhs_t_rel_to_max", (a - b).abs() / b.abs().max().clamp_min(1e-300), rep)
    del a, b
    g = n_cells + 2
    fields, fields_l2, mom = {}, {}, {}
    s32, s64 = g32.momentum_sums(), g64.momentum_sums()
    for i, name in enumerate(("C", "RHS_RU_x", "RHS_RU_y", "RHS_RU_z", "RHS_Part_Temp")):
        a = torch.empty(g ** 3, dtype=torch.float64, device=dev)
        b = torch.empty(g ** 3, dtype=torch.float64, device=dev)
        g32.field(name, out=a)
        g64.field(name, out=b)
        a = a.view(g, g, g)[1:-1, 1:-1, 1:-1]
        b = b.view(g, g, g)[1:-1, 1:-1, 1:-1]
        fields[name] = float((a - b).abs().max() / b.abs().max().clamp_min(1e-300))
        fields_l2[name] = float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b).clamp_min(1e-300))
        if 1 <= i <= 3:
            mom[name] = abs(s32[i - 1] - s64[i - 1]) / max(float(b.abs().sum()), 1e-300)
        del a, b
    rep["fields"] = fields
    rep["fields_l2"] = fields_l2
    rep["momentum_rel_to_abs"] = mom
    e32, e64 = g32.energy_mean(), g64.energy_mean()
    rep["energy_mean_rel"] = abs(e32 - e64) / max(abs(e64), 1e-300)
    torch.cuda.empty_cache()
    return rep


def particle_stats(g, u_fields_dev, L: float, n_cells: int) -> dict:
    """Slip-velocity and particle-temperature statistics of a population, on the device:
    the slip is u_p - U(x_p) with U the bound gas velocity interpolated at the particle's
    position as gas2part_velocity does (particle.cpp:340-360: face-normal linear, ghosted
    index (int)(x/dx) + 1). u_fields_dev: the three ghosted velocity fields as flat fp64
    device tensors."""
    import torch
    dev = "cuda"
    n = g.np
    gs = n_cells + 2
    idx = n_cells / L

    def arr(name):
        t = torch.empty(n, dtype=torch.float64, device=dev)
        g.array(name, out=t)
        return t

    pos = [arr(k) for k in ("x", "y", "z")]
    # clamped into the ghosted range so that no index can leave the arrays (a position at
    # x = L, which the FP64 form flags as out of range, reads the last interior face pair)
    cell = [torch.floor(p * idx).clamp(0, n_cells - 1) for p in pos]
    frac = [(p * idx - c).clamp(0.0, 1.0) for p, c in zip(pos, cell)]
    ci = [c.to(torch.int64) + 1 for c in cell]
    del pos, cell
    slip2 = torch.zeros(n, dtype=torch.float64, device=dev)
    for d, name in enumerate(("u", "v", "w")):
        lo = (ci[2] * gs + ci[1]) * gs + ci[0]
        step = (1, gs, gs * gs)[d]
        f = u_fields_dev[d]
        ug = frac[d] * f[lo + step] + (1 - frac[d]) * f[lo]
        slip2 += (arr(name) - ug) ** 2
        del lo, ug
    t = arr("T")
    out = {"slip_rms": float(torch.sqrt(slip2.mean())), "slip_mean": float(torch.sqrt(slip2).mean()),
           "T_mean": float(t.mean()), "T_rms": float(torch.sqrt(((t - t.mean()) ** 2).mean())),
           "T_max": float(t.max())}
    del slip2, t, frac, ci
    torch.cuda.empty_cache()
    return out


def stats_difference(a: dict, b: dict) -> dict:
    """a - b and (a - b) / |b| for each statistic"""
    return {k: {"diff": a[k] - b[k], "rel": (a[k] - b[k]) / abs(b[k]) if b[k] else None} for k in a}


def cpu_sample_rate(n_cells=160, count=1 << 22, steps=2, seed=77, clustered=True):
    """Oracle (single thread) on a bounded sample with the workload's density and construction."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    case = gen.make_case(n_cells, count, seed, clustered)
    bp = config.box_params(n_cells, count)
    o = pyoracle.Oracle(bp.step_config(), count)
    o.load(case["x"], case["y"], case["z"], case["u"], case["v"], case["w"], case["t"], case["flag"])
    ux, uy, uz, tf = (gen.ghost(case[k]) for k in ("ux", "uy", "uz", "T"))
    o.prime(tf)
    t0 = time.perf_counter()
    o.run(steps, ux, uy, uz, tf)
    dt = time.perf_counter() - t0
    return count * steps / dt, dt


def _ref_worker(args):
    n_cells, count, steps, seed = args
    rate, dt = cpu_sample_rate(n_cells, count, steps, seed)
    return rate, dt


def run_reference(args, wl):
    rank, _, world = rank_info()
    if rank != 0:
        return
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    n_cells, count = 128, 1 << 21
    ctx = mp.get_context("spawn")
    rates = []
    t_all = []
    # warm-up: one step on one core (builds nothing new; page-in of the library)
    for _ in range(max(1, args.warmup // 3)):
        cpu_sample_rate(32, 1 << 15, 1)
    with ctx.Pool(cores) as pool:
        for s in range(args.steps):
            t0 = time.perf_counter()
            res = pool.map(_ref_worker, [(n_cells, count, 1, 1000 + 7 * i + s) for i in range(cores)])
            wall = time.perf_counter() - t0
            slowest = max(r[1] for r in res)
            rates.append(cores * count / slowest)
            t_all.append(wall)
    value = float(np.median(rates))
    # ms_per_step and steps describe what ran: each timed step is one RK4 step of every
    # instance (all cores at once), and its time is the wall time of that step
    step_ms = 1e3 * float(np.median(t_all))
    line = {
        "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "impl": "reference",
        "config": {"workload": wl.name, "cells": wl.n ** 3, "particles": wl.n_particles,
                   "same_config": False,
                   "sample": f"{cores} independent single-rank instances x {count} particles on {n_cells}^3 "
                             "(the workload's particle density and construction), 1 RK4 step each per timed step; "
                             "the reference cannot be constructed at the workload's size (int Buffer_max_size "
                             "overflows, particle.cpp:23-26), so the rate is a per-particle-step CPU rate"},
        "per_particle_step_extrapolation": {
            "ms_per_workload_step": 1e3 * wl.n_particles / value,
            "note": f"time one step of the workload's {wl.n_particles} particles would take at the sample's rate "
                    "(not measured)"},
        "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": cores, "kind": "port",
                         "sample": f"{cores} x {count} particles on {n_cells}^3, 1 RK4 step per instance and "
                                   f"timed step, {args.steps} timed steps",
                         "note": "the oracle port (C restatement of the reference's particle step); measured on "
                                 "x86 it runs 1.44-1.53x faster than the reference's own build on the same cases, "
                                 "so this baseline favours the CPU"},
        "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="box512_corrected", choices=sorted(config.WORKLOADS))
    ap.add_argument("--form", default="fp32mlp", choices=["fp64", "fp32", "fp32mlp"])
    ap.add_argument("--no-fp64-line", action="store_true", help="skip timing the FP64 drop-in beside the FP32 form")
    ap.add_argument("--no-fp32-line", action="store_true", help="skip timing the plain FP32 step beside fp32mlp")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--c4-steps", type=int, default=100,
                    help="steps after which the corrected step's slip and temperature statistics are compared with "
                         "the FP64 drop-in's (untimed; needs the FP64 line; one GPU only, so that a multi-GPU run "
                         "holds its GPUs no longer than its timing needs)")
    args = ap.parse_args()
    wl = config.WORKLOADS[args.workload]
    if args.impl == "reference":
        run_reference(args, wl)
        return

    rank, local, world = rank_info()
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")

    from first_repo_gb300 import pstep
    case, bp, fields, gen_s = make_inputs(wl)
    form = pstep.FP64 if args.form == "fp64" else pstep.FP32
    flags = pstep.TRACK_ORDER if form == pstep.FP64 else 0
    n = wl.n_particles
    arrs = [np.ascontiguousarray(case[k]) for k in ("x", "y", "z", "u", "v", "w", "t", "flag")]
    corr_model = None
    if args.form == "fp32mlp":
        from first_repo_gb300 import learn
        corr_model = learn.load_model()
    nu_gas = bp.mu0 / bp.rho0

    tau = wl.tau_p()

    def make_step(frm, flg, with_model):
        h = pstep.ParticleStep(bp.step_config(), n, frm, flg)
        h.load(*arrs)
        if tau is not None:
            h.set_tau_p(tau)
        if with_model:
            h.set_correction(corr_model, nu_gas)
        h.bind_velocity(*fields[:3])
        h.bind_temperature(fields[3])
        h.prime()
        return h

    g = pstep.ParticleStep(bp.step_config(), n, form, flags)
    g.load(*arrs)
    if tau is not None:
        g.set_tau_p(tau)
    if corr_model is not None:
        g.set_correction(corr_model, nu_gas)
    g.bind_velocity(*fields[:3])
    g.bind_temperature(fields[3])
    g.prime()
    for _ in range(args.warmup):
        g.run(1)
    rc, wflags = g.check()
    if rc != 0:
        raise SystemExit(f"device check failed after warm-up: {wflags}")

    def barrier():
        if dist is not None:
            dist.barrier()

    clocks = Clocks(local)
    g.profile(True)
    g.profile_read()
    l0 = g.launches()
    clocks.start()
    barrier()
    g.run(args.steps)
    ms = g.last_run_ms()
    barrier()
    clocks.stop()
    launches = g.launches() - l0
    prof = g.profile_read()
    g.profile(False)
    ms = max_over_ranks(ms, dist, "cuda")
    ms_per_step = ms / args.steps
    value = job_rate(world, n, ms_per_step)

    # roofline of the dominant phase (live CUDA-event time of its launches in the timed region)
    peak, peak_kind = peaks()
    dom = max(prof, key=lambda p: prof[p][0])
    dom_ms, dom_cnt = prof[dom]
    roof = None
    model = PHASE_BYTES.get((args.form, dom))
    if model and dom_cnt:
        per_launch = n * model[0] + model[1] * (wl.n + 2) ** 3
        achieved = per_launch / (dom_ms / dom_cnt / 1e3) / 1e9
        traffic = None
        tf_path = os.path.join(ROOT, "profiles", "ncu_traffic.json")
        if os.path.exists(tf_path):
            with open(tf_path) as f:
                traffic = json.load(f).get(f"{args.form}_{dom}_{wl.name}")
        roof = {"kernel_phase": dom, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": per_launch, "mean_launch_ms": dom_ms / dom_cnt,
                "launches": dom_cnt}
    phases = {p: {"ms_per_step": v[0] / args.steps, "launch_groups": v[1]} for p, v in prof.items()}

    # slip-velocity and particle-temperature statistics after --c4-steps steps from the
    # inputs (the corrected step's report; the steps beyond warm-up + timed ones are run
    # here, untimed), compared below with the plain FP64 drop-in after as many steps
    stats_steps = args.warmup + args.steps
    c4_extra = 0
    if form == pstep.FP32 and not args.no_fp64_line and args.c4_steps > stats_steps and world == 1:
        c4_extra = args.c4_steps - stats_steps
        g.run(c4_extra)
        stats_steps = args.c4_steps
    import torch
    u_dev = [torch.from_numpy(np.ascontiguousarray(fields[d]).ravel()).to("cuda") for d in range(3)]
    stats_main = particle_stats(g, u_dev, bp.l, wl.n)

    # end to end through the C ABI with host buffers (pinned): a time-stepping loop
    # through host memory -- each step uploads the particles and the gas fields, primes,
    # runs one step and reads back every particle array (ids included) and every
    # deposited field; the particles read back are the next step's inputs, in the order
    # returned. The copies that do not depend on the step run beside it on two copy
    # streams: the next step's gas fields go up while this step computes (into the other
    # of two device slots, bound in place), and the deposited fields come back (through
    # a device slot) while the next step's particles go up.
    e2e = None
    # (per-particle tau_p would have to follow the particles' order through the host loop;
    # the workloads that carry it are error-report workloads and skip the loop)
    if not args.no_e2e and tau is None:
        import torch
        hpart = [torch.from_numpy(pinned_like(a)) for a in arrs]  # the particles' host copy
        hf = [torch.from_numpy(pinned_like(f)) for f in fields]
        out_f = [torch.from_numpy(pinned_like(np.empty_like(fields[0]))) for _ in range(5)]
        dev_in = [torch.empty(a.shape, dtype=a.dtype, device="cuda") for a in hpart]
        dev_out = [torch.empty(a.shape, dtype=a.dtype, device="cuda") for a in hpart]
        dev_f = [[torch.empty(f.shape, dtype=torch.float64, device="cuda") for f in hf] for _ in range(2)]
        dev_dep = [torch.empty(out_f[0].shape, dtype=torch.float64, device="cuda") for _ in range(5)]
        main_s, up_s, down_s = torch.cuda.Stream(), torch.cuda.Stream(), torch.cuda.Stream()
        torch.cuda.synchronize()
        g.set_stream(main_s.cuda_stream)
        ev_f = [torch.cuda.Event(), torch.cuda.Event()]
        ev_arr = [torch.cuda.Event() for _ in hpart]
        ev_in, ev_out = torch.cuda.Event(), torch.cuda.Event()
        ev_dep_ready, ev_dep_free = torch.cuda.Event(), torch.cuda.Event()
        slot = [0]

        def upload_fields(sl):
            with torch.cuda.stream(up_s):
                for d in range(4):
                    dev_f[sl][d].copy_(hf[d], non_blocking=True)
                ev_f[sl].record(up_s)

        def one_step():
            # (the correction set above persists across uploads; an upload clears its drive state)
            sl = slot[0]
            main_s.wait_event(ev_in)  # this step's particles, up from the host copy
            g.load(*dev_in)
            main_s.wait_event(ev_f[sl])
            g.bind_velocity(*dev_f[sl][:3])
            g.bind_temperature(dev_f[sl][3])
            g.prime()
            g.run(1)
            upload_fields(1 - sl)  # the next step's gas fields, while this step computes
            main_s.wait_event(ev_dep_free)
            for i, fname in enumerate(pstep.FIELD_IDS):
                g.field(fname, dev_dep[i])
            ev_dep_ready.record(main_s)
            g.download(*dev_out)
            ev_out.record(main_s)
            # the particles through the host copy, array by array: each array goes up as
            # soon as it is down, the two directions overlapping; the deposited fields come
            # down once the particles are back up (while the next step computes), so they
            # do not take link bandwidth from the particles' round trip
            with torch.cuda.stream(down_s):
                down_s.wait_event(ev_out)
                for a in range(len(hpart)):
                    hpart[a].copy_(dev_out[a], non_blocking=True)
                    ev_arr[a].record(down_s)
            with torch.cuda.stream(up_s):
                for a in range(len(hpart)):
                    up_s.wait_event(ev_arr[a])
                    dev_in[a].copy_(hpart[a], non_blocking=True)
                ev_in.record(up_s)
            with torch.cuda.stream(down_s):
                down_s.wait_event(ev_in)
                down_s.wait_event(ev_dep_ready)
                for i in range(5):
                    out_f[i].copy_(dev_dep[i], non_blocking=True)
                ev_dep_free.record(down_s)
            slot[0] = 1 - sl

        with torch.cuda.stream(up_s):
            for a in range(len(hpart)):
                dev_in[a].copy_(hpart[a], non_blocking=True)
            ev_in.record(up_s)
        upload_fields(0)
        one_step()
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        ke = max(1, args.steps)
        for _ in range(ke):
            one_step()
        torch.cuda.synchronize()  # the last round trip and read-back included
        barrier()
        e2e_s = max_over_ranks((time.perf_counter() - t0) / ke, dist, "cuda")
        g.set_stream(0)
        h2d = sum(a.numel() * a.element_size() for a in hpart) + sum(f.numel() * 8 for f in hf)
        d2h = sum(a.numel() * a.element_size() for a in hpart) + sum(f.numel() * 8 for f in out_f)
        e2e = {"value": job_rate(world, n, e2e_s * 1e3), "unit": "particle-steps/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s * 1e3,
               "loop": "host time-stepping: each step's particles go down to a pinned host copy and back up as "
                       "the next step's inputs (array by array, both directions overlapping); gas-field uploads "
                       "and deposited-field read-backs overlap the step on copy streams"}
        del dev_f, dev_dep, dev_in, dev_out

    # the plain FP32 step and the FP64 drop-in on the same inputs, timed the same way
    # (the comparison the metric names)
    fp32_plain = None
    if args.form == "fp32mlp" and not args.no_fp32_line:
        g.close()
        g = make_step(pstep.FP32, 0, False)
        for _ in range(args.warmup):
            g.run(1)
        barrier()
        g.run(args.steps)
        ms32 = g.last_run_ms() / args.steps
        fp32_plain = {"value": world * n / (ms32 / 1e3), "ms_per_step": ms32, "form": "fp32 plain interpolation"}
    fp64 = None
    c4_stats = None
    fp32_error = None
    if form == pstep.FP32 and not args.no_fp64_line:
        g.close()
        g = make_step(pstep.FP64, pstep.TRACK_ORDER, False)
        for _ in range(args.warmup):
            g.run(1)
        barrier()
        g.run(args.steps)
        ms64 = g.last_run_ms() / args.steps
        fp64 = {"value": world * n / (ms64 / 1e3), "ms_per_step": ms64, "form": "fp64 drop-in (reference order)"}
        if c4_extra:
            g.run(c4_extra)
        stats64 = particle_stats(g, u_dev, bp.l, wl.n)
        c4_stats = {"steps": stats_steps, "fields": "held fixed (the bound synthetic gas fields)",
                    args.form: stats_main, "fp64_plain": stats64,
                    "difference": stats_difference(stats_main, stats64)}
    # the FP32 form's error against the FP64 step on the same inputs (one step from the
    # inputs), for the workloads with per-particle tau_p
    if form == pstep.FP32 and wl.tau_p_range is not None and not args.no_fp64_line:
        g.close()
        g = make_step(pstep.FP32, 0, False)
        g64 = make_step(pstep.FP64, 0, False)
        g.run(1)
        g64.run(1)
        fp32_error = {"steps": 1, "against": "fp64 drop-in, same inputs and per-particle tau_p",
                      **fp32_error_report(g, g64, bp.l, wl.n)}
        g64.close()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        rate, dt = cpu_sample_rate()
        cpu = {"value": rate, "unit": "particle-steps/s", "cores": 1, "kind": "port",
               "sample": f"{1 << 22} particles on 160^3 (the workload's density and construction), 2 RK4 steps, "
                         f"{dt:.1f} s"}

    if rank == 0:
        line = {
            "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if form == pstep.FP64 else ("f32+bf16" if corr_model is not None else "f32"),
            "data": "synthetic",
            "config": {"workload": wl.name, "cells": wl.n ** 3, "particles": n, "form": args.form,
                       "learned_correction": corr_model is not None, "dp_over_dx": wl.dp_over_dx,
                       "mass_loading": wl.mass_loading,
                       "order_tracking": bool(flags & pstep.TRACK_ORDER), "clustered": wl.clustered, "blobs": wl.nblobs if wl.clustered else 0,
                       "l2": "inputs larger than L2 (particle state alone is several GB)",
                       "parallelism": f"replicas x{world}", "input_generation_s": round(gen_s, 2)},
            "roofline": roof, "phases": phases, "fp32_plain": fp32_plain, "fp64_dropin": fp64, "cpu_baseline": cpu,
            "c4_stats": c4_stats, "fp32_error": fp32_error,
            "e2e": e2e,
            "gpu_launches": launches,
            "clocks": clocks.summary(),
        }
        print(json.dumps(line), flush=True)
    g.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
