"""Benchmark of the SPH-DEM per-step hot path on one GB300 (one JSON line).

Workload: the 3D coupled SPH-DEM sedimentation configuration -- 1,024,000
fluid particles (dx = 2.5 mm, h = 1.5 dx, periodic x/y box 0.2 x 0.2 x 0.4
with a bottom wall of 6,400 repulsive boundary particles) and 50,000 DEM
spheres of radius 0.5 dx seeded in the top half; Wendland C2, Morris
viscosity, Omega correction, porosity-weighted Tait EOS, Di Felice drag,
linear spring-dashpot contacts, fixed dt.  Synthetic, seeded inputs.

  value     particle-steps/s of the mixed-precision path, state resident in
            HBM (1.08M particles, ~2.7 GB of state and lists, larger than
            L2), K steps timed with CUDA events around replays of the
            captured step graph
  e2e       the same metric through the C ABI with host buffers: create the
            simulation from pinned host arrays, then every step run it and
            read positions and densities back into pinned host arrays
  fp64      the plain-FP64 GPU path on the same input (--fp64-steps steps)
  error_vs_fp64  mixed vs FP64 after --error-steps steps from the same
            input: max |drho| / rho0 and max |df| / max |f| (fluid), DEM
            position error / R
  roofline  the dominant kernel (largest device time per step) from live
            per-launch CUDA events: HBM fraction of its algorithmic bytes
            and, for the pair passes, FP32-pipe fraction of its pair FLOPs
  configs   the other configurations at full size: the 2D dam break
            (mixed and FP64 rates, error after 1000 steps) and the 50k-sphere
            DEM settling (mixed and FP64 rates, error after 2000 steps)
  cpu_baseline  the CPU oracle port (a restatement of the reference's own
            C++ step) on a 1/16 periodic sub-box of the same workload

  python bench.py [--steps K] [--warmup W] [--gpus N] [--impl reference]

With --gpus N > 1 and no launcher environment (RANK / WORLD_SIZE), the
script starts its own N worker processes, one per GPU.
"""
from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import statistics
import socket
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "sph-dem_gb300"))
sys.path.insert(0, REPO)

import numpy as np  # noqa: E402

METRIC = "particle-steps/s (mixed-precision SPH-DEM step, 1 GPU)"
UNIT = "particle-steps/s"
SM_COUNT = 152
FP32_LANES = 128
# FLOPs per listed pair of the force pass (kernel evaluations for h_a and h_b,
# Morris viscosity, pressure; counted from k_force32's FP32 instruction mix)
FORCE_FLOP_PER_PAIR = 80.0


def workload_case(small: bool = False, quarter: bool = False):
    from sphdem import cases
    if small:
        # 1/16 periodic sub-box of the same workload: same dx, height, DEM density
        return cases.sediment3d(nx=20, L=0.05, height=0.4, n_dem=3125, seed=3, nsteps=2)
    if quarter:
        # 1/4 periodic sub-box (270k particles): profiler captures
        return cases.sediment3d(nx=40, L=0.1, height=0.4, n_dem=12500, seed=3, nsteps=2)
    return cases.sediment3d(seed=3)


def run_profile(args):
    """Mixed path only: warm-up steps then `steps` graph replays (the command
    to run under a profiler)."""
    import __graft_entry__
    __graft_entry__.build()
    from sphdem import capi, cases
    lib = capi.Library()
    case = workload_case(quarter=args.quarter)
    sim = capi.Simulation(lib, case.cfg, case.particles, precision=cases.PREC_MIXED)
    sim.step(args.warmup)
    ms = sim.time_steps(args.steps)
    st = sim.stats()
    sim.kernel_times_reset(True)
    sim.step(2)
    kt = {k: round(m / 2, 4) for k, (m, _) in sorted(sim.kernel_times().items(), key=lambda kv: -kv[1][0])}
    sim.kernel_times_reset(False)
    print(json.dumps({"profile": True, "n": case.n, "ms_per_step": ms / args.steps, "kernel_ms_per_step": kt,
                      "list_pairs": st.n_list_pairs, "h_max": st.h_max,
                      "search_radius": st.search_radius, "n_sph_cells": st.n_sph_cells,
                      "band_candidates": st.n_band_candidates, "band_queue_capacity": st.band_queue_capacity}))


def workload_config(case, nsteps, world: int = 1):
    n = case.n
    nd = int((case.particles["iam"] == 11).sum())
    return {
        "workload": "sediment3d_coupled_1M: 3D SPH-DEM sedimentation, periodic x/y 0.2x0.2x0.4 box",
        "n_particles": n, "n_fluid": case.notes["n_fluid"], "n_boundary": case.notes["n_boundary"],
        "n_dem": nd, "dx": case.cfg["psep"], "dt": case.cfg["maxdt"],
        "dem_radius": case.notes["dem_radius"], "coupling_radius": case.notes["coupling_radius"],
        "viscosity_kinematic": case.cfg["viscosity"], "steps": nsteps,
        "precision": "mixed (FP32 pair math on FP64-cell-origin offsets, FP64 integration)",
        "l2_policy": "inputs larger than L2 (state > 1 GB, L2 129 MB)",
        "parallelism": "single GPU" if world == 1 else f"{world} independent replicas, one per GPU",
    }


# --------------------------------------------------------------------------
# N > 1: independent replicas, one per GPU (the step does not shard); the
# timed region is bracketed by barriers and its time is the maximum over ranks
def dist_setup(world: int):
    """torch.distributed for N > 1 replicas: NCCL on GPUs, gloo otherwise
    (env:// rendezvous from the launcher).  None for a single process."""
    if world <= 1:
        return None
    import torch
    import torch.distributed as dist
    if not dist.is_initialized():
        dist.init_process_group(backend="nccl" if torch.cuda.is_available() else "gloo")
    return dist


def barrier(dist) -> None:
    if dist is not None:
        dist.barrier()


def max_over_ranks(x: float, dist) -> float:
    """The largest x over all ranks (the slowest rank's time)."""
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank: float, world: int, seconds_max: float) -> float:
    """Whole-job rate: the units all ranks processed over the slowest rank's time."""
    return units_per_rank * world / seconds_max


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, path):
        self.path = path
        self.proc = None

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i, v in enumerate(r) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def measured_peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            return json.load(fh), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "sm_max_mhz": 2070.0}, "fallback"


# Algorithmic bytes and FLOPs of one launch of each list pass (mixed
# precision, 3D), per the compulsory-traffic rule: every field a pass needs
# read once and every field it produces written once, plus 4 B per list entry
# the pass reads or writes.  `owners` = sph + sphBoundary particles (the list
# owners), `entries` = list entries of one build, `fluid` = sph particles.
#   nlist32   reads each owner's packed position (16 B), writes its count
#             (4 B) and its list (4 B per entry)
#   force32   reads cell id + offset (4 + 12), vhat (12), rho, pdr2, m, h,
#             type (4 each), porosity and Omega (4 each) and writes f (12):
#             68 B per owner, + 4 B per entry; ~80 FLOP per entry
#   dddt32    reads cell id + offset, vhat, m, h, type, Omega, writes dddt:
#             52 B per owner, + 4 B per entry; ~40 FLOP per entry
PASS_MODELS = {
    "nlist32": lambda owners, entries: (20.0 * owners + 4.0 * entries, None),
    "force32": lambda owners, entries: (68.0 * owners + 4.0 * entries, 80.0 * entries),
    "dddt32": lambda owners, entries: (52.0 * owners + 4.0 * entries, 40.0 * entries),
}
# DRAM bytes (read + write) of one launch per particle of the whole state,
# from ncu captures of the 270k sub-box of the same workload (traffic grows
# in proportion to the particle count at fixed density)
PASS_DRAM_BYTES_PER_PARTICLE = {
    "force32": (163.309824e6 + 12.316928e6) / 270100,
    "nlist32": (37.5e6 + 121.9e6) / 270100,
}


# --------------------------------------------------------------------------
def cpu_sample_worker(args):
    """Time the CPU oracle port on the sub-box sample (test infrastructure as
    the CPU baseline)."""
    steps, warm = args
    from oracle.port_api import OracleSim
    case = workload_case(small=True)
    o = OracleSim(case.cfg, case.particles)
    o.step(warm)
    t0 = time.perf_counter()
    o.step(steps)
    t = time.perf_counter() - t0
    return case.n, steps, t


def cpu_baseline(steps=2, warm=1, procs=1):
    from oracle import build_oracle
    build_oracle.build()
    if procs == 1:
        n, s, t = cpu_sample_worker((steps, warm))
        return n * s / t, n, s, t
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs) as pool:
        res = pool.map(cpu_sample_worker, [(steps, warm)] * procs)
    agg = sum(n * s / t for n, s, t in res)
    return agg, res[0][0], steps, max(t for _, _, t in res)


# --------------------------------------------------------------------------
def _time_adjoint(lib, capi, cases, case, nsteps, ckpt, seed_fn, precisions=("fp64", "mixed"), tape_mem=0):
    """(plain forward, adjoint forward, adjoint backward) wall times of the
    same nsteps from the same state, FP64 and / or mixed (each call returns
    after the device finished).  tape_mem: sphdem_adjoint_set_tape_memory
    (0: one segment's tape, earlier segments replayed in the backward pass;
    -1: the tapes of every segment that fits in half of the free memory)."""
    out = {}
    for name in precisions:
        prec = cases.PREC_FP64 if name == "fp64" else cases.PREC_MIXED
        sim = capi.Simulation(lib, case.cfg, case.particles, precision=prec)
        sim.step(2)
        t0 = time.perf_counter()
        sim.step(nsteps)
        t_fwd = time.perf_counter() - t0
        sim.close()
        sim = capi.Simulation(lib, case.cfg, case.particles, precision=prec)
        sim.step(2)
        seeds = seed_fn(sim)
        sim.adjoint_set_tape_memory(tape_mem)
        t0 = time.perf_counter()
        sim.adjoint_forward(nsteps, ckpt)
        t_af = time.perf_counter() - t0
        sim.adjoint_backward(**seeds)
        t_ab = time.perf_counter() - t0 - t_af
        sim.close()
        out[name] = {"forward_s": t_fwd, "adjoint_forward_s": t_af, "adjoint_backward_s": t_ab,
                     "ratio": (t_af + t_ab) / t_fwd}
    return out


def measure_adjoint(lib, capi, cases, nsteps=100, ckpt=10):
    """Wall time of sphdem_adjoint_forward + sphdem_adjoint_backward over the
    wall time of the same steps stepped plainly, for the three step families
    the adjoint covers: DEM-only settling (4,913 spheres), the 2D dam break
    at its full size (dx = 0.01, artificial viscosity), both FP64 and mixed,
    and the coupled SPH-DEM workload of 100k fluid + 5k DEM particles
    (mixed)."""
    out = {}
    dem = cases.dem_settling3d(lattice=(17, 17, 17), box=(0.067, 0.067, 0.067), spread=0.0,
                               nsteps=nsteps, vel_amp=0.3)

    def dem_seed(sim):
        a = sim.get(capi.FIELD_IAM)
        seed = np.zeros((sim.n, 3))
        m = a["iam"] == cases.DEM
        seed[m, 2] = 1.0 / max(1, m.sum())
        return {"dL_dr": seed}

    out["dem"] = _time_adjoint(lib, capi, cases, dem, nsteps, ckpt, dem_seed)
    out["dem"]["workload"] = (f"DEM-only settling, {dem.n} spheres, {nsteps} steps, "
                              f"checkpoint every {ckpt}")
    fluid = cases.workload("dambreak2d")

    def fluid_seed(sim):
        a = sim.get(capi.FIELD_IAM)
        seed = np.zeros((sim.n, 3))
        m = a["iam"] == cases.SPH
        seed[m, 1] = 1.0 / max(1, m.sum())
        return {"dL_dr": seed}

    out["fluid"] = _time_adjoint(lib, capi, cases, fluid, nsteps, ckpt, fluid_seed)
    out["fluid"]["workload"] = (f"2D dam break, {fluid.n} particles (artificial viscosity), "
                                f"{nsteps} steps, checkpoint every {ckpt}")
    # the differentiated coupled workload: 100k fluid + 5k DEM (periodic x/y,
    # fixed boundary floor, porosity, two-way drag, contacts), mixed precision
    cpl = cases.workload("sediment3d_adjoint")
    cpl_steps, cpl_ckpt = 100, 50

    def cpl_seed(sim):
        a = sim.get(capi.FIELD_IAM)
        seed = np.zeros((sim.n, 3))
        m = a["iam"] == cases.DEM
        seed[m, 2] = 1.0 / max(1, m.sum())
        return {"dL_dr": seed}

    # checkpoints every 50 steps; the tapes of the segments are kept in
    # device memory from the forward pass (they fit: ~10 GB per 50 steps)
    out["coupled"] = _time_adjoint(lib, capi, cases, cpl, cpl_steps, cpl_ckpt, cpl_seed, precisions=("mixed",),
                                   tape_mem=-1)
    out["coupled"]["workload"] = (f"coupled SPH-DEM, {cpl.n} particles ({cpl.notes['n_fluid']} fluid, "
                                  f"{cpl.notes['n_dem']} DEM), {cpl_steps} steps, checkpoint every {cpl_ckpt}, "
                                  f"segment tapes kept in device memory")
    # the same with one segment's tape: the backward pass replays the first
    # segment from its checkpoint
    out["coupled_replay"] = _time_adjoint(lib, capi, cases, cpl, cpl_steps, cpl_ckpt, cpl_seed,
                                          precisions=("mixed",), tape_mem=0)
    out["coupled_replay"]["workload"] = (f"as coupled, one segment's tape kept (earlier segments replayed "
                                         f"from their checkpoints)")
    # the same with one segment (checkpoint interval = run length)
    out["coupled_one_segment"] = _time_adjoint(lib, capi, cases, cpl, cpl_steps, cpl_steps, cpl_seed,
                                               precisions=("mixed",))
    out["coupled_one_segment"]["workload"] = (f"as coupled, {cpl_steps} steps in one checkpoint segment "
                                              f"(tape recorded in the forward pass, no replay)")
    # the differentiated run's own length: 500 steps, checkpoints every 50
    out["coupled_500"] = _time_adjoint(lib, capi, cases, cpl, 500, 50, cpl_seed, precisions=("mixed",),
                                       tape_mem=-1)
    out["coupled_500"]["workload"] = ("as coupled, 500 steps, checkpoint every 50, segment tapes kept in "
                                      "device memory")
    # the coupled configuration's own VAR_H_CORRECTION (h following density,
    # the 1/Omega gradient correction): 100 steps, checkpoints every 50
    cplv = cases.workload("sediment3d_adjoint_varh")
    out["coupled_varh"] = _time_adjoint(lib, capi, cases, cplv, cpl_steps, cpl_ckpt, cpl_seed, precisions=("mixed",),
                                        tape_mem=-1)
    out["coupled_varh"]["workload"] = ("as coupled, with VAR_H_CORRECTION (h = 1.5 (m / rho)^(1/3), gradients "
                                       "over Omega), segment tapes kept in device memory")
    out["ratio"] = max(out["dem"]["mixed"]["ratio"], out["fluid"]["mixed"]["ratio"],
                       out["coupled"]["mixed"]["ratio"], out["coupled_varh"]["mixed"]["ratio"])
    return out


def run_adjoint_profile(args):
    """The differentiated coupled workload (100k fluid + 5k DEM, mixed) for
    profiler captures: 2 plain steps, then sphdem_adjoint_forward over
    args.steps steps with one checkpoint segment and sphdem_adjoint_backward
    of the mean DEM height; prints the wall times."""
    import __graft_entry__
    __graft_entry__.build()
    from sphdem import capi, cases
    lib = capi.Library()
    case = cases.workload("sediment3d_adjoint")
    sim = capi.Simulation(lib, case.cfg, case.particles, precision=cases.PREC_MIXED)
    sim.step(2)
    a = sim.get(capi.FIELD_IAM)
    seed = np.zeros((sim.n, 3))
    m = a["iam"] == cases.DEM
    seed[m, 2] = 1.0 / m.sum()
    t0 = time.perf_counter()
    sim.adjoint_forward(args.steps, args.steps)
    t1 = time.perf_counter()
    g = sim.adjoint_backward(dL_dr=seed)[0]
    t2 = time.perf_counter()
    sim.close()
    print(json.dumps({"workload": "sediment3d_adjoint (coupled, %d particles)" % case.n, "steps": args.steps,
                      "adjoint_forward_ms_per_step": 1e3 * (t1 - t0) / args.steps,
                      "adjoint_backward_ms_per_step": 1e3 * (t2 - t1) / args.steps,
                      "grad_viscosity": g.viscosity, "grad_drag_scale": g.drag_scale}), flush=True)


def full_box_step_1core(warm: int = 0):
    """One step of the CPU oracle port on the full 1.08M-particle workload on
    one core (after `warm` warm-up steps; the oracle builds its lists at
    creation, outside the timed step): checks that the per-particle cost of
    the 1/16 sub-box sample carries over to the full box."""
    from oracle.port_api import OracleSim
    case = workload_case()
    t0 = time.perf_counter()
    o = OracleSim(case.cfg, case.particles)
    t_setup = time.perf_counter() - t0
    if warm:
        o.step(warm)
    t0 = time.perf_counter()
    o.step(1)
    t = time.perf_counter() - t0
    return {"n": case.n, "setup_s": t_setup, "step_s": t, "particle_steps_per_s": case.n / t}


def run_reference_arm(args, rank, world):
    """The reference's CPU step (the oracle port, a restatement of its C++
    step pinned to the compiled reference) on all host cores: one process per
    core, each on a 1/16 periodic sub-box of the workload (16 sub-boxes make
    the full 1.08M-particle box), W warm-up and K timed steps each; the value
    is the particles of all processes times K over the slowest process's
    time.  Then one full-box step on one core checks the per-particle cost."""
    if rank != 0:
        return
    procs = os.cpu_count() or 1
    value, n, s, t = cpu_baseline(steps=args.steps, warm=args.warmup, procs=procs)
    sample = (f"CPU oracle port (restatement of the reference's C++ step, single-threaded per "
              f"process) on 1/16 periodic sub-boxes of the workload ({n} particles each, "
              f"{procs} processes = {procs / 16:.2f} full boxes), {s} timed steps after {args.warmup} "
              f"warm-up steps each")
    full = None if args.no_full_box else full_box_step_1core()
    per_core_sub = value / procs
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / s,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded)", "config": workload_config(workload_case(), args.steps),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": procs, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "per_core_sub_box": per_core_sub,
        "full_box_check": None if full is None else dict(
            full, sub_box_per_core_over_full_box=per_core_sub / full["particle_steps_per_s"]),
    }
    print(json.dumps(line), flush=True)


def select_device(world: int) -> None:
    """One GPU per rank: the launcher's LOCAL_RANK, set as the current device
    of the CUDA runtime the library uses (and of torch, whose NCCL calls need
    it)."""
    if world <= 1:
        return
    import ctypes as C
    local = int(os.environ.get("LOCAL_RANK", os.environ.get("RANK", "0")))
    rt = C.CDLL("libcudart.so.13")
    rc = rt.cudaSetDevice(local)
    if rc != 0:
        raise RuntimeError(f"cudaSetDevice({local}) failed with {rc}")
    try:
        import torch
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
    except ImportError:
        pass


def _kernel_split(sim, steps=2):
    """Per-kernel device ms per step and launches per step over `steps` steps."""
    sim.kernel_times_reset(True)
    sim.step(steps)
    kt = sim.kernel_times()
    sim.kernel_times_reset(False)
    return {k: (m / steps, c / steps) for k, (m, c) in kt.items()}


def _errors(a, b, cases, rho0, R):
    """Mixed (a) against FP64 (b), tag order: fluid density and force, DEM
    position."""
    iam = b["iam"]
    fl = (iam == cases.SPH) | (iam == cases.SPH_BOUNDARY)
    dem = iam == cases.DEM
    out = {}
    if fl.any():
        out["max_abs_drho_over_rho0"] = float(np.abs(a["dens"][fl] - b["dens"][fl]).max() / rho0)
        out["max_abs_df_over_max_f"] = float(np.abs(a["f"][fl] - b["f"][fl]).max() / np.abs(b["f"][fl]).max())
    if dem.any():
        out["dem_max_abs_dr_over_R"] = float(np.abs(a["r"][dem] - b["r"][dem]).max() / R)
        out["dem_max_abs_df_over_max_f"] = float(np.abs(a["f"][dem] - b["f"][dem]).max()
                                                 / max(np.abs(b["f"][dem]).max(), 1e-300))
    return out


def measure_config(lib, capi, cases, case, mixed_steps, fp64_steps, err_steps, R):
    """Mixed and FP64 rates (graph replays timed with CUDA events) of one
    configuration and the mixed error against FP64 after err_steps steps."""
    n = case.n
    mixed = capi.Simulation(lib, case.cfg, case.particles, precision=cases.PREC_MIXED)
    fp64 = capi.Simulation(lib, case.cfg, case.particles, precision=cases.PREC_FP64)
    ms_m = mixed.time_steps(mixed_steps)
    ms_f = fp64.time_steps(fp64_steps)
    mixed.step(err_steps - mixed_steps - 1)
    fp64.step(err_steps - fp64_steps - 1)
    a, b = mixed.get(), fp64.get()
    mixed.close()
    fp64.close()
    return {"n_particles": n,
            "mixed": {"value": n * mixed_steps / (ms_m * 1e-3), "unit": UNIT, "steps": mixed_steps},
            "fp64": {"value": n * fp64_steps / (ms_f * 1e-3), "unit": UNIT, "steps": fp64_steps},
            "mixed_over_fp64": (ms_f / fp64_steps) / (ms_m / mixed_steps),
            "error_vs_fp64": dict(_errors(a, b, cases, case.cfg["dens"], R), steps=err_steps)}


def run_ours(args, rank, world):
    import __graft_entry__
    __graft_entry__.build()
    select_device(world)
    from sphdem import capi, cases
    lib = capi.Library()
    case = workload_case()
    n = case.n
    scratch = tempfile.mkdtemp(prefix="sphdem_bench_")

    # ---- mixed precision, device-resident --------------------------------
    dist = dist_setup(world)
    sim = capi.Simulation(lib, case.cfg, case.particles, precision=cases.PREC_MIXED)
    sim.step(args.warmup)
    barrier(dist)
    with ClockSampler(os.path.join(scratch, "clocks.csv")) as clk:
        ms = sim.time_steps(args.steps)   # CUDA events on the handle's stream, synchronised
    barrier(dist)
    ms = max_over_ranks(ms, dist)
    clocks = clk.summary()
    value = aggregate_rate(n * args.steps, world, ms * 1e-3)
    st = sim.stats()

    # per-kernel device times (CUDA events around each launch on the
    # handle's stream), 2 steps
    split = _kernel_split(sim, 2)
    launches_per_step = sum(c for _, c in split.values())
    total_ms = sum(m for m, _ in split.values())
    top = sorted(split.items(), key=lambda kv: -kv[1][0])

    # ---- roofline of the dominant list pass -------------------------------
    peaks, peak_kind = measured_peaks()
    owners = case.notes["n_fluid"] + case.notes["n_boundary"]
    entries = float(st.n_list_pairs)
    dom = next((k for k, _ in top if k in PASS_MODELS), None)
    roof = None
    if dom is not None:
        ms_step, launches = split[dom]
        ms_launch = ms_step / max(launches, 1e-9)
        alg_bytes, flops = PASS_MODELS[dom](owners, entries)
        achieved = alg_bytes / (ms_launch * 1e-3) / 1e9
        sm_mhz = clocks.get("sm_max_mhz") or peaks.get("sm_max_mhz", 2070.0)
        fp32_peak = SM_COUNT * FP32_LANES * 2 * sm_mhz * 1e6 / 1e12
        traffic = PASS_DRAM_BYTES_PER_PARTICLE.get(dom)
        roof = {
            "kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peaks.get("hbm_gbs"),
            "unit": "GB/s", "frac": achieved / peaks.get("hbm_gbs", 6800.0),
            "traffic": None if traffic is None else traffic * n,
            "peak_kind": peak_kind, "alg_bytes_per_launch": alg_bytes, "ms_per_launch": ms_launch,
            "launches_per_step": launches, "share_of_step": ms_step / total_ms,
            "list_entries": entries, "owners": owners,
            "h_max": st.h_max, "search_radius": st.search_radius, "n_sph_cells": st.n_sph_cells,
            "band_candidates": st.n_band_candidates,
        }
        if flops is not None:
            achieved_tf = flops / (ms_launch * 1e-3) / 1e12
            roof["fp32_pipe"] = {"achieved": achieved_tf, "peak": fp32_peak, "unit": "TFLOP/s",
                                 "frac": achieved_tf / fp32_peak,
                                 "peak_basis": f"{SM_COUNT} SMs x {FP32_LANES} lanes x 2 x {sm_mhz:.0f} MHz"}
    passes = {}
    for k in PASS_MODELS:
        if k in split:
            ms_step, launches = split[k]
            b_, f_ = PASS_MODELS[k](owners, entries)
            ms_launch = ms_step / max(launches, 1e-9)
            passes[k] = {"ms_per_launch": ms_launch, "launches_per_step": launches,
                         "hbm_frac": b_ / (ms_launch * 1e-3) / 1e9 / peaks.get("hbm_gbs", 6800.0)}

    # ---- FP64 path and mixed-vs-FP64 error on the same input -------------
    fp64_steps = max(1, args.fp64_steps)
    err_steps = max(args.error_steps, fp64_steps + 2, args.warmup + args.steps + 3)
    ref = capi.Simulation(lib, case.cfg, case.particles, precision=cases.PREC_FP64)
    ref.step(1)
    ms64 = ref.time_steps(fp64_steps)   # advances fp64_steps + 1 steps
    fp64_value = n * fp64_steps / (ms64 * 1e-3)
    # a fresh mixed handle from the same input, compared at checkpoints every
    # 20 steps up to err_steps (the maxima over particles at each)
    cmp = capi.Simulation(lib, case.cfg, case.particles, precision=cases.PREC_MIXED)
    at = fp64_steps + 2
    cmp.step(at)
    mask = capi.FIELD_DENS | capi.FIELD_F | capi.FIELD_R | capi.FIELD_IAM
    checkpoints = []
    while True:
        e = _errors(cmp.get(mask), ref.get(mask), cases, case.cfg["dens"], case.notes["dem_radius"])
        checkpoints.append(dict(e, steps=at))
        if at >= err_steps:
            break
        k = min(20, err_steps - at)
        cmp.step(k)
        ref.step(k)
        at += k
    err = dict(checkpoints[-1],
               against="the FP64 GPU path from the same input (pinned to the CPU oracle on the small cases)",
               checkpoints=checkpoints,
               note="the suspension amplifies any difference at an e-folding time of ~30 steps; the FP64 path "
                    "run from inputs one bit apart separates as far within ~700 steps (tests/test_gpu_precision.py)")
    cmp.close()
    ref.close()

    # ---- the other configurations at full size ---------------------------
    configs = None
    if not args.no_configs:
        db = cases.workload("dambreak2d")
        dem = cases.workload("dem_settling3d")
        configs = {
            "dambreak2d": dict(measure_config(lib, capi, cases, db, 200, 50, 1000, db.cfg["psep"]),
                               workload=f"2D dam break, {db.notes['n_fluid']} fluid + {db.notes['n_boundary']} "
                                        f"wall particles, dx 0.01, artificial viscosity, dt 0.25 h/c0"),
            "dem_settling3d": dict(measure_config(lib, capi, cases, dem, 200, 200, 2000, dem.cfg["dem_radius"]),
                                   workload="DEM settling, 50,000 spheres radius 1 mm x U[0.9, 1.1], walled "
                                            "0.1 x 0.1 x 0.3 m box, k 1e4, e 0.5, dt 1e-5"),
            "ensemble_dambreak256": measure_ensemble(lib, capi, cases, args.instances, args.steps, args.warmup),
        }

    # ---- adjoint / forward ------------------------------------------------
    adjoint = measure_adjoint(lib, capi, cases) if not args.no_adjoint else None

    # ---- end to end through the C ABI with host buffers -------------------
    e2e_steps = args.steps
    init = capi.ParticleBuffers(n, case.particles, pinned=lib)
    # two pinned result buffers: the copy of step k's result overlaps step k+1
    outbufs = [capi.ParticleBuffers(n, pinned=lib, fields=("r", "dens")) for _ in range(2)]
    import ctypes as C
    cfgs = capi.config_struct(case.cfg, cases.PREC_MIXED)
    barrier(dist)
    t0 = time.perf_counter()
    h = C.c_void_p()
    lib.check(lib.lib.sphdem_create(C.byref(cfgs), init.ref(), n, C.byref(h)), None, "create")
    for k in range(e2e_steps):
        lib.check(lib.lib.sphdem_step(h, 1), h, "step")
        lib.check(lib.lib.sphdem_get_fields_async(h, capi.FIELD_R | capi.FIELD_DENS, outbufs[k % 2].ref()), h,
                  "get_fields_async")
    lib.check(lib.lib.sphdem_fields_wait(h), h, "fields_wait")
    t_e2e = max_over_ranks(time.perf_counter() - t0, dist)
    lib.lib.sphdem_destroy(h)
    e2e_value = aggregate_rate(n * e2e_steps, world, t_e2e)
    h2d_bytes = n * (4 * 3 * 8 + 4 * 8 + 12)  # r, v, norms x3 (3 comps) + mass, dens, h, radius + ints
    d2h_bytes = n * (3 * 8 + 8)

    # ---- CPU baseline (oracle port, 1 core, bounded sample) ---------------
    cpu = None
    if rank == 0 and not args.no_cpu:
        cv, cn, cs, ct = cpu_baseline(steps=args.cpu_steps, warm=1, procs=1)
        cpu = {"value": cv, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"CPU oracle port on a 1/16 periodic sub-box of the workload ({cn} particles, "
                         f"same dx/physics), {cs} steps after 1 warm-up step, {ct:.1f} s"}

    sim.close()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32/f64", "data": "synthetic (seeded)",
        "config": workload_config(case, args.steps, world),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d_bytes / e2e_steps),
                "d2h_bytes_per_step": int(d2h_bytes),
                "what": "sphdem_create from pinned host arrays + per step sphdem_step + sphdem_get_fields_async(r, "
                        "dens) into two alternating pinned host arrays (each step's copy overlaps the next step), "
                        "sphdem_fields_wait at the end; wall clock"},
        "fp64": {"value": fp64_value, "unit": UNIT, "steps": fp64_steps,
                 "mixed_over_fp64": value / fp64_value},
        "error_vs_fp64": err,
        "configs": configs,
        "adjoint_over_forward": adjoint["ratio"] if adjoint else None,
        "adjoint": adjoint,
        "roofline": roof,
        "passes": passes,
        "kernels_ms_per_step": {k: v[0] for k, v in top[:14]},
        "kernel_share": {k: v[0] / total_ms for k, v in top[:14]},
        "gpu_launches": int(round(launches_per_step * args.steps)),
        "clocks": clocks,
        "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def measure_ensemble(lib, capi, cases, instances, steps, warmup, err_steps=1000, err_every=16):
    """The batched dam-break ensemble: `instances` independent 2D dam breaks
    of uneven size stepped by one CUDA graph per step (sphdem_batch_*),
    against the same instances each graph-replayed alone; and the mixed
    path's error against the FP64 path after err_steps steps on every
    err_every-th instance (both precisions batched)."""
    ens = cases.dambreak_ensemble(instances, seed=5)
    n_total = sum(c.n for c in ens)
    t0 = time.time()
    sims = [capi.Simulation(lib, c.cfg, c.particles, precision=cases.PREC_MIXED) for c in ens]
    batch = capi.Batch(lib, sims)
    chosen = batch.tune(steps_per_trial=2)
    setup_s = time.time() - t0
    batch.step(warmup)
    ms_batch = batch.time_steps(steps)
    ms_seq = sum(sim.time_steps(steps) for sim in sims)
    batch.close()
    for sim in sims:
        sim.close()
    pick = list(range(0, instances, err_every))
    runs = {}
    for prec in (cases.PREC_MIXED, cases.PREC_FP64):
        ss = [capi.Simulation(lib, ens[k].cfg, ens[k].particles, precision=prec) for k in pick]
        b = capi.Batch(lib, ss)
        b.step(err_steps)
        runs[prec] = [x.get(capi.FIELD_DENS | capi.FIELD_F | capi.FIELD_IAM) for x in ss]
        b.close()
        for x in ss:
            x.close()
    errs = [_errors(a, f, cases, ens[k].cfg["dens"], 1.0)
            for k, a, f in zip(pick, runs[cases.PREC_MIXED], runs[cases.PREC_FP64])]
    return {
        "workload": f"{instances} independent 2D dam breaks, fluid count log-uniform in [2k, 40k], "
                    f"column height U[1.0, 2.5], seed 5",
        "n_particles_total": n_total, "n_instances": instances,
        "min_particles": min(c.n for c in ens), "max_particles": max(c.n for c in ens),
        "batched": {"value": n_total * steps / (ms_batch * 1e-3), "unit": UNIT, "ms_per_step": ms_batch / steps},
        "sequential": {"value": n_total * steps / (ms_seq * 1e-3), "unit": UNIT, "ms_per_step": ms_seq / steps},
        "batched_over_sequential": ms_seq / ms_batch,
        "autotuner": {"blk_pair_64": sum(1 for x in chosen if x[0] == 64),
                      "grid_div_4": sum(1 for x in chosen if x[1] == 4),
                      "staged_tiles": sum(1 for x in chosen if x[2]), "setup_s": setup_s},
        "error_vs_fp64": {"steps": err_steps, "instances": len(pick),
                          "max_abs_drho_over_rho0": max(e["max_abs_drho_over_rho0"] for e in errs),
                          "max_abs_df_over_max_f": max(e["max_abs_df_over_max_f"] for e in errs)},
    }


def run_ensemble(args):
    """Batched ensemble: independent 2D dam breaks of uneven size stepped by
    one CUDA graph per step (sphdem_batch_*), against the same instances run
    one at a time; per-instance error of the mixed path against the FP64
    path after the timed steps."""
    import __graft_entry__
    __graft_entry__.build()
    from sphdem import capi, cases
    lib = capi.Library()
    ens = cases.dambreak_ensemble(args.instances, seed=5)
    n_total = sum(c.n for c in ens)
    t0 = time.time()
    sims = [capi.Simulation(lib, c.cfg, c.particles, precision=cases.PREC_MIXED) for c in ens]
    batch = capi.Batch(lib, sims)
    chosen = batch.tune(steps_per_trial=2)
    setup_s = time.time() - t0
    batch.step(args.warmup)
    ms_batch = batch.time_steps(args.steps)
    # the same instances one at a time (each timed alone, graph-replayed)
    ms_seq = 0.0
    for sim in sims:
        ms_seq += sim.time_steps(args.steps)
    # error against the FP64 path for every instance, same step count
    steps_done = [sim.globals().sph_step for sim in sims]
    errs = []
    for c, sim, k in zip(ens, sims, steps_done):
        ref = capi.Simulation(lib, c.cfg, c.particles, precision=cases.PREC_FP64)
        ref.step(int(k))
        a, b = sim.get(), ref.get()
        errs.append(float(np.abs(a["dens"] - b["dens"]).max() / c.cfg["dens"]))
        ref.close()
    batch.close()
    line = {
        "metric": "particle-steps/s (batched dam-break ensemble, 1 GPU)",
        "value": n_total * args.steps / (ms_batch * 1e-3), "unit": "particle-steps/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_batch / args.steps, "higher_is_better": True, "dtype": "f32/f64",
        "data": "synthetic (seeded)",
        "config": {"workload": f"{args.instances} independent 2D dam breaks, fluid count log-uniform "
                               f"in [2k, 40k], column height U[1.0, 2.5], seed 5",
                   "n_particles_total": n_total, "n_instances": args.instances,
                   "min_particles": min(c.n for c in ens), "max_particles": max(c.n for c in ens)},
        "sequential": {"value": n_total * args.steps / (ms_seq * 1e-3), "ms_per_step": ms_seq / args.steps},
        "batched_over_sequential": ms_seq / ms_batch,
        "autotuner": {"blk_pair_64": sum(1 for b, _, _ in chosen if b == 64),
                      "grid_div_4": sum(1 for _, d, _ in chosen if d == 4),
                      "staged_tiles": sum(1 for _, _, t in chosen if t), "setup_s": setup_s},
        "max_drho_over_rho0_vs_fp64": max(errs),
    }
    print(json.dumps(line), flush=True)


def replica_env(rank: int, world: int, port: int, base: dict | None = None) -> dict:
    """Environment of worker `rank` of `world` self-started replicas (the
    variables torch.distributed.run would set; rendezvous on 127.0.0.1)."""
    env = dict(os.environ if base is None else base)
    env.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), LOCAL_WORLD_SIZE=str(world),
               MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    return env


def spawn_replicas(world: int) -> int:
    """bench.py --gpus N without a launcher: start N copies of this command,
    one per GPU; rank 0 prints the line.  Returns the worst exit code."""
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    procs = [subprocess.Popen([sys.executable, os.path.abspath(__file__), *sys.argv[1:]],
                              env=replica_env(r, world, port)) for r in range(world)]
    return max(p.wait() for p in procs)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--fp64-steps", type=int, default=20)
    ap.add_argument("--error-steps", type=int, default=100,
                    help="steps after which the mixed path is compared with the FP64 path")
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-configs", action="store_true", help="skip the dam-break and DEM-settling legs")
    ap.add_argument("--no-full-box", action="store_true", help="reference arm: skip the full-box step")
    ap.add_argument("--profile", action="store_true", help="mixed path only (for profiler captures)")
    ap.add_argument("--quarter", action="store_true", help="with --profile: 1/4 sub-box of the workload")
    ap.add_argument("--ensemble", action="store_true", help="batched dam-break ensemble instead")
    ap.add_argument("--adjoint-profile", action="store_true",
                    help="coupled adjoint over --steps steps only (for profiler captures)")
    ap.add_argument("--instances", type=int, default=256)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    launched = "RANK" in os.environ and "WORLD_SIZE" in os.environ
    if args.gpus > 1 and not launched and args.impl == "ours" and not (
            args.profile or args.ensemble or args.adjoint_profile):
        sys.exit(spawn_replicas(args.gpus))
    rank = int(os.environ.get("RANK", "0")) if launched else 0
    world = int(os.environ.get("WORLD_SIZE", "1")) if launched else 1
    if args.adjoint_profile:
        run_adjoint_profile(args)
    elif args.profile:
        run_profile(args)
    elif args.ensemble:
        run_ensemble(args)
    elif args.impl == "reference":
        run_reference_arm(args, rank, world)
    else:
        run_ours(args, rank, world)


if __name__ == "__main__":
    main()
