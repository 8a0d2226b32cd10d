#!/usr/bin/env python3
"""Benchmark of the SDPD step: particle-steps/s on the 3D 1M workload.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (configs.c3_poiseuille_3d): 100^3 = 1,000,000 fluid particles on a
unit lattice between two solid walls in y (4 layers of 100x100 wall
particles per side, 80,000 in total), quintic kernel rc = 3dx, Hu-Adams
force, Morris EOS c = 20, eta = 0.5, g_x = 0.1, kT = 1e-4 with the Philox
Wiener increments, dt = 5e-5.  Synthetic inputs, generated with the
reference's lattice rule.  A step is one velocity-Verlet step (kick, drift,
wrap, cell list, density, pressure, pair force, body force, kick); the
metric counts fluid particles.

`value` is the FP32-mixed path with the state resident in HBM (device time,
CUDA events on the library's stream), with neighbour-list reuse on
(mcfg_params.reserved[1]): the candidates within rc + skin are rebuilt on the
device only when a particle has moved more than skin/2, every step re-tests
them exactly (config.list_reuse gives the skin, the rebuilds inside the timed
steps and the same step with MCF's cell list rebuilt every step;
--no-list-reuse times that mode as the headline).  `fp64` is the plain FP64
path on the same workload.  `e2e` is the same metric through the C-ABI with host
buffers: every step is one mcfg_step_vv_host call that hands x, v over from
the caller's arrays (page-locked once with mcfg_host_register, as MCF's own
x, v would be), runs the step and copies x, v back (the positions' copy
overlapping the sweeps on a second stream); masses, ids and the initial
forces go over once, before the timed steps.  `output_write` times MCF's
particle output file of the workload written through mcfg_write_particles
(E16.8 text formatted on the device).  `lees_edwards` times a sheared box
of the same size (y faces sliding along x, bcdef 10) with the cell list
rebuilt every step and with the candidate list kept across steps.
`mcf_scalability_deck` runs the physics of MCF's own 1M-particle
scalability input (cut-off 4 dx, Batchelor equation of state, Hu-Adams
angular force) read from an MCF deck by mcf_config.load_mcf_deck.
`fp32_error_vs_fp64` runs the workload for --accuracy-steps (5000, the
whole C3 run) in FP32-mixed and in FP64 from the same state with the same
Philox keys and states the errors of the mean velocity, the u_x(y) profile,
the wall shear stress and the shear stress S_xy (over --accuracy-seeds
seeds), then the same on a developed Poiseuille channel (--channel-steps,
two viscous times).  `colloid_suspension` is C4: a 96^3 lattice with 200
rigid spheres integrated on the device (Adams-Bashforth), FP32-mixed
particle-steps/s and the colloids' velocity and angular-velocity errors
against FP64 over --c4-steps steps.  `cpu_baseline` is the CPU
restatement of MCF's path (the oracle; MCF itself cannot be built here) on
the host cores in MCF's symmetric loop mode (symmetry = T, each pair once;
x-slabs of cells in two colours over the threads), with the full-stencil
mode and one core beside it.  With --impl reference only that CPU path is
timed.

With torchrun (N > 1) every rank runs an independent replica on its own GPU
("replicas only": this workload is not decomposed across GPUs); value sums
the ranks' particle-steps over the slowest rank's time.  The single-GPU
studies (accuracy, C4, adjoint, Lees-Edwards, MCF deck, output file) run at
N = 1 only; the N-GPU line keeps the headline, FP64 and e2e.
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
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "particle-steps/s, 3D SDPD 1M: FP32-mixed vs FP64 at stated error; adjoint/fwd"
UNIT = "particle-steps/s"

# GB300's L2 (bytes): the headline workload's state is ~13x this
L2_BYTES = 129_000_000

# algorithmic bytes per particle and pass (minimum HBM traffic with every
# per-particle array read or written once), FP32-mixed / FP64
ALGO_BYTES = {
    "list": (128, 184),
    "density": (20, 32),
    "force": (64, 92),
    "update": (80, 120),
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n-side", type=int, default=100)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--no-list-reuse", action="store_true")
    ap.add_argument("--no-output", action="store_true")
    ap.add_argument("--no-lees-edwards", action="store_true")
    ap.add_argument("--no-mcf-deck", action="store_true")
    ap.add_argument("--no-colloids", action="store_true")
    ap.add_argument("--c4-steps", type=int, default=2000,
                    help="VV steps of the FP32-vs-FP64 colloid run (C4's 2000)")
    ap.add_argument("--precision", choices=["fp32", "fp64"], default="fp32",
                    help="path of the headline value (fp64: the plain FP64 path, for profiling "
                         "its sweeps; the FP64 comparison line is then left out)")
    ap.add_argument("--accuracy-steps", type=int, default=5000,
                    help="VV steps of the FP32-vs-FP64 run on the headline workload (the "
                         "5000 of its configuration)")
    ap.add_argument("--accuracy-seeds", type=int, default=1,
                    help="Philox keys of the FP32-vs-FP64 run (errors: mean and max)")
    ap.add_argument("--channel-steps", type=int, default=40000,
                    help="VV steps of the developed-channel FP32-vs-FP64 run")
    ap.add_argument("--cpu-sample-steps", type=int, default=2)
    return ap.parse_args()


# ---------------------------------------------------------------- dist
def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist

        backend = "nccl"
        try:
            import torch

            if not torch.cuda.is_available():
                backend = "gloo"
            else:
                torch.cuda.set_device(local)
        except Exception:
            backend = "gloo"
        dist.init_process_group(backend=backend)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(val: float, ws: int) -> float:
    if ws == 1:
        return val
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([val], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_throughput(per_rank_units: float, max_seconds: float, ws: int) -> float:
    """Whole-job particle-steps/s: all ranks' work over the slowest rank."""
    return per_rank_units * ws / max_seconds


# -------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 8:
                    continue
                try:
                    sm.append(float(parts[0]))
                    smax.append(float(parts[1]))
                except ValueError:
                    continue
                for nm, val in zip(names, parts[4:8]):
                    if val.lower() == "active":
                        reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------- CPU baseline
def cpu_baseline(w, steps: int, threads: int | None = None) -> dict:
    """The CPU restatement of MCF's step on the host cores, in MCF's own loop
    mode (symmetry = T: each pair once, half-shell cell pairs, ghost put),
    parallelised over x-slabs of cells in two colours; beside it the
    full-stencil loops (symmetry = F, every pair from both sides) and one
    core with the symmetric loops (one MCF MPI rank's work)."""
    from oracle.oracle import Oracle

    threads = threads or os.cpu_count() or 1

    def timed(symmetry):
        p = w.params.copy()
        p.symmetry = symmetry
        o = Oracle(p, threads=threads)
        o.upload(w.x, w.v, w.m, w.id)
        o.marching_init_force(0)
        t0 = time.perf_counter()
        o.run_vv(0, steps, w.dt)
        return time.perf_counter() - t0

    dt = timed(1)
    out = {"value": w.n_fluid * steps / dt, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"{w.name}: {steps} full VV steps of all {w.n} particles "
                     f"({w.n_fluid} fluid), MCF's symmetric loops (symmetry = T) on "
                     f"{threads} threads, {dt:.1f} s",
           "seconds_per_step": dt / steps, "cpu_model": cpu_model()}
    if threads > 1:
        dtf = timed(0)
        out["full_stencil"] = {"value": w.n_fluid * steps / dtf, "unit": UNIT, "cores": threads,
                               "seconds_per_step": dtf / steps,
                               "sample": "the same steps with the full-stencil loops "
                                         "(symmetry = F, each pair from both sides)"}
        # one core, MCF's symmetric loops: the work of one MCF MPI rank,
        # on a 40^3 sub-box of the same workload (one step, a few seconds)
        from mcf_gb300 import configs
        ws_ = configs.c3_poiseuille_3d(n_side=40)
        o1 = Oracle(ws_.params, threads=1)
        o1.upload(ws_.x, ws_.v, ws_.m, ws_.id)
        o1.marching_init_force(0)
        t0 = time.perf_counter()
        o1.run_vv(0, 1, ws_.dt)
        t1 = time.perf_counter() - t0
        out["single_core"] = {"value": ws_.n_fluid / t1, "unit": UNIT, "cores": 1,
                              "sample": f"1 full VV step of the 40^3 + walls sub-box "
                                        f"({ws_.n} particles), symmetric loops, {t1:.1f} s"}
    return out


def cpu_model() -> str:
    """The host CPU's model name (Linux /proc/cpuinfo; Arm hosts may only
    name the implementer and part), with the core count."""
    name = ""
    try:
        for line in open("/proc/cpuinfo"):
            k = line.split(":", 1)[0].strip().lower()
            if k in ("model name", "cpu model", "hardware") and not name:
                name = line.split(":", 1)[1].strip()
            elif k == "cpu part" and not name:
                part = line.split(":", 1)[1].strip()
                name = {"0xd4f": "Arm Neoverse V2", "0xd40": "Arm Neoverse V1",
                        "0xd0c": "Arm Neoverse N1"}.get(part, "Arm cpu part " + part)
    except OSError:
        pass
    import platform
    return f"{name or platform.processor() or platform.machine()} ({os.cpu_count()} cores)"


def run_reference(args, ws, rank):
    """Reference arm: the CPU path on all host cores.  A step is one full VV
    step of a slice of the same workload: the full 100 sites along x (the
    threads take x-slabs of cells in two colours, so a narrower box would
    leave cores idle) and fewer along y and z, sized from a one-step
    calibration so that warm-up plus timed steps take about two minutes."""
    from mcf_gb300 import configs
    from oracle.oracle import Oracle

    if rank != 0:
        return
    threads = os.cpu_count() or 1

    def make(n_yz):
        w = configs.c3_poiseuille_3d(n_side=args.n_side, n_yz=n_yz)
        p = w.params.copy()
        p.symmetry = 1  # MCF's own loop mode: half-shell pairs, each once
        o = Oracle(p, threads=threads)
        o.upload(w.x, w.v, w.m, w.id)
        o.marching_init_force(0)
        return w, o

    n_yz = min(args.n_side, 24)
    w, o = make(n_yz)
    t0 = time.perf_counter()
    o.run_vv(0, 1, w.dt)
    t1 = time.perf_counter() - t0
    budget = 120.0
    nsteps = args.warmup + args.steps
    scale = (budget / max(nsteps * t1, 1e-9)) ** 0.5
    n_new = int(max(12, min(args.n_side, n_yz * scale)))
    if n_new != n_yz:
        w, o = make(n_new)
        o.run_vv(0, 1, w.dt)
    o.run_vv(1, args.warmup, w.dt)
    t0 = time.perf_counter()
    o.run_vv(1 + args.warmup, args.steps, w.dt)
    dt = time.perf_counter() - t0
    value = w.n_fluid * args.steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": w.name + " with y-walls (CPU slice of the 100^3 workload)",
                   "n_fluid": w.n_fluid, "n_wall": w.n - w.n_fluid,
                   "note": "CPU restatement of MCF's FP64 SDPD step (MCF is Fortran+MPI and "
                           "cannot be built here) with MCF's symmetric loops (symmetry = T), "
                           "x-slabs of cells in two colours over all host cores"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{args.steps} timed full VV steps of a {w.n_fluid}-fluid "
                                   f"sub-box of the 1M workload ({w.n} particles)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------- GPU arm
def timed_run(sd, torch, nsteps, step0, dt, ws):
    stream = torch.cuda.ExternalStream(sd.stream())
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    barrier(ws)
    torch.cuda.synchronize()
    l0 = sd.info()["kernel_launches"]
    e0.record(stream)
    sd.run_vv(step0, nsteps, dt)
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    barrier(ws)
    launches = sd.info()["kernel_launches"] - l0
    return e0.elapsed_time(e1) / 1e3, launches


def roofline_for(sd, torch, w, prec_idx, peaks, step0, clock_mhz=None):
    sd.set_profiling(2)
    sd.set_profiling(1)
    sd.run_vv(step0, 5, w.dt)
    sd.set_profiling(0)
    ph = sd.phase_times()
    phases = {k: v for k, v in ph.items() if k in ALGO_BYTES and v[1] > 0}
    top = max(phases, key=lambda k: phases[k][0])
    avg_ms = phases[top][0] / phases[top][1]
    algo = ALGO_BYTES[top][prec_idx] * w.n
    achieved = algo / (avg_ms / 1e3) / 1e9
    peak = peaks.get("hbm_gbs")
    share = {k: round(v[0] / sum(x[0] for x in phases.values()), 4) for k, v in phases.items()}
    # DRAM bytes per particle of this kernel from the committed ncu summary
    # (a smaller case of the same workload, scaled by the particles)
    traffic = None
    issue = None
    tf = ROOT / "profiles" / "traffic.json"
    if tf.exists():
        prof = json.loads(tf.read_text())
        per = prof.get("fp64" if prec_idx else "fp32", {}).get(top)
        if per:
            traffic = per * w.n
        # the pair sweeps are bound by instruction issue, not HBM: warp
        # instructions per particle of the same ncu capture over this
        # launch's time, against 4 warp instructions per clock per SM at
        # the clock sampled during the timed steps
        wi = prof.get("warp_instructions_per_particle", {}).get(
            "fp64" if prec_idx else "fp32", {}).get(top)
        if wi and clock_mhz:
            sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
            ach = wi * w.n / (avg_ms / 1e3)
            pk = 4.0 * sms * clock_mhz * 1e6
            issue = {"achieved": ach, "peak": pk, "unit": "warp instructions/s", "frac": ach / pk,
                     "warp_instructions_per_launch": wi * w.n, "sms": sms,
                     "clock_mhz": clock_mhz}
    fp64_pipe = None
    if prec_idx and tf.exists():
        # the FP64 path is bound by the FP64 pipe: its busy fraction and the
        # FLOP rate (ncu FLOPs per particle of the same sweep on 64^3 x this
        # launch's particles / its event time) against 2 DFMA a clock per SM
        fp = json.loads(tf.read_text()).get("fp64_pipe", {}).get(top)
        if fp:
            sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
            clk = clock_mhz or 2070.0
            ach = fp["flop_per_particle"] * w.n / (avg_ms / 1e3)
            pk = 4.0 * sms * clk * 1e6
            fp64_pipe = {"kernel": fp["kernel"], "pipe_active_ncu": fp["pipe_active"],
                         "flop_frac_ncu": fp["flop_frac"], "achieved": ach / 1e12, "peak": pk / 1e12,
                         "unit": "TFLOP/s", "frac": ach / pk,
                         "peak_source": f"nominal: {sms} SMs x 2 DFMA x 2 FLOP x {clk:.0f} MHz"}
    fp32_flops = None
    if not prec_idx and tf.exists():
        # FP32 (non-tensor) FLOP rate of the FP32 sweep: ncu's FADD + FMUL +
        # 2 FFMA per particle of the same sweep on 64^3 x this launch's
        # particles / its event time, against 128 FP32 lanes x 2 FLOP per
        # clock per SM; beside it the pair-body model of the algorithmic
        # FLOPs (~80 a pair side for the Hu-Adams force, ~25 for the
        # density, without the noise's integer work)
        fl = json.loads(tf.read_text()).get("fp32_flop_per_particle", {}).get(top)
        if fl:
            sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
            clk = clock_mhz or 2070.0
            ach = fl * w.n / (avg_ms / 1e3)
            pk = 256.0 * sms * clk * 1e6
            per_pair = {"force": 80, "density": 25}.get(top)
            info = sd.info()
            pairs = info["num_pairs"] / max(w.n, 1)
            fp32_flops = {"achieved": ach / 1e12, "peak": pk / 1e12, "unit": "TFLOP/s",
                          "frac": ach / pk, "flop_per_particle_ncu": fl,
                          "algorithmic_flop_per_particle":
                              (per_pair * pairs) if per_pair else None,
                          "peak_source": f"nominal: {sms} SMs x 128 FP32 lanes x 2 FLOP x "
                                         f"{clk:.0f} MHz"}
    return {"kernel_phase": top, "bound": "fp64 pipe" if prec_idx else "hbm",
            "achieved": achieved, "peak": peak,
            "unit": "GB/s", "frac": (achieved / peak) if peak else None, "traffic": traffic,
            "avg_ms": avg_ms, "algo_bytes_per_launch": algo,
            "peak_source": peaks.get("source"), "phase_share": share, "issue": issue,
            "fp64_pipe": fp64_pipe, "fp32_flops": fp32_flops}


def adjoint_cost(torch, w, T, K, local, wts):
    """Wall time of mcfg_adjoint_run (J and dJ/d(eta, tau, c) over T steps,
    checkpoints every K) against the forward trajectory it differentiates
    (mcfg_init_force + mcfg_run_vv of the same T steps), both after a warm-up
    call; returns the ratio and both times."""
    from mcf_gb300 import SDPD

    w.params.device = local
    w.params.stress_tensor = 1
    sd = SDPD(w.params)

    def fwd():
        sd.upload(w.x, w.v, w.m, w.id)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sd.marching_init_force(0)
        sd.run_vv(0, T, w.dt)
        sd.synchronize()
        return time.perf_counter() - t0

    def adj():
        sd.upload(w.x, w.v, w.m, w.id)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        J, g = sd.adjoint_run(0, T, w.dt, wts, checkpoint_every=K)
        return time.perf_counter() - t0, J, g

    fwd()
    adj()
    tf = min(fwd() for _ in range(3))
    ta, J, g = min((adj() for _ in range(3)), key=lambda r: r[0])
    return {"workload": w.name, "n": w.n, "steps": T, "checkpoint_every": K,
            "forward_ms": 1e3 * tf, "adjoint_ms": 1e3 * ta, "adjoint_over_forward": ta / tf,
            "reverse_over_forward": (ta - tf) / tf,
            "J": J, "dJ_deta_tau_c": [float(x) for x in g],
            "timing": "wall clock, best of 3 after a warm-up call; adjoint_over_forward is the "
                      "whole gradient (its own forward pass with checkpoints, the segment "
                      "recomputation and the reverse sweep) over the forward trajectory; "
                      "reverse_over_forward leaves out the forward pass that evaluates J"}


def fp32_accuracy(w, steps, local, seeds=(0,), samples=20, floor_seed=None):
    """FP32-mixed against FP64 over `steps` VV steps from the same state,
    for each seed offset in `seeds` (the Philox key of the Wiener increments
    is params.seed + offset, the same in both precisions, so the only
    difference is FP32 pair arithmetic).  Per seed: the bulk mean velocity
    and the velocity profile u_x(y) in unit slabs at the end; averaged over
    `samples` snapshots of the second half of the run, the wall shear stress
    (x-force of the fluid on each wall's particles per wall area) and the
    shear-stress profile tau_xy(y) (per-particle stresses s_xy summed per
    unit slab over the slab volume).  Errors are relative to the FP64
    run's scale; mean and max over the seeds are reported.  With floor_seed,
    the same errors between the FP64 run and an FP64 run with the Philox key
    offset by floor_seed (another noise realisation) are reported beside them
    as the statistical floor: once the trajectories have decorrelated, the
    FP32-vs-FP64 differences of time-averaged quantities are thermal noise
    unless they exceed that floor."""
    import numpy as np

    from mcf_gb300 import SDPD
    from mcf_gb300.params import PRECISION_FP32_MIXED, PRECISION_FP64

    sid = w.id[:, 1]
    fl = sid == 0
    P = w.params
    d = int(P.num_dim)
    lx = P.max_phys[0] - P.min_phys[0]
    lz = (P.max_phys[2] - P.min_phys[2]) if d == 3 else 1.0
    area = lx * lz
    nb = int(round(P.max_phys[1] - P.min_phys[1]))
    wall_sids = sorted(set(int(q) for q in np.unique(sid) if q < 0))

    def slab(x):
        return np.clip(np.floor(x[:, 1] - P.min_phys[1]).astype(int), 0, nb - 1)

    def run(prec, seed):
        p = P.copy()
        p.precision = prec
        p.stress_tensor = 1
        p.device = local
        p.seed = P.seed + seed
        sd = SDPD(p)
        sd.upload(w.x, w.v, w.m, w.id)
        sd.marching_init_force(0)
        half = steps // 2
        sd.run_vv(0, half, w.dt)
        walls, taus = [], []
        every = max(1, (steps - half) // samples)
        s0 = half
        while s0 + every <= steps:
            sd.run_vv(s0, every, w.dt)
            s0 += every
            st = sd.download("x", "f", "s")
            f, x = st["f"], st["x"]
            walls.append([float((w.m[sid == q] * f[sid == q, 0]).sum() / area) for q in wall_sids])
            sxy = 0.5 * (st["s"][:, 1] + st["s"][:, d])
            taus.append(np.bincount(slab(x[fl]), weights=sxy[fl], minlength=nb) / area)
        if s0 < steps:
            sd.run_vv(s0, steps - s0, w.dt)
        e = sd.download("x", "v")
        del sd
        prof = np.bincount(slab(e["x"][fl]), weights=e["v"][fl, 0], minlength=nb) / np.maximum(
            np.bincount(slab(e["x"][fl]), minlength=nb), 1)
        return {"u": float(e["v"][fl, 0].mean()), "prof": prof,
                "walls": np.mean(walls, axis=0) if walls else np.zeros(0),
                "tau": np.mean(taus, axis=0) if taus else np.zeros(nb)}

    def compare(a, b, errs):
        errs["mean_velocity_rel"].append(abs(a["u"] - b["u"]) / abs(b["u"]))
        errs["velocity_profile_rel"].append(
            float(np.max(np.abs(a["prof"] - b["prof"])) / np.max(np.abs(b["prof"]))))
        if len(b["walls"]):
            errs["wall_shear_stress_rel"].append(
                float(np.max(np.abs(a["walls"] - b["walls"]) / np.abs(b["walls"]))))
        errs["shear_stress_profile_rel"].append(
            float(np.max(np.abs(a["tau"] - b["tau"])) / np.max(np.abs(b["tau"]))))

    keys = ("mean_velocity_rel", "velocity_profile_rel", "wall_shear_stress_rel",
            "shear_stress_profile_rel")
    errs = {k: [] for k in keys}
    floor = {k: [] for k in keys}
    ref = {"mean_velocity_fp64": [], "wall_shear_stress_fp64": [], "max_shear_stress_fp64": []}
    for sd_off in seeds:
        a, b = run(PRECISION_FP32_MIXED, sd_off), run(PRECISION_FP64, sd_off)
        compare(a, b, errs)
        if floor_seed is not None:
            compare(run(PRECISION_FP64, sd_off + floor_seed), b, floor)
        ref["mean_velocity_fp64"].append(b["u"])
        ref["wall_shear_stress_fp64"].append([float(q) for q in b["walls"]])
        ref["max_shear_stress_fp64"].append(float(np.max(np.abs(b["tau"]))))
    out = {"steps": steps, "dt": w.dt, "seeds": len(seeds), "samples": samples}
    for k, vals in errs.items():
        if vals:
            out[k] = {"mean": float(np.mean(vals)), "max": float(np.max(vals))}
    if floor_seed is not None:
        out["fp64_other_seed"] = {k: {"mean": float(np.mean(v)), "max": float(np.max(v))}
                                  for k, v in floor.items() if v}
        out["fp64_other_seed"]["what"] = (
            "the same errors between FP64 runs with different Philox keys: the thermal-noise "
            "floor of the time averages")
    out.update(ref)
    out["reference"] = "the FP64 GPU path (itself within 1e-12 of the CPU oracle per step)"
    return out


def developed_channel(local, steps=40000):
    """FP32-mixed against FP64 on a developed Poiseuille flow: a 3D channel
    of 20 x 20 x 20 lattice sites between solid y walls (Morris no-slip, 4
    wall layers per side), C3's fluid (c = 20, eta = 0.5, kT = 1e-4 with the
    Wiener increments) driven by g_x = 0.005 (u_max ~ 0.5, Mach 0.025), dt =
    0.01 (MCF's criteria allow 0.0125), run to t = 400, two viscous times
    L^2/nu (the slowest transient mode has decayed to e^-10)."""
    from mcf_gb300 import configs

    w = configs.poiseuille_channel(dim=3, n_side=20, force=0.005)
    p = w.params
    p.c = 20.0
    p.eta = 0.5
    p.kt = 1e-4
    p.Brownian = 1
    w.dt = 0.01
    p.dt = 0.01
    out = fp32_accuracy(w, steps, local, seeds=(0,), samples=40, floor_seed=1000)
    out["workload"] = ("developed Poiseuille channel 20^3 + walls (c 20, eta 0.5, kT 1e-4, "
                       "g_x 0.005, dt 0.01)")
    nu = p.eta / 1.0
    out["u_max_analytic"] = 0.005 * 20.0 ** 2 / (8.0 * nu)
    return out


def colloid_suspension(args, local, ws, torch):
    """C4: 96^3 lattice with 200 rigid spheres (radius 4 dx, DLVO repulsion,
    g_x = 0.05, kT = 1e-3), the colloids integrated on the device
    (Adams-Bashforth order 2, mcfg_set_colloid_dynamics).  FP32-mixed with
    list reuse: particle-steps/s over the timed steps (all particles: solvent
    and boundary).  Then FP32-mixed against FP64 over args.c4_steps steps
    from the same state and Philox key: the colloids' velocities V and
    angular velocities Omega, error relative to each quantity's largest
    FP64 magnitude."""
    import math

    import numpy as np

    from mcf_gb300 import SDPD, configs
    from mcf_gb300.params import PRECISION_FP32_MIXED, PRECISION_FP64, ColloidDynamics

    w, cs = configs.c4_colloids()
    cd = ColloidDynamics()
    cd.integrate_AB = 2
    cd.sub_time_step = 1
    cd.body_force_type = 1
    cd.body_force[0] = w.params.body_force[0]
    m = 4.0 / 3.0 * math.pi * cs.radius ** 3.0
    mmi = np.repeat((0.4 * m * cs.radius ** 2)[:, None], 3, 1)

    def make(prec, reuse):
        p = w.params.copy()
        p.precision = prec
        p.device = local
        p.reserved[1] = reuse
        sd = SDPD(p)
        sd.upload(w.x, w.v, w.m, w.id)
        sd.set_colloids(cs.params, cs.x, cs.v, cs.omega, cs.radius)
        sd.set_colloid_dynamics(cd, m, mmi)
        sd.marching_init_force(0)
        return sd

    sd = make(PRECISION_FP32_MIXED, 1)
    sd.run_vv(0, args.warmup, w.dt)
    k = max(3, min(args.steps, 100))
    t, launches = timed_run(sd, torch, k, args.warmup, w.dt, ws)
    t = max_over_ranks(t, ws)
    out = {"workload": f"{w.name} (the colloids integrated on the device, AB2), FP32-mixed "
                       "with list reuse",
           "n": w.n, "n_boundary": int((w.id[:, 1] > 0).sum()), "n_colloid": int(cs.x.shape[0]),
           "value": aggregate_throughput(w.n * k, t, ws), "unit": UNIT,
           "ms_per_step": 1e3 * t / k, "steps": k, "gpu_launches": int(launches)}
    del sd
    if args.c4_steps > 0:
        res = {}
        for name, prec in (("fp32", PRECISION_FP32_MIXED), ("fp64", PRECISION_FP64)):
            sd = make(prec, 1)
            sd.run_vv(0, args.c4_steps, w.dt)
            res[name] = sd.colloid_state()
            del sd
        a, b = res["fp32"], res["fp64"]
        out["fp32_error_vs_fp64"] = {
            "steps": args.c4_steps,
            "velocity_rel": float(np.max(np.abs(a["v"][0] - b["v"][0])) /
                                  np.max(np.abs(b["v"][0]))),
            "angular_velocity_rel": float(np.max(np.abs(a["omega"][0] - b["omega"][0])) /
                                          np.max(np.abs(b["omega"][0]))),
            "centre_abs": float(np.max(np.abs(a["x"] - b["x"]))),
            "max_velocity_fp64": float(np.max(np.abs(b["v"][0]))),
            "max_angular_velocity_fp64": float(np.max(np.abs(b["omega"][0])))}
    return out


def run_ours(args, ws, rank, local):
    import numpy as np
    import torch

    from mcf_gb300 import SDPD, configs
    from mcf_gb300.params import PRECISION_FP32_MIXED, PRECISION_FP64

    torch.cuda.set_device(local)
    # with several ranks every replica would repeat the single-GPU studies
    # (minutes each, all GPUs held): the N-GPU line keeps the headline, the
    # FP64 line and e2e; the studies run at N = 1
    single_gpu_studies = ws == 1
    if not single_gpu_studies:
        args.no_accuracy = args.no_lees_edwards = args.no_colloids = True
        args.no_mcf_deck = args.no_adjoint = args.no_output = True
    peaks = {}
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists():
        peaks = json.loads(pk.read_text())
        peaks["source"] = "measured (MEASURED_PEAKS.json)"
    else:
        peaks = {"hbm_gbs": 6800.0, "source": "fallback 6.8 TB/s"}

    head64 = args.precision == "fp64"
    w = configs.c3_poiseuille_3d(n_side=args.n_side,
                                 precision=PRECISION_FP64 if head64 else PRECISION_FP32_MIXED)
    w.params.device = local
    reuse = 0 if args.no_list_reuse else 1
    w.params.reserved[1] = reuse
    sd = SDPD(w.params)
    sd.upload(w.x, w.v, w.m, w.id)
    sd.marching_init_force(0)
    sd.run_vv(0, args.warmup, w.dt)
    r0 = sd.info()["list_rebuilds"]
    clk = ClockSampler(local)
    clk.start()
    t, launches = timed_run(sd, torch, args.steps, args.warmup, w.dt, ws)
    clocks = clk.stop()
    tmax = max_over_ranks(t, ws)
    value = aggregate_throughput(w.n_fluid * args.steps, tmax, ws)
    info = sd.info()
    list_reuse = None
    if reuse:
        list_reuse = {"skin": info["skin"], "rebuilds_in_timed_steps": info["list_rebuilds"] - r0,
                      "rebuilds_total": info["list_rebuilds"]}
    roof = roofline_for(sd, torch, w, 1 if head64 else 0, peaks, args.warmup + args.steps,
                        clocks.get("sm_mhz") if clocks else None)
    # the same FP32-mixed step with MCF's cell list rebuilt every step
    every_step = None
    if reuse:
        p1 = w.params.copy()
        p1.reserved[1] = 0
        sd1 = SDPD(p1)
        sd1.upload(w.x, w.v, w.m, w.id)
        sd1.marching_init_force(0)
        sd1.run_vv(0, args.warmup, w.dt)
        t1, _ = timed_run(sd1, torch, args.steps, args.warmup, w.dt, ws)
        t1 = max_over_ranks(t1, ws)
        every_step = {"value": aggregate_throughput(w.n_fluid * args.steps, t1, ws),
                      "unit": UNIT, "ms_per_step": 1e3 * t1 / args.steps}
        list_reuse["rebuild_every_step"] = every_step
        del sd1
    # FP32-mixed error against the FP64 path on the same state
    err = None
    fp64 = None
    if not args.no_fp64 and not head64:
        w64 = configs.c3_poiseuille_3d(n_side=args.n_side, precision=PRECISION_FP64)
        w64.params.device = local
        w64.params.reserved[1] = reuse
        sd64 = SDPD(w64.params)
        sd64.upload(w.x, w.v, w.m, w.id)
        sd64.marching_init_force(0)
        sd32 = SDPD(w.params)
        sd32.upload(w.x, w.v, w.m, w.id)
        sd32.marching_init_force(0)
        a = sd32.download("rho", "f")
        b = sd64.download("rho", "f")
        fl = w.id[:, 1] == 0
        err = {"density_max_rel": float(np.max(np.abs(a["rho"] - b["rho"]) / b["rho"])),
               "accel_rms_rel": float(np.sqrt(np.mean((a["f"][fl] - b["f"][fl]) ** 2)) /
                                      np.sqrt(np.mean(b["f"][fl] ** 2)))}
        del sd32
        k64 = max(20, args.steps // 20)
        sd64.run_vv(0, 2, w.dt)
        t64, _ = timed_run(sd64, torch, k64, 2, w.dt, ws)
        t64 = max_over_ranks(t64, ws)
        v64 = aggregate_throughput(w.n_fluid * k64, t64, ws)
        roof64 = roofline_for(sd64, torch, w64, 1, peaks, 2 + k64,
                              clocks.get("sm_mhz") if clocks else None)
        fp64 = {"value": v64, "unit": UNIT, "steps": k64, "ms_per_step": 1e3 * t64 / k64,
                "fp32_mixed_speedup": value / v64, "roofline": roof64}
        del sd64
        if not args.no_accuracy:
            err["long_run"] = fp32_accuracy(w, args.accuracy_steps, local,
                                            seeds=tuple(range(args.accuracy_seeds)))
            err["long_run"]["workload"] = w.name + " with y-walls"
            err["developed_channel"] = developed_channel(local, args.channel_steps)
    # end to end through the C-ABI with host buffers
    e2e = None
    if not args.no_e2e:
        n, d = w.n, 3
        # the caller's ordinary host arrays (as MCF's x, v are), page-locked
        # once through the library's mcfg_host_register
        st = sd.download("x", "v", "f")
        hx, hv, hf = (np.ascontiguousarray(st[k]) for k in ("x", "v", "f"))
        hm, hid = np.ascontiguousarray(w.m), np.ascontiguousarray(w.id)
        # each array is unregistered only if its own registration succeeded;
        # page-locking refused: the same steps on pageable arrays
        locked = []
        for a in (hx, hv):
            try:
                sd.host_register(a)
                locked.append(a)
            except Exception:
                break
        registered = len(locked) == 2
        ke = max(3, min(args.steps, 20))
        step = args.warmup + args.steps + 10

        import ctypes as C
        dp = C.POINTER(C.c_double)

        def step_e2e(s):
            # MCF's per-step drop-in, one call: x, v over, the step, x, v back
            # (the positions' copy back overlaps the sweeps on a second stream)
            rc = sd.lib.mcfg_step_vv_host(sd._h, s, w.dt, hx.ctypes.data_as(dp),
                                          hv.ctypes.data_as(dp))
            if rc != 0:
                raise RuntimeError(sd.lib.mcfg_last_error(sd._h).decode())

        # the particle set (masses, ids) and the initial forces go over once;
        # every step carries x, v both ways, the forces stay on the device
        sd.upload(hx, hv, hm, hid)
        sd.upload_force(hf)
        for q in range(2):
            step_e2e(step + q)
        try:
            barrier(ws)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for q in range(ke):
                step_e2e(step + 2 + q)
            torch.cuda.synchronize()
            te = max_over_ranks(time.perf_counter() - t0, ws)
        finally:
            for a in locked:
                sd.host_unregister(a)
        e2e = {"value": aggregate_throughput(w.n_fluid * ke, te, ws), "unit": UNIT,
               "h2d_bytes_per_step": int(n * 3 * 8 * 2),
               "d2h_bytes_per_step": int(n * 3 * 8 * 2), "steps": ke,
               "path": "mcfg_step_vv_host(x, v) per step on the caller's numpy arrays, "
                       + ("page-locked once with mcfg_host_register" if registered else
                          "pageable (mcfg_host_register refused)") +
                       ": x, v to the device, the step, "
                       "x, v back (masses, ids and the initial forces uploaded once before; the "
                       "forces stay on the device between steps)"}
    output = None
    if rank == 0 and not args.no_output:
        # MCF's particle output file of the whole workload, formatted on the
        # device (E16.8, io_write_particles.F90), copied once, written once
        import shutil
        tmpd = tempfile.mkdtemp(prefix="mcfg_out_")
        try:
            path = os.path.join(tmpd, "mcf_particles00000001.out")
            sd.write_particles(path)  # buffers allocated on the first call
            t0 = time.perf_counter()
            sd.write_particles(path)
            tw = time.perf_counter() - t0
            nbytes = os.path.getsize(path)
        finally:
            shutil.rmtree(tmpd, ignore_errors=True)
        output = {"particles": int(w.n), "bytes": int(nbytes), "seconds": tw,
                  "path": "mcfg_write_particles: device E16.8 formatting, one device-to-host "
                          "copy, one fwrite (to a temporary file)"}
    # Lees-Edwards shear (y faces sliding along x) on the same box: MCF's
    # cell list rebuilt every step, and the candidate list kept while the
    # images across the faces move less than the skin
    lees_edwards = None
    if not args.no_lees_edwards:
        kle = max(3, min(args.steps, 50))
        lees_edwards = {"workload": f"Lees-Edwards 3D {args.n_side}^3 FP32-mixed, shear rate 0.05, "
                                    "kT 1e-4, dt 1e-3", "steps": kle}
        for name, ru in (("rebuild_every_step", 0), ("list_reuse", 1)):
            wl = configs.lees_edwards(dim=3, n_side=args.n_side, shear_rate=0.05,
                                      precision=PRECISION_FP32_MIXED, kt=1e-4)
            wl.params.device = local
            wl.params.reserved[1] = ru
            sl = SDPD(wl.params)
            sl.upload(wl.x, wl.v, wl.m, wl.id)
            sl.marching_init_force(0)
            sl.run_vv(0, args.warmup, wl.dt)
            rb0 = sl.info()["list_rebuilds"]
            tl, _ = timed_run(sl, torch, kle, args.warmup, wl.dt, ws)
            tl = max_over_ranks(tl, ws)
            lees_edwards[name] = {"value": aggregate_throughput(wl.n * kle, tl, ws), "unit": UNIT,
                                  "ms_per_step": 1e3 * tl / kle}
            if ru:
                lees_edwards[name]["rebuilds_in_timed_steps"] = sl.info()["list_rebuilds"] - rb0
                lees_edwards[name]["skin"] = sl.info()["skin"]
            del sl
    # MCF's own 1M-particle scalability deck (cut-off 4 dx, Batchelor
    # equation of state, Hu-Adams angular force), read through
    # mcf_config.load_mcf_deck from a deck written in MCF's format
    colloids = None
    if not args.no_colloids:
        colloids = colloid_suspension(args, local, ws, torch)
    mcf_deck = None
    if not args.no_mcf_deck:
        from mcf_gb300.configs import write_mcf_scalability_deck
        from mcf_gb300.mcf_config import load_mcf_deck

        tmpd = tempfile.mkdtemp(prefix="mcfg_deck_")
        try:
            deck = load_mcf_deck(write_mcf_scalability_deck(tmpd, n_side=args.n_side),
                                 precision=PRECISION_FP32_MIXED, list_reuse=True)
        finally:
            import shutil
            shutil.rmtree(tmpd, ignore_errors=True)
        wd_ = deck.workload
        wd_.params.device = local
        sk = SDPD(wd_.params)
        sk.upload(wd_.x, wd_.v, wd_.m, wd_.id)
        sk.marching_init_force(0)
        sk.run_vv(0, args.warmup, deck.dt)
        kd = max(3, min(args.steps, 100))
        td, _ = timed_run(sk, torch, kd, args.warmup, deck.dt, ws)
        td = max_over_ranks(td, ws)
        inf = sk.info()
        mcf_deck = {"workload": f"MCF scalability deck {args.n_side}^3 (rc 4 dx, Batchelor gamma 7, "
                                "Hu-Adams angular), FP32-mixed with list reuse",
                    "value": aggregate_throughput(wd_.n * kd, td, ws), "unit": UNIT,
                    "ms_per_step": 1e3 * td / kd, "steps": kd, "dt": deck.dt,
                    "max_neigh": inf["max_neigh"], "pairs_per_step": inf["num_pairs"]}
        del sk
    adjoint = None
    if not args.no_adjoint:
        w5 = configs.c5_oldroyd_b_2d()
        w5.v = np.random.default_rng(55).normal(0, 1e-3, w5.v.shape)
        adjoint = adjoint_cost(torch, w5, 200, 20, local, [0.0, 0.5, 0.5, 0.0])
        w3 = configs.c2_fluctuating_3d(n_side=args.n_side)
        adjoint["periodic_3d"] = adjoint_cost(torch, w3, 20, 10, local,
                                              [0, 0.5, 0, 0.5, 0, 0, 0, 0, 0])
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(w, args.cpu_sample_steps)
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * tmax / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if head64 else "f32 (FP32-mixed; f64 state)",
        "data": "synthetic",
        "config": {"workload": w.name + " with y-walls", "n_fluid": w.n_fluid,
                   "n_wall": w.n - w.n_fluid, "precision": "FP64" if head64 else "FP32-mixed",
                   "kernel": "quintic rc=3dx", "force": "Hu-Adams + Philox Wiener",
                   "parallelism": f"replicas x{ws}",
                   "l2": (("inputs larger than L2" if info["device_bytes"] > L2_BYTES else
                           "inputs fit in L2 (not flushed between steps)") +
                          f" ({info['device_bytes'] / 1e6:.0f} MB device state, "
                          f"L2 {L2_BYTES / 1e6:.0f} MB)"),
                   "neighbour_capacity": info["neigh_capacity"], "max_neigh": info["max_neigh"],
                   "pairs_per_step": info["num_pairs"], "list_reuse": list_reuse},
        "roofline": roof, "fp64": fp64, "fp32_error_vs_fp64": err, "e2e": e2e,
        "adjoint": adjoint, "output_write": output, "lees_edwards": lees_edwards,
        "mcf_scalability_deck": mcf_deck, "colloid_suspension": colloids,
        "cpu_baseline": cpu, "clocks": clocks, "gpu_launches": int(launches),
        "single_gpu_studies": "in this line" if single_gpu_studies else
                              "run at N = 1 only (accuracy, C4, adjoint, Lees-Edwards, deck, output)",
        "pair_interactions_per_s": info["num_pairs"] * args.steps * ws / tmax,
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        run_ours(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
