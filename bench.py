"""Benchmark: D3Q19 CHT lattice throughput (MLUPS) on one GB300.

Workload (default): the pin-fin heat sink, 256x128x128 cells (4,194,304), base
plate + 16x8 jittered cylinders of radius 3.5 and height 80, interpolated
bounce-back with analytic link fractions, MRT collision, FP16 shifted
populations with FP32 collision, velocity inlet u = 0.08, pressure outlet,
walls at +-z, periodic in y, outlet sponge of 40 cells.  One step = one fused
pass + the inlet/outlet plane kernels.  The same case with FP32 populations
is timed as the plain-precision comparison, and the thermal MG-Krylov solve
time to a 1e-8 FP64 residual is reported beside it when available.  The
geometry set-up (voxel SDF, boundary links, Bouzidi fractions) is timed on the
384x192x192 gyroid and the 768x384x384 pin + gyroid hybrid, with scipy's host
distance transform on the gyroid as its CPU baseline; snapshot and checkpoint
I/O is timed on the pin-fin case.  The accuracy report compares FP16 and FP32
storage runs with an FP64 run of the plain method (velocity, temperature, wall
heat flow, Nusselt number) on a reduced pin fin.

The populations (2 x 159 MB at FP16) exceed the 129 MB L2, so no L2 flush is
inserted between steps.

--impl reference times the oracle's C restatement of the reference's CUDA-path
step (collide, sponge, stream, bounce-back, plane BCs) on the host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
RESULT_OUT = sys.stdout
sys.path.insert(0, ROOT)

METRIC = "D3Q19 CHT MLUPS + thermal ms to 1e-8 residual, mixed/learned vs plain, 1 GB300"
WORKLOAD = "pin-fin heat sink 256x128x128 (16x8 pins r=3.5 h=80, seed 1), MRT + Bouzidi IBB, u=0.08, Re=200"


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), float(d.get("bf16_tflops", 1900.0)), "measured"
    return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


KERNEL = {
    "tma": "k_fused_tma<FP16 shifted, MRT> (TMA-staged tiles: pull + link slots + packed collide of cell pairs + sponge)",
    "direct": "k_fused_step<FP16 shifted, MRT> (per-thread pull + bounce-back + collide + sponge)",
}
PROFILE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "profiles",
                       "k_fused_tma_fp16_mrt_pinfin_256x128x128.md")


def profiled_traffic(args):
    """DRAM bytes (read + write) of one launch of the dominant kernel, from the committed ncu
    summary of this workload (line 'dram_bytes_per_launch: N'), or (None, reason)."""
    default = (args.nx, args.ny, args.nz, args.collision, args.staging) == (256, 128, 128, "mrt", "tma")
    if not default or not os.path.exists(PROFILE):
        return None, "no ncu capture of this configuration"
    for line in open(PROFILE):
        if line.startswith("dram_bytes_per_launch:"):
            return int(line.split(":")[1].strip()), os.path.relpath(PROFILE, os.path.dirname(PROFILE) + "/..")
    return None, "no dram_bytes_per_launch line in the ncu summary"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def host_case(args):
    """The workload's lattice state built on the host cores alone, for the CPU legs: the same level
    set, mask and initial state as the device case, links from the oracle's link builder, fractions
    by the same FP64 bisection of the analytic level set on the CPU, Bouzidi weights from the oracle.
    No device library is loaded on this path."""
    import torch
    from fluxcore3d_gb300 import case as cases
    from fluxcore3d_gb300 import geometry as geo
    from oracle import geometry as og

    def host_ibb(solid, G):
        s = solid.cpu().numpy()
        ff, di, do, fff, fv = og.links_from_mask(s)
        q = geo.level_set_fractions(G, torch.from_numpy(ff), torch.from_numpy(di), s.shape).numpy()
        ge, w1, w2 = og.weights_from_q(q)
        t = torch.from_numpy
        return geo.IBBData(int(ff.size), t(ff), t(di), t(do), t(ge), t(w1), t(w2), t(fff), t(fv))

    sim = cases.pin_fin(device="cpu", collision=args.collision, storage="fp32", nx=args.nx, ny=args.ny, nz=args.nz,
                        ibb_builder=host_ibb)
    return sim


def oracle_of(sim, real="f32"):
    """The oracle lattice started from the case's state."""
    from oracle.lbm import OracleLBM
    d = sim.ibb_data
    links = {k: getattr(d, k).cpu().numpy() for k in
             ("fluid_flat", "dir_i", "dir_opp", "w_i", "w_second", "q_ge_half", "ff_flat", "ff_valid")}
    return OracleLBM(sim.nx, sim.ny, sim.nz, sim.f.cpu().numpy(), sim.solid_flow.cpu().numpy(),
                     collision=sim.cfg.collision, omega=float(sim.omega_plus),
                     S=sim._mrt_S.cpu().numpy() if hasattr(sim, "_mrt_S") else None,
                     sigma=sim._sponge_sigma.cpu().numpy() if sim.cfg.sponge_length > 0 else None, links=links,
                     domain_walls=sim.cfg.domain_walls, u_in_lat=sim.u_in_lat, real=real)


def bench_config(args):
    """The `config` object both arms print (one workload, whatever the storage precision)."""
    return {"workload": WORKLOAD, "cells": args.nx * args.ny * args.nz, "collision": args.collision,
            "macro_stride": args.macro_stride,
            "l2_flush": "inputs larger than L2 (2 x 159 MB FP16 / 2 x 319 MB FP32 populations)",
            "parallelism": "replicas"}


def make_case(device, storage, args):
    from fluxcore3d_gb300 import case as cases
    sim = cases.pin_fin(device=device, collision=args.collision, storage=storage, nx=args.nx, ny=args.ny,
                        nz=args.nz)
    sim.cfg.macro_stride = args.macro_stride
    sim.cfg.lbm_cells_per_thread = getattr(args, "cells_per_thread", 1)
    sim.cfg.lbm_staging = getattr(args, "staging", "tma")
    sim.cfg.lbm_link_pass = getattr(args, "link_pass", "inline")
    return sim


def lbm_traffic(sim, fc, storage_bytes):
    """Algorithmic bytes of one step's two fused passes.

    main pass : every fluid cell without links and off the inlet/outlet planes
                reads and writes its 19 populations once; every cell's flag byte is read.
    link pass : each link cell reads its 19 populations, its flag, list entry and
                link offset, writes 19 populations; each link reads 9 bytes of
                table (w1, w2, meta) and 2 extra populations of the cell."""
    N = sim.nx * sim.ny * sim.nz
    fl = fc.flags
    fluid = (fl & 1) == 0
    deferred = (fl & 4) != 0
    link = (fl & 2) != 0
    s = storage_bytes
    n_main = int((fluid & ~deferred & ~link).sum())
    n_lc = int((fluid & link).sum())
    main = n_main * 38 * s + N
    links = n_lc * (38 * s + 9) + fc.n_links * (9 + 2 * s)
    if not fc.separate_link_pass:        # link cells run inside the main pass
        main, links = main + links, 0
    return {"main": main, "links": links, "n_main": n_main, "n_link_cells": n_lc,
            "n_fluid": int(fluid.sum())}


class Restarter:
    """Keeps a timed lattice run inside its physically valid start-up window: plain MRT on the
    pin fin at Re = 200 diverges after about 600 steps (FP32 and FP64 alike), so before a block of
    steps would take the run past `max_age` steps since its start, the state is reset to the
    initial populations (outside the timed region; the engine is re-primed there too).  The cost
    of a step does not depend on the state, only on the geometry."""

    def __init__(self, sim, max_age):
        self.sim = sim
        self.max_age = int(max_age)
        self.f0 = sim.f.detach().clone()
        self.age = 0
        self.restarts = 0

    def before(self, steps):
        if self.max_age <= 0 or self.age + steps <= self.max_age:
            self.age += steps
            return
        self.sim.f.copy_(self.f0)
        self.sim._fc.invalidate()
        self.sim._fc._prime()
        self.age = steps
        self.restarts += 1


def time_steps(sim, steps, dev, min_seconds=1.0, ws=1, restarter=None):
    """Device time (ms) of `steps` solver steps, CUDA events on the current stream.  One untimed
    block of `steps` steps sizes the count R of timed blocks so that they add up to at least
    `min_seconds` (long enough for the clock sampler); every rank then times the same R blocks,
    each bracketed by a barrier and a synchronize.  A block longer than the restarter's window is
    timed as consecutive sub-blocks that each fit in it, the state being reset between them
    outside the timed regions, so every timed step runs on a finite state.  Returns the median
    block time and R."""
    import torch
    st = torch.cuda.current_stream()
    window = restarter.max_age if (restarter and restarter.max_age > 0) else steps
    parts = []
    left = steps
    while left > 0:
        parts.append(min(left, window))
        left -= parts[-1]

    def block():
        ms = 0.0
        for n in parts:
            if restarter:
                restarter.before(n)
            t0 = torch.cuda.Event(enable_timing=True)
            t1 = torch.cuda.Event(enable_timing=True)
            if ws > 1:
                torch.distributed.barrier()
            torch.cuda.synchronize()
            t0.record(st)
            for _ in range(n):
                sim.step(do_thermal=False)
            t1.record(st)
            torch.cuda.synchronize()
            ms += t0.elapsed_time(t1)
        return ms

    t = time.perf_counter()
    block()
    est = max(time.perf_counter() - t, 1e-6)
    reps = torch.tensor([max(1, min(20000, int(min_seconds / est) + 1))], device=dev)
    if ws > 1:
        torch.distributed.all_reduce(reps, op=torch.distributed.ReduceOp.MAX)
    blocks = [block() for _ in range(int(reps))]
    return statistics.median(blocks), len(blocks)


def run_reference(args):
    """CPU baseline: the oracle's C restatement of the reference step on all host cores, with the
    case built on the host (nothing of the device library is loaded)."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    sim = host_case(args)
    orc = oracle_of(sim)
    orc.step(args.warmup)
    t = time.perf_counter()
    orc.step(args.steps)
    dt = time.perf_counter() - t
    N = sim.nx * sim.ny * sim.nz
    v = N * args.steps / dt / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": round(v, 3), "unit": "MLUPS", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt * 1e3 / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": bench_config(args),
        "cpu_baseline": {"value": round(v, 3), "unit": "MLUPS", "cores": cores, "kind": "port",
                         "sample": f"{args.steps} full steps of the 256x128x128 workload with FP32 populations "
                                   f"(oracle C restatement of the reference's CUDA-path step, OpenMP)"},
        "e2e": {"value": round(v, 3), "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), file=RESULT_OUT, flush=True)


def _velocity_of(sim):
    """(3, N) FP64 velocity of the fused engine's current post-stream populations, on the device."""
    import torch
    from fluxcore3d_gb300.geometry import C_NP
    sim.sync_f()
    f = sim.f.reshape(19, -1).double()
    c = torch.tensor(C_NP, dtype=torch.float64, device=f.device)
    return (c.t() @ f) / f.sum(0)


def accuracy_run(args, dev):
    """FP32-, FP16- and BF16-storage runs of the fused engine against an FP64 run of the plain method
    (fluxcore3d_gb300.lattice64: the reference step sequence in double precision on the device), from
    the same initial state, on the full 256x128x128 pin fin with MRT-Smagorinsky, to steady state
    (`accuracy_steps` steps): velocity error, then the thermal system of each velocity field solved to a
    1e-10 FP64 residual, and the temperature, wall heat flow and Nusselt number of each against the
    FP64 run's.  Plain MRT at this Reynolds number does not reach a steady state (it diverges in FP32
    and FP64 alike after about 600 steps), so the steady-state comparison uses the reference's own
    default collision, MRT with the Smagorinsky model."""
    import torch
    from fluxcore3d_gb300 import case as cases
    from fluxcore3d_gb300 import thermal_bench
    from fluxcore3d_gb300.diagnostics import heat_balance, lbm_mass, wall_heat
    from fluxcore3d_gb300.lattice64 import Lattice64
    from fluxcore3d_gb300.solver import mg_pcg
    from fluxcore3d_gb300.solver.lbm_cuda_ext import LBMCUDAUpgrade
    steps = args.accuracy_steps
    shape = (args.nx, args.ny, args.nz)
    sims = {}
    for storage in ("fp32", "fp16", "bf16"):
        sim = cases.pin_fin(device=dev, storage=storage, collision="mrt_smag", nx=args.nx, ny=args.ny, nz=args.nz)
        sim.cfg.macro_stride = args.macro_stride
        if storage == "fp32":
            lat = Lattice64(sim)
        LBMCUDAUpgrade.patch(sim)
        sims[storage] = sim
    ref = sims["fp32"]
    torch.cuda.synchronize()
    t = time.perf_counter()
    lat.step(steps - 1000)
    prev = lat.velocity()
    lat.step(1000)
    torch.cuda.synchronize()
    fp64_s = time.perf_counter() - t
    lat.check()
    vel = {"fp64": lat.velocity()}
    fluid = ~ref.solid_flow.reshape(-1)
    steady = float(torch.linalg.norm((vel["fp64"] - prev)[:, fluid]) / torch.linalg.norm(vel["fp64"][:, fluid]))
    mass = {}
    for storage, sim in sims.items():
        m0 = lbm_mass(sim)
        for _ in range(steps):
            sim.step(do_thermal=False)
        mass[storage] = (lbm_mass(sim) - m0) / m0
        if sim._fc.check_device_error():
            raise RuntimeError(f"accuracy run ({storage}): device error word set")
        vel[storage] = _velocity_of(sim)
    U64 = vel["fp64"][:, fluid]
    out = {"workload": "pin fin 256x128x128 (16x8 pins r=3.5 h=80, seed 1), MRT-Smagorinsky (Cs=0.1) + Bouzidi "
                       "IBB, u=0.08, Re=200",
           "steps": steps, "fp64_run": f"device FP64 run of the reference step sequence, {fp64_s:.1f} s",
           "fp64_velocity_change_last_1000_steps": steady,
           "velocity_rel_l2": {}, "velocity_rel_max": {}, "temperature_rel_max": {}, "temperature_rel_l2": {},
           "wall_heat_flow_rel": {}, "nusselt": {}, "nusselt_rel": {}, "heat_balance": {}, "mass_rel_change": {}}
    k = ref.k.cpu().numpy().astype("float64")
    solid = ref.solid.cpu().numpy()
    T, heat = {}, {}
    for name in ("fp64", "fp32", "fp16", "bf16"):
        if name != "fp64":
            U = vel[name][:, fluid]
            out["velocity_rel_l2"][name] = float(torch.linalg.norm(U - U64) / torch.linalg.norm(U64))
            out["velocity_rel_max"][name] = float((U - U64).abs().max() / U64.abs().max())
        u = vel[name].to(torch.float32).reshape((3,) + shape)
        mg, b = thermal_bench.thermal_system(ref, u[0], u[1], u[2])
        x, info = mg_pcg.bicgstab_mg_f64(mg, b, tol=1e-10, max_it=600)
        T[name] = x.reshape(shape).cpu().numpy().astype("float64")
        hb = heat_balance(mg, x, b / 1000.0, 1000.0)
        out["heat_balance"][name] = {kk: (float(f"{vv:.6g}")) for kk, vv in hb.items()}
        heat[name] = wall_heat(T[name], k, solid, 2 * 3.5)
        out["nusselt"][name] = round(heat[name][2], 6)
    import numpy as np
    for name in ("fp32", "fp16", "bf16"):
        dT = T[name] - T["fp64"]
        out["temperature_rel_max"][name] = float(np.abs(dT).max() / np.abs(T["fp64"]).max())
        out["temperature_rel_l2"][name] = float(np.linalg.norm(dT) / np.linalg.norm(T["fp64"]))
        out["wall_heat_flow_rel"][name] = float(abs(heat[name][0] - heat["fp64"][0]) / abs(heat["fp64"][0]))
        out["nusselt_rel"][name] = float(abs(heat[name][2] - heat["fp64"][2]) / abs(heat["fp64"][2]))
    out["wall_faces"] = heat["fp64"][1]
    out["mass_rel_change"] = {kk: float(f"{vv:.6g}") for kk, vv in mass.items()}
    return out


def cpu_baseline_sample(args):
    """A bounded sample of the same workload on the host cores (oracle, FP32), case built on the host."""
    sim = host_case(args)
    orc = oracle_of(sim)
    orc.step(1)
    n = args.cpu_steps
    t = time.perf_counter()
    orc.step(n)
    dt = time.perf_counter() - t
    N = sim.nx * sim.ny * sim.nz
    return {"value": round(N * n / dt / 1e6, 3), "unit": "MLUPS", "cores": os.cpu_count() or 1, "kind": "port",
            "sample": f"{n} steps of the same 256x128x128 MRT+IBB workload, FP32 oracle C (OpenMP)"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="fluxcore3d_gb300")
    ap.add_argument("--collision", default="mrt")
    ap.add_argument("--nx", type=int, default=256)
    ap.add_argument("--ny", type=int, default=128)
    ap.add_argument("--nz", type=int, default=128)
    ap.add_argument("--macro-stride", type=int, default=100)
    ap.add_argument("--cells-per-thread", type=int, default=1, choices=(1, 2))
    ap.add_argument("--staging", default="tma", choices=("tma", "direct"),
                    help="main pass: TMA-staged tiles (default) or per-thread global loads")
    ap.add_argument("--link-pass", default="inline", choices=("inline", "separate"),
                    help="link cells inside the main pass (default) or in their own kernel (direct pass only)")
    ap.add_argument("--restart-every", type=int, default=400,
                    help="reset the lattice to its initial state (untimed) before it passes this many steps "
                         "(plain MRT at this Reynolds number diverges after ~600 steps); 0 = never")
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-thermal", action="store_true")
    ap.add_argument("--no-geometry", action="store_true", help="skip the voxel SDF / link builder timings")
    ap.add_argument("--no-io", action="store_true", help="skip the snapshot / checkpoint timings")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the FP16/FP32 vs FP64 accuracy report")
    ap.add_argument("--no-gyroid", action="store_true",
                    help="skip the gyroid TPMS block (TRT lattice, FP64 error, 5-level thermal solve)")
    ap.add_argument("--gyroid-steps", type=int, default=6000, help="steps of the gyroid accuracy runs")
    ap.add_argument("--no-coupled", action="store_true",
                    help="skip the coupled flow + heat run on the 768x384x384 hybrid heat sink")
    ap.add_argument("--coupled-steps", type=int, default=200, help="timed lattice steps of the coupled run")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-preconditioner training / A-B")
    ap.add_argument("--accuracy-steps", type=int, default=10000)
    ap.add_argument("--storages", default="fp16,fp32", help="population storages to time (first = headline)")
    ap.add_argument("--profile", action="store_true",
                    help="short run for ncu captures: headline storage only, no e2e / thermal / CPU legs")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.profile:
        args.storages = args.storages.split(",")[0]
        args.no_e2e = args.no_cpu = args.no_thermal = args.no_geometry = args.no_io = args.no_accuracy = True
        args.no_gyroid = args.no_coupled = True
        args.no_learned = True
    if args.impl == "reference":
        run_reference(args)
        return

    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from fluxcore3d_gb300 import _build
    _build.build()
    from fluxcore3d_gb300.solver.lbm_cuda_ext import LBMCUDAUpgrade

    hbm_peak, _, peak_kind = peaks()
    results = {}
    storages = args.storages.split(",")
    for storage in storages:
        sim = make_case(dev, storage, args)
        LBMCUDAUpgrade.patch(sim)
        restarter = Restarter(sim, args.restart_every)
        restarter.before(args.warmup)
        for _ in range(args.warmup):
            sim.step(do_thermal=False)
        torch.cuda.synchronize()
        sampler = ClockSampler(local) if storage == storages[0] else None
        if sampler:
            sampler.start()
        total_ms, blocks = time_steps(sim, args.steps, dev, min_seconds=0.0 if args.profile else 1.0, ws=ws,
                                      restarter=restarter)
        if ws > 1:
            tt = torch.tensor([total_ms], device=dev)
            torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
            total_ms = float(tt)
        clocks = sampler.stop() if sampler else None
        sbytes = 4 if storage == "fp32" else 2
        traffic = lbm_traffic(sim, sim._fc, sbytes)
        err = sim._fc.check_device_error()
        import math
        from fluxcore3d_gb300.diagnostics import lbm_mass
        finite = math.isfinite(lbm_mass(sim))            # FP64 sum of every population of the state
        n_pass = max(20, min(args.steps, 200))
        restarter.before(n_pass)
        passes = sim._fc.time_passes(n_pass)
        per_step = sim._fc.launches_per_step()
        results[storage] = dict(total_ms=total_ms, blocks=blocks, restarts=restarter.restarts, finite=finite,
                                passes=passes, traffic=traffic, clocks=clocks,
                                launches=per_step,
                                N=sim.nx * sim.ny * sim.nz, planes=len(sim._fc.planes),
                                links=sim._fc.n_links, err=err)
        del sim
    r = results[storages[0]]
    N = r["N"]
    traffic, traffic_src = profiled_traffic(args)
    mlups = N * args.steps / (r["total_ms"] / 1e3) / 1e6 * ws
    tr, ps = r["traffic"], r["passes"]
    achieved = tr["main"] / (ps["main"] / 1e3) / 1e9
    link_gbs = tr["links"] / (ps["links"] / 1e3) / 1e9 if ps.get("links") else None
    step_gbs = (tr["main"] + tr["links"]) / (r["total_ms"] / args.steps / 1e3) / 1e9
    launches_per_step = r["launches"]

    # end to end through the public API with host buffers
    e2e = None
    if not args.no_e2e:
        e2e = e2e_run(args, dev)

    line = {
        "metric": METRIC,
        "value": round(mlups, 1),
        "unit": "MLUPS",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(r["total_ms"] / args.steps, 5),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f16-storage/f32-compute",
        "data": "synthetic",
        "config": bench_config(args),
        "case": {"fluid_cells": tr["n_fluid"], "links": r["links"], "link_cells": tr["n_link_cells"],
                 "storage": storages[0], "timed_blocks": r["blocks"], "restarts": r["restarts"],
                 "state_finite_after_timing": r["finite"],
                 "restart_every": args.restart_every,
                 "timing": f"median of {r['blocks']} blocks of {args.steps} steps (CUDA events), "
                           f"blocks repeated to span >= 1 s; blocks longer than the restart window are timed "
                           f"as sub-blocks of at most {args.restart_every} steps"},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm_peak, "unit": "GB/s",
                     "frac": round(achieved / hbm_peak, 4), "traffic": traffic,
                     "kernel": KERNEL[args.staging],
                     "traffic_source": traffic_src,
                     "kernel_ms": round(ps["main"], 5),
                     "algorithmic_bytes": tr["main"], "peak_kind": peak_kind,
                     "link_pass": {"ms": round(ps.get("links", 0.0), 5), "algorithmic_bytes": tr["links"],
                                   "achieved": None if link_gbs is None else round(link_gbs, 1)},
                     "step_achieved": round(step_gbs, 1)},

        "clocks": r["clocks"],
        "gpu_launches": r["blocks"] * args.steps * launches_per_step,
        "device_error": r["err"],
    }
    for st_name in storages[1:]:
        q = results[st_name]
        line[st_name] = {"mlups": round(q["N"] * args.steps / (q["total_ms"] / 1e3) / 1e6, 1),
                         "main_ms": round(q["passes"]["main"], 5), "links_ms": round(q["passes"].get("links", 0), 5),
                         "main_achieved_gbs": round(q["traffic"]["main"] / (q["passes"]["main"] / 1e3) / 1e9, 1)}
    if "fp32" in line:
        line["fp16_over_fp32"] = round(line["value"] / max(line["fp32"]["mlups"], 1e-9), 3)
    if e2e:
        line["e2e"] = e2e
    if not args.no_thermal:
        try:
            th = thermal_run(args, dev)
            if th:
                if th.get("mixed_bicgstab_ms"):
                    th["mixed_speedup_over_plain"] = round(th["plain_bicgstab_ms"] / th["mixed_bicgstab_ms"], 3)
                line["thermal"] = th
        except ImportError:
            pass
    if not args.no_geometry:
        from fluxcore3d_gb300 import geometry_bench
        cpu_vox = None
        if rank == 0 and not args.no_cpu:
            from oracle import voxelizer as ov

            def cpu_vox(tri, origin, dims, pitch, ids):
                return ov.voxelize(tri, origin, dims, pitch, ray_ids=ids)
        line["geometry"] = geometry_bench.run(dev, cpu_baseline=(rank == 0 and not args.no_cpu),
                                              cpu_voxelize=cpu_vox)
    if not args.no_io:
        from fluxcore3d_gb300 import io_bench
        line["io"] = io_bench.run(dev)
    if rank == 0 and not args.no_learned:
        from fluxcore3d_gb300 import conv_bench, learned_bench
        line["learned"] = learned_bench.run(dev, eval_seeds=(1001, 1002))
        # the network's tcgen05 convolution alone: FLOP/s against the measured bf16 peak
        line["learned"]["conv_fwd"] = conv_bench.run(dev, bf16_peak_tflops=peaks()[1])
    if rank == 0 and not args.no_accuracy:
        line["accuracy"] = accuracy_run(args, dev)
    if rank == 0 and not args.no_coupled:
        from fluxcore3d_gb300 import coupled_bench
        line["coupled"] = coupled_bench.run(dev, steps=args.coupled_steps)
    if rank == 0 and not args.no_gyroid:
        from fluxcore3d_gb300 import gyroid_bench
        line["gyroid"] = gyroid_bench.run(dev, accuracy_steps=args.gyroid_steps, peak_gbs=peaks()[0])
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline_sample(args)
    if rank == 0:
        print(json.dumps(line), file=RESULT_OUT, flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def e2e_run(args, dev, min_seconds=1.0):
    """Public API end to end: initial populations uploaded from pinned host memory, K steps
    through sim.step(), final macro fields read back into pinned host memory; bytes are reported
    per step.  The block is repeated until the blocks span `min_seconds`; the median is reported."""
    import torch
    from fluxcore3d_gb300.solver.lbm_cuda_ext import LBMCUDAUpgrade
    sim = make_case(dev, "fp16", args)
    host_f = sim.f.cpu().pin_memory()
    out = torch.empty((4,) + tuple(sim.rho.shape), dtype=torch.float32).pin_memory()
    LBMCUDAUpgrade.patch(sim)
    for _ in range(args.warmup):
        sim.step(do_thermal=False)
    torch.cuda.synchronize()

    def block():
        t = time.perf_counter()
        sim.f.copy_(host_f, non_blocking=True)
        sim._fc.invalidate()
        for _ in range(args.steps):
            sim.step(do_thermal=False)
        out[0].copy_(sim.rho, non_blocking=True)
        out[1].copy_(sim.u, non_blocking=True)
        out[2].copy_(sim.v, non_blocking=True)
        out[3].copy_(sim.wv, non_blocking=True)
        torch.cuda.synchronize()
        return time.perf_counter() - t

    times = [block()]
    while sum(times) < min_seconds and len(times) < 20000:
        times.append(block())
    dt = statistics.median(times)
    N = sim.nx * sim.ny * sim.nz
    return {"value": round(N * args.steps / dt / 1e6, 1), "unit": "MLUPS",
            "h2d_bytes_per_step": int(host_f.numel() * 4 // args.steps),
            "d2h_bytes_per_step": int(out.numel() * 4 // args.steps),
            "blocks": len(times),
            "block": f"upload of the FP32 populations, {args.steps} sim.step() calls, read-back of rho/u/v/w; "
                     f"median over the blocks (wall clock)"}


def thermal_run(args, dev):
    from fluxcore3d_gb300 import thermal_bench
    return thermal_bench.run(dev)


if __name__ == "__main__":
    # stdout carries only the result line; progress lines of the solvers go to stderr
    RESULT_OUT = sys.stdout
    sys.stdout = sys.stderr
    main()
