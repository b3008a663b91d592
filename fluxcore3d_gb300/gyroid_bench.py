"""Gyroid TPMS heat sink benchmark: 384x192x192 (L = 48, t = 0.3), TRT with magic parameter 1/4,
link fractions from the linear interpolation of the level set, inlet u = 0.05, k_s/k_f = 200.

Reported:
  lattice      MLUPS of the fused engine at FP16 shifted storage and at FP32, with the main pass's
               device time and its achieved bandwidth against the measured copy peak;
  accuracy     FP32 and FP16 storage runs against the device FP64 run of the plain method
               (fluxcore3d_gb300.lattice64) from the same initial state after `steps` steps: velocity
               (relative L2 over fluid cells) and the temperature that each velocity field gives
               (relative max and L2), the thermal system solved to a 1e-10 FP64 residual, with the
               wall heat flow and the Nusselt number on the gyroid's L/4 = 12 cells;
  thermal      the steady thermal solve on the FP64 velocity with the 5-level geometric multigrid to
               a 1e-8 FP64 relative residual: plain FP64 BiCGSTAB around the FP32 V-cycle, the mixed
               solver (FP64 refinement around FP32 BiCGSTAB), and the plain solver with the exact FP64
               coarsest-level solve (coarse_solve="fp64").
"""
from __future__ import annotations

import time

import torch

SHAPE = (384, 192, 192)
WORKLOAD = ("gyroid TPMS 384x192x192 (L=48, t=0.3, linear-interpolation link fractions), TRT Lambda=1/4, "
            "u=0.05, Re=20 on L/4")


def _velocity(sim):
    from .geometry import C_NP
    sim.sync_f()
    f = sim.f.reshape(19, -1).double()
    c = torch.tensor(C_NP, dtype=torch.float64, device=f.device)
    return (c.t() @ f) / f.sum(0)


def _bytes_main(sim) -> int:
    """Algorithmic bytes of one main pass: 38 s per fluid cell off the planes, 1 flag byte per cell,
    9 B per link cell and 9 + 2 s per link (the same count as the pin-fin bench's roofline)."""
    s = 4 if sim.cfg.lbm_storage == "fp32" else 2
    N = sim.nx * sim.ny * sim.nz
    fluid = int((~sim.solid_flow).sum())
    d = sim.ibb_data
    links = int(d.n_links) if d is not None else 0
    link_cells = int(torch.unique(d.fluid_flat).numel()) if links else 0
    return 38 * s * fluid + N + 9 * link_cells + (9 + 2 * s) * links


def lattice_block(dev, storage, steps=200, min_seconds=1.0, peak_gbs=None, **kw):
    from . import case as cases
    from .solver.lbm_cuda_ext import LBMCUDAUpgrade
    sim = cases.gyroid(device=dev, storage=storage, **kw)
    sim.cfg.macro_stride = 100
    LBMCUDAUpgrade.patch(sim)
    for _ in range(50):
        sim.step(do_thermal=False)
    torch.cuda.synchronize()
    times = []
    while sum(times) < min_seconds * 1e3 and len(times) < 200:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            sim.step(do_thermal=False)
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) / steps)
    times.sort()
    ms = times[len(times) // 2]
    if not bool(torch.isfinite(_velocity(sim)).all()) or sim._fc.check_device_error():
        raise RuntimeError(f"gyroid lattice ({storage}): state not finite or device error")
    main_ms = sim._fc.time_passes(50)["main"]
    nbytes = _bytes_main(sim)
    N = sim.nx * sim.ny * sim.nz
    out = {"mlups": round(N / ms / 1e3, 1), "ms_per_step": round(ms, 5), "timed_blocks": len(times),
           "main_ms": round(main_ms, 5), "main_algorithmic_bytes": nbytes,
           "main_achieved_gbs": round(nbytes / main_ms / 1e6, 1)}
    if peak_gbs:
        out["main_frac_of_measured_hbm"] = round(nbytes / main_ms / 1e6 / peak_gbs, 4)
    del sim
    torch.cuda.empty_cache()
    return out


def _temperature(ref, u):
    from . import thermal_bench
    from .solver import mg_pcg
    uu = u.to(torch.float32).reshape((3,) + (ref.nx, ref.ny, ref.nz))
    mg, b = thermal_bench.thermal_system(ref, uu[0], uu[1], uu[2])
    x, info = mg_pcg.bicgstab_mg_f64(mg, b, tol=1e-10, max_it=800)
    if not info["converged"]:
        raise RuntimeError(f"gyroid thermal solve did not converge: {info['res_rel']:.3e}")
    return x.double(), mg, b


def accuracy_block(dev, steps, **kw):
    from . import case as cases
    from .lattice64 import Lattice64
    from .solver.lbm_cuda_ext import LBMCUDAUpgrade
    ref = cases.gyroid(device=dev, storage="fp32", **kw)
    lat = Lattice64(ref)
    t = time.perf_counter()
    lat.step(steps - 500)
    prev = lat.velocity()
    lat.step(500)
    torch.cuda.synchronize()
    fp64_s = time.perf_counter() - t
    lat.check()
    fluid = ~ref.solid_flow.reshape(-1)
    vel = {"fp64": lat.velocity()}
    change = float(torch.linalg.norm((vel["fp64"] - prev)[:, fluid]) / torch.linalg.norm(vel["fp64"][:, fluid]))
    del lat
    for storage in ("fp32", "fp16"):
        sim = cases.gyroid(device=dev, storage=storage, **kw)
        sim.cfg.macro_stride = 100
        LBMCUDAUpgrade.patch(sim)
        for _ in range(steps):
            sim.step(do_thermal=False)
        if sim._fc.check_device_error():
            raise RuntimeError(f"gyroid accuracy run ({storage}): device error word set")
        vel[storage] = _velocity(sim)
        del sim
    U64 = vel["fp64"][:, fluid]
    out = {"steps": steps, "fp64_run_s": round(fp64_s, 2), "fp64_velocity_change_last_500_steps": change,
           "velocity_rel_l2": {}, "temperature_rel_max": {}, "temperature_rel_l2": {}, "wall_heat_flow_rel": {},
           "nusselt": {}, "nusselt_rel": {}}
    from .diagnostics import wall_heat
    T, heat = {}, {}
    k_np = ref.k.cpu().numpy().astype("float64")
    solid_np = ref.solid.cpu().numpy()
    for name, u in vel.items():
        T[name] = _temperature(ref, u)[0]
        heat[name] = wall_heat(T[name].reshape(ref.nx, ref.ny, ref.nz).cpu().numpy(), k_np, solid_np, 12.0)
        out["nusselt"][name] = round(heat[name][2], 6)
    for name in ("fp32", "fp16"):
        out["velocity_rel_l2"][name] = float(torch.linalg.norm(vel[name][:, fluid] - U64) / torch.linalg.norm(U64))
        dT = T[name] - T["fp64"]
        out["temperature_rel_max"][name] = float(dT.abs().max() / T["fp64"].abs().max())
        out["temperature_rel_l2"][name] = float(torch.linalg.norm(dT) / torch.linalg.norm(T["fp64"]))
        out["wall_heat_flow_rel"][name] = abs(heat[name][0] - heat["fp64"][0]) / abs(heat["fp64"][0])
        out["nusselt_rel"][name] = abs(heat[name][2] - heat["fp64"][2]) / abs(heat["fp64"][2])
    return out, ref, vel["fp64"]


def thermal_block(dev, ref, u64, repeats=3):
    """Steady 5-level multigrid thermal solve to a 1e-8 FP64 residual on the FP64 velocity field."""
    from . import thermal_bench
    from .solver import mg_pcg
    uu = u64.to(torch.float32).reshape((3,) + (ref.nx, ref.ny, ref.nz))
    mg, b = thermal_bench.thermal_system(ref, uu[0], uu[1], uu[2], max_levels=5)
    out = {"levels": len(mg._levels), "coarsest_level": list(mg._levels[-1]["shape"]), "tol": 1e-8}

    def timed(fn):
        fn()
        ms, info = thermal_bench.time_solver(fn, repeats)
        return round(ms, 3), info

    ms, info = timed(lambda: mg_pcg.bicgstab_mg_f64(mg, b, tol=1e-8, max_it=400))
    out.update(plain_bicgstab_ms=ms, plain_bicgstab_it=info["it"], plain_res=info["res_rel"])
    ms, info = timed(lambda: mg_pcg.bicgstab_mg_mixed(mg, b, tol=1e-8, max_it=400))
    out.update(mixed_bicgstab_ms=ms, mixed_it=info["it"], mixed_res=info["res_rel"])
    # the same system with the exact FP64 solve of the coarsest level (24 x 12 x 12)
    torch.cuda.synchronize()
    t = time.perf_counter()
    mg64, b64 = thermal_bench.thermal_system(ref, uu[0], uu[1], uu[2], max_levels=5, coarse_solve="fp64")
    torch.cuda.synchronize()
    out["fp64_coarse_build_ms"] = round((time.perf_counter() - t) * 1e3, 1)
    ms, info = timed(lambda: mg_pcg.bicgstab_mg_f64(mg64, b64, tol=1e-8, max_it=400))
    out.update(fp64_coarse_bicgstab_ms=ms, fp64_coarse_bicgstab_it=info["it"], fp64_coarse_res=info["res_rel"])
    return out


def run(dev, accuracy_steps=6000, peak_gbs=None):
    out = {"workload": WORKLOAD, "cells": SHAPE[0] * SHAPE[1] * SHAPE[2]}
    lat = {s: lattice_block(dev, s, peak_gbs=peak_gbs) for s in ("fp16", "fp32")}
    out["lattice"] = lat
    out["fp16_over_fp32"] = round(lat["fp16"]["mlups"] / lat["fp32"]["mlups"], 3)
    acc, ref, u64 = accuracy_block(dev, accuracy_steps)
    out["accuracy"] = acc
    out["thermal"] = thermal_block(dev, ref, u64)
    return out
