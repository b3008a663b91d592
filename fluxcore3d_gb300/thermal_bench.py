"""Thermal solve benchmark: time to a 1e-8 FP64 relative residual on the pin-fin heat sink.

The velocity field comes from the fused lattice solver run on the same
geometry; the thermal system is the reference's pseudo-time operator
A = I + dt L (harmonic-mean conduction, first-order upwind convection) with a
large pseudo-time step, the inlet plane Dirichlet and a uniform heat flux into
the bottom layer of the base plate.  Plain method: FP64 BiCGSTAB (and FGMRES)
preconditioned by one FP32 V-cycle of the geometric multigrid.  Mixed method:
FP64 iterative refinement around an FP32 BiCGSTAB with the same preconditioner.
"""
from __future__ import annotations

import statistics
import time

import torch


def thermal_system(sim, u, v, w, dt=1000.0, flux=5e-3, max_levels=None, coarse_solve="jacobi"):
    """A = I + dt L for the velocity (u, v, w) on sim's geometry (zero velocity in flow-solid
    cells), inlet plane (x = 0) Dirichlet, a uniform heat flux into the bottom layer of the solid;
    returns (mg, b)."""
    from .solver.nlevel_mg_cuda import NLevelGeometricMGSolver
    dev = sim.device
    nx, ny, nz = sim.nx, sim.ny, sim.nz
    mask = torch.ones((nx, ny, nz), dtype=torch.bool, device=dev)
    mask[0] = False                                   # inlet plane (flow +X) is Dirichlet
    src = torch.zeros((nx, ny, nz), device=dev)
    src[:, :, 0] = flux                               # heat flux into the bottom layer of the base plate
    src[~sim.solid] = 0.0
    b = (mask.float() * dt * src).contiguous()
    mg = NLevelGeometricMGSolver(dev, torch.float32, 0, +1, 1.0, omega=0.6, n_pre=2, n_post=2, n_coarse=20,
                                 max_levels=max_levels, coarse_solve=coarse_solve)
    vel = []
    for t in (u, v, w):
        if not bool(torch.isfinite(t).all()):
            raise ValueError("thermal_system: the velocity field is not finite (did the lattice run diverge?)")
        t = t.to(device=dev, dtype=torch.float32).clone()
        t[sim.solid_flow] = 0.0
        vel.append(t)
    mg.build_if_needed(sim.k, sim.rho_cp, *vel, mask, dt)
    return mg, b


def build_system(dev, nx=256, ny=128, nz=128, lbm_steps=3000, dt=1000.0, flux=5e-3, k_ratio=200.0):
    """Velocity from `lbm_steps` steps of the FP16 lattice with MRT-Smagorinsky (plain MRT at Re = 200
    on this pin fin diverges after about 600 steps), then the thermal system on it."""
    from . import case as cases
    from .solver.lbm_cuda_ext import LBMCUDAUpgrade
    sim = cases.pin_fin(device=dev, nx=nx, ny=ny, nz=nz, storage="fp16", collision="mrt_smag", k_ratio=k_ratio)
    LBMCUDAUpgrade.patch(sim)
    for _ in range(lbm_steps):
        sim.step(do_thermal=False)
    torch.cuda.synchronize()
    mg, b = thermal_system(sim, sim.u, sim.v, sim.wv, dt, flux)
    return sim, mg, b


def time_solver(fn, repeats=5):
    times, info = [], None
    for _ in range(repeats):
        torch.cuda.synchronize()
        t = time.perf_counter()
        x, info = fn()
        torch.cuda.synchronize()
        times.append((time.perf_counter() - t) * 1e3)
    return statistics.median(times), info


def run(dev, repeats=5):
    from .solver import mg_pcg
    sim, mg, b = build_system(dev)
    out = {"workload": "pin-fin 256x128x128 thermal, A = I + dt L, dt = 1000, 5-level MG", "tol": 1e-8}
    # warm-up
    mg_pcg.bicgstab_mg_f64(mg, b, tol=1e-8, max_it=300)
    ms, info = time_solver(lambda: mg_pcg.bicgstab_mg_f64(mg, b, tol=1e-8, max_it=300), repeats)
    out["plain_bicgstab_ms"] = round(ms, 3)
    out["plain_bicgstab_it"] = info["it"]
    out["plain_bicgstab_res"] = info["res_rel"]
    mg_pcg.bicgstab_mg_mixed(mg, b, tol=1e-8, max_it=300)
    ms, info = time_solver(lambda: mg_pcg.bicgstab_mg_mixed(mg, b, tol=1e-8, max_it=300), repeats)
    out["mixed_bicgstab_ms"] = round(ms, 3)
    out["mixed_bicgstab_it"] = info["it"]
    out["mixed_bicgstab_outer"] = info["outer"]
    out["mixed_bicgstab_res"] = info["res_rel"]
    ms, info = time_solver(lambda: mg_pcg.fgmres_mg_f64(mg, b, tol=1e-8, max_it=300, restart=30), repeats)
    out["plain_fgmres_ms"] = round(ms, 3)
    out["plain_fgmres_it"] = info["it"]
    out["plain_fgmres_res"] = info["res_rel"]
    # V-cycle cost alone (the preconditioner application)
    lv0 = mg._levels[0]
    lv0["b_buf"].copy_(b)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(20):
        mg._vcycle(0, zero_guess=True)
    e1.record()
    torch.cuda.synchronize()
    out["vcycle_ms"] = round(e0.elapsed_time(e1) / 20, 4)
    return out
