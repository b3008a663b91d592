"""Coupled CHT benchmark at scale: the pin-fin / gyroid hybrid heat sink 768x384x384 (113 M cells),
MRT-Smagorinsky with Bouzidi links at FP16 shifted storage, inlet u = 0.06, Re = 500, k_s/k_f = 200,
a thermal pseudo-time step (dt = 200) every 20 lattice steps on the current velocity, each solved to
a 1e-8 FP64 residual, with the FP64 heat balance of every thermal step (fluxcore3d_gb300.coupled).

A bounded sample of the 20000-step run is timed: `steps` lattice steps after a warm-up block."""
from __future__ import annotations

import statistics
import time

import torch

SHAPE = (768, 384, 384)
WORKLOAD = ("pin-fin / gyroid hybrid 768x384x384 (pins r=5 on 16x16-cell pitch, gyroid L=64 t=0.3 infill, seed 2), "
            "MRT-Smagorinsky + Bouzidi IBB, FP16 shifted populations, u=0.06, Re=500, k_s/k_f=200, "
            "thermal step every 20 lattice steps")


def run(dev, steps=200, every=20, shape=SHAPE, storage="fp16"):
    from . import case as cases
    from .coupled import CoupledCHT
    t = time.perf_counter()
    sim = cases.hybrid(device=dev, storage=storage, nx=shape[0], ny=shape[1], nz=shape[2])
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t
    cp = CoupledCHT(sim, thermal_every=every, dt_thermal=200.0, tol=1e-8, max_it=300, max_levels=5)
    cp.run(every + 1)                    # warm-up: graphs, hierarchy, one thermal step
    h0, ms0 = len(cp.history), cp.lattice_ms
    t = time.perf_counter()
    cp.run(steps)
    wall = time.perf_counter() - t
    hist = cp.history[h0:]
    N = shape[0] * shape[1] * shape[2]
    lat_ms = cp.lattice_ms - ms0
    out = {"workload": WORKLOAD, "cells": N, "links": int(sim.ibb_data.n_links), "setup_s": round(setup_s, 2),
           "lattice_steps": steps, "thermal_steps": len(hist),
           "lattice_mlups": round(N * steps / lat_ms / 1e3, 1),
           "coupled_mlups": round(N * steps / wall / 1e6, 1),
           "thermal_solve_ms_median": round(statistics.median(h["solve_ms"] for h in hist), 2),
           "thermal_step_ms_median": round(statistics.median(h["thermal_step_ms"] for h in hist), 2),
           "thermal_it_median": statistics.median(h["it"] for h in hist),
           "all_converged": all(h["converged"] for h in hist),
           "heat_imbalance_rel_max": max(h["imbalance_rel"] for h in hist),
           "heat_last": {k: hist[-1][k] for k in ("heat_generated", "heat_out", "heat_stored")},
           "Tmax_last": hist[-1]["Tmax"], "levels": len(sim._mg_solver._levels)}
    del cp, sim
    torch.cuda.empty_cache()
    return out
