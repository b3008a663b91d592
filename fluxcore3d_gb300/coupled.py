"""Coupled conjugate-heat-transfer run: the fused lattice engine advances the flow, and every
`thermal_every` lattice steps the fused pseudo-time thermal step (the drop-in
_temperature_step_mg) advances the temperature on the current velocity.

The reference keeps flow and heat apart (run_flow_to_steady_v2, then solve_thermal_steady_only,
LBM_CHT.py:2388-2569 with the step of :2571-2712); this driver interleaves the same two
operations.  Each thermal step:
  - rebuilds the multigrid operator from the velocity the lattice exposes (the pre-collision
    macros of the previous state, written every `thermal_every` steps by the fused engine);
  - solves A theta = rhs (A = I + dt L) to an FP64-certified relative residual `tol`, with
    FP64 BiCGSTAB around the FP32 V-cycle, or, when a learned preconditioner network is given,
    with FGMRES preconditioned by one V-cycle plus the network (LearnedCorrection) and the plain
    V-cycle taking over when an inner cycle stalls; a solve that does not converge is finished by
    the plain BiCGSTAB (the fallback, recorded);
  - records the FP64 heat balance of the discrete step over the non-Dirichlet cells:
    heat generated = sum src, outflow = sum L(T0 + theta), stored = sum (theta - theta_old) / dt,
    and the relative imbalance |generated - outflow - stored| / generated.
"""
from __future__ import annotations

import time
import types
from typing import Optional

import torch

from .diagnostics import heat_balance
from .solver import mg_pcg
from .solver.lbm_cuda_ext import LBMCUDAUpgrade
from .solver.nlevel_mg_cuda import NLevelGeometricMGSolver
from .solver.thermal_cuda_ext import patch_thermal_fused


class CoupledCHT:
    def __init__(self, sim, thermal_every: int = 20, dt_thermal: float = 200.0, tol: float = 1e-8,
                 max_it: int = 300, learned_net=None, max_levels: Optional[int] = None, fgmres_restart: int = 20):
        if thermal_every < 2:
            raise ValueError("thermal_every must be at least 2")
        self.sim = sim
        self.every = int(thermal_every)
        self.dt = float(dt_thermal)
        self.tol = float(tol)
        self.max_it = int(max_it)
        self.net = learned_net
        self.restart = int(fgmres_restart)
        sim.cfg.macro_stride = self.every
        if not hasattr(sim, "_fc"):
            LBMCUDAUpgrade.patch(sim)
        patch_thermal_fused(sim)
        cfg = sim.cfg
        sim._mg_solver = NLevelGeometricMGSolver(
            device=sim.device, dtype=torch.float32, flow_axis=sim.ax, flow_sign=sim.sign,
            thermal_dt_scale=float(sim.thermal_dt_scale), omega=float(getattr(cfg, "mg_omega", 0.6)),
            n_pre=int(getattr(cfg, "mg_pre_smooth", 2)), n_post=int(getattr(cfg, "mg_post_smooth", 2)),
            n_coarse=int(getattr(cfg, "mg_coarse_iters", 20)), min_coarse_cells=4, max_levels=max_levels)
        sim._mg_solver.solve = types.MethodType(self._solve, sim._mg_solver)
        self.k = 0
        self.history = []
        self.lattice_ms = 0.0

    # bound as the multigrid solver's solve(b, x0, max_cycles, tol) inside the fused thermal step
    def _solve(self, mg, b, x0=None, max_cycles=0, tol=0.0):
        sim = self.sim
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fell_back = False
        if self.net is not None:
            from .learned import LearnedCorrection
            pc = LearnedCorrection(self.net, mg, sim.k)
            x, info = mg_pcg.fgmres_mg_f64(mg, b, x0, tol=self.tol, max_it=self.max_it, restart=self.restart,
                                           precond=pc, stall_fallback=mg_pcg._vcycle_pc(mg))
            fell_back = bool(info.get("fell_back", False))
            if not info["converged"]:
                x, info = mg_pcg.bicgstab_mg_f64(mg, b, x, tol=self.tol, max_it=self.max_it)
                fell_back = True
        else:
            x, info = mg_pcg.bicgstab_mg_f64(mg, b, x0, tol=self.tol, max_it=self.max_it)
        torch.cuda.synchronize()
        ms = (time.perf_counter() - t0) * 1e3
        theta = x.to(torch.float32).reshape(b.shape)
        cs = sim._cached_thermal_setup
        src = cs["src_vol"]
        hb = heat_balance(mg, cs["T0"] + theta, src, self.dt)
        x_old = x0 if x0 is not None else torch.zeros_like(theta)
        stored = heat_balance(mg, theta - x_old.reshape(b.shape), src, self.dt)["heat_stored"]
        gen, out = hb["heat_generated"], hb["heat_out_through_boundaries"]
        self.history.append({"step": self.k, "it": int(info["it"]), "res_rel": float(info["res_rel"]),
                             "converged": bool(info["converged"]), "solve_ms": round(ms, 3),
                             "learned_fell_back": fell_back if self.net is not None else None,
                             "heat_generated": gen, "heat_out": out, "heat_stored": stored,
                             "imbalance_rel": abs(gen - out - stored) / max(abs(gen), 1e-300)})
        return theta, {"converged": bool(info["converged"]), "it": int(info["it"]), "res_rel": float(info["res_rel"]),
                       "diverged": False}

    def thermal_step(self) -> dict:
        sim = self.sim
        sim._mg_solver._ready = False          # the velocity changed: rebuild the operator
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = sim._temperature_step_mg(self.dt, tol=self.tol, max_cycles=self.max_it)
        torch.cuda.synchronize()
        self.history[-1]["thermal_step_ms"] = round((time.perf_counter() - t0) * 1e3, 3)
        self.history[-1]["Tmax"] = out.get("Tmax")
        return out

    def run(self, n_steps: int) -> list:
        """Advance n_steps lattice steps; a thermal step follows every lattice step k with
        (k - 1) % thermal_every == 0, k > 1 (where the engine exposes fresh macros).  The lattice
        steps between thermal steps are timed as blocks with CUDA events (lattice_ms)."""
        sim = self.sim
        left = int(n_steps)
        while left > 0:
            # lattice steps up to the next thermal step (or the end)
            nxt = self.k + 1
            while not (nxt > 1 and (nxt - 1) % self.every == 0):
                nxt += 1
            n = min(left, nxt - self.k)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(n):
                sim.step(do_thermal=False)
            e1.record()
            torch.cuda.synchronize()
            self.lattice_ms += e0.elapsed_time(e1)
            self.k += n
            left -= n
            if self.k > 1 and (self.k - 1) % self.every == 0:
                self.thermal_step()
        if sim._fc.check_device_error():
            raise RuntimeError("coupled run: device error word set")
        return self.history
