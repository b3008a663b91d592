"""FP64 run of the plain method on the device.

`Lattice64(sim)` advances the reference's CUDA-path step sequence
(solver/lbm_cuda_ext.py:445-517: collide writing the pre-collision macros,
sponge on the post-collision populations, pull stream, interpolated
bounce-back and reset of the flow-solid cells, plane boundary conditions in the
reference face order) with double populations and macros, through the
library's fc_lbm64_* kernels.  It starts from the solver object's initial
state (sim.f, before any step) and reads the same geometry, rates, sponge
profile and link data, so the FP32 and FP16/BF16 runs of the fused engine can
report their error against it (velocity, and through the thermal solve
temperature, wall heat flow and Nusselt number).

It is a measurement device, not a solver for production runs: every step is
the six to nine per-operation launches of the reference sequence.
"""
from __future__ import annotations

import torch

from . import _lib
from ._torch import ptr, stream_ptr
from .solver.face_roles import periodic_flags
from .solver.lbm_cuda_ext import _bc_plan, _prepare_ibb_tensors

_COLLISION = {"bgk": 0, "trt": 1, "mrt": 2, "mrt_smag": 3}
_C = ((0, 0, 0), (1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1), (1, 1, 0), (1, -1, 0),
      (-1, 1, 0), (-1, -1, 0), (1, 0, 1), (1, 0, -1), (-1, 0, 1), (-1, 0, -1), (0, 1, 1), (0, 1, -1), (0, -1, 1),
      (0, -1, -1))


class Lattice64:
    def __init__(self, sim, f0: torch.Tensor | None = None):
        cfg = sim.cfg
        dev = sim.device
        self.nx, self.ny, self.nz = sim.nx, sim.ny, sim.nz
        self.N = N = sim.nx * sim.ny * sim.nz
        self.mode = str(getattr(cfg, "collision", "bgk")).lower()
        if self.mode not in _COLLISION:
            raise ValueError(f"collision {self.mode!r} has no FP64 kernel")
        ibb = getattr(sim, "ibb_data", None)
        if ibb is None or int(ibb.n_links) == 0:
            raise ValueError("Lattice64 runs the interpolated bounce-back path: the case needs link data")
        src = sim.f if f0 is None else f0
        self.f = src.reshape(19, N).to(device=dev, dtype=torch.float64).contiguous().clone()
        self.fp = torch.empty_like(self.f)
        self.rho = torch.ones(N, dtype=torch.float64, device=dev)
        self.u = torch.zeros(N, dtype=torch.float64, device=dev)
        self.v = torch.zeros_like(self.u)
        self.w = torch.zeros_like(self.u)
        self.solid = sim.solid_flow.reshape(N).to(device=dev, dtype=torch.uint8).contiguous()
        self.omega = float(sim.omega_plus)
        self.omega_minus = float(getattr(sim, "omega_minus", sim.omega_plus))
        self.S = (sim._mrt_S.to(device=dev, dtype=torch.float32).contiguous()
                  if self.mode in ("mrt", "mrt_smag") else None)
        self.Cs_dx2 = float(getattr(cfg, "smag_Cs", 0.1)) ** 2
        self.sigma = (sim._sponge_sigma.reshape(N).to(device=dev, dtype=torch.float32).contiguous()
                      if int(getattr(cfg, "sponge_length", 0)) > 0 and hasattr(sim, "_sponge_sigma") else None)
        self.periodic = tuple(int(p) for p in periodic_flags(cfg))
        self.links = _prepare_ibb_tensors(ibb, dev, torch.float32)
        self.n_links = int(self.links.fluid_flat.numel())
        self.plan = _bc_plan(sim)
        self.err = torch.zeros(1, dtype=torch.int32, device=dev)
        self.ws = {}
        self.steps = 0

    def _ws(self, n1, n2):
        need = int(_lib.call("fc_lbm_convective_workspace_bytes", int(n1), int(n2)))
        w = self.ws.get((n1, n2))
        if w is None:
            w = torch.empty(need, dtype=torch.uint8, device=self.f.device)
            self.ws[(n1, n2)] = w
        return w

    def step(self, n: int = 1) -> None:
        st = stream_ptr()
        N = self.N
        t = self.links
        for _ in range(int(n)):
            _lib.call("fc_lbm64_macro_collide", _COLLISION[self.mode], ptr(self.f), ptr(self.fp), ptr(self.rho),
                      ptr(self.u), ptr(self.v), ptr(self.w), ptr(self.solid), self.omega, self.omega,
                      self.omega_minus, ptr(self.S), self.Cs_dx2, self.omega, N, st)
            if self.sigma is not None:
                _lib.call("fc_lbm64_sponge", ptr(self.fp), ptr(self.rho), ptr(self.u), ptr(self.v), ptr(self.w),
                          ptr(self.sigma), N, st)
            _lib.call("fc_lbm64_stream_pull", ptr(self.fp), ptr(self.f), self.nx, self.ny, self.nz, *self.periodic,
                      st)
            _lib.call("fc_lbm64_ibb", ptr(self.fp), ptr(self.f), ptr(t.fluid_flat), ptr(t.dir_i), ptr(t.dir_opp),
                      ptr(t.w_i), ptr(t.w_second), ptr(t.q_ge_half), ptr(t.ff_flat), ptr(t.ff_valid),
                      self.n_links, N, ptr(self.err), st)
            _lib.call("fc_lbm64_reset_solid", ptr(self.f), ptr(self.solid), N, st)
            for kind, ax, pidx, iidx, code, u_signed, rho_out, sign, n1, n2 in self.plan:
                if kind == "zou_he":
                    _lib.call("fc_lbm64_zou_he_bc", ptr(self.f), ptr(self.solid), self.nx, self.ny, self.nz, ax,
                              pidx, iidx, code, float(u_signed), float(rho_out), sign, st)
                else:
                    ws = self._ws(n1, n2)
                    _lib.call("fc_lbm64_convective_bc", ptr(self.f), ptr(self.solid), self.nx, self.ny, self.nz,
                              ax, pidx, iidx, code, float(rho_out), n1, n2, ptr(ws), ws.numel(), st)
            self.steps += 1

    def check(self) -> None:
        e = int(self.err.item())
        if e:
            raise RuntimeError(f"Lattice64: device error word {e:#x} (link index out of range)")

    def velocity(self) -> torch.Tensor:
        """(3, N) FP64 velocity of the current post-stream populations (zero where rho is zero)."""
        rho = self.f.sum(0)
        c = torch.tensor(_C, dtype=torch.float64, device=self.f.device)
        j = c.t() @ self.f
        return j / rho
