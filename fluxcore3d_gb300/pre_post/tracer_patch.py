"""Drop-in for the reference's pre_post/tracer_patch.py on the library's tracer kernel.

  TracerField(sim, flow_dir, inject_depth, dissipation)   tracer_patch.py:26-97
  attach_tracer(sim, flow_dir, inject_depth, dissipation) :100-124

Same fields, methods and printed lines.  `step()` is one launch of fc_tracer_step
(ping-pong buffers; `field` is rebound to the new one, as the reference rebinds it),
`inject()` one launch of fc_tracer_inject.  The tracer reads sim.u / sim.v / sim.wv
after every step, so attaching it makes the fused lattice engine write the macro
fields every step (macro stride 1), as the reference's step does.

On the fused lattice engine, attach_tracer(..., fuse=True) (the default) hands the
tracer to the engine: each sim.step() then advances it inside the lattice main pass,
reading the velocity the step exposes, instead of launching fc_tracer_step after the
step.  The field is the same bit for bit; tracer.step() on its own (warmup) still
launches the kernel.
"""
from __future__ import annotations

import types

import numpy as np
import torch

from .. import _lib
from .._torch import ptr, stream_ptr


class TracerField:
    def __init__(self, sim, flow_dir="-Z", inject_depth=6, dissipation=0.9995):
        self.sim = sim
        self.fd = flow_dir.strip().upper()
        self.diss = dissipation
        nx, ny, nz = sim.nx, sim.ny, sim.nz
        self.nx, self.ny, self.nz = nx, ny, nz
        self._buf = [torch.zeros(nx, ny, nz, device=sim.device, dtype=torch.float32) for _ in range(2)]
        self._cur = 0
        self.fluid = ~sim.solid_flow
        self._solid_u8 = sim.solid_flow.to(torch.uint8).contiguous()
        d = inject_depth
        m = torch.zeros(nx, ny, nz, dtype=torch.bool, device=sim.device)
        if self.fd == "+Z":
            m[:, :, :d] = True
        elif self.fd == "-Z":
            m[:, :, nz - d:] = True
        elif self.fd == "+Y":
            m[:, :d, :] = True
        elif self.fd == "-Y":
            m[:, ny - d:, :] = True
        elif self.fd == "+X":
            m[:d, :, :] = True
        elif self.fd == "-X":
            m[nx - d:, :, :] = True
        self._inlet = m & self.fluid
        self._inlet_u8 = self._inlet.to(torch.uint8).contiguous()
        print(f"[Tracer] flow_dir={flow_dir}  inject_depth={inject_depth}  "
              f"dissipation={dissipation}  inlet_voxels={int(self._inlet.sum()):,}")

    @property
    def field(self) -> torch.Tensor:
        return self._buf[self._cur]

    @field.setter
    def field(self, value: torch.Tensor):
        self._buf[self._cur].copy_(value)

    def inject(self):
        _lib.call("fc_tracer_inject", ptr(self.field), ptr(self._inlet_u8), self.field.numel(), stream_ptr())

    def step(self):
        sim = self.sim
        u, v, w = (t.contiguous() for t in (sim.u, sim.v, sim.wv))
        for t in (u, v, w):
            if t.dtype != torch.float32:
                raise RuntimeError("the tracer needs float32 velocity fields")
        src, dst = self._buf[self._cur], self._buf[1 - self._cur]
        _lib.call("fc_tracer_step", ptr(src), ptr(dst), ptr(u), ptr(v), ptr(w), ptr(self._solid_u8), self.nx,
                  self.ny, self.nz, float(np.float32(self.diss)), stream_ptr())
        self._cur = 1 - self._cur

    def warmup(self, n_steps=300):
        print(f"[Tracer] warming up {n_steps} steps to fill domain...")
        self.inject()
        for i in range(n_steps):
            if i % 30 == 0:
                self.inject()
            self.step()
        print(f"[Tracer] warmup done — max density: {float(self.field.max()):.4f}")

    def get(self):
        return self.field.detach().cpu().numpy().astype(np.float32)


def attach_tracer(sim, flow_dir="-Z", inject_depth=6, dissipation=0.9995, *, fuse=True):
    tracer = TracerField(sim, flow_dir=flow_dir, inject_depth=inject_depth, dissipation=dissipation)
    fc = getattr(sim, "_fc", None)
    if fc is not None:
        fc.macro_stride = 1
        if fuse:
            fc.tracer = tracer
    _lbm_step = sim.step

    def _step_with_tracer(self_, do_thermal=False):
        if fc is not None and fc.tracer is tracer:
            return _lbm_step(do_thermal=do_thermal)   # the lattice pass advanced the tracer
        result = _lbm_step(do_thermal=do_thermal)
        tracer.step()
        return result

    sim.step = types.MethodType(_step_with_tracer, sim)
    print("[Tracer] attached — tracer.step() runs after every sim.step()")
    return tracer
