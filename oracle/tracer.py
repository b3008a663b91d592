"""CPU restatement of the passive tracer (pre_post/tracer_patch.py:55-82).

TEST INFRASTRUCTURE ONLY.  FP32 numpy, one rounding per operation: upwind
differences with periodic neighbours (np.roll), phi - ((u*ax + v*ay) + w*az),
clamp to [0, 1], times the FP32 dissipation, 0 in flow-solid cells.  Pinned by
tests/golden/tracer.npz, written by the reference's TracerField on the torch CPU path.
"""
from __future__ import annotations

import numpy as np

f32 = np.float32


def step(phi, u, v, w, solid_flow, diss=0.9995):
    phi = np.asarray(phi, dtype=np.float32)

    def adv(vel, ax):
        back = phi - np.roll(phi, 1, ax)
        fwd = np.roll(phi, -1, ax) - phi
        return np.where(vel >= 0, back, fwd)
    s = (u * adv(u, 0) + v * adv(v, 1)) + w * adv(w, 2)
    n = np.clip(phi - s, f32(0.0), f32(1.0)) * f32(diss)
    n[np.asarray(solid_flow, dtype=bool)] = f32(0.0)
    return n.astype(np.float32)


def inject(phi, inlet_mask):
    phi = phi.copy()
    phi[np.asarray(inlet_mask, dtype=bool)] = f32(1.0)
    return phi
