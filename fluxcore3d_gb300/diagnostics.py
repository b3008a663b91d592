"""FP64 conservation diagnostics on the device.

`lbm_mass(sim)`: the mass of the fused lattice state, sum over fluid cells of
sum_q f_q, decoded from the storage format and accumulated in FP64
(fc_lbm_mass).  `heat_balance(mg, T, src, dt)`: the heat budget of the thermal
pseudo-time step A T = b (A = I + dt L, b = dt src on the non-Dirichlet cells)
in FP64 (fc_mg_heat_balance): heat generated (sum src), heat leaving through
the boundaries (sum L(T), which telescopes to the boundary fluxes), heat stored
(sum T / dt), and the relative imbalance.  The reference tracks neither in FP64.
"""
from __future__ import annotations

import torch

from . import _lib
from ._torch import ptr, stream_ptr


def lbm_mass(sim) -> float:
    fc = sim._fc
    if not fc.primed:
        fc._prime()
    ws = torch.empty(int(_lib.lib().fc_lbm_mass_workspace_bytes()), dtype=torch.uint8, device=sim.device)
    out = torch.zeros(1, dtype=torch.float64, device=sim.device)
    _lib.call("fc_lbm_mass", ptr(fc.P[fc.cur]), int(fc.storage), ptr(fc.flags), fc.N, ptr(ws), ws.numel(), ptr(out),
              stream_ptr())
    return float(out.item())


def heat_balance(mg, T: torch.Tensor, src: torch.Tensor, dt: float) -> dict:
    lv = mg._levels[0]
    nx, ny, nz = lv["shape"]
    n = nx * ny * nz
    T32 = T.reshape(lv["shape"]).to(torch.float32).contiguous()
    s32 = src.reshape(lv["shape"]).to(device=T32.device, dtype=torch.float32).contiguous()
    ws = torch.empty(int(_lib.call("fc_mg_heat_balance_workspace_bytes", n)), dtype=torch.uint8, device=T32.device)
    out = torch.zeros(3, dtype=torch.float64, device=T32.device)
    _lib.call("fc_mg_heat_balance", ptr(T32), ptr(s32), ptr(lv["mask_f"]), *mg._cptrs(lv), nx, ny, nz, mg.ax,
              lv["out_idx"], ptr(ws), ws.numel(), ptr(out), stream_ptr())
    q_src, q_out, t_sum = (float(v) for v in out.cpu())
    q_store = t_sum / float(dt)
    return {"heat_generated": q_src, "heat_out_through_boundaries": q_out, "heat_stored": q_store,
            "imbalance_rel": abs(q_src - q_out - q_store) / max(abs(q_src), 1e-300)}


def wall_heat(T, k, solid, D):
    """Host-side post-processing of a solved temperature field (numpy arrays T, k, solid): heat flow through the solid/fluid faces (harmonic-mean conductance times the temperature
    jump, summed over the 6-neighbour faces), the face count, and the Nusselt number
    Nu = (Q / A) * D / (k_f * mean wall temperature rise over the inlet)."""
    import numpy as np
    q, n, tw = 0.0, 0, 0.0
    for ax in range(3):
        a = [slice(None)] * 3
        b = [slice(None)] * 3
        a[ax] = slice(0, -1)
        b[ax] = slice(1, None)
        sa, sb = solid[tuple(a)], solid[tuple(b)]
        face = sa != sb
        ka, kb = k[tuple(a)], k[tuple(b)]
        kh = 2.0 * ka * kb / (ka + kb)
        Ta, Tb = T[tuple(a)], T[tuple(b)]
        ts = np.where(sa, Ta, Tb)
        tf = np.where(sa, Tb, Ta)
        q += float((kh * (ts - tf))[face].sum())
        n += int(face.sum())
        tw += float((0.5 * (ts + tf))[face].sum())
    k_f = float(k[~solid].min())
    tw /= max(n, 1)
    return q, n, (q / n) * D / (k_f * tw)
