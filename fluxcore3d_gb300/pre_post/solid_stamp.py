"""Device stamp of voxelized bodies into the solver's solid mask and material fields.

`SolidStampUpgrade.patch(sim)` replaces LBMCHT3D_Torch.add_solid_body
(LBM_CHT.py:959-1023) on the solver object with the same arguments, checks and
printed line: the body's voxel npz (from STLVoxelizer / gpu_voxelize_mesh) is placed
with voxel (0, 0, 0) at `offset_ijk`, clamped to the domain, OR-ed into sim.solid,
and k / rho_cp are set to the body's lattice values where its voxels are solid -- one
kernel (fc_geom_stamp_body), which also returns the cells this body added, the
per-body mask SolidAssembly.stamp (pre_post/solid_assembly.py:164-184) records.
"""
from __future__ import annotations

import numpy as np
import torch

from .. import _lib
from .._torch import ptr, stream_ptr


def stamp_voxels(sim, vox: torch.Tensor, offset_ijk, k_lat: float, rho_cp_lat: float):
    """Stamp a uint8/bool voxel block on sim's device; returns (body mask bool (nx,ny,nz), cells stamped)."""
    nx, ny, nz = sim.nx, sim.ny, sim.nz
    if sim.solid.dtype != torch.bool or not sim.solid.is_contiguous():
        raise RuntimeError("sim.solid must be a contiguous bool tensor")
    for name in ("k", "rho_cp"):
        t = getattr(sim, name)
        if t.dtype != torch.float32 or not t.is_contiguous():
            raise RuntimeError(f"sim.{name} must be a contiguous float32 tensor")
    v = vox.to(device=sim.solid.device, dtype=torch.uint8).contiguous()
    gx, gy, gz = v.shape
    body = torch.zeros((nx, ny, nz), dtype=torch.uint8, device=sim.solid.device)
    count = torch.zeros(1, dtype=torch.int64, device=sim.solid.device)
    i0, j0, k0 = (int(x) for x in offset_ijk)
    _lib.call("fc_geom_stamp_body", ptr(v), gx, gy, gz, i0, j0, k0, nx, ny, nz, ptr(sim.solid.view(torch.uint8)),
              ptr(sim.k), ptr(sim.rho_cp), float(np.float32(k_lat)), float(np.float32(rho_cp_lat)), ptr(body),
              ptr(count), stream_ptr())
    return body.bool(), int(count.item())


class SolidStampUpgrade:
    @staticmethod
    def patch(sim):
        def add_solid_body(npz_path: str, offset_ijk: tuple, solid_props, name: str = "solid"):
            data = np.load(npz_path, allow_pickle=True)
            vox = data["voxel_solid"].astype(bool)
            pitch_mm = float(data["pitch_mm"])
            dx_mm = sim.dx_phys_m * 1000.0
            if abs(pitch_mm - dx_mm) / dx_mm > 0.01:
                raise ValueError(f"[{name}] STL pitch {pitch_mm:.4f} mm != LBM dx {dx_mm:.4f} mm. "
                                 f"Re-voxelize with pitch_mm={dx_mm:.4f}.")
            Gx, Gy, Gz = vox.shape
            i0, j0, k0 = (int(x) for x in offset_ijk)
            outside = (min(i0 + Gx, sim.nx) <= max(i0, 0) or min(j0 + Gy, sim.ny) <= max(j0, 0)
                       or min(k0 + Gz, sim.nz) <= max(k0, 0))
            if outside:
                print(f"[{name}] WARNING: body is entirely outside domain — skipped.")
                return
            rho_cp_lat = float(solid_props.rho_cp_J_m3K) / sim.rho_cp_ref_J_m3K
            k_lat = float(solid_props.k_W_mK) / sim.k_ref_W_mK
            _, n = stamp_voxels(sim, torch.from_numpy(vox), (i0, j0, k0), k_lat, rho_cp_lat)
            print(f"[{name}] stamped {n} cells  offset=({i0},{j0},{k0})  voxel_grid={Gx}×{Gy}×{Gz}  "
                  f"k={solid_props.k_W_mK} W/mK")
        sim.add_solid_body = add_solid_body
        return sim
