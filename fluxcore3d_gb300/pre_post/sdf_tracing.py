"""Drop-in for the reference's pre_post/sdf_tracing.py voxel path, on the device.

Same names, arguments and results as sdf_tracing.py:
  IBBData                        :9-18
  build_links_from_mask_gpu      :20-85   (link order included)
  bfl_weights_from_q             :188-205
  build_ibb_from_sdf_gpu         :208-259 (sets sim.ibb_data, prints the same summary line)
  build_phi_from_voxel_mask_mm   :312-340 (scipy's host EDT replaced by the device transform;
                                           the FP32 phi is the same bit for bit)
The STL path (build_phi_from_stl_mm, :262-308) needs trimesh and is not provided.
Everything runs on a CUDA device; without one the functions raise.
"""
from __future__ import annotations

import numpy as np
import torch

from .. import geometry as _geo
from ..geometry import IBBData  # noqa: F401  (re-exported under the reference's name)


def _check_lattice(c_np, opp_np) -> None:
    if not (np.array_equal(np.asarray(c_np), _geo.C_NP) and np.array_equal(np.asarray(opp_np), _geo.OPP_NP)):
        raise ValueError("c_np / opp_np must be the D3Q19 set of the solver (LBMCHT3D_Torch.c_np / opp_np)")


def build_links_from_mask_gpu(solid_geom: torch.Tensor, c_np, opp_np):
    _check_lattice(c_np, opp_np)
    return _geo.build_links(solid_geom)


def bfl_weights_from_q(q: torch.Tensor):
    return _geo.bfl_weights_from_q(q)


def build_phi_from_voxel_mask_mm(voxel_solid, pitch_mm: float, device="cuda", dtype=torch.float32):
    print("[SDF] Building SDF from voxel mask (distance transform)...")
    solid = torch.as_tensor(np.asarray(voxel_solid).astype(bool), device=device)
    phi = _geo.signed_distance(solid, float(pitch_mm))
    print("[SDF] Done.")
    print(f"[SDF] phi range: min={float(phi.min()):.6f}, max={float(phi.max()):.6f}")
    return phi.to(dtype)


def build_ibb_from_sdf_gpu(sim, voxel_origin_mm, pitch_mm, offset_ijk, c_np, opp_np):
    _check_lattice(c_np, opp_np)
    origin = (torch.tensor(voxel_origin_mm, dtype=torch.float32)
              - float(pitch_mm) * torch.tensor(offset_ijk, dtype=torch.float32))
    ibb, q = _geo.ibb_from_phi(sim.solid, sim.phi, float(pitch_mm), tuple(origin.tolist()), return_q=True)
    sim.ibb_data = ibb
    with torch.no_grad():
        qv = q[torch.isfinite(q)]
        if qv.numel():
            print(f"[SDF-IBB] links={ibb.n_links} q[min,med,max]=({float(qv.min()):.4f},{float(qv.median()):.4f},"
                  f"{float(qv.max()):.4f}) q<0.5={int((q < 0.5).sum())}")
