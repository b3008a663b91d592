"""Drop-in for the reference's pre_post/gpu_voxelizer.py, on the library's kernels.

  gpu_voxelize_mesh(mesh, pitch_mm, ...)   gpu_voxelizer.py:81-170
  patch_stl_voxelizer(cls, method="gpu")   :210-256
  unpatch_stl_voxelizer(cls)               :266-269

`mesh` is anything with `vertices` (V, 3) and `faces` (T, 3) -- a trimesh object, or
`stl.MeshData` from `stl.read_stl` when trimesh is not installed.  The grid (origin
half a pitch below the mesh's lower corner, two cells of margin) and the ray set
(+z rays through the (i, j) cell corners shifted by 1.3e-5 pitch times (sqrt 2,
sqrt 3)) are the reference's; the parity count runs in two kernels
(fc_vox_prepare_triangles, fc_vox_parity_z) over all triangles at once, with the
same FP32 rounding, so the returned voxel grid is the reference's bit for bit.

Mesh repair (trimesh.repair on a mesh that is not watertight) runs only when trimesh
is importable; the PyVista fallback is not provided.
"""
from __future__ import annotations

from datetime import datetime

import numpy as np
import torch

from .. import _lib
from .._torch import ptr, stream_ptr


def _log(msg):
    print(f"[ {datetime.now().strftime('%I:%M:%S %p')} ] [GPUVox] {msg}")


def _repair_mesh(mesh, verbose=True):
    if getattr(mesh, "is_watertight", True):
        return mesh
    try:
        import trimesh
    except ImportError:
        if verbose:
            _log("WARNING: mesh is not watertight and trimesh is unavailable; voxelizing it as is")
        return mesh
    trimesh.repair.fix_normals(mesh)
    trimesh.repair.fill_holes(mesh)
    trimesh.repair.fix_winding(mesh)
    if not mesh.is_watertight:
        _log("WARNING: repair failed, using convex hull approximation")
        mesh = mesh.convex_hull
    return mesh


def voxel_grid(verts: np.ndarray, pitch_mm: float):
    """(origin FP32 (3,), nx, ny, nz) of the voxel grid around FP32 vertices: origin half a pitch
    below the lower corner, size ceil(extent / pitch) + 2 per axis, in FP32 numpy arithmetic."""
    bmin = verts.min(0)
    bmax = verts.max(0)
    origin = bmin - pitch_mm * 0.5
    dims = [int(np.ceil((bmax[a] - origin[a]) / pitch_mm)) + 2 for a in range(3)]
    return origin, dims[0], dims[1], dims[2]


def ray_perturbation(pitch_mm: float):
    """Offsets of the ray origins from the cell corners (keeps rays off shared triangle edges)."""
    p = 1.3e-5 * pitch_mm
    return p * np.sqrt(2), p * np.sqrt(3)


def voxelize_triangles(tri: torch.Tensor, origin, dims, pitch_mm: float) -> torch.Tensor:
    """Parity voxelization of FP32 triangles (T, 3, 3) on their CUDA device -> uint8 (nx, ny, nz)."""
    if not tri.is_cuda:
        raise RuntimeError("voxelization runs on a CUDA device")
    nx, ny, nz = dims
    tri = tri.contiguous().to(torch.float32).reshape(-1, 9)
    T = tri.shape[0]
    L = _lib.lib()
    prep = torch.empty(max(1, int(L.fc_vox_prepared_floats(T))), dtype=torch.float32, device=tri.device)
    out = torch.empty((nx, ny, nz), dtype=torch.uint8, device=tri.device)
    st = stream_ptr()
    z0 = float(np.float32(origin[2]))
    _lib.call("fc_vox_prepare_triangles", ptr(tri), T, z0, ptr(prep), st)
    px, py = ray_perturbation(pitch_mm)
    _lib.call("fc_vox_parity_z", ptr(prep), T, nx, ny, nz, float(origin[0]), float(origin[1]), z0,
              float(pitch_mm), float(px), float(py), ptr(out), st)
    return out


def gpu_voxelize_mesh(mesh, pitch_mm: float, device: str = "cuda", ray_chunk: int = 2048, tri_chunk: int = 32768,
                      t_inner: int = 512, verbose: bool = False):
    """(voxel_solid uint8 (nx, ny, nz), voxel_origin_mm float64 (3,)); the chunk sizes of the
    reference are accepted and unused (one launch covers every ray and triangle)."""
    if device != "cuda" or not torch.cuda.is_available():
        raise RuntimeError("gpu_voxelize_mesh runs on a CUDA device")
    mesh = _repair_mesh(mesh, verbose=verbose)
    verts = np.array(mesh.vertices, dtype=np.float32)
    faces = np.array(mesh.faces, dtype=np.int64)
    if verbose:
        _log(f"Mesh: {len(verts)} verts, {faces.shape[0]} triangles | pitch={pitch_mm} mm")
    origin, nx, ny, nz = voxel_grid(verts, pitch_mm)
    if verbose:
        _log(f"Grid: {nx}x{ny}x{nz} = {nx * ny * nz / 1e6:.2f} M cells")
    tri = torch.from_numpy(verts[faces]).to("cuda")
    vox = voxelize_triangles(tri, origin, (nx, ny, nz), pitch_mm).cpu().numpy()
    if verbose:
        _log(f"Done.  Solid: {int(vox.sum()):,}  ({vox.mean() * 100:.1f}% fill)")
    return vox, origin.astype(np.float64)


def patch_stl_voxelizer(cls, method: str = "gpu", device: str = "cuda", ray_chunk: int = 2048):
    """Replace STLVoxelizer._voxelize with the device voxelizer (method "gpu" only)."""
    if method != "gpu":
        raise NotImplementedError("only the GPU voxelizer is provided (PyVista is not installed)")

    def _vox(self):
        v, o = gpu_voxelize_mesh(self.mesh, self.pitch_mm, device=device, ray_chunk=ray_chunk)
        self.voxel_origin_mm = o
        return v
    cls._voxelize = _vox
    return cls


def _original_voxelize(self) -> np.ndarray:
    """trimesh's own voxelizer (needs trimesh)."""
    vox = self.mesh.voxelized(pitch=self.pitch_mm).fill()
    self.voxel_origin_mm = vox.transform[:3, 3].copy()
    return vox.matrix.astype(np.uint8)


def unpatch_stl_voxelizer(cls):
    cls._voxelize = _original_voxelize
    return cls
