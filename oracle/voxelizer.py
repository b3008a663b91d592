"""CPU restatement of the reference's ray-parity STL voxelizer and body stamp.

TEST INFRASTRUCTURE ONLY: the oracle the device kernels are compared with.

  grid                gpu_voxelize_mesh's grid (pre_post/gpu_voxelizer.py:103-110):
                      origin = min corner - pitch/2 (FP32), n = ceil(extent/pitch) + 2
  voxelize            the parity count of gpu_voxelize_mesh (:112-165) and
                      _mt_intersect_z (:39-70): +z rays from FP64 origins
                      (+1.3e-5 pitch * (sqrt 2, sqrt 3)) cast to FP32, Moller-Trumbore
                      in FP32 numpy (one rounding per operation), a cell solid when an
                      odd number of hits lies below its FP32 centre
  stamp               LBMCHT3D_Torch.add_solid_body's stamp (LBM_CHT.py:959-1023)

Pinned by tests/golden/voxels.npz, written by the reference's own gpu_voxelize_mesh
(torch CPU path) on three closed meshes.
"""
from __future__ import annotations

import numpy as np

f32 = np.float32


def grid(verts: np.ndarray, pitch: float):
    v = np.asarray(verts, dtype=np.float32)
    lo, hi = v.min(0), v.max(0)
    origin = lo - f32(pitch * 0.5)
    dims = tuple(int(np.ceil(f32(hi[a] - origin[a]) / f32(pitch))) + 2 for a in range(3))
    return origin.astype(np.float32), dims


def voxelize(tri: np.ndarray, origin, dims, pitch: float, ray_chunk: int = 0, ray_ids=None) -> np.ndarray:
    """uint8 (nx, ny, nz) parity grid of FP32 triangles (T, 3, 3); with ray_ids (flat i*ny + j),
    only those columns, as (len(ray_ids), nz)."""
    tri = np.asarray(tri, dtype=np.float32)
    nx, ny, nz = dims
    ray_chunk = ray_chunk or max(1, (1 << 21) // max(1, tri.shape[0]))
    o = np.asarray(origin, dtype=np.float32)
    z0 = float(o[2])
    zc = (z0 + (np.arange(nz) + 0.5) * pitch).astype(np.float32)
    pert = 1.3e-5 * pitch
    gx, gy = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    ox = (np.float64(o[0]) + gx.ravel() * pitch + pert * np.sqrt(2)).astype(np.float32)
    oy = (np.float64(o[1]) + gy.ravel() * pitch + pert * np.sqrt(3)).astype(np.float32)
    if ray_ids is not None:
        ox, oy = ox[ray_ids], oy[ray_ids]
    nr = ox.size
    v0, v1, v2 = tri[:, 0], tri[:, 1], tri[:, 2]
    e1 = v1 - v0
    e2 = v2 - v0
    hx = -e2[:, 1]
    hy = e2[:, 0]
    det = e1[:, 0] * hx + e1[:, 1] * hy
    valid = np.abs(det) > f32(1e-7)
    with np.errstate(divide="ignore"):
        inv = np.where(valid, f32(1.0) / np.where(valid, det, f32(1.0)), f32(0.0)).astype(np.float32)
    szt = f32(z0) - v0[:, 2]
    a_y = szt * e1[:, 1]
    a_x = szt * e1[:, 0]
    out = np.zeros((nr, nz), dtype=np.uint8)
    for r0 in range(0, nr, ray_chunk):
        sx = ox[r0:r0 + ray_chunk, None] - v0[None, :, 0]
        sy = oy[r0:r0 + ray_chunk, None] - v0[None, :, 1]
        u = (sx * hx + sy * hy) * inv
        qz = sx * e1[:, 1] - sy * e1[:, 0]
        v = qz * inv
        qx = sy * e1[:, 2] - a_y
        qy = a_x - sx * e1[:, 2]
        t = (e2[:, 0] * qx + e2[:, 1] * qy + e2[:, 2] * qz) * inv
        hit = valid & (u >= 0) & (u <= 1) & (v >= 0) & (u + v <= 1) & (t >= 0)
        hz = f32(z0) + t
        rows, cols = np.nonzero(hit)
        flips = np.zeros((sx.shape[0], nz + 1), dtype=np.uint8)
        k = np.searchsorted(zc, hz[rows, cols], side="right")
        np.bitwise_xor.at(flips, (rows, k), 1)
        out[r0:r0 + sx.shape[0]] = np.bitwise_xor.accumulate(flips[:, :nz], axis=1)
    return out if ray_ids is not None else out.reshape(nx, ny, nz)


def stamp(solid: np.ndarray, k: np.ndarray, rho_cp: np.ndarray, vox: np.ndarray, offset, k_val, rho_cp_val):
    """In place; returns the body mask (cells this body added)."""
    nx, ny, nz = solid.shape
    gx, gy, gz = vox.shape
    i0, j0, k0 = (int(x) for x in offset)
    d0 = (max(i0, 0), max(j0, 0), max(k0, 0))
    d1 = (min(i0 + gx, nx), min(j0 + gy, ny), min(k0 + gz, nz))
    body = np.zeros_like(solid, dtype=bool)
    if any(d1[a] <= d0[a] for a in range(3)):
        return body
    sl = tuple(slice(d0[a], d1[a]) for a in range(3))
    src = tuple(slice(d0[a] - o, d1[a] - o) for a, o in enumerate((i0, j0, k0)))
    patch = vox[src].astype(bool)
    before = solid.copy()
    solid[sl] |= patch
    k[sl][patch] = f32(k_val)
    rho_cp[sl][patch] = f32(rho_cp_val)
    body = solid & ~before
    return body
