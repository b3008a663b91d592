"""Triangle meshes without trimesh: STL reading / writing and a few closed test solids.

The reference loads meshes with trimesh (absent from this image); the voxelizer only
needs the triangle corners, so `read_stl` returns (vertices, faces) with one vertex
per triangle corner (binary or ASCII STL).  `MeshData` carries them with the
attributes gpu_voxelize_mesh reads from a trimesh object (`vertices`, `faces`,
`is_watertight`).

The generators build closed, consistently wound meshes for tests and benchmarks:
an axis-aligned box, an icosphere and a finned heat sink (base plate plus a row of
fins, each a separate closed box resting on the plate).
"""
from __future__ import annotations

import struct
from dataclasses import dataclass

import numpy as np


@dataclass
class MeshData:
    vertices: np.ndarray        # (V, 3) float
    faces: np.ndarray           # (T, 3) int
    is_watertight: bool = True

    @property
    def triangles(self) -> np.ndarray:
        return np.asarray(self.vertices, dtype=np.float32)[np.asarray(self.faces, dtype=np.int64)]


def read_stl(path: str) -> MeshData:
    """Binary or ASCII STL -> MeshData (three vertices per triangle, in file order)."""
    with open(path, "rb") as fh:
        data = fh.read()
    tri = None
    if len(data) >= 84:
        n = struct.unpack_from("<I", data, 80)[0]
        if 84 + 50 * n == len(data):
            rec = np.frombuffer(data, dtype=np.dtype([("n", "<f4", 3), ("v", "<f4", (3, 3)), ("a", "<u2")]),
                                count=n, offset=84)
            tri = np.array(rec["v"], dtype=np.float32)
    if tri is None:
        words = data.decode("ascii", errors="replace").split()
        pts = []
        for i, w in enumerate(words):
            if w == "vertex":
                pts.append((float(words[i + 1]), float(words[i + 2]), float(words[i + 3])))
        tri = np.array(pts, dtype=np.float32).reshape(-1, 3, 3)
    T = tri.shape[0]
    return MeshData(tri.reshape(-1, 3), np.arange(3 * T, dtype=np.int64).reshape(T, 3))


def write_stl(path: str, mesh: MeshData) -> None:
    """Binary STL (normals from the winding)."""
    tri = mesh.triangles.astype(np.float32)
    nrm = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    ln = np.linalg.norm(nrm, axis=1, keepdims=True)
    nrm = (nrm / np.where(ln > 0, ln, 1)).astype(np.float32)
    rec = np.zeros(tri.shape[0], dtype=np.dtype([("n", "<f4", 3), ("v", "<f4", (3, 3)), ("a", "<u2")]))
    rec["n"] = nrm
    rec["v"] = tri
    with open(path, "wb") as fh:
        fh.write(b"fluxcore3d_gb300".ljust(80, b" "))
        fh.write(struct.pack("<I", tri.shape[0]))
        fh.write(rec.tobytes())


def box_mesh(lo, hi) -> MeshData:
    """Closed axis-aligned box, outward winding."""
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    v = np.array([[x0, y0, z0], [x1, y0, z0], [x1, y1, z0], [x0, y1, z0],
                  [x0, y0, z1], [x1, y0, z1], [x1, y1, z1], [x0, y1, z1]], dtype=np.float64)
    f = np.array([[0, 2, 1], [0, 3, 2], [4, 5, 6], [4, 6, 7], [0, 1, 5], [0, 5, 4],
                  [1, 2, 6], [1, 6, 5], [2, 3, 7], [2, 7, 6], [3, 0, 4], [3, 4, 7]], dtype=np.int64)
    return MeshData(v, f)


def merge(*meshes: MeshData) -> MeshData:
    vs, fs, off = [], [], 0
    for m in meshes:
        vs.append(np.asarray(m.vertices, dtype=np.float64))
        fs.append(np.asarray(m.faces, dtype=np.int64) + off)
        off += len(m.vertices)
    return MeshData(np.concatenate(vs), np.concatenate(fs))


def icosphere_mesh(radius: float = 1.0, subdivisions: int = 2, center=(0.0, 0.0, 0.0)) -> MeshData:
    t = (1.0 + 5 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
         (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    verts = [np.array(p, dtype=np.float64) / np.linalg.norm(p) for p in v]
    faces = list(f)
    for _ in range(subdivisions):
        cache = {}

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]
        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    V = np.array(verts) * radius + np.asarray(center, dtype=np.float64)
    return MeshData(V, np.array(faces, dtype=np.int64))


def fin_heatsink_mesh(base=(40.0, 30.0, 3.0), n_fins=8, fin_t=1.5, fin_h=20.0, origin=(0.0, 0.0, 0.0)) -> MeshData:
    """Base plate plus n_fins plates along x, each a closed box resting on the base."""
    ox, oy, oz = origin
    bx, by, bz = base
    parts = [box_mesh((ox, oy, oz), (ox + bx, oy + by, oz + bz))]
    pitch = bx / n_fins
    for i in range(n_fins):
        x0 = ox + (i + 0.5) * pitch - fin_t / 2
        parts.append(box_mesh((x0, oy, oz + bz), (x0 + fin_t, oy + by, oz + bz + fin_h)))
    return merge(*parts)
