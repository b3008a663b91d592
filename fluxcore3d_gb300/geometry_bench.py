"""Geometry set-up benchmark: voxel SDF, boundary links and Bouzidi fractions on the device.

Workloads: the 384x192x192 gyroid heat sink (L = 48, t = 0.3) and the
768x384x384 pin + gyroid hybrid (113M cells).  Every timed call is preceded by an L2 flush (a
256 MB write) and bracketed by CUDA events on the current stream; medians of
five runs after three warm-ups.  Algorithmic bytes of the distance transform:
pass z reads the mask and writes one int32 (5 B/cell), passes y and x read the
int32 and the mask and write an int32 / the FP32 phi (9 B/cell each): 23 B per
cell.  The reference computes phi with scipy.ndimage.distance_transform_edt on
the host; that call is timed on the same mask as the CPU baseline.
"""
from __future__ import annotations

import statistics
import time

import torch

from . import geometry as geo

EDT_BYTES_PER_CELL = 23


def _timed(fn, flush, reps=5, warm=3):
    for _ in range(warm):
        fn()
    ts = []
    for _ in range(reps):
        flush.fill_(1.0)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record()
        fn()
        b.record()
        torch.cuda.synchronize()
        ts.append(a.elapsed_time(b))
    return statistics.median(ts)


def _measure(solid, flush):
    phi = geo.signed_distance(solid)
    edt_ms = _timed(lambda: geo.signed_distance(solid), flush)
    links = geo.build_links(solid)
    links_ms = _timed(lambda: geo.build_links(solid), flush)
    ibb_ms = _timed(lambda: geo.ibb_from_phi(solid, phi), flush)
    n = int(solid.numel())
    return phi, {"cells": n, "links": int(links[0].numel()), "solid_fraction": round(float(solid.float().mean()), 4),
                 "edt_ms": round(edt_ms, 3), "edt_achieved_gbs": round(n * EDT_BYTES_PER_CELL / (edt_ms / 1e3) / 1e9, 1),
                 "links_ms": round(links_ms, 3), "links_and_fractions_ms": round(ibb_ms, 3),
                 "q_ms": round(max(ibb_ms - links_ms, 0.0), 3)}


def voxelizer_run(dev, flush, cpu_voxelize=None):
    """Ray-parity voxelization of two closed meshes: a 20,480-triangle sphere (r = 10 mm, 0.05 mm
    pitch, 65M cells) and a finned heat sink (108 triangles, 0.06 mm pitch, 129M cells).  Device
    time of the prepare + parity kernels (median of 5, L2 flushed).  `cpu_voxelize(tri, origin,
    dims, pitch, ray_ids)`, when given, is timed on 2,000 columns of the sphere as the CPU
    baseline."""
    import numpy as np
    from .pre_post import gpu_voxelizer as gv
    from .pre_post import stl
    res = {}
    for name, mesh, pitch in (("sphere_20480_tri", stl.icosphere_mesh(10.0, 5), 0.05),
                              ("fin_sink_108_tri", stl.fin_heatsink_mesh(), 0.06)):
        verts = np.asarray(mesh.vertices, dtype=np.float32)
        origin, nx, ny, nz = gv.voxel_grid(verts, pitch)
        tri = torch.from_numpy(mesh.triangles).to(dev)
        ms = _timed(lambda: gv.voxelize_triangles(tri, origin, (nx, ny, nz), pitch), flush)
        pairs = nx * ny * tri.shape[0]
        r = {"cells": nx * ny * nz, "rays": nx * ny, "triangles": int(tri.shape[0]), "ms": round(ms, 3),
             "ray_triangle_tests_per_s": float(f"{pairs / (ms / 1e3):.4g}")}
        if cpu_voxelize is not None and name.startswith("sphere"):
            ids = np.arange(0, nx * ny, max(1, (nx * ny) // 2000))[:2000]
            t = time.perf_counter()
            cpu_voxelize(mesh.triangles, origin, (nx, ny, nz), pitch, ids)
            cpu_s = time.perf_counter() - t
            r["cpu_rays_per_s"] = round(len(ids) / cpu_s, 1)
            r["gpu_rays_per_s"] = round(nx * ny / (ms / 1e3), 1)
            r["cpu_sample"] = f"{len(ids)} columns, the CPU restatement (numpy), 1 host core"
        res[name] = r
    return res


def run(dev, cpu_baseline=True, large=True, cpu_voxelize=None):
    flush = torch.empty(64 << 20, dtype=torch.float32, device=dev)
    out = {"workload": "gyroid heat sink 384x192x192 (L=48, t=0.3), voxel SDF + links + trilinear q",
           "edt_bytes_per_cell": EDT_BYTES_PER_CELL}
    solid = geo.mask_from_levelset((384, 192, 192), geo.gyroid_levelset(48.0, 0.3), device=dev)
    phi, r = _measure(solid, flush)
    out.update(r)
    if cpu_baseline:
        from scipy.ndimage import distance_transform_edt
        s = solid.cpu().numpy()
        t = time.perf_counter()
        d_out = distance_transform_edt(~s)
        d_in = distance_transform_edt(s)
        cpu_ms = (time.perf_counter() - t) * 1e3
        ref = d_out
        ref[s] = -d_in[s]
        out["scipy_edt_ms"] = round(cpu_ms, 1)
        out["scipy_edt_cores"] = 1
        out["edt_speedup_over_scipy"] = round(cpu_ms / out["edt_ms"], 1)
        out["edt_equals_scipy"] = bool(torch.equal(phi.cpu(), torch.from_numpy(ref.astype("float32"))))
    del phi, solid
    out["voxelizer"] = voxelizer_run(dev, flush, cpu_voxelize if cpu_baseline else None)
    if large:
        G = geo.pin_gyroid_levelset(768, 384, 384, device=dev)
        solid = geo.mask_from_levelset((768, 384, 384), G, device=dev)
        _, r = _measure(solid, flush)
        r["workload"] = "pin + gyroid hybrid 768x384x384 (pins r=5, gyroid L=64, t=0.3, seed 2)"
        out["large"] = r
        del solid
    torch.cuda.empty_cache()
    return out


if __name__ == "__main__":
    import json
    print(json.dumps(run(torch.device("cuda"))))
