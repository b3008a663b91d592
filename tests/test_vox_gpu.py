"""STL voxelizer and body stamp kernels against the reference's voxel grids and the oracle."""
import os
import types

import numpy as np
import pytest
import torch

from fluxcore3d_gb300.pre_post import gpu_voxelizer as gv
from fluxcore3d_gb300.pre_post import stl
from fluxcore3d_gb300.pre_post.solid_stamp import SolidStampUpgrade, stamp_voxels
from oracle import voxelizer as ov

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden():
    d = np.load(os.path.join(GOLD, "voxels.npz"))
    for name in ("box", "sphere", "finsink"):
        dims = tuple(int(x) for x in d[f"{name}_dims"])
        want = np.unpackbits(d[f"{name}_bits"])[:np.prod(dims)].reshape(dims)
        yield name, d[f"{name}_tri"], float(d[f"{name}_pitch"]), d[f"{name}_origin"], dims, want


def test_voxel_grids_match_reference_golden(cuda):
    for name, tri, pitch, origin, dims, want in golden():
        o32 = origin.astype(np.float32)
        got = gv.voxelize_triangles(torch.from_numpy(tri).to(cuda), o32, dims, pitch).cpu().numpy()
        assert np.array_equal(got, want), name
        # the drop-in entry: same grid, origin and voxels from the mesh itself
        mesh = stl.MeshData(tri.reshape(-1, 3), np.arange(tri.shape[0] * 3).reshape(-1, 3))
        v, o = gv.gpu_voxelize_mesh(mesh, pitch)
        assert v.shape == dims and np.array_equal(o, origin) and np.array_equal(v, want), name


def random_meshes(seed=1):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(4):
        c = rng.uniform(-5, 5, 3)
        out.append((stl.icosphere_mesh(rng.uniform(2, 6), int(rng.integers(1, 4)), center=c),
                    float(rng.uniform(0.15, 0.6))))
    lo = rng.uniform(-3, 3, 3)
    out.append((stl.box_mesh(lo, lo + rng.uniform(1, 8, 3)), 0.25))
    out.append((stl.fin_heatsink_mesh(base=(30.0, 12.0, 2.5), n_fins=9, fin_t=0.9, fin_h=17.0,
                                      origin=tuple(rng.uniform(-4, 4, 3))), 0.21))
    # two overlapping bodies: parity of the union (double hits cancel inside the overlap)
    out.append((stl.merge(stl.icosphere_mesh(3.0, 2), stl.icosphere_mesh(3.0, 2, center=(2.5, 0.3, -0.4))), 0.3))
    # a degenerate (zero-area) triangle mixed in
    m = stl.box_mesh((0, 0, 0), (3, 4, 5))
    m = stl.MeshData(np.concatenate([m.vertices, [[1, 1, 1], [2, 2, 2], [3, 3, 3]]]),
                     np.concatenate([m.faces, [[8, 9, 10]]]))
    out.append((m, 0.33))
    return out


def test_voxel_grids_match_oracle_on_seeded_meshes(cuda):
    for mesh, pitch in random_meshes():
        tri = mesh.triangles
        origin, dims = ov.grid(mesh.vertices, pitch)
        got = gv.voxelize_triangles(torch.from_numpy(tri).to(cuda), origin, dims, pitch).cpu().numpy()
        want = ov.voxelize(tri, origin, dims, pitch)
        assert np.array_equal(got, want), (dims, pitch)


def test_large_mesh_sampled_columns_and_volume(cuda):
    """A 20,480-triangle sphere and a finned heat sink at fine pitch (tens of millions of cells):
    2,000 sampled columns equal the oracle's, and the solid volume is the analytic one."""
    rng = np.random.default_rng(0)
    sph = stl.icosphere_mesh(10.0, 5)
    sink = stl.fin_heatsink_mesh(base=(40.0, 30.0, 3.0), n_fins=8, fin_t=1.5, fin_h=20.0)
    for mesh, pitch, vol in ((sph, 0.05, None), (sink, 0.06, 40 * 30 * 3 + 8 * 1.5 * 30 * 20)):
        tri = mesh.triangles
        origin, dims = ov.grid(mesh.vertices, pitch)
        got = gv.voxelize_triangles(torch.from_numpy(tri).to(cuda), origin, dims, pitch)
        ids = rng.choice(dims[0] * dims[1], 2000, replace=False)
        want = ov.voxelize(tri, origin, dims, pitch, ray_ids=ids)
        assert np.array_equal(got.reshape(-1, dims[2])[torch.from_numpy(ids).to(cuda)].cpu().numpy(), want)
        if vol is not None:
            v = float(got.sum()) * pitch ** 3
            assert abs(v - vol) / vol < 0.01


def test_stamp_matches_oracle(cuda):
    rng = np.random.default_rng(3)
    nx, ny, nz = 30, 22, 17
    solid = rng.random((nx, ny, nz)) < 0.1
    k = rng.random((nx, ny, nz)).astype(np.float32)
    rcp = rng.random((nx, ny, nz)).astype(np.float32)
    sim = types.SimpleNamespace(nx=nx, ny=ny, nz=nz, solid=torch.from_numpy(solid.copy()).to(cuda),
                                k=torch.from_numpy(k.copy()).to(cuda), rho_cp=torch.from_numpy(rcp.copy()).to(cuda))
    for offset, shape in (((4, 3, 2), (9, 8, 7)), ((-3, 15, 10), (12, 10, 12)), ((25, -4, -6), (9, 9, 9)),
                          ((40, 0, 0), (3, 3, 3))):
        vox = rng.random(shape) < 0.5
        kv, rv = float(rng.uniform(1, 400)), float(rng.uniform(0.5, 3))
        body, n = stamp_voxels(sim, torch.from_numpy(vox), offset, kv, rv)
        want_body = ov.stamp(solid, k, rcp, vox, offset, kv, rv)
        assert np.array_equal(sim.solid.cpu().numpy(), solid), offset
        assert np.array_equal(sim.k.cpu().numpy(), k) and np.array_equal(sim.rho_cp.cpu().numpy(), rcp)
        assert np.array_equal(body.cpu().numpy(), want_body)
        i0, j0, k0 = offset
        inside = vox[max(0, -i0):max(0, min(shape[0], nx - i0)), max(0, -j0):max(0, min(shape[1], ny - j0)),
                     max(0, -k0):max(0, min(shape[2], nz - k0))]
        assert n == int(inside.sum())


def test_add_solid_body_drop_in(cuda, tmp_path, capsys):
    nx, ny, nz = 20, 16, 12
    sim = types.SimpleNamespace(nx=nx, ny=ny, nz=nz, dx_phys_m=0.5e-3, rho_cp_ref_J_m3K=4.0e6, k_ref_W_mK=0.6,
                                solid=torch.zeros((nx, ny, nz), dtype=torch.bool, device=cuda),
                                k=torch.ones((nx, ny, nz), device=cuda), rho_cp=torch.ones((nx, ny, nz), device=cuda))
    SolidStampUpgrade.patch(sim)
    mesh = stl.box_mesh((0, 0, 0), (3.0, 2.0, 1.5))
    v, o = gv.gpu_voxelize_mesh(mesh, 0.5)
    path = str(tmp_path / "body.npz")
    np.savez(path, voxel_solid=v, pitch_mm=0.5, voxel_origin_mm=o)
    props = types.SimpleNamespace(k_W_mK=400.0, rho_cp_J_m3K=3.45e6)
    sim.add_solid_body(path, (2, 3, 1), props, name="cu")
    assert "[cu] stamped" in capsys.readouterr().out
    assert int(sim.solid.sum()) == int(v.sum())
    assert float(sim.k[sim.solid].unique()) == float(np.float32(400.0 / 0.6))
    with pytest.raises(ValueError):
        np.savez(path, voxel_solid=v, pitch_mm=0.9, voxel_origin_mm=o)
        sim.add_solid_body(path, (0, 0, 0), props, name="bad")
