"""The C-ABI library builds, loads without a GPU and exports every symbol the header declares;
host-side logic (face roles, link tables, sponge profile, BC plan) on CPU tensors."""
import os
import re
import types

import numpy as np
import pytest
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for fn in os.listdir(inc):
        if fn.endswith(".h"):
            src = open(os.path.join(inc, fn)).read()
            names |= set(re.findall(r"^\s*(?:int|long long|void)\s+(fc_\w+)\s*\(", src, re.M))
    return names


def test_library_exports_every_declared_symbol(native_lib):
    from fluxcore3d_gb300 import _lib
    decl = declared_symbols()
    assert len(decl) >= 30
    missing = [n for n in decl if not hasattr(native_lib, n)]
    assert not missing, missing
    assert set(_lib.SIGNATURES) >= decl
    assert native_lib.fc_abi_version() == 1


def test_workspace_queries_without_gpu(native_lib):
    from fluxcore3d_gb300 import _lib
    assert _lib.call("fc_lbm_convective_workspace_bytes", 128, 128) > 0
    assert _lib.call("fc_lbm_convective_workspace_bytes", 0, 4) == -1
    assert _lib.call("fc_vec_workspace_bytes", 1000) >= 8 * 2
    assert _lib.call("fc_mg_reduce_workspace_bytes", 1 << 20) > 0


def test_argument_checks_return_status_without_gpu(native_lib):
    from fluxcore3d_gb300 import _lib
    # null pointers and bad modes are rejected before any launch
    assert native_lib.fc_lbm_stream_pull(None, None, 4, 4, 4, 0, 0, 0, None) == 1
    assert native_lib.fc_lbm_zou_he_bc(None, None, 4, 4, 4, 5, 0, 1, 0, 0.05, 1.0, 1, None) == 1
    args = _lib.StepArgs()
    args.storage = 7
    assert native_lib.fc_lbm_fused_step(args, None) == 1


def test_face_roles_table():
    from fluxcore3d_gb300.solver.face_roles import periodic_flags, resolve_face_roles
    from oracle.lbm import resolve_face_roles as oracle_roles
    cases = [("+X", [], [], False), ("-Y", ["+Z"], [], False), ("+Z", ["-Z"], ["+X"], True),
             ("+X", ["+Z", "-Z"], [], False)]
    for fd, walls, outs, legacy in cases:
        cfg = types.SimpleNamespace(flow_dir=fd, domain_walls=walls, domain_outlets=outs, transverse_walls=legacy)
        r = resolve_face_roles(cfg)
        assert r == oracle_roles(fd, walls, outs, legacy)
        assert list(r) == ["+X", "-X", "+Y", "-Y", "+Z", "-Z"]
    cfg = types.SimpleNamespace(flow_dir="+X", domain_walls=["+Z", "-Z"], domain_outlets=[], transverse_walls=False)
    assert periodic_flags(cfg) == (False, True, False)


def test_link_table_groups_links_by_cell():
    from fluxcore3d_gb300 import geometry as geo
    from fluxcore3d_gb300.solver.fused_lbm import build_link_table
    solid = geo.cube_mask((12, 10, 9), (6, 5, 4), (4, 4, 4))
    phi = torch.tensor(geo.phi_from_voxels(solid.numpy()), dtype=torch.float32)
    ibb = geo.ibb_from_phi_trilinear(solid, phi)
    off, meta, w, counts = build_link_table(ibb, solid.to(torch.uint8).reshape(-1), 12, 10, 9)
    assert int(counts.sum()) == ibb.n_links
    # every link reachable from its cell and terminated by the last bit
    seen = 0
    for cell in torch.nonzero(counts).reshape(-1).tolist():
        l0 = int(off[cell])
        c = int(counts[cell])
        dirs = [int(meta[l0 + t]) & 31 for t in range(c)]
        assert all(int(meta[l0 + t]) & 0x80 == 0 for t in range(c - 1)) and int(meta[l0 + c - 1]) & 0x80
        ref = sorted(int(d) for d, f in zip(ibb.dir_i.tolist(), ibb.fluid_flat.tolist()) if f == cell)
        assert dirs == ref
        seen += c
    assert seen == ibb.n_links


def test_link_table_rejects_inconsistent_data():
    from fluxcore3d_gb300 import geometry as geo
    from fluxcore3d_gb300.solver.fused_lbm import build_link_table
    solid = geo.cube_mask((8, 8, 8), (4, 4, 4), (2, 2, 2))
    phi = torch.tensor(geo.phi_from_voxels(solid.numpy()), dtype=torch.float32)
    ibb = geo.ibb_from_phi_trilinear(solid, phi)
    bad = geo.IBBData(ibb.n_links, ibb.fluid_flat, ibb.dir_i, ibb.dir_i.clone(), ibb.q_ge_half, ibb.w_i,
                      ibb.w_second, ibb.ff_flat, ibb.ff_valid)
    with pytest.raises(ValueError):
        build_link_table(bad, solid.to(torch.uint8).reshape(-1), 8, 8, 8)


def test_fused_engine_flags_and_sponge_profile_on_cpu_state():
    """Plan built from a CPU solver state: deferred inlet/outlet planes, export planes, sponge profile."""
    from fluxcore3d_gb300 import case as cases
    from fluxcore3d_gb300.solver.fused_lbm import FusedLBM
    sim = cases.channel_cube(device="cpu", nx=20, ny=8, nz=8, cube=4, cube_x=8, sponge_length=5,
                             outlet="pressure")
    sim._solid_u8 = sim.solid_flow.to(torch.uint8)
    fc = FusedLBM(sim)
    fl = fc.flags.view(20, 8, 8)
    assert bool(((fl[0] & 4) != 0).all()) and bool(((fl[19] & 4) != 0).all())
    assert bool(((fl[1] & 8) != 0).all()) and bool(((fl[18] & 8) != 0).all())
    assert fc.planes == [(0, 19), (0, 0)]          # +X outlet first, then -X inlet (face order)
    assert torch.allclose(fc.sponge[-5:], torch.tensor([((k + 1) / 5) ** 2 * 0.3 for k in range(5)]))
    assert float(fc.sponge[:-5].abs().sum()) == 0.0
