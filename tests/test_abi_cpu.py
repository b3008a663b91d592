"""The C-ABI library builds, loads without a GPU and exports every symbol the header declares;
host-side logic (face roles, link tables, sponge profile, BC plan) on CPU tensors."""
import ctypes
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
    assert native_lib.fc_abi_version() == _lib.ABI_VERSION
    assert native_lib.fc_lbm_step_args_size() == ctypes.sizeof(_lib.StepArgs)


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
    assert native_lib.fc_lbm_wait_selftest(16, 0, None, None) == 1
    # a carried tracer needs every buffer, and distinct in / out buffers and velocity / macro outputs
    # (the step checks the argument block before it touches any pointer)
    good = _lib.StepArgs()
    good.nx, good.ny, good.nz = 16, 8, 16
    good.pop_in, good.pop_out, good.cell_flags = 0x10000, 0x20000, 0x30000
    for bad in ({"tracer_out": None}, {"tracer_solid": None}, {"tracer_out": 0x40000},
                {"u": 0x50000, "v": 0x51000, "w": 0x52000, "rho": 0x53000}):
        a = _lib.StepArgs.from_buffer_copy(good)
        a.tracer_in, a.tracer_out = 0x40000, 0x41000
        a.tracer_u, a.tracer_v, a.tracer_w, a.tracer_solid = 0x50000, 0x51000, 0x52000, 0x60000
        assert native_lib.fc_lbm_tile_links(a, None, 0, None, 0, None, 0, None) > 0   # accepted as is
        for k, v in bad.items():
            setattr(a, k, v)
        assert native_lib.fc_lbm_tile_links(a, None, 0, None, 0, None, 0, None) == -1, bad
        assert native_lib.fc_lbm_fused_step(a, None) == 1, bad


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


def oracle_ibb(solid: np.ndarray, phi: np.ndarray):
    """IBBData on CPU tensors from the geometry oracle (host-side table tests need no GPU)."""
    from fluxcore3d_gb300 import geometry as geo
    from oracle import geometry as og
    r = og.ibb_from_sdf(solid, phi)
    t = {k: torch.from_numpy(np.ascontiguousarray(v)) for k, v in r.items()}
    return geo.IBBData(int(r["fluid_flat"].size), t["fluid_flat"], t["dir_i"], t["dir_opp"], t["q_ge_half"],
                       t["w_i"], t["w_second"], t["ff_flat"], t["ff_valid"])


def test_link_table_groups_links_by_cell():
    from fluxcore3d_gb300.solver.fused_lbm import build_link_table
    d = np.load(os.path.join(ROOT, "tests", "golden", "ibb_links.npz"))
    solid = torch.from_numpy(d["heatsink_solid"])
    ibb = oracle_ibb(d["heatsink_solid"], d["heatsink_phi"])
    nx, ny, nz = solid.shape
    t = build_link_table(ibb, solid.to(torch.uint8).reshape(-1), nx, ny, nz)
    assert t["n_links"] == ibb.n_links and int(t["counts"].sum()) == ibb.n_links
    ref = {}
    for f, dd, g, fv, w1, w2 in zip(ibb.fluid_flat.tolist(), ibb.dir_i.tolist(), ibb.q_ge_half.tolist(),
                                    ibb.ff_valid.tolist(), ibb.w_i.tolist(), ibb.w_second.tolist()):
        ref[(f, dd)] = (g, fv, w1, w2)
    hdr = t["link_hdr"].numpy().astype(np.int64)
    lw = t["link_w"].numpy()
    cells = t["link_cells"].numpy()
    assert np.all(np.diff(cells) > 0)
    n_modes = {"ge": 0, "ff": 0, "fallback": 0}
    for o, cell in enumerate(cells):
        assert int(t["link_off"][cell]) == o
        mask, smask, w0 = hdr[o, 0], hdr[o, 1], hdr[o, 2]
        dirs = [q for q in range(1, 19) if (mask >> q) & 1]
        for r, q in enumerate(dirs):
            g, fv, w1, w2 = ref[(int(cell), q)]
            second = bool((smask >> q) & 1)
            if g:
                assert not second and (lw[w0 + r] == np.float32([w1, w2])).all()
                n_modes["ge"] += 1
            elif fv:
                assert second and (lw[w0 + r] == np.float32([w1, w2])).all()
                n_modes["ff"] += 1
            else:
                assert not second and (lw[w0 + r] == np.float32([1.0, 0.0])).all()
                n_modes["fallback"] += 1
    assert sum(n_modes.values()) == ibb.n_links and n_modes["ff"] > 0


def test_link_table_rejects_inconsistent_data():
    from fluxcore3d_gb300 import geometry as geo
    from fluxcore3d_gb300.solver.fused_lbm import build_link_table
    from oracle import geometry as og
    solid = geo.cube_mask((8, 8, 8), (4, 4, 4), (2, 2, 2))
    ibb = oracle_ibb(solid.numpy(), og.signed_edt(solid.numpy()))
    bad = geo.IBBData(ibb.n_links, ibb.fluid_flat, ibb.dir_i, ibb.dir_i.clone(), ibb.q_ge_half, ibb.w_i,
                      ibb.w_second, ibb.ff_flat, ibb.ff_valid)
    with pytest.raises(ValueError):
        build_link_table(bad, solid.to(torch.uint8).reshape(-1), 8, 8, 8)


def test_fused_engine_flags_and_sponge_profile_on_cpu_state():
    """Plan built from a CPU solver state: deferred inlet/outlet planes, export planes, sponge profile."""
    from fluxcore3d_gb300 import case as cases
    from fluxcore3d_gb300.solver.fused_lbm import FusedLBM
    sim = cases.channel_cube(device="cpu", nx=20, ny=8, nz=8, cube=4, cube_x=8, sponge_length=5,
                             outlet="pressure", with_links=False)
    sim._solid_u8 = sim.solid_flow.to(torch.uint8)
    fc = FusedLBM(sim)
    fl = fc.flags.view(20, 8, 8)
    assert bool(((fl[0] & 4) != 0).all()) and bool(((fl[19] & 4) != 0).all())
    assert bool(((fl[1] & 8) != 0).all()) and bool(((fl[18] & 8) != 0).all())
    assert fc.planes == [(0, 19), (0, 0)]          # +X outlet first, then -X inlet (face order)
    assert torch.allclose(fc.sponge[-5:], torch.tensor([((k + 1) / 5) ** 2 * 0.3 for k in range(5)]))
    assert float(fc.sponge[:-5].abs().sum()) == 0.0
