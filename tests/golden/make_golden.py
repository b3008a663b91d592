"""Generate the golden fixtures in tests/golden/ by running the reference's own
Python implementation (fluxcore3D, torch CPU path) on small seeded inputs.

Run in a container where the reference tree is available:
    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py /path/to/fluxcore3D

Stub modules stand in for pyvista / trimesh (only the viewers and STL loading
use them).  Fixtures written (all small .npz files):
  mrt_matrix.npz      M and M^-1 of flow_solver_upgrade.py:98-125
  lbm_ops.npz         collide (BGK, TRT via LBM_CHT._collide; MRT via
                      FlowSolverUpgrade._collide_mrt), stream (LBM_CHT._stream),
                      interpolated bounce-back + reset (LBM_CHT._interp_bounce_back_from_post)
  ibb_links.npz       build_ibb_from_sdf_gpu link arrays and q on a cube and on a
                      crop of fluxcore3D_web/Heatsink.npz (phi from build_phi_from_voxel_mask_mm)
  ibb_pitch.npz       the same with a non-unit pitch, a shifted voxel origin and a
                      non-zero offset_ijk, and the fractions q themselves (captured
                      from bfl_q_from_sdf); written alone by `--only ibb_pitch`
  tracer.npz          TracerField (pre_post/tracer_patch.py) on seeded velocity and
                      solid fields: the field after 1 and after 25 steps with
                      injections; written alone by `--only tracer`
  voxels.npz          gpu_voxelize_mesh (pre_post/gpu_voxelizer.py, torch CPU path)
                      on three closed meshes built by fluxcore3d_gb300.pre_post.stl
                      (box, icosphere, finned heat sink): triangles, grid and the
                      packed voxel grids; written alone by `--only voxels`
  thermal_steady.npz  steady temperature of a heated channel from the reference's fused
                      pseudo-time thermal step with its FP64 torch multigrid and its thermal
                      kernels built for the host (oracle/build_ref.py); written alone by
                      `--only thermal_steady`
  mg_solve.npz        NLevelGeometricMGSolver (torch fallback, float64): coefficients,
                      L_apply_fine, V-cycle solve, pcg_mg and bicgstab_mg results
"""
from __future__ import annotations

import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _stub_modules():
    for name in ("pyvista", "trimesh", "trimesh.proximity"):
        m = types.ModuleType(name)
        m.Trimesh = object
        m.ProximityQuery = object
        sys.modules[name] = m
    sys.modules["trimesh"].proximity = sys.modules["trimesh.proximity"]


def main(ref_root: str):
    os.environ["PYTHONDONTWRITEBYTECODE"] = "1"
    sys.dont_write_bytecode = True
    _stub_modules()
    sys.path.insert(0, ref_root)
    import torch
    torch.set_num_threads(max(1, os.cpu_count() or 1))
    import LBM_CHT as R
    from solver import flow_solver_upgrade as FSU
    from solver.nlevel_mg_cuda import NLevelGeometricMGSolver
    from solver import mg_pcg
    from pre_post import sdf_tracing as SDF

    np.savez(os.path.join(HERE, "mrt_matrix.npz"), M=FSU._M_D3Q19, Minv=FSU._M_INV_D3Q19)

    # ---------------- lattice operations on a 10x8x6 box with a cube --------------
    def make_sim(collision):
        cfg = R.SimConfig3D(nx=10, ny=8, nz=6, Lx_m=0.01, Ly_m=0.008, Lz_m=0.006, u_in_mps=0.05,
                            device="cpu", collision=collision, transverse_walls=False, sponge_length=0,
                            obstacle={"type": "cube", "cx": 5, "cy": 4, "cz": 3, "wx": 2, "wy": 2, "wz": 2})
        cfg.dx_mm = 1.0
        fl = R.FluidPropsSI(nu_m2_s=1e-5)
        return R.LBMCHT3D_Torch(cfg, fl, R.SolidPropsSI())

    g = torch.Generator().manual_seed(11)
    out = {}
    for col in ("bgk", "trt", "mrt"):
        sim = make_sim(col)
        f0 = (torch.rand((19, 10, 8, 6), generator=g, dtype=torch.float32) * 0.02
              + torch.tensor(R.LBMCHT3D_Torch.w_np)[:, None, None, None])
        sim.f = f0.clone()
        sim._macroscopic()
        if col == "mrt":
            FSU.FlowSolverUpgrade._init_mrt(sim)
            FSU.FlowSolverUpgrade._collide_mrt(sim)
            out["mrt_S"] = sim._mrt_S.numpy()
        else:
            sim._collide()
        out[f"{col}_f0"] = f0.numpy()
        out[f"{col}_fpost"] = sim.f.numpy()
        out[f"{col}_omega"] = np.float64(float(sim.omega_plus))
        if col == "trt":
            out["trt_omega_minus"] = np.float64(float(sim.omega_minus))
    out["solid"] = sim.solid.numpy()
    # streaming with the face roles of the default config (+X flow, periodic y/z)
    sim = make_sim("bgk")
    fs = torch.rand((19, 10, 8, 6), generator=g, dtype=torch.float32)
    sim.f = fs.clone()
    sim._stream()
    out["stream_in"] = fs.numpy()
    out["stream_out"] = sim.f.numpy()
    # interpolated bounce-back from a voxel SDF
    sim = make_sim("bgk")
    phi = SDF.build_phi_from_voxel_mask_mm(sim.solid.numpy(), 1.0, device="cpu")
    sim.phi = phi
    SDF.build_ibb_from_sdf_gpu(sim, voxel_origin_mm=(0.0, 0.0, 0.0), pitch_mm=1.0, offset_ijk=(0, 0, 0),
                               c_np=sim.c_np, opp_np=sim.opp_np)
    fpost = torch.rand((19, 10, 8, 6), generator=g, dtype=torch.float32)
    fstr = torch.rand((19, 10, 8, 6), generator=g, dtype=torch.float32)
    sim.f = fstr.clone()
    sim._interp_bounce_back_from_post(fpost.contiguous())
    d = sim.ibb_data
    out.update(ibb_fpost=fpost.numpy(), ibb_fstream=fstr.numpy(), ibb_out=sim.f.numpy(),
               ibb_fluid_flat=d.fluid_flat.numpy(), ibb_dir_i=d.dir_i.numpy(), ibb_dir_opp=d.dir_opp.numpy(),
               ibb_w_i=d.w_i.numpy(), ibb_w_second=d.w_second.numpy(), ibb_q_ge_half=d.q_ge_half.numpy(),
               ibb_ff_flat=d.ff_flat.numpy(), ibb_ff_valid=d.ff_valid.numpy())
    np.savez_compressed(os.path.join(HERE, "lbm_ops.npz"), **out)

    # ---------------- link arrays + q on two voxel geometries ------------------------
    links = {}
    hs = np.load(os.path.join(ref_root, "fluxcore3D_web", "Heatsink.npz"))["voxel_solid"].astype(bool)
    crop = np.zeros((40, 36, 24), bool)
    crop[4:36, 2:34, 2:22] = hs[30:62, 40:72, 0:20]
    cube = np.zeros((12, 10, 9), bool)
    cube[4:8, 3:7, 2:6] = True
    for name, solid in (("cube", cube), ("heatsink", crop)):
        s = types.SimpleNamespace(device=torch.device("cpu"), nx=solid.shape[0], ny=solid.shape[1],
                                  nz=solid.shape[2])
        s.solid = torch.from_numpy(solid)
        s.phi = SDF.build_phi_from_voxel_mask_mm(solid, 1.0, device="cpu")
        SDF.build_ibb_from_sdf_gpu(s, voxel_origin_mm=(0.0, 0.0, 0.0), pitch_mm=1.0, offset_ijk=(0, 0, 0),
                                   c_np=R.LBMCHT3D_Torch.c_np, opp_np=R.LBMCHT3D_Torch.opp_np)
        d = s.ibb_data
        links[f"{name}_solid"] = solid
        links[f"{name}_phi"] = s.phi.numpy()
        for k in ("fluid_flat", "dir_i", "dir_opp", "q_ge_half", "w_i", "w_second", "ff_flat", "ff_valid"):
            links[f"{name}_{k}"] = getattr(d, k).numpy()
    np.savez_compressed(os.path.join(HERE, "ibb_links.npz"), **links)

    # ---------------- multigrid (float64 torch path) ---------------------------------
    rng = np.random.default_rng(7)
    shape = (24, 12, 12)
    k = np.where(rng.random(shape) < 0.3, 200.0, 1.0) * 0.005
    rcp = np.where(rng.random(shape) < 0.5, 1.0, 2.0)
    u = rng.random(shape) * 0.05
    v = (rng.random(shape) - 0.5) * 0.02
    w = (rng.random(shape) - 0.5) * 0.02
    mask = np.ones(shape, bool)
    mask[0] = False
    b = rng.random(shape) * mask
    T = rng.random(shape)
    t = lambda a: torch.tensor(a, dtype=torch.float64)
    mgo = {"k": k, "rcp": rcp, "u": u, "v": v, "w": w, "mask": mask, "b": b, "T": T, "dt": 3.0, "s": 1.5}
    mg = NLevelGeometricMGSolver(torch.device("cpu"), torch.float64, 0, 1, 1.5, omega=0.6)
    mg.build_if_needed(t(k), t(rcp), t(u), t(v), t(w), torch.tensor(mask), 3.0)
    for li, lv in enumerate(mg._levels):
        for key in ("aE", "aW", "aN", "aS", "aU", "aD", "diagL", "inv_diagM", "mask_f"):
            mgo[f"L{li}_{key}"] = lv[key].numpy()
    mgo["nlevels"] = len(mg._levels)
    mgo["LT"] = mg.L_apply_fine(t(T)).numpy()
    x, info = mg.solve(t(b), None, max_cycles=6, tol=0.0)
    mgo["solve_x"] = x.numpy()
    mgo["solve_res"] = info["res_rel"]
    x, info = mg_pcg.bicgstab_mg(mg, t(b), None, tol=1e-9, max_it=8)
    mgo["bicgstab_x"] = x.numpy()
    mgo["bicgstab_it"] = info["it"]
    x, info = mg_pcg.pcg_mg(mg, t(b), None, tol=1e-9, max_it=6)
    mgo["pcg_x"] = x.numpy()
    mgo["pcg_it"] = info["it"]
    np.savez_compressed(os.path.join(HERE, "mg_solve.npz"), **mgo)
    print("golden fixtures written to", HERE)


def ibb_pitch(ref_root: str):
    """Voxel SDF, link arrays, weights and fractions at pitches 0.37 and 0.5 (torch CPU path)."""
    os.environ["PYTHONDONTWRITEBYTECODE"] = "1"
    sys.dont_write_bytecode = True
    _stub_modules()
    sys.path.insert(0, ref_root)
    import torch
    import LBM_CHT as R
    from pre_post import sdf_tracing as SDF

    captured = {}
    orig_q = SDF.bfl_q_from_sdf

    def capture_q(*a, **kw):
        q = orig_q(*a, **kw)
        captured["q"] = q
        return q
    SDF.bfl_q_from_sdf = capture_q
    hs = np.load(os.path.join(ref_root, "fluxcore3D_web", "Heatsink.npz"))["voxel_solid"].astype(bool)
    crop = np.zeros((30, 26, 22), bool)
    crop[3:27, 2:24, 0:18] = hs[10:34, 20:42, 0:18]
    I, J, K = np.indices((24, 20, 18))
    balls = ((I - 9.3) ** 2 + (J - 8.1) ** 2 + (K - 7.7) ** 2 < 5.2 ** 2) | \
            ((I - 17.6) ** 2 + (J - 13.2) ** 2 + (K - 10.4) ** 2 < 3.9 ** 2)
    out = {}
    cases = (("crop", crop, 0.37, (1.5, -2.25, 0.125), (2, 1, 3)),
             ("balls", balls, 0.5, (-0.75, 0.3, 4.0), (0, 2, 1)))
    for name, solid, pitch, vo, off in cases:
        s = types.SimpleNamespace(device=torch.device("cpu"), nx=solid.shape[0], ny=solid.shape[1],
                                  nz=solid.shape[2])
        s.solid = torch.from_numpy(solid)
        s.phi = SDF.build_phi_from_voxel_mask_mm(solid, pitch, device="cpu")
        SDF.build_ibb_from_sdf_gpu(s, voxel_origin_mm=vo, pitch_mm=pitch, offset_ijk=off,
                                   c_np=R.LBMCHT3D_Torch.c_np, opp_np=R.LBMCHT3D_Torch.opp_np)
        d = s.ibb_data
        out[f"{name}_solid"] = solid
        out[f"{name}_phi"] = s.phi.numpy()
        out[f"{name}_pitch"] = np.float64(pitch)
        out[f"{name}_voxel_origin"] = np.array(vo, np.float64)
        out[f"{name}_offset_ijk"] = np.array(off, np.int64)
        out[f"{name}_q"] = captured["q"].numpy()
        for k in ("fluid_flat", "dir_i", "dir_opp", "q_ge_half", "w_i", "w_second", "ff_flat", "ff_valid"):
            out[f"{name}_{k}"] = getattr(d, k).numpy()
    SDF.bfl_q_from_sdf = orig_q
    np.savez_compressed(os.path.join(HERE, "ibb_pitch.npz"), **out)
    print("ibb_pitch.npz written to", HERE)


def voxels(ref_root: str):
    """Reference voxel grids of three procedural meshes (triangles stored, so no mesh file travels)."""
    os.environ["PYTHONDONTWRITEBYTECODE"] = "1"
    sys.dont_write_bytecode = True
    _stub_modules()
    sys.path.insert(0, ref_root)
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from pre_post import gpu_voxelizer as GV
    from fluxcore3d_gb300.pre_post import stl
    meshes = {
        "box": (stl.box_mesh((0.0, 0.0, 0.0), (10.0, 20.0, 5.0)), 0.5),
        "sphere": (stl.icosphere_mesh(5.0, 3, center=(1.3, -0.7, 2.1)), 0.45),
        "finsink": (stl.fin_heatsink_mesh(base=(24.0, 16.0, 2.0), n_fins=6, fin_t=1.2, fin_h=9.0,
                                          origin=(-3.1, 2.2, 0.4)), 0.37),
    }
    out = {}
    for name, (mesh, pitch) in meshes.items():
        v, o = GV.gpu_voxelize_mesh(mesh, pitch, device="cpu")
        out[f"{name}_tri"] = mesh.triangles.astype(np.float32)
        out[f"{name}_pitch"] = np.float64(pitch)
        out[f"{name}_origin"] = o
        out[f"{name}_dims"] = np.array(v.shape, np.int64)
        out[f"{name}_bits"] = np.packbits(v.astype(bool).ravel())
        out[f"{name}_count"] = np.int64(v.sum())
    np.savez_compressed(os.path.join(HERE, "voxels.npz"), **out)
    print("voxels.npz written to", HERE)


def tracer(ref_root: str):
    os.environ["PYTHONDONTWRITEBYTECODE"] = "1"
    sys.dont_write_bytecode = True
    _stub_modules()
    sys.path.insert(0, ref_root)
    import torch
    from pre_post import tracer_patch as TP
    g = torch.Generator().manual_seed(21)
    nx, ny, nz = 20, 14, 11
    solid = torch.rand((nx, ny, nz), generator=g) < 0.15
    out = {"solid_flow": solid.numpy()}
    sim = types.SimpleNamespace(nx=nx, ny=ny, nz=nz, device=torch.device("cpu"), solid_flow=solid)
    vel = []
    for s in range(5):
        f = [(torch.rand((nx, ny, nz), generator=g) - 0.45) * 0.3 for _ in range(3)]
        vel.append(f)
        for a, name in enumerate(("u", "v", "w")):
            out[f"{name}{s}"] = f[a].numpy()
    tr = TP.TracerField(sim, flow_dir="+X", inject_depth=3, dissipation=0.9995)
    tr.inject()
    out["inlet"] = tr._inlet.numpy()
    for it in range(25):
        sim.u, sim.v, sim.wv = vel[it // 5]
        if it % 7 == 6:
            tr.inject()
        tr.step()
        if it == 0:
            out["field1"] = tr.field.numpy().copy()
    out["field25"] = tr.field.numpy().copy()
    np.savez_compressed(os.path.join(HERE, "tracer.npz"), **out)
    print("tracer.npz written to", HERE)


def thermal_steady(ref_root: str):
    """Steady temperature of a heated channel from the reference's own fused pseudo-time thermal step
    (solver/thermal_cuda_ext.py:55-201, _temperature_step_mg_fused, the path the reference takes on a
    GPU) with its multigrid in FP64 (solver/nlevel_mg_cuda.py, torch path) and its
    thermal_reconstruct / physics_check kernels (solver/thermal_kernels.cu) compiled for the host in
    FP64 by oracle/build_ref.py, iterated with the ramped pseudo-time step of
    solve_thermal_steady_only (LBM_CHT.py:2388-2569: dt from 5, times 1.5 per step, at most 200)
    until a step changes T by less than 2e-13; T after the first three steps is kept too.
    Channel 24x16x16, solid cube 6^3 centred at (8, 8, 8), k_s/k_f = 100, velocity 0.02 along +x in
    the fluid (zero in the solid and in the wall planes z = 0, 15), heat source 0.05 in the cube,
    inlet x = 0 at Tin = 25."""
    import ctypes as C
    os.environ["PYTHONDONTWRITEBYTECODE"] = "1"
    sys.dont_write_bytecode = True
    _stub_modules()
    sys.path.insert(0, ref_root)
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    import torch
    import LBM_CHT as R
    from oracle import build_ref
    from solver import thermal_cuda_ext as TCE

    lib = C.CDLL(build_ref.build_thermal(ref_root))
    vp, i32, f64 = C.c_void_p, C.c_int, C.c_double
    lib.ref_thermal_reconstruct64.argtypes = [vp, vp, vp, i32, i32, i32, i32, i32]
    lib.ref_physics_check64.argtypes = [vp, f64, f64, i32]
    lib.ref_physics_check64.restype = i32

    class _HostThermal:
        """THERMAL_CUDA's calls of the fused step, on the host kernels (FP64 tensors)."""

        @staticmethod
        def thermal_reconstruct(T0, theta, nx, ny, nz, ax, out_idx):
            a, b = T0.contiguous(), theta.contiguous()
            out = torch.empty_like(a)
            lib.ref_thermal_reconstruct64(a.data_ptr(), b.data_ptr(), out.data_ptr(), nx, ny, nz, ax, out_idx)
            return out

        @staticmethod
        def physics_check(T, T_min, T_max):
            t = T.contiguous()
            return torch.tensor([lib.ref_physics_check64(t.data_ptr(), T_min, T_max, t.numel())], dtype=torch.int32)

        @staticmethod
        def convergence_metrics(T_new, T_old, solid_u8):
            dT = (T_new - T_old).abs()
            s = solid_u8.bool()
            return [dT[s].max().reshape(1), dT[~s].max().reshape(1)]

    TCE.THERMAL_CUDA, TCE.THERMAL_CUDA_AVAILABLE = _HostThermal(), True

    nx, ny, nz = 24, 16, 16
    solid = torch.zeros((nx, ny, nz), dtype=torch.bool)
    solid[5:11, 5:11, 5:11] = True
    solid_flow = solid.clone()
    solid_flow[:, :, 0] = True
    solid_flow[:, :, -1] = True
    nu = 0.05 * 6 / 50.0
    alpha_f = nu / 0.71
    k = torch.full((nx, ny, nz), alpha_f, dtype=torch.float32)
    k[solid] = alpha_f * 100.0
    u = torch.full((nx, ny, nz), 0.02, dtype=torch.float32)
    u[solid_flow] = 0.0
    src = torch.zeros((nx, ny, nz), dtype=torch.float32)
    src[solid] = 0.05

    class _Host:
        pass

    h = _Host()
    h.cfg = types.SimpleNamespace(flow_dir="+X", temp_bc="fixed", mg_omega=0.6, mg_pre_smooth=2, mg_post_smooth=2,
                                  mg_coarse_iters=20, domain_walls=["+Z", "-Z"], domain_outlets=[],
                                  transverse_walls=False, flow_bc="inlet_outlet")
    h.nx, h.ny, h.nz = nx, ny, nz
    h.fluid = types.SimpleNamespace(tin_C=25.0)
    h.thermal_dt_scale = 1.0
    h.ax, h.sign = 0, +1
    h.solid = solid
    d = torch.float64
    h.T = torch.full((nx, ny, nz), 25.0, dtype=d)
    h.k, h.rho_cp = k.to(d), torch.ones((nx, ny, nz), dtype=d)
    h.u, h.v, h.wv = u.to(d), torch.zeros((nx, ny, nz), dtype=d), torch.zeros((nx, ny, nz), dtype=d)
    h._compute_surface_flux_sources = lambda: torch.zeros((nx, ny, nz), dtype=d)
    h._compute_heat_source = lambda: src.to(d)
    for name in ("_build_update_mask_thermal", "_build_T_dirichlet_field"):
        setattr(h, name, types.MethodType(getattr(R.LBMCHT3D_Torch, name), h))
    step = types.MethodType(TCE._temperature_step_mg_fused, h)
    dt, T3, dT, it = 5.0, None, float("inf"), 0
    for it in range(400):
        Tprev = h.T.clone()
        step(dt=dt, tol=1e-13, max_cycles=200)
        dT = float((h.T - Tprev).abs().max())
        dt = min(200.0, 1.5 * dt)
        if it == 2:
            T3 = h.T.clone()
        if dT < 2e-13:
            break
    print(f"thermal_steady: {it + 1} pseudo-time steps, last dT {dT:.3e}")
    np.savez_compressed(os.path.join(HERE, "thermal_steady.npz"), T=h.T.numpy(), T3=T3.numpy(), k=k.numpy(),
                        u=u.numpy(), src=src.numpy(), solid=solid.numpy(), solid_flow=solid_flow.numpy(),
                        steps=np.array(it + 1))
    print("thermal_steady.npz written to", HERE)


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("reference_root", help="root of the fluxcore3D source tree (read only)")
    ap.add_argument("--only", choices=("main", "ibb_pitch", "voxels", "tracer", "thermal_steady"), default=None)
    a = ap.parse_args()
    root = a.reference_root
    if a.only == "main":
        main(root)
    elif a.only == "ibb_pitch":
        ibb_pitch(root)
    elif a.only == "voxels":
        voxels(root)
    elif a.only == "tracer":
        tracer(root)
    elif a.only == "thermal_steady":
        thermal_steady(root)
    else:
        main(root)
        ibb_pitch(root)
        voxels(root)
        tracer(root)
        thermal_steady(root)
