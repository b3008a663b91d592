"""Pin the oracle (and the link/q builder) against fixtures produced by the reference's own
Python implementation (tests/golden/make_golden.py).  CPU only."""
import os

import numpy as np
import pytest
import torch

from oracle import lbm as olbm
from oracle import mg as omg

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
W_TORCH = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12, dtype=np.float32)  # LBM_CHT.py:550-553


def load(name):
    return np.load(os.path.join(G, name))


def test_mrt_matrix_matches_reference():
    d = load("mrt_matrix.npz")
    M = olbm.mrt_matrix()
    assert np.array_equal(M, d["M"])
    assert np.allclose(np.linalg.inv(M), d["Minv"], rtol=0, atol=1e-14)
    # rows are orthogonal, so M^-1 = M^T diag(1/|M_k|^2) (the fused kernel relies on this)
    assert np.allclose(M @ M.T, np.diag(np.diag(M @ M.T)))


@pytest.mark.parametrize("col", ["bgk", "trt", "mrt"])
def test_collide_matches_reference(col):
    d = load("lbm_ops.npz")
    f0 = d[f"{col}_f0"].reshape(19, -1)
    solid = d["solid"].reshape(-1)
    N = f0.shape[1]
    om = float(d[f"{col}_omega"])
    orc = olbm.OracleLBM(10, 8, 6, f0, solid, collision=col, omega=om,
                         omega_minus=float(d["trt_omega_minus"]) if col == "trt" else None,
                         S=d["mrt_S"] if col == "mrt" else None, real="f64", weights=W_TORCH)
    orc.collide()
    fluid = ~solid.astype(bool)
    got = orc.fp[:, fluid]
    ref = d[f"{col}_fpost"].reshape(19, N)[:, fluid]
    # FP64 oracle against an FP32 torch result: a few FP32 ulps
    assert np.abs(got - ref).max() / np.abs(ref).max() < 1e-6


def test_stream_matches_reference_exactly():
    d = load("lbm_ops.npz")
    orc = olbm.OracleLBM(10, 8, 6, np.zeros((19, 480)), np.zeros(480), real="f32")
    src = np.ascontiguousarray(d["stream_in"].reshape(19, -1))
    out = np.empty_like(src)
    # default config: +X flow, no walls -> x non-periodic, y and z periodic
    orc.L.or_stream_pull(olbm._p(src), olbm._p(out), 10, 8, 6, 0, 1, 1)
    assert np.array_equal(out, d["stream_out"].reshape(19, -1))


def test_ibb_and_reset_match_reference_exactly():
    d = load("lbm_ops.npz")
    links = {k: d[f"ibb_{k}"] for k in ("fluid_flat", "dir_i", "dir_opp", "w_i", "w_second", "q_ge_half",
                                        "ff_flat", "ff_valid")}
    solid = d["solid"].reshape(-1)
    orc = olbm.OracleLBM(10, 8, 6, d["ibb_fstream"], solid, links=links, real="f32", weights=W_TORCH)
    fp = np.ascontiguousarray(d["ibb_fpost"].reshape(19, -1))
    k = orc.links
    orc.L.or_ibb(olbm._p(fp), olbm._p(orc.f), olbm._p(k["fluid_flat"]), olbm._p(k["dir_i"]),
                 olbm._p(k["dir_opp"]), olbm._p(k["w1"]), olbm._p(k["w2"]), olbm._p(k["ge"]),
                 olbm._p(k["ff_flat"]), olbm._p(k["ff_valid"]), len(k["fluid_flat"]), orc.N)
    orc.L.or_reset_solid(olbm._p(orc.f), olbm._p(orc.solid), orc.N)
    assert np.array_equal(orc.f, d["ibb_out"].reshape(19, -1))


@pytest.mark.parametrize("name", ["cube", "heatsink"])
def test_link_list_and_q_bit_exact(name):
    """The oracle's link list (order included) and Bouzidi weights equal the reference's bit for bit,
    in both ways of rounding (x - origin) / dx (they agree at pitch 1)."""
    from oracle import geometry as og
    d = load("ibb_links.npz")
    for mode in ("reciprocal", "divide"):
        r = og.ibb_from_sdf(d[f"{name}_solid"], d[f"{name}_phi"], 1.0, scalar_div=mode)
        for k in ("fluid_flat", "dir_i", "dir_opp", "ff_flat", "q_ge_half", "ff_valid"):
            assert np.array_equal(r[k], d[f"{name}_{k}"]), k
        for k in ("w_i", "w_second"):
            assert np.array_equal(r[k].view(np.uint32), d[f"{name}_{k}"].view(np.uint32)), k


@pytest.mark.parametrize("name", ["crop", "balls"])
def test_fractions_at_non_unit_pitch_match_reference(name):
    """Pitch 0.37 / 0.5 with a shifted origin: the oracle's CPU-rounding mode reproduces the
    reference's torch-CPU q, weights and phi exactly."""
    from oracle import geometry as og
    d = load("ibb_pitch.npz")
    pitch = float(d[f"{name}_pitch"])
    org = (d[f"{name}_voxel_origin"].astype(np.float32)
           - np.float32(pitch) * d[f"{name}_offset_ijk"].astype(np.float32))
    phi = og.signed_edt(d[f"{name}_solid"], pitch)
    assert np.array_equal(phi.view(np.uint32), d[f"{name}_phi"].view(np.uint32))
    r = og.ibb_from_sdf(d[f"{name}_solid"], d[f"{name}_phi"], pitch, org, scalar_div="divide")
    for k in ("fluid_flat", "dir_i", "dir_opp", "ff_flat", "q_ge_half", "ff_valid"):
        assert np.array_equal(r[k], d[f"{name}_{k}"]), k
    for k in ("q", "w_i", "w_second"):
        assert np.array_equal(r[k].view(np.uint32), d[f"{name}_{k}"].view(np.uint32)), k


def test_phi_from_voxels_matches_reference():
    from oracle import geometry as og
    d = load("ibb_links.npz")
    for name in ("cube", "heatsink"):
        phi = og.signed_edt(d[f"{name}_solid"])
        assert np.array_equal(phi.view(np.uint32), d[f"{name}_phi"].view(np.uint32))


def test_signed_edt_oracle_matches_scipy():
    """The separable restatement against scipy.ndimage.distance_transform_edt itself (the routine
    build_phi_from_voxel_mask_mm calls), on seeded masks, two pitches and both degenerate masks."""
    edt = pytest.importorskip("scipy.ndimage").distance_transform_edt
    from oracle import geometry as og
    rng = np.random.default_rng(5)
    masks = [rng.random(tuple(rng.integers(1, 26, size=3))) < rng.uniform(0.005, 0.7) for _ in range(10)]
    masks += [np.zeros((4, 5, 6), bool), np.ones((4, 5, 6), bool), np.zeros((1, 1, 7), bool)]
    for s in masks:
        for pitch in (1.0, 0.37):
            ref = edt(~s) * pitch
            ref[s] = -(edt(s) * pitch)[s]
            got = og.signed_edt(s, pitch)
            assert np.array_equal(got.view(np.uint32), ref.astype(np.float32).view(np.uint32)), (s.shape, pitch)


def _golden_mg():
    d = load("mg_solve.npz")
    mg = omg.OracleMG(d["k"], d["rcp"], d["u"], d["v"], d["w"], d["mask"], 0, 1, float(d["s"]), omega=0.6,
                      real=np.float64)
    mg.set_dt(float(d["dt"]))
    return d, mg


def test_mg_coefficients_match_reference():
    d, mg = _golden_mg()
    assert len(mg.levels) == int(d["nlevels"])
    for li, lv in enumerate(mg.levels):
        for key, rk in (("aE", "E"), ("aW", "W"), ("aN", "N"), ("aS", "S"), ("aU", "U"), ("aD", "D")):
            # the oracle builds from FP32 inputs as the CUDA path does; the golden ran in FP64
            assert np.allclose(lv["a"][rk], d[f"L{li}_{key}"], rtol=1e-6, atol=0), (li, key)
        assert np.array_equal(lv["mask"], d[f"L{li}_mask_f"])
        assert np.allclose(lv["inv"], d[f"L{li}_inv_diagM"], rtol=1e-6, atol=0)


def test_mg_apply_and_solves_match_reference():
    d, mg = _golden_mg()
    assert np.allclose(mg.L_apply_fine(d["T"]), d["LT"], rtol=1e-5, atol=1e-9)
    x, info = mg.solve(d["b"], None, max_cycles=6, tol=0.0)
    assert np.linalg.norm(x - d["solve_x"]) / np.linalg.norm(d["solve_x"]) < 1e-6
    assert abs(info["res_rel"] - float(d["solve_res"])) < 1e-6
    xb, ib = omg.bicgstab(mg, d["b"], None, tol=1e-9, max_it=8)
    assert ib["it"] == int(d["bicgstab_it"])
    assert np.linalg.norm(xb - d["bicgstab_x"]) / np.linalg.norm(d["bicgstab_x"]) < 1e-5


def test_voxelizer_oracle_matches_reference_grids():
    """The restated ray-parity voxelizer reproduces gpu_voxelize_mesh's grids, origins and sizes."""
    from oracle import voxelizer as ov
    d = load("voxels.npz")
    for name in ("box", "sphere", "finsink"):
        tri, pitch = d[f"{name}_tri"], float(d[f"{name}_pitch"])
        origin, dims = ov.grid(tri.reshape(-1, 3), pitch)
        assert dims == tuple(int(x) for x in d[f"{name}_dims"])
        assert np.array_equal(origin.astype(np.float64), d[f"{name}_origin"])
        want = np.unpackbits(d[f"{name}_bits"])[:np.prod(dims)].reshape(dims)
        assert np.array_equal(ov.voxelize(tri, origin, dims, pitch), want), name


def test_stl_round_trip_and_grid_helper(tmp_path):
    from fluxcore3d_gb300.pre_post import gpu_voxelizer as gv
    from fluxcore3d_gb300.pre_post import stl
    from oracle import voxelizer as ov
    m = stl.fin_heatsink_mesh()
    p = str(tmp_path / "sink.stl")
    stl.write_stl(p, m)
    r = stl.read_stl(p)
    assert np.array_equal(r.triangles, m.triangles.astype(np.float32))
    ascii_path = str(tmp_path / "tri.stl")
    with open(ascii_path, "w") as fh:
        fh.write("solid t\nfacet normal 0 0 1\nouter loop\nvertex 0 0 0\nvertex 1 0 0\nvertex 0 1 0\n"
                 "endloop\nendfacet\nendsolid t\n")
    assert stl.read_stl(ascii_path).triangles.shape == (1, 3, 3)
    o1, *d1 = gv.voxel_grid(m.vertices.astype(np.float32), 0.37)
    o2, d2 = ov.grid(m.vertices, 0.37)
    assert tuple(d1) == d2 and np.array_equal(o1, o2)


def test_tracer_oracle_matches_reference():
    from oracle import tracer as ot
    d = load("tracer.npz")
    phi = ot.inject(np.zeros(d["solid_flow"].shape, np.float32), d["inlet"])
    for it in range(25):
        s = it // 5
        if it % 7 == 6:
            phi = ot.inject(phi, d["inlet"])
        phi = ot.step(phi, d[f"u{s}"], d[f"v{s}"], d[f"w{s}"], d["solid_flow"])
        if it == 0:
            assert np.array_equal(phi.view(np.uint32), d["field1"].view(np.uint32))
    assert np.array_equal(phi.view(np.uint32), d["field25"].view(np.uint32))


def test_oracle_flux_form_equals_reference_form_in_fp64():
    """The flux form of the operator (sum_n a_n (T - T_n), what the CUDA kernels evaluate) equals the
    reference's diag*T - sum_n a_n T_n in FP64 on the golden multigrid problem: same operator."""
    d = load("mg_solve.npz")
    args = (d["k"], d["rcp"], d["u"], d["v"], d["w"], d["mask"], 0, 1, float(d["s"]))
    ref = omg.OracleMG(*args, omega=0.6, real=np.float64)
    flx = omg.OracleMG(*args, omega=0.6, real=np.float64, flux=True)
    T = np.random.default_rng(0).random(d["k"].shape) + 25.0
    for lr, lf in zip(ref.levels, flx.levels):
        Tl = T[tuple(slice(0, n) for n in lr["shape"])]
        a, b = ref.L(lr, Tl), flx.L(lf, Tl)
        assert float(np.abs(a - b).max()) <= 1e-12 * float(np.abs(a).max() + 1.0)


# ---- the reference's own plane and Smagorinsky kernels, run on the host (ref_lbm.npz) ----------

def _plane_cells(shape, axis, idx):
    i, j, k = np.meshgrid(*(np.arange(n) for n in shape), indexing="ij")
    flat = (i * shape[1] + j) * shape[2] + k
    return np.take(flat, idx, axis=axis).reshape(-1)


ZH_CASES = ("inlet_x_low", "outlet_x_high", "inlet_y_high", "outlet_y_low", "outlet_z_low", "inlet_z_low")
CV_CASES = ("x_high", "z_low", "x_high_two_blocks")


def _close(got, want, tol):
    return float(np.abs(got.astype(np.float64) - want).max()) <= tol * float(np.abs(want).max())


@pytest.mark.parametrize("case", ZH_CASES)
def test_oracle_zou_he_matches_reference_kernel(case):
    """or_zou_he (oracle/lbm_oracle.c) against lbm_zou_he_bc_kernel (solver/lbm_kernels.cu:791-969)
    run on the host: boundary plane within FP32 rounding, solid and backflow nodes included."""
    d = load("ref_lbm.npz")
    a = d[f"zh_{case}_args"]
    shape = tuple(int(x) for x in a[:3])
    axis, plane, inter, bct = (int(x) for x in a[3:7])
    uin, rout, sign = float(a[7]), float(a[8]), int(a[9])
    orc = olbm.OracleLBM(*shape, d[f"zh_{case}_in"], d["solid_%dx%dx%d" % shape])
    f = orc.f.copy()
    orc.L.or_zou_he(olbm._p(f), olbm._p(orc.solid), *shape, axis, plane, inter, bct, float(np.float32(uin)),
                    float(np.float32(rout)), sign)
    assert _close(f[:, _plane_cells(shape, axis, plane)], d[f"zh_{case}_plane"], 2e-6)


@pytest.mark.parametrize("case", CV_CASES)
def test_oracle_convective_matches_reference_kernel(case):
    """or_convective against lbm_convective_bc_reduce_kernel + lbm_convective_mass_correct_kernel
    (solver/lbm_kernels.cu:1170-1344) run on the host; the reference sums rho in FP32 with one
    atomicAdd per block, the oracle in FP64, so the plane agrees to FP32 summation order."""
    d = load("ref_lbm.npz")
    a = d[f"cv_{case}_args"]
    shape = tuple(int(x) for x in a[:3])
    axis, o, inter, ucax = (int(x) for x in a[3:7])
    rout = float(a[7])
    orc = olbm.OracleLBM(*shape, d[f"cv_{case}_in"], d["solid_%dx%dx%d" % shape])
    f = orc.f.copy()
    orc.L.or_convective(olbm._p(f), olbm._p(orc.solid), *shape, axis, o, inter, ucax, float(np.float32(rout)))
    assert _close(f[:, _plane_cells(shape, axis, o)], d[f"cv_{case}_plane"], 2e-6)


def test_oracle_mrt_smagorinsky_matches_reference_kernel():
    """Mode 3 of or_macro_collide against lbm_macro_collide_mrt_smag_kernel (solver/lbm_kernels.cu:
    1018-1117) run on the host: post-collision populations and macros within FP32 rounding."""
    d = load("ref_lbm.npz")
    shape = tuple(int(x) for x in d["smag_shape"])
    cs2, om0 = (float(x) for x in d["smag_params"])
    orc = olbm.OracleLBM(*shape, d["smag_f"], d["solid_%dx%dx%d" % shape], collision="mrt_smag", omega=om0,
                         S=d["smag_S"], Cs_dx2=float(np.float32(cs2)))
    orc.params[4] = float(np.float32(om0))
    orc.collide()
    assert _close(orc.fp, d["smag_out_fp"], 2e-6)
    for got, want in zip((orc.rho, orc.u, orc.v, orc.w), d["smag_out_macro"]):
        assert _close(got, want, 2e-6)


def test_oracle_thermal_step_matches_reference_fused_step():
    """The oracle's restatement of the pseudo-time thermal step (oracle/mg.py thermal_step) against the
    reference's own fused step (solver/thermal_cuda_ext.py:55-201 with its FP64 torch multigrid and its
    thermal kernels built for the host; thermal_steady.npz): three ramped steps, FP64."""
    d = load("thermal_steady.npz")
    k, u, src = d["k"], d["u"], d["src"].astype(np.float64)
    shape = k.shape
    mask = np.ones(shape, bool)
    mask[0] = False
    z = np.zeros(shape, np.float32)
    ref = omg.OracleMG(k, np.ones(shape, np.float32), u, z, z, mask, 0, 1, 1.0, omega=0.6, real=np.float64)
    T = np.full(shape, 25.0)
    T0 = np.full(shape, 25.0)
    dt = 5.0
    for _ in range(3):
        ref.set_dt(dt)
        T, _ = omg.thermal_step(ref, T, T0, src, mask, dt, 1e-13, 200, 0, shape[0] - 1)
        dt *= 1.5
    assert float(np.abs(T - d["T3"]).max()) < 1e-12


def test_oracle_fp32_flux_form_steady_temperature_within_1e6():
    """The steady temperature of the thermal step iterated in FP32 with the flux form (60 ramped steps,
    FP32 V-cycles) is within 1e-6 relative L2 of the reference's own FP64 steady state
    (thermal_steady.npz).  With the reference's diag form in FP32 it is ~4e-6 away: its rounded diagL
    acts as a source proportional to T ~ 25."""
    d = load("thermal_steady.npz")
    k, u, src = d["k"], d["u"], d["src"]
    shape = k.shape
    mask = np.ones(shape, np.float32)
    mask[0] = 0
    z = np.zeros(shape, np.float32)
    mg = omg.OracleMG(k, np.ones(shape, np.float32), u, z, z, mask, 0, 1, 1.0, omega=0.6, real=np.float32, flux=True)
    T = np.full(shape, 25.0, np.float32)
    T0 = np.full(shape, 25.0, np.float32)
    dt = 5.0
    for _ in range(60):
        mg.set_dt(dt)
        T, _ = omg.thermal_step(mg, T, T0, src, mask, dt, 1e-7, 100, 0, shape[0] - 1)
        dt = min(200.0, 1.5 * dt)
    Tr = d["T"]
    assert np.linalg.norm(T.astype(np.float64) - Tr) / np.linalg.norm(Tr) < 1e-6
