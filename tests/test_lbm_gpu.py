"""GPU parity of the lattice kernels against the C oracle (reference CUDA-path semantics).

Tolerances: FP32 paths must agree with the FP32 oracle within 1e-5 relative L2
on populations after the stated number of steps (the oracle differs only in
FMA contraction and division rounding); FP16/BF16 shifted storage is compared
with the FP64 oracle and must stay within 1e-3 relative error on velocity.
"""
import numpy as np
import pytest
import torch

from fluxcore3d_gb300 import case as cases
from fluxcore3d_gb300.solver.lbm_cuda_ext import LBM_CUDA, LBMCUDAUpgrade
from oracle.lbm import OracleLBM

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def oracle_for(sim, real="f32"):
    cfg = sim.cfg
    links = None
    if sim.ibb_data is not None and sim.ibb_data.n_links > 0:
        d = sim.ibb_data
        links = {k: getattr(d, k).cpu().numpy() for k in
                 ("fluid_flat", "dir_i", "dir_opp", "w_i", "w_second", "q_ge_half", "ff_flat", "ff_valid")}
    sigma = sim._sponge_sigma.cpu().numpy() if getattr(cfg, "sponge_length", 0) > 0 else None
    om_minus = float(sim.omega_minus) if hasattr(sim, "omega_minus") else None
    S = sim._mrt_S.cpu().numpy() if hasattr(sim, "_mrt_S") else None
    return OracleLBM(sim.nx, sim.ny, sim.nz, sim.f.cpu().numpy(), sim.solid_flow.cpu().numpy(),
                     collision=cfg.collision, omega=float(sim.omega_plus), omega_minus=om_minus, S=S,
                     Cs_dx2=cfg.smag_Cs ** 2, sigma=sigma, links=links, flow_dir=cfg.flow_dir,
                     domain_walls=cfg.domain_walls, domain_outlets=cfg.domain_outlets,
                     transverse_walls=cfg.transverse_walls, u_in_lat=sim.u_in_lat,
                     rho_out_lat=cfg.rho_out_lat, u_lat_max=cfg.u_lat_max,
                     outlet_bc_mode=cfg.outlet_bc_mode, real=real)


def run_pair(sim, steps, real="f32"):
    orc = oracle_for(sim, real)
    LBMCUDAUpgrade.patch(sim)
    for _ in range(steps):
        sim.step(do_thermal=False)
    sim.sync_f()
    torch.cuda.synchronize()
    orc.step(steps)
    assert sim._fc.check_device_error() == 0
    return orc


@pytest.mark.parametrize("collision", ["bgk", "trt", "mrt", "mrt_smag"])
def test_fused_step_fp32_matches_oracle_small(cuda, collision):
    sim = cases.channel_cube(device=cuda, collision=collision, nx=32, ny=16, nz=16, cube=6, cube_x=10,
                             sponge_length=8, outlet="pressure")
    orc = run_pair(sim, 200)
    N = sim.nx * sim.ny * sim.nz
    e = rel_l2(sim.f.reshape(19, N).cpu().numpy(), orc.f)
    assert e < 1e-5, e
    assert rel_l2(sim.u.reshape(-1).cpu().numpy(), orc.u) < 1e-4
    assert rel_l2(sim.rho.reshape(-1).cpu().numpy(), orc.rho) < 1e-5


@pytest.mark.parametrize("storage,cpt,staging", [("fp32", 1, "tma"), ("fp16", 1, "tma"), ("bf16", 1, "tma"),
                                                 ("fp16", 1, "direct"), ("fp32", 2, "direct"),
                                                 ("bf16", 2, "direct")])
def test_pin_fin_all_link_modes(cuda, storage, cpt, staging):
    """Small pin-fin heat sink with analytic link fractions: q >= 1/2, q < 1/2 with a second
    fluid node, and q < 1/2 without one all occur; MRT, pressure outlet, sponge.  nz = 48 is
    a partial 32-cell chunk per row for the TMA-staged pass."""
    sim = cases.pin_fin(device=cuda, collision="mrt", storage=storage, nx=48, ny=32, nz=48,
                        n_pins=(3, 2), radius=3.5, height=24, base=4, sponge_length=8)
    sim.cfg.lbm_cells_per_thread = cpt
    sim.cfg.lbm_staging = staging
    d = sim.ibb_data
    ge, fv = d.q_ge_half.bool(), d.ff_valid.bool()
    assert bool(ge.any()) and bool((~ge & fv).any())
    orc = run_pair(sim, 200, real="f32" if storage == "fp32" else "f64")
    N = sim.nx * sim.ny * sim.nz
    e = rel_l2(sim.f.reshape(19, N).cpu().numpy(), orc.f)
    assert e < {"fp32": 1e-5, "fp16": 2e-4, "bf16": 2e-3}[storage], e


def periodic_box(cuda, collision, storage, nx=40, ny=20, nz=32):
    """Cube with IBB links in a box periodic along y and z (no walls): fluid cells sit on every
    k and j boundary, so the staged pass wraps rows inside its tiles and the edge rows take
    the direct path; ny = 20 leaves a partial last tile."""
    from fluxcore3d_gb300 import geometry as geo
    from fluxcore3d_gb300.case import CaseConfig, LatticeCase, stamp_walls
    cfg = CaseConfig(nx=nx, ny=ny, nz=nz, collision=collision, lbm_storage=storage, domain_walls=[],
                     outlet_bc_mode="pressure", sponge_length=6)
    solid = geo.cube_mask((nx, ny, nz), (14, ny // 2, nz // 2), (6, 6, 6), device=cuda)
    ibb = geo.ibb_from_voxels(solid)
    return LatticeCase(cfg, 0.05, 0.05 * 6 / 50, solid, stamp_walls(cfg, solid), ibb, device=cuda, seed=0)


@pytest.mark.parametrize("collision", ["trt", "mrt"])
def test_staged_pass_periodic_box_matches_oracle(cuda, collision):
    sim = periodic_box(cuda, collision, "fp32")
    sim.cfg.lbm_staging = "tma"
    orc = run_pair(sim, 150)
    N = sim.nx * sim.ny * sim.nz
    assert rel_l2(sim.f.reshape(19, N).cpu().numpy(), orc.f) < 1e-5


@pytest.mark.parametrize("storage,collision", [("fp16", "mrt"), ("fp32", "trt"), ("bf16", "mrt_smag"),
                                               ("fp16", "bgk")])
def test_staged_pass_bit_identical_to_direct(cuda, storage, collision):
    """The TMA-staged and the direct main pass run the same per-cell arithmetic on the same
    values, so their populations and macros agree bit for bit."""
    out = {}
    for staging in ("tma", "direct"):
        sim = periodic_box(cuda, collision, storage)
        sim.cfg.lbm_staging = staging
        LBMCUDAUpgrade.patch(sim)
        for _ in range(60):
            sim.step(do_thermal=False)
        torch.cuda.synchronize()
        assert sim._fc.check_device_error() == 0
        P = sim._fc.P[sim._fc.cur]
        out[staging] = (P.view(torch.uint8).cpu().numpy(), P.float().cpu().numpy(), sim.rho.cpu().numpy(),
                        sim.u.cpu().numpy())
    assert np.array_equal(out["tma"][0], out["direct"][0]), \
        float(np.abs(out["tma"][1].astype(np.float64) - out["direct"][1]).max())
    for a, b in zip(out["tma"][2:], out["direct"][2:]):
        assert np.array_equal(a, b), float(np.abs(a.astype(np.float64) - b.astype(np.float64)).max())


@pytest.mark.parametrize("storage,nz", [("fp16", 288), ("fp32", 320), ("bf16", 512)])
def test_staged_pass_long_rows_bit_identical_to_direct(cuda, storage, nz):
    """Rows longer than one TMA box (256 elements) are staged as 2 segments through a 5-D tensor
    map; the staged pass must still be taken (tile records exist) and agree with the direct pass
    bit for bit, links, periodic z wrap and partial tiles included."""
    out = {}
    for staging in ("tma", "direct"):
        sim = periodic_box(cuda, "mrt", storage, nx=24, ny=6, nz=nz)
        sim.cfg.lbm_staging = staging
        LBMCUDAUpgrade.patch(sim)
        if staging == "tma":
            assert sim._fc.tile_links is not None
        for _ in range(30):
            sim.step(do_thermal=False)
        torch.cuda.synchronize()
        assert sim._fc.check_device_error() == 0
        P = sim._fc.P[sim._fc.cur]
        out[staging] = (P.view(torch.uint8).cpu().numpy(), sim.rho.cpu().numpy(), sim.u.cpu().numpy())
    for a, b in zip(out["tma"], out["direct"]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("flow_dir,shape,storage", [("+X", (40, 16, 64), "fp16"), ("+Z", (20, 16, 64), "bf16"),
                                                    ("+Y", (24, 20, 32), "fp32"), ("-X", (30, 8, 64), "fp16"),
                                                    ("+X", (40, 16, 32), "bf16")])
def test_staged_pass_wrapped_edges_bit_identical_to_direct(cuda, flow_dir, shape, storage):
    """Periodic axes staged by the tensor copies themselves: the plane coordinate of a periodic x
    wraps, and with full tiles whose rows keep 128-byte alignment the first and last tile of each
    plane load the periodic y wrap as a box of tj - 1 rows plus a one-row box (no direct loads for
    those rows); other shapes keep the direct-load path for the edge rows.  Bit for bit the same as
    the direct pass, links included."""
    from fluxcore3d_gb300 import geometry as geo
    from fluxcore3d_gb300.case import CaseConfig, LatticeCase, stamp_walls
    nx, ny, nz = shape
    out = {}
    for staging in ("tma", "direct"):
        cfg = CaseConfig(nx=nx, ny=ny, nz=nz, flow_dir=flow_dir, collision="mrt", lbm_storage=storage,
                         domain_walls=[], outlet_bc_mode="pressure")
        solid = geo.cube_mask(shape, (nx // 2, ny // 2, nz // 2), (6, 6, 6), device=cuda)
        sim = LatticeCase(cfg, 0.05, 0.05 * 6 / 50, solid, stamp_walls(cfg, solid), geo.ibb_from_voxels(solid),
                          device=cuda, seed=0)
        sim.cfg.lbm_staging = staging
        LBMCUDAUpgrade.patch(sim)
        if staging == "tma":
            assert sim._fc.tile_links is not None
        for _ in range(40):
            sim.step(do_thermal=False)
        torch.cuda.synchronize()
        assert sim._fc.check_device_error() == 0
        P = sim._fc.P[sim._fc.cur]
        out[staging] = (P.view(torch.uint8).cpu().numpy(), sim.rho.cpu().numpy(), sim.u.cpu().numpy())
    for a, b in zip(out["tma"], out["direct"]):
        assert np.array_equal(a, b)


def test_fused_planes_and_concurrent_gather_bit_identical(cuda, monkeypatch):
    """Fused Zou/He + collision of the inlet/outlet planes (one launch) and the next step's link
    gather on a second stream give the same bits as the reference-order plane sequence with the
    gather inside the step."""
    from fluxcore3d_gb300.solver.fused_lbm import FusedLBM
    out = {}
    for mode in ("fused", "sequential"):
        sim = cases.pin_fin(device=cuda, collision="mrt", storage="fp16", nx=48, ny=32, nz=48,
                            n_pins=(3, 2), radius=3.5, height=24, base=4, sponge_length=8)
        if mode == "sequential":
            monkeypatch.setattr(FusedLBM, "_plane_set", lambda self: None)
        LBMCUDAUpgrade.patch(sim)
        if mode == "sequential":
            sim._fc.concurrent_gather = False
        else:
            assert sim._fc.concurrent_gather and sim._fc._plane_set() is not None
        for _ in range(40):
            sim.step(do_thermal=False)
        sim.sync_f()
        torch.cuda.synchronize()
        assert sim._fc.check_device_error() == 0
        P = sim._fc.P[sim._fc.cur]
        out[mode] = (P.view(torch.uint8).cpu().numpy(), sim.f.cpu().numpy(), sim.rho.cpu().numpy())
        monkeypatch.undo()
    for a, b in zip(out["fused"], out["sequential"]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("concurrent", [True, False])
def test_alternating_tile_and_gather_order_bit_identical(cuda, concurrent):
    """The staged pass alternates its tile order every step and each link gather runs opposite to
    the pass that wrote its input; the populations, plane states and macros are the same bits as
    with every pass and gather in ascending order (links, sponge and inlet/outlet planes included)."""
    out = {}
    for alt in (True, False):
        sim = cases.pin_fin(device=cuda, collision="mrt", storage="fp16", nx=48, ny=32, nz=48,
                            n_pins=(3, 2), radius=3.5, height=24, base=4, sponge_length=8)
        LBMCUDAUpgrade.patch(sim)
        sim._fc.alternate_order = alt
        sim._fc.concurrent_gather = concurrent and sim._fc.concurrent_gather
        assert sim._fc.tile_links is not None
        for _ in range(41):
            sim.step(do_thermal=False)
        sim.sync_f()
        torch.cuda.synchronize()
        assert sim._fc.check_device_error() == 0
        P = sim._fc.P[sim._fc.cur]
        out[alt] = (P.view(torch.uint8).cpu().numpy(), sim.f.cpu().numpy(), sim.rho.cpu().numpy(),
                    sim.u.cpu().numpy())
    for a, b in zip(out[True], out[False]):
        assert np.array_equal(a, b)


def test_bounded_mbarrier_wait_times_out_and_context_survives(cuda):
    """Failure detection without a GPU fault: the staged pass's bounded mbarrier wait gives up
    when nothing arrives and reports the timeout bit (4) to the host; with an arrival it completes;
    the context stays usable (a lattice step runs and matches the oracle afterwards)."""
    from fluxcore3d_gb300 import _lib
    from fluxcore3d_gb300._torch import ptr, stream_ptr
    status = torch.zeros(1, dtype=torch.int32, device=cuda)
    _lib.call("fc_lbm_wait_selftest", 1024, 0, ptr(status), stream_ptr())
    torch.cuda.synchronize()
    assert int(status.item()) == 4
    status.zero_()
    _lib.call("fc_lbm_wait_selftest", 1024, 1, ptr(status), stream_ptr())
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    sim = cases.channel_cube(device=cuda, collision="bgk", nx=24, ny=12, nz=10, cube=4, cube_x=8,
                             outlet="pressure")
    orc = run_pair(sim, 20)
    N = sim.nx * sim.ny * sim.nz
    assert rel_l2(sim.f.reshape(19, N).cpu().numpy(), orc.f) < 1e-5


def test_fused_step_c1_channel_1000_steps(cuda):
    """Plain method, small channel (64x32x32, BGK FP32, convective outlet, cube IBB): 1000 steps."""
    sim = cases.channel_cube(device=cuda, collision="bgk")
    orc = run_pair(sim, 1000)
    N = sim.nx * sim.ny * sim.nz
    e = rel_l2(sim.f.reshape(19, N).cpu().numpy(), orc.f)
    assert e < 1e-5, e


def test_fused_step_separate_link_pass_matches(cuda):
    """The two-pass variant (link cells in their own kernel) gives the same result."""
    sim = cases.channel_cube(device=cuda, collision="mrt", nx=32, ny=16, nz=16, cube=6, cube_x=10,
                             sponge_length=8, outlet="pressure")
    sim.cfg.lbm_link_pass = "separate"
    orc = run_pair(sim, 100)
    N = sim.nx * sim.ny * sim.nz
    assert rel_l2(sim.f.reshape(19, N).cpu().numpy(), orc.f) < 1e-5


def test_fused_step_no_links_periodic(cuda):
    """No IBB links: flow-solid cells act through the in-cell swap; two periodic axes."""
    sim = cases.channel_cube(device=cuda, collision="mrt", nx=24, ny=12, nz=10, cube=4, cube_x=8,
                             with_links=False, outlet="pressure")
    sim.cfg.domain_walls = []
    orc = run_pair(sim, 100)
    N = sim.nx * sim.ny * sim.nz
    assert rel_l2(sim.f.reshape(19, N).cpu().numpy(), orc.f) < 1e-5


def test_fused_step_convective_and_macro_lag(cuda):
    sim = cases.channel_cube(device=cuda, collision="trt", nx=32, ny=12, nz=12, cube=4, cube_x=10)
    orc = run_pair(sim, 50)
    # macros after step k are those of the step's input state (reference semantics)
    assert rel_l2(sim.v.reshape(-1).cpu().numpy(), orc.v) < 1e-4
    assert rel_l2(sim.rho.reshape(-1).cpu().numpy(), orc.rho) < 1e-5


@pytest.mark.parametrize("storage", ["fp16", "bf16"])
def test_shifted_storage_vs_fp64(cuda, storage):
    sim = cases.channel_cube(device=cuda, collision="mrt", storage=storage, nx=48, ny=16, nz=16, cube=6,
                             cube_x=14, outlet="pressure", sponge_length=8)
    orc = run_pair(sim, 300, real="f64")
    u_ref = orc.u
    err = np.abs(sim.u.reshape(-1).cpu().numpy() - u_ref).max() / np.abs(u_ref).max()
    tol = 1e-3 if storage == "fp16" else 2e-2
    assert err < tol, err


def test_per_op_kernels_match_oracle(cuda):
    """The LBM_CUDA per-operation surface reproduces one oracle step op by op."""
    sim = cases.channel_cube(device=cuda, collision="mrt", nx=20, ny=10, nz=10, cube=4, cube_x=6,
                             sponge_length=6, outlet="pressure")
    orc = oracle_for(sim)
    LBMCUDAUpgrade.patch(sim)
    for _ in range(5):
        LBMCUDAUpgrade._step_unfused(sim)
    torch.cuda.synchronize()
    orc.step(5)
    N = sim.nx * sim.ny * sim.nz
    assert rel_l2(sim.f.reshape(19, N).cpu().numpy(), orc.f) < 1e-6
    # and the fused engine picks up from the unfused state
    for _ in range(5):
        sim.step(do_thermal=False)
    sim.sync_f()
    orc.step(5)
    assert rel_l2(sim.f.reshape(19, N).cpu().numpy(), orc.f) < 1e-6


def test_stream_pull_exact(cuda):
    nx, ny, nz = 7, 5, 6
    g = torch.Generator().manual_seed(3)
    f = torch.rand((19, nx * ny * nz), generator=g).to(cuda)
    out = torch.empty_like(f)
    LBM_CUDA.stream_pull(f, out, nx, ny, nz, 0, 1, 0)
    orc = OracleLBM(nx, ny, nz, np.zeros((19, nx * ny * nz)), np.zeros(nx * ny * nz), real="f32")
    fo = np.empty((19, nx * ny * nz), np.float32)
    from oracle.lbm import _p
    src = np.ascontiguousarray(f.cpu().numpy())
    orc.L.or_stream_pull(_p(src), _p(fo), nx, ny, nz, 0, 1, 0)
    assert np.array_equal(out.cpu().numpy(), fo)


def test_argument_errors_raise(cuda):
    f = torch.zeros((19, 8), device=cuda)
    with pytest.raises(RuntimeError):
        LBM_CUDA.stream_pull(f, f.t().contiguous().t(), 2, 2, 2, 0, 0, 0)
    with pytest.raises(RuntimeError):
        LBM_CUDA.macro_collide_mrt(f, f.clone(), torch.zeros(8, device=cuda), torch.zeros(8, device=cuda),
                                   torch.zeros(8, device=cuda), torch.zeros(8, device=cuda),
                                   torch.zeros(8, dtype=torch.uint8, device=cuda), torch.zeros(5, device=cuda))


def test_gyroid_trt_fp32_matches_oracle(cuda):
    """Reduced gyroid (48x24x32, L = 12, linear-interpolation link fractions), TRT with magic
    parameter 1/4 at FP32 storage: 200 steps of the fused engine against the FP32 oracle."""
    sim = cases.gyroid(device=cuda, storage="fp32", nx=48, ny=24, nz=32, L=12.0)
    orc = run_pair(sim, 200)
    N = sim.nx * sim.ny * sim.nz
    assert rel_l2(sim.f.reshape(19, N).cpu().numpy(), orc.f) < 1e-5


def _fp64_gate(cuda, make, steps):
    """Storage runs of the fused engine against the device FP64 run of the plain method from the
    same initial state: velocity rel. L2 over fluid cells and the temperature of each velocity field
    (the thermal system of the heat-sink benchmarks, solved to a 1e-10 FP64 residual) in max norm."""
    from fluxcore3d_gb300 import thermal_bench
    from fluxcore3d_gb300.lattice64 import Lattice64
    from fluxcore3d_gb300.solver import mg_pcg
    ref = make("fp32")
    lat = Lattice64(ref)
    lat.step(steps)
    lat.check()
    shape = (ref.nx, ref.ny, ref.nz)
    fluid = ~ref.solid_flow.reshape(-1)
    c = torch.tensor(cases.geo.C_NP, dtype=torch.float64, device=cuda)
    vel = {"fp64": lat.velocity()}
    for storage in ("fp16", "bf16"):
        sim = make(storage)
        LBMCUDAUpgrade.patch(sim)
        for _ in range(steps):
            sim.step(do_thermal=False)
        sim.sync_f()
        assert sim._fc.check_device_error() == 0
        f = sim.f.reshape(19, -1).double()
        vel[storage] = (c.t() @ f) / f.sum(0)
    T = {}
    for name, u in vel.items():
        uu = u.to(torch.float32).reshape((3,) + shape)
        mg, b = thermal_bench.thermal_system(ref, uu[0], uu[1], uu[2])
        x, info = mg_pcg.bicgstab_mg_f64(mg, b, tol=1e-10, max_it=600)
        assert info["converged"]
        T[name] = x.double()
    out = {}
    for s in ("fp16", "bf16"):
        out[s] = (float(torch.linalg.norm((vel[s] - vel["fp64"])[:, fluid]) / torch.linalg.norm(vel["fp64"][:, fluid])),
                  float((T[s] - T["fp64"]).abs().max() / T["fp64"].abs().max()))
    return out


def test_pin_fin_fp16_bf16_gate_against_fp64(cuda):
    """FP16/BF16 shifted storage on a reduced pin fin (128x64x64, 8x4 pins r = 3.5, h = 40, MRT with
    the Smagorinsky model, Re = 200, u = 0.08) after 4000 steps against the FP64 run: FP16
    temperature error <= 1e-3 (max norm, the brief's target) and velocity <= 3e-3 rel. L2; BF16 (8
    significant bits against FP16's 11) is held to 1e-2 on temperature and 5e-2 on velocity."""
    def make(storage):
        return cases.pin_fin(device=cuda, storage=storage, collision="mrt_smag", nx=128, ny=64, nz=64, n_pins=(8, 4),
                             height=40, base=4, sponge_length=20)
    err = _fp64_gate(cuda, make, 4000)
    assert err["fp16"][1] <= 1e-3 and err["fp16"][0] <= 3e-3, err
    assert err["bf16"][1] <= 1e-2 and err["bf16"][0] <= 5e-2, err


def test_gyroid_trt_fp16_bf16_error_against_fp64(cuda):
    """The reduced gyroid (96x48x48, L = 24, TRT, tau = 0.545) at its steady state (4000 steps; the
    FP64 velocity changes by < 3e-6 per 2000 steps beyond) against the FP64 run.  Measured: FP16
    velocity 5.9e-3 rel. L2 and temperature 2.1e-3 in max norm (the FP16 rounding of f - w_q settles
    into a fixed bias near tau = 1/2), BF16 4.1e-2 and 1.2e-2; held to 1.5x those."""
    def make(storage):
        return cases.gyroid(device=cuda, storage=storage, nx=96, ny=48, nz=48, L=24.0)
    err = _fp64_gate(cuda, make, 4000)
    assert err["fp16"][1] <= 3.2e-3 and err["fp16"][0] <= 9e-3, err
    assert err["bf16"][1] <= 1.8e-2 and err["bf16"][0] <= 6.2e-2, err
