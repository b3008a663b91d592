"""GPU parity of the multigrid / Krylov / thermal kernels against the numpy oracle.

Tolerances: operator coefficients and single V-cycles within 1e-6 relative
(FP32, different summation order in the 2x2x2 mean); multi-cycle solves within
1e-5; FP64-certified Krylov solvers must reach a 1e-8 true relative residual.
"""
import numpy as np
import pytest
import torch

from fluxcore3d_gb300.solver.nlevel_mg_cuda import NLevelGeometricMGSolver
from fluxcore3d_gb300.solver import mg_pcg
from fluxcore3d_gb300.solver.mg_cuda_ext import MG_CUDA
from fluxcore3d_gb300.solver.thermal_cuda_ext import THERMAL_CUDA
from oracle import mg as omg

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def problem(shape=(32, 16, 16), ax=0, sign=1, seed=0, kratio=200.0):
    rng = np.random.default_rng(seed)
    k = np.where(rng.random(shape) < 0.3, kratio, 1.0).astype(np.float32) * 0.005
    rcp = np.where(rng.random(shape) < 0.5, 1.0, 2.0).astype(np.float32)
    u = (rng.random(shape) * 0.05).astype(np.float32)
    v = ((rng.random(shape) - 0.5) * 0.02).astype(np.float32)
    w = ((rng.random(shape) - 0.5) * 0.02).astype(np.float32)
    mask = np.ones(shape, bool)
    sl = [slice(None)] * 3
    sl[ax] = 0 if sign > 0 else -1
    mask[tuple(sl)] = False
    b = (rng.random(shape) * mask).astype(np.float32)
    return k, rcp, u, v, w, mask, b


def both(prob, ax=0, sign=1, dt=3.0, s=1.0, **kw):
    k, rcp, u, v, w, mask, b = prob
    dev = torch.device("cuda")
    mg = NLevelGeometricMGSolver(dev, torch.float32, ax, sign, s, omega=0.6, **kw)
    T = lambda a: torch.tensor(a, device=dev)
    mg.build_if_needed(T(k), T(rcp), T(u), T(v), T(w), T(mask), dt)
    ref = omg.OracleMG(k, rcp, u, v, w, mask, ax, sign, s, omega=0.6, real=np.float32, flux=True, **kw)
    ref.set_dt(dt)
    return mg, ref


@pytest.mark.parametrize("ax,sign", [(0, 1), (1, -1), (2, 1)])
def test_coefficients_and_hierarchy(cuda, ax, sign):
    prob = problem((24, 20, 16), ax, sign)
    mg, ref = both(prob, ax, sign)
    assert len(mg._levels) == len(ref.levels)
    for lg, lr in zip(mg._levels, ref.levels):
        for key, rk in (("aE", "E"), ("aW", "W"), ("aN", "N"), ("aS", "S"), ("aU", "U"), ("aD", "D")):
            assert rel(lg[key].cpu().numpy(), lr["a"][rk]) < 1e-6, key
        assert rel(lg["diagL"].cpu().numpy(), lr["diag"]) < 1e-6
        assert np.array_equal(lg["mask_f"].cpu().numpy(), lr["mask"])
        assert rel(lg["inv_diagM"].cpu().numpy(), lr["inv"]) < 1e-6


def test_mop_jacobi_and_L_apply(cuda):
    prob = problem()
    mg, ref = both(prob)
    lv = mg._levels[0]
    rng = np.random.default_rng(1)
    T = rng.random(lv["shape"]).astype(np.float32)
    Tt = torch.tensor(T, device="cuda")
    Lo = torch.empty_like(Tt)
    MG_CUDA.mop_fused(Tt, lv["aE"], lv["aW"], lv["aN"], lv["aS"], lv["aU"], lv["aD"], lv["diagL"], Lo,
                      mg._dt_cache, 0, lv["out_idx"])
    assert rel(Lo.cpu().numpy(), ref.mop(ref.levels[0], T)) < 1e-6
    assert rel(mg.L_apply_fine(Tt).cpu().numpy(), ref.L_apply_fine(T)) < 1e-5
    x = Tt.clone()
    b = torch.ones_like(x)
    MG_CUDA.jacobi_smooth(x, b, Lo, lv["inv_diagM"])
    xr = T + ref.levels[0]["inv"] * (1.0 - ref.mop(ref.levels[0], T))
    assert rel(x.cpu().numpy(), xr) < 1e-6


@pytest.mark.parametrize("shape", [(32, 16, 16), (40, 24, 20)])
def test_vcycle_solve_matches_oracle(cuda, shape):
    prob = problem(shape)
    mg, ref = both(prob)
    b = prob[-1]
    x, info = mg.solve(torch.tensor(b, device="cuda"), None, max_cycles=8, tol=0.0)
    xr, ir = ref.solve(b, None, max_cycles=8, tol=0.0)
    assert rel(x.cpu().numpy(), xr) < 1e-5
    assert abs(info["res_rel"] - ir["res_rel"]) < 1e-5 * max(1.0, ir["res_rel"])
    assert info["it"] == ir["it"] == 8


@pytest.mark.parametrize("ax,sign", [(0, 1), (2, -1)])
def test_coarse_fp64_solve_is_exact(cuda, ax, sign):
    """coarse_solve='fp64': the coarsest level's FP64 inverse applied to a right-hand side equals the
    exact FP64 solution of A x = b on the cells with mask 1 (numpy dense solve of the oracle's
    flux-form operator), within the FP32 rounding of the output."""
    prob = problem((32, 24, 20), ax, sign, seed=3)
    mg, ref = both(prob, ax, sign, coarse_solve="fp64")
    lv, lr = mg._levels[-1], ref.levels[-1]
    assert lv["mask_f"].numel() == 8 * 6 * 5
    rng = np.random.default_rng(4)
    b = rng.random(lv["shape"]).astype(np.float32)
    lv["b_buf"].copy_(torch.tensor(b, device="cuda"))
    lr["b"] = b.astype(np.float64)
    mg._vcycle(len(mg._levels) - 1, zero_guess=True)
    xr = ref.coarse_exact(lr)
    got = lv["x"].cpu().numpy()
    assert rel(got, xr) < 1e-6
    assert np.all(got[lr["mask"] == 0] == 0)


def test_vcycle_fp64_coarse_matches_oracle_and_converges_no_slower(cuda):
    """Six V-cycles with the exact FP64 coarse solve match the oracle's, and reach a residual no
    larger than the reference's 20 FP32 Jacobi sweeps on the coarsest level."""
    prob = problem((40, 24, 20), seed=5)
    mg, ref = both(prob, coarse_solve="fp64")
    b = prob[-1]
    x, info = mg.solve(torch.tensor(b, device="cuda"), None, max_cycles=6, tol=0.0)
    xr, ir = ref.solve(b, None, max_cycles=6, tol=0.0)
    assert rel(x.cpu().numpy(), xr) < 1e-5
    mj, _ = both(prob)
    _, ij = mj.solve(torch.tensor(b, device="cuda"), None, max_cycles=6, tol=0.0)
    assert info["res_rel"] <= ij["res_rel"] * (1 + 1e-4)


@pytest.mark.parametrize("shape,from_zero", [((24, 16, 16), False), ((24, 16, 16), True), ((12, 8, 8), True),
                                              ((10, 6, 4), False)])
def test_small_level_smoother_equals_sweep_sequence(cuda, shape, from_zero):
    """fc_mg_smooth_small (all sweeps in one CTA) gives the same bits as fc_mg_smooth_from_zero +
    fc_mg_smooth launched once per sweep."""
    from fluxcore3d_gb300 import _lib
    from fluxcore3d_gb300._torch import ptr, stream_ptr
    prob = problem(shape)
    mg, _ = both(prob)
    lv = mg._levels[0]
    nx, ny, nz = lv["shape"]
    rng = np.random.default_rng(5)
    x0 = torch.tensor(rng.random(lv["shape"]).astype(np.float32), device="cuda")
    lv["b_buf"].copy_(torch.tensor(prob[-1], device="cuda"))
    cp = mg._cptrs(lv)
    dt = float(mg._dt_cache)
    n = 7
    xa = x0.clone()
    _lib.call("fc_mg_smooth_small", ptr(xa), ptr(lv["b_buf"]), ptr(lv["inv_diagM"]), *cp, dt, nx, ny, nz, mg.ax,
              lv["out_idx"], n, int(from_zero), stream_ptr())
    cur, alt = x0.clone(), torch.empty_like(x0)
    start = 0
    if from_zero:
        _lib.call("fc_mg_smooth_from_zero", ptr(alt), ptr(lv["b_buf"]), ptr(lv["inv_diagM"]), cur.numel(),
                  stream_ptr())
        cur, alt = alt, cur
        start = 1
    for _ in range(start, n):
        _lib.call("fc_mg_smooth", ptr(cur), ptr(alt), ptr(lv["b_buf"]), ptr(lv["inv_diagM"]), *cp, dt, nx, ny, nz,
                  mg.ax, lv["out_idx"], stream_ptr())
        cur, alt = alt, cur
    torch.cuda.synchronize()
    assert np.array_equal(xa.cpu().numpy(), cur.cpu().numpy())


def test_first_two_sweeps_fused(cuda):
    """fc_mg_smooth_first2 equals fc_mg_smooth_from_zero followed by one fc_mg_smooth (same
    arithmetic; FMA contraction may differ, so within a few FP32 ulps)."""
    from fluxcore3d_gb300 import _lib
    from fluxcore3d_gb300._torch import ptr, stream_ptr
    prob = problem((40, 24, 20))
    mg, _ = both(prob)
    lv = mg._levels[0]
    nx, ny, nz = lv["shape"]
    lv["b_buf"].copy_(torch.tensor(prob[-1], device="cuda"))
    cp = mg._cptrs(lv)
    dt = float(mg._dt_cache)
    fused = torch.empty_like(lv["x"])
    _lib.call("fc_mg_smooth_first2", ptr(fused), ptr(lv["b_buf"]), ptr(lv["inv_diagM"]), *cp, dt, nx, ny, nz,
              mg.ax, lv["out_idx"], stream_ptr())
    x1, x2 = torch.empty_like(fused), torch.empty_like(fused)
    _lib.call("fc_mg_smooth_from_zero", ptr(x1), ptr(lv["b_buf"]), ptr(lv["inv_diagM"]), x1.numel(), stream_ptr())
    _lib.call("fc_mg_smooth", ptr(x1), ptr(x2), ptr(lv["b_buf"]), ptr(lv["inv_diagM"]), *cp, dt, nx, ny, nz,
              mg.ax, lv["out_idx"], stream_ptr())
    torch.cuda.synchronize()
    assert rel(fused.cpu().numpy(), x2.cpu().numpy()) < 1e-6


def test_bicgstab_and_pcg_dropins_match_oracle(cuda):
    prob = problem()
    mg, ref = both(prob)
    b = torch.tensor(prob[-1], device="cuda")
    x, info = mg_pcg.bicgstab_mg(mg, b, None, tol=1e-5, max_it=12)
    xr, ir = omg.bicgstab(ref, prob[-1], None, tol=1e-5, max_it=12)
    assert info["it"] == ir["it"]
    assert rel(x.cpu().numpy(), xr) < 1e-4
    x2, i2 = mg_pcg.pcg_mg(mg, b, None, tol=1e-3, max_it=10)
    assert np.isfinite(x2.cpu().numpy()).all()


def test_certified_solvers_reach_1e8(cuda):
    prob = problem((48, 24, 24))
    mg, ref = both(prob)
    b = torch.tensor(prob[-1], device="cuda")
    x, info = mg_pcg.bicgstab_mg_f64(mg, b, tol=1e-8, max_it=200)
    assert info["converged"], info
    assert omg.true_residual(ref, x.cpu().numpy(), prob[-1]) < 2e-8
    x2, i2 = mg_pcg.fgmres_mg_f64(mg, b, tol=1e-8, max_it=200, restart=30)
    assert i2["converged"], i2
    assert omg.true_residual(ref, x2.cpu().numpy(), prob[-1]) < 2e-8
    x3, i3 = mg_pcg.bicgstab_mg_mixed(mg, b, tol=1e-8, max_it=300)
    assert i3["converged"] and i3["outer"] >= 2, i3
    assert omg.true_residual(ref, x3.cpu().numpy(), prob[-1]) < 2e-8


def test_thermal_kernels(cuda):
    rng = np.random.default_rng(3)
    shape = (12, 10, 8)
    T0 = rng.random(shape).astype(np.float32)
    th = rng.random(shape).astype(np.float32)
    d = lambda a: torch.tensor(a, device="cuda")
    for ax, out_idx in ((0, 11), (0, 0), (1, 9), (2, 0)):
        Tn = THERMAL_CUDA.thermal_reconstruct(d(T0), d(th), *shape, ax, out_idx).cpu().numpy()
        ref = T0 + th
        val = ref.copy()
        nx, ny, nz = shape
        for i in range(nx):
            for j in range(ny):
                for k in range(nz):
                    s = None
                    if i == nx - 1:
                        s = (i - 1, j, k)
                    elif i == 0 and (ax != 0 or out_idx == 0):
                        s = (1, j, k)
                    elif j == ny - 1:
                        s = (i, j - 1, k)
                    elif j == 0 and (ax != 1 or out_idx == 0):
                        s = (i, 1, k)
                    elif k == nz - 1:
                        s = (i, j, k - 1)
                    elif k == 0 and (ax != 2 or out_idx == 0):
                        s = (i, j, 1)
                    if s is not None:
                        val[i, j, k] = ref[s]
        assert np.array_equal(Tn, val)
    To = rng.random(shape).astype(np.float32)
    solid = (rng.random(shape) < 0.3).astype(np.uint8)
    rs, rf = THERMAL_CUDA.convergence_metrics(d(T0), d(To), d(solid))
    dT = np.abs(T0 - To)
    assert float(rs) == dT[solid == 1].max() and float(rf) == dT[solid == 0].max()
    flag = THERMAL_CUDA.physics_check(d(T0), 0.0, 0.5)
    assert int(flag) == 1
    assert int(THERMAL_CUDA.physics_check(d(T0), -1.0, 2.0)) == 0


def test_thermal_pseudo_time_steps_match_oracle(cuda):
    """Three fused pseudo-time steps (_temperature_step_mg_fused) on a small heated channel against the
    oracle's restatement of the same step; fixed cycle count (tol = 0)."""
    from fluxcore3d_gb300 import case as cases
    from fluxcore3d_gb300.solver.thermal_cuda_ext import patch_thermal_fused
    sim = cases.channel_cube(device=cuda, nx=24, ny=16, nz=16, cube=6, cube_x=8, with_links=False)
    sim.u.fill_(0.02)
    sim.u[sim.solid_flow] = 0.0
    src = torch.zeros_like(sim.T)
    src[sim.solid] = 0.05
    sim.heat_source = src
    patch_thermal_fused(sim)
    ref = omg.OracleMG(sim.k.cpu().numpy(), sim.rho_cp.cpu().numpy(), sim.u.cpu().numpy(), sim.v.cpu().numpy(),
                       sim.wv.cpu().numpy(), sim._build_update_mask_thermal().cpu().numpy(), 0, 1, 1.0, omega=0.6,
                       real=np.float32, flux=True)
    T = sim.T.cpu().numpy()
    T0 = sim._build_T_dirichlet_field().cpu().numpy()
    mask = sim._build_update_mask_thermal().cpu().numpy()
    for it, dt in enumerate((2.0, 3.0, 4.5)):
        info = sim._temperature_step_mg(dt, tol=0.0, max_cycles=4)
        ref.set_dt(dt)
        T, rinfo = omg.thermal_step(ref, T, T0, src.cpu().numpy(), mask, dt, 0.0, 4, 0, 23)
        assert info["it"] == rinfo["it"] == 4
        got = sim.T.cpu().numpy()
        # theta is carried on top of T0 = 25, so FP32 rounding of T alone is ulp(25) ~ 2e-6: bound the
        # difference by a few ulps of T plus 1e-5 of the largest temperature rise
        rise = float(np.abs(T - 25.0).max())
        assert rise > 1e-2
        assert float(np.abs(got - T).max()) <= 8 * float(np.spacing(np.float32(32.0))) + 1e-5 * rise, it
    assert np.isfinite(info["r_rel"])



def test_prolongation_four_and_two_cells_per_thread_bit_identical(cuda):
    """fc_mg_prolong_correct takes four cells per thread on 16-byte aligned levels with nz >= 128
    and two cells per thread on 8-byte aligned ones: the same interpolation, the same bits."""
    from fluxcore3d_gb300 import _lib
    from fluxcore3d_gb300._torch import ptr, stream_ptr
    nx, ny, nz = 16, 12, 128
    N = nx * ny * nz
    g = torch.Generator(device="cpu").manual_seed(3)
    xc = torch.randn((nx // 2) * (ny // 2) * (nz // 2), generator=g).to(cuda)
    x0 = torch.randn(N, generator=g).to(cuda)
    m0 = (torch.rand(N, generator=g) > 0.2).float().to(cuda)
    out = []
    for off in (0, 2):   # float offset 0: 16-byte aligned; 2: 8-byte aligned only
        bx = torch.zeros(N + 4, device=cuda)
        bm = torch.zeros(N + 4, device=cuda)
        x, m = bx[off:off + N], bm[off:off + N]
        x.copy_(x0)
        m.copy_(m0)
        _lib.call("fc_mg_prolong_correct", ptr(x), ptr(xc), ptr(m), nx, ny, nz, nx // 2, ny // 2, nz // 2, 0.6,
                  stream_ptr())
        torch.cuda.synchronize()
        out.append(x.clone())
    assert torch.equal(out[0].view(torch.int32), out[1].view(torch.int32))
    assert not torch.equal(out[0], x0)


@pytest.mark.parametrize("solver", ["fp64_krylov", "fp32_vcycles"])
def test_steady_temperature_matches_reference(cuda, solver):
    """The drop-in fused pseudo-time thermal step (_temperature_step_mg after patch_thermal_fused)
    driven to steady state with the ramped step of solve_thermal_steady_only (dt from 5, times 1.5
    per step, at most 200) on the heated channel of tests/golden/thermal_steady.npz, against the
    steady temperature of the reference's own fused step with its FP64 multigrid: within 1e-6
    relative L2 (the accuracy the plain FP32 path is held to) with either solver:
      fp64_krylov : each step solved by the FP64-certified BiCGSTAB around the FP32 V-cycle
                    (patch_mg_pcg(method="bicgstab_f64"));
      fp32_vcycles: the reference's FP32 stationary V-cycle iteration.
    Both rely on the flux form of the operator: with the reference's diag*T - sum a_n T_n the FP32
    rounding of diagL alone moves this steady state by ~4e-6 (the oracle in FP32 shows it)."""
    import os
    from fluxcore3d_gb300 import case as cases
    from fluxcore3d_gb300.solver.thermal_cuda_ext import patch_thermal_fused
    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "thermal_steady.npz"))
    sim = cases.channel_cube(device=cuda, nx=24, ny=16, nz=16, cube=6, cube_x=8, with_links=False)
    sim.u.fill_(0.02)
    sim.u[sim.solid_flow] = 0.0
    src = torch.zeros_like(sim.T)
    src[sim.solid] = 0.05
    sim.heat_source = src
    assert np.array_equal(sim.k.cpu().numpy(), d["k"]) and np.array_equal(sim.u.cpu().numpy(), d["u"])
    assert np.array_equal(src.cpu().numpy(), d["src"])
    patch_thermal_fused(sim)
    dt = 5.0
    tol, cycles = (1e-10, 200) if solver == "fp64_krylov" else (1e-7, 100)
    for it in range(int(d["steps"]) + 20):
        sim._temperature_step_mg(dt, tol=tol, max_cycles=cycles)
        if it == 0 and solver == "fp64_krylov":
            mg_pcg.patch_mg_pcg(sim._mg_solver, method="bicgstab_f64")
        dt = min(200.0, 1.5 * dt)
    got = sim.T.cpu().numpy().astype(np.float64)
    T = d["T"]
    assert rel(got, T) < 1e-6
    assert float(np.abs(got - T).max()) < 1e-5 * float((T - 25.0).max())


def test_solver_graphs_follow_a_rebuilt_hierarchy(cuda):
    """A hierarchy rebuilt with new coefficients (the reference's `_ready = False` pattern, used when
    the velocity changes) must not replay solver graphs captured on the old one, even when the
    allocator returns the same addresses: the FP64 BiCGSTAB on the rebuilt solver gives the result of
    a fresh solver on the new coefficients."""
    prob = problem((32, 16, 16), seed=7)
    k, rcp, u, v, w, mask, b = prob
    dev = torch.device("cuda")
    T = lambda a: torch.tensor(a, device=dev)
    mg = NLevelGeometricMGSolver(dev, torch.float32, 0, 1, 1.0, omega=0.6)
    mg.build_if_needed(T(k), T(rcp), T(u), T(v), T(w), T(mask), 50.0)
    x1, i1 = mg_pcg.bicgstab_mg_f64(mg, T(b), tol=1e-10, max_it=200)
    assert i1["converged"]
    u2 = (u * 3.0).astype(np.float32)
    mg._ready = False
    mg.build_if_needed(T(k), T(rcp), T(u2), T(v), T(w), T(mask), 50.0)
    x2, i2 = mg_pcg.bicgstab_mg_f64(mg, T(b), tol=1e-10, max_it=200)
    fresh = NLevelGeometricMGSolver(dev, torch.float32, 0, 1, 1.0, omega=0.6)
    fresh.build_if_needed(T(k), T(rcp), T(u2), T(v), T(w), T(mask), 50.0)
    x3, i3 = mg_pcg.bicgstab_mg_f64(fresh, T(b), tol=1e-10, max_it=200)
    assert i2["converged"] and i3["converged"]
    assert rel(x2.cpu().numpy(), x3.cpu().numpy()) < 1e-8
    assert rel(x2.cpu().numpy(), x1.cpu().numpy()) > 1e-4


@pytest.mark.parametrize("shape", [(16, 12, 128), (10, 6, 64), (8, 20, 256), (6, 8, 48)])
def test_prolongation_tma_staged_bit_identical(cuda, shape):
    """The TMA-staged prolongation (taken for a 16-byte aligned coarse field, nz a multiple of 8 up to
    256) and the direct-load kernels (taken when the coarse field is only 4-byte aligned) give the same
    bits, partial last row-blocks and the clamped first/last coarse rows and planes included."""
    from fluxcore3d_gb300 import _lib
    from fluxcore3d_gb300._torch import ptr, stream_ptr
    nx, ny, nz = shape
    N = nx * ny * nz
    nc = (nx // 2) * (ny // 2) * (nz // 2)
    g = torch.Generator(device="cpu").manual_seed(5)
    xc0 = torch.randn(nc, generator=g).to(cuda)
    x0 = torch.randn(N, generator=g).to(cuda)
    m0 = (torch.rand(N, generator=g) > 0.2).float().to(cuda)
    out = []
    for off in (0, 1):   # coarse offset 0: 16-byte aligned (TMA); 1: 4-byte aligned (direct loads)
        bc = torch.zeros(nc + 4, device=cuda)
        xc = bc[off:off + nc]
        xc.copy_(xc0)
        x = x0.clone()
        _lib.call("fc_mg_prolong_correct", ptr(x), ptr(xc), ptr(m0), nx, ny, nz, nx // 2, ny // 2, nz // 2, 0.75,
                  stream_ptr())
        torch.cuda.synchronize()
        out.append(x)
    assert torch.equal(out[0].view(torch.int32), out[1].view(torch.int32))
    assert not torch.equal(out[0], x0)


def test_operator_transpose_dot_identity(cuda):
    """fc_mg_mop_transpose_f32 is the transpose of the fine-level operator fc_mg_mop_f32 applies,
    ghosting included (the outlet-side self coupling on the flow axis, mirrors elsewhere):
    <M x, y> = <x, M^T y> for a masked y."""
    from fluxcore3d_gb300 import _lib
    from fluxcore3d_gb300._torch import ptr, stream_ptr
    from fluxcore3d_gb300 import learned_bench as lb
    mg, k, solid = lb.make_problem(16, 77, cuda)
    lv0 = mg._levels[0]
    nx, ny, nz = lv0["shape"]
    mask = lv0["mask_f"]
    g = torch.Generator(device="cpu").manual_seed(5)
    x = torch.randn((nx, ny, nz), generator=g).to(cuda).contiguous()
    y = (torch.randn((nx, ny, nz), generator=g).to(cuda) * mask).contiguous()
    mx = torch.empty_like(x)
    _lib.call("fc_mg_mop_f32", ptr(x), *mg._cptrs(lv0), float(mg._dt_cache), nx, ny, nz, mg.ax, lv0["out_idx"],
              None, None, ptr(mx), stream_ptr())
    mty = torch.empty_like(y)
    _lib.call("fc_mg_mop_transpose_f32", ptr(y), *mg._cptrs(lv0)[:6], float(mg._dt_cache), nx, ny, nz, mg.ax,
              lv0["out_idx"], ptr(mask), ptr(mty), stream_ptr())
    lhs = float((mx.double() * y.double()).sum())
    rhs = float((x.double() * mty.double()).sum())
    scale = float((mx.double().abs() * y.double().abs()).sum())
    assert abs(lhs - rhs) <= 1e-5 * scale, (lhs, rhs, scale)


def test_residual_loss_training_runs_and_descends(cuda):
    """The learned correction's residual-norm loss (gradient through the operator transpose)
    trains: finite and lower after a few dozen Adam steps on a handful of 16^3 problems."""
    import numpy as np
    from fluxcore3d_gb300 import learned_bench as lb
    from fluxcore3d_gb300.learned import UNetPreconditioner
    rng = np.random.default_rng(1)
    data = []
    for s in range(2):
        mg, k, solid = lb.make_problem(16, 400 + s, cuda)
        lv0 = mg._levels[0]
        op = {"coef": mg._cptrs(lv0), "dt": mg._dt_cache, "ax": mg.ax, "out_idx": lv0["out_idx"],
              "mask": lv0["mask_f"], "keep": mg}
        for _ in range(2):
            r1 = lb.residual_after_vcycle(mg, lb.random_rhs(16, rng, cuda, solid)).contiguous()
            data.append((r1, k, op))
    net = UNetPreconditioner(device=cuda, seed=3, zero_last=True)
    losses = []
    for it in range(40):
        b = [data[(2 * it) % 4], data[(2 * it + 1) % 4]]
        loss, _ = net.residual_loss_and_grad(torch.stack([d[0] for d in b]), torch.stack([d[1] for d in b]),
                                             [d[2] for d in b])
        net.adam_step(lr=1e-3)
        losses.append(loss)
    assert all(np.isfinite(losses))
    assert abs(losses[0] - 1.0) < 1e-3          # zero output: the residual is the right-hand side
    assert np.mean(losses[-8:]) < losses[0]
    assert net.check_device_error() == 0
