"""FP64 conservation integrals (mass of the lattice state, heat balance of the thermal step)."""
import numpy as np
import pytest
import torch

from fluxcore3d_gb300 import case as cases
from fluxcore3d_gb300.diagnostics import heat_balance, lbm_mass
from fluxcore3d_gb300.solver import mg_pcg
from fluxcore3d_gb300.solver.lbm_cuda_ext import LBMCUDAUpgrade
from fluxcore3d_gb300.solver.nlevel_mg_cuda import NLevelGeometricMGSolver
from oracle.mg import shift

pytestmark = pytest.mark.gpu
W = np.array([0.33333333] + [0.05555556] * 6 + [0.02777778] * 12, dtype=np.float32)


@pytest.mark.parametrize("storage", ["fp32", "fp16", "bf16"])
def test_lbm_mass_matches_fp64_host_sum(cuda, storage):
    sim = cases.channel_cube(device=cuda, collision="mrt", storage=storage, nx=40, ny=20, nz=24, cube=6, cube_x=12,
                             outlet="pressure")
    LBMCUDAUpgrade.patch(sim)
    for _ in range(7):
        sim.step(do_thermal=False)
    fc = sim._fc
    P = fc.P[fc.cur]
    if storage == "fp32":
        f = P.cpu().numpy().astype(np.float64)
    else:
        f = P.float().cpu().numpy().astype(np.float64) + W.astype(np.float64)[:, None]
    fluid = (fc.flags.cpu().numpy() & 1) == 0
    want = f[:, fluid].sum()
    got = lbm_mass(sim)
    assert abs(got - want) <= 1e-12 * abs(want)


def test_heat_balance_integrals_and_closure(cuda):
    g = torch.Generator(device=cuda).manual_seed(5)
    shape = (32, 16, 16)
    k = torch.where(torch.rand(shape, generator=g, device=cuda) < 0.3, 200.0, 1.0) * 0.005
    rcp = torch.ones(shape, device=cuda)
    u = torch.rand(shape, generator=g, device=cuda) * 0.05
    z = torch.zeros(shape, device=cuda)
    mask = torch.ones(shape, dtype=torch.bool, device=cuda)
    mask[0] = False
    dt = 50.0
    mg = NLevelGeometricMGSolver(cuda, torch.float32, 0, +1, 1.0, omega=0.6)
    mg.build_if_needed(k, rcp, u, z, z, mask, dt)
    src = torch.rand(shape, generator=g, device=cuda) * mask
    T = torch.rand(shape, generator=g, device=cuda)
    hb = heat_balance(mg, T, src, dt)
    lv = mg._levels[0]
    a = {key: lv[key].cpu().numpy().astype(np.float64) for key in ("aE", "aW", "aN", "aS", "aU", "aD", "diagL")}
    Tn = T.cpu().numpy().astype(np.float64)
    ax, oi = mg.ax, lv["out_idx"]
    # the operator in flux form sum_n a_n (T - T_n), as the kernels evaluate it
    L = (a["aE"] * (Tn - shift(Tn, 0, 1, ax, oi)) + a["aW"] * (Tn - shift(Tn, 0, -1, ax, oi))
         + a["aN"] * (Tn - shift(Tn, 1, 1, ax, oi)) + a["aS"] * (Tn - shift(Tn, 1, -1, ax, oi))
         + a["aU"] * (Tn - shift(Tn, 2, 1, ax, oi)) + a["aD"] * (Tn - shift(Tn, 2, -1, ax, oi)))
    m = mask.cpu().numpy()
    assert abs(hb["heat_out_through_boundaries"] - L[m].sum()) <= 1e-9 * np.abs(L[m]).sum()
    assert abs(hb["heat_generated"] - src.cpu().numpy().astype(np.float64)[m].sum()) <= 1e-9 * hb["heat_generated"]
    assert abs(hb["heat_stored"] - Tn[m].sum() / dt) <= 1e-9 * Tn[m].sum() / dt
    # the solution of A T = dt src balances generated = outflow + stored to the solve's accuracy
    b = (mask.float() * dt * src).contiguous()
    x, info = mg_pcg.bicgstab_mg_f64(mg, b, tol=1e-10, max_it=400)
    assert info["converged"]
    hb2 = heat_balance(mg, x, src, dt)
    assert hb2["imbalance_rel"] < 1e-5, hb2
