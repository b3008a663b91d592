"""The coupled flow + heat driver (fluxcore3d_gb300.coupled.CoupledCHT) against the oracle's
lattice run and the oracle's pseudo-time thermal step on the velocities that run produces.

A 32x16x16 channel with a heated cube (BGK, FP32 storage, Bouzidi links): thermal steps with
dt = 50 after lattice steps 11 and 21 (every 10 steps, on the pre-collision macros of the state
before, as the engine exposes them).  Temperatures agree within 1e-5 relative L2 of the rise
(FP32 lattice against FP32 oracle velocities, both thermal systems solved far below that); every
recorded FP64 heat balance closes to 1e-6 of the heat generated."""
import numpy as np
import pytest
import torch

from fluxcore3d_gb300 import case as cases
from fluxcore3d_gb300.coupled import CoupledCHT
from oracle import mg as omg
from test_lbm_gpu import oracle_for

pytestmark = pytest.mark.gpu


def test_coupled_run_matches_oracle_lattice_and_thermal(cuda):
    sim = cases.channel_cube(device=cuda, collision="bgk", storage="fp32", nx=32, ny=16, nz=16, cube=6, cube_x=10)
    src = torch.zeros_like(sim.T)
    src[sim.solid] = 0.05
    sim.heat_source = src
    orc = oracle_for(sim)
    k = sim.k.cpu().numpy()
    rcp = sim.rho_cp.cpu().numpy()
    solid_flow = sim.solid_flow.cpu().numpy()
    mask = sim._build_update_mask_thermal().cpu().numpy()
    cp = CoupledCHT(sim, thermal_every=10, dt_thermal=50.0, tol=1e-11, max_it=400)
    cp.run(21)
    assert [h["step"] for h in cp.history] == [11, 21]
    assert all(h["converged"] for h in cp.history)
    assert all(h["imbalance_rel"] < 1e-6 for h in cp.history), cp.history
    shape = (sim.nx, sim.ny, sim.nz)
    T = np.full(shape, 25.0)
    T0 = np.full(shape, 25.0)
    done = 0
    for kk in (11, 21):
        orc.step(kk - done)
        done = kk
        vel = [np.asarray(a, np.float32).reshape(shape).copy() for a in (orc.u, orc.v, orc.w)]
        for a in vel:
            a[solid_flow] = 0.0
        ref = omg.OracleMG(k, rcp, *vel, mask, 0, 1, 1.0, omega=0.6, real=np.float64, flux=True)
        ref.set_dt(50.0)
        T, _ = omg.thermal_step(ref, T, T0, src.cpu().numpy().astype(np.float64), mask, 50.0, 1e-12, 600, 0,
                                shape[0] - 1)
    got = sim.T.cpu().numpy().astype(np.float64)
    rise = T - 25.0
    assert float(np.abs(rise).max()) > 1e-3
    assert np.linalg.norm(got - T) / np.linalg.norm(rise) < 1e-5
