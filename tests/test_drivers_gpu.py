"""The drop-in driven by the reference's own outer-loop pattern.

run_flow_to_steady_v2 (solver/flow_solver_upgrade.py:537-723) steps the solver and, every
`check_every` loop iterations (it % check_every == 0, i.e. after steps 1, 1 + check_every, ...),
reads sim.u / sim.v / sim.wv / sim.rho into an exponential moving average, a domain mass rate
(with rho_prev.copy_(sim.rho)), the mean density error and the peak speed.  Here that loop runs
on the fused engine with cfg.macro_stride = check_every (the engine writes the macros only where
such a monitor reads them, and rebinds the macro attributes every step) and on the oracle, whose
macros are written every step; the monitor values must agree to FP32 accuracy."""
import numpy as np
import pytest
import torch

from fluxcore3d_gb300 import case as cases
from fluxcore3d_gb300.solver.lbm_cuda_ext import LBMCUDAUpgrade
from test_lbm_gpu import oracle_for

pytestmark = pytest.mark.gpu


class _Monitor:
    """The monitor arithmetic of run_flow_to_steady_v2 (EMA residual, mass rate, density error, umax)."""

    def __init__(self, u, v, w, rho, fluid, rho_out, ema_window=200):
        self.alpha = 2.0 / (ema_window + 1)
        self.fluid = fluid
        self.rho_out = rho_out
        self.ema = [np.array(a, np.float64) for a in (u, v, w)]
        self.rho_prev = np.array(rho, np.float64)
        self.hist = []

    def check(self, it, u, v, w, rho):
        prev = [e.copy() for e in self.ema]
        self.ema = [self.alpha * np.asarray(x, np.float64) + (1 - self.alpha) * e for x, e in zip((u, v, w), self.ema)]
        du = max(float(np.abs(e - p).max()) for e, p in zip(self.ema, prev))
        mag = float(np.sqrt(sum(e ** 2 for e in self.ema)).max())
        umax = float(np.sqrt(sum(np.asarray(x, np.float64) ** 2 for x in (u, v, w))).max())
        rho = np.asarray(rho, np.float64)
        m_now, m_prev = rho[self.fluid].sum(), self.rho_prev[self.fluid].sum()
        self.hist.append({"step": it, "R_ema": du / (mag + 1e-12), "R_dm": abs(m_now - m_prev) / (m_prev + 1e-12),
                          "rho_mean_err": abs(rho[self.fluid].mean() - self.rho_out), "umax": umax})
        self.rho_prev = rho.copy()


def test_flow_monitor_loop_on_the_drop_in_matches_oracle(cuda):
    check_every, n = 10, 61
    sim = cases.channel_cube(device=cuda, collision="mrt", storage="fp32", nx=48, ny=24, nz=32, cube=8, cube_x=16)
    sim.cfg.macro_stride = check_every
    orc = oracle_for(sim)
    shape = (sim.nx, sim.ny, sim.nz)
    fluid = ~sim.solid_flow.cpu().numpy()
    rho_out = float(sim.cfg.rho_out_lat)
    LBMCUDAUpgrade.patch(sim)
    mon_dev = _Monitor(*(t.cpu().numpy() for t in (sim.u, sim.v, sim.wv, sim.rho)), fluid, rho_out)
    mon_orc = _Monitor(*(t.cpu().numpy() for t in (sim.u, sim.v, sim.wv, sim.rho)), fluid, rho_out)
    rho_prev = sim.rho.clone()            # the reference keeps its own copy and refreshes it in place
    for it in range(n):
        sim.step(do_thermal=False)
        orc.step(1)
        if it % check_every != 0:
            continue
        mon_dev.check(it, *(t.cpu().numpy() for t in (sim.u, sim.v, sim.wv, sim.rho)))
        mon_orc.check(it, *(a.reshape(shape) for a in (orc.u, orc.v, orc.w, orc.rho)))
        rho_prev.copy_(sim.rho)
        last_rho = sim.rho.clone()
    assert sim._fc.check_device_error() == 0
    # the caller's copy is its own storage: later steps rebind and rewrite the engine's macros only
    assert rho_prev.data_ptr() != sim.rho.data_ptr() and torch.equal(rho_prev, last_rho)
    assert [h["step"] for h in mon_dev.hist] == list(range(0, n, check_every))
    for a, b in zip(mon_dev.hist, mon_orc.hist):
        assert abs(a["umax"] - b["umax"]) <= 1e-5 * b["umax"]
        assert abs(a["rho_mean_err"] - b["rho_mean_err"]) <= 1e-6
        assert abs(a["R_ema"] - b["R_ema"]) <= 1e-4 * b["R_ema"] + 1e-9
        assert abs(a["R_dm"] - b["R_dm"]) <= 1e-6
