"""The FP64 run of the plain method on the device (fluxcore3d_gb300.lattice64) against the
oracle's FP64 C restatement of the same step sequence.

Both evaluate the reference's CUDA-path step in double precision; they differ only in
rounding order (the device contracts multiply-adds, the oracle uses a generic moment
matrix for MRT), so the populations must agree within 1e-11 relative L2 after the stated
number of steps, and within 1e-9 with the Smagorinsky model, whose square root of the
non-equilibrium stress amplifies rounding differences where that stress is near zero.
"""
import numpy as np
import pytest
import torch

from fluxcore3d_gb300 import case as cases
from fluxcore3d_gb300.lattice64 import Lattice64
from test_lbm_gpu import oracle_for, rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("collision,outlet", [("bgk", "convective"), ("trt", "pressure"), ("mrt", "pressure"),
                                              ("mrt_smag", "pressure")])
def test_lattice64_matches_fp64_oracle_channel(cuda, collision, outlet):
    sim = cases.channel_cube(device=cuda, collision=collision, nx=32, ny=16, nz=16, cube=6, cube_x=10,
                             sponge_length=8 if outlet == "pressure" else 0, outlet=outlet)
    orc = oracle_for(sim, real="f64")
    lat = Lattice64(sim)
    lat.step(150)
    orc.step(150)
    lat.check()
    e = rel_l2(lat.f.cpu().numpy(), orc.f)
    tol = 1e-9 if collision == "mrt_smag" else 1e-11
    assert e < tol, e
    assert rel_l2(lat.u.cpu().numpy(), orc.u) < 100 * tol   # velocities near zero carry the relative error


def test_lattice64_matches_fp64_oracle_pin_fin(cuda):
    """All three interpolated bounce-back link modes, MRT-Smagorinsky, pressure outlet, sponge."""
    sim = cases.pin_fin(device=cuda, collision="mrt_smag", storage="fp32", nx=48, ny=32, nz=48, n_pins=(3, 2),
                        radius=3.5, height=24, base=4, sponge_length=8)
    orc = oracle_for(sim, real="f64")
    lat = Lattice64(sim)
    lat.step(100)
    orc.step(100)
    lat.check()
    assert rel_l2(lat.f.cpu().numpy(), orc.f) < 1e-9


def test_lattice64_velocity_is_macros_of_f(cuda):
    sim = cases.channel_cube(device=cuda, collision="mrt", nx=24, ny=12, nz=16, cube=4, cube_x=8)
    lat = Lattice64(sim)
    lat.step(20)
    u = lat.velocity().cpu().numpy()
    f = lat.f.cpu().numpy()
    c = np.array(cases.geo.C_NP, dtype=np.float64)
    ref = (c.T @ f) / f.sum(0)
    assert np.allclose(u, ref, rtol=1e-13, atol=1e-15)
    assert torch.isfinite(lat.f).all()
