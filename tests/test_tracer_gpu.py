"""Passive tracer kernel against the reference's TracerField fixtures and the oracle."""
import os
import types

import numpy as np
import pytest
import torch

from fluxcore3d_gb300 import case as cases
from fluxcore3d_gb300.pre_post.tracer_patch import TracerField, attach_tracer
from fluxcore3d_gb300.solver.lbm_cuda_ext import LBMCUDAUpgrade
from oracle import tracer as ot

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


def test_tracer_matches_reference_fixture(cuda):
    d = np.load(os.path.join(GOLD, "tracer.npz"))
    nx, ny, nz = d["solid_flow"].shape
    sim = types.SimpleNamespace(nx=nx, ny=ny, nz=nz, device=cuda, solid_flow=torch.from_numpy(d["solid_flow"]).to(cuda))
    tr = TracerField(sim, flow_dir="+X", inject_depth=3, dissipation=0.9995)
    assert np.array_equal(tr._inlet.cpu().numpy(), d["inlet"])
    tr.inject()
    for it in range(25):
        s = it // 5
        sim.u, sim.v, sim.wv = (torch.from_numpy(d[f"{n}{s}"]).to(cuda) for n in ("u", "v", "w"))
        if it % 7 == 6:
            tr.inject()
        tr.step()
        if it == 0:
            assert np.array_equal(bits(tr.get()), bits(d["field1"]))
    assert np.array_equal(bits(tr.get()), bits(d["field25"]))


@pytest.mark.parametrize("shape", [(33, 1, 300), (1, 40, 17), (64, 48, 40)])
def test_tracer_matches_oracle_on_seeded_fields(cuda, shape):
    rng = np.random.default_rng(sum(shape))
    solid = rng.random(shape) < 0.2
    u, v, w = ((rng.random(shape).astype(np.float32) - 0.5) * 0.4 for _ in range(3))
    u[0, 0, 0] = np.nan                                  # NaN velocity: the other branch, NaN kept
    sim = types.SimpleNamespace(nx=shape[0], ny=shape[1], nz=shape[2], device=cuda,
                                solid_flow=torch.from_numpy(solid).to(cuda))
    for fd in ("-Z", "+Y"):
        tr = TracerField(sim, flow_dir=fd, inject_depth=2, dissipation=0.998)
        sim.u, sim.v, sim.wv = (torch.from_numpy(a).to(cuda) for a in (u, v, w))
        phi = np.zeros(shape, np.float32)
        tr.inject()
        phi = ot.inject(phi, tr._inlet.cpu().numpy())
        for it in range(12):
            tr.step()
            phi = ot.step(phi, u, v, w, solid, 0.998)
        got = tr.get()
        assert np.array_equal(np.isnan(got), np.isnan(phi))
        assert np.array_equal(bits(np.nan_to_num(got)), bits(np.nan_to_num(phi)))


def test_attach_tracer_follows_the_lattice_velocity(cuda):
    sim = cases.channel_cube(device=cuda, collision="mrt", storage="fp16", nx=48, ny=24, nz=24, cube=6, cube_x=14,
                             outlet="pressure")
    sim.cfg.macro_stride = 10
    LBMCUDAUpgrade.patch(sim)
    tr = attach_tracer(sim, flow_dir="+X", inject_depth=4)
    assert sim._fc.macro_stride == 1
    tr.inject()
    phi = tr.get()
    solid = sim.solid_flow.cpu().numpy()
    for _ in range(15):
        sim.step(do_thermal=False)
        u, v, w = (t.cpu().numpy() for t in (sim.u, sim.v, sim.wv))
        phi = ot.step(phi, u, v, w, solid)
    assert np.array_equal(bits(tr.get()), bits(phi))
    assert float(tr.field.max()) > 0.5


@pytest.mark.parametrize("storage,collision", [("fp16", "mrt"), ("fp32", "trt")])
def test_tracer_carried_by_the_staged_pass(cuda, storage, collision):
    """attach_tracer hands the tracer to the lattice engine, whose staged main pass advances it:
    the field equals the separate kernel's (fuse=False) and the oracle's step on the exposed
    velocity, bit for bit, including injections between steps."""
    def make(fuse):
        sim = cases.channel_cube(device=cuda, collision=collision, storage=storage, nx=64, ny=32, nz=32, cube=8,
                                 cube_x=20, outlet="pressure")
        sim.cfg.macro_stride = 10
        LBMCUDAUpgrade.patch(sim)
        tr = attach_tracer(sim, flow_dir="+X", inject_depth=4, fuse=fuse)
        return sim, tr
    sim, tr = make(True)
    ref_sim, ref_tr = make(False)
    assert sim._fc.tracer is tr and ref_sim._fc.tracer is None
    assert sim._fc.tile_links is not None          # the staged pass runs on this grid
    solid = sim.solid_flow.cpu().numpy()
    phi = None
    for it in range(24):
        if it % 10 == 0:
            tr.inject()
            ref_tr.inject()
            phi = tr.get() if phi is None else np.where(tr._inlet.cpu().numpy(), np.float32(1.0), phi)
        sim.step(do_thermal=False)
        ref_sim.step(do_thermal=False)
        u, v, w = (t.cpu().numpy() for t in (sim.u, sim.v, sim.wv))
        phi = ot.step(phi, u, v, w, solid)
        got = tr.get()
        assert np.array_equal(bits(got), bits(ref_tr.get())), it
        assert np.array_equal(bits(got), bits(phi)), it
    assert sim._fc.check_device_error() == 0
    assert float(tr.field.max()) > 0.5
    # a tracer step on its own (warm-up style) still runs the kernel
    tr.step()
    ref_tr.step()
    assert np.array_equal(bits(tr.get()), bits(ref_tr.get()))
