"""Checkpoint / resume of the fused lattice engine and the device snapshot file."""
import numpy as np
import pytest
import torch

from fluxcore3d_gb300 import case as cases
from fluxcore3d_gb300.snapshots import SnapshotUpgrade, load_checkpoint, save_checkpoint
from fluxcore3d_gb300.solver.lbm_cuda_ext import LBMCUDAUpgrade

pytestmark = pytest.mark.gpu


def make(cuda, storage, outlet, collision="mrt"):
    sim = cases.channel_cube(device=cuda, collision=collision, storage=storage, nx=48, ny=24, nz=32, cube=8,
                             cube_x=16, sponge_length=10, outlet=outlet)
    sim.cfg.macro_stride = 3
    LBMCUDAUpgrade.patch(sim)
    return sim


def run(sim, n):
    for _ in range(n):
        sim.step(do_thermal=False)


def state_bytes(sim):
    st = sim._fc.export_state()
    return st["P"].view(torch.uint8).cpu().numpy().copy()


@pytest.mark.parametrize("storage,outlet", [("fp16", "convective"), ("bf16", "pressure"), ("fp32", "pressure")])
def test_resume_from_checkpoint_is_bit_identical(cuda, tmp_path, storage, outlet):
    """K steps, checkpoint, a fresh solver loads it and runs K more: populations, the exposed
    macro fields, sim.f after sync_f and T equal a 2K-step run bit for bit."""
    K = 23
    a = make(cuda, storage, outlet)
    b = make(cuda, storage, outlet)
    g = torch.Generator(device=cuda).manual_seed(4)
    T0 = 25.0 + torch.rand(a.T.shape, generator=g, device=cuda)
    a.T.copy_(T0)
    b.T.copy_(T0)
    run(a, 2 * K)
    run(b, K)
    path = str(tmp_path / "ck.npz")
    save_checkpoint(b, path, it=K)
    c = make(cuda, storage, outlet)
    meta = load_checkpoint(c, path)
    assert meta["it"] == K and meta["k"] == K
    run(c, K)
    torch.cuda.synchronize()
    assert np.array_equal(state_bytes(a), state_bytes(c))
    for name in ("rho", "u", "v", "wv", "T"):
        assert torch.equal(getattr(a, name), getattr(c, name)), name
    a.sync_f()
    c.sync_f()
    assert torch.equal(a.f, c.f)
    assert a._fc.check_device_error() == 0 and c._fc.check_device_error() == 0


def test_checkpoint_rejects_other_geometry(cuda, tmp_path):
    a = make(cuda, "fp16", "pressure")
    run(a, 3)
    path = str(tmp_path / "ck.npz")
    save_checkpoint(a, path)
    other = cases.channel_cube(device=cuda, collision="mrt", storage="fp16", nx=48, ny=24, nz=32, cube=6,
                               cube_x=16, sponge_length=10, outlet="pressure")
    LBMCUDAUpgrade.patch(other)
    with pytest.raises(ValueError, match="geometry"):
        load_checkpoint(other, path)
    wrong = make(cuda, "bf16", "pressure")
    with pytest.raises(ValueError, match="storage"):
        load_checkpoint(wrong, path)


def test_snapshot_file_has_reference_layout_and_values(cuda, tmp_path):
    """_alloc_snapshot_buffers / _save_snapshot / _flush_snapshots through the device store: the
    archive has the reference's keys, dtypes and shapes, and every frame equals the fields at the
    step it was taken (speed = sqrt(u*u + v*v + w*w) as torch rounds it)."""
    sim = make(cuda, "fp16", "convective")
    sim.cfg.macro_stride = 1
    SnapshotUpgrade.patch(sim)
    sim.cfg.snap_stride = 5
    sim.cfg.out_dir = str(tmp_path)
    sim.cfg.snapshot_file = "snaps.npz"
    sim._alloc_snapshot_buffers(nsteps=12)
    want = []
    g = torch.Generator(device=cuda).manual_seed(2)
    for it in range(13):
        if it % 5 == 0:
            sim.T.add_(torch.rand(sim.T.shape, generator=g, device=cuda))
            sim._save_snapshot(it)
            u, v, w = sim.u, sim.v, sim.wv
            want.append({"u": u.cpu(), "v": v.cpu(), "w": w.cpu(), "rho": sim.rho.cpu(), "T": sim.T.cpu(),
                         "speed": torch.sqrt(u * u + v * v + w * w).cpu()})
        sim.step(do_thermal=False)
    out = sim._flush_snapshots()
    d = np.load(out)
    assert set(d.files) == {"u", "v", "w", "speed", "rho", "T", "solid", "_iters", "fluid_k0"}
    nx, ny, nz = sim.nx, sim.ny, sim.nz
    assert d["solid"].shape == (1, nx, ny, nz) and d["solid"].dtype == np.uint8
    assert np.array_equal(d["solid"][0], sim.solid.cpu().numpy().astype(np.uint8))
    assert d["_iters"].dtype == np.int64 and d["_iters"].tolist() == [0, 5, 10]
    assert d["fluid_k0"].tolist() == [0]
    for f in ("u", "v", "w", "speed", "rho", "T"):
        assert d[f].shape == (3, nx, ny, nz) and d[f].dtype == np.float32
        for s in range(3):
            assert np.array_equal(d[f][s].view(np.uint32), want[s][f].numpy().view(np.uint32)), (f, s)


def test_snapshot_past_allocated_frames_raises_like_reference(cuda, tmp_path):
    sim = make(cuda, "fp32", "pressure")
    SnapshotUpgrade.patch(sim)
    sim.cfg.snap_stride = 10
    sim.cfg.out_dir = str(tmp_path)
    sim._alloc_snapshot_buffers(nsteps=0)
    sim._save_snapshot(0)
    with pytest.raises(IndexError):
        sim._save_snapshot(1)
