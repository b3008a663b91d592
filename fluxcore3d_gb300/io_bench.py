"""Snapshot and checkpoint timings on the pin-fin heat sink (256x128x128, FP16 shifted MRT).

* snapshot: one frame of u, v, w, speed, rho, T (6 x 16.8 MB).  `pack_ms` is the
  device time of the pack kernel (mean of 20 back-to-back launches, CUDA events;
  44 B/cell algorithmic: 5 fields in, 6 out); `host_call_ms` the wall time of the
  `_save_snapshot` call (the loop does not wait for the copy); `landed_ms` the time
  until the frame is in pinned host memory.  `reference_style_ms` times the
  reference's own sequence (LBM_CHT.py:2749-2769: speed from torch temporaries and
  six blocking .cpu() copies into numpy frames) on the same fields.
* steps_with_snapshots: the time loop with a snapshot every 10 steps against the
  same loop without snapshots (device time per step).
* tracer: device time of one fc_tracer_step (21 B/cell algorithmic) and of the
  reference's tensor sequence for TracerField.step on the same fields; and the
  lattice step with macros written every step (what a tracer needs) alone, followed
  by the separate tracer launch, and with the tracer carried by the main pass.
* checkpoint: save_checkpoint / load_checkpoint wall time and size, file in /tmp.
"""
from __future__ import annotations

import os
import statistics
import tempfile
import time

import numpy as np
import torch


def run(dev, steps=200):
    from . import case as cases
    from .snapshots import SnapshotUpgrade, load_checkpoint, save_checkpoint
    from .solver.lbm_cuda_ext import LBMCUDAUpgrade
    sim = cases.pin_fin(device=dev, storage="fp16")
    LBMCUDAUpgrade.patch(sim)
    SnapshotUpgrade.patch(sim)
    sim.cfg.macro_stride = 1
    for _ in range(20):
        sim.step(do_thermal=False)
    tmp = tempfile.mkdtemp(prefix="fc_io_")
    sim.cfg.out_dir = tmp
    sim.cfg.snap_stride = 10
    sim._alloc_snapshot_buffers(nsteps=10 * 40)
    n = sim.nx * sim.ny * sim.nz
    out = {"workload": "pin-fin 256x128x128, FP16 shifted MRT, frames of u, v, w, speed, rho, T",
           "frame_bytes": 6 * 4 * n}
    # pack device time and host call time
    pk, hc, land = [], [], []
    for i in range(8):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t = time.perf_counter()
        e0.record()
        sim._save_snapshot(i)
        e1.record()
        hc.append((time.perf_counter() - t) * 1e3)
        sim._snap_store.wait()
        land.append((time.perf_counter() - t) * 1e3)
        torch.cuda.synchronize()
        pk.append(e0.elapsed_time(e1))
    # the pack kernel alone: 20 back-to-back launches into the staging slot, CUDA events around them
    from . import _lib
    from ._torch import ptr, stream_ptr
    slot = sim._snap_store._slots[0]
    args = (ptr(sim.rho), ptr(sim.u), ptr(sim.v), ptr(sim.wv), ptr(sim.T), n, 63, ptr(slot))
    for _ in range(3):
        _lib.call("fc_snapshot_pack", *args, stream_ptr())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(20):
        _lib.call("fc_snapshot_pack", *args, stream_ptr())
    e1.record()
    torch.cuda.synchronize()
    out["pack_ms"] = round(e0.elapsed_time(e1) / 20, 4)
    out["pack_achieved_gbs"] = round(44 * n / (out["pack_ms"] / 1e3) / 1e9, 1)
    out["save_call_device_ms"] = round(statistics.median(pk[2:]), 4)
    out["host_call_ms"] = round(statistics.median(hc[2:]), 4)
    out["landed_ms"] = round(statistics.median(land[2:]), 3)
    # the reference's sequence on the same fields
    frames = {f: np.zeros((2, sim.nx, sim.ny, sim.nz), np.float32) for f in ("u", "v", "w", "speed", "rho", "T")}
    ref = []
    for i in range(6):
        torch.cuda.synchronize()
        t = time.perf_counter()
        frames["u"][i % 2] = sim.u.detach().cpu().numpy()
        frames["v"][i % 2] = sim.v.detach().cpu().numpy()
        frames["w"][i % 2] = sim.wv.detach().cpu().numpy()
        sp = torch.sqrt(sim.u * sim.u + sim.v * sim.v + sim.wv * sim.wv)
        frames["speed"][i % 2] = sp.detach().cpu().numpy()
        frames["rho"][i % 2] = sim.rho.detach().cpu().numpy()
        frames["T"][i % 2] = sim.T.detach().cpu().numpy()
        ref.append((time.perf_counter() - t) * 1e3)
    out["reference_style_ms"] = round(statistics.median(ref[1:]), 3)
    # time loop with and without snapshots every 10 steps
    sim.cfg.macro_stride = 10
    sim._fc.macro_stride = 10

    def loop(with_snaps):
        sim._snap_count = 0
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for s in range(steps):
            sim.step(do_thermal=False)
            if with_snaps and s % 10 == 9:
                sim._save_snapshot(s)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps
    loop(False)
    base = statistics.median([loop(False) for _ in range(3)])
    snap = statistics.median([loop(True) for _ in range(3)])
    out["step_ms_without_snapshots"] = round(base, 5)
    out["step_ms_with_snapshot_every_10"] = round(snap, 5)
    # passive tracer: one fused kernel per step against the reference's tensor sequence
    from .pre_post.tracer_patch import TracerField
    sim._fc.macro_stride = 1
    sim.step(do_thermal=False)
    tr = TracerField(sim, flow_dir="+X", inject_depth=6)
    tr.inject()

    def ref_step(phi):
        u, v, w = sim.u, sim.v, sim.wv
        ax = torch.where(u >= 0, phi - torch.roll(phi, 1, 0), torch.roll(phi, -1, 0) - phi)
        ay = torch.where(v >= 0, phi - torch.roll(phi, 1, 1), torch.roll(phi, -1, 1) - phi)
        az = torch.where(w >= 0, phi - torch.roll(phi, 1, 2), torch.roll(phi, -1, 2) - phi)
        phi = torch.clamp(phi - (u * ax + v * ay + w * az), 0.0, 1.0)
        phi *= 0.9995
        phi[~tr.fluid] = 0.0
        return phi

    def timed(fn, n=50):
        for _ in range(5):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(n):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / n
    out["tracer_step_ms"] = round(timed(tr.step), 4)
    out["tracer_achieved_gbs"] = round(21 * n / (out["tracer_step_ms"] / 1e3) / 1e9, 1)
    holder = [tr.field.clone()]

    def ref():
        holder[0] = ref_step(holder[0])
    out["tracer_reference_sequence_ms"] = round(timed(ref), 4)
    # the lattice step with the tracer after it (separate launch) and carried by the main pass
    fc = sim._fc

    def plain():
        sim.step(do_thermal=False)

    def separate():
        sim.step(do_thermal=False)
        tr.step()

    def fused():
        fc.tracer = tr
        try:
            sim.step(do_thermal=False)
        finally:
            fc.tracer = None
    for name, fn in (("step_ms_macros_every_step", plain), ("step_ms_with_tracer_separate", separate),
                     ("step_ms_with_tracer_fused", fused)):
        out[name] = round(statistics.median([timed(fn, n=200) for _ in range(3)]), 4)
    # checkpoint
    path = os.path.join(tmp, "ck.npz")
    ts, tl = [], []
    for _ in range(3):
        torch.cuda.synchronize()
        t = time.perf_counter()
        save_checkpoint(sim, path, it=steps)
        ts.append(time.perf_counter() - t)
        t = time.perf_counter()
        load_checkpoint(sim, path)
        torch.cuda.synchronize()
        tl.append(time.perf_counter() - t)
    size = os.path.getsize(path)
    out["checkpoint_bytes"] = int(size)
    out["checkpoint_save_s"] = round(statistics.median(ts), 3)
    out["checkpoint_load_s"] = round(statistics.median(tl), 3)
    out["checkpoint_save_gbs"] = round(size / statistics.median(ts) / 1e9, 2)
    for fn in os.listdir(tmp):
        os.remove(os.path.join(tmp, fn))
    os.rmdir(tmp)
    return out


if __name__ == "__main__":
    import json
    print(json.dumps(run(torch.device("cuda"))))
