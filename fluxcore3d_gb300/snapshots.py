"""Snapshot files and checkpoints, written from the device.

Snapshots
---------
`SnapshotUpgrade.patch(sim)` replaces the reference's one-file snapshot store
(LBMCHT3D_Torch._alloc_snapshot_buffers / _save_snapshot / _flush_snapshots,
LBM_CHT.py:2717-2791) on the solver object.  The file is the same: one
np.savez_compressed archive with the keys of `cfg.store_fields` (frames
[n, nx, ny, nz] FP32, "solid" [1, nx, ny, nz] uint8), "_iters" (int64 step
numbers), "fluid_k0" and, when the solver carries a solid assembly, "body_names"
and "solid_<name>" masks, so the reference's viewers and web app read it
unchanged.  What changes is how a frame leaves the GPU: the reference copies
each field to the host with a blocking copy (and computes speed with three
temporaries); here one kernel (fc_snapshot_pack) packs the selected fields,
speed included, into one of two device staging slots, and a copy stream moves
the slot to pinned host memory while the time loop goes on.  The loop waits only
when it reuses a slot whose copy has not finished (two frames in flight).

Checkpoints
-----------
`save_checkpoint(sim, path, it)` / `load_checkpoint(sim, path)` (no counterpart
in the reference, which cannot resume a run).  For a solver patched with the
fused lattice engine the checkpoint holds the engine's exact state -- the latest
post-collision populations in their storage format (FP16/BF16 shifted or
FP32), both macro buffers, the step count, and the sim.f populations of the
inlet/outlet plane cells (the only part of sim.f a step reads before writing) --
plus the temperature field, so a run resumed from it continues bit for bit.  An
unpatched solver stores sim.f and the macro fields.  The container is an
uncompressed .npz with a JSON "meta" entry (sizes, storage, collision, a CRC of
the cell-flag array) that loading checks against the receiving solver.
"""
from __future__ import annotations

import json
import os
import zlib

import numpy as np
import torch

from . import _lib
from ._torch import ptr, stream_ptr

FIELD_BITS = {"u": 1, "v": 2, "w": 4, "speed": 8, "rho": 16, "T": 32}
FIELD_ORDER = ("u", "v", "w", "speed", "rho", "T")
CKPT_VERSION = 1


def _f32(t: torch.Tensor) -> torch.Tensor:
    if t.dtype != torch.float32:
        raise RuntimeError("snapshot fields must be float32 (the reference stores FP32 frames for FP32 solvers)")
    return t.contiguous()


class SnapshotStore:
    """The snapshot buffers of one solver object (see the module docstring)."""

    def __init__(self, sim):
        self.sim = sim
        self._slots = None
        self._copy_stream = None
        self._ev_packed = None
        self._ev_copied = None
        self._frames = {}

    # LBMCHT3D_Torch._alloc_snapshot_buffers (LBM_CHT.py:2717-2747)
    def alloc(self, nsteps: int):
        sim = self.sim
        cfg = sim.cfg
        if int(getattr(cfg, "snap_stride", 200)) <= 0:
            sim._snapshots = None
            return
        if sim.dtype != torch.float32:
            raise NotImplementedError("device snapshots are implemented for FP32 solvers")
        nsnaps = (int(nsteps) // int(cfg.snap_stride)) + 1
        nx, ny, nz = sim.nx, sim.ny, sim.nz
        snaps = {}
        self._frames = {}
        for f in getattr(cfg, "store_fields", ("u", "v", "w", "speed", "rho", "T", "solid")):
            if f == "solid":
                snaps["solid"] = np.zeros((1, nx, ny, nz), dtype=np.uint8)
            else:
                host = torch.empty((nsnaps, nx, ny, nz), dtype=torch.float32, pin_memory=True)
                self._frames[f] = host
                snaps[f] = host.numpy()
        snaps["_iters"] = np.zeros((nsnaps,), dtype=np.int64)
        sim._snapshots = snaps
        sim._snap_count = 0
        if "solid" in snaps:
            snaps["solid"][0] = sim.solid.detach().cpu().numpy().astype(np.uint8)
        snaps["fluid_k0"] = np.array([getattr(cfg, "fluid_k0", 0)], dtype=np.int64)
        asm = getattr(sim, "_assembly", None)
        if asm is not None and hasattr(asm, "_body_masks"):
            snaps["body_names"] = np.array(list(asm._body_masks.keys()))
            for name, mask in asm._body_masks.items():
                snaps[f"solid_{name}"] = mask.cpu().numpy().astype(np.uint8)[np.newaxis]
        self._slots = None

    def _fields(self):
        return [f for f in FIELD_ORDER if f in self._frames]

    def _ensure_slots(self, nf: int, n: int):
        dev = self.sim.device
        if self._slots is None or self._slots[0].shape != (nf, n):
            self._slots = [torch.empty((nf, n), dtype=torch.float32, device=dev) for _ in range(2)]
            self._copy_stream = torch.cuda.Stream(device=dev)
            self._ev_packed = [torch.cuda.Event() for _ in range(2)]
            self._ev_copied = [None, None]

    # LBMCHT3D_Torch._save_snapshot (LBM_CHT.py:2749-2769)
    def save(self, it: int):
        sim = self.sim
        snaps = getattr(sim, "_snapshots", None)
        if snaps is None:
            return
        sidx = sim._snap_count
        snaps["_iters"][sidx] = it              # IndexError past the allocated frames, as the reference
        fields = self._fields()
        if fields:
            n = sim.nx * sim.ny * sim.nz
            self._ensure_slots(len(fields), n)
            s = sidx % 2
            main = torch.cuda.current_stream()
            if self._ev_copied[s] is not None:
                main.wait_event(self._ev_copied[s])
            mask = 0
            for f in fields:
                mask |= FIELD_BITS[f]
            rho = _f32(sim.rho) if "rho" in fields else None
            T = _f32(sim.T) if "T" in fields else None
            uvw = any(f in fields for f in ("u", "v", "w", "speed"))
            u, v, w = (_f32(sim.u), _f32(sim.v), _f32(sim.wv)) if uvw else (None, None, None)
            _lib.call("fc_snapshot_pack", ptr(rho), ptr(u), ptr(v), ptr(w), ptr(T), n, mask, ptr(self._slots[s]),
                      stream_ptr())
            self._ev_packed[s].record(main)
            cs = self._copy_stream
            cs.wait_event(self._ev_packed[s])
            with torch.cuda.stream(cs):
                for r, f in enumerate(fields):
                    self._frames[f][sidx].view(-1).copy_(self._slots[s][r], non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(cs)
            self._ev_copied[s] = ev
            # the slot is read by the copy stream: keep the caching allocator from reusing it early
            self._slots[s].record_stream(cs)
        sim._snap_count += 1

    def wait(self):
        for ev in (self._ev_copied or []):
            if ev is not None:
                ev.synchronize()

    def payload(self) -> dict:
        """The archive's arrays, as LBMCHT3D_Torch._flush_snapshots (LBM_CHT.py:2771-2788) builds them."""
        sim = self.sim
        self.wait()
        ns = sim._snap_count
        out = {}
        for k, v in sim._snapshots.items():
            if k == "solid" or k == "fluid_k0" or k == "body_names" or k.startswith("solid_"):
                out[k] = v
            else:
                out[k] = v[:ns]
        return out

    # LBMCHT3D_Torch._flush_snapshots (LBM_CHT.py:2771-2788)
    def flush(self):
        sim = self.sim
        if getattr(sim, "_snapshots", None) is None:
            return
        os.makedirs(sim.cfg.out_dir, exist_ok=True)
        out_path = os.path.join(sim.cfg.out_dir, sim.cfg.snapshot_file)
        np.savez_compressed(out_path, **self.payload())
        return out_path


class SnapshotUpgrade:
    """Install the device snapshot store on a solver object (LBMCHT3D_Torch or LatticeCase)."""

    @staticmethod
    def patch(sim):
        store = SnapshotStore(sim)
        sim._snap_store = store
        sim._alloc_snapshot_buffers = store.alloc
        sim._save_snapshot = store.save
        sim._flush_snapshots = store.flush
        for name, default in (("snap_stride", 200), ("out_dir", "."), ("snapshot_file", "snapshots3d.npz"),
                              ("store_fields", ("u", "v", "w", "speed", "rho", "T", "solid"))):
            if not hasattr(sim.cfg, name):
                setattr(sim.cfg, name, default)
        return sim


# ---------------------------------------------------------------------------
# checkpoints
# ---------------------------------------------------------------------------
def _to_host(t: torch.Tensor) -> np.ndarray:
    h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
    h.copy_(t, non_blocking=True)
    return h


def _np(h: torch.Tensor) -> np.ndarray:
    if h.dtype in (torch.float16, torch.bfloat16):
        return h.view(torch.int16).numpy().view(np.uint16)
    return h.numpy()


def _flags_crc(fc) -> int:
    return zlib.crc32(fc.flags.cpu().numpy().tobytes()) & 0xFFFFFFFF


def save_checkpoint(sim, path: str, it: int = 0) -> str:
    """Write the state a resumed run needs to continue this one exactly; returns the path."""
    fc = getattr(sim, "_fc", None)
    meta = {"version": CKPT_VERSION, "it": int(it), "nx": sim.nx, "ny": sim.ny, "nz": sim.nz}
    dev_arrays = {}
    if fc is not None:
        stt = fc.export_state()
        idx = fc.plane_cells()
        cols = torch.empty((19, idx.numel()), dtype=torch.float32, device=sim.device)
        err = torch.zeros(1, dtype=torch.int32, device=sim.device)
        _lib.call("fc_columns_gather", ptr(sim.f), 19, fc.N, ptr(idx), idx.numel(), ptr(cols), ptr(err),
                  stream_ptr())
        meta.update(kind="fused", k=int(stt["k"]), storage=fc.storage_name, collision=fc.collision,
                    macro_stride=fc.macro_stride, flags_crc=_flags_crc(fc), n_links=fc.n_links)
        dev_arrays.update(P=stt["P"], M0=stt["M0"], M1=stt["M1"], f_plane_idx=idx, f_plane=cols)
    else:
        meta.update(kind="plain")
        dev_arrays.update(f=sim.f, rho=sim.rho, u=sim.u, v=sim.v, wv=sim.wv)
    if getattr(sim, "T", None) is not None:
        dev_arrays["T"] = sim.T
    scalars = {}
    for name in ("thermal_dt_scale",):
        if hasattr(sim, name):
            scalars[name] = float(getattr(sim, name))
    meta["scalars"] = scalars
    host = {k: _to_host(v.detach()) for k, v in dev_arrays.items()}
    torch.cuda.synchronize(sim.device)
    if fc is not None and int(err.item()):
        raise RuntimeError("checkpoint: plane-cell index out of range")
    arrays = {k: _np(v) for k, v in host.items()}
    arrays["meta"] = np.array(json.dumps(meta))
    with open(path, "wb") as fh:
        np.savez(fh, **arrays)
    return path


def load_checkpoint(sim, path: str) -> dict:
    """Restore a checkpoint into a solver built for the same case; returns its metadata
    (meta["it"] is the step number the caller passed to save_checkpoint)."""
    d = np.load(path, allow_pickle=False)
    meta = json.loads(str(d["meta"]))
    if meta.get("version") != CKPT_VERSION:
        raise ValueError(f"checkpoint version {meta.get('version')} is not {CKPT_VERSION}")
    if (meta["nx"], meta["ny"], meta["nz"]) != (sim.nx, sim.ny, sim.nz):
        raise ValueError("checkpoint grid size differs from the solver's")
    dev = sim.device
    fc = getattr(sim, "_fc", None)

    def up(name, like):
        a = np.ascontiguousarray(d[name])
        if like.dtype in (torch.float16, torch.bfloat16):
            t = torch.from_numpy(a.view(np.int16)).view(like.dtype)
        else:
            t = torch.from_numpy(a)
        if t.dtype != like.dtype:
            raise ValueError(f"checkpoint array {name} has dtype {t.dtype}, expected {like.dtype}")
        return t.to(dev).reshape(like.shape)

    if meta["kind"] == "fused":
        if fc is None:
            raise ValueError("fused-engine checkpoint: patch the solver (LBMCUDAUpgrade.patch) before loading")
        if meta["storage"] != fc.storage_name or meta["collision"] != fc.collision:
            raise ValueError("checkpoint storage / collision differ from the solver's")
        if meta["flags_crc"] != _flags_crc(fc) or meta["n_links"] != fc.n_links:
            raise ValueError("checkpoint geometry (cell flags / links) differs from the solver's")
        idx = torch.from_numpy(d["f_plane_idx"]).to(dev)
        cols = torch.from_numpy(d["f_plane"]).to(dev)
        err = torch.zeros(1, dtype=torch.int32, device=dev)
        _lib.call("fc_columns_scatter", ptr(sim.f), 19, fc.N, ptr(idx), idx.numel(), ptr(cols), ptr(err),
                  stream_ptr())
        P = up("P", fc.P[0])
        M0 = up("M0", torch.empty((4, fc.N), dtype=torch.float32))
        M1 = up("M1", torch.empty((4, fc.N), dtype=torch.float32))
        fc.import_state(meta["k"], P, M0, M1)
        if int(err.item()):
            raise RuntimeError("checkpoint: plane-cell index out of range")
    else:
        sim.f.copy_(torch.from_numpy(d["f"]).to(dev).reshape(sim.f.shape))
        for name in ("rho", "u", "v", "wv"):
            getattr(sim, name).copy_(torch.from_numpy(d[name]).to(dev))
        if fc is not None:
            fc.invalidate()
    if "T" in d.files and getattr(sim, "T", None) is not None:
        sim.T.copy_(torch.from_numpy(d["T"]).to(dev).reshape(sim.T.shape))
    for name, v in meta.get("scalars", {}).items():
        setattr(sim, name, v)
    return meta
