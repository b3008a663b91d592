"""Fused step engine behind LBMCUDAUpgrade.patch(sim).step.

State kept between steps
------------------------
The reference stores post-stream populations S_k in `sim.f` and recollides
them at the start of every step.  This engine stores the post-collision
populations P_{k+1} = C(S_k) instead (two ping-pong buffers, FP32 or FP16/BF16
shifted by w_q) so that one pass per step can pull, bounce back, collide and
store: step k reads P_k and writes P_{k+1}.  S_k is not stored; `sync_f()`
rebuilds it into `sim.f` from P_k on demand.

Observable behaviour compared with the reference step (solver/lbm_cuda_ext.py:445-517)
  - sim.rho/u/v/wv after step k hold the macros of S_{k-1}, exactly as in the
    reference (its collide writes the pre-collision macros).  They are written
    every step unless `cfg.macro_stride = s > 1`, in which case only the
    macros needed after steps k with (k-1) % s == 0 are written (the cadence of
    a monitor that reads every s steps starting after the first).  The macro
    tensors are double-buffered, so the attributes are rebound each step.
  - sim.f is only current after `sim.sync_f()` (and on inlet/outlet planes,
    which the plane BCs update in place every step).
  - The collision of step k+1 happens inside step k, so parameters changed on
    the solver object between steps take effect one step later; call
    `sim._fc.invalidate()` after editing sim.f or the collision parameters.
"""
from __future__ import annotations

import ctypes as C

import torch

from .. import _lib
from .._lib import StepArgs
from .._torch import capture_graph, ptr, stream_ptr
from .face_roles import periodic_flags, resolve_face_roles, _face_ax_idx_fsign

CF_SOLID, CF_LINK, CF_DEFER, CF_WRITE_S = 1, 2, 4, 8  # low nibble; high nibble = link count
STORAGE = {"fp32": 0, "float32": 0, "f32": 0, "fp16": 1, "float16": 1, "f16": 1, "bf16": 2, "bfloat16": 2}
STORAGE_DTYPE = {0: torch.float32, 1: torch.float16, 2: torch.bfloat16}
COLLISION = {"bgk": 0, "trt": 1, "mrt": 2, "mrt_smag": 3}
_CX = (0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1, 0, 0, 0, 0)
_CY = (0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1)
_CZ = (0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1)
_OPP = (0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15)


def build_link_table(ibb, solid_flow_u8: torch.Tensor, nx: int, ny: int, nz: int):
    """Per-cell interpolated-bounce-back tables from the reference's link-major IBBData.

    Returns a dict with
      link_off [N] int32   ordinal of the cell among link cells (-1 elsewhere)
      link_hdr [C, 4] int32 per link cell: mask of link directions (bit d), mask of
                           links whose second term is the opposite population at
                           x_f - c_d (q < 1/2 with a fluid second node), offset of the
                           cell's first (w1, w2) pair, 0
      link_w   [L, 2] float32 (w1, w2) per link, cells in ordinal order, directions ascending;
                           q < 1/2 links without a second node become (1, 0): the
                           plain bounce-back value f_opp(x_f) of the reference
      link_cells [C] int32 cell index of each link cell (ascending)
      counts   [N] links per cell
    Links whose fluid cell is a flow solid are dropped: the reference resets those
    cells right after the bounce-back pass.
    """
    dev = solid_flow_u8.device
    N = nx * ny * nz
    nynz = ny * nz
    ff = ibb.fluid_flat.to(device=dev, dtype=torch.int64).reshape(-1)
    d = ibb.dir_i.to(device=dev, dtype=torch.int64).reshape(-1)
    do = ibb.dir_opp.to(device=dev, dtype=torch.int64).reshape(-1)
    ge = ibb.q_ge_half.to(device=dev).reshape(-1).bool()
    fv = ibb.ff_valid.to(device=dev).reshape(-1).bool()
    fff = ibb.ff_flat.to(device=dev, dtype=torch.int64).reshape(-1)
    w1 = ibb.w_i.to(device=dev, dtype=torch.float32).reshape(-1)
    w2 = ibb.w_second.to(device=dev, dtype=torch.float32).reshape(-1)
    if ff.numel() and (int(ff.min()) < 0 or int(ff.max()) >= N):
        raise ValueError("IBB fluid_flat index out of range")
    if d.numel() and (int(d.min()) < 1 or int(d.max()) > 18):
        raise ValueError("IBB dir_i must lie in 1..18")
    opp = torch.tensor(_OPP, device=dev)
    if not torch.equal(opp[d], do):
        raise ValueError("IBB dir_opp is not the opposite of dir_i")
    cxyz = torch.tensor([[_CX[q] * nynz + _CY[q] * nz + _CZ[q]] for q in range(19)], device=dev).reshape(-1)
    need_ff = (~ge) & fv
    if need_ff.any() and not torch.equal(fff[need_ff], ff[need_ff] - cxyz[d[need_ff]]):
        raise ValueError("IBB ff_flat must be the cell x_f - c_dir for valid second nodes")
    keep = solid_flow_u8.reshape(-1)[ff] == 0
    ff, d, ge, fv, w1, w2 = ff[keep], d[keep], ge[keep], fv[keep], w1[keep], w2[keep]
    key = ff * 32 + d
    if key.numel() != torch.unique(key).numel():
        raise ValueError("IBB links repeat a (cell, direction) pair")
    order = torch.argsort(key)
    ff, d, ge, fv, w1, w2 = ff[order], d[order], ge[order], fv[order], w1[order], w2[order]
    fallback = (~ge) & (~fv)
    w1 = torch.where(fallback, torch.ones_like(w1), w1)
    w2 = torch.where(fallback, torch.zeros_like(w2), w2)
    second_ff = (~ge) & fv
    L = ff.numel()
    cells, inv, counts_c = torch.unique_consecutive(ff, return_inverse=True, return_counts=True)
    C = cells.numel()
    bit = torch.ones_like(d) << d
    dmask = torch.zeros(C, dtype=torch.int64, device=dev).index_add_(0, inv, bit)
    smask = torch.zeros(C, dtype=torch.int64, device=dev).index_add_(0, inv, bit * second_ff.to(torch.int64))
    first = torch.cumsum(counts_c, 0) - counts_c
    hdr = torch.stack([dmask, smask, first, torch.zeros_like(first)], dim=1).to(torch.int32).contiguous()
    link_off = torch.full((N,), -1, dtype=torch.int32, device=dev)
    link_off[cells] = torch.arange(C, device=dev, dtype=torch.int32)
    counts = torch.zeros(N, dtype=torch.int64, device=dev)
    counts[cells] = counts_c
    return {"link_off": link_off, "link_hdr": hdr, "link_w": torch.stack([w1, w2], dim=1).contiguous(),
            "link_cells": cells.to(torch.int32).contiguous(), "counts": counts, "n_links": L}


class FusedLBM:
    def __init__(self, sim):
        self.sim = sim
        cfg = sim.cfg
        dev = sim.device
        nx, ny, nz = sim.nx, sim.ny, sim.nz
        self.N = N = nx * ny * nz
        self.storage = STORAGE[str(getattr(cfg, "lbm_storage", "fp32")).lower()]
        self.storage_name = {0: "fp32", 1: "fp16-shifted", 2: "bf16-shifted"}[self.storage]
        mode = getattr(cfg, "collision", "bgk").lower()
        self.collision = COLLISION.get(mode, 0)
        self.macro_stride = max(1, int(getattr(cfg, "macro_stride", 1)))

        solid = sim._solid_u8.reshape(N)
        flags = solid.clone()
        # links
        self.has_links = bool(getattr(sim, "ibb_data", None) is not None and int(sim.ibb_data.n_links) > 0)
        if self.has_links:
            t = build_link_table(sim.ibb_data, solid, nx, ny, nz)
            self.link_off, self.link_hdr, self.link_w = t["link_off"], t["link_hdr"], t["link_w"]
            self.link_cells = t["link_cells"]
            # bit1 = has links, high nibble = link count (15 = 15 or more; informational)
            flags |= (t["counts"] > 0).to(torch.uint8) * CF_LINK
            flags |= (t["counts"].clamp(max=15).to(torch.uint8) << 4)
            self.n_links = int(t["n_links"])
        else:
            self.link_off = self.link_hdr = self.link_w = None
            self.link_cells = None
            self.n_links = 0
        # link cells are handled inside the main pass unless cfg.lbm_link_pass == "separate"
        self.separate_link_pass = str(getattr(cfg, "lbm_link_pass", "inline")).lower() == "separate"
        # inlet/outlet planes are finished by the plane BC kernels after the fused pass
        f3 = flags.view(nx, ny, nz)
        self.planes = []
        for face, role in resolve_face_roles(cfg).items():
            if role not in ("inlet", "outlet"):
                continue
            ax, pidx, _ = _face_ax_idx_fsign(sim, face)
            iidx = pidx - 1 if pidx > 0 else 1
            sl = [slice(None)] * 3
            sl[ax] = pidx
            f3[tuple(sl)] |= CF_DEFER
            sl[ax] = iidx
            f3[tuple(sl)] |= CF_WRITE_S
            self.planes.append((ax, pidx))
        self.flags = flags.contiguous()
        # sponge: sigma must be a profile along one axis
        self.sponge = None
        self.sponge_axis = 0
        sig = getattr(sim, "_sponge_sigma", None)
        if int(getattr(cfg, "sponge_length", 0)) > 0 and sig is not None:
            ax = int(getattr(sim, "_sponge_axis", 0))
            prof = sig.to(torch.float32).movedim(ax, 0).reshape(sig.shape[ax], -1)
            if not torch.equal(prof, prof[:, :1].expand_as(prof)):
                raise NotImplementedError("sponge sigma must be constant on planes normal to the sponge axis")
            self.sponge = prof[:, 0].contiguous().to(dev)
            self.sponge_axis = ax
        # buffers
        sdt = STORAGE_DTYPE[self.storage]
        self.P = [torch.empty((19, N), dtype=sdt, device=dev) for _ in range(2)]
        self.M = [[torch.empty(N, dtype=torch.float32, device=dev) for _ in range(4)] for _ in range(2)]
        self.dev_err = torch.zeros(1, dtype=torch.int32, device=dev)
        self.periodic = periodic_flags(cfg)
        self.k = 0          # steps taken since priming
        self.cur = 0        # P[cur] holds the latest post-collision populations
        self.primed = False
        self.use_graphs = bool(getattr(cfg, "lbm_cuda_graph", True))
        self._graphs = {}
        self._eager_steps = 0
        self.tracer = None  # a TracerField the main pass advances once per step (attach_tracer sets it)
        self.alternate_order = True   # alternate the staged pass's tile order (and the gathers') per step
        self.args = StepArgs()
        self._fill_static_args()

    # -- argument block ------------------------------------------------------
    def _fill_static_args(self):
        sim, a = self.sim, self.args
        a.storage = self.storage
        a.collision = self.collision
        a.nx, a.ny, a.nz = sim.nx, sim.ny, sim.nz
        for d in range(3):
            a.periodic[d] = int(self.periodic[d])
        a.f32 = ptr(sim.f)
        a.cell_flags = ptr(self.flags)
        a.link_off = ptr(self.link_off)
        a.link_hdr = ptr(self.link_hdr)
        a.link_w = ptr(self.link_w)
        a.n_links = self.n_links
        a.sponge = ptr(self.sponge)
        a.sponge_axis = self.sponge_axis
        a.has_links = int(self.has_links)
        a.phase_mask = 3
        a.separate_link_pass = int(self.separate_link_pass)
        a.cells_per_thread = int(getattr(self.sim.cfg, "lbm_cells_per_thread", 1))
        a.staging = {"tma": 0, "direct": 1}[str(getattr(self.sim.cfg, "lbm_staging", "tma"))]
        a.link_cells = ptr(self.link_cells)
        a.n_link_cells = 0 if self.link_cells is None else int(self.link_cells.numel())
        a.dev_err = ptr(self.dev_err)
        # per-step gathered link values (storage form), the staged pass's tile records
        # and the staged-tile element each link value replaces
        self.link_val = None
        self.tile_links = None
        self.link_pos = None
        self.link_src = None
        N = self.N
        if self.has_links and self.n_links > 0:
            self.link_val = torch.zeros(self.n_links + 8, dtype=STORAGE_DTYPE[self.storage], device=sim.device)
            a.link_val = ptr(self.link_val)
            a.n_link_val = self.link_val.numel()
        nt = 0
        if sim.device.type == "cuda":
            nt = int(_lib.lib().fc_lbm_tile_links(C.byref(a), None, 0, None, 0, None, 0, stream_ptr()))
        if nt > 0:
            self.tile_links = torch.zeros((nt, 8), dtype=torch.int32, device=sim.device)
            pos_ptr, pos_cap, src_ptr, src_cap = None, 0, None, 0
            if self.n_links > 0:
                self.link_pos = torch.zeros(self.n_links + 8, dtype=torch.int16, device=sim.device)
                pos_ptr, pos_cap = ptr(self.link_pos), self.link_pos.numel()
                if 19 * N < 2 ** 31:
                    self.link_src = torch.zeros((self.n_links + 8, 2), dtype=torch.int32, device=sim.device)
                    src_ptr, src_cap = ptr(self.link_src), self.n_links + 8
            got = int(_lib.lib().fc_lbm_tile_links(C.byref(a), ptr(self.tile_links), nt, pos_ptr, pos_cap,
                                                   src_ptr, src_cap, stream_ptr()))
            if got != nt:
                raise RuntimeError(f"fc_lbm_tile_links failed: {got}")
            a.tile_links = ptr(self.tile_links)
            a.n_tile_links = nt
            if self.link_pos is not None:
                a.link_pos = ptr(self.link_pos)
                a.n_link_pos = pos_cap
            if self.link_src is not None:
                a.link_src = ptr(self.link_src)
                a.n_link_src = src_cap
        # The link gather for step k+1 may run on a second stream while step k's plane
        # work runs when no link reads a cell of an inlet/outlet plane.
        # Links that read a cell of such a plane are marked (bit 31 of their second element)
        # and gathered after the plane work.
        self.concurrent_gather = False
        self._side = None
        self.late_links = None
        if self.link_src is not None and self.planes:
            src = self.link_src[: self.n_links].long()
            e1 = (src[:, 0] & 0x7FFFFFFF) % N
            e2 = (src[:, 1] & 0x7FFFFFFF) % N
            defer = (self.flags.long() & CF_DEFER) != 0
            late = defer[e1] | defer[e2]
            if bool(late.any()):
                self.late_links = torch.nonzero(late).flatten().to(torch.int32).contiguous()
                marked = self.link_src[: self.n_links, 1].long() | (1 << 31)
                self.link_src[: self.n_links, 1] = torch.where(late, marked - (1 << 32),
                                                               self.link_src[: self.n_links, 1].long()).to(torch.int32)
            self.concurrent_gather = True
        self.refresh_params()

    def refresh_params(self):
        """Re-read the collision parameters from the solver object."""
        sim, a = self.sim, self.args
        a.omega = float(getattr(sim, "omega", 1.0))
        a.omega_plus = float(getattr(sim, "omega_plus", a.omega))
        a.omega_minus = float(sim.omega_minus) if hasattr(sim, "omega_minus") else 1.0
        S = getattr(sim, "_mrt_S", None)
        vals = [float(x) for x in S.tolist()] if S is not None else [0.0] * 19
        for q in range(19):
            a.S[q] = vals[q]
        a.Cs_dx2 = float(getattr(sim, "_cuda_Cs_dx2", None) or 0.0)
        a.omega0 = float(getattr(sim, "_cuda_omega0", None) or a.omega_plus)

    def _set_macros(self, m):
        a = self.args
        if m is None:
            a.rho = a.u = a.v = a.w = None
        else:
            a.rho, a.u, a.v, a.w = (ptr(t) for t in m)

    def _arm_tracer(self, tr, m):
        """Point the step's tracer arguments at `tr`'s buffers, advected by the velocity in
        macro set m (None clears them)."""
        a = self.args
        if tr is None:
            a.tracer_in = a.tracer_out = a.tracer_u = a.tracer_v = a.tracer_w = a.tracer_solid = None
            return
        a.tracer_in = ptr(tr._buf[tr._cur])
        a.tracer_out = ptr(tr._buf[1 - tr._cur])
        a.tracer_u, a.tracer_v, a.tracer_w = (ptr(t) for t in m[1:])
        a.tracer_solid = ptr(tr._solid_u8)
        a.tracer_dissipation = float(tr.diss)

    def _expose(self, m):
        sim = self.sim
        shp = (sim.nx, sim.ny, sim.nz)
        sim.rho, sim.u, sim.v, sim.wv = (t.view(shp) for t in m)

    def invalidate(self):
        """Forget the stored post-collision state; the next step re-primes from sim.f."""
        self.primed = False
        self._graphs.clear()
        self._eager_steps = 0

    # -- stepping --------------------------------------------------------------
    def _prime(self):
        """P_1 = C(S_0) from sim.f; macros of S_0; solid cells pinned in both buffers."""
        sim, a = self.sim, self.args
        self.refresh_params()
        if sim.f.dtype != torch.float32 or not sim.f.is_contiguous():
            raise RuntimeError("sim.f must be a contiguous float32 tensor")
        a.f32 = ptr(sim.f)
        self._graphs.clear()
        self._eager_steps = 0
        st = stream_ptr()
        for m in self.M:
            for t in m:
                t.zero_()
        for b in range(2):
            a.pop_out = ptr(self.P[b])
            self._set_macros(self.M[b])
            _lib.call("fc_lbm_pin_solid", a, st)
        self.cur = 0
        a.pop_out = ptr(self.P[0])
        self._set_macros(self.M[0])
        _lib.call("fc_lbm_collide_from_f32", a, -1, 0, st)
        if self.concurrent_gather:
            a.pop_in = ptr(self.P[0])
            _lib.call("fc_lbm_link_gather", a, None, 0, 0, st)
        self.k = 0
        self.primed = True

    def _plane_set(self):
        """Fused plane descriptors when every inlet/outlet condition is node-local (Zou/He) on
        distinct planes of one axis, else None (the sequential reference-order path runs)."""
        from .lbm_cuda_ext import _bc_plan
        plan = _bc_plan(self.sim)
        if not plan or len(plan) > 6 or any(b[0] != "zou_he" for b in plan):
            return None
        axes = {b[1] for b in plan}
        pidx = [b[2] for b in plan]
        if len(axes) != 1 or len(set(pidx)) != len(pidx) or any(b[3] in pidx for b in plan):
            return None
        if sorted((b[1], b[2]) for b in plan) != sorted(self.planes):
            return None
        arr = (_lib.PlaneBC * len(plan))()
        for d, (_, ax, p, ii, code, u, rho, sign, _n1, _n2) in zip(arr, plan):
            d.axis, d.plane_idx, d.interior_idx, d.bc_type = ax, p, ii, code
            d.u_in_lat, d.rho_out_lat, d.sign = u, rho, sign
        return arr

    def launches_per_step(self) -> int:
        """Kernels one step launches (main pass, link gathers, link-cell pass, plane work)."""
        n = 1
        if self.link_val is not None:
            n += 1 + (1 if self.late_links is not None and self.concurrent_gather else 0)
        if self.separate_link_pass and self.link_cells is not None:
            n += 1
        if self.planes:
            if self._plane_set() is not None:
                n += 1
            else:
                from .lbm_cuda_ext import _bc_plan
                n += sum(2 if b[0] == "convective" else 1 for b in _bc_plan(self.sim)) + len(self.planes)
        return n

    def _side_stream(self):
        if self._side is None:
            self._side = torch.cuda.Stream(device=self.sim.device)
            self._ev_fork = torch.cuda.Event()
            self._ev_join = torch.cuda.Event()
        return self._side

    def _enqueue(self, cur, m_out, phase_event=None):
        """Launch one step's kernels: fused pass P[cur] -> P[1-cur], then the plane BCs (and,
        concurrently with those, the next step's link gather)."""
        sim, a = self.sim, self.args
        st = stream_ptr()
        a.pop_in = ptr(self.P[cur])
        a.pop_out = ptr(self.P[1 - cur])
        a.f32 = ptr(sim.f)
        self._set_macros(m_out)
        # the staged pass alternates its tile order every step, and each link gather runs opposite
        # to the pass that wrote its input, so both start on what is still in L2
        alt = 1 if self.alternate_order else 0
        a.tile_order = cur * alt
        a.gather_order = cur * alt      # the in-step gather reads P[cur], written in order 1 - cur
        a.skip_link_gather = 1 if self.concurrent_gather else 0
        _lib.call("fc_lbm_fused_step", a, st)
        a.skip_link_gather = 0
        a.gather_order = (1 - cur) * alt   # the gathers below read P[1 - cur], written in order cur
        if phase_event is not None:
            phase_event.record()
        if self.concurrent_gather:
            main = torch.cuda.current_stream()
            side = self._side_stream()
            self._ev_fork.record(main)
            side.wait_event(self._ev_fork)
            a.pop_in = ptr(self.P[1 - cur])   # the next step's input
            _lib.call("fc_lbm_link_gather", a, None, 0, 1, side.cuda_stream)
            a.pop_in = ptr(self.P[cur])
            self._ev_join.record(side)
        if self.planes:
            ps = self._plane_set()
            rc = 3
            if ps is not None:
                rc = _lib.lib().fc_lbm_planes_zou_he_collide(C.byref(a), ps, len(ps), st)
                if rc not in (0, 3):
                    _lib.check(rc, "fc_lbm_planes_zou_he_collide")
            if rc != 0:
                from .lbm_cuda_ext import _apply_flow_bcs_cuda
                _apply_flow_bcs_cuda(sim)
                for ax, pidx in self.planes:
                    _lib.call("fc_lbm_collide_from_f32", a, ax, pidx, st)
        if self.concurrent_gather:
            if self.late_links is not None:
                a.pop_in = ptr(self.P[1 - cur])
                _lib.call("fc_lbm_link_gather", a, ptr(self.late_links), self.late_links.numel(), 0, st)
                a.pop_in = ptr(self.P[cur])
            torch.cuda.current_stream().wait_event(self._ev_join)

    def _graph(self, cur):
        """CUDA graph of one step without macro output, captured on first use (per parity)."""
        key = (cur, self.sim.f.data_ptr())
        g = self._graphs.get(key)
        if g is None:
            g = capture_graph(lambda: self._enqueue(cur, None))
            self._graphs[key] = g
        return g

    def step(self, phase_event=None):
        if not self.primed:
            self._prime()
        k = self.k + 1          # reference step number being completed
        nxt = 1 - self.cur
        write_m = (k % self.macro_stride) == 0
        tr = self.tracer
        if tr is not None:
            # the tracer step that follows step k in the reference reads the macros exposed after
            # step k: the ones the previous step wrote
            self._arm_tracer(tr, self.M[(k - 1) % 2])
        if self.use_graphs and not write_m and phase_event is None and self._eager_steps >= 1 and tr is None:
            self._graph(self.cur).replay()
        else:
            try:
                self._enqueue(self.cur, self.M[k % 2] if write_m else None, phase_event)
            finally:
                if tr is not None:
                    self._arm_tracer(None, None)
            self._eager_steps += 1
            if tr is not None:
                tr._cur = 1 - tr._cur
        self.cur = nxt
        self.k = k
        # the reference exposes the pre-collision macros of this step's input state
        self._expose(self.M[(k - 1) % 2])

    def time_passes(self, n: int):
        """Mean device time (ms) of the main fused pass and of the link-cell pass over n launches,
        measured with CUDA events on the current stream.  Leaves the populations advanced by
        n steps without plane boundary conditions: call it after the measured run."""
        a = self.args
        out = {}
        for name, mask in (("main", 1), ("links", 2)):
            if mask == 2 and not (a.n_link_cells and a.separate_link_pass):
                continue
            a.phase_mask = mask
            a.skip_link_gather = 1 if self.concurrent_gather else 0
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n)]
            cur = self.cur
            for e0, e1 in ev:
                a.pop_in = ptr(self.P[cur])
                a.pop_out = ptr(self.P[1 - cur])
                a.tile_order = cur if self.alternate_order else 0
                self._set_macros(None)
                e0.record()
                _lib.call("fc_lbm_fused_step", a, stream_ptr())
                e1.record()
                cur = 1 - cur
            torch.cuda.synchronize()
            out[name] = sum(e0.elapsed_time(e1) for e0, e1 in ev) / n
        a.phase_mask = 3
        a.skip_link_gather = 0
        return out

    def sync_f(self):
        """Write the current post-stream populations S_k into sim.f."""
        if not self.primed or self.k == 0:
            return
        a = self.args
        a.pop_in = ptr(self.P[1 - self.cur])
        a.f32 = ptr(self.sim.f)
        _lib.call("fc_lbm_materialize", a, stream_ptr())

    def post_collision(self) -> torch.Tensor:
        """Latest post-collision populations as FP32 [19, N] (unshifted)."""
        P = self.P[self.cur]
        if self.storage == 0:
            return P.clone()
        return P.float() + _W.to(P.device)[:, None]

    def check_device_error(self) -> int:
        return int(self.dev_err.item())

    # -- checkpoint support ----------------------------------------------------
    def plane_cells(self) -> torch.Tensor:
        """Cells whose sim.f populations carry state from one step to the next: the deferred
        inlet/outlet plane cells and the cells exporting their post-stream values to them."""
        return torch.nonzero((self.flags & (CF_DEFER | CF_WRITE_S)) != 0).flatten().to(torch.int64)

    def export_state(self) -> dict:
        """Device tensors that determine every later step exactly (no copies are made)."""
        if not self.primed:
            self._prime()
        return {"k": self.k, "P": self.P[self.cur], "M0": torch.stack(self.M[0]), "M1": torch.stack(self.M[1])}

    def import_state(self, k: int, P: torch.Tensor, M0: torch.Tensor, M1: torch.Tensor):
        """Resume from export_state's tensors: the next step continues the saved run bit for bit.
        sim.f must already hold the saved plane-cell populations."""
        sim, a = self.sim, self.args
        if P.shape != self.P[0].shape or P.dtype != self.P[0].dtype:
            raise ValueError("checkpoint populations do not match this engine's storage or size")
        self._prime()                       # static arguments, pinned solid cells in both buffers
        self.P[0].copy_(P)
        for b, Mb in enumerate((M0, M1)):
            for q in range(4):
                self.M[b][q].copy_(Mb[q])
        self.cur = 0
        self.k = int(k)
        self._graphs.clear()
        self._eager_steps = 0
        if self.concurrent_gather:          # link values of the next step come from P_k
            a.pop_in = ptr(self.P[0])
            a.f32 = ptr(sim.f)
            _lib.call("fc_lbm_link_gather", a, None, 0, 0, stream_ptr())
        if self.k > 0:
            self._expose(self.M[(self.k - 1) % 2])


_W = torch.tensor([0.33333333] + [0.05555556] * 6 + [0.02777778] * 12, dtype=torch.float32)
