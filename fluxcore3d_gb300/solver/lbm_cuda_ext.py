"""Drop-in replacement for the reference's solver/lbm_cuda_ext.py.

Module surface kept from the reference (solver/lbm_cuda_ext.py):
  LBM_CUDA, LBM_CUDA_AVAILABLE              (:51-94)
  _prepare_ibb_tensors(ibb_data, device, dtype)   (:100-123)
  LBMCUDAUpgrade.patch(sim)                 (:151-265)
  _apply_flow_bcs_cuda(sim)                 (:628-687)
  add_step_profiler(sim, print_every)       (:693-748)

`LBM_CUDA` exposes the reference module functions with the same argument
order and meaning, backed by the sm_103a kernels of libfluxcore3d_gb300.so.
`LBMCUDAUpgrade.patch(sim)` sets the same attributes and bound methods on the
solver object as the reference, but `sim.step()` runs the fused step engine
(fused_lbm.FusedLBM): one pass per step instead of 6-9 launches.  Differences a
caller can observe are listed on FusedLBM.

There is no torch fallback: without the native library or without CUDA,
`LBM_CUDA_AVAILABLE` is False and `patch` raises instead of silently running
something else.
"""
from __future__ import annotations

import types

import torch

from .. import _lib
from .._torch import ptr, require, stream_ptr
from .face_roles import _face_ax_idx_fsign, periodic_flags, resolve_face_roles

__all__ = [
    "LBM_CUDA", "LBM_CUDA_AVAILABLE", "LBMCUDAUpgrade", "_prepare_ibb_tensors",
    "_apply_flow_bcs_cuda", "add_step_profiler",
]


class _LBMKernels:
    """Reference LBM_CUDA call surface (solver/lbm_kernels.cu:1347-1386)."""

    @staticmethod
    def _collide_checks(f, f_post, rho, u, v, w, solid):
        require(f, "f", torch.float32)
        N = f_post.numel() // 19
        for t, n in ((f_post, "f_post"), (rho, "rho_out"), (u, "u_out"), (v, "v_out"), (w, "w_out")):
            require(t, n, torch.float32)
        require(solid, "solid", torch.uint8)
        if f.numel() != 19 * N or rho.numel() != N or solid.numel() != N:
            raise RuntimeError("population / macro / solid sizes disagree")
        return N

    def macro_collide_bgk(self, f, f_post, rho, u, v, w, solid, omega):
        N = self._collide_checks(f, f_post, rho, u, v, w, solid)
        _lib.call("fc_lbm_macro_collide_bgk", ptr(f), ptr(f_post), ptr(rho), ptr(u), ptr(v), ptr(w),
                  ptr(solid), float(omega), N, stream_ptr())

    def macro_collide_trt(self, f, f_post, rho, u, v, w, solid, omega_plus, omega_minus):
        N = self._collide_checks(f, f_post, rho, u, v, w, solid)
        _lib.call("fc_lbm_macro_collide_trt", ptr(f), ptr(f_post), ptr(rho), ptr(u), ptr(v), ptr(w),
                  ptr(solid), float(omega_plus), float(omega_minus), N, stream_ptr())

    def macro_collide_mrt(self, f, f_post, rho, u, v, w, solid, S_rates):
        N = self._collide_checks(f, f_post, rho, u, v, w, solid)
        require(S_rates, "S_rates", torch.float32, 19)
        _lib.call("fc_lbm_macro_collide_mrt", ptr(f), ptr(f_post), ptr(rho), ptr(u), ptr(v), ptr(w),
                  ptr(solid), ptr(S_rates), N, stream_ptr())

    def macro_collide_mrt_smag(self, f, f_post, rho, u, v, w, solid, S_rates, Cs_dx2, omega0):
        N = self._collide_checks(f, f_post, rho, u, v, w, solid)
        require(S_rates, "S_rates", torch.float32, 19)
        _lib.call("fc_lbm_macro_collide_mrt_smag", ptr(f), ptr(f_post), ptr(rho), ptr(u), ptr(v), ptr(w),
                  ptr(solid), ptr(S_rates), float(Cs_dx2), float(omega0), N, stream_ptr())

    def stream_pull(self, f_in, f_out, nx, ny, nz, periodic_x, periodic_y, periodic_z):
        require(f_in, "f_in", torch.float32)
        require(f_out, "f_out", torch.float32)
        if f_in.numel() != 19 * nx * ny * nz or f_out.numel() != f_in.numel():
            raise RuntimeError("f_in / f_out must hold 19*nx*ny*nz values")
        _lib.call("fc_lbm_stream_pull", ptr(f_in), ptr(f_out), int(nx), int(ny), int(nz),
                  int(periodic_x), int(periodic_y), int(periodic_z), stream_ptr())

    def sponge(self, f, rho, u, v, w, sigma):
        require(f, "f", torch.float32)
        N = rho.numel()
        for t, n in ((rho, "rho"), (u, "u"), (v, "v"), (w, "w"), (sigma, "sigma")):
            require(t, n, torch.float32, N)
        _lib.call("fc_lbm_sponge", ptr(f), ptr(rho), ptr(u), ptr(v), ptr(w), ptr(sigma), N, stream_ptr())

    def ibb(self, f_post, f_stream, fluid_flat, dir_i, dir_opp, w1, w2, q_ge_half, ff_flat, ff_valid,
            dev_err=None):
        require(f_post, "f_post", torch.float32)
        require(f_stream, "f_stream", torch.float32)
        n = fluid_flat.numel()
        if n == 0:
            return
        for t, nm, dt in ((fluid_flat, "fluid_flat", torch.int32), (dir_i, "dir_i", torch.int32),
                          (dir_opp, "dir_opp", torch.int32), (w1, "w1", torch.float32),
                          (w2, "w2", torch.float32), (q_ge_half, "q_ge_half", torch.uint8),
                          (ff_flat, "ff_flat", torch.int32), (ff_valid, "ff_valid", torch.uint8)):
            require(t, nm, dt, n)
        _lib.call("fc_lbm_ibb", ptr(f_post), ptr(f_stream), ptr(fluid_flat), ptr(dir_i), ptr(dir_opp),
                  ptr(w1), ptr(w2), ptr(q_ge_half), ptr(ff_flat), ptr(ff_valid), n, f_post.numel() // 19,
                  ptr(dev_err), stream_ptr())

    def reset_solid(self, f, solid):
        require(f, "f", torch.float32)
        require(solid, "solid", torch.uint8)
        _lib.call("fc_lbm_reset_solid", ptr(f), ptr(solid), solid.numel(), stream_ptr())

    def zou_he_bc(self, f, solid, nx, ny, nz, axis, plane_idx, interior_idx, bc_type, u_in_lat,
                  rho_out_lat, sign):
        require(f, "f", torch.float32)
        require(solid, "solid", torch.uint8)
        _lib.call("fc_lbm_zou_he_bc", ptr(f), ptr(solid), int(nx), int(ny), int(nz), int(axis),
                  int(plane_idx), int(interior_idx), int(bc_type), float(u_in_lat), float(rho_out_lat),
                  int(sign), stream_ptr())

    def convective_bc(self, f, solid, nx, ny, nz, axis, outlet_idx, interior_idx, unknown_cax,
                      rho_out_lat, n1, n2, workspace=None):
        require(f, "f", torch.float32)
        require(solid, "solid", torch.uint8)
        need = _lib.call("fc_lbm_convective_workspace_bytes", int(n1), int(n2))
        if need < 0:
            raise RuntimeError("convective_bc: bad plane size")
        if workspace is None or workspace.numel() < need:
            workspace = torch.empty(int(need), dtype=torch.uint8, device=f.device)
        _lib.call("fc_lbm_convective_bc", ptr(f), ptr(solid), int(nx), int(ny), int(nz), int(axis),
                  int(outlet_idx), int(interior_idx), int(unknown_cax), float(rho_out_lat), int(n1), int(n2),
                  ptr(workspace), workspace.numel(), stream_ptr())


def _available() -> bool:
    return torch.cuda.is_available() and _lib.load_error() is None


LBM_CUDA = _LBMKernels()
LBM_CUDA_AVAILABLE = _available()


def _require_available():
    if not torch.cuda.is_available():
        raise RuntimeError("[LBM_CUDA] CUDA is not available; fluxcore3d_gb300 has no CPU path")
    _lib.lib()


def _prepare_ibb_tensors(ibb_data, device, dtype):
    """int32 / float32 / uint8 copies of the link arrays, cached on ibb_data._cuda_tensors
    (reference solver/lbm_cuda_ext.py:100-123)."""
    if hasattr(ibb_data, "_cuda_tensors"):
        return ibb_data._cuda_tensors

    def _to(t, dt):
        return t.to(device=device, dtype=dt).contiguous()

    t = types.SimpleNamespace(
        fluid_flat=_to(ibb_data.fluid_flat, torch.int32),
        dir_i=_to(ibb_data.dir_i, torch.int32),
        dir_opp=_to(ibb_data.dir_opp, torch.int32),
        w_i=_to(ibb_data.w_i, torch.float32),
        w_second=_to(ibb_data.w_second, torch.float32),
        q_ge_half=_to(ibb_data.q_ge_half.to(torch.uint8), torch.uint8),
        ff_flat=_to(ibb_data.ff_flat, torch.int32),
        ff_valid=_to(ibb_data.ff_valid.to(torch.uint8), torch.uint8),
    )
    ibb_data._cuda_tensors = t
    return t


def _has_links(sim) -> bool:
    d = getattr(sim, "ibb_data", None)
    return d is not None and int(d.n_links) > 0


class LBMCUDAUpgrade:
    """Patches a LBMCHT3D_Torch-like solver object in place (call after FlowSolverUpgrade.patch)."""

    @staticmethod
    def patch(sim):
        _require_available()
        from .fused_lbm import FusedLBM

        cfg = sim.cfg
        sim._solid_u8 = sim.solid_flow.to(dtype=torch.uint8, device=sim.device).contiguous()
        mode = getattr(cfg, "collision", "bgk").lower()
        sim._S_cuda = (sim._mrt_S.to(device=sim.device, dtype=torch.float32).contiguous()
                       if mode in ("mrt", "mrt_smag") else None)
        if mode == "mrt_smag":
            Cs = float(getattr(cfg, "smag_Cs", 0.1))
            sim._cuda_Cs_dx2 = float(Cs ** 2)
            sim._cuda_omega0 = float(sim.omega_plus)
        else:
            sim._cuda_Cs_dx2 = None
            sim._cuda_omega0 = None
        if not hasattr(sim, "_f_post") or sim._f_post.shape != sim.f.shape:
            sim._f_post = torch.empty_like(sim.f)
        sim._f_stream = None
        sim._cuda_periodic = periodic_flags(cfg)
        has_sponge = int(getattr(cfg, "sponge_length", 0)) > 0 and hasattr(sim, "_sponge_sigma")
        sim._sponge_sigma_flat = sim._sponge_sigma.reshape(-1).contiguous() if has_sponge else None

        sim._macroscopic_python = sim._macroscopic
        sim._macroscopic = types.MethodType(LBMCUDAUpgrade._macroscopic_noop, sim)
        sim._collide = types.MethodType(LBMCUDAUpgrade._make_collide(mode), sim)
        sim._stream = types.MethodType(LBMCUDAUpgrade._stream_cuda, sim)
        if _has_links(sim):
            _prepare_ibb_tensors(sim.ibb_data, sim.device, sim.dtype)
            sim._interp_bounce_back_from_post = types.MethodType(LBMCUDAUpgrade._ibb_cuda, sim)
        if has_sponge:
            sim._apply_sponge_zone = types.MethodType(LBMCUDAUpgrade._sponge_cuda, sim)
        sim._apply_flow_bcs = types.MethodType(_apply_flow_bcs_cuda, sim)
        sim._original_step_thermal = sim.step
        sim._cuda_debug_nan = bool(getattr(cfg, "cuda_debug_nan", False))

        sim._fc = FusedLBM(sim)
        sim.step = types.MethodType(LBMCUDAUpgrade._step_fused, sim)
        sim.sync_f = types.MethodType(lambda s: s._fc.sync_f(), sim)
        print(f"[LBM_CUDA] fluxcore3d_gb300 fused step: collision={mode} storage={sim._fc.storage_name} "
              f"links={sim._fc.n_links} periodic={sim._cuda_periodic} deferred_planes={len(sim._fc.planes)}")

    # -- single-operation methods (reference semantics, per-op kernels) ------
    @staticmethod
    def _macroscopic_noop(sim_self):
        pass

    @staticmethod
    def _make_collide(mode: str):
        def _collide(sim_self):
            N = sim_self.nx * sim_self.ny * sim_self.nz
            f = sim_self.f.reshape(19, N).contiguous()
            fp = sim_self._f_post.reshape(19, N)
            args = (f, fp, sim_self.rho.reshape(N), sim_self.u.reshape(N), sim_self.v.reshape(N),
                    sim_self.wv.reshape(N), sim_self._solid_u8.reshape(N))
            if mode == "trt":
                LBM_CUDA.macro_collide_trt(*args, float(sim_self.omega_plus), float(sim_self.omega_minus))
            elif mode == "mrt":
                LBM_CUDA.macro_collide_mrt(*args, sim_self._S_cuda)
            elif mode == "mrt_smag":
                LBM_CUDA.macro_collide_mrt_smag(*args, sim_self._S_cuda, float(sim_self._cuda_Cs_dx2),
                                                float(sim_self._cuda_omega0))
            else:
                LBM_CUDA.macro_collide_bgk(*args, float(sim_self.omega))
            # the collide kernels already write (1,0,0,0) macros at flow-solid cells
        return _collide

    @staticmethod
    def _stream_cuda(sim_self):
        px, py, pz = sim_self._cuda_periodic
        LBM_CUDA.stream_pull(sim_self._f_post.contiguous(), sim_self.f, sim_self.nx, sim_self.ny,
                             sim_self.nz, int(px), int(py), int(pz))

    @staticmethod
    def _ibb_cuda(sim_self, f_post):
        ibb = sim_self.ibb_data
        if ibb.n_links == 0:
            return
        t = ibb._cuda_tensors
        N = sim_self.nx * sim_self.ny * sim_self.nz
        LBM_CUDA.ibb(f_post.reshape(19, N).contiguous(), sim_self.f.reshape(19, N), t.fluid_flat, t.dir_i,
                     t.dir_opp, t.w_i, t.w_second, t.q_ge_half, t.ff_flat, t.ff_valid)
        LBM_CUDA.reset_solid(sim_self.f.reshape(19, N), sim_self._solid_u8.reshape(N))

    @staticmethod
    def _sponge_cuda(sim_self, target_f=None):
        if sim_self._sponge_sigma_flat is None:
            return
        N = sim_self.nx * sim_self.ny * sim_self.nz
        f = (target_f if target_f is not None else sim_self.f).reshape(19, N)
        LBM_CUDA.sponge(f, sim_self.rho.reshape(N), sim_self.u.reshape(N), sim_self.v.reshape(N),
                        sim_self.wv.reshape(N), sim_self._sponge_sigma_flat)

    @staticmethod
    def _step_unfused(sim_self, do_thermal: bool = True):
        """The reference launch sequence (collide, sponge, stream, ibb/reset, BCs) on the
        per-operation kernels; kept for A/B measurements against the fused step."""
        sim_self._fc.sync_f()
        sim_self._fc.invalidate()
        sim_self._collide()
        if sim_self._sponge_sigma_flat is not None:
            sim_self._apply_sponge_zone(sim_self._f_post)
        sim_self._stream()
        if _has_links(sim_self):
            sim_self._interp_bounce_back_from_post(sim_self._f_post)
        else:
            sim_self._bounce_back_post_stream()
        sim_self._apply_flow_bcs()
        return (0, 0)

    @staticmethod
    def _step_fused(sim_self, do_thermal: bool = True):
        sim_self._fc.step()
        if sim_self._cuda_debug_nan:
            sim_self._fc.sync_f()
            if not torch.isfinite(sim_self.f).all():
                bad = torch.nonzero(~torch.isfinite(sim_self.f), as_tuple=False)[0]
                print("[LBM_CUDA NaN] after BCs: (q,x,y,z)=", tuple(int(v) for v in bad.tolist()))
                raise FloatingPointError("Non-finite f after BCs")
        if do_thermal and hasattr(sim_self, "_original_step_thermal"):
            return sim_self._original_step_thermal()
        return (0, 0)


def _bc_plan(sim):
    """Ordered list of plane BC calls (reference _apply_flow_bcs_cuda, lbm_cuda_ext.py:628-687)."""
    cfg = sim.cfg
    u_max = float(getattr(cfg, "u_lat_max", 0.5))
    rho_out = float(cfg.rho_out_lat)
    fdir = cfg.flow_dir.upper().strip()
    flow_sign = +1 if fdir[0] == "+" else -1
    flow_axis = {"X": 0, "Y": 1, "Z": 2}[fdir[1]]
    u_signed = float(max(-u_max, min(u_max, float(sim.u_in_lat) * flow_sign)))
    outlet_mode = getattr(cfg, "outlet_bc_mode", "pressure").lower()
    dims = {0: (sim.ny, sim.nz), 1: (sim.nx, sim.nz), 2: (sim.nx, sim.ny)}
    plan = []
    for face, role in resolve_face_roles(cfg).items():
        if role not in ("inlet", "outlet"):
            continue
        ax, plane_idx, fsign = _face_ax_idx_fsign(sim, face)
        interior_idx = plane_idx - 1 if plane_idx > 0 else 1
        n1, n2 = dims[ax]
        if role == "inlet":
            plan.append(("zou_he", ax, plane_idx, interior_idx, 0, u_signed, rho_out, flow_sign, n1, n2))
        elif outlet_mode == "convective" and ax == flow_axis:
            unknown = +1 if plane_idx == 0 else -1
            plan.append(("convective", ax, plane_idx, interior_idx, unknown, u_signed, rho_out, fsign, n1, n2))
        else:
            plan.append(("zou_he", ax, plane_idx, interior_idx, 1, u_signed, rho_out, fsign, n1, n2))
    return plan


def _apply_flow_bcs_cuda(sim_self):
    """Plane boundary conditions on sim.f in the reference face order."""
    N = sim_self.nx * sim_self.ny * sim_self.nz
    f = sim_self.f.reshape(19, N)
    s = sim_self._solid_u8.reshape(N)
    for kind, ax, pidx, iidx, code, u_signed, rho_out, sign, n1, n2 in _bc_plan(sim_self):
        if kind == "zou_he":
            LBM_CUDA.zou_he_bc(f, s, sim_self.nx, sim_self.ny, sim_self.nz, ax, pidx, iidx, code, u_signed,
                               rho_out, sign)
        else:
            ws = getattr(sim_self, "_fc_conv_ws", None)
            need = _lib.call("fc_lbm_convective_workspace_bytes", int(n1), int(n2))
            if ws is None or ws.numel() < need:
                ws = torch.empty(int(need), dtype=torch.uint8, device=sim_self.f.device)
                sim_self._fc_conv_ws = ws
            LBM_CUDA.convective_bc(f, s, sim_self.nx, sim_self.ny, sim_self.nz, ax, pidx, iidx, code, rho_out,
                                   n1, n2, workspace=ws)


def add_step_profiler(sim, print_every: int = 200):
    """Per-phase step timer with CUDA events on the current stream (reference lbm_cuda_ext.py:693-748
    times with host syncs; here the phases are the fused pass and the plane BC work)."""
    sim._prof = {"fused": 0.0, "planes": 0.0, "total": 0.0, "n": 0}

    def _timed_step(self, do_thermal=True):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        ev[0].record()
        self._fc.step(phase_event=ev[1])
        ev[2].record()
        ev[2].synchronize()
        p = self._prof
        p["fused"] += ev[0].elapsed_time(ev[1])
        p["planes"] += ev[1].elapsed_time(ev[2])
        p["total"] += ev[0].elapsed_time(ev[2])
        p["n"] += 1
        if p["n"] % print_every == 0:
            n = p["n"]
            print(f"[PROFILE] {n} steps  (ms/step)")
            for k in ("fused", "planes", "total"):
                print(f"  {k:10s}: {p[k] / n:.4f} ms")
            print(f"  it/s      : {1e3 * n / p['total']:.1f}")
        if do_thermal and hasattr(self, "_original_step_thermal"):
            return self._original_step_thermal()
        return (0, 0)

    sim.step = types.MethodType(_timed_step, sim)
    print(f"[PROFILER] Injected. Prints every {print_every} steps.")
