"""Drop-in replacement for the reference's solver/thermal_cuda_ext.py.

THERMAL_CUDA keeps the reference module functions (solver/thermal_kernels.cu:258-263):
  thermal_rhs(T_old, T0, src_step, LT0, mask_f, rhs, theta0, dt)
  thermal_reconstruct(T0, theta, nx, ny, nz, ax, out_idx) -> new T
  convergence_metrics(T_new, T_old, solid_u8) -> [dT_solid_max (1,), dT_fluid_max (1,)]
  physics_check(T, T_min, T_max) -> int32 flag tensor (1,)
`_temperature_step_mg_fused(self, dt, tol, max_cycles)` and
`patch_thermal_fused(sim)` follow thermal_cuda_ext.py:55-234: the Dirichlet
lifting field, update mask and volumetric source are cached; the right-hand
side, the reconstruction with Neumann faces, the physics range check, the
convergence metrics and the steady residual each run as one native kernel.
"""
from __future__ import annotations

import types

import torch

from .. import _lib
from .._torch import ptr, require, stream_ptr


class _ThermalKernels:
    def _ws(self, n, device):
        need = int(_lib.call("fc_thermal_workspace_bytes", n))
        ws = getattr(self, "_wsbuf", None)
        if ws is None or ws.numel() < need or ws.device != device:
            ws = torch.empty(need, dtype=torch.uint8, device=device)
            self._wsbuf = ws
        return ws

    def thermal_rhs(self, T_old, T0, src_step, LT0, mask_float, rhs, theta0, dt):
        n = T_old.numel()
        for t, nm in ((T_old, "T_old"), (T0, "T0"), (src_step, "src_step"), (LT0, "LT0"),
                      (mask_float, "mask_float"), (rhs, "rhs"), (theta0, "theta0")):
            require(t, nm, torch.float32, n)
        _lib.call("fc_thermal_rhs", ptr(T_old), ptr(T0), ptr(src_step), ptr(LT0), ptr(mask_float), ptr(rhs),
                  ptr(theta0), float(dt), n, stream_ptr())

    def thermal_reconstruct(self, T0, theta, nx, ny, nz, ax, out_idx):
        require(T0, "T0", torch.float32)
        require(theta, "theta", torch.float32, T0.numel())
        T_new = torch.empty_like(T0)
        _lib.call("fc_thermal_reconstruct", ptr(T0), ptr(theta), ptr(T_new), int(nx), int(ny), int(nz), int(ax),
                  int(out_idx), stream_ptr())
        return T_new

    def convergence_metrics(self, T_new, T_old, solid_u8):
        n = T_new.numel()
        require(T_new, "T_new", torch.float32)
        require(T_old, "T_old", torch.float32, n)
        require(solid_u8, "solid_u8", torch.uint8, n)
        ws = self._ws(n, T_new.device)
        out = torch.empty(2, dtype=torch.float32, device=T_new.device)
        _lib.call("fc_thermal_convergence_metrics", ptr(T_new), ptr(T_old), ptr(solid_u8), n, ptr(ws), ws.numel(),
                  ptr(out), stream_ptr())
        return [out[0:1], out[1:2]]

    def physics_check(self, T, T_min, T_max):
        require(T, "T", torch.float32)
        flag = torch.zeros(1, dtype=torch.int32, device=T.device)
        _lib.call("fc_thermal_physics_check", ptr(T), ptr(flag), float(T_min), float(T_max), T.numel(),
                  stream_ptr())
        return flag

    def steady_residual(self, mg, T, src_step, mask_f, dt):
        lv = mg._levels[0]
        nx, ny, nz = lv["shape"]
        n = T.numel()
        ws = self._ws(n, T.device)
        out = torch.empty(2, dtype=torch.float32, device=T.device)
        _lib.call("fc_thermal_steady_residual", ptr(T), *mg._cptrs(lv), ptr(src_step), ptr(mask_f), float(dt), nx,
                  ny, nz, mg.ax, lv["out_idx"], ptr(ws), ws.numel(), ptr(out), stream_ptr())
        return out


THERMAL_CUDA = _ThermalKernels()
THERMAL_CUDA_AVAILABLE = torch.cuda.is_available() and _lib.load_error() is None


def _temperature_step_mg_fused(self, dt: float, tol: float = 1e-3, max_cycles: int = 20) -> dict:
    """One pseudo-time step A theta = rhs, A = I + dt L, T = T0 + theta (thermal_cuda_ext.py:55-201)."""
    from .nlevel_mg_cuda import NLevelGeometricMGSolver

    dt = float(dt)
    T_old = self.T
    if not hasattr(self, "_cached_thermal_setup"):
        update_mask = self._build_update_mask_thermal()
        T0 = self._build_T_dirichlet_field()
        src_vol = self._compute_heat_source() if hasattr(self, "_compute_heat_source") else None
        if src_vol is None:
            src_vol = torch.zeros_like(T_old)
        ax, sign = self.ax, self.sign
        n_ax = (self.nx, self.ny, self.nz)[ax]
        self._cached_thermal_setup = dict(
            update_mask=update_mask, T0=T0.contiguous(), src_vol=src_vol, mask_f=update_mask.to(T_old.dtype).contiguous(),
            solid_u8=self.solid.to(torch.uint8).contiguous(), out_idx=(n_ax - 1 if sign == +1 else 0))
    cs = self._cached_thermal_setup
    T0, mask_f, solid_u8, out_idx = cs["T0"], cs["mask_f"], cs["solid_u8"], cs["out_idx"]
    src_step = cs["src_vol"]
    if hasattr(self, "_compute_surface_flux_sources"):
        src_step = src_step + self._compute_surface_flux_sources()
    src_step = src_step.contiguous()
    if not hasattr(self, "_mg_solver"):
        self._mg_solver = NLevelGeometricMGSolver(
            device=T_old.device, dtype=T_old.dtype, flow_axis=self.ax, flow_sign=self.sign,
            thermal_dt_scale=float(self.thermal_dt_scale), omega=float(getattr(self.cfg, "mg_omega", 0.8)),
            n_pre=int(getattr(self.cfg, "mg_pre_smooth", 2)), n_post=int(getattr(self.cfg, "mg_post_smooth", 2)),
            n_coarse=int(getattr(self.cfg, "mg_coarse_iters", 20)), min_coarse_cells=4)
    mg = self._mg_solver
    mg.build_if_needed(k=self.k, rho_cp=self.rho_cp, u=self.u, v=self.v, w=self.wv, mask=cs["update_mask"], dt=dt)
    LT0 = mg.L_apply_fine(T0)
    # rhs = mask ((T_old + dt src) - (T0 + dt LT0)); theta0 = mask (T_old - T0)
    ALT0 = torch.empty_like(T0)
    _lib.call("fc_vec_axpby", 0, ptr(ALT0), ptr(LT0), T0.numel(), dt, None, None, 0.0, None, stream_ptr())
    _lib.call("fc_vec_axpby", 0, ptr(ALT0), ptr(T0), T0.numel(), 1.0, None, None, 1.0, None, stream_ptr())
    rhs = torch.empty_like(T0)
    theta0 = torch.empty_like(T0)
    THERMAL_CUDA.thermal_rhs(T_old.contiguous(), T0, src_step, ALT0, mask_f, rhs, theta0, dt)
    theta, info = mg.solve(b=rhs, x0=theta0, max_cycles=max_cycles, tol=tol)
    Tin = float(self.fluid.tin_C)
    cand = torch.empty_like(T0)
    _lib.call("fc_vec_axpby", 0, ptr(cand), ptr(theta), T0.numel(), 1.0, None, None, 0.0, ptr(mask_f), stream_ptr())
    _lib.call("fc_vec_axpby", 0, ptr(cand), ptr(T0), T0.numel(), 1.0, None, None, 1.0, None, stream_ptr())
    flag = THERMAL_CUDA.physics_check(cand, Tin - 500.0, Tin + 2000.0)
    T_new = THERMAL_CUDA.thermal_reconstruct(T0, theta, self.nx, self.ny, self.nz, self.ax, out_idx)
    if int(flag.item()):
        return dict(converged=False, it=info["it"], res_rel=info["res_rel"], r_rel=float("inf"),
                    r_inf=float("inf"), src_inf=float("nan"), Tmax=float("nan"), diverged=True)
    self.T = T_new
    rs, rf = THERMAL_CUDA.convergence_metrics(T_new, T_old.contiguous(), solid_u8)
    self._async_dT_solid = rs
    self._async_dT_fluid = rf
    res = THERMAL_CUDA.steady_residual(mg, self.T, src_step, mask_f, dt).tolist()
    r_inf, src_inf = res[0], (res[1] if res[1] > 0 else 1e-30)
    return dict(converged=info["converged"], it=info["it"], res_rel=info["res_rel"],
                r_rel=r_inf / max(src_inf, 1e-30), r_inf=r_inf, src_inf=src_inf,
                Tmax=float(torch.amax(self.T).item()))


def patch_thermal_fused(sim):
    """Bind _temperature_step_mg_fused as sim._temperature_step_mg (thermal_cuda_ext.py:204-234)."""
    if not THERMAL_CUDA_AVAILABLE:
        raise RuntimeError("[THERMAL_CUDA] native library or CUDA unavailable; no fallback path exists")
    sim._temperature_step_mg = types.MethodType(_temperature_step_mg_fused, sim)
    print("[THERMAL_FUSED] Patched _temperature_step_mg with fluxcore3d_gb300 kernels.")
