"""Lattice-unit solver state with the attribute surface of the reference's
LBMCHT3D_Torch (LBM_CHT.py:525-729), so that the drop-in patch layer can be
driven, tested and benchmarked without the reference package.

Only the state the hot path reads is built: populations, macro fields, flow
and thermal solid masks, relaxation rates, MRT rates (flow_solver_upgrade.py:
216-274), the outlet sponge profile (flow_solver_upgrade.py:327-377), the
interpolated-bounce-back link data and the thermal material fields.  The
configuration object carries the reference's SimConfig3D attribute names.
"""
from __future__ import annotations

import math
import types
from dataclasses import dataclass, field

import numpy as np
import torch

from . import geometry as geo

W_CUDA = torch.tensor([0.33333333] + [0.05555556] * 6 + [0.02777778] * 12, dtype=torch.float32)
_C = torch.tensor(geo.C_NP, dtype=torch.float32)


@dataclass
class CaseConfig:
    nx: int = 64
    ny: int = 32
    nz: int = 32
    flow_dir: str = "+X"
    flow_bc: str = "inlet_outlet"
    transverse_walls: bool = False
    domain_walls: list = field(default_factory=list)
    domain_outlets: list = field(default_factory=list)
    collision: str = "bgk"
    trt_lambda: float = 0.1875
    rho_out_lat: float = 1.0
    u_lat_max: float = 0.12
    outlet_bc_mode: str = "pressure"
    sponge_length: int = 0
    sponge_strength: float = 0.3
    mrt_s_e: float = 1.19
    mrt_s_bulk: float = 1.4
    mrt_s_ghost: float = 1.2
    smag_Cs: float = 0.10
    cuda_debug_nan: bool = False
    lbm_storage: str = "fp32"
    macro_stride: int = 1
    temp_bc: str = "fixed"
    mg_omega: float = 0.6
    mg_pre_smooth: int = 2
    mg_post_smooth: int = 2
    mg_coarse_iters: int = 20


def equilibrium(rho, u, v, w, weights=W_CUDA):
    c = _C.to(rho.device)
    wt = weights.to(rho.device, rho.dtype)
    cu = 3.0 * (c[:, 0, None, None, None] * u + c[:, 1, None, None, None] * v + c[:, 2, None, None, None] * w)
    u2 = u * u + v * v + w * w
    return wt[:, None, None, None] * rho * (1.0 + cu + 0.5 * cu * cu - 1.5 * u2)


class LatticeCase:
    """Solver state in lattice units (dx = dt = 1)."""

    def __init__(self, cfg: CaseConfig, u_in_lat: float, nu_lat: float, solid: torch.Tensor,
                 solid_flow: torch.Tensor | None = None, ibb_data=None, device="cuda", seed: int | None = 0,
                 rho_noise: float = 1e-4, k_ratio: float = 100.0, prandtl: float = 0.71):
        self.cfg = cfg
        self.device = torch.device(device)
        self.dtype = torch.float32
        self.nx, self.ny, self.nz = cfg.nx, cfg.ny, cfg.nz
        nx, ny, nz = self.nx, self.ny, self.nz
        self.u_in_lat = float(u_in_lat)
        self.nu_lat = float(nu_lat)
        self.tau_plus = 0.5 + 3.0 * nu_lat
        self.omega_plus = torch.tensor(1.0 / self.tau_plus, dtype=torch.float32)
        self.omega = self.omega_plus
        if cfg.collision == "trt":
            tau_minus = 0.5 + cfg.trt_lambda / (self.tau_plus - 0.5)
            self.omega_minus = torch.tensor(1.0 / tau_minus, dtype=torch.float32)
        self.solid = solid.to(self.device).bool()
        sf = self.solid.clone() if solid_flow is None else solid_flow.to(self.device).bool()
        self.solid_flow = sf
        self.ibb_data = ibb_data
        g = torch.Generator().manual_seed(seed) if seed is not None else None
        rho0 = torch.ones((nx, ny, nz), dtype=torch.float32)
        if seed is not None and rho_noise > 0:
            rho0 = rho0 + (torch.rand((nx, ny, nz), generator=g, dtype=torch.float32) * 2 - 1) * rho_noise
        self.rho = rho0.to(self.device)
        self.u = torch.zeros((nx, ny, nz), device=self.device)
        self.v = torch.zeros_like(self.u)
        self.wv = torch.zeros_like(self.u)
        self.f = equilibrium(self.rho, self.u, self.v, self.wv).contiguous()
        if cfg.collision in ("mrt", "mrt_smag"):
            S = torch.zeros(19, dtype=torch.float32)
            S[[9, 11, 13, 14, 15]] = float(self.omega_plus)
            S[1] = cfg.mrt_s_e
            S[[2, 4, 6, 8, 10, 12]] = cfg.mrt_s_bulk
            S[[16, 17, 18]] = cfg.mrt_s_ghost
            self._mrt_S = S.to(self.device)
        if cfg.sponge_length > 0:
            self._init_sponge()
        # thermal material fields (lattice-scaled as LBM_CHT.py:680-687)
        pr = float(prandtl)
        alpha_f = self.nu_lat / pr
        self.rho_cp = torch.ones((nx, ny, nz), device=self.device)
        self.k = torch.full((nx, ny, nz), alpha_f, device=self.device)
        self.k[self.solid] = alpha_f * float(k_ratio)
        self.T = torch.full((nx, ny, nz), 25.0, device=self.device)
        self.thermal_dt_scale = 1.0
        self.fluid = types.SimpleNamespace(tin_C=25.0)

    def _init_sponge(self):
        """Quadratic outlet ramp (flow_solver_upgrade.py:327-377)."""
        cfg = self.cfg
        d = cfg.flow_dir.upper().strip()
        sign = 1 if d[0] == "+" else -1
        axis = "XYZ".index(d[1])
        n = (self.nx, self.ny, self.nz)[axis]
        out = n - 1 if sign > 0 else 0
        L = int(cfg.sponge_length)
        sig = np.zeros((self.nx, self.ny, self.nz), dtype=np.float32)
        for kk in range(L):
            ramp = ((kk + 1) / L) ** 2 * float(cfg.sponge_strength)
            c = out - (L - 1 - kk) if sign > 0 else out + (L - 1 - kk)
            if 0 <= c < n:
                sl = [slice(None)] * 3
                sl[axis] = c
                sig[tuple(sl)] = ramp
        self._sponge_sigma = torch.tensor(sig, device=self.device)
        self._sponge_axis = axis
        self._sponge_outlet_idx = out

    # thermal set-up used by the pseudo-time step (LBM_CHT.py:2133-2167, 2361-2386)
    @property
    def ax(self):
        return "XYZ".index(self.cfg.flow_dir.upper().strip()[1])

    @property
    def sign(self):
        return +1 if self.cfg.flow_dir.upper().strip()[0] == "+" else -1

    def _build_update_mask_thermal(self):
        m = torch.ones((self.nx, self.ny, self.nz), dtype=torch.bool, device=self.device)
        if self.cfg.temp_bc == "periodic":
            return m
        n = (self.nx, self.ny, self.nz)[self.ax]
        sl = [slice(None)] * 3
        sl[self.ax] = 0 if self.sign > 0 else n - 1
        m[tuple(sl)] = False
        return m

    def _build_T_dirichlet_field(self):
        return torch.full((self.nx, self.ny, self.nz), float(self.fluid.tin_C), device=self.device)

    def _compute_heat_source(self):
        return getattr(self, "heat_source", None)

    def _compute_surface_flux_sources(self):
        return torch.zeros((self.nx, self.ny, self.nz), device=self.device)

    # methods the patch layer saves or replaces
    def _macroscopic(self):
        N = self.nx * self.ny * self.nz
        f = self.f.reshape(19, N)
        c = _C.to(self.device)
        self.rho = f.sum(0).view(self.nx, self.ny, self.nz)
        inv = 1.0 / (self.rho + 1e-12)
        self.u = (c[:, 0, None] * f).sum(0).view_as(self.rho) * inv
        self.v = (c[:, 1, None] * f).sum(0).view_as(self.rho) * inv
        self.wv = (c[:, 2, None] * f).sum(0).view_as(self.rho) * inv

    def _bounce_back_post_stream(self):
        s = self.solid_flow.reshape(-1)
        if not bool(s.any()):
            return
        N = self.nx * self.ny * self.nz
        f = self.f.reshape(19, N)
        opp = torch.as_tensor(geo.OPP_NP, device=self.device)
        f[:, s] = f[:, s][opp]

    def step(self, do_thermal: bool = True):
        raise RuntimeError("LatticeCase has no unpatched step; apply LBMCUDAUpgrade.patch first")

    def _collide(self):
        raise RuntimeError("unpatched")

    def _stream(self):
        raise RuntimeError("unpatched")

    def _apply_flow_bcs(self):
        raise RuntimeError("unpatched")


def stamp_walls(cfg: CaseConfig, solid_flow: torch.Tensor) -> torch.Tensor:
    """Wall planes of every face whose role is 'wall' (LBM_CHT.py _apply_transverse_flow_walls)."""
    from .solver.face_roles import resolve_face_roles
    s = solid_flow.clone()
    for face, role in resolve_face_roles(cfg).items():
        if role != "wall":
            continue
        ax = "XYZ".index(face[1])
        sl = [slice(None)] * 3
        sl[ax] = -1 if face[0] == "+" else 0
        s[tuple(sl)] = True
    return s


# --------------------------------------------------------------------------
# benchmark / parity workloads
# --------------------------------------------------------------------------
def channel_cube(device="cuda", collision="bgk", storage="fp32", nx=64, ny=32, nz=32, u=0.05, Re=50.0,
                 cube=12, cube_x=20, seed=0, sponge_length=0, outlet="convective", with_links=True):
    """Channel with a heated solid cube: velocity inlet, zero-gradient outlet, periodic y,
    walls at +-z; nu = u * cube / Re."""
    cfg = CaseConfig(nx=nx, ny=ny, nz=nz, collision=collision, lbm_storage=storage,
                     domain_walls=["+Z", "-Z"], outlet_bc_mode=outlet, sponge_length=sponge_length)
    solid = geo.cube_mask((nx, ny, nz), (cube_x, ny // 2, nz // 2), (cube, cube, cube), device=device)
    ibb = None
    if with_links:
        ibb = geo.ibb_from_voxels(solid)
    sf = stamp_walls(cfg, solid)
    return LatticeCase(cfg, u, u * cube / Re, solid, sf, ibb, device=device, seed=seed)


def pin_fin(device="cuda", collision="mrt", storage="fp16", nx=256, ny=128, nz=128, u=0.08, Re=200.0,
            radius=3.5, height=80, base=8, seed=1, sponge_length=40, k_ratio=200.0, n_pins=(16, 8),
            ibb_builder=None):
    """Pin-fin heat sink: base plate + 16x8 jittered cylinders, analytic link fractions.
    `ibb_builder(solid, G)` makes the link data (default: the device link builder and FP64
    bisection of the level set G)."""
    cfg = CaseConfig(nx=nx, ny=ny, nz=nz, collision=collision, lbm_storage=storage,
                     domain_walls=["+Z", "-Z"], sponge_length=sponge_length)
    G = geo.pin_fin_levelset(nx, ny, nz, n_pins=n_pins, radius=radius, height=height, base=base, seed=seed,
                             device=device)
    solid = geo.mask_from_levelset((nx, ny, nz), G, device=device)
    ibb = (ibb_builder or geo.ibb_from_level_set)(solid, G)
    sf = stamp_walls(cfg, solid)
    nu = u * (2 * radius) / Re
    return LatticeCase(cfg, u, nu, solid, sf, ibb, device=device, seed=seed, k_ratio=k_ratio)


def gyroid(device="cuda", collision="trt", storage="fp16", nx=384, ny=192, nz=192, u=0.05, L=48.0, t=0.3,
           Re=20.0, seed=0, k_ratio=200.0, q_method="linear"):
    """Gyroid TPMS block: solid where sin(2 pi x/L) cos(2 pi y/L) + sin(2 pi y/L) cos(2 pi z/L) +
    sin(2 pi z/L) cos(2 pi x/L) > t, four open fluid planes at the inlet and at the outlet, walls at
    +-z; TRT with magic parameter 1/4, nu = u (L/4) / Re.  Re = 20 by default, where the flow
    settles to a steady state (at Re = 100 TRT diverges on this geometry after about 650 steps, at
    Re = 50 the flow stays weakly unsteady).  Link fractions from the linear interpolation of the
    level set between the link's nodes (q_method="bisect": its exact crossing)."""
    cfg = CaseConfig(nx=nx, ny=ny, nz=nz, collision=collision, lbm_storage=storage, trt_lambda=0.25,
                     domain_walls=["+Z", "-Z"])
    G = geo.gyroid_levelset(L, t)
    solid = geo.mask_from_levelset((nx, ny, nz), G, device=device)
    # keep an inlet/outlet buffer of fluid so the planes are open
    solid[:4] = False
    solid[-4:] = False
    ibb = geo.ibb_from_level_set(solid, lambda x: torch.where(
        (x[..., 0] < 3.5) | (x[..., 0] > nx - 4.5), torch.full_like(x[..., 0], -1.0), G(x)), method=q_method)
    sf = stamp_walls(cfg, solid)
    nu = u * L / 4 / Re
    return LatticeCase(cfg, u, nu, solid, sf, ibb, device=device, seed=seed, k_ratio=k_ratio)


def hybrid(device="cuda", collision="mrt_smag", storage="fp16", nx=768, ny=384, nz=384, u=0.06, Re=500.0,
           radius=5.0, height=80, base=8, L=64.0, t=0.3, seed=2, n_pins=None, k_ratio=200.0, sponge_length=40,
           heat_flux=5e-3):
    """Pin-fin / gyroid hybrid heat sink: the base plate of the pin fin, jittered cylindrical pins of
    radius 5 (one per 16 x 16 cells of the plate unless n_pins is given) and gyroid (L = 64, t = 0.3)
    infill between the pins from the plate top to the pin tops; inlet u = 0.06, Re = 500 on the pin
    diameter, walls at +-z, periodic y, k_s/k_f = 200, and a uniform heat flux `heat_flux` into the
    bottom layer of the plate (the case's heat_source).  MRT with the Smagorinsky model by default:
    at Re = 500 (tau = 0.5036) plain MRT is not stable.  Link fractions from the analytic level set
    (FP64 bisection)."""
    if n_pins is None:
        n_pins = (max(1, nx // 16), max(1, ny // 16))
    cfg = CaseConfig(nx=nx, ny=ny, nz=nz, collision=collision, lbm_storage=storage,
                     domain_walls=["+Z", "-Z"], sponge_length=sponge_length)
    G = geo.pin_gyroid_levelset(nx, ny, nz, n_pins=n_pins, radius=radius, height=height, base=base, L=L, t=t,
                                seed=seed, device=device)
    solid = geo.mask_from_levelset((nx, ny, nz), G, device=device)
    ibb = geo.ibb_from_level_set(solid, G)
    sf = stamp_walls(cfg, solid)
    nu = u * (2 * radius) / Re
    sim = LatticeCase(cfg, u, nu, solid, sf, ibb, device=device, seed=seed, k_ratio=k_ratio)
    src = torch.zeros((nx, ny, nz), device=sim.device)
    src[:, :, 0] = float(heat_flux)
    src[~sim.solid] = 0.0
    sim.heat_source = src
    return sim
