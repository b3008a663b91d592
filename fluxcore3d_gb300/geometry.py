"""Voxel geometry and interpolated-bounce-back (Bouzidi) link data.

`IBBData` has the field layout of the reference's pre_post/sdf_tracing.py:9-18.
The set-up runs on the device through the library's geometry kernels:

* `signed_distance` -- the voxel SDF of build_phi_from_voxel_mask_mm
  (sdf_tracing.py:312-340): exact Euclidean distance to the nearest cell of the
  other kind times the pitch, negative in the solid, FP32 equal bit for bit to
  the host scipy.ndimage.distance_transform_edt result the reference casts.
* `build_links` -- build_links_from_mask_gpu (sdf_tracing.py:20-85): a link is a
  fluid cell x_f whose neighbour x_f + c_q (q = 1..18, no wrap) is solid; the
  arrays are grouped by q = 1..18 with cells in row-major order inside each q,
  and x_ff = x_f - c_q is the second fluid node (valid when inside the box and
  fluid).
* `ibb_from_phi` -- build_ibb_from_sdf_gpu's fractions (bfl_q_from_sdf /
  sdf_trilinear, sdf_tracing.py:89-184: 6 coarse samples and 10 bisections of
  the trilinear level set in FP32) and bfl_weights_from_q (:188-205).

The synthetic heat-sink geometries (cube channel, pin fin, gyroid, random
spheres) are generated here on the device; their link fractions come either
from the trilinear path above or from the exact level set of the analytic
surface (cylinders, planes, gyroid), refined in FP64.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from ._torch import ptr, stream_ptr

C_NP = np.array([[0, 0, 0], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
                 [1, 1, 0], [1, -1, 0], [-1, 1, 0], [-1, -1, 0], [1, 0, 1], [1, 0, -1], [-1, 0, 1],
                 [-1, 0, -1], [0, 1, 1], [0, 1, -1], [0, -1, 1], [0, -1, -1]], dtype=np.int64)
OPP_NP = np.array([0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15], dtype=np.int64)


@dataclass
class IBBData:
    n_links: int
    fluid_flat: torch.Tensor
    dir_i: torch.Tensor
    dir_opp: torch.Tensor
    q_ge_half: torch.Tensor
    w_i: torch.Tensor
    w_second: torch.Tensor
    ff_flat: torch.Tensor
    ff_valid: torch.Tensor


def _mask_u8(solid: torch.Tensor) -> torch.Tensor:
    if not isinstance(solid, torch.Tensor) or solid.dim() != 3:
        raise ValueError("solid must be a (nx, ny, nz) tensor")
    if not solid.is_cuda:
        raise RuntimeError("geometry set-up runs on a CUDA device: move the solid mask to the GPU")
    return solid.contiguous().to(torch.uint8)


def _check_errword(err: torch.Tensor, what: str) -> None:
    e = int(err.item())
    if e:
        raise RuntimeError(f"{what}: device error word {e:#x} (link index out of range)")


def signed_distance(solid: torch.Tensor, pitch: float = 1.0) -> torch.Tensor:
    """Signed distance of a voxel mask (positive in fluid) times `pitch`, FP32 on the mask's
    device: build_phi_from_voxel_mask_mm (sdf_tracing.py:312-340)."""
    s = _mask_u8(solid)
    nx, ny, nz = s.shape
    L = _lib.lib()
    ws = torch.empty(max(1, int(L.fc_geom_edt_workspace_bytes(nx, ny, nz))), dtype=torch.uint8, device=s.device)
    phi = torch.empty((nx, ny, nz), dtype=torch.float32, device=s.device)
    _lib.call("fc_geom_signed_edt", ptr(s), nx, ny, nz, float(pitch), ptr(phi), ptr(ws), ws.numel(), stream_ptr())
    return phi


def build_links(solid: torch.Tensor):
    """(fluid_flat, dir_i, dir_opp, ff_flat, ff_valid) of build_links_from_mask_gpu (sdf_tracing.py:20-85),
    int64 / bool on the mask's device, in the reference's order."""
    s = _mask_u8(solid)
    nx, ny, nz = s.shape
    dev = s.device
    L = _lib.lib()
    ws = torch.empty(int(L.fc_ibb_links_workspace_bytes(nx, ny, nz)), dtype=torch.uint8, device=dev)
    total = torch.zeros(1, dtype=torch.int64, device=dev)
    st = stream_ptr()
    _lib.call("fc_ibb_count_links", ptr(s), nx, ny, nz, ptr(ws), ws.numel(), ptr(total), st)
    n = int(total.item())
    out = [torch.empty(n, dtype=torch.int64, device=dev) for _ in range(4)]
    ff_valid = torch.empty(n, dtype=torch.bool, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    _lib.call("fc_ibb_build_links", ptr(s), nx, ny, nz, ptr(ws), ws.numel(), n, *(ptr(t) for t in out),
              ptr(ff_valid), ptr(err), st)
    _check_errword(err, "fc_ibb_build_links")
    fluid_flat, dir_i, dir_opp, ff_flat = out
    return fluid_flat, dir_i, dir_opp, ff_flat, ff_valid


def bfl_weights_from_q(q: torch.Tensor):
    """(q >= 1/2, w1, w2) of bfl_weights_from_q (sdf_tracing.py:188-205) for FP32 fractions on the GPU."""
    if not q.is_cuda:
        raise RuntimeError("q must be on CUDA")
    q = q.contiguous().to(torch.float32)
    n = q.numel()
    ge = torch.empty(n, dtype=torch.bool, device=q.device)
    w1 = torch.empty(n, dtype=torch.float32, device=q.device)
    w2 = torch.empty(n, dtype=torch.float32, device=q.device)
    _lib.call("fc_ibb_weights_from_q", ptr(q), n, ptr(ge), ptr(w1), ptr(w2), stream_ptr())
    return ge, w1, w2


def ibb_from_phi(solid: torch.Tensor, phi: torch.Tensor, pitch: float = 1.0, origin=(0.0, 0.0, 0.0),
                 return_q: bool = False, host_division: bool = False):
    """Links of `solid` with fractions from the trilinear level set `phi` (build_ibb_from_sdf_gpu,
    sdf_tracing.py:208-259; the fluid cell (i,j,k) sits at origin + pitch*(i,j,k)).  `origin` holds
    the three FP32 coordinates of the domain origin.  The grid coordinate (x - origin) / pitch is
    rounded as torch rounds it on a CUDA device (times the FP32 reciprocal of the pitch), or as on
    the CPU (one division) with host_division=True; the two agree for power-of-two pitches."""
    ff, di, do, fff, fv = build_links(solid)
    nx, ny, nz = solid.shape
    if tuple(phi.shape) != (nx, ny, nz):
        raise ValueError("phi must have the shape of solid")
    ph = phi.to(device=ff.device, dtype=torch.float32).contiguous()
    n = ff.numel()
    dev = ff.device
    ge = torch.empty(n, dtype=torch.bool, device=dev)
    w1 = torch.empty(n, dtype=torch.float32, device=dev)
    w2 = torch.empty(n, dtype=torch.float32, device=dev)
    q = torch.empty(n, dtype=torch.float32, device=dev) if return_q else None
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    ox, oy, oz = (float(np.float32(v)) for v in origin)
    _lib.call("fc_ibb_q_from_sdf", ptr(ph), nx, ny, nz, ox, oy, oz, float(pitch), int(bool(host_division)),
              ptr(ff), ptr(di), n, ptr(q),
              ptr(ge), ptr(w1), ptr(w2), ptr(err), stream_ptr())
    _check_errword(err, "fc_ibb_q_from_sdf")
    ibb = IBBData(int(n), ff, di, do, ge, w1, w2, fff, fv)
    return (ibb, q) if return_q else ibb


def ibb_from_voxels(solid: torch.Tensor, pitch: float = 1.0, origin=(0.0, 0.0, 0.0)) -> IBBData:
    """Voxel SDF then links and fractions: build_phi_from_voxel_mask_mm followed by build_ibb_from_sdf_gpu."""
    return ibb_from_phi(solid, signed_distance(solid, pitch), pitch, origin)


def ibb_from_level_set(solid: torch.Tensor, levelset, n_bisect: int = 40, method: str = "bisect") -> IBBData:
    """Links of `solid` with q from an analytic level set G(x) (negative = fluid, positive =
    solid, G(cell centre) > 0 <=> solid): method "bisect" refines the crossing by FP64 bisection,
    "linear" interpolates G linearly between the link's two nodes."""
    ff, di, do, fff, fv = build_links(solid)
    if method == "linear":
        q = linear_level_set_fractions(levelset, ff, di, solid.shape)
    elif method == "bisect":
        q = level_set_fractions(levelset, ff, di, solid.shape, n_bisect)
    else:
        raise ValueError("method must be 'bisect' or 'linear'")
    ge, w1, w2 = bfl_weights_from_q(q)
    return IBBData(int(ff.numel()), ff, di, do, ge, w1, w2, fff, fv)


def level_set_fractions(levelset, fluid_flat: torch.Tensor, dir_i: torch.Tensor, shape,
                        n_bisect: int = 40) -> torch.Tensor:
    """FP32 link fractions q in (0, 1]: FP64 bisection of G along x_f + t c_q for t in [0, 1] (the
    crossing lies in that interval because x_f is fluid and x_f + c_q solid), on the links' device."""
    dev = fluid_flat.device
    nx, ny, nz = shape
    ff = fluid_flat
    i = (ff // (ny * nz)).to(torch.float64)
    j = ((ff // nz) % ny).to(torch.float64)
    k = (ff % nz).to(torch.float64)
    x0 = torch.stack([i, j, k], dim=1)
    c = torch.tensor(C_NP, device=dev, dtype=torch.float64)[dir_i]
    lo = torch.zeros(ff.numel(), device=dev, dtype=torch.float64)
    hi = torch.ones_like(lo)
    for _ in range(n_bisect):
        mid = 0.5 * (lo + hi)
        inside = levelset(x0 + mid[:, None] * c) > 0
        hi = torch.where(inside, mid, hi)
        lo = torch.where(inside, lo, mid)
    return hi.clamp(1e-6, 1.0).to(torch.float32)


def linear_level_set_fractions(levelset, fluid_flat: torch.Tensor, dir_i: torch.Tensor, shape) -> torch.Tensor:
    """FP32 link fractions q = G_f / (G_f - G_s) in (0, 1]: the zero of G interpolated linearly
    between the fluid node x_f (G_f <= 0) and the solid node x_f + c_q (G_s > 0), in FP64."""
    dev = fluid_flat.device
    nx, ny, nz = shape
    ff = fluid_flat
    x0 = torch.stack([(ff // (ny * nz)).double(), ((ff // nz) % ny).double(), (ff % nz).double()], dim=1)
    c = torch.tensor(C_NP, device=dev, dtype=torch.float64)[dir_i]
    gf = levelset(x0)
    gs = levelset(x0 + c)
    q = gf / (gf - gs)
    return q.clamp(1e-6, 1.0).to(torch.float32)


# --------------------------------------------------------------------------
# synthetic geometries (level sets are positive inside the solid)
# --------------------------------------------------------------------------
def _grid(shape, device):
    nx, ny, nz = shape
    X = torch.arange(nx, device=device, dtype=torch.float64).view(nx, 1, 1).expand(shape)
    Y = torch.arange(ny, device=device, dtype=torch.float64).view(1, ny, 1).expand(shape)
    Z = torch.arange(nz, device=device, dtype=torch.float64).view(1, 1, nz).expand(shape)
    return torch.stack([X, Y, Z], dim=-1)


def cube_mask(shape, center, width, device="cpu") -> torch.Tensor:
    """Cube obstacle as ObstacleFactory3D.cube (LBM_CHT.py:171-181)."""
    s = torch.zeros(shape, dtype=torch.bool, device=device)
    sl = []
    for n, c, w in zip(shape, center, width):
        sl.append(slice(max(0, c - w // 2), min(n, c + (w - w // 2))))
    s[tuple(sl)] = True
    return s


def pin_fin_levelset(nx, ny, nz, n_pins=(16, 8), radius=3.5, height=80, base=8, seed=1, device="cpu"):
    """Base plate z < base plus n_pins[0] x n_pins[1] cylinders of `radius` up to z < base + height,
    centres on a regular grid jittered uniformly by +-1 voxel (seed).  Cell (i,j,k) has its
    centre at (i,j,k); the plate top and pin tops sit half a cell below the first fluid layer."""
    g = torch.Generator().manual_seed(seed)
    px, py = n_pins
    sx, sy = nx / px, ny / py
    ax = torch.arange(px, dtype=torch.float64)
    by = torch.arange(py, dtype=torch.float64)
    cx = ((ax[:, None] + 0.5) * sx).expand(px, py).clone() - 0.5
    cy = ((by[None, :] + 0.5) * sy).expand(px, py).clone() - 0.5
    cx = cx + (torch.rand((px, py), generator=g, dtype=torch.float64) * 2 - 1)
    cy = cy + (torch.rand((px, py), generator=g, dtype=torch.float64) * 2 - 1)
    cx, cy = cx.to(device), cy.to(device)
    top = float(base + height) - 0.5
    zb = float(base) - 0.5
    r = float(radius)

    def G(x):
        X, Y, Z = x[..., 0], x[..., 1], x[..., 2]
        plate = zb - Z
        a0 = torch.floor((X + 0.5) / sx).long()
        b0 = torch.floor((Y + 0.5) / sy).long()
        best = torch.full_like(X, -1e30)
        for da in (-1, 0, 1):
            ia = (a0 + da).clamp(0, px - 1)
            for db in (-1, 0, 1):
                ib = (b0 + db).clamp(0, py - 1)
                dxv = X - cx[ia, ib]
                dyv = Y - cy[ia, ib]
                best = torch.maximum(best, r - torch.sqrt(dxv * dxv + dyv * dyv))
        pins = torch.minimum(best, top - Z)
        return torch.maximum(plate, pins)
    return G


def pin_gyroid_levelset(nx, ny, nz, n_pins=(48, 24), radius=5.0, height=80, base=8, L=64.0, t=0.3, seed=2,
                        device="cpu"):
    """Pin-fin / TPMS hybrid: the base plate and jittered cylinders of pin_fin_levelset with gyroid
    (level t, period L) infill between the pins, from the plate top to the pin tops."""
    pins = pin_fin_levelset(nx, ny, nz, n_pins=n_pins, radius=radius, height=height, base=base, seed=seed,
                            device=device)
    gyr = gyroid_levelset(L, t)
    top = float(base + height) - 0.5
    zb = float(base) - 0.5

    def G(x):
        Z = x[..., 2]
        band = torch.minimum(torch.minimum(gyr(x), top - Z), Z - zb)
        return torch.maximum(pins(x), band)
    return G


def gyroid_levelset(L=48.0, t=0.3):
    w = 2 * math.pi / L

    def G(x):
        X, Y, Z = x[..., 0] * w, x[..., 1] * w, x[..., 2] * w
        return torch.sin(X) * torch.cos(Y) + torch.sin(Y) * torch.cos(Z) + torch.sin(Z) * torch.cos(X) - t
    return G


def mask_from_levelset(shape, G, device="cpu", chunk=1 << 22) -> torch.Tensor:
    nx, ny, nz = shape
    out = torch.empty(nx * ny * nz, dtype=torch.bool, device=device)
    idx = torch.arange(nx * ny * nz, device=device)
    for s in range(0, idx.numel(), chunk):
        fl = idx[s:s + chunk]
        x = torch.stack([(fl // (ny * nz)).double(), ((fl // nz) % ny).double(), (fl % nz).double()], dim=1)
        out[s:s + chunk] = G(x) > 0
    return out.view(shape)


def random_spheres_mask(n: int, seed: int, rmin=4.0, rmax=16.0, frac_lo=0.2, frac_hi=0.4, device="cpu"):
    """Binary solid of random non-overlapping spheres with a target solid fraction in [frac_lo, frac_hi]."""
    rng = np.random.default_rng(seed)
    target = rng.uniform(frac_lo, frac_hi)
    centers, radii = [], []
    vol = 0.0
    tries = 0
    while vol / n ** 3 < target and tries < 20000:
        tries += 1
        r = rng.uniform(rmin, rmax)
        c = rng.uniform(r, n - r, size=3)
        if any(np.linalg.norm(c - c2) < r + r2 + 1.0 for c2, r2 in zip(centers, radii)):
            continue
        centers.append(c)
        radii.append(r)
        vol += 4.0 / 3.0 * math.pi * r ** 3
    g = _grid((n, n, n), device)
    s = torch.zeros((n, n, n), dtype=torch.bool, device=device)
    for c, r in zip(centers, radii):
        ct = torch.tensor(c, device=device, dtype=torch.float64)
        s |= ((g - ct) ** 2).sum(-1) <= r * r
    return s
