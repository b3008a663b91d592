"""Voxel geometry and interpolated-bounce-back (Bouzidi) link data.

`IBBData` has the field layout of the reference's pre_post/sdf_tracing.py:9-18.
`build_links_from_mask` follows sdf_tracing.py:20-85: a link is a fluid cell
x_f whose neighbour x_f + c_q (q = 1..18, no wrap) is solid; the arrays are
concatenated over q = 1..18 with cells in row-major order inside each q, and
x_ff = x_f - c_q is the second fluid node (valid when inside the box and fluid).
`bfl_weights_from_q` follows sdf_tracing.py:188-205.
`q_from_sdf_trilinear` restates bfl_q_from_sdf / sdf_trilinear
(sdf_tracing.py:89-184): 6 coarse samples along the link and 10 bisections of
the trilinearly interpolated level set, each operation rounded separately in
FP32 as the reference's elementwise torch ops are.

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


def build_links_from_mask(solid: torch.Tensor):
    nx, ny, nz = solid.shape
    dev = solid.device
    fluid = ~solid
    I = torch.arange(nx, device=dev).view(nx, 1, 1).expand(nx, ny, nz)
    J = torch.arange(ny, device=dev).view(1, ny, 1).expand(nx, ny, nz)
    K = torch.arange(nz, device=dev).view(1, 1, nz).expand(nx, ny, nz)
    flats, dirs, ffs, oks = [], [], [], []
    for q in range(1, 19):
        cx, cy, cz = (int(v) for v in C_NP[q])
        nb = torch.zeros_like(solid)
        # neighbour x + c (no wrap)
        xs = slice(max(0, -cx), nx - max(0, cx))
        ys = slice(max(0, -cy), ny - max(0, cy))
        zs = slice(max(0, -cz), nz - max(0, cz))
        xd = slice(max(0, cx), nx - max(0, -cx))
        yd = slice(max(0, cy), ny - max(0, -cy))
        zd = slice(max(0, cz), nz - max(0, -cz))
        nb[xs, ys, zs] = solid[xd, yd, zd]
        m = fluid & nb
        if not bool(m.any()):
            continue
        i, j, k = I[m], J[m], K[m]
        flat = (i * (ny * nz) + j * nz + k).to(torch.int64)
        iff, jff, kff = i - cx, j - cy, k - cz
        inb = (iff >= 0) & (iff < nx) & (jff >= 0) & (jff < ny) & (kff >= 0) & (kff < nz)
        ok = inb.clone()
        ok[inb] = fluid[iff[inb], jff[inb], kff[inb]]
        fff = (iff.clamp(0, nx - 1) * (ny * nz) + jff.clamp(0, ny - 1) * nz + kff.clamp(0, nz - 1)).to(torch.int64)
        flats.append(flat)
        dirs.append(torch.full_like(flat, q))
        ffs.append(fff)
        oks.append(ok)
    if not flats:
        e = torch.zeros(0, dtype=torch.int64, device=dev)
        return e, e.clone(), e.clone(), e.clone(), torch.zeros(0, dtype=torch.bool, device=dev)
    fluid_flat = torch.cat(flats)
    dir_i = torch.cat(dirs)
    ff_flat = torch.cat(ffs)
    ff_valid = torch.cat(oks)
    dir_opp = torch.as_tensor(OPP_NP, device=dev)[dir_i]
    return fluid_flat, dir_i, dir_opp, ff_flat, ff_valid


def bfl_weights_from_q(q: torch.Tensor):
    ge = q >= 0.5
    qg = torch.where(ge, q, torch.ones_like(q))
    w1_ge = 1.0 / (2.0 * qg)
    w2_ge = 1.0 - w1_ge
    ql = torch.where(~ge, q, 0.25 * torch.ones_like(q))
    w1_lt = 2.0 * ql
    w2_lt = 1.0 - 2.0 * ql
    return ge, torch.where(ge, w1_ge, w1_lt), torch.where(ge, w2_ge, w2_lt)


def _trilinear(phi: torch.Tensor, origin: torch.Tensor, dx: float, x: torch.Tensor) -> torch.Tensor:
    g = (x - origin) / dx
    gx = g[..., 0].clamp(0.0, phi.shape[0] - 1.001)
    gy = g[..., 1].clamp(0.0, phi.shape[1] - 1.001)
    gz = g[..., 2].clamp(0.0, phi.shape[2] - 1.001)
    i0, j0, k0 = gx.floor().long(), gy.floor().long(), gz.floor().long()
    fx, fy, fz = gx - i0.to(gx.dtype), gy - j0.to(gy.dtype), gz - k0.to(gz.dtype)
    i1 = (i0 + 1).clamp_max(phi.shape[0] - 1)
    j1 = (j0 + 1).clamp_max(phi.shape[1] - 1)
    k1 = (k0 + 1).clamp_max(phi.shape[2] - 1)
    c000, c100 = phi[i0, j0, k0], phi[i1, j0, k0]
    c010, c110 = phi[i0, j1, k0], phi[i1, j1, k0]
    c001, c101 = phi[i0, j0, k1], phi[i1, j0, k1]
    c011, c111 = phi[i0, j1, k1], phi[i1, j1, k1]
    a00 = c000 + fx * (c100 - c000)
    a10 = c010 + fx * (c110 - c010)
    a01 = c001 + fx * (c101 - c001)
    a11 = c011 + fx * (c111 - c011)
    b0 = a00 + fy * (a10 - a00)
    b1 = a01 + fy * (a11 - a01)
    return b0 + fz * (b1 - b0)


def q_from_sdf_trilinear(phi, origin, dx, x0, d, L, n_coarse: int = 6, n_bisect: int = 10):
    n = x0.shape[0]
    tv = torch.linspace(0.0, 1.0, steps=n_coarse + 1, device=x0.device, dtype=x0.dtype)
    t = tv[None, :] * L[:, None]
    xs = x0[:, None, :] + t[:, :, None] * d[:, None, :]
    ph = _trilinear(phi, origin, dx, xs.reshape(-1, 3)).reshape(n, -1)
    s = ph > 0
    cross = s[:, :-1] & (~s[:, 1:])
    q = torch.full((n,), 0.5, device=x0.device, dtype=x0.dtype)
    anyc = cross.any(dim=1)
    if bool(anyc.any()):
        idx = cross.float().argmax(dim=1).long()
        lo = t.gather(1, idx[:, None]).squeeze(1)
        hi = t.gather(1, (idx + 1)[:, None]).squeeze(1)
        for _ in range(n_bisect):
            mid = 0.5 * (lo + hi)
            pm = _trilinear(phi, origin, dx, x0 + mid[:, None] * d)
            lo = torch.where(pm > 0, mid, lo)
            hi = torch.where(pm > 0, hi, mid)
        q = torch.where(anyc, hi / (L + 1e-30), q)
    return q


def phi_from_voxels(solid: np.ndarray, pitch: float = 1.0) -> np.ndarray:
    """Signed distance of a voxel mask (positive in fluid): exact Euclidean
    distance transform, as build_phi_from_voxel_mask_mm (sdf_tracing.py:312-340)."""
    from scipy.ndimage import distance_transform_edt
    s = solid.astype(bool)
    out = distance_transform_edt(~s) * pitch
    inn = distance_transform_edt(s) * pitch
    phi = out
    phi[s] = -inn[s]
    return phi


def ibb_from_phi_trilinear(solid: torch.Tensor, phi: torch.Tensor, pitch: float = 1.0,
                           origin=(0.0, 0.0, 0.0)) -> IBBData:
    """Links of `solid` with q from the trilinear level set `phi` (build_ibb_from_sdf_gpu semantics)."""
    dev = solid.device
    nx, ny, nz = solid.shape
    ff, di, do, fff, fv = build_links_from_mask(solid)
    org = torch.tensor(origin, device=dev, dtype=torch.float32)
    i = (ff // (ny * nz)).to(torch.float32)
    j = ((ff // nz) % ny).to(torch.float32)
    k = (ff % nz).to(torch.float32)
    x0 = torch.stack([i, j, k], dim=1) * float(pitch) + org[None, :]
    c = torch.tensor(C_NP, device=dev, dtype=torch.float32)
    draw = c[di]
    cn = torch.linalg.norm(draw, dim=1)
    d = draw / (cn[:, None] + 1e-30)
    L = float(pitch) * cn
    q = q_from_sdf_trilinear(phi.to(dev, torch.float32), org, float(pitch), x0, d, L)
    ge, w1, w2 = bfl_weights_from_q(q)
    return IBBData(int(ff.numel()), ff, di, do, ge, w1.float(), w2.float(), fff, fv)


def ibb_from_level_set(solid: torch.Tensor, levelset, n_bisect: int = 40) -> IBBData:
    """Links of `solid` with q from an analytic level set G(x) (negative = fluid, positive =
    solid, G(cell centre) > 0 <=> solid), refined by FP64 bisection to the exact crossing."""
    dev = solid.device
    nx, ny, nz = solid.shape
    ff, di, do, fff, fv = build_links_from_mask(solid)
    i = (ff // (ny * nz)).to(torch.float64)
    j = ((ff // nz) % ny).to(torch.float64)
    k = (ff % nz).to(torch.float64)
    x0 = torch.stack([i, j, k], dim=1)
    c = torch.tensor(C_NP, device=dev, dtype=torch.float64)[di]
    lo = torch.zeros(ff.numel(), device=dev, dtype=torch.float64)
    hi = torch.ones_like(lo)
    for _ in range(n_bisect):
        mid = 0.5 * (lo + hi)
        inside = levelset(x0 + mid[:, None] * c) > 0
        hi = torch.where(inside, mid, hi)
        lo = torch.where(inside, lo, mid)
    q = hi.clamp(1e-6, 1.0).to(torch.float32)
    ge, w1, w2 = bfl_weights_from_q(q)
    return IBBData(int(ff.numel()), ff, di, do, ge, w1.float(), w2.float(), fff, fv)


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
