"""CPU restatement of the geometry set-up for interpolated bounce-back.

TEST INFRASTRUCTURE ONLY: the oracle that the device kernels are compared
with.  Nothing on the product path imports it.

  signed_edt        build_phi_from_voxel_mask_mm (pre_post/sdf_tracing.py:312-340):
                    scipy.ndimage.distance_transform_edt of the fluid and of the
                    solid (a third-party routine, scipy 1.18.1 in the build
                    container; the reference pins no version), times the pitch,
                    negative in the solid, cast to FP32.  Restated as three
                    separable min-plus passes over exact squared integer
                    distances (the published algorithm of Saito and Toriwaki),
                    then numpy's FP64 sqrt and product.  With no cell of the
                    other kind anywhere, scipy's feature transform reports the
                    point (-1, 0, 0) for every cell; restated here too.
  links_from_mask   build_links_from_mask_gpu (sdf_tracing.py:20-85)
  q_from_sdf        bfl_q_from_sdf + sdf_trilinear (sdf_tracing.py:89-184) in
                    FP32 numpy, one rounding per tensor operation.  `scalar_div`
                    picks how (x - origin) / dx is evaluated: "reciprocal" as a
                    tensor-by-host-scalar division runs on a CUDA device (times
                    the FP32 reciprocal), "divide" as it runs on the CPU.  The two
                    agree whenever dx is a power of two.
  weights_from_q    bfl_weights_from_q (sdf_tracing.py:188-205)

Pinned by tests/golden/ibb_links.npz (the reference's own link arrays, weights
and phi on a cube and a heat-sink crop, pitch 1) and, for the distance
transform, by scipy itself on seeded random masks.
"""
from __future__ import annotations

import numpy as np

C_NP = np.array([[0, 0, 0], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
                 [1, 1, 0], [1, -1, 0], [-1, 1, 0], [-1, -1, 0], [1, 0, 1], [1, 0, -1], [-1, 0, 1],
                 [-1, 0, -1], [0, 1, 1], [0, 1, -1], [0, -1, 1], [0, -1, -1]], dtype=np.int64)
OPP_NP = np.array([0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15], dtype=np.int64)

_INF = np.int64(1) << 40
f32 = np.float32


def _min_plus_axis(g: np.ndarray, axis: int, chunk_elems: int = 1 << 24) -> np.ndarray:
    """out[..., x, ...] = min_y g[..., y, ...] + (x - y)^2 along `axis`."""
    g = np.moveaxis(g, axis, -1)
    shp = g.shape
    L = shp[-1]
    flat = g.reshape(-1, L)
    x = np.arange(L, dtype=np.int64)
    d2 = (x[:, None] - x[None, :]) ** 2          # (out, in)
    out = np.empty_like(flat)
    step = max(1, chunk_elems // (L * L))
    for s in range(0, flat.shape[0], step):
        blk = flat[s:s + step]
        out[s:s + step] = np.min(blk[:, None, :] + d2[None, :, :], axis=2)
    out = np.minimum(out, _INF)
    return np.moveaxis(out.reshape(shp), -1, axis)


def squared_edt(feature: np.ndarray) -> np.ndarray:
    """Exact squared Euclidean distance (int64) from every cell to the nearest True cell;
    values >= 2**40 where the mask has no True cell."""
    g = np.where(feature, 0, _INF).astype(np.int64)
    for ax in (2, 1, 0):
        g = _min_plus_axis(g, ax)
    return g


def _degenerate_d2(shape) -> np.ndarray:
    i, j, k = np.indices(shape, dtype=np.int64)
    return (i + 1) ** 2 + j ** 2 + k ** 2


def signed_edt(solid: np.ndarray, pitch: float = 1.0) -> np.ndarray:
    """phi of build_phi_from_voxel_mask_mm: FP32, positive in fluid, negative in solid."""
    s = np.asarray(solid).astype(bool)
    d_out = squared_edt(s) if s.any() else _degenerate_d2(s.shape)      # fluid -> nearest solid
    d_in = squared_edt(~s) if (~s).any() else _degenerate_d2(s.shape)   # solid -> nearest fluid
    phi = np.sqrt(d_out.astype(np.float64)) * float(pitch)
    phi[s] = -(np.sqrt(d_in[s].astype(np.float64)) * float(pitch))
    return phi.astype(np.float32)


def links_from_mask(solid: np.ndarray):
    """(fluid_flat, dir_i, dir_opp, ff_flat, ff_valid) in the reference's order."""
    s = np.asarray(solid).astype(bool)
    nx, ny, nz = s.shape
    fluid = ~s
    I, J, K = np.indices(s.shape)
    out = [[], [], [], []]
    for q in range(1, 19):
        cx, cy, cz = (int(v) for v in C_NP[q])
        a, b, c = I + cx, J + cy, K + cz
        valid = (a >= 0) & (a < nx) & (b >= 0) & (b < ny) & (c >= 0) & (c < nz)
        nb = s[a.clip(0, nx - 1), b.clip(0, ny - 1), c.clip(0, nz - 1)]
        m = valid & fluid & nb
        if not m.any():
            continue
        i, j, k = I[m], J[m], K[m]
        iff, jff, kff = i - cx, j - cy, k - cz
        inb = (iff >= 0) & (iff < nx) & (jff >= 0) & (jff < ny) & (kff >= 0) & (kff < nz)
        ic, jc, kc = iff.clip(0, nx - 1), jff.clip(0, ny - 1), kff.clip(0, nz - 1)
        out[0].append((i * ny * nz + j * nz + k).astype(np.int64))
        out[1].append(np.full(i.size, q, dtype=np.int64))
        out[2].append((ic * ny * nz + jc * nz + kc).astype(np.int64))
        out[3].append(inb & fluid[ic, jc, kc])
    if not out[0]:
        e = np.zeros(0, dtype=np.int64)
        return e, e.copy(), e.copy(), e.copy(), np.zeros(0, dtype=bool)
    ff = np.concatenate(out[0])
    di = np.concatenate(out[1])
    return ff, di, OPP_NP[di], np.concatenate(out[2]), np.concatenate(out[3])


def linspace7() -> np.ndarray:
    """torch.linspace(0, 1, 7) in FP32: start + step*i below the midpoint, end - step*(6-i) from it."""
    step = f32(1.0) / f32(6.0)
    v = [f32(0.0), step, step * f32(2.0), f32(1.0) - step * f32(3.0), f32(1.0) - step * f32(2.0),
         f32(1.0) - step, f32(1.0)]
    return np.array(v, dtype=np.float32)


def _trilinear(phi: np.ndarray, origin: np.ndarray, dx: float, x: np.ndarray, scalar_div: str) -> np.ndarray:
    """sdf_trilinear (sdf_tracing.py:89-125)."""
    if scalar_div == "reciprocal":
        g = (x - origin) * (f32(1.0) / f32(dx))
    else:
        g = (x - origin) / f32(dx)
    n = phi.shape
    gx = np.clip(g[..., 0], f32(0.0), f32(n[0] - 1.001))
    gy = np.clip(g[..., 1], f32(0.0), f32(n[1] - 1.001))
    gz = np.clip(g[..., 2], f32(0.0), f32(n[2] - 1.001))
    i0, j0, k0 = np.floor(gx).astype(np.int64), np.floor(gy).astype(np.int64), np.floor(gz).astype(np.int64)
    fx, fy, fz = gx - i0.astype(np.float32), gy - j0.astype(np.float32), gz - k0.astype(np.float32)
    i1 = np.minimum(i0 + 1, n[0] - 1)
    j1 = np.minimum(j0 + 1, n[1] - 1)
    k1 = np.minimum(k0 + 1, n[2] - 1)
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


def q_from_sdf(phi: np.ndarray, fluid_flat: np.ndarray, dir_i: np.ndarray, pitch: float = 1.0,
               origin=(0.0, 0.0, 0.0), scalar_div: str = "reciprocal", n_bisect: int = 10) -> np.ndarray:
    """Fractions of build_ibb_from_sdf_gpu (sdf_tracing.py:208-259) for the given links."""
    phi = np.asarray(phi, dtype=np.float32)
    nx, ny, nz = phi.shape
    org = np.asarray(origin, dtype=np.float32)
    pf = f32(pitch)
    i = (fluid_flat // (ny * nz)).astype(np.float32)
    j = ((fluid_flat // nz) % ny).astype(np.float32)
    k = (fluid_flat % nz).astype(np.float32)
    x0 = np.stack([i, j, k], axis=1) * pf + org[None, :]
    c = C_NP[dir_i].astype(np.float32)
    cn = np.sqrt((c * c).sum(axis=1, dtype=np.float32)).astype(np.float32)
    d = c / (cn + f32(1e-30))[:, None]
    L = pf * cn
    t = linspace7()[None, :] * L[:, None]
    xs = x0[:, None, :] + t[:, :, None] * d[:, None, :]
    ph = _trilinear(phi, org, pitch, xs.reshape(-1, 3), scalar_div).reshape(t.shape)
    s = ph > 0
    cross = s[:, :-1] & ~s[:, 1:]
    anyc = cross.any(axis=1)
    idx = np.argmax(cross, axis=1)
    lo = np.take_along_axis(t, idx[:, None], 1)[:, 0]
    hi = np.take_along_axis(t, (idx + 1)[:, None], 1)[:, 0]
    for _ in range(n_bisect):
        mid = f32(0.5) * (lo + hi)
        pm = _trilinear(phi, org, pitch, x0 + mid[:, None] * d, scalar_div)
        lo = np.where(pm > 0, mid, lo)
        hi = np.where(pm > 0, hi, mid)
    return np.where(anyc, hi / (L + f32(1e-30)), f32(0.5)).astype(np.float32)


def weights_from_q(q: np.ndarray):
    q = np.asarray(q, dtype=np.float32)
    ge = q >= f32(0.5)
    qg = np.where(ge, q, f32(1.0))
    w1_ge = f32(1.0) / (f32(2.0) * qg)
    w2_ge = f32(1.0) - w1_ge
    ql = np.where(~ge, q, f32(0.25))
    w1_lt = f32(2.0) * ql
    w2_lt = f32(1.0) - f32(2.0) * ql
    return ge, np.where(ge, w1_ge, w1_lt).astype(np.float32), np.where(ge, w2_ge, w2_lt).astype(np.float32)


def ibb_from_sdf(solid: np.ndarray, phi: np.ndarray, pitch: float = 1.0, origin=(0.0, 0.0, 0.0),
                 scalar_div: str = "reciprocal") -> dict:
    """Every IBBData array of build_ibb_from_sdf_gpu, plus q."""
    ff, di, do, fff, fv = links_from_mask(solid)
    q = q_from_sdf(phi, ff, di, pitch, origin, scalar_div)
    ge, w1, w2 = weights_from_q(q)
    return dict(fluid_flat=ff, dir_i=di, dir_opp=do, q_ge_half=ge, w_i=w1, w_second=w2, ff_flat=fff, ff_valid=fv,
                q=q)
