"""Geometry set-up kernels (voxel SDF, boundary links, Bouzidi fractions) against the oracle and the
reference's golden fixtures, through the C ABI."""
import os
import types

import numpy as np
import pytest
import torch

from fluxcore3d_gb300 import geometry as geo
from oracle import geometry as og

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLD, name))


def same_bits(a, b):
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = np.ascontiguousarray(b, dtype=np.float32)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def golden_cases():
    d1, d2 = load("ibb_links.npz"), load("ibb_pitch.npz")
    out = []
    for n in ("cube", "heatsink"):
        out.append((n, d1, 1.0, np.zeros(3, np.float32)))
    for n in ("crop", "balls"):
        pitch = float(d2[f"{n}_pitch"])
        org = (d2[f"{n}_voxel_origin"].astype(np.float32)
               - np.float32(pitch) * d2[f"{n}_offset_ijk"].astype(np.float32))
        out.append((n, d2, pitch, org))
    return out


def random_masks(seed=3):
    rng = np.random.default_rng(seed)
    shapes = [(37, 29, 33), (20, 18, 100), (64, 48, 40), (5, 7, 1), (1, 9, 64), (16, 1, 16),
              (800, 3, 5), (3, 800, 5), (1700, 2, 3), (3200, 1, 2), (1, 2, 4096)]
    masks = []
    for shp in shapes:
        masks.append(rng.random(shp) < rng.uniform(0.002, 0.5))
    one = np.zeros((30, 26, 21), bool)
    one[3, 20, 17] = True
    masks += [one, ~one, np.zeros((6, 7, 8), bool), np.ones((6, 7, 8), bool)]
    return masks


# ------------------------------------------------------------------ voxel SDF
def test_signed_distance_matches_reference_golden(cuda):
    for name, d, pitch, _ in golden_cases():
        phi = geo.signed_distance(torch.from_numpy(d[f"{name}_solid"]).to(cuda), pitch)
        assert same_bits(phi.cpu().numpy(), d[f"{name}_phi"]), name


def test_signed_distance_matches_oracle_on_seeded_masks(cuda):
    """Every staging width of the line passes (long x and y lines), ragged rows (nz = 1, 33, 100,
    4096), a single solid cell, its complement, and both one-kind masks (scipy's (-1,0,0) rule)."""
    for s in random_masks():
        for pitch in (1.0, 0.37):
            phi = geo.signed_distance(torch.from_numpy(s).to(cuda), pitch)
            assert same_bits(phi.cpu().numpy(), og.signed_edt(s, pitch)), (s.shape, pitch)


def test_signed_distance_rejects_rows_beyond_limit(cuda):
    with pytest.raises(RuntimeError, match="unsupported"):
        geo.signed_distance(torch.zeros((2, 2, 4097), dtype=torch.bool, device=cuda))


def _window_check(solid: np.ndarray, phi: np.ndarray, cells: np.ndarray) -> None:
    """Exact distance of sampled cells by a search of the cube of radius ceil(|phi|) around each."""
    nx, ny, nz = solid.shape
    for c in cells:
        i, j, k = np.unravel_index(int(c), solid.shape)
        kind = solid[i, j, k]
        r = int(np.ceil(abs(float(phi[i, j, k])))) + 1
        a0, a1 = max(0, i - r), min(nx, i + r + 1)
        b0, b1 = max(0, j - r), min(ny, j + r + 1)
        c0, c1 = max(0, k - r), min(nz, k + r + 1)
        w = solid[a0:a1, b0:b1, c0:c1] != kind
        I, J, K = np.nonzero(w)
        d2 = ((I + a0 - i) ** 2 + (J + b0 - j) ** 2 + (K + c0 - k) ** 2).min()
        want = np.float32(np.sqrt(np.float64(d2)))
        assert np.float32(abs(phi[i, j, k])) == want, (i, j, k)


@pytest.mark.parametrize("case", ["gyroid_384x192x192", "pinfin_256x128x128"])
def test_signed_distance_full_size_properties(cuda, case):
    """Full-size geometries: sign = kind, |phi| >= 1, 1-Lipschitz between same-kind neighbours, and
    the exact distance of 3000 sampled cells by a local brute-force search."""
    if case.startswith("gyroid"):
        solid = geo.mask_from_levelset((384, 192, 192), geo.gyroid_levelset(48.0, 0.3), device=cuda)
    else:
        G = geo.pin_fin_levelset(256, 128, 128, device=cuda)
        solid = geo.mask_from_levelset((256, 128, 128), G, device=cuda)
    phi = geo.signed_distance(solid)
    assert torch.equal(phi < 0, solid)
    assert float(phi.abs().min()) >= 1.0
    a = phi.abs()
    for ax in range(3):
        n = solid.shape[ax]
        lo, hi = a.narrow(ax, 0, n - 1), a.narrow(ax, 1, n - 1)
        same = solid.narrow(ax, 0, n - 1) == solid.narrow(ax, 1, n - 1)
        assert float(((lo - hi).abs() - 1.0 - 1e-5 * torch.maximum(lo, hi))[same].max()) <= 0.0
    s_np, p_np = solid.cpu().numpy(), phi.cpu().numpy()
    rng = np.random.default_rng(0)
    near = np.flatnonzero(np.abs(p_np).ravel() <= 6.0)
    far = np.flatnonzero(np.abs(p_np).ravel() > 6.0)
    cells = rng.choice(near, 2900, replace=False)
    if far.size:
        cells = np.concatenate([cells, rng.choice(far, min(100, far.size), replace=False)])
    _window_check(s_np, p_np, cells)


# ------------------------------------------------------------------ link list
def _links_np(solid, cuda):
    ff, di, do, fff, fv = geo.build_links(torch.from_numpy(solid).to(cuda))
    return [t.cpu().numpy() for t in (ff, di, do, fff, fv)]


def test_links_match_reference_golden(cuda):
    for name, d, _, _ in golden_cases():
        got = _links_np(d[f"{name}_solid"], cuda)
        for k, v in zip(("fluid_flat", "dir_i", "dir_opp", "ff_flat", "ff_valid"), got):
            assert np.array_equal(v, d[f"{name}_{k}"]), (name, k)


def test_links_match_oracle_on_seeded_masks(cuda):
    for s in random_masks(11):
        got = _links_np(s, cuda)
        want = og.links_from_mask(s)
        for g, w in zip(got, want):
            assert np.array_equal(g, w), s.shape


def test_links_full_size_order_and_counts(cuda):
    """384x192x192 gyroid: per-q counts equal a shifted-mask count, cells strictly increase inside
    every q block, every link is fluid -> solid, and ff / ff_valid follow x_f - c_q."""
    solid = geo.mask_from_levelset((384, 192, 192), geo.gyroid_levelset(48.0, 0.3), device=cuda)
    nx, ny, nz = solid.shape
    ff, di, do, fff, fv = geo.build_links(solid)
    assert torch.all(di[1:] >= di[:-1])
    fl = solid.reshape(-1)
    start = 0
    for q in range(1, 19):
        cx, cy, cz = (int(v) for v in geo.C_NP[q])
        nb = torch.zeros_like(solid)
        nb[max(0, -cx):nx - max(0, cx), max(0, -cy):ny - max(0, cy), max(0, -cz):nz - max(0, cz)] = \
            solid[max(0, cx):nx - max(0, -cx), max(0, cy):ny - max(0, -cy), max(0, cz):nz - max(0, -cz)]
        cnt = int((~solid & nb).sum())
        blk = ff[start:start + cnt]
        assert int((di[start:start + cnt] == q).sum()) == cnt
        assert bool(torch.all(blk[1:] > blk[:-1]))
        i, j, k = blk // (ny * nz), (blk // nz) % ny, blk % nz
        assert not bool(fl[blk].any())
        assert bool(fl[(i + cx) * ny * nz + (j + cy) * nz + (k + cz)].all())
        a, b, e = i - cx, j - cy, k - cz
        inb = (a >= 0) & (a < nx) & (b >= 0) & (b < ny) & (e >= 0) & (e < nz)
        flat = a.clamp(0, nx - 1) * ny * nz + b.clamp(0, ny - 1) * nz + e.clamp(0, nz - 1)
        assert torch.equal(fff[start:start + cnt], flat)
        assert torch.equal(fv[start:start + cnt], inb & ~fl[flat])
        assert bool(torch.all(do[start:start + cnt] == int(geo.OPP_NP[q])))
        start += cnt
    assert start == ff.numel()


# ------------------------------------------------------------------ fractions
def test_fractions_match_reference_golden_with_host_division(cuda):
    """The reference's fixtures were produced by its torch CPU path: with host_division the kernel
    reproduces their q, weights and flags bit for bit, at pitch 1, 0.37 and 0.5."""
    for name, d, pitch, org in golden_cases():
        solid = torch.from_numpy(d[f"{name}_solid"]).to(cuda)
        phi = torch.from_numpy(d[f"{name}_phi"]).to(cuda)
        ibb, q = geo.ibb_from_phi(solid, phi, pitch, tuple(org.tolist()), return_q=True, host_division=True)
        for k in ("fluid_flat", "dir_i", "dir_opp", "ff_flat", "ff_valid", "q_ge_half"):
            assert np.array_equal(getattr(ibb, k).cpu().numpy(), d[f"{name}_{k}"]), (name, k)
        for k in ("w_i", "w_second"):
            assert same_bits(getattr(ibb, k).cpu().numpy(), d[f"{name}_{k}"]), (name, k)
        if f"{name}_q" in d:
            assert same_bits(q.cpu().numpy(), d[f"{name}_q"]), name


def test_fractions_match_oracle_in_device_rounding(cuda):
    rng = np.random.default_rng(8)
    cases = [(m, p, rng.uniform(-3, 3, 3).astype(np.float32)) for m, p in
             ((random_masks(5)[0], 0.37), (random_masks(5)[2], 0.2), (random_masks(5)[1], 1.0))]
    d = load("ibb_pitch.npz")
    cases.append((d["crop_solid"], float(d["crop_pitch"]), np.array([0.76, -2.62, -0.985], np.float32)))
    thin = np.zeros((12, 1, 10), bool)      # one-cell axis: the trilinear lookup wraps index -1
    thin[5:8, 0, 3:6] = True
    cases.append((thin, 0.5, np.zeros(3, np.float32)))
    for s, pitch, org in cases:
        phi = og.signed_edt(s, pitch)
        ibb, q = geo.ibb_from_phi(torch.from_numpy(s).to(cuda), torch.from_numpy(phi).to(cuda), pitch,
                                  tuple(org.tolist()), return_q=True)
        want = og.ibb_from_sdf(s, phi, pitch, org, scalar_div="reciprocal")
        assert same_bits(q.cpu().numpy(), want["q"]), (s.shape, pitch)
        assert same_bits(ibb.w_i.cpu().numpy(), want["w_i"])
        assert same_bits(ibb.w_second.cpu().numpy(), want["w_second"])
        assert np.array_equal(ibb.q_ge_half.cpu().numpy(), want["q_ge_half"])


def test_torch_cuda_divides_by_host_scalar_through_its_reciprocal(cuda):
    """The rounding the default mode follows: a CUDA tensor divided by a Python float is the tensor
    times the FP32 reciprocal of the scalar, not a correctly rounded quotient."""
    x = (torch.rand(1 << 16, generator=torch.Generator().manual_seed(0)) * 60 - 5).to(cuda)
    dx = 0.37
    got = (x / dx).cpu().numpy()
    xn = x.cpu().numpy()
    recip = xn * (np.float32(1.0) / np.float32(dx))
    quot = xn / np.float32(dx)
    assert same_bits(got, recip)
    assert not same_bits(got, quot)


def test_weights_from_q_kernel(cuda):
    q = torch.rand(100003, generator=torch.Generator().manual_seed(1)).clamp_min(1e-6)
    q[:4] = torch.tensor([0.5, 1.0, 0.4999999, 1e-6])
    ge, w1, w2 = geo.bfl_weights_from_q(q.to(cuda))
    wg, wa, wb = og.weights_from_q(q.numpy())
    assert np.array_equal(ge.cpu().numpy(), wg)
    assert same_bits(w1.cpu().numpy(), wa) and same_bits(w2.cpu().numpy(), wb)


# ------------------------------------------------------------------ reference-named module
def test_sdf_tracing_module_drop_in(cuda, capsys):
    from fluxcore3d_gb300.pre_post import sdf_tracing as SDF
    d = load("ibb_pitch.npz")
    name = "crop"
    pitch = float(d[f"{name}_pitch"])
    sim = types.SimpleNamespace(device=cuda, nx=0, ny=0, nz=0)
    sim.solid = torch.from_numpy(d[f"{name}_solid"]).to(cuda)
    sim.phi = SDF.build_phi_from_voxel_mask_mm(d[f"{name}_solid"], pitch, device=cuda)
    assert same_bits(sim.phi.cpu().numpy(), d[f"{name}_phi"])
    SDF.build_ibb_from_sdf_gpu(sim, tuple(d[f"{name}_voxel_origin"]), pitch, tuple(d[f"{name}_offset_ijk"]),
                               geo.C_NP, geo.OPP_NP)
    out = capsys.readouterr().out
    assert "[SDF-IBB] links=" in out
    org = (d[f"{name}_voxel_origin"].astype(np.float32)
           - np.float32(pitch) * d[f"{name}_offset_ijk"].astype(np.float32))
    want = og.ibb_from_sdf(d[f"{name}_solid"], d[f"{name}_phi"], pitch, org, scalar_div="reciprocal")
    assert sim.ibb_data.n_links == want["fluid_flat"].size
    assert same_bits(sim.ibb_data.w_i.cpu().numpy(), want["w_i"])
    links = SDF.build_links_from_mask_gpu(sim.solid, geo.C_NP, geo.OPP_NP)
    assert np.array_equal(links[0].cpu().numpy(), want["fluid_flat"])
    with pytest.raises(ValueError):
        SDF.build_links_from_mask_gpu(sim.solid, geo.C_NP[::-1].copy(), geo.OPP_NP)
