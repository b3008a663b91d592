"""Golden fixtures from the reference's own CUDA kernels run on the host (TEST INFRASTRUCTURE).

oracle/build_ref.py compiles the unmodified text of fluxcore3D solver/lbm_kernels.cu's
regularised Zou/He (lbm_zou_he_bc_kernel), convective outlet (lbm_convective_bc_reduce_kernel
+ lbm_convective_mass_correct_kernel) and MRT-Smagorinsky collision
(lbm_macro_collide_mrt_smag_kernel) for the CPU; this script runs them on seeded inputs and
writes tests/golden/ref_lbm.npz:
  zh_<case>_{in,plane}, zh_<case>_args   Zou/He planes: velocity inlets and pressure outlets on
                                       low and high faces of each axis, backflow nodes and solid
                                       nodes in the planes (`plane`: the [19][n1*n2] populations of
                                       the boundary plane after the kernel; nothing else changes)
  cv_<case>_{in,plane}, cv_<case>_args   convective outlets (one and two blocks of plane nodes),
                                       with the reference's plane sums (sum of rho, count)
  smag_{f,solid,S,out_fp,out_macro}    one MRT-Smagorinsky collision of a perturbed state
Every case shares one solid mask per lattice shape (`solid_<nx>x<ny>x<nz>`).

Usage:  python tests/golden/make_ref_fixtures.py /path/to/fluxcore3D
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

CX = np.array([0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1, 0, 0, 0, 0])
CY = np.array([0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1])
CZ = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1])
W = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)


def state(shape, rng, umean=(0.05, 0.0, 0.0), spread=0.06):
    """Equilibrium of a random (rho, u) field plus non-equilibrium noise, FP32, [19][N]."""
    n = int(np.prod(shape))
    rho = 1.0 + 0.02 * (rng.random(n) - 0.5)
    u = [m + spread * (rng.random(n) - 0.5) for m in umean]
    cu = 3.0 * (CX[:, None] * u[0] + CY[:, None] * u[1] + CZ[:, None] * u[2])
    usq = 1.5 * (u[0] ** 2 + u[1] ** 2 + u[2] ** 2)
    f = W[:, None] * rho * (1 + cu + 0.5 * cu * cu - usq)
    f *= 1.0 + 0.01 * (rng.random(f.shape) - 0.5)
    return np.ascontiguousarray(f.astype(np.float32))


def plane_cells(shape, axis, idx):
    """Flat indices of plane `idx` normal to `axis`, in the kernels' (a, b) order."""
    i, j, k = np.meshgrid(*(np.arange(n) for n in shape), indexing="ij")
    flat = (i * shape[1] + j) * shape[2] + k
    return np.ascontiguousarray(np.take(flat, idx, axis=axis).reshape(-1))


def main(ref_root: str) -> None:
    from oracle import build_ref
    from oracle.lbm import mrt_rates
    lib = C.CDLL(build_ref.build(ref_root))
    vp, i32, f32 = C.c_void_p, C.c_int, C.c_float
    lib.ref_zou_he_bc.argtypes = [vp, vp, i32, i32, i32, i32, i32, i32, i32, f32, f32, i32]
    lib.ref_convective_bc.argtypes = [vp, vp, i32, i32, i32, i32, i32, i32, i32, f32, i32, i32, vp, vp]
    lib.ref_macro_collide_mrt_smag.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, f32, f32, i32]
    rng = np.random.default_rng(7)
    out = {}
    solids = {}

    def solid_of(shape):
        key = "solid_%dx%dx%d" % shape
        if key not in solids:
            solids[key] = np.ascontiguousarray((rng.random(shape) < 0.15).astype(np.uint8).reshape(-1))
            out[key] = solids[key]
        return solids[key]

    # Zou/He: (name, shape, axis, plane, interior, bc_type, u_in, rho_out, sign, mean velocity of the state)
    zh = [("inlet_x_low", (4, 10, 8), 0, 0, 1, 0, 0.05, 1.0, 1, (0.05, 0, 0)),
          ("outlet_x_high", (4, 10, 8), 0, 3, 2, 1, 0.0, 1.0, 1, (0.01, 0, 0)),
          ("inlet_y_high", (10, 4, 8), 1, 3, 2, 0, -0.04, 1.0, -1, (0, -0.04, 0)),
          ("outlet_y_low", (10, 4, 8), 1, 0, 1, 1, 0.0, 1.002, -1, (0, -0.01, 0)),
          ("outlet_z_low", (8, 10, 4), 2, 0, 1, 1, 0.0, 0.998, -1, (0, 0, -0.01)),
          ("inlet_z_low", (8, 10, 4), 2, 0, 1, 0, 0.06, 1.0, 1, (0, 0, 0.06))]
    for name, shape, axis, plane, inter, bct, uin, rout, sign, um in zh:
        f = state(shape, rng, um)
        s = solid_of(shape)
        g = f.copy()
        lib.ref_zou_he_bc(g.ctypes.data, s.ctypes.data, *shape, axis, plane, inter, bct, uin, rout, sign)
        pc = plane_cells(shape, axis, plane)
        assert np.array_equal(np.delete(g, pc, axis=1), np.delete(f, pc, axis=1))
        out[f"zh_{name}_in"], out[f"zh_{name}_plane"] = f, g[:, pc]
        out[f"zh_{name}_args"] = np.array([*shape, axis, plane, inter, bct, uin, rout, sign], dtype=np.float64)
    # convective: (name, shape, axis, outlet, interior, unknown_cax, rho_out)
    cv = [("x_high", (4, 10, 8), 0, 3, 2, -1, 1.0),
          ("z_low", (8, 10, 4), 2, 0, 1, 1, 1.001),
          ("x_high_two_blocks", (3, 24, 20), 0, 2, 1, -1, 0.999)]
    for name, shape, axis, o, inter, ucax, rout in cv:
        f = state(shape, rng, (0.03, 0.01, 0.0))
        s = solid_of(shape)
        g = f.copy()
        n1, n2 = {0: (shape[1], shape[2]), 1: (shape[0], shape[2]), 2: (shape[0], shape[1])}[axis]
        ssum, cnt = C.c_float(0), C.c_int(0)
        lib.ref_convective_bc(g.ctypes.data, s.ctypes.data, *shape, axis, o, inter, ucax, rout, n1, n2,
                              C.byref(ssum), C.byref(cnt))
        pc = plane_cells(shape, axis, o)
        assert np.array_equal(np.delete(g, pc, axis=1), np.delete(f, pc, axis=1))
        out[f"cv_{name}_in"], out[f"cv_{name}_plane"] = f, g[:, pc]
        out[f"cv_{name}_args"] = np.array([*shape, axis, o, inter, ucax, rout, n1, n2, ssum.value, cnt.value],
                                          dtype=np.float64)
    # MRT-Smagorinsky collision
    shape = (6, 10, 8)
    N = int(np.prod(shape))
    f = state(shape, rng, (0.05, 0.01, -0.01), spread=0.1)
    s = solid_of(shape)
    S = mrt_rates(1.0 / 0.56).astype(np.float32)
    fp = np.zeros_like(f)
    mac = np.zeros((4, N), np.float32)
    lib.ref_macro_collide_mrt_smag(f.ctypes.data, fp.ctypes.data, mac[0].ctypes.data, mac[1].ctypes.data,
                                   mac[2].ctypes.data, mac[3].ctypes.data, s.ctypes.data, S.ctypes.data,
                                   0.01, 1.0 / 0.56, N)
    out.update(smag_f=f, smag_shape=np.array(shape), smag_S=S, smag_params=np.array([0.01, 1.0 / 0.56]),
               smag_out_fp=fp, smag_out_macro=mac)
    np.savez_compressed(os.path.join(HERE, "ref_lbm.npz"), **out)
    print("ref_lbm.npz written to", HERE, "with", len(out), "arrays")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_ref_fixtures.py /path/to/fluxcore3D")
    main(sys.argv[1])
