"""TEST INFRASTRUCTURE: numpy restatement of the reference's multigrid thermal solver
and its Krylov wrappers (fluxcore3D solver/nlevel_mg_cuda.py, solver/mg_kernels.cu,
solver/mg_pcg.py, and the thermal step of LBM_CHT.py:2571-2712 / solver/thermal_kernels.cu).

CUDA-path semantics are followed where the reference's torch and CUDA paths
differ: M(T) = T + dt L(T) is evaluated as the fused kernel does
(mg_kernels.cu:92-105) and L_apply_fine as (M(T) - T)/dt (nlevel_mg_cuda.py:169-174).
Runs in float32 (parity) or float64 (plain-method reference).
Parity status: pinned against fixtures from the reference's own torch
NLevelGeometricMGSolver / pcg_mg / bicgstab_mg (tests/golden/make_golden.py).
"""
from __future__ import annotations

import numpy as np


def _ghost_low(ax: int, out_idx: int, axis: int) -> int:
    """mg_kernels.cu:37-44: low-face ghost index."""
    return 0 if (ax == axis and out_idx != 0) else 1


def shift(A: np.ndarray, dim: int, step: int, ax: int, out_idx: int) -> np.ndarray:
    """Neighbour field with the operator's ghosting (nlevel_mg_cuda.py:431-469)."""
    B = np.empty_like(A)
    n = A.shape[dim]
    src = np.arange(n)
    if step == +1:
        idx = np.minimum(src + 1, n - 1)
        idx[n - 1] = n - 2
    else:
        idx = src - 1
        idx[0] = _ghost_low(ax, out_idx, dim)
    B[...] = np.take(A, idx, axis=dim)
    return B


def build_coeffs(k, rcp, u, v, w, ax, out_idx, dx, s, dtype):
    """nlevel_mg_cuda.py:417-507 (harmonic face k, upwind convection)."""
    k = k.astype(dtype)
    one = dtype(1.0)
    tiny = dtype(1e-30)
    inv_rcp = one / (rcp.astype(dtype) + tiny)
    two = dtype(2.0)
    cd = dtype(s / (dx * dx))
    ca = dtype(s / dx)
    out = {}
    for name, dim, st in (("E", 0, 1), ("W", 0, -1), ("N", 1, 1), ("S", 1, -1), ("U", 2, 1), ("D", 2, -1)):
        kn = shift(k, dim, st, ax, out_idx)
        kf = (two * k * kn) / (k + kn + tiny)
        out[name] = cd * kf * inv_rcp
    zero = dtype(0)
    uu, vv, ww = (t.astype(dtype) for t in (u, v, w))
    out["W"] = out["W"] + ca * np.maximum(uu, zero)
    out["E"] = out["E"] + ca * np.maximum(-uu, zero)
    out["S"] = out["S"] + ca * np.maximum(vv, zero)
    out["N"] = out["N"] + ca * np.maximum(-vv, zero)
    out["D"] = out["D"] + ca * np.maximum(ww, zero)
    out["U"] = out["U"] + ca * np.maximum(-ww, zero)
    diag = out["E"] + out["W"] + out["N"] + out["S"] + out["U"] + out["D"]
    return out, diag


def restrict_mean(x: np.ndarray) -> np.ndarray:
    """nlevel_mg_cuda.py:511-519 (2x mean over the even-cropped block)."""
    n0, n1, n2 = (d // 2 for d in x.shape)
    v = x[:2 * n0, :2 * n1, :2 * n2].reshape(n0, 2, n1, 2, n2, 2)
    return v.mean(axis=(1, 3, 5), dtype=np.float64).astype(x.dtype)


def _src_index(nf: int, nc: int):
    scale = np.float32(nc) / np.float32(nf)
    s = np.maximum(scale * (np.arange(nf, dtype=np.float32) + np.float32(0.5)) - np.float32(0.5), np.float32(0))
    i0 = np.minimum(s.astype(np.int64), nc - 1)
    i1 = i0 + (i0 < nc - 1)
    l1 = (s - i0).astype(np.float32)
    return i0, i1, l1


def prolong(xc: np.ndarray, shape) -> np.ndarray:
    """Trilinear interpolation with align_corners=False (nlevel_mg_cuda.py:531-537)."""
    (i0, i1, li), (j0, j1, lj), (k0, k1, lk) = (_src_index(nf, nc) for nf, nc in zip(shape, xc.shape))
    dt = xc.dtype
    li, lj, lk = li.astype(dt)[:, None, None], lj.astype(dt)[None, :, None], lk.astype(dt)[None, None, :]

    def X(a, b, c):
        return xc[np.ix_(a, b, c)]
    one = dt.type(1)
    return ((one - li) * ((one - lj) * ((one - lk) * X(i0, j0, k0) + lk * X(i0, j0, k1)) +
                          lj * ((one - lk) * X(i0, j1, k0) + lk * X(i0, j1, k1))) +
            li * ((one - lj) * ((one - lk) * X(i1, j0, k0) + lk * X(i1, j0, k1)) +
                  lj * ((one - lk) * X(i1, j1, k0) + lk * X(i1, j1, k1))))


class OracleMG:
    """NLevelGeometricMGSolver (nlevel_mg_cuda.py:38-307) on numpy arrays."""

    def __init__(self, k, rcp, u, v, w, mask, ax, sign, s, omega=0.8, n_pre=2, n_post=2, n_coarse=20,
                 min_coarse_cells=4, max_levels=None, real=np.float64, flux=False, coarse_solve="jacobi"):
        self.dt_ = real
        self.flux = flux
        self.coarse_solve = coarse_solve
        self.ax, self.sign, self.s, self.omega = ax, sign, s, omega
        self.n_pre, self.n_post, self.n_coarse = n_pre, n_post, n_coarse
        self.levels = []
        fields = [np.asarray(t, dtype=np.float32) for t in (k, rcp, u, v, w)]
        msk = np.asarray(mask, dtype=np.float32)
        while True:
            shape = fields[0].shape
            out_idx = (shape[ax] - 1) if sign == +1 else 0
            dx = float(2 ** len(self.levels))
            a, diag = build_coeffs(*fields, ax, out_idx, dx, s, real)
            self.levels.append({"shape": shape, "out_idx": out_idx, "a": a, "diag": diag,
                                "mask": msk.astype(real), "x": np.zeros(shape, real), "b": np.zeros(shape, real)})
            if min(d // 2 for d in shape) <= min_coarse_cells:
                break
            if max_levels is not None and len(self.levels) >= max_levels:
                break
            fields = [restrict_mean(t) for t in fields]
            msk = (restrict_mean(msk) >= np.float32(0.999)).astype(np.float32)
        self.dt = None

    def set_dt(self, dt):
        self.dt = float(dt)
        r = self.dt_
        for lv in self.levels:
            d = np.maximum(r(1.0) + r(dt) * lv["diag"], r(1e-12))
            lv["inv"] = (r(self.omega) / d) * lv["mask"]

    def L(self, lv, x):
        """The 7-point operator.  flux=False: diag*x - sum_n a_n x_n, the reference's form
        (mg_kernels.cu:55-106); flux=True: sum_n a_n (x - x_n), equal in exact arithmetic
        (diag = sum_n a_n) and the form the CUDA kernels evaluate, which stays exact on
        constant fields once the coefficients are rounded."""
        a = lv["a"]
        ax, oi = self.ax, lv["out_idx"]
        if self.flux:
            s = None
            for name, dim, st in (("E", 0, 1), ("W", 0, -1), ("N", 1, 1), ("S", 1, -1), ("U", 2, 1), ("D", 2, -1)):
                t = a[name] * (x - shift(x, dim, st, ax, oi))
                s = t if s is None else s + t
            return s
        return (lv["diag"] * x - a["E"] * shift(x, 0, 1, ax, oi) - a["W"] * shift(x, 0, -1, ax, oi)
                - a["N"] * shift(x, 1, 1, ax, oi) - a["S"] * shift(x, 1, -1, ax, oi)
                - a["U"] * shift(x, 2, 1, ax, oi) - a["D"] * shift(x, 2, -1, ax, oi))

    def mop(self, lv, x):
        return x + self.dt_(self.dt) * self.L(lv, x)

    def L_apply_fine(self, T):
        lv = self.levels[0]
        T = np.asarray(T, self.dt_)
        return (self.mop(lv, T) - T) / self.dt_(self.dt)

    def smooth(self, lv, n):
        for _ in range(n):
            lv["x"] = lv["x"] + lv["inv"] * (lv["b"] - self.mop(lv, lv["x"]))

    def coarse_matrix(self, lv):
        """A = I + dt L of a level as a dense FP64 matrix, column j = the operator applied (in FP64) to
        the unit vector e_j, so the operator's ghosting is whatever L does."""
        n = int(np.prod(lv["shape"]))
        a64 = {kk: np.asarray(vv, np.float64) for kk, vv in lv["a"].items()}
        lv64 = dict(lv, a=a64, diag=np.asarray(lv["diag"], np.float64))
        A = np.empty((n, n))
        e = np.zeros(n)
        for j in range(n):
            e[j] = 1.0
            x = e.reshape(lv["shape"])
            A[:, j] = (x + float(self.dt) * self.L(lv64, x)).reshape(-1)
            e[j] = 0.0
        return A

    def coarse_exact(self, lv):
        """The 'fp64' coarse solve: A x = b exactly in FP64 on the cells with mask 1, x = 0 elsewhere."""
        m = np.asarray(lv["mask"]).reshape(-1) != 0
        A = self.coarse_matrix(lv)
        b = np.asarray(lv["b"], np.float64).reshape(-1)
        x = np.zeros(b.size)
        x[m] = np.linalg.solve(A[np.ix_(m, m)], b[m])
        return x.reshape(lv["shape"]).astype(self.dt_)

    def vcycle(self, level=0):
        lv = self.levels[level]
        if level == len(self.levels) - 1:
            if self.coarse_solve == "fp64" and level > 0:
                lv["x"] = self.coarse_exact(lv)
            else:
                self.smooth(lv, self.n_coarse)
            return
        self.smooth(lv, self.n_pre)
        r = (lv["b"] - self.mop(lv, lv["x"])) * lv["mask"]
        lc = self.levels[level + 1]
        lc["b"] = restrict_mean(r)
        lc["x"] = np.zeros(lc["shape"], self.dt_)
        self.vcycle(level + 1)
        lv["x"] = (lv["x"] + self.dt_(0.75) * prolong(lc["x"], lv["shape"])) * lv["mask"]
        self.smooth(lv, self.n_post)

    def solve(self, b, x0=None, max_cycles=50, tol=1e-6):
        """nlevel_mg_cuda.py:102-162 (residual norm includes the unmasked Dirichlet rows)."""
        lv = self.levels[0]
        m = lv["mask"]
        b = np.asarray(b, self.dt_)
        lv["x"] = (np.asarray(x0, self.dt_) * m) if x0 is not None else np.zeros(lv["shape"], self.dt_)
        lv["b"] = b * m
        bn = float(np.linalg.norm(b.astype(np.float64))) + 1e-30
        res = res0 = float("inf")
        conv = False
        cyc = 0
        for cyc in range(max_cycles):
            self.vcycle(0)
            r = lv["b"] - self.mop(lv, lv["x"])
            res = float(np.linalg.norm(r.astype(np.float64))) / bn
            if cyc == 0:
                res0 = res
            if not res < float("inf"):
                break
            if cyc > 2 and res > 10.0 * res0:
                break
            if res < tol:
                conv = True
                break
        return lv["x"] * m, {"converged": conv, "it": cyc + 1, "res_rel": res, "res0_rel": res0}

    def precond(self, r):
        """One V-cycle from zero (mg_pcg.py:178-187)."""
        lv = self.levels[0]
        lv["x"] = np.zeros(lv["shape"], self.dt_)
        lv["b"] = np.asarray(r, self.dt_) * lv["mask"]
        self.vcycle(0)
        return lv["x"] * lv["mask"]


def bicgstab(mg: OracleMG, b, x0=None, tol=1e-3, max_it=15):
    """mg_pcg.py:103-175 (preconditioned BiCGSTAB, one V-cycle per application)."""
    lv = mg.levels[0]
    m = lv["mask"]
    r_ = mg.dt_
    b = np.asarray(b, r_)
    x = (np.asarray(x0, r_) if x0 is not None else np.zeros_like(b)) * m
    r = (b - mg.mop(lv, x)) * m
    rh = r.copy()
    bn = float(np.sqrt(np.dot(b.ravel().astype(np.float64), b.ravel()))) + 1e-30
    rho = alpha = omega = 1.0
    v = np.zeros_like(b)
    p = np.zeros_like(b)
    conv = False
    it = 0
    dot = lambda a, c: float(np.dot(a.ravel().astype(np.float64), c.ravel().astype(np.float64)))
    for it in range(max_it):
        if np.sqrt(dot(r, r)) / bn < tol:
            conv = True
            break
        rho_new = dot(rh, r)
        if abs(rho_new) < 1e-30:
            break
        beta = (rho_new / (rho + 1e-30)) * (alpha / (omega + 1e-30))
        p = r + r_(beta) * (p - r_(omega) * v)
        ph = mg.precond(p)
        v = mg.mop(lv, ph)
        alpha = rho_new / (dot(rh, v) + 1e-30)
        s = (r - r_(alpha) * v) * m
        if np.sqrt(dot(s, s)) / bn < tol:
            x = x + r_(alpha) * ph
            conv = True
            break
        sh = mg.precond(s)
        t = mg.mop(lv, sh)
        omega = dot(t, s) / (dot(t, t) + 1e-30)
        x = (x + r_(alpha) * ph + r_(omega) * sh) * m
        r = (s - r_(omega) * t) * m
        rho = rho_new
    return x * m, {"converged": conv, "it": it + 1, "res_rel": float(np.sqrt(dot(r, r)) / bn)}


def true_residual(mg: OracleMG, x, b):
    """||mask (b - A x)|| / ||mask b|| in float64."""
    lv = mg.levels[0]
    m = lv["mask"].astype(np.float64)
    saved = mg.dt_
    mg.dt_ = np.float64
    r = (np.asarray(b, np.float64) - mg.mop(lv, np.asarray(x, np.float64))) * m
    mg.dt_ = saved
    return float(np.linalg.norm(r) / (np.linalg.norm(np.asarray(b, np.float64) * m) + 1e-300))


def reconstruct(T0, theta, ax, out_idx):
    """thermal_kernels.cu:61-114: T = T0 + theta with Neumann copies on every face except the inlet."""
    val = T0 + theta
    nx, ny, nz = val.shape
    out = val.copy()
    for i in range(nx):
        for j in range(ny):
            for k in range(nz):
                s = None
                if i == nx - 1:
                    s = (i - 1, j, k)
                elif i == 0 and (ax != 0 or out_idx == 0):
                    s = (1, j, k)
                elif j == ny - 1:
                    s = (i, j - 1, k)
                elif j == 0 and (ax != 1 or out_idx == 0):
                    s = (i, 1, k)
                elif k == nz - 1:
                    s = (i, j, k - 1)
                elif k == 0 and (ax != 2 or out_idx == 0):
                    s = (i, j, 1)
                if s is not None:
                    out[i, j, k] = val[s]
    return out


def thermal_step(mg: OracleMG, T_old, T0, src, mask, dt, tol, max_cycles, ax, out_idx):
    """One pseudo-time step of thermal_cuda_ext.py:55-201 (fused variant)."""
    r = mg.dt_
    m = np.asarray(mask, r)
    LT0 = mg.L_apply_fine(T0)
    rhs = m * ((np.asarray(T_old, r) + r(dt) * np.asarray(src, r)) - (np.asarray(T0, r) + r(dt) * LT0))
    theta0 = m * (np.asarray(T_old, r) - np.asarray(T0, r))
    theta, info = mg.solve(rhs, theta0, max_cycles=max_cycles, tol=tol)
    return reconstruct(np.asarray(T0, r), theta * m, ax, out_idx), info
